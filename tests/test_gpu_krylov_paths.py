"""The Krylov loops' entry and exit paths through the C-ABI.

The CG graph decides on the device whether to iterate at all (k_cg_begin)
and the host reads the outcome once, after the true residual; the batched
BiCGStab keeps its instantiated graph across calls while its buffers and
scalars stay the same.  So: a zero right-hand side and an exact initial guess
take no CG iteration and return at once; a non-finite right-hand side is
reported as SEMO_ERR_NAN after the graph; one context alternating BiCGStab
systems of different sizes and right-hand-side counts solves each correctly
(the kept graph is replaced whenever a baked pointer or size changes); a
zero component of the momentum overload stays inactive (no iteration, x = 0)
while the others converge.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def semo():
    import semo_mesh_gb300 as S
    S.load_library()
    return S


def coo_sorted(r, c, v, n):
    """Diagonal entries first, then each row's off-diagonals by column."""
    d = r == c
    off = np.lexsort((c[~d], r[~d]))
    dr = np.argsort(r[d], kind="stable")
    return (np.concatenate([r[d][dr], r[~d][off]]).astype(np.int32),
            np.concatenate([c[d][dr], c[~d][off]]).astype(np.int32),
            np.concatenate([v[d][dr], v[~d][off]]))


def poisson3d(m, shift=0.05):
    """SPD 7-point Laplacian on an m^3 grid plus shift * I."""
    n = m ** 3
    idx = np.arange(n)
    x, y, z = idx % m, (idx // m) % m, idx // (m * m)
    rows, cols, vals = [idx], [idx], [np.full(n, 6.0 + shift)]
    for d, coord in ((1, x), (m, y), (m * m, z)):
        for sgn in (-1, 1):
            ok = (coord + sgn >= 0) & (coord + sgn < m)
            rows.append(idx[ok]); cols.append(idx[ok] + sgn * d); vals.append(np.full(ok.sum(), -1.0))
    return coo_sorted(np.concatenate(rows), np.concatenate(cols), np.concatenate(vals), n) + (n,)


def convection2d(m, seed):
    """Non-symmetric, diagonally dominant upwind convection-diffusion on an m^2
    grid with a BDF2-like mass term (the momentum and volume-fraction shape)."""
    rng = np.random.default_rng(seed)
    n = m * m
    idx = np.arange(n)
    x, y = idx % m, idx // m
    rows, cols, vals = [], [], []
    diag = np.full(n, 3.0)
    for d, coord in ((1, x), (m, y)):
        for sgn in (-1, 1):
            ok = (coord + sgn >= 0) & (coord + sgn < m)
            w = 1.0 + (0.8 * rng.random(ok.sum()) if sgn < 0 else np.zeros(ok.sum()))
            rows.append(idx[ok]); cols.append(idx[ok] + sgn * d); vals.append(-w)
            np.add.at(diag, idx[ok], w)
    rows.append(idx); cols.append(idx); vals.append(diag)
    return coo_sorted(np.concatenate(rows), np.concatenate(cols), np.concatenate(vals), n) + (n,)


def dense_solve(r, c, v, n, b):
    A = np.zeros((n, n))
    np.add.at(A, (r, c), v)
    return np.linalg.solve(A, b)


def test_cg_zero_rhs_and_exact_guess(semo):
    r, c, v, n = poisson3d(12)
    ctx = semo.Context(precision="mixed", tol=1e-10)
    res = ctx.solve_amgcl("pressure", 1, r, c, v, np.zeros(n))
    assert res.info["iterations"] == 0
    assert res.info["rel_residual"] == 0.0
    assert np.array_equal(res.x, np.zeros(n))
    b = np.random.default_rng(1).standard_normal(n)
    first = ctx.solve_amgcl("pressure", 1, r, c, v, b)
    assert first.info["iterations"] > 0 and first.info["rel_residual"] <= 1e-10
    ref = dense_solve(r, c, v, n, b)
    assert np.linalg.norm(first.x - ref) / np.linalg.norm(ref) < 1e-8
    # from the converged solution: the initial residual already meets the tolerance
    again = ctx.solve_amgcl("pressure", 1, r, c, v, b, first.x)
    assert again.info["iterations"] == 0
    assert again.info["rel_residual"] <= 1e-10
    ctx.close()


def test_cg_nan_rhs_reported_after_graph(semo):
    r, c, v, n = poisson3d(8)
    ctx = semo.Context(precision="fp64", tol=1e-10)
    b = np.ones(n)
    b[5] = np.nan
    with pytest.raises(semo.SemoError) as e:
        ctx.solve_amgcl("pressure", 1, r, c, v, b)
    assert e.value.status == 6
    # the context stays usable
    ok = ctx.solve_amgcl("pressure", 1, r, c, v, np.ones(n))
    assert ok.info["rel_residual"] <= 1e-10
    ctx.close()


def test_bicgstab_kept_graph_across_systems(semo):
    """Alternate volume-fraction (1 RHS) and momentum (3 RHS) systems of two
    sizes in one context; every solution matches a dense solve."""
    ctx = semo.Context(precision="fp64", mom_tol=1e-11)
    rng = np.random.default_rng(7)
    systems = [convection2d(20, 1), convection2d(27, 2)]
    for rep in range(2):
        for k, (r, c, v, n) in enumerate(systems):
            b = rng.standard_normal(n)
            res = ctx.solve_amgcl("volume_fraction", 1, r, c, v, b)
            ref = dense_solve(r, c, v, n, b)
            assert res.info["rel_residual"] <= 1e-11, (rep, k)
            assert np.linalg.norm(res.x - ref) / np.linalg.norm(ref) < 1e-9, (rep, k)
            B = [rng.standard_normal(n) for _ in range(3)]
            out = ctx.solve_amgcl("momentum", 1, r, c, v, *B)
            for j in range(3):
                refj = dense_solve(r, c, v, n, B[j])
                assert out[j].info["rel_residual"] <= 1e-11, (rep, k, j)
                assert np.linalg.norm(out[j].x - refj) / np.linalg.norm(refj) < 1e-9, (rep, k, j)
    ctx.close()


def test_bicgstab_zero_and_nan_components(semo):
    r, c, v, n = convection2d(16, 3)
    ctx = semo.Context(precision="fp64", mom_tol=1e-11)
    b1 = np.random.default_rng(4).standard_normal(n)
    out = ctx.solve_amgcl("momentum", 1, r, c, v, np.zeros(n), b1, np.zeros(n))
    assert out[0].info["iterations"] == 0 and out[2].info["iterations"] == 0
    assert np.array_equal(out[0].x, np.zeros(n)) and np.array_equal(out[2].x, np.zeros(n))
    ref = dense_solve(r, c, v, n, b1)
    assert out[1].info["iterations"] > 0
    assert np.linalg.norm(out[1].x - ref) / np.linalg.norm(ref) < 1e-9
    bad = b1.copy()
    bad[3] = np.inf
    with pytest.raises(semo.SemoError) as e:
        ctx.solve_amgcl("momentum", 1, r, c, v, b1, bad, b1)
    assert e.value.status == 6
    ok = ctx.solve_amgcl("volume_fraction", 1, r, c, v, b1)
    assert np.linalg.norm(ok.x - ref) / np.linalg.norm(ref) < 1e-9
    ctx.close()
