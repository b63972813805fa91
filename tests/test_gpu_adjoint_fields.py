"""Discrete adjoint of the pressure equation with respect to the cell fields
(semo_vjp_fields, GPU, C-ABI).

J = sum of x_i^2 over the cells on the z = 1 patch, x the pressure-correction
solution of A x = b(U, V, W, P).  A depends only on geometry, dt and the
densities, so dJ/dphi = (db/dphi)^T lambda, lambda = A^-T dJ/dx: the
transposed face-flux kernel (skew-corrected, stencil-limited face velocity
and the Rhie-Chow pressure terms) applied to lambda.  Checked against

* the oracle's own Jacobian: every column db/dphi_k of the oracle's FP64
  assembly by central differences (b is piecewise linear, so a column is
  exact unless the step crosses a limiter kink, which shows as a column that
  changes between h and h/2 and is left out), contracted with the oracle's
  lambda, on a small case with random fields and every boundary rule (slip,
  no-slip, fixed velocity, fixed and zero-gradient pressure): this covers the
  clamped reconstructions, whose derivative goes to the stencil cell holding
  the limit;
* central finite differences (h = 1e-6) along 16 seeded directions (seeds
  100-115) in (U, V, W, P) on the jittered 64^3 mesh, with U, V, W linear in
  space (no reconstruction near a limiter kink, so J is exactly quadratic
  along every direction) and P random.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 1e-6
FD_TOL = 1e-6       # relative, over the 16 directional derivatives
JAC_TOL = 1e-7      # relative (max norm) against the oracle's Jacobian-transpose product
SOLVE_TOL = 1e-12
FIELDS = ("U", "V", "W", "P")


@pytest.fixture(scope="module")
def semo():
    import semo_mesh_gb300 as S
    S.load_library()
    return S


def small_case():
    from semo_mesh_gb300.cases import vof_case, with_fields
    c = with_fields(vof_case(5), seed=41, p_scale=100.0)
    names = c.mesh.patch_names
    c.bc_type[names.index("xmin"), 1] = 3                 # slip
    c.bc_type[names.index("ymin"), 1] = 2                 # no-slip
    c.bc_type[names.index("ymax"), 1] = 1                 # fixed velocity
    c.bc_value[names.index("ymax")] = (0.0, 0.5, -0.2, 0.1, 0.0)
    return c


def oracle_jt_lambda(case, zc):
    """(db/dphi)^T lambda from the oracle's assembled b, column by column;
    the mask marks the columns left out (kink within the step)."""
    from oracle.oracle import Oracle
    n = case.mesh.n_cells
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble()
    x = o.solve(False, 1e-13, 1000)["x"]
    g = np.zeros(n)
    g[zc] = 2.0 * x[zc]
    o.set("B", g)
    lam = o.solve(False, 1e-13, 1000)["x"]        # A is symmetric
    F = np.array([case.U, case.V, case.W, case.P], dtype=np.float64)

    def b_of(f):
        for q, nm in enumerate(FIELDS):
            o.set(nm, f[q])
        o.set("VF", case.VF)
        o.assemble()
        return o.get("B")

    jt = np.zeros((4, n))
    keep = np.ones((4, n), bool)
    for q in range(4):
        for k in range(n):
            sc = max(1.0, abs(F[q, k]))

            def col(h):
                fp = F.copy(); fp[q, k] += h * sc
                fm = F.copy(); fm[q, k] -= h * sc
                return (b_of(fp) - b_of(fm)) / (2.0 * h * sc)
            c1, c2 = col(1e-7), col(5e-8)
            keep[q, k] = np.abs(c1 - c2).max() <= 1e-6 * max(np.abs(c1).max(), 1e-300)
            jt[q, k] = c1 @ lam
    return x, lam, jt, keep


def test_vjp_fields_matches_oracle_jacobian(semo):
    case = small_case()
    zc = np.unique(case.mesh.patch_cells("zmax"))
    x_o, lam_o, jt, keep = oracle_jt_lambda(case, zc)
    assert keep.sum() >= 0.95 * keep.size
    ctx = semo.Context(precision="fp64", tol=SOLVE_TOL, max_iter=1000)
    ctx.set_case(case)
    ctx.assemble()
    res = ctx.solve()
    assert np.linalg.norm(res.x - x_o) <= 1e-9 * np.linalg.norm(x_o)
    g = np.zeros(case.mesh.n_cells)
    g[zc] = 2.0 * res.x[zc]
    lam, grads, info = ctx.vjp_fields(g)
    assert info["rel_residual"] <= SOLVE_TOL
    assert np.linalg.norm(lam - lam_o) <= 1e-9 * np.linalg.norm(lam_o)
    scale = np.abs(jt).max()
    for q, nm in enumerate(FIELDS):
        err = np.abs(grads[nm] - jt[q])[keep[q]].max() / scale
        assert err < JAC_TOL, (nm, err)
    ctx.close()


def linear_fields(case):
    from semo_mesh_gb300.cases import approx_cell_centres
    cc = approx_cell_centres(case.mesh)
    x, y, z = cc[:, 0], cc[:, 1], cc[:, 2]
    case.U = 0.3 + 1.0 * x - 0.5 * y + 0.25 * z
    case.V = -0.2 + 0.4 * x + 0.8 * y - 0.6 * z
    case.W = 0.1 - 0.7 * x + 0.3 * y + 0.9 * z
    case.P = 50.0 * np.random.default_rng(7).standard_normal(case.mesh.n_cells)
    return case


def test_vjp_fields_matches_central_differences(semo):
    from semo_mesh_gb300.cases import box_case
    case = linear_fields(box_case(64, jitter=0.2))
    n = case.mesh.n_cells
    zc = np.unique(case.mesh.patch_cells("zmax"))
    ctx = semo.Context(precision="fp64", tol=SOLVE_TOL, max_iter=1000)
    ctx.set_case(case)

    def J(f):
        ctx.set_fields(f[3], f[0], f[1], f[2], case.VF)
        ctx.assemble()
        r = ctx.solve()
        assert r.info["rel_residual"] <= SOLVE_TOL
        return float(np.sum(r.x[zc] ** 2)), r.x

    F = np.array([case.U, case.V, case.W, case.P])
    _, x = J(F)
    g = np.zeros(n)
    g[zc] = 2.0 * x[zc]
    _, grads, info = ctx.vjp_fields(g)
    G = np.array([grads[nm] for nm in FIELDS])
    fd, ad = [], []
    for seed in range(100, 116):
        d = np.random.default_rng(seed).standard_normal((4, n))
        jp, _ = J(F + H * d)
        jm, _ = J(F - H * d)
        fd.append((jp - jm) / (2.0 * H))
        ad.append(float(np.sum(G * d)))
    fd, ad = np.array(fd), np.array(ad)
    err = np.linalg.norm(ad - fd) / np.linalg.norm(fd)
    assert err < FD_TOL, (err, ad, fd)
    ctx.close()


def test_vjp_fields_needs_forward(semo):
    from semo_mesh_gb300.cases import vof_case
    case = vof_case(4)
    ctx = semo.Context()
    ctx.set_case(case)
    with pytest.raises(semo.SemoError) as e:
        ctx.vjp_fields(np.ones(case.mesh.n_cells))
    assert e.value.status == 8   # SEMO_ERR_STATE
    ctx.close()
