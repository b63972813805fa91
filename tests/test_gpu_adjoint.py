"""Discrete adjoint of the pressure solve with a per-cell source (GPU, C-ABI).

The source s enters the pressure right-hand side as b_i += s_i V_i and the
objective is J = sum of x_i^2 over the cells on the z = 1 patch, x the
pressure-correction solution.  semo_vjp_source returns lambda = A^-T dJ/dx
and dJ/ds = V lambda, solved on the forward hierarchy.  It is checked against

* central finite differences (h = 1e-6) along 16 seeded directions
  (seeds 100-115), and
* the oracle's FP64 gradient formed from its own assembled A, which is
  symmetric: a face's off-diagonal coefficient is written to both of its
  rows (eqPressure.cpp:538-548), so A^T lambda = A lambda.

J is exactly quadratic in s, so central differences carry no truncation
error; what is left is rounding in J and the solve error divided by h, hence
the tight FP64 tolerance of the forward solves.  The reference itself has no adjoint.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 1e-6
FD_TOL = 1e-6         # relative, over the 16 directional derivatives
ORACLE_TOL = 1e-7     # relative L2 of dJ/ds against the oracle's gradient
SOLVE_TOL = 1e-12


@pytest.fixture(scope="module")
def semo():
    import semo_mesh_gb300 as S
    S.load_library()
    return S


@pytest.fixture(scope="module")
def adj_case():
    from semo_mesh_gb300.cases import box_case
    case = box_case(64, jitter=0.2)
    s = np.random.default_rng(4).standard_normal(case.mesh.n_cells)
    zc = np.unique(case.mesh.patch_cells("zmax"))
    return case, s, zc


def objective(x, zc):
    return float(np.sum(x[zc] ** 2))


def forward(ctx, s):
    ctx.set_source(s)
    ctx.assemble()
    res = ctx.solve()
    assert res.info["rel_residual"] <= SOLVE_TOL
    return res.x


@pytest.fixture(scope="module")
def oracle_grad(adj_case):
    from oracle.oracle import Oracle
    case, s, zc = adj_case
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble()
    vol = o.get("cell_vol")
    b0 = o.get("B")
    o.set("B", b0 + s * vol)
    x = o.solve(False, 1e-13, 1000)["x"]
    g = np.zeros_like(x)
    g[zc] = 2.0 * x[zc]
    o.set("B", g)
    lam = o.solve(False, 1e-13, 1000)["x"]
    ptr, col, val = o.get("csr_ptr"), o.get("csr_col"), o.get("csr_val")
    return x, lam * vol, (ptr, col, val)


def test_oracle_matrix_symmetric(oracle_grad):
    sp = pytest.importorskip("scipy.sparse")
    _, _, (ptr, col, val) = oracle_grad
    a = sp.csr_matrix((val, col, ptr))
    assert (a != a.T).nnz == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_vjp_matches_oracle_gradient(semo, adj_case, oracle_grad, precision):
    case, s, zc = adj_case
    x_ref, djds_ref, _ = oracle_grad
    ctx = semo.Context(precision=precision, tol=SOLVE_TOL, max_iter=1000)
    ctx.set_case(case)
    x = forward(ctx, s)
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < ORACLE_TOL
    g = np.zeros(case.mesh.n_cells)
    g[zc] = 2.0 * x[zc]
    lam, djds, info = ctx.vjp_source(g)
    assert info["rel_residual"] <= SOLVE_TOL
    err = np.linalg.norm(djds - djds_ref) / np.linalg.norm(djds_ref)
    assert err < ORACLE_TOL, err
    vol = ctx.get_array("geometry:cell_vol", case.mesh.n_cells)
    assert np.array_equal(djds, lam * vol)


def test_vjp_matches_central_differences(semo, adj_case):
    case, s, zc = adj_case
    ctx = semo.Context(precision="fp64", tol=SOLVE_TOL, max_iter=1000)
    ctx.set_case(case)
    x = forward(ctx, s)
    g = np.zeros(case.mesh.n_cells)
    g[zc] = 2.0 * x[zc]
    _, djds, _ = ctx.vjp_source(g)
    fd, ad = [], []
    for seed in range(100, 116):
        d = np.random.default_rng(seed).standard_normal(case.mesh.n_cells)
        jp = objective(forward(ctx, s + H * d), zc)
        jm = objective(forward(ctx, s - H * d), zc)
        fd.append((jp - jm) / (2.0 * H))
        ad.append(float(djds @ d))
    fd, ad = np.array(fd), np.array(ad)
    err = np.linalg.norm(ad - fd) / np.linalg.norm(fd)
    assert err < FD_TOL, (err, ad, fd)
