"""The benchmark configurations at full size where the oracle finishes in seconds.

Config 0 as written: the plain method on an unjittered 32^3 hex box
(32,768 cells), U, V, W uniform[-1, 1], density 1, viscosity 1e-3, p = 0,
dt = 1, p fixed on zmax; the pressure-correction Laplacian with the
discrete divergence as right-hand side, AMG-preconditioned CG to 1e-8.
Config 2's coupled 5x5 ideal-gas system on the largest tetrahedral case
the oracle assembles and solves in seconds (6 x 32^3 = 196,608 cells).

Bars: CSR pattern and RCM permutation bit-exact; coefficients and
right-hand sides within 1e-12 relative (max norm); solutions within 1e-7
relative L2 of the oracle's FP64 solve, at the FP64 relative residual asked
for, with the iteration counts of both sides printed.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COEF_TOL = 1e-12
SOL_TOL = 1e-7


def relmax(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.abs(b).max() if b.size else 0.0
    return float(np.abs(a - b).max() / (s if s > 0 else 1.0)) if a.size else 0.0


@pytest.fixture(scope="module")
def semo():
    import semo_mesh_gb300 as S
    S.load_library()
    return S


@pytest.fixture(scope="module")
def config0():
    from semo_mesh_gb300.cases import box_case
    from oracle.oracle import Oracle
    case = box_case(32)
    assert case.mesh.n_cells == 32768 and case.mesh.n_faces == 101376
    assert case.rho == (1.0, 1.0) and case.dt == 1.0 and not case.use_gravity
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble()
    return case, o


def test_config0_system(semo, config0):
    case, o = config0
    ctx = semo.Context(precision="fp64", tol=1e-8)
    ctx.set_case(case)
    ctx.assemble()
    sysm = ctx.system_rcm()
    assert np.array_equal(sysm["ptr"], o.get("rcm_csr_ptr"))
    assert np.array_equal(sysm["col"], o.get("rcm_csr_col"))
    assert relmax(sysm["val"], o.get("rcm_csr_val")) < COEF_TOL
    assert relmax(sysm["b"], o.get("rcm_B")) < COEF_TOL
    perm, iperm = ctx.lib_rcm()
    assert np.array_equal(perm, o.get("rcm_perm"))
    ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_config0_solve(semo, config0, precision):
    case, o = config0
    ctx = semo.Context(precision=precision, tol=1e-8)
    ctx.set_case(case)
    ctx.assemble()
    res = ctx.solve()
    ref = o.solve(False, 1e-12)
    ref8 = o.solve(False, 1e-8)
    err = np.linalg.norm(res.x - ref["x"]) / np.linalg.norm(ref["x"])
    print(f"config 0 {precision}: GPU {res.info['iterations']} iterations (rel. residual "
          f"{res.info['rel_residual']:.2e}), oracle {ref8['iters']} at 1e-8; solution rel L2 {err:.2e}")
    assert res.info["rel_residual"] <= 1e-8
    assert err < SOL_TOL, err
    ctx.close()


def test_config0_pressure_pass(semo, config0):
    """The whole calcPressureEq (solve, Gauss-Green, update) on config 0."""
    from semo_mesh_gb300.cases import box_case
    from oracle.oracle import Oracle
    case = box_case(32)
    o = Oracle(case.mesh)
    sol = o.pressure_pass(case, 1e-12)
    ctx = semo.Context(precision="mixed", tol=1e-10)
    ctx.set_case(case)
    norm, info = ctx.calc_pressure_eq()
    f = ctx.fields()
    for k in ("P", "U", "V", "W"):
        ref = o.get(k)
        assert np.linalg.norm(f[k] - ref) <= SOL_TOL * np.linalg.norm(ref), k
    assert abs(norm - sol["norm"]) <= 1e-6 * abs(sol["norm"])
    ctx.close()


@pytest.fixture(scope="module")
def config2():
    from semo_mesh_gb300.cases import coupled_case
    from oracle.oracle import Oracle
    case = coupled_case(32)
    o = Oracle(case.mesh)
    o.set_coupled(case)
    o.assemble_coupled()
    return case, o


def test_config2_system(semo, config2):
    case, o = config2
    ctx = semo.Context(precision="fp64", tol=1e-8)
    ctx.set_coupled_case(case)
    ctx.assemble_coupled()
    sysm = ctx.coupled_system()
    ptr, col, val = o.coupled_bsr()
    assert np.array_equal(sysm["ptr"], ptr)
    assert np.array_equal(sysm["col"], col)
    scale = np.abs(val).max(axis=0)
    scale[scale == 0] = 1.0
    err = (np.abs(sysm["val"] - val) / scale).max()
    assert err < COEF_TOL, err
    B = o.get("cpl_B").reshape(5, -1)
    for a in range(5):
        assert np.abs(sysm["b"][a] - B[a]).max() <= COEF_TOL * np.abs(B[a]).max(), a
    ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_config2_solve(semo, config2, precision):
    case, o = config2
    ref = o.solve_coupled(1e-13, 5000)
    ctx = semo.Context(precision=precision, tol=1e-8, max_iter=3000)
    ctx.set_coupled_case(case)
    ctx.assemble_coupled()
    res = ctx.solve_coupled()
    err = np.linalg.norm(res.x - ref["x"]) / np.linalg.norm(ref["x"])
    print(f"config 2 (6 x 32^3 tets) {precision}: GPU {res.info['iterations']} iterations (rel. residual "
          f"{res.info['rel_residual']:.2e}), oracle block-Jacobi BiCGStab {ref['iters']} to 1e-13; "
          f"solution rel L2 {err:.2e}")
    assert res.info["rel_residual"] <= 1e-8
    assert err < SOL_TOL, err
    ctx.close()
