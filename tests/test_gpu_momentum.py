"""GPU momentum equation and outer iteration (through the C-ABI) against the reference.

The outer_* fixtures hold the reference's own outputs for one outer iteration
(calcMomentumEqs, then calcPressureEq on the updated velocity).  Bars: the
momentum CSR pattern (rows, in-row order, dropped entries) bit-exact;
coefficients and right-hand sides within 1e-12 relative; cell viscosity and
stencil limits bit-exact; solutions within 1e-7 relative L2 of AMGCL's.
Larger cases compare with the CPU oracle, pinned bit-exactly to the fixtures.
"""
import numpy as np
import pytest

from golden_io import load, outer_names

pytestmark = pytest.mark.gpu

COEF_TOL = 1e-12
SOL_TOL = 1e-7
OUTER = outer_names()


def relmax(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.abs(b).max() if b.size else 0.0
    return float(np.abs(a - b).max() / (s if s > 0 else 1.0)) if a.size else 0.0


def coo_to_csr(rows, cols, vals, n):
    """solveAMGCL's COO -> CSR (solveAMGCL.cpp:1129-1172): stable scatter, rows keep COO order."""
    order = np.argsort(rows, kind="stable")
    ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(ptr, rows + 1, 1)
    return np.cumsum(ptr), cols[order], vals[order]


@pytest.fixture(scope="module")
def semo():
    import semo_mesh_gb300 as S
    S.load_library()
    return S


def make_ctx(semo, case, precision="fp64"):
    ctx = semo.Context(precision=precision, tol=1e-10, mom_tol=1e-11)
    ctx.set_case(case)
    return ctx


@pytest.mark.parametrize("gname", OUTER)
def test_momentum_system_matches_reference(semo, gname):
    case, ref = load(gname)
    n = case.mesh.n_cells
    ctx = make_ctx(semo, case)
    ctx.assemble_momentum()
    sysm = ctx.momentum_system()
    ptr, col, val = coo_to_csr(ref["mom_A_rows"], ref["mom_A_cols"], ref["mom_A_vals"], n)
    assert np.array_equal(sysm["ptr"], ptr)
    assert np.array_equal(sysm["col"], col)
    assert relmax(sysm["val"], val) < COEF_TOL
    for j in range(3):
        assert relmax(sysm["b"][j], ref[f"mom_B{j}"]) < COEF_TOL, j
    assert np.array_equal(ctx.get_array("mu", n), ref["mu"])
    assert np.array_equal(ctx.get_array("minmax_p", 2 * n), ref["mom_minmax_p"])
    for g in ("P", "U", "V", "W", "VF"):
        assert relmax(ctx.get_array("grad_" + g, 3 * n), ref["mom_grad_" + g]) < COEF_TOL, g


@pytest.mark.parametrize("gname", OUTER)
def test_momentum_solution_matches_reference(semo, gname):
    case, ref = load(gname)
    ctx = make_ctx(semo, case)
    ctx.assemble_momentum()
    x, info = ctx.solve_momentum()
    for j in range(3):
        assert info[j]["rel_residual"] <= 1e-11
        xr = ref[f"mom_x{j}"]
        assert np.linalg.norm(x[j] - xr) / np.linalg.norm(xr) < SOL_TOL, j


@pytest.mark.parametrize("gname", OUTER)
def test_outer_iteration_matches_reference(semo, gname):
    case, ref = load(gname)
    ctx = make_ctx(semo, case)
    (nm, npres), info = ctx.outer_iteration()
    assert abs(nm - ref["mom_norm"][0]) <= 1e-7 * abs(ref["mom_norm"][0])
    assert info[3]["rel_residual"] <= 1e-10
    out = ctx.fields()
    for k in ("P", "U", "V", "W"):
        assert relmax(out[k], ref[f"{k}_new"]) < 1e-7, k
    assert abs(npres - ref["norm"][0]) <= 1e-6 * abs(ref["norm"][0])


@pytest.fixture(scope="module")
def vof24():
    from semo_mesh_gb300.cases import vof_case, with_history, with_fields
    from oracle.oracle import Oracle
    case = with_history(with_fields(vof_case(24), seed=21, p_scale=200.0), seed=22)
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble_momentum()
    return case, o


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_vof24_momentum_vs_oracle(semo, vof24, precision):
    case, o = vof24
    n = case.mesh.n_cells
    ctx = make_ctx(semo, case, precision)
    ctx.assemble_momentum()
    sysm = ctx.momentum_system()
    assert np.array_equal(sysm["ptr"], o.get("mom_csr_ptr"))
    assert np.array_equal(sysm["col"], o.get("mom_csr_col"))
    assert relmax(sysm["val"], o.get("mom_csr_val")) < COEF_TOL
    B = o.get("mom_B").reshape(3, n)
    for j in range(3):
        assert relmax(sysm["b"][j], B[j]) < COEF_TOL
    x, info = ctx.solve_momentum()
    ref = o.solve_momentum(1e-12)
    for j in range(3):
        assert np.linalg.norm(x[j] - ref["x"][j]) / np.linalg.norm(ref["x"][j]) < SOL_TOL
        assert info[j]["iterations"] <= 20


def test_momentum_deterministic(semo):
    from semo_mesh_gb300.cases import vof_case, with_history
    case = with_history(vof_case(16), seed=3)
    outs = []
    for _ in range(2):
        ctx = make_ctx(semo, case, "mixed")
        norm, _ = ctx.calc_momentum_eqs()
        outs.append((norm, ctx.fields()))
    assert outs[0][0] == outs[1][0]
    for k in ("U", "V", "W"):
        assert np.array_equal(outs[0][1][k], outs[1][1][k])


def test_old_velocity_arguments(semo):
    """All six history arrays or none (status 1 otherwise)."""
    import ctypes
    from semo_mesh_gb300.cases import vof_case
    case = vof_case(6)
    ctx = make_ctx(semo, case)
    u = np.zeros(case.mesh.n_cells)
    p = u.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert ctx.L.semo_set_old_velocity(ctx.h, p, None, None, None, None, None) == 1
    assert ctx.L.semo_set_old_velocity(ctx.h, None, None, None, None, None, None) == 0


@pytest.mark.parametrize("precision,sigma", [("fp64", 0.0), ("mixed", 0.0), ("mixed", 0.05)])
@pytest.mark.parametrize("reuse", [False, True])
def test_overlapped_setup_is_bit_identical(semo, precision, sigma, reuse):
    """The pressure hierarchy built on the second stream during the momentum
    pass (semo_params.overlap_setup) gives the serial path's results bit for
    bit, over several outer iterations (with and without hierarchy reuse, and
    with a surface tension)."""
    from semo_mesh_gb300.cases import vof_case, with_history, with_fields
    case = with_history(with_fields(vof_case(20, jitter=0.2), seed=31, p_scale=50.0), seed=32)
    case.sigma = sigma
    runs = []
    for overlap in (True, False):
        ctx = semo.Context(precision=precision, tol=1e-8, reuse_hierarchy=reuse, overlap_setup=overlap)
        ctx.set_case(case)
        norms, iters = [], []
        for _ in range(3):
            nm, info = ctx.outer_iteration()
            norms.append(nm)
            iters.append(info[3]["iterations"])
        runs.append((norms, iters, ctx.fields(), ctx.system_rcm()))
    (n1, i1, f1, s1), (n2, i2, f2, s2) = runs
    assert n1 == n2 and i1 == i2
    for k in ("P", "U", "V", "W"):
        assert np.array_equal(f1[k], f2[k]), k
    assert np.array_equal(s1["val"], s2["val"]) and np.array_equal(s1["b"], s2["b"])


def test_overlapped_setup_with_profiling(semo):
    """Stage timers recorded from both host threads (setup on the second stream)."""
    from semo_mesh_gb300.cases import vof_case, with_history
    case = with_history(vof_case(16), seed=33)
    ctx = semo.Context(precision="mixed", reuse_hierarchy=False)
    ctx.set_case(case)
    ctx.set_profiling(True)
    for _ in range(2):
        ctx.outer_iteration()
    st = ctx.stage_times()
    assert st["amg_setup"][1] == 2 and st["amg_setup"][0] > 0.0
    assert st["setup_galerkin"][1] > 0 and st["mface"][1] == 2
