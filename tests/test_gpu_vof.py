"""GPU volume-fraction sub-iteration (through the C-ABI) against the reference.

The vofeq_* fixtures hold the reference's own outputs for one sub-iteration
(MSTACS reconstruction + calcVolfracEq + AMGCL solve + VF update).  Bars:
the CSR pattern (with the upwind drops) bit-exact; MSTACS face values,
coefficients and right-hand side within 1e-12 relative; the solution within
1e-7 relative L2 of AMGCL's.  Larger cases compare with the CPU oracle, pinned
bit-exactly to the fixtures.
"""
import numpy as np
import pytest

from golden_io import load, vofeq_names

pytestmark = pytest.mark.gpu

COEF_TOL = 1e-12
SOL_TOL = 1e-7
VOFEQ = vofeq_names()


def relmax(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.abs(b).max() if b.size else 0.0
    return float(np.abs(a - b).max() / (s if s > 0 else 1.0)) if a.size else 0.0


def coo_to_csr(rows, cols, vals, n):
    """solveAMGCL's COO -> CSR (solveAMGCL.cpp:206-251): stable scatter, rows keep COO order."""
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


@pytest.mark.parametrize("gname", VOFEQ)
def test_vof_system_matches_reference(semo, gname):
    case, ref = load(gname)
    n, nf = case.mesh.n_cells, case.mesh.n_faces
    ctx = make_ctx(semo, case)
    ctx.assemble_vof()
    lr = ctx.get_array("face_VF_LR", 2 * nf).reshape(nf, 2)
    assert relmax(lr[:, 0], ref["vof_face_vfL"]) < COEF_TOL
    assert relmax(lr[:, 1], ref["vof_face_vfR"]) < COEF_TOL
    sysm = ctx.vof_system()
    ptr, col, val = coo_to_csr(ref["vof_A_rows"], ref["vof_A_cols"], ref["vof_A_vals"], n)
    assert np.array_equal(sysm["ptr"], ptr)
    assert np.array_equal(sysm["col"], col)
    assert relmax(sysm["val"], val) < COEF_TOL
    assert relmax(sysm["b"], ref["vof_B"]) < COEF_TOL
    assert relmax(ctx.get_array("grad_VF", 3 * n), ref["vof_grad_VF"]) < COEF_TOL


@pytest.mark.parametrize("gname", VOFEQ)
def test_vof_solution_and_update(semo, gname):
    case, ref = load(gname)
    ctx = make_ctx(semo, case)
    ctx.assemble_vof()
    res = ctx.solve_vof()
    assert res.info["rel_residual"] <= 1e-11
    assert np.linalg.norm(res.x - ref["vof_x"]) / np.linalg.norm(ref["vof_x"]) < SOL_TOL
    ctx2 = make_ctx(semo, case)
    norm, info = ctx2.calc_volfrac_eq()
    assert abs(norm - ref["vof_norm"][0]) <= 1e-7 * ref["vof_norm"][0]
    vf = ctx2.get_array("VF", case.mesh.n_cells)
    assert np.abs(vf - ref["vof_VF_new"]).max() < 1e-9
    f = ctx2.fields()
    for k in ("P", "U", "V", "W"):
        assert np.array_equal(f[k], getattr(case, k)), k


@pytest.fixture(scope="module")
def vof24():
    from semo_mesh_gb300.cases import vof_case, with_fields, with_vf_history
    from oracle.oracle import Oracle
    case = with_vf_history(with_fields(vof_case(24), seed=31, p_scale=200.0), seed=32)
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble_vof()
    return case, o


def test_vof24_vs_oracle(semo, vof24):
    case, o = vof24
    n, nf = case.mesh.n_cells, case.mesh.n_faces
    ctx = make_ctx(semo, case)
    ctx.assemble_vof()
    lr = ctx.get_array("face_VF_LR", 2 * nf).reshape(nf, 2)
    assert relmax(lr[:, 0], o.get("vof_face_vfL")) < COEF_TOL
    assert relmax(lr[:, 1], o.get("vof_face_vfR")) < COEF_TOL
    sysm = ctx.vof_system()
    assert np.array_equal(sysm["ptr"], o.get("vof_csr_ptr"))
    assert np.array_equal(sysm["col"], o.get("vof_csr_col"))
    assert relmax(sysm["val"], o.get("vof_csr_val")) < COEF_TOL
    assert relmax(sysm["b"], o.get("vof_B")) < COEF_TOL
    res = ctx.solve_vof()
    ref = o.solve_vof(1e-13)
    assert np.linalg.norm(res.x - ref["x"]) / np.linalg.norm(ref["x"]) < SOL_TOL


def test_vof_deterministic(semo):
    from semo_mesh_gb300.cases import vof_case, with_vf_history
    case = with_vf_history(vof_case(16), seed=3)
    outs = []
    for _ in range(2):
        ctx = make_ctx(semo, case, "mixed")
        norm, _ = ctx.calc_volfrac_eq()
        ctx.assemble_vof()
        outs.append((norm, ctx.vof_system()["b"]))
    assert outs[0][0] == outs[1][0]
    assert np.array_equal(outs[0][1], outs[1][1])
