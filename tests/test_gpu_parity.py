"""GPU path (through the C-ABI) against the reference's own outputs.

Golden fixtures come from the reference's compiled code (tests/golden/);
larger cases compare against the CPU oracle, which is pinned bit-exactly to
those fixtures by tests/test_oracle_golden.py.

Tolerances: geometry, RCM and the CSR pattern are bit-exact; assembled FP64
coefficients and gradients agree within 1e-12 relative (the face kernel
reassociates the Rhie-Chow terms and uses FMA); solutions converge to the FP64
relative residual asked for and agree with the reference's solution within
1e-7 relative L2.
"""
import numpy as np
import pytest

from golden_io import load, names

pytestmark = pytest.mark.gpu

GEOM = ["face_area", "face_n", "face_c", "face_wC", "face_magPN", "face_alphaF", "face_ePN", "face_skew",
        "face_vecPF", "face_vecNF", "cell_vol", "cell_c", "lsq_minv"]
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


def make_ctx(semo, case, precision="fp64", tol=1e-10):
    ctx = semo.Context(precision=precision, tol=tol)
    ctx.set_case(case)
    return ctx


def cell_count(name, case):
    n, f = case.mesh.n_cells, case.mesh.n_faces
    return {"face_area": f, "face_n": 3 * f, "face_c": 3 * f, "face_wC": f, "face_magPN": f, "face_alphaF": f,
            "face_ePN": 3 * f, "face_skew": 3 * f, "face_vecPF": 3 * f, "face_vecNF": 3 * f, "cell_vol": n,
            "cell_c": 3 * n, "lsq_minv": 6 * n}[name]


@pytest.mark.parametrize("gname", names())
def test_geometry_bit_exact(semo, gname):
    case, ref = load(gname)
    ctx = make_ctx(semo, case)
    for k in GEOM:
        got = ctx.get_array("geometry:" + k, cell_count(k, case))
        assert np.array_equal(got, ref[k]), f"{gname}:{k} max rel {relmax(got, ref[k])}"


@pytest.mark.parametrize("gname", names())
def test_rcm_bit_exact(semo, gname):
    case, ref = load(gname)
    ctx = make_ctx(semo, case)
    perm, iperm = ctx.lib_rcm()
    assert np.array_equal(perm, ref["rcm_perm"])
    assert np.array_equal(iperm, ref["rcm_iperm"])


def reference_csr_rcm(case, ref):
    """The reference's COO system -> CSR (solveAMGCL order) -> RCM permutation."""
    from oracle.oracle import Oracle
    o = Oracle(case.mesh)
    o.set_case(case)
    o.set("A_rows", ref["A_rows"]); o.set("A_cols", ref["A_cols"])
    o.set("A_vals", ref["A_vals"]); o.set("B", ref["B"])
    from oracle.oracle import lib
    lib().orc_coo_to_csr(o.h)
    lib().orc_permute_csr(o.h)
    return {k: o.get(k) for k in ("rcm_csr_ptr", "rcm_csr_col", "rcm_csr_val", "rcm_B")}


@pytest.mark.parametrize("gname", names())
def test_assembly_matches_reference(semo, gname):
    case, ref = load(gname)
    ctx = make_ctx(semo, case)
    ctx.assemble()
    sysm = ctx.system_rcm()
    exp = reference_csr_rcm(case, ref)
    assert np.array_equal(sysm["ptr"], exp["rcm_csr_ptr"])
    assert np.array_equal(sysm["col"], exp["rcm_csr_col"])
    assert relmax(sysm["val"], exp["rcm_csr_val"]) < COEF_TOL
    assert relmax(sysm["b"], exp["rcm_B"]) < COEF_TOL
    n = case.mesh.n_cells
    for g in ("grad_P", "grad_U", "grad_V", "grad_W", "grad_VF"):
        got = ctx.get_array(g, 3 * n)
        assert relmax(got, ref[g]) < COEF_TOL, g
    assert np.array_equal(ctx.get_array("minmax_uvw", 6 * n), ref["minmax_uvw"])
    assert relmax(ctx.get_array("rho", n), ref["rho"]) == 0.0
    assert relmax(ctx.get_array("src_grav", 4 * n), ref["src_grav"]) < COEF_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("gname", names())
def test_solution_matches_reference(semo, gname, precision):
    case, ref = load(gname)
    ctx = make_ctx(semo, case, precision=precision, tol=1e-10)
    ctx.assemble()
    res = ctx.solve()
    assert res.info["rel_residual"] <= 1e-10
    err = np.linalg.norm(res.x - ref["x"]) / np.linalg.norm(ref["x"])
    assert err < SOL_TOL, err


@pytest.mark.parametrize("gname", names())
def test_pressure_pass_matches_reference(semo, gname):
    case, ref = load(gname)
    ctx = make_ctx(semo, case, precision="mixed", tol=1e-11)
    norm, info = ctx.calc_pressure_eq()
    f = ctx.fields()
    for k in ("P", "U", "V", "W"):
        assert relmax(f[k], ref[k + "_new"]) < SOL_TOL, k
    assert abs(norm - ref["norm"][0]) <= SOL_TOL * abs(ref["norm"][0])


@pytest.mark.parametrize("gname", names())
def test_solve_amgcl_coo_boundary(semo, gname):
    """The solveAMGCL-shaped entry: SEMO's own COO triple in, solution out."""
    case, ref = load(gname)
    ctx = semo.Context(precision="fp64", tol=1e-10)
    res = ctx.solve_amgcl("pressure", 1, ref["A_rows"], ref["A_cols"], ref["A_vals"], ref["B"])
    err = np.linalg.norm(res.x - ref["x"]) / np.linalg.norm(ref["x"])
    assert err < SOL_TOL


# ---------------------------------------------------------------- larger cases
@pytest.fixture(scope="module")
def vof32():
    from semo_mesh_gb300.cases import vof_case
    from oracle.oracle import Oracle
    case = vof_case(32)
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble()
    return case, o


def test_vof32_assembly_vs_oracle(semo, vof32):
    case, o = vof32
    ctx = make_ctx(semo, case)
    ctx.assemble()
    sysm = ctx.system_rcm()
    assert np.array_equal(sysm["ptr"], o.get("rcm_csr_ptr"))
    assert np.array_equal(sysm["col"], o.get("rcm_csr_col"))
    assert relmax(sysm["val"], o.get("rcm_csr_val")) < COEF_TOL
    assert relmax(sysm["b"], o.get("rcm_B")) < COEF_TOL
    perm, iperm = ctx.lib_rcm()
    assert np.array_equal(perm, o.get("rcm_perm"))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_vof32_solve_vs_oracle(semo, vof32, precision):
    case, o = vof32
    ctx = make_ctx(semo, case, precision=precision, tol=1e-8)
    ctx.assemble()
    res = ctx.solve()
    assert res.info["rel_residual"] <= 1e-8
    ref = o.solve(False, 1e-12)
    err = np.linalg.norm(res.x - ref["x"]) / np.linalg.norm(ref["x"])
    assert err < SOL_TOL, err


def test_deterministic(semo):
    from semo_mesh_gb300.cases import vof_case
    case = vof_case(16)
    out = []
    for _ in range(2):
        ctx = make_ctx(semo, case, precision="mixed", tol=1e-8)
        norm, info = ctx.calc_pressure_eq()
        out.append((norm, ctx.fields(), info["iterations"]))
    assert out[0][0] == out[1][0]
    assert out[0][2] == out[1][2]
    for k in ("P", "U", "V", "W"):
        assert np.array_equal(out[0][1][k], out[1][1][k])


def test_not_converged_status(semo):
    from semo_mesh_gb300.cases import vof_case
    case = vof_case(12)
    ctx = semo.Context(precision="fp64", tol=1e-12, max_iter=1)
    ctx.set_case(case)
    ctx.assemble()
    with pytest.raises(semo.SemoError) as e:
        ctx.solve()
    assert e.value.status == 5


def test_bad_mesh_rejected(semo):
    from semo_mesh_gb300.meshgen import hex_box
    m = hex_box(3)
    m.owner = m.owner.copy()
    m.owner[5] = m.n_cells + 7
    ctx = semo.Context()
    with pytest.raises(semo.SemoError) as e:
        ctx.upload_mesh(m)
    assert e.value.status == 2
