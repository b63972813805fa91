"""GPU compressible coupled 5x5 system (through the C-ABI) against the oracle.

The reference's calcCompCoupledEq is commented out, so the oracle's
restatement of its last live state is the only thing to compare with (see
tests/test_oracle_coupled.py for what pins the oracle).  Bars: the block
pattern bit-exact; every block entry and the right-hand side within 1e-12
of the oracle, relative to the largest magnitude of that entry over the
mesh (the entries mix pressure, velocity and temperature units); the
solution within 1e-7 relative L2 of the oracle's FP64 solve; the update and
its norm within 1e-9.
"""
import numpy as np
import pytest

from semo_mesh_gb300.cases import coupled_case

pytestmark = pytest.mark.gpu

COEF_TOL = 1e-12
SOL_TOL = 1e-7


@pytest.fixture(scope="module")
def semo():
    import semo_mesh_gb300 as S
    S.load_library()
    return S


def build(case):
    from oracle.oracle import Oracle
    o = Oracle(case.mesh)
    o.set_coupled(case)
    o.assemble_coupled()
    return o


CASES = {
    "tet5": lambda: coupled_case(5),
    "hex6j": lambda: coupled_case(6, tets=False),
    "tet4_fixed": lambda: _fixed(coupled_case(4)),
}


def _fixed(case):
    """Exercises the other boundary branches: fixed p and T on zmax, slip on xmin, fixed U on ymax, gravity."""
    names = case.mesh.patch_names
    case.bc_type[names.index("zmax")] = (1, 0, 1)
    case.bc_value[names.index("zmax")] = (1.01e5, 0.0, 0.0, 0.0, 305.0)
    case.bc_type[names.index("xmin"), 1] = 3
    case.bc_type[names.index("ymax"), 1] = 1
    case.bc_value[names.index("ymax")] = (0.0, 5.0, -3.0, 1.0, 0.0)
    case.gravity = (0.0, 0.0, -9.81)
    return case


@pytest.mark.parametrize("name", sorted(CASES))
def test_coupled_system_matches_oracle(semo, name):
    case = CASES[name]()
    o = build(case)
    ctx = semo.Context(precision="fp64", tol=1e-10)
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
def test_coupled_solution(semo, precision):
    case = coupled_case(5)
    o = build(case)
    ref = o.solve_coupled(1e-13, 3000)
    ctx = semo.Context(precision=precision, tol=1e-10)
    ctx.set_coupled_case(case)
    ctx.assemble_coupled()
    res = ctx.solve_coupled()
    assert res.info["rel_residual"] <= 1e-10
    assert np.linalg.norm(res.x - ref["x"]) <= SOL_TOL * np.linalg.norm(ref["x"])
    ctx.close()


def test_coupled_pass_update_and_norm(semo):
    case = coupled_case(5)
    case.urf = 0.7
    o = build(case)
    ctx = semo.Context(precision="mixed", tol=1e-11)
    ctx.set_coupled_case(case)
    norm, info = ctx.calc_comp_coupled_eq()
    ref = o.solve_coupled(1e-13, 3000)
    onorm = o.update_coupled(ref["x"], case.limits)
    f = ctx.coupled_fields()
    for k in ("P", "U", "V", "W", "T"):
        np.testing.assert_allclose(f[k], o.get("cpl_" + k), rtol=1e-9, atol=1e-9 * np.abs(o.get("cpl_" + k)).max())
    assert abs(norm - onorm) <= 1e-7 * onorm
    ctx.close()


def test_coupled_deterministic(semo):
    case = coupled_case(4)
    outs = []
    for _ in range(2):
        ctx = semo.Context(precision="mixed", tol=1e-9)
        ctx.set_coupled_case(case)
        ctx.assemble_coupled()
        sysm = ctx.coupled_system()
        res = ctx.solve_coupled()
        outs.append((sysm["val"], sysm["b"], res.x))
        ctx.close()
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)


def test_coupled_state_errors(semo):
    case = coupled_case(3)
    ctx = semo.Context(precision="mixed")
    ctx.upload_mesh(case.mesh)
    with pytest.raises(semo.SemoError) as e:
        ctx.assemble_coupled()
    assert e.value.status == 8
    ctx.set_coupled_case(case)
    with pytest.raises(semo.SemoError) as e:
        ctx.solve_coupled()
    assert e.value.status == 8
    ctx.close()
