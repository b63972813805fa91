"""solveAMGCL's other live call forms through the C-ABI (semo_solve_coo_multi).

The momentum overload with three right-hand sides (calcMomentumEqs,
src/solvers/eqMomentum.cpp:1017) and the volume-fraction form with one
(calcVolfracEq, src/solvers/eqVolfrac.cpp:766), fed the reference's own COO
systems from the golden fixtures; solutions within 1e-7 relative L2 of
AMGCL's.  An initial guess is honoured (the correction is solved), and a row
without a diagonal entry is refused.
"""
import numpy as np
import pytest

from golden_io import load, outer_names, vofeq_names

pytestmark = pytest.mark.gpu

SOL_TOL = 1e-7


@pytest.fixture(scope="module")
def semo():
    import semo_mesh_gb300 as S
    S.load_library()
    return S


@pytest.mark.parametrize("gname", outer_names())
def test_momentum_overload(semo, gname):
    _, ref = load(gname)
    ctx = semo.Context(precision="fp64", mom_tol=1e-11)
    res = ctx.solve_amgcl("momentum", 1, ref["mom_A_rows"], ref["mom_A_cols"], ref["mom_A_vals"],
                          ref["mom_B0"], ref["mom_B1"], ref["mom_B2"])
    for j in range(3):
        assert res[j].info["rel_residual"] <= 1e-11
        xr = ref[f"mom_x{j}"]
        assert np.linalg.norm(res[j].x - xr) / np.linalg.norm(xr) < SOL_TOL, j
    # from a guess (AMGCL's solution, perturbed): the same solutions
    rng = np.random.default_rng(3)
    guess = [ref[f"mom_x{j}"] * (1.0 + 0.01 * rng.standard_normal(len(ref["mom_x0"]))) for j in range(3)]
    res2 = ctx.solve_amgcl("momentum", 1, ref["mom_A_rows"], ref["mom_A_cols"], ref["mom_A_vals"],
                           ref["mom_B0"], ref["mom_B1"], ref["mom_B2"], *guess)
    for j in range(3):
        xr = ref[f"mom_x{j}"]
        assert np.linalg.norm(res2[j].x - xr) / np.linalg.norm(xr) < SOL_TOL, j
    ctx.close()


@pytest.mark.parametrize("gname", vofeq_names())
def test_volume_fraction_form(semo, gname):
    _, ref = load(gname)
    ctx = semo.Context(precision="fp64", mom_tol=1e-11)
    res = ctx.solve_amgcl("volume_fraction", 1, ref["vof_A_rows"], ref["vof_A_cols"], ref["vof_A_vals"],
                          ref["vof_B"])
    assert res.info["rel_residual"] <= 1e-11
    xr = ref["vof_x"]
    assert np.linalg.norm(res.x - xr) <= SOL_TOL * max(np.linalg.norm(xr), 1e-300)
    ctx.close()


def test_missing_diagonal_refused(semo):
    n = 6
    rows = np.array([0, 1, 2, 3, 4, 5, 0], np.int32)
    cols = np.array([0, 1, 2, 3, 5, 5, 1], np.int32)   # row 4 has no diagonal entry
    vals = np.ones(7)
    ctx = semo.Context()
    with pytest.raises(semo.SemoError) as e:
        ctx.solve_amgcl("volume_fraction", 1, rows, cols, vals, np.ones(n))
    assert e.value.status == 1
    assert "diagonal" in str(e.value)
    ctx.close()
