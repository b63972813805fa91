"""Multicolour Gauss-Seidel smoothing of the pressure AMG (semo_params.smoother = 1).

The smoother of AMGCL's relaxation/gauss_seidel.hpp family made parallel by
colouring: the rows of the finest level (above 16,384 rows) are coloured by
synchronous Jones-Plassmann rounds (hashed priorities), a forward sweep
(colours ascending) smooths before the coarse correction and a backward
sweep after it, so the V-cycle stays symmetric for CG; the coarser levels
keep Chebyshev.  The oracle restates the same colouring, sweeps and rule.

Bars: solutions within 1e-7 relative L2 of AMGCL's (the reference's own
fixtures) and of the oracle's FP64 solve; the FP64 GPU iteration count
within one of the oracle's Gauss-Seidel count; bitwise reproducible.
"""
import numpy as np
import pytest

from golden_io import load, names

pytestmark = pytest.mark.gpu

SOL_TOL = 1e-7


@pytest.fixture(scope="module")
def semo():
    import semo_mesh_gb300 as S
    S.load_library()
    return S


@pytest.mark.parametrize("gname", names())
def test_gs_option_small_systems(semo, gname):
    """Systems below the Gauss-Seidel size keep Chebyshev under the option."""
    _, ref = load(gname)
    ctx = semo.Context(precision="fp64", tol=1e-10, smoother="gauss_seidel")
    res = ctx.solve_amgcl("pressure", 1, ref["A_rows"], ref["A_cols"], ref["A_vals"], ref["B"])
    assert res.info["rel_residual"] <= 1e-10
    assert np.linalg.norm(res.x - ref["x"]) / np.linalg.norm(ref["x"]) < SOL_TOL
    ctx.close()


@pytest.fixture(scope="module")
def vof32():
    from semo_mesh_gb300.cases import vof_case
    from oracle.oracle import Oracle
    case = vof_case(32)
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble()
    ref = o.solve(False, 1e-12)
    gs8 = o.solve(False, 1e-8, smoother="gauss_seidel")
    return case, ref, gs8


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gs_solve_vs_oracle(semo, vof32, precision):
    case, ref, gs8 = vof32
    ctx = semo.Context(precision=precision, tol=1e-8, smoother="gauss_seidel")
    ctx.set_case(case)
    ctx.assemble()
    res = ctx.solve()
    assert res.info["rel_residual"] <= 1e-8
    err = np.linalg.norm(res.x - ref["x"]) / np.linalg.norm(ref["x"])
    assert err < SOL_TOL, err
    print(f"Gauss-Seidel {precision}: GPU {res.info['iterations']} iterations, oracle {gs8['iters']}")
    if precision == "fp64":
        assert abs(res.info["iterations"] - gs8["iters"]) <= 1, (res.info["iterations"], gs8["iters"])
    ctx.close()


def test_gs_deterministic_and_outer_iteration(semo):
    from semo_mesh_gb300.cases import vof_case, with_history
    case = with_history(vof_case(28), seed=9)
    out = []
    for _ in range(2):
        ctx = semo.Context(precision="mixed", tol=1e-8, smoother="gauss_seidel")
        ctx.set_case(case)
        norms, info = ctx.outer_iteration()
        assert info[3]["rel_residual"] <= 1e-8
        out.append((norms, info[3]["iterations"], ctx.fields()))
        ctx.close()
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    for k in ("P", "U", "V", "W"):
        assert np.array_equal(out[0][2][k], out[1][2][k])


def test_bad_smoother_refused(semo):
    with pytest.raises(semo.SemoError):
        semo.Context(smoother="jacobi")
