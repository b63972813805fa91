"""The oracle's momentum equation and whole outer iteration against the reference.

The outer_* fixtures hold the reference's own outputs for one outer iteration
of src/solvers/pressureBased.cpp:200-213: calcMomentumEqs (transport, face
values, gradients, BDF2 + convection + diffusion assembly, the 3-RHS AMGCL
solve, update) followed by calcPressureEq on the updated velocity.  The
oracle's restatement must reproduce every assembled array bit for bit.
"""
import numpy as np
import pytest

from golden_io import load, outer_names

OUTER = outer_names()


@pytest.fixture(scope="module", params=OUTER)
def outer(request):
    from oracle.oracle import Oracle
    case, ref = load(request.param)
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble_momentum()
    return request.param, case, ref, o


def test_fixtures_present():
    assert len(OUTER) >= 2


def test_viscosity_and_pressure_limits(outer):
    _, _, ref, o = outer
    assert np.array_equal(o.get("mu"), ref["mu"])
    assert np.array_equal(o.get("mom_minmax_p"), ref["mom_minmax_p"])


@pytest.mark.parametrize("field", ["P", "U", "V", "W", "VF"])
def test_gradients_bit_exact(outer, field):
    _, _, ref, o = outer
    assert np.array_equal(o.get("mom_grad_" + field), ref["mom_grad_" + field])


def test_coo_bit_exact(outer):
    _, _, ref, o = outer
    for k in ("rows", "cols", "vals"):
        assert np.array_equal(o.get("mom_A_" + k), ref["mom_A_" + k]), k


def test_rhs_bit_exact(outer):
    _, case, ref, o = outer
    B = o.get("mom_B").reshape(3, case.mesh.n_cells)
    for j in range(3):
        assert np.array_equal(B[j], ref[f"mom_B{j}"]), j


def test_csr_is_coo_scatter(outer):
    """CSR rows keep COO order (solveAMGCL.cpp:1129-1172): diagonal first."""
    _, case, ref, o = outer
    ptr, col, val = o.get("mom_csr_ptr"), o.get("mom_csr_col"), o.get("mom_csr_val")
    n = case.mesh.n_cells
    assert ptr[-1] == ref["mom_A_vals"].size
    assert np.array_equal(col[ptr[:-1]], np.arange(n))
    rows = np.repeat(np.arange(n), np.diff(ptr))
    dense = {(int(r), int(c)): v for r, c, v in zip(rows, col, val)}
    for r, c, v in zip(ref["mom_A_rows"], ref["mom_A_cols"], ref["mom_A_vals"]):
        assert dense[(int(r), int(c))] == v


def test_solution_matches_reference(outer):
    _, _, ref, o = outer
    sol = o.solve_momentum(1e-12, 2000)
    for j in range(3):
        x, xr = sol["x"][j], ref[f"mom_x{j}"]
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-7, j


def test_update_and_following_pressure_pass(outer):
    name, case, ref, o = outer
    norm = o.update_momentum([ref[f"mom_x{j}"] for j in range(3)])
    assert norm == ref["mom_norm"][0]
    for c in "UVW":
        assert np.array_equal(o.get(c), ref[f"mom_{c}_new"]), c
    o.assemble()
    assert np.array_equal(o.get("A_vals"), ref["A_vals"])
    assert np.array_equal(o.get("B"), ref["B"])
