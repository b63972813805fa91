"""The oracle's volume-fraction sub-iteration against the reference.

The vofeq_* fixtures hold the reference's own outputs for one sub-iteration
of the VOF loop of src/solvers/pressureBased.cpp:104-112: the MSTACS face
reconstruction (src/solvers/reconIncom.cpp:345-429, src/solvers/NVD.cpp:
1098-1790) and calcVolfracEq (src/solvers/eqVolfrac.cpp:9-795) with its AMGCL
solve and the VF update.  The oracle's restatement must reproduce every
assembled array bit for bit.
"""
import numpy as np
import pytest

from golden_io import load, vofeq_names

VOFEQ = vofeq_names()


@pytest.fixture(scope="module", params=VOFEQ)
def vofeq(request):
    from oracle.oracle import Oracle
    case, ref = load(request.param)
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble_vof()
    return request.param, case, ref, o


def test_fixtures_present():
    assert len(VOFEQ) >= 2


@pytest.mark.parametrize("name", ["vof_face_vfL", "vof_face_vfR"])
def test_mstacs_face_values_bit_exact(vofeq, name):
    _, _, ref, o = vofeq
    assert np.array_equal(o.get(name), ref[name])


@pytest.mark.parametrize("field", ["P", "U", "V", "W", "VF"])
def test_gradients_bit_exact(vofeq, field):
    _, _, ref, o = vofeq
    assert np.array_equal(o.get("vof_grad_" + field), ref["vof_grad_" + field])


def test_system_bit_exact(vofeq):
    _, _, ref, o = vofeq
    for k in ("vof_A_rows", "vof_A_cols", "vof_A_vals", "vof_B"):
        assert np.array_equal(o.get(k), ref[k]), k


def test_upwind_drops_one_entry_per_face(vofeq):
    """First-order upwind keeps one off-diagonal per internal face (the other is exactly 0)."""
    _, case, ref, o = vofeq
    assert ref["vof_A_vals"].size <= case.mesh.n_cells + case.mesh.n_internal


def test_solution_and_update(vofeq):
    _, _, ref, o = vofeq
    sol = o.solve_vof(1e-13, 1000)
    xr = ref["vof_x"]
    assert np.linalg.norm(sol["x"] - xr) / np.linalg.norm(xr) < 1e-7
    norm = o.update_vof(xr)
    assert norm == ref["vof_norm"][0]
    assert np.array_equal(o.get("VF"), ref["vof_VF_new"])
