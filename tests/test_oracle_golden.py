"""The CPU checker against the reference's own outputs (golden fixtures).

Every intermediate of one pressure-correction pass must be bit-identical to
what the reference's compiled code produced on the same inputs.
"""
import numpy as np
import pytest

from golden_io import load, names
from oracle.oracle import Oracle

EXACT = ["face_area", "face_n", "face_c", "face_wC", "face_magPN", "face_alphaF", "face_ePN",
         "face_skew", "face_vecPF", "face_vecNF", "face_dist", "cell_vol", "cell_c", "lsq_minv",
         "stencil_ptr", "stencil_idx", "rho", "src_grav", "max_vf", "min_vf", "face_rhoL", "face_rhoR",
         "face_pL", "face_pR", "face_uL", "face_uR", "CRS_ptr", "CRS_col", "CRS_dig", "CRS_LR", "CRS_RL",
         "grad_P", "grad_U", "grad_V", "grad_W", "grad_VF", "minmax_uvw", "A_rows", "A_cols", "A_vals",
         "B", "rcm_perm", "rcm_iperm"]


@pytest.fixture(scope="module", params=names())
def golden(request):
    case, ref = load(request.param)
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble()
    return case, ref, o


@pytest.mark.parametrize("key", EXACT)
def test_bit_exact(golden, key):
    case, ref, o = golden
    got = o.get(key)
    assert got.shape == ref[key].shape
    assert np.array_equal(got, ref[key]), f"{case.name}:{key} differs"


def test_update_from_reference_solution(golden):
    case, ref, _ = golden
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble()
    norm = o.update(ref["x"])
    for k in ("P", "U", "V", "W"):
        assert np.array_equal(o.get(k), ref[k + "_new"])
    assert norm == ref["norm"][0]


def test_solution_matches_reference_amgcl(golden):
    case, ref, o = golden
    s = o.solve(False, 1e-10)
    assert s["rel_res"] <= 1e-10
    err = np.linalg.norm(s["x"] - ref["x"]) / np.linalg.norm(ref["x"])
    assert err < 1e-7, err
