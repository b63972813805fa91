"""Error statuses for bad host inputs, through the C-ABI.

Every failure here is made on the host (a NaN in a caller array, a face
whose neighbour is its owner, a mirrored mesh whose cells have negative
volume, a negative-definite matrix); the library must turn each into its
status code and leave the context usable.  Nothing here faults the GPU.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def semo():
    import semo_mesh_gb300 as S
    S.load_library()
    return S


def test_nan_in_host_fields(semo):
    from semo_mesh_gb300.cases import vof_case
    case = vof_case(6)
    ctx = semo.Context()
    ctx.set_case(case)
    U = case.U.copy()
    U[17] = np.nan
    with pytest.raises(semo.SemoError) as e:
        ctx.set_fields(case.P, U, case.V, case.W, case.VF)
    assert e.value.status == 6   # SEMO_ERR_NAN
    VF = case.VF.copy()
    VF[3] = np.inf
    with pytest.raises(semo.SemoError) as e:
        ctx.set_fields(case.P, case.U, case.V, case.W, VF)
    assert e.value.status == 6
    # the context still works with good fields
    ctx.set_fields(case.P, case.U, case.V, case.W, case.VF)
    norm, info = ctx.calc_pressure_eq()
    assert np.isfinite(norm) and info["rel_residual"] <= 1e-8
    ctx.close()


def test_nan_in_old_velocity_and_coo(semo):
    from semo_mesh_gb300.cases import vof_case
    case = vof_case(5)
    ctx = semo.Context()
    ctx.set_case(case)
    old = [case.U.copy(), case.V.copy(), case.W.copy()]
    old[1][2] = np.nan
    with pytest.raises(semo.SemoError) as e:
        ctx.set_old_velocity(old, old)
    assert e.value.status == 6
    n = 8
    rows = np.arange(n, dtype=np.int32)
    vals = np.ones(n)
    vals[4] = np.nan
    with pytest.raises(semo.SemoError) as e:
        ctx.solve_amgcl("pressure", 1, rows, rows, vals, np.ones(n))
    assert e.value.status == 6
    ctx.close()


def test_neighbour_equals_owner(semo):
    from semo_mesh_gb300.meshgen import hex_box
    m = hex_box(3)
    m.neighbour = m.neighbour.copy()
    m.neighbour[4] = m.owner[4]
    ctx = semo.Context()
    with pytest.raises(semo.SemoError) as e:
        ctx.upload_mesh(m)
    assert e.value.status == 2   # SEMO_ERR_MESH
    assert "neighbour == owner" in str(e.value)
    ctx.close()


def test_non_positive_volume(semo):
    """A mirrored mesh keeps its face lists, so every face normal points into
    its owner and every cell volume comes out negative."""
    from semo_mesh_gb300.meshgen import hex_box
    m = hex_box(3)
    m.points = m.points.copy()
    m.points[:, 0] *= -1.0
    ctx = semo.Context()
    with pytest.raises(semo.SemoError) as e:
        ctx.upload_mesh(m)
    assert e.value.status == 2
    assert "volume" in str(e.value)
    # the same context takes a good mesh afterwards
    ctx.upload_mesh(hex_box(3))
    ctx.close()


@pytest.mark.parametrize("n", [40, 3000])
def test_breakdown_on_negative_definite(semo, n):
    """CG on -L (L the 1-D Laplacian): p.Ap < 0 at the first iteration, which
    the device check reports as SEMO_ERR_BREAKDOWN (the loop stops there)."""
    rows, cols, vals = [], [], []
    for i in range(n):
        rows.append(i); cols.append(i); vals.append(-2.0)
    for i in range(n):
        for j in (i - 1, i + 1):
            if 0 <= j < n:
                rows.append(i); cols.append(j); vals.append(1.0)
    ctx = semo.Context(precision="fp64", tol=1e-10)
    with pytest.raises(semo.SemoError) as e:
        ctx.solve_amgcl("pressure", 1, np.array(rows, np.int32), np.array(cols, np.int32), np.array(vals),
                        np.ones(n))
    assert e.value.status == 7   # SEMO_ERR_BREAKDOWN
    ctx.close()
