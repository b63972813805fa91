"""Every assembled system in RCM order through the C-ABI (semo_get_system_rcm_eq).

The pressure, momentum (three right-hand sides), volume-fraction and coupled
5x5 systems come out on the mesh's RCM-ordered CSR pattern.  Permuted back to
the caller's numbering (RCM row r is caller cell perm[r]), each must equal the
oracle's assembled system: coefficients and right-hand sides within 1e-12
relative, entries SEMO leaves out of the momentum and volume-fraction
matrices present as exact zeros.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def semo():
    import semo_mesh_gb300 as S
    S.load_library()
    return S


def to_caller(sysm, perm, n, block=False):
    """(rows, cols, vals) in the caller's numbering from an RCM CSR export."""
    ptr, col, val = sysm["ptr"], sysm["col"], sysm["val"]
    rows = np.repeat(np.arange(n), np.diff(ptr))
    return perm[rows], perm[col], val


def dense_from(rows, cols, vals, n, shape=()):
    a = np.zeros((n, n) + shape)
    np.add.at(a, (rows, cols), vals)
    return a


def test_pressure_export_equals_pressure_getter(semo):
    from semo_mesh_gb300.cases import vof_case
    case = vof_case(6)
    ctx = semo.Context(precision="fp64")
    ctx.set_case(case)
    ctx.assemble()
    a = ctx.system_rcm()
    b = ctx.system_rcm_eq("pressure")
    for k in ("ptr", "col", "val", "b"):
        assert np.array_equal(a[k], b[k]), k
    ctx.close()


def test_momentum_and_vof_exports_match_oracle(semo):
    from semo_mesh_gb300.cases import vof_case, with_history, with_vf_history
    from oracle.oracle import Oracle
    case = with_vf_history(with_history(vof_case(7), seed=12), seed=13)
    n = case.mesh.n_cells
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble_momentum()
    ctx = semo.Context(precision="fp64")
    ctx.set_case(case)
    perm, _ = ctx.lib_rcm()
    ctx.assemble_momentum()
    m = ctx.system_rcm_eq("momentum")
    r, c, v = to_caller(m, perm, n)
    A = dense_from(r, c, v, n)
    optr, ocol, oval = o.get("mom_csr_ptr"), o.get("mom_csr_col"), o.get("mom_csr_val")
    Aref = dense_from(np.repeat(np.arange(n), np.diff(optr)), ocol, oval, n)
    assert np.abs(A - Aref).max() <= TOL * np.abs(Aref).max()
    # the entries SEMO drops are stored, as zeros
    kept = np.zeros((n, n), bool)
    kept[np.repeat(np.arange(n), np.diff(optr)), ocol] = True
    assert np.all(v[~kept[r, c]] == 0.0)
    B = o.get("mom_B").reshape(3, n)
    for j in range(3):
        bj = np.empty(n)
        bj[perm] = m["b"][j]
        assert np.abs(bj - B[j]).max() <= TOL * np.abs(B[j]).max(), j
    # volume fraction
    o.assemble_vof()
    ctx.assemble_vof()
    w = ctx.system_rcm_eq("volume_fraction")
    r, c, v = to_caller(w, perm, n)
    A = dense_from(r, c, v, n)
    optr, ocol, oval = o.get("vof_csr_ptr"), o.get("vof_csr_col"), o.get("vof_csr_val")
    Aref = dense_from(np.repeat(np.arange(n), np.diff(optr)), ocol, oval, n)
    assert np.abs(A - Aref).max() <= TOL * np.abs(Aref).max()
    bj = np.empty(n)
    bj[perm] = w["b"]
    Bv = o.get("vof_B")
    assert np.abs(bj - Bv).max() <= TOL * np.abs(Bv).max()
    ctx.close()


def test_coupled_export_matches_oracle(semo):
    from semo_mesh_gb300.cases import coupled_case
    from oracle.oracle import Oracle
    case = coupled_case(3)
    n = case.mesh.n_cells
    o = Oracle(case.mesh)
    o.set_coupled(case)
    o.assemble_coupled()
    ctx = semo.Context(precision="fp64")
    ctx.set_coupled_case(case)
    perm, _ = ctx.lib_rcm()
    ctx.assemble_coupled()
    s = ctx.system_rcm_eq("coupled")
    r, c, v = to_caller(s, perm, n)
    A = dense_from(r, c, v, n, (5, 5))
    optr, ocol, oval = o.coupled_bsr()
    Aref = dense_from(np.repeat(np.arange(n), np.diff(optr)), ocol, oval, n, (5, 5))
    scale = np.abs(Aref).max(axis=(0, 1))
    scale[scale == 0] = 1.0
    assert (np.abs(A - Aref) / scale).max() <= TOL
    B = o.get("cpl_B").reshape(5, n)
    for a in range(5):
        ba = np.empty(n)
        ba[perm] = s["b"][a]
        assert np.abs(ba - B[a]).max() <= TOL * np.abs(B[a]).max(), a
    ctx.close()


def test_export_state_errors(semo):
    from semo_mesh_gb300.cases import vof_case
    case = vof_case(4)
    ctx = semo.Context()
    ctx.set_case(case)
    for eq in ("momentum", "volume_fraction", "coupled"):
        with pytest.raises(semo.SemoError) as e:
            ctx.system_rcm_eq(eq)
        assert e.value.status == 8
    ctx.close()
