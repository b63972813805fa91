"""The 16-bit-column SELL layout at bandwidths beyond 16-bit row offsets.

A 5-point Laplacian (plus a mass term) on a 70,000 x 3 grid (210,000 rows) couples row i to
i +- 70,000.  No slice fits signed 16-bit offsets from the row; most fit
unsigned offsets from their (slice, entry) group base, and the slices where
a row gains its i - 70,000 neighbour have a group spanning ~70,000 columns
and keep 32-bit columns.  The finest operator of the V-cycle (FP32) and the
FP64 outer operator both take this layout; the solution must match a direct
sparse solve.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def grid_laplacian(nx, ny):
    """COO of the Dirichlet 5-point Laplacian plus 0.5 I (a time term), the
    diagonal entries first and then each row's off-diagonals by ascending
    column, as SEMO's COO lists them."""
    rows, cols, vals = [], [], []
    n = nx * ny
    idx = np.arange(n)
    x = idx % nx
    y = idx // nx
    rows.append(idx); cols.append(idx); vals.append(np.full(n, 4.5))   # + a mass term: well conditioned
    for dx, dy in ((-1, 0), (1, 0), (0, -1), (0, 1)):
        ok = (x + dx >= 0) & (x + dx < nx) & (y + dy >= 0) & (y + dy < ny)
        rows.append(idx[ok]); cols.append(idx[ok] + dx + dy * nx); vals.append(np.full(ok.sum(), -1.0))
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    v = np.concatenate(vals)
    # diagonal entries first (the first n), then off-diagonals row by row
    off = np.lexsort((c[n:], r[n:]))
    return (np.concatenate([r[:n], r[n:][off]]).astype(np.int32), np.concatenate([c[:n], c[n:][off]]).astype(np.int32),
            np.concatenate([v[:n], v[n:][off]]), n)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_wide_bandwidth_solve(precision):
    scipy_sparse = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    import semo_mesh_gb300 as S
    rows, cols, vals, n = grid_laplacian(70000, 3)
    assert np.abs(cols.astype(np.int64) - rows).max() == 70000
    rng = np.random.default_rng(11)
    b = rng.standard_normal(n)
    A = scipy_sparse.csr_matrix((vals, (rows, cols)), shape=(n, n))
    ref = spla.spsolve(A.tocsc(), b)
    ctx = S.Context(precision=precision, tol=1e-10, max_iter=1000)
    res = ctx.solve_amgcl("pressure", 1, rows, cols, vals, b)
    assert res.info["rel_residual"] <= 1e-10
    err = np.linalg.norm(res.x - ref) / np.linalg.norm(ref)
    assert err < 1e-7, err
    # the finest V-cycle operator took the 16-bit-column layout
    lev = ctx.hierarchy_levels()
    assert lev[0]["rows"] == n and lev[0]["layout"] == 2
    ctx.close()
