"""The adjoint formulation, checked on the oracle alone (CPU).

With a per-cell source s entering the pressure right-hand side as
b_i += s_i V_i and J = sum of x_i^2 over the z = 1 cells, the gradient is
dJ/ds = V A^-T (2 x on those cells).  The oracle's assembled A is symmetric
bit for bit (a face's off-diagonal coefficient goes to both of its rows,
eqPressure.cpp:538-548), so the transpose solve is a plain solve.  Central
differences (h = 1e-6, seeds 100-115) confirm the gradient; the GPU's VJP is
compared with this same gradient in the GPU tests.
"""
import numpy as np
import pytest

from semo_mesh_gb300.cases import box_case


@pytest.fixture(scope="module")
def small():
    from oracle.oracle import Oracle
    case = box_case(12, jitter=0.2)
    s = np.random.default_rng(4).standard_normal(case.mesh.n_cells)
    zc = np.unique(case.mesh.patch_cells("zmax"))
    o = Oracle(case.mesh)
    o.set_case(case)
    o.assemble()
    return case, s, zc, o, o.get("cell_vol"), o.get("B")


def test_assembled_matrix_symmetric(small):
    sp = pytest.importorskip("scipy.sparse")
    o = small[3]
    a = sp.csr_matrix((o.get("csr_val"), o.get("csr_col"), o.get("csr_ptr")))
    assert (a != a.T).nnz == 0


def test_source_gradient_matches_central_differences(small):
    case, s, zc, o, vol, b0 = small

    def forward(src):
        o.set("B", b0 + src * vol)
        r = o.solve(False, 1e-13, 1000)
        assert r["rel_res"] <= 1e-13
        return r["x"]

    x = forward(s)
    g = np.zeros_like(x)
    g[zc] = 2.0 * x[zc]
    o.set("B", g)
    djds = o.solve(False, 1e-13, 1000)["x"] * vol
    h = 1e-6
    fd, ad = [], []
    for seed in range(100, 116):
        d = np.random.default_rng(seed).standard_normal(case.mesh.n_cells)
        jp = np.sum(forward(s + h * d)[zc] ** 2)
        jm = np.sum(forward(s - h * d)[zc] ** 2)
        fd.append((jp - jm) / (2.0 * h))
        ad.append(djds @ d)
    fd, ad = np.array(fd), np.array(ad)
    assert np.linalg.norm(ad - fd) / np.linalg.norm(fd) < 1e-6
