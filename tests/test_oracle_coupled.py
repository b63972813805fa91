"""The oracle's compressible coupled 5x5 block system (no reference to pin).

The reference's calcCompCoupledEq (src/solvers/compressible/coupled.cpp) is
commented out from its first to its last line, so the oracle restates the
state its body was in when last live.  Nothing compiled from the reference
can check it; these tests check what can be derived independently:

* the ideal-gas EOS against its closed forms;
* the diagonal time block against a central finite difference of the cell
  part of the right-hand side (the reference's Newton form A dW = B makes
  the time block -dB/dW when the bounded BDF2 falls back to first order);
* conservation of the face terms: each face adds equal and opposite
  amounts to its two cells, so the face part of every column sums to zero
  and the face part of B sums to zero;
* the block structure the reference's live lines give (zero cross-momentum
  blocks, zero continuity-velocity entries in the time block);
* the block-Jacobi BiCGStab solution reaches its residual.
"""
import numpy as np
import pytest

from semo_mesh_gb300.cases import coupled_case


@pytest.fixture(scope="module")
def small():
    from oracle.oracle import Oracle
    case = coupled_case(5)
    o = Oracle(case.mesh)
    o.set_coupled(case)
    return case, o


def dense(o, n):
    """The BSR system as a dense (5n x 5n) matrix in field-split order."""
    ptr, col, val = o.coupled_bsr()
    A = np.zeros((5 * n, 5 * n))
    for i in range(n):
        for k in range(ptr[i], ptr[i + 1]):
            j = col[k]
            for a in range(5):
                A[a * n + i, np.arange(5) * n + j] += val[k, a, :]
    return A


def test_tet_mesh_is_closed_and_positive(small):
    case, o = small
    vol = o.get("cell_vol")
    assert vol.min() > 0.0
    assert abs(vol.sum() - 1.0) < 1e-12
    m = case.mesh
    assert m.n_cells == 6 * 5 ** 3
    assert m.n_faces - m.n_internal == 12 * 5 ** 2
    assert np.all(m.owner[:m.n_internal] < m.neighbour)


def test_eos_closed_forms(small):
    case, o = small
    o.assemble_coupled()
    e = o.get("cpl_eos").reshape(-1, 7)
    R = (case.gamma - 1.0) * case.cv
    rho = case.P / (R * case.T)
    usq = case.U ** 2 + case.V ** 2 + case.W ** 2
    np.testing.assert_allclose(e[:, 0], rho, rtol=1e-14)
    np.testing.assert_allclose(e[:, 1], np.sqrt(case.gamma * R * case.T), rtol=1e-14)
    np.testing.assert_allclose(e[:, 2], case.gamma * case.cv * case.T + 0.5 * usq, rtol=1e-14)
    np.testing.assert_allclose(e[:, 3], 1.0 / (R * case.T), rtol=1e-14)
    np.testing.assert_allclose(e[:, 4], -rho / case.T, rtol=1e-14)
    assert np.all(e[:, 5] == 0.0)
    np.testing.assert_allclose(e[:, 6], case.gamma * case.cv, rtol=1e-15)


def test_time_block_is_the_derivative_of_the_cell_terms():
    """Monotone history (n-2 < n-1 < n) makes the bounded BDF2 first order."""
    from oracle.oracle import Oracle
    case = coupled_case(3)
    cur = np.stack([case.P, case.U, case.V, case.W, case.T])
    case.old = cur * (1.0 - 1e-3)
    case.old2 = cur * (1.0 - 2e-3)
    case.gravity = (0.3, -0.2, -9.81)
    o = Oracle(case.mesh)
    o.set_coupled(case)
    o.assemble_coupled(terms=1)
    D = o.get("cpl_diag").reshape(-1, 5, 5)
    names = ("P", "U", "V", "W", "T")
    n = case.mesh.n_cells
    cells = [0, n // 2, n - 1]
    for b, nm in enumerate(names):
        base = getattr(case, nm).copy()
        h = 1e-6 * max(1.0, float(np.abs(base).max()))
        cols = []
        for sgn in (1.0, -1.0):
            f = base.copy()
            f[cells] += sgn * h
            setattr(case, nm, f)
            o.set_coupled(case)
            o.assemble_coupled(terms=1)
            cols.append(o.get("cpl_B").reshape(5, n)[:, cells])
        setattr(case, nm, base)
        fd = -(cols[0] - cols[1]) / (2.0 * h)          # -dB/dW_b, shape (5, len(cells))
        for ci, i in enumerate(cells):
            scale = np.abs(D[i]).max()
            np.testing.assert_allclose(D[i][:, b], fd[:, ci], rtol=0, atol=2e-6 * scale, err_msg=f"{nm} cell {i}")


def test_face_terms_conserve(small):
    case, o = small
    n = case.mesh.n_cells
    o.assemble_coupled(terms=2)
    A = dense(o, n)
    B = o.get("cpl_B").reshape(5, n)
    colsum = np.abs(A.sum(axis=0)).max()
    assert colsum <= 1e-12 * np.abs(A).max()
    for a in range(5):
        assert abs(B[a].sum()) <= 1e-11 * np.abs(B[a]).sum()


def test_block_structure(small):
    case, o = small
    o.assemble_coupled()
    LR = o.get("cpl_LR").reshape(-1, 5, 5)
    RL = o.get("cpl_RL").reshape(-1, 5, 5)
    for a, b in ((1, 2), (1, 3), (2, 1), (2, 3), (3, 1), (3, 2)):
        assert np.all(LR[:, a, b] == 0.0) and np.all(RL[:, a, b] == 0.0)
    o.assemble_coupled(terms=1)
    D = o.get("cpl_diag").reshape(-1, 5, 5)
    assert np.all(D[:, 0, 1:4] == 0.0)
    assert np.all(D[:, 1, 2:4] == 0.0)


def test_solution_residual(small):
    case, o = small
    o.assemble_coupled()
    sol = o.solve_coupled(1e-12, 2000)
    assert sol["rel_res"] < 1e-10
    n = case.mesh.n_cells
    A = dense(o, n)
    b = o.get("cpl_B")
    x = np.linalg.solve(A, b)
    assert np.linalg.norm(sol["x"] - x) <= 1e-9 * np.linalg.norm(x)


def test_update_and_norm(small):
    case, o = small
    o.set_coupled(case)
    o.assemble_coupled()
    sol = o.solve_coupled(1e-12, 2000)
    norm = o.update_coupled(sol["x"], case.limits)
    x = sol["x"].reshape(5, -1)
    new = np.stack([o.get("cpl_" + k) for k in ("P", "U", "V", "W", "T")])
    old = np.stack([case.P, case.U, case.V, case.W, case.T])
    np.testing.assert_allclose(new, old + case.urf * x, rtol=1e-15, atol=1e-9)
    ref = np.sqrt((x ** 2).sum()) / np.sqrt((new ** 2).sum()) / 5.0
    assert abs(norm - ref) <= 1e-12 * ref
    o.set_coupled(case)
