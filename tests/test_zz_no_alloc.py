"""The allocation-free residual norm against the solver's own residual check.

semo_residual_norm_static is for callers that cannot call cudaMalloc (code
running inside a caller-managed memory arena or under a fixed device-memory
budget, or loops that must not synchronise through allocation calls): it keeps
its partial sums in a fixed array in the library's static device memory.  Its
result must equal the FP64 relative residual that semo_solve_coo reports for
the solution it returns, call after call (the static array is reused).

This file is collected last so a failure here does not hide the other tests.
"""
import ctypes

import numpy as np
import pytest

from golden_io import load

pytestmark = pytest.mark.gpu

TOL = 1e-10   # relative; both sides are the same FP64 sums in a different order


def coo_to_csr(n, rows, cols, vals):
    """SEMO's COO -> CSR (solveAMGCL.cpp:206-251): in-row order = COO order."""
    order = np.argsort(rows, kind="stable")
    ptr = np.zeros(n + 1, dtype=np.int32)
    np.add.at(ptr, rows.astype(np.int64) + 1, 1)
    return np.cumsum(ptr).astype(np.int32), cols[order].astype(np.int32), vals[order].astype(np.float64)


def numpy_rel_residual(ptr, col, val, x, b):
    """FP64 ||b - A x|| / ||b|| on the host, row by row from the CSR arrays."""
    rows = np.repeat(np.arange(len(ptr) - 1), np.diff(ptr))
    ax = np.zeros(len(b))
    np.add.at(ax, rows, val * x[col])
    return np.linalg.norm(b - ax) / np.linalg.norm(b)


def random_csr(n, seed):
    """A diagonally dominant random CSR of n rows with 1-9 off-diagonals a row."""
    rng = np.random.default_rng(seed)
    counts = rng.integers(1, 10, n)
    ptr = np.zeros(n + 1, np.int32)
    ptr[1:] = np.cumsum(counts + 1)
    rows = np.repeat(np.arange(n), counts + 1)
    first = np.zeros(ptr[-1], bool)
    first[ptr[:-1]] = True                                   # the diagonal leads each row
    col = np.where(first, rows, rng.integers(0, n, ptr[-1])).astype(np.int32)
    val = np.where(first, 0.0, rng.uniform(-1.0, 1.0, ptr[-1]))
    val[ptr[:-1]] = 1.0 + np.add.reduceat(np.abs(val), ptr[:-1])
    return ptr, col, val


def systems():
    case, ref = load("box7j")
    yield "box7j", ref["A_rows"], ref["A_cols"], ref["A_vals"], ref["B"]
    from semo_mesh_gb300.cases import vof_case
    from oracle.oracle import Oracle
    c = vof_case(16)
    o = Oracle(c.mesh)
    o.set_case(c)
    o.assemble()
    yield "vof16", o.get("A_rows"), o.get("A_cols"), o.get("A_vals"), o.get("B")


@pytest.mark.parametrize("name,rows,cols,vals,B", [pytest.param(*s, id=s[0]) for s in systems()])
def test_static_residual_matches_solver(name, rows, cols, vals, B):
    import torch
    import semo_mesh_gb300 as S
    L = S.load_library()
    L.semo_residual_norm_static.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] + [ctypes.c_void_p] * 4
    n = len(B)
    ctx = S.Context(precision="fp64", tol=1e-10)
    res = ctx.solve_amgcl("pressure", 1, rows, cols, vals, B)
    existing = res.info["rel_residual"]
    ptr, col, val = coo_to_csr(n, rows, cols, vals)
    dev = torch.device("cuda:0")
    d = {k: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
         for k, a in (("ptr", ptr), ("col", col), ("val", val), ("x", res.x), ("b", np.asarray(B, np.float64)))}
    out = torch.full((3,), -1.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    got = []
    for _ in range(2):                      # two calls in a row share the static scratch
        out.fill_(-1.0)
        st = L.semo_residual_norm_static(d["ptr"].data_ptr(), d["col"].data_ptr(), d["val"].data_ptr(), n,
                                         d["x"].data_ptr(), d["b"].data_ptr(), out.data_ptr(),
                                         ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, S.STATUS.get(st, st)
        torch.cuda.synchronize()
        got.append(out.cpu().numpy().copy())
    host = numpy_rel_residual(ptr, col, val, np.asarray(res.x, np.float64), np.asarray(B, np.float64))
    for g in got:
        assert abs(g[0] - existing) <= TOL * existing, (g[0], existing)
        assert abs(g[0] - host) <= 1e-6 * host, (g[0], host)   # a converged residual cancels ~8 digits
        assert abs(g[2] - np.linalg.norm(B)) <= TOL * np.linalg.norm(B)
    assert np.array_equal(got[0], got[1])


@pytest.mark.parametrize("n", [100_003, 2_097_152 - 5])
def test_static_residual_matches_numpy(n):
    """Rows not a multiple of 32 (a ragged last block) and more than 256 partial
    sums (the finishing kernel's strided loop), against NumPy FP64, twice."""
    import torch
    import semo_mesh_gb300 as S
    L = S.load_library()
    L.semo_residual_norm_static.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] + [ctypes.c_void_p] * 4
    ptr, col, val = random_csr(n, 7)
    rng = np.random.default_rng(8)
    x = rng.standard_normal(n)
    b = rng.standard_normal(n)
    host = numpy_rel_residual(ptr, col, val, x, b)
    dev = torch.device("cuda:0")
    d = [torch.from_numpy(a).to(dev) for a in (ptr, col, val, x, b)]
    out = torch.full((3,), -1.0, dtype=torch.float64, device=dev)
    got = []
    for _ in range(2):
        out.fill_(-1.0)
        st = L.semo_residual_norm_static(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), n, d[3].data_ptr(),
                                         d[4].data_ptr(), out.data_ptr(), None)
        assert st == 0, S.STATUS.get(st, st)
        torch.cuda.synchronize()
        got.append(out.cpu().numpy().copy())
    for g in got:
        assert abs(g[0] - host) <= 1e-12 * host, (g[0], host)
        assert abs(g[2] - np.linalg.norm(b)) <= 1e-12 * np.linalg.norm(b)
    assert np.array_equal(got[0], got[1])


def test_static_residual_rejects_oversize():
    import torch
    import semo_mesh_gb300 as S
    L = S.load_library()
    L.semo_residual_norm_static.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] + [ctypes.c_void_p] * 4
    t = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    i = torch.zeros(8, dtype=torch.int32, device="cuda:0")
    st = L.semo_residual_norm_static(i.data_ptr(), i.data_ptr(), t.data_ptr(), 2097152 + 1, t.data_ptr(),
                                     t.data_ptr(), t.data_ptr(), None)
    assert st == 1   # SEMO_ERR_ARGUMENT: beyond the static scratch, nothing launched
