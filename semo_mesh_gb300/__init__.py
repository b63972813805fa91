"""GB300 (sm_103a) drop-in for SEMO's per-outer-iteration pressure path.

Python mirror of the reference's interface for this path, over the C-ABI of
include/semo_gb300.h (libsemo_gb300.so, built in-tree by
``semo_mesh_gb300.build``):

* ``Context.calc_pressure_eq()``   -- SEMO_Solvers_Builder::calcPressureEq
  (src/solvers/eqPressure.cpp:8-942), returning SEMO's ||dprim||/||prim||;
* ``Context.solve_amgcl(...)``     -- SEMO_Solvers_Builder::solveAMGCL for the
  scalar "pressure" equation (src/solvers/solveAMGCL.cpp:179-1108): SEMO's
  COO triple in, solution vector out;
* ``Context.lib_rcm()``            -- SEMO_Utility_Math::lib_RCM
  (src/math/RCM.cpp:34-218): (cells[i].RCM, cells[i].invRCM).

There is no CPU fallback: without the built library (or without a GB300) the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsemo_gb300.so")

SEMO_OK = 0
STATUS = {0: "SEMO_OK", 1: "SEMO_ERR_ARGUMENT", 2: "SEMO_ERR_MESH", 3: "SEMO_ERR_CUDA",
          4: "SEMO_ERR_OUT_OF_MEMORY", 5: "SEMO_ERR_NOT_CONVERGED", 6: "SEMO_ERR_NAN",
          7: "SEMO_ERR_BREAKDOWN", 8: "SEMO_ERR_STATE", 9: "SEMO_ERR_NO_DEVICE"}
PREC_FP64 = 0
PREC_MIXED = 1


class SemoError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Params(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("tol", C.c_double), ("max_iter", C.c_int),
                ("eps_strong", C.c_double), ("coarse_enough", C.c_int), ("max_levels", C.c_int),
                ("cheb_degree", C.c_int), ("reuse_hierarchy", C.c_int), ("mom_tol", C.c_double),
                ("mom_max_iter", C.c_int), ("overlap_setup", C.c_int), ("smoother", C.c_int)]


class Physics(C.Structure):
    _fields_ = [("dt", C.c_double), ("rho", C.c_double * 2), ("gravity", C.c_double * 3),
                ("use_gravity", C.c_int), ("urf_p", C.c_double), ("urf_u", C.c_double),
                ("p_min", C.c_double), ("p_max", C.c_double), ("u_min", C.c_double), ("u_max", C.c_double),
                ("v_min", C.c_double), ("v_max", C.c_double), ("w_min", C.c_double), ("w_max", C.c_double),
                ("mu", C.c_double * 2), ("urf_mom", C.c_double), ("urf_vof", C.c_double),
                ("sigma", C.c_double)]


class CoupledPhysics(C.Structure):
    _fields_ = [("cv", C.c_double), ("gamma", C.c_double), ("mu", C.c_double), ("dt", C.c_double),
                ("dt_old", C.c_double), ("dt_old2", C.c_double), ("gravity", C.c_double * 3),
                ("urf", C.c_double), ("limits", C.c_double * 10)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("rel_residual", C.c_double), ("levels", C.c_int),
                ("coarse_size", C.c_int), ("operator_complexity", C.c_double),
                ("setup_ms", C.c_double), ("solve_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load the C-ABI library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m semo_mesh_gb300.build` "
                          "(there is no CPU fallback)")
    L = C.CDLL(path)
    vp, i32p, f64p = C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_double)
    L.semo_params_default.argtypes = [C.POINTER(Params)]
    L.semo_physics_default.argtypes = [C.POINTER(Physics)]
    L.semo_ctx_create.argtypes = [C.POINTER(vp), C.POINTER(Params)]
    L.semo_ctx_destroy.argtypes = [vp]
    L.semo_last_error.restype = C.c_char_p
    L.semo_last_error.argtypes = [vp]
    L.semo_stream.restype = vp
    L.semo_stream.argtypes = [vp]
    L.semo_mesh_upload.argtypes = [vp, C.c_int, f64p, C.c_int, C.c_int, C.c_int, i32p, i32p, i32p, i32p,
                                   C.c_int, i32p, i32p]
    L.semo_rcm.argtypes = [vp, i32p, i32p]
    L.semo_set_physics.argtypes = [vp, C.POINTER(Physics), i32p, f64p]
    L.semo_set_fields.argtypes = [vp, f64p, f64p, f64p, f64p, f64p]
    L.semo_get_fields.argtypes = [vp, f64p, f64p, f64p, f64p]
    L.semo_pressure_pass.argtypes = [vp, f64p, C.POINTER(SolveInfo)]
    L.semo_assemble_pressure.argtypes = [vp]
    L.semo_get_system_rcm.argtypes = [vp, i32p, i32p, f64p, f64p]
    L.semo_get_system_rcm_eq.argtypes = [vp, C.c_int, i32p, i32p, f64p, f64p]
    L.semo_get_array.argtypes = [vp, C.c_char_p, f64p, C.c_int64]
    L.semo_solve_pressure.argtypes = [vp, f64p, C.POINTER(SolveInfo)]
    L.semo_solve_coo.argtypes = [vp, C.c_int, C.c_int64, i32p, i32p, f64p, f64p, f64p, C.POINTER(SolveInfo)]
    L.semo_solve_coo_multi.argtypes = [vp, C.c_int, C.c_int, C.c_int64, i32p, i32p, f64p, f64p, f64p,
                                       C.POINTER(SolveInfo)]
    L.semo_set_source.argtypes = [vp, f64p]
    L.semo_vjp_source.argtypes = [vp, f64p, f64p, f64p, C.POINTER(SolveInfo)]
    L.semo_vjp_fields.argtypes = [vp, f64p, f64p, f64p, f64p, f64p, f64p, C.POINTER(SolveInfo)]
    L.semo_set_profiling.argtypes = [vp, C.c_int]
    L.semo_stage_time.argtypes = [vp, C.c_char_p, f64p, C.POINTER(C.c_int64)]
    L.semo_reset_stats.argtypes = [vp]
    L.semo_kernel_launches.restype = C.c_int64
    L.semo_mesh_info.argtypes = [vp, C.POINTER(C.c_int64)]
    L.semo_time_spmv.argtypes = [vp, C.c_int, C.c_int, f64p]
    L.semo_hierarchy_levels.argtypes = [vp, C.POINTER(C.c_int64), C.c_int, C.POINTER(C.c_int)]
    L.semo_set_old_velocity.argtypes = [vp, f64p, f64p, f64p, f64p, f64p, f64p]
    L.semo_momentum_pass.argtypes = [vp, f64p, C.POINTER(SolveInfo)]
    L.semo_assemble_momentum.argtypes = [vp]
    L.semo_get_momentum_system.argtypes = [vp, i32p, i32p, f64p, f64p, C.POINTER(C.c_int64)]
    L.semo_solve_momentum.argtypes = [vp, f64p, C.POINTER(SolveInfo)]
    L.semo_outer_iteration.argtypes = [vp, f64p, C.POINTER(SolveInfo)]
    L.semo_set_old_vf.argtypes = [vp, f64p, f64p]
    L.semo_vof_pass.argtypes = [vp, f64p, C.POINTER(SolveInfo)]
    L.semo_assemble_vof.argtypes = [vp]
    L.semo_source_surface_tension.argtypes = [vp]
    L.semo_get_surface_tension.argtypes = [vp, f64p, f64p, f64p]
    L.semo_get_vof_system.argtypes = [vp, i32p, i32p, f64p, f64p, C.POINTER(C.c_int64)]
    L.semo_solve_vof.argtypes = [vp, f64p, C.POINTER(SolveInfo)]
    L.semo_foam_sizes.argtypes = [C.c_char_p, C.POINTER(C.c_int64)]
    L.semo_foam_read.argtypes = [C.c_char_p, f64p, i32p, i32p, i32p, i32p, i32p, i32p, C.c_char_p]
    L.semo_foam_last_error.restype = C.c_char_p
    L.semo_mesh_load_foam.argtypes = [vp, C.c_char_p]
    L.semo_set_coupled_physics.argtypes = [vp, C.POINTER(CoupledPhysics), i32p, f64p]
    L.semo_set_coupled_fields.argtypes = [vp, f64p, f64p, f64p, f64p, f64p, f64p, f64p]
    L.semo_get_coupled_fields.argtypes = [vp, f64p, f64p, f64p, f64p, f64p]
    L.semo_assemble_coupled.argtypes = [vp]
    L.semo_get_coupled_system.argtypes = [vp, i32p, i32p, f64p, f64p, C.POINTER(C.c_int64)]
    L.semo_solve_coupled.argtypes = [vp, f64p, C.POINTER(SolveInfo)]
    L.semo_coupled_pass.argtypes = [vp, f64p, C.POINTER(SolveInfo)]
    _lib = L
    return L


def _i32(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int32))


def _f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


@dataclass
class SolveResult:
    x: np.ndarray
    info: dict


class Context:
    """One GPU context (semo_ctx) holding a mesh, its fields and the solver."""

    def __init__(self, precision: str = "mixed", tol: float = 1e-8, max_iter: int = 500, device: int = 0,
                 eps_strong: float = 0.03, coarse_enough: int = 64, cheb_degree: int = 2, max_levels: int = 24,
                 mom_tol: float = 1e-9, mom_max_iter: int = 1000, reuse_hierarchy: bool = True,
                 overlap_setup: bool = True, smoother: str = "chebyshev"):
        self.L = load_library()
        p = Params()
        self.L.semo_params_default(C.byref(p))
        p.device = device
        p.precision = PREC_MIXED if precision == "mixed" else PREC_FP64
        p.tol = tol
        p.max_iter = max_iter
        p.eps_strong = eps_strong
        p.coarse_enough = coarse_enough
        p.cheb_degree = cheb_degree
        p.max_levels = max_levels
        p.reuse_hierarchy = 1 if reuse_hierarchy else 0
        p.mom_tol = mom_tol
        p.mom_max_iter = mom_max_iter
        p.overlap_setup = 1 if overlap_setup else 0
        if smoother not in ("chebyshev", "gauss_seidel"):
            raise SemoError(1, f"unknown smoother '{smoother}' (chebyshev or gauss_seidel)")
        p.smoother = 1 if smoother == "gauss_seidel" else 0
        h = C.c_void_p()
        st = self.L.semo_ctx_create(C.byref(h), C.byref(p))
        if st != SEMO_OK:
            raise SemoError(st, "semo_ctx_create failed (no GB300 / CUDA device?)")
        self.h = h
        self.mesh = None
        self.n_cells = 0

    def _check(self, st: int, allow=()):
        if st != SEMO_OK and st not in allow:
            raise SemoError(st, self.L.semo_last_error(self.h).decode(errors="replace"))
        return st

    def close(self):
        if getattr(self, "h", None):
            self.L.semo_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(self.L.semo_stream(self.h) or 0)

    # ---- mesh / case -----------------------------------------------------
    def upload_mesh(self, mesh) -> None:
        pts, pp = _f64(mesh.points.reshape(-1))
        keep = [_i32(mesh.face_ptr), _i32(mesh.face_pts), _i32(mesh.owner), _i32(mesh.neighbour),
                _i32(mesh.patch_start), _i32(mesh.patch_size)]
        self._check(self.L.semo_mesh_upload(self.h, mesh.n_points, pp, mesh.n_faces, mesh.n_internal, mesh.n_cells,
                                            keep[0][1], keep[1][1], keep[2][1], keep[3][1],
                                            len(mesh.patch_names), keep[4][1], keep[5][1]))
        self.mesh = mesh
        self.n_cells = mesh.n_cells

    def load_foam(self, directory: str, mesh=None) -> None:
        """Read an OpenFOAM polyMesh directory and upload it (semo_mesh_load_foam).

        ``mesh`` (a PolyMesh of the same directory, e.g. from
        ``foam.read_polymesh``) is kept for the case helpers that need the
        patch layout."""
        from .foam import read_polymesh
        self._check(self.L.semo_mesh_load_foam(self.h, directory.encode()))
        self.mesh = mesh if mesh is not None else read_polymesh(directory)
        self.n_cells = self.mesh.n_cells

    def set_physics(self, case) -> None:
        ph = Physics()
        self.L.semo_physics_default(C.byref(ph))
        ph.dt = case.dt
        ph.rho[0], ph.rho[1] = case.rho
        ph.gravity[0], ph.gravity[1], ph.gravity[2] = case.gravity
        ph.use_gravity = 1 if case.use_gravity else 0
        ph.urf_p = case.pre_p_urf
        ph.urf_u = case.pre_u_urf
        ph.mu[0], ph.mu[1] = case.mu
        ph.urf_mom = case.mom_u_urf
        ph.urf_vof = case.vof_urf
        ph.sigma = case.sigma
        bt, btp = _i32(case.bc_type.reshape(-1))
        bv, bvp = _f64(case.bc_value.reshape(-1))
        self._check(self.L.semo_set_physics(self.h, C.byref(ph), btp, bvp))

    def set_fields(self, P, U, V, W, VF) -> None:
        arrs = [_f64(a) for a in (P, U, V, W, VF)]
        self._check(self.L.semo_set_fields(self.h, *[a[1] for a in arrs]))

    def set_case(self, case) -> None:
        if self.mesh is not case.mesh:
            self.upload_mesh(case.mesh)
        self.set_physics(case)
        self.set_fields(case.P, case.U, case.V, case.W, case.VF)
        if case.old is None and case.old2 is None:
            self.set_old_velocity(None)
        else:
            h = case.history()
            self.set_old_velocity(h[:3], h[3:])
        if case.old_vf is None and case.old2_vf is None:
            self.set_old_vf(None)
        else:
            self.set_old_vf(*case.vf_history())

    def set_old_vf(self, old_vf, old2_vf=None) -> None:
        """BDF2 history of the volume fraction (n-1, n-2); None clears it."""
        if old_vf is None:
            self._check(self.L.semo_set_old_vf(self.h, None, None))
            return
        a, ap = _f64(old_vf)
        b, bp = _f64(old2_vf)
        self._check(self.L.semo_set_old_vf(self.h, ap, bp))

    def set_old_velocity(self, old, old2=None) -> None:
        """BDF2 history: old = (U, V, W) at n-1, old2 at n-2; None clears both."""
        if old is None:
            self._check(self.L.semo_set_old_velocity(self.h, None, None, None, None, None, None))
            return
        arrs = [_f64(a) for a in (*old, *old2)]
        self._check(self.L.semo_set_old_velocity(self.h, *[a[1] for a in arrs]))

    def fields(self, out: dict | None = None) -> dict:
        """P, U, V, W in the caller's cell order (into `out`'s arrays if given, e.g. pinned buffers)."""
        n = self.n_cells
        if out is None:
            out = {k: np.empty(n) for k in ("P", "U", "V", "W")}
        for k in ("P", "U", "V", "W"):
            if out[k].dtype != np.float64 or not out[k].flags.c_contiguous or out[k].shape != (n,):
                raise ValueError(f"output array {k} must be contiguous float64 of length {n}")
        ptrs = [out[k].ctypes.data_as(C.POINTER(C.c_double)) for k in ("P", "U", "V", "W")]
        self._check(self.L.semo_get_fields(self.h, *ptrs))
        return out

    def set_source(self, s) -> None:
        if s is None:
            self._check(self.L.semo_set_source(self.h, None))
        else:
            a, ap = _f64(s)
            self._check(self.L.semo_set_source(self.h, ap))

    # ---- the reference's entry points -------------------------------------
    def calc_pressure_eq(self) -> tuple:
        """calcPressureEq: one pressure-correction pass; returns (norm, info)."""
        norm = C.c_double()
        info = SolveInfo()
        self._check(self.L.semo_pressure_pass(self.h, C.byref(norm), C.byref(info)))
        return norm.value, info.as_dict()

    def calc_momentum_eqs(self) -> tuple:
        """calcMomentumEqs: one momentum pass; returns (norm, [info x, y, z])."""
        norm = C.c_double()
        info = (SolveInfo * 3)()
        self._check(self.L.semo_momentum_pass(self.h, C.byref(norm), info))
        return norm.value, [i.as_dict() for i in info]

    def outer_iteration(self) -> tuple:
        """Momentum then pressure (one pressure correction): ((norm_mom, norm_p), [4 infos])."""
        norms = (C.c_double * 2)()
        info = (SolveInfo * 4)()
        self._check(self.L.semo_outer_iteration(self.h, norms, info))
        return (norms[0], norms[1]), [i.as_dict() for i in info]

    def calc_volfrac_eq(self) -> tuple:
        """One volume-fraction sub-iteration (MSTACS + calcVolfracEq): (norm, info)."""
        norm = C.c_double()
        info = SolveInfo()
        self._check(self.L.semo_vof_pass(self.h, C.byref(norm), C.byref(info)))
        return norm.value, info.as_dict()

    def assemble_vof(self) -> None:
        self._check(self.L.semo_assemble_vof(self.h))

    def calc_source_surface_tension(self) -> None:
        """Curvature and surface-tension source from the current fields (sigma != 0)."""
        self._check(self.L.semo_source_surface_tension(self.h))

    def surface_tension(self) -> dict:
        """The last curvature / source: kappa, ls (n_cells each), src (n_cells x 4)."""
        n = self.n_cells
        kap, ls, src = np.empty(n), np.empty(n), np.empty(4 * n)
        p = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        self._check(self.L.semo_get_surface_tension(self.h, p(kap), p(ls), p(src)))
        return {"kappa": kap, "ls": ls, "src": src.reshape(n, 4)}

    def vof_system(self) -> dict:
        """The volume-fraction system in SEMO's layout (caller numbering, COO-scatter rows)."""
        n = self.n_cells
        nnz = C.c_int64()
        self._check(self.L.semo_get_vof_system(self.h, None, None, None, None, C.byref(nnz)))
        ptr = np.empty(n + 1, dtype=np.int32)
        col = np.empty(nnz.value, dtype=np.int32)
        val = np.empty(nnz.value)
        b = np.empty(n)
        self._check(self.L.semo_get_vof_system(self.h, ptr.ctypes.data_as(C.POINTER(C.c_int32)),
                                               col.ctypes.data_as(C.POINTER(C.c_int32)),
                                               val.ctypes.data_as(C.POINTER(C.c_double)),
                                               b.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nnz)))
        return {"ptr": ptr, "col": col, "val": val, "b": b}

    def solve_vof(self) -> SolveResult:
        x = np.empty(self.n_cells)
        info = SolveInfo()
        self._check(self.L.semo_solve_vof(self.h, x.ctypes.data_as(C.POINTER(C.c_double)), C.byref(info)))
        return SolveResult(x=x, info=info.as_dict())

    # ---- compressible coupled system (calcCompCoupledEq) --------------------
    def set_coupled_case(self, case) -> None:
        """Mesh (if new), physics, boundary conditions and fields of a CoupledCase."""
        if self.mesh is not case.mesh:
            self.upload_mesh(case.mesh)
        ph = CoupledPhysics()
        ph.cv, ph.gamma, ph.mu = case.cv, case.gamma, case.mu
        ph.dt, ph.dt_old, ph.dt_old2 = case.dt, case.dt_old, case.dt_old2
        for k in range(3):
            ph.gravity[k] = case.gravity[k]
        ph.urf = case.urf
        for k in range(10):
            ph.limits[k] = float(case.limits[k])
        bt, btp = _i32(case.bc_type)
        bv, bvp = _f64(case.bc_value)
        self._check(self.L.semo_set_coupled_physics(self.h, C.byref(ph), btp, bvp))
        self.set_coupled_fields(case.P, case.U, case.V, case.W, case.T, *case.history())

    def set_coupled_fields(self, P, U, V, W, T, old=None, old2=None) -> None:
        arrs = [_f64(a) for a in (P, U, V, W, T)]
        o = _f64(old) if old is not None else (None, None)
        o2 = _f64(old2) if old2 is not None else (None, None)
        self._check(self.L.semo_set_coupled_fields(self.h, *[a[1] for a in arrs], o[1], o2[1]))

    def coupled_fields(self) -> dict:
        n = self.n_cells
        out = {k: np.empty(n) for k in ("P", "U", "V", "W", "T")}
        self._check(self.L.semo_get_coupled_fields(self.h, *[_f64(out[k])[1] for k in ("P", "U", "V", "W", "T")]))
        return out

    def assemble_coupled(self) -> None:
        self._check(self.L.semo_assemble_coupled(self.h))

    def coupled_system(self) -> dict:
        """(ptr, col, val[nnz, 5, 5], b[5, n]) in the caller's numbering."""
        n = self.n_cells
        nnz = C.c_int64()
        self._check(self.L.semo_get_coupled_system(self.h, None, None, None, None, C.byref(nnz)))
        ptr = np.empty(n + 1, dtype=np.int32)
        col = np.empty(nnz.value, dtype=np.int32)
        val = np.empty(25 * nnz.value)
        b = np.empty(5 * n)
        self._check(self.L.semo_get_coupled_system(self.h, ptr.ctypes.data_as(C.POINTER(C.c_int32)),
                                                   col.ctypes.data_as(C.POINTER(C.c_int32)),
                                                   val.ctypes.data_as(C.POINTER(C.c_double)),
                                                   b.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nnz)))
        return {"ptr": ptr, "col": col, "val": val.reshape(-1, 5, 5), "b": b.reshape(5, n)}

    def solve_coupled(self) -> SolveResult:
        x = np.empty(5 * self.n_cells)
        info = SolveInfo()
        self._check(self.L.semo_solve_coupled(self.h, x.ctypes.data_as(C.POINTER(C.c_double)), C.byref(info)))
        return SolveResult(x=x, info=info.as_dict())

    def calc_comp_coupled_eq(self) -> tuple:
        """One calcCompCoupledEq: assemble, solve, update p, U, T; (norm, info)."""
        norm = C.c_double()
        info = SolveInfo()
        self._check(self.L.semo_coupled_pass(self.h, C.byref(norm), C.byref(info)))
        return norm.value, info.as_dict()

    def assemble_momentum(self) -> None:
        self._check(self.L.semo_assemble_momentum(self.h))

    def momentum_system(self) -> dict:
        """The momentum system in SEMO's layout (caller numbering, COO-scatter rows)."""
        n = self.n_cells
        nnz = C.c_int64()
        self._check(self.L.semo_get_momentum_system(self.h, None, None, None, None, C.byref(nnz)))
        ptr = np.empty(n + 1, dtype=np.int32)
        col = np.empty(nnz.value, dtype=np.int32)
        val = np.empty(nnz.value)
        b = np.empty(3 * n)
        self._check(self.L.semo_get_momentum_system(self.h, ptr.ctypes.data_as(C.POINTER(C.c_int32)),
                                                    col.ctypes.data_as(C.POINTER(C.c_int32)),
                                                    val.ctypes.data_as(C.POINTER(C.c_double)),
                                                    b.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nnz)))
        return {"ptr": ptr, "col": col, "val": val, "b": b.reshape(3, n)}

    def solve_momentum(self) -> tuple:
        """Solve the assembled momentum system: (x of shape (3, n), [3 infos])."""
        x = np.empty(3 * self.n_cells)
        info = (SolveInfo * 3)()
        self._check(self.L.semo_solve_momentum(self.h, x.ctypes.data_as(C.POINTER(C.c_double)), info))
        return x.reshape(3, self.n_cells), [i.as_dict() for i in info]

    def lib_rcm(self) -> tuple:
        """lib_RCM: (perm, iperm) = (cells[i].RCM, cells[i].invRCM)."""
        perm = np.empty(self.n_cells, dtype=np.int32)
        iperm = np.empty(self.n_cells, dtype=np.int32)
        self._check(self.L.semo_rcm(self.h, perm.ctypes.data_as(C.POINTER(C.c_int32)),
                                    iperm.ctypes.data_as(C.POINTER(C.c_int32))))
        return perm, iperm

    def solve_amgcl(self, equation: str, B_n: int, A_rows, A_cols, A_vals, *args):
        """solveAMGCL with SEMO's argument lists (src/solvers/build.h:225-239).

        solve_amgcl("pressure", 1, rows, cols, vals, B[, resiVar]): AMG-CG
        (semo_solve_coo); solve_amgcl("volume_fraction", 1, rows, cols, vals,
        B[, resiVar]): BiCGStab (semo_solve_coo_multi, one right-hand side);
        solve_amgcl("momentum", 1, rows, cols, vals, B0, B1, B2[, resiVar0,
        resiVar1, resiVar2]): the three-right-hand-side overload, returns a
        list of three SolveResult.  resiVar is the initial guess (zeros when
        left out)."""
        if B_n != 1:
            raise SemoError(1, "only scalar systems (B_n == 1) have a live SEMO caller; the 5x5 coupled system "
                               "goes through semo_solve_coupled")
        r, rp = _i32(A_rows)
        c, cp = _i32(A_cols)
        v, vp = _f64(A_vals)
        if equation in ("pressure", "volume_fraction"):
            if len(args) not in (1, 2):
                raise SemoError(1, f"solveAMGCL('{equation}') takes B and optionally resiVar")
            B = args[0]
            n = len(B)
            x = np.zeros(n) if len(args) == 1 or args[1] is None else np.array(args[1], dtype=np.float64)
            b, bp = _f64(B)
            if equation == "pressure":
                info = SolveInfo()
                self._check(self.L.semo_solve_coo(self.h, n, len(r), rp, cp, vp, bp,
                                                  x.ctypes.data_as(C.POINTER(C.c_double)), C.byref(info)))
                return SolveResult(x=x, info=info.as_dict())
            info = (SolveInfo * 1)()
            self._check(self.L.semo_solve_coo_multi(self.h, 1, n, len(r), rp, cp, vp, bp,
                                                    x.ctypes.data_as(C.POINTER(C.c_double)), info))
            return SolveResult(x=x, info=info[0].as_dict())
        if equation == "momentum":
            if len(args) not in (3, 6):
                raise SemoError(1, "solveAMGCL('momentum') takes B0, B1, B2 and optionally three resiVar")
            n = len(args[0])
            b = np.ascontiguousarray(np.concatenate([np.asarray(a, dtype=np.float64) for a in args[:3]]))
            x = (np.zeros(3 * n) if len(args) == 3
                 else np.ascontiguousarray(np.concatenate([np.asarray(a, dtype=np.float64) for a in args[3:]])))
            info = (SolveInfo * 3)()
            self._check(self.L.semo_solve_coo_multi(self.h, 3, n, len(r), rp, cp, vp,
                                                    b.ctypes.data_as(C.POINTER(C.c_double)),
                                                    x.ctypes.data_as(C.POINTER(C.c_double)), info))
            return [SolveResult(x=x[j * n:(j + 1) * n].copy(), info=info[j].as_dict()) for j in range(3)]
        raise SemoError(1, f"equation '{equation}' is not on this path")

    # ---- pieces ----------------------------------------------------------
    def assemble(self) -> None:
        self._check(self.L.semo_assemble_pressure(self.h))

    def system_rcm(self) -> dict:
        n = self.n_cells
        nnz = n + 2 * self.mesh.n_internal
        ptr = np.empty(n + 1, dtype=np.int32)
        col = np.empty(nnz, dtype=np.int32)
        val = np.empty(nnz)
        b = np.empty(n)
        self._check(self.L.semo_get_system_rcm(self.h, ptr.ctypes.data_as(C.POINTER(C.c_int32)),
                                               col.ctypes.data_as(C.POINTER(C.c_int32)),
                                               val.ctypes.data_as(C.POINTER(C.c_double)),
                                               b.ctypes.data_as(C.POINTER(C.c_double))))
        return {"ptr": ptr, "col": col, "val": val, "b": b}

    EQUATIONS = {"pressure": 0, "momentum": 1, "volume_fraction": 2, "coupled": 3}

    def system_rcm_eq(self, equation: str) -> dict:
        """An assembled system in RCM order on the mesh's CSR pattern (dropped
        momentum / volume-fraction entries as 0.0; 5x5 blocks for "coupled")."""
        eq = self.EQUATIONS[equation]
        n = self.n_cells
        nnz = n + 2 * self.mesh.n_internal
        per, planes = (25, 5) if eq == 3 else (1, 3 if eq == 1 else 1)
        ptr = np.empty(n + 1, dtype=np.int32)
        col = np.empty(nnz, dtype=np.int32)
        val = np.empty(per * nnz)
        b = np.empty(planes * n)
        self._check(self.L.semo_get_system_rcm_eq(self.h, eq, ptr.ctypes.data_as(C.POINTER(C.c_int32)),
                                                  col.ctypes.data_as(C.POINTER(C.c_int32)),
                                                  val.ctypes.data_as(C.POINTER(C.c_double)),
                                                  b.ctypes.data_as(C.POINTER(C.c_double))))
        return {"ptr": ptr, "col": col, "val": val.reshape(-1, 5, 5) if eq == 3 else val,
                "b": b.reshape(planes, n) if planes > 1 else b}

    def solve(self) -> SolveResult:
        x = np.empty(self.n_cells)
        info = SolveInfo()
        self._check(self.L.semo_solve_pressure(self.h, x.ctypes.data_as(C.POINTER(C.c_double)), C.byref(info)))
        return SolveResult(x=x, info=info.as_dict())

    def get_array(self, name: str, count: int) -> np.ndarray:
        out = np.empty(count)
        self._check(self.L.semo_get_array(self.h, name.encode(), out.ctypes.data_as(C.POINTER(C.c_double)), count))
        return out

    # ---- measurement hooks -------------------------------------------------
    STAGES = ("face_values", "gravity", "stencil", "pface", "pbface", "pcell", "amg_setup", "pcg",
              "gauss_green", "update", "vcycle", "setup_aggregate", "setup_prolong", "setup_galerkin",
              "setup_level", "setup_coarse", "mface", "mcell", "msolve", "mupdate", "mstacs", "vface",
              "vsolve", "vupdate", "stencil_uvw", "mbface", "cgrad", "cface", "ccell", "csolve", "cupdate",
              "surface_tension", "setup_cycle")

    def set_profiling(self, on: bool) -> None:
        self.L.semo_set_profiling(self.h, 1 if on else 0)

    def reset_stats(self) -> None:
        self._check(self.L.semo_reset_stats(self.h))

    def stage_times(self) -> dict:
        out = {}
        for st in self.STAGES:
            ms = C.c_double()
            n = C.c_int64()
            self._check(self.L.semo_stage_time(self.h, st.encode(), C.byref(ms), C.byref(n)))
            out[st] = (ms.value, n.value)
        return out

    def kernel_launches(self) -> int:
        return int(self.L.semo_kernel_launches())

    def mesh_info(self) -> dict:
        out = (C.c_int64 * 6)()
        self._check(self.L.semo_mesh_info(self.h, out))
        keys = ("cells", "faces", "internal_faces", "boundary_faces", "stencil_nnz", "nnz")
        return {k: int(v) for k, v in zip(keys, out)}

    def time_spmv(self, which: int, reps: int = 20) -> float:
        """ms per y = A x launch on the last pressure hierarchy: which 0 the
        finest V-cycle operator (its layout and precision), 1 the FP64 outer one."""
        ms = C.c_double()
        self._check(self.L.semo_time_spmv(self.h, int(which), int(reps), C.byref(ms)))
        return ms.value

    def hierarchy_levels(self) -> list:
        """Per level of the last pressure hierarchy: rows, nnz of A, P and R,
        the V-cycle layout of A and the value bytes."""
        out = (C.c_int64 * (6 * 64))()
        nl = C.c_int()
        self._check(self.L.semo_hierarchy_levels(self.h, out, 64, C.byref(nl)))
        keys = ("rows", "nnz_A", "nnz_P", "nnz_R", "layout", "value_bytes")
        return [{k: int(out[6 * l + j]) for j, k in enumerate(keys)} for l in range(nl.value)]

    def vjp_fields(self, dJ_dx) -> tuple:
        """lambda = A^-T dJ/dx and dJ/d(U, V, W, P) through the pressure
        equation's face-flux right-hand side (a dict of four arrays)."""
        g, gp = _f64(dJ_dx)
        out = {k: np.empty(self.n_cells) for k in ("lambda", "U", "V", "W", "P")}
        ptr = [out[k].ctypes.data_as(C.POINTER(C.c_double)) for k in ("lambda", "U", "V", "W", "P")]
        info = SolveInfo()
        self._check(self.L.semo_vjp_fields(self.h, gp, *ptr, C.byref(info)))
        lam = out.pop("lambda")
        return lam, out, info.as_dict()

    def vjp_source(self, dJ_dx) -> tuple:
        """lambda = A^-T dJ/dx and dJ/ds (s entering as b_i += s_i V_i)."""
        g, gp = _f64(dJ_dx)
        lam = np.empty(self.n_cells)
        djds = np.empty(self.n_cells)
        info = SolveInfo()
        self._check(self.L.semo_vjp_source(self.h, gp, lam.ctypes.data_as(C.POINTER(C.c_double)),
                                           djds.ctypes.data_as(C.POINTER(C.c_double)), C.byref(info)))
        return lam, djds, info.as_dict()
