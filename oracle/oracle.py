"""ctypes binding of the CPU checker (oracle/semo_oracle.c).

Test infrastructure: used by tests/, __graft_entry__.smoke() and the CPU
baseline legs of bench.py only.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "semo_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               "-o", LIB, SRC, "-lm"]
        subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        vp = C.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.c_int, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, C.c_int, vp, vp]
        L.orc_destroy.argtypes = [vp]
        L.orc_len.restype = C.c_longlong
        L.orc_len.argtypes = [vp, C.c_char_p]
        L.orc_type.argtypes = [vp, C.c_char_p]
        L.orc_get.argtypes = [vp, C.c_char_p, vp]
        L.orc_set.argtypes = [vp, C.c_char_p, C.c_int, C.c_longlong, vp]
        L.orc_set_case.argtypes = [vp, vp, vp, vp]
        L.orc_assemble_pressure.argtypes = [vp]
        L.orc_coo_to_csr.argtypes = [vp]
        L.orc_permute_csr.argtypes = [vp]
        L.orc_solve.restype = C.c_int
        L.orc_solve.argtypes = [vp, C.c_int, C.c_double, C.c_int, vp]
        L.orc_update.restype = C.c_double
        L.orc_update.argtypes = [vp, vp]
        L.orc_assemble_momentum.argtypes = [vp]
        L.orc_solve_momentum.restype = C.c_int
        L.orc_solve_momentum.argtypes = [vp, C.c_int, C.c_double, C.c_int, vp, vp]
        L.orc_update_momentum.restype = C.c_double
        L.orc_update_momentum.argtypes = [vp, vp, vp, vp]
        L.orc_assemble_vof.argtypes = [vp]
        L.orc_solve_vof.restype = C.c_int
        L.orc_solve_vof.argtypes = [vp, C.c_double, C.c_int, vp, vp]
        L.orc_update_vof.restype = C.c_double
        L.orc_update_vof.argtypes = [vp, vp]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_smoother.argtypes = [C.c_int]
        L.orc_set_coupled.argtypes = [vp, vp, vp, vp]
        L.orc_curvature.argtypes = [vp]
        L.orc_surface_tension.argtypes = [vp, C.c_double]
        L.orc_coupled_terms.argtypes = [C.c_int]
        L.orc_assemble_coupled.argtypes = [vp]
        L.orc_coupled_bsr.argtypes = [vp, vp]
        L.orc_solve_coupled.restype = C.c_int
        L.orc_solve_coupled.argtypes = [vp, C.c_double, C.c_int, vp, vp]
        L.orc_update_coupled.restype = C.c_double
        L.orc_update_coupled.argtypes = [vp, vp, vp]
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """The reference's pressure pass restated on the CPU, for one mesh."""

    def __init__(self, mesh):
        L = lib()
        self._keep = [np.ascontiguousarray(mesh.points, dtype=np.float64),
                      np.ascontiguousarray(mesh.face_ptr, dtype=np.int32),
                      np.ascontiguousarray(mesh.face_pts, dtype=np.int32),
                      np.ascontiguousarray(mesh.owner, dtype=np.int32),
                      np.ascontiguousarray(mesh.neighbour, dtype=np.int32),
                      np.ascontiguousarray(mesh.patch_start, dtype=np.int32),
                      np.ascontiguousarray(mesh.patch_size, dtype=np.int32)]
        k = self._keep
        self.mesh = mesh
        self.h = L.orc_create(mesh.n_points, _p(k[0]), mesh.n_faces, mesh.n_internal, mesh.n_cells,
                              _p(k[1]), _p(k[2]), _p(k[3]), _p(k[4]), len(mesh.patch_names), _p(k[5]), _p(k[6]))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def get(self, name: str) -> np.ndarray:
        L = lib()
        n = L.orc_len(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        t = L.orc_type(self.h, name.encode())
        out = np.empty(n, dtype=np.float64 if t == 0 else np.int32)
        L.orc_get(self.h, name.encode(), _p(out))
        return out

    def set(self, name: str, arr: np.ndarray) -> None:
        if arr.dtype == np.int32:
            a = np.ascontiguousarray(arr)
            lib().orc_set(self.h, name.encode(), 1, a.size, _p(a))
        else:
            a = np.ascontiguousarray(arr, dtype=np.float64)
            lib().orc_set(self.h, name.encode(), 0, a.size, _p(a))

    def set_case(self, case) -> None:
        bt = np.ascontiguousarray(case.bc_type, dtype=np.int32)
        bv = np.ascontiguousarray(case.bc_value, dtype=np.float64)
        prm = np.zeros(16)
        prm[:12] = [case.dt, case.rho[0], case.rho[1], case.mu[0], case.mu[1], case.sigma,
                    case.gravity[0], case.gravity[1], case.gravity[2], case.pre_p_urf, case.pre_u_urf,
                    1.0 if case.use_gravity else 0.0]
        prm[12] = case.mom_u_urf
        prm[13] = case.vof_urf
        lib().orc_set_case(self.h, _p(bt), _p(bv), _p(prm))
        for nm in ("P", "U", "V", "W", "VF"):
            self.set(nm, getattr(case, nm))
        for nm, a in zip(("oldU", "oldV", "oldW", "old2U", "old2V", "old2W"), case.history()):
            self.set(nm, a)
        for nm, a in zip(("oldVF", "old2VF"), case.vf_history()):
            self.set(nm, a)
        if case.sigma != 0.0:
            # curvature and source from the case's fields, once per pass
            # (src/solvers/pressureBased.cpp:142)
            self.surface_tension(case.sigma)

    def assemble(self) -> None:
        lib().orc_assemble_pressure(self.h)
        lib().orc_coo_to_csr(self.h)
        lib().orc_permute_csr(self.h)

    def solve(self, use_rcm: bool = False, tol: float = 1e-8, maxiter: int = 500,
              smoother: str = "chebyshev") -> dict:
        """SA-AMG CG on the assembled system; smoother "chebyshev" or
        "gauss_seidel" (multicolour, the GPU's colouring and sweep order)."""
        info = np.zeros(16)
        lib().orc_set_smoother(1 if smoother == "gauss_seidel" else 0)
        try:
            it = lib().orc_solve(self.h, 1 if use_rcm else 0, tol, maxiter, _p(info))
        finally:
            lib().orc_set_smoother(0)
        if it < 0:
            raise RuntimeError("oracle AMG setup failed")
        x = self.get("rcm_x_orc" if use_rcm else "x_orc")
        nlev = int(info[2])
        return {"x": x, "iters": int(info[0]), "rel_res": float(info[1]), "levels": nlev,
                "operator_complexity": float(info[3]), "coarse_n": int(info[4]),
                "level_sizes": [int(v) for v in info[5:5 + min(nlev, 10)]]}

    def update(self, x: np.ndarray) -> float:
        xa = np.ascontiguousarray(x, dtype=np.float64)
        return float(lib().orc_update(self.h, _p(xa)))

    def assemble_momentum(self) -> None:
        """calcMomentumEqs assembly: COO (mom_A_*), CSR (mom_csr_*), RHS planes mom_B."""
        lib().orc_assemble_momentum(self.h)

    def solve_momentum(self, tol: float = 1e-9, maxiter: int = 1000) -> dict:
        """Jacobi-BiCGStab on each of the three right-hand sides (x0 = 0)."""
        n = self.mesh.n_cells
        xs, its, res = [], [], []
        for j in range(3):
            x = np.empty(n)
            rr = np.zeros(1)
            its.append(int(lib().orc_solve_momentum(self.h, j, tol, maxiter, _p(x), _p(rr))))
            xs.append(x)
            res.append(float(rr[0]))
        return {"x": xs, "iters": its, "rel_res": res}

    def update_momentum(self, xs) -> float:
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in xs]
        return float(lib().orc_update_momentum(self.h, _p(a[0]), _p(a[1]), _p(a[2])))

    def momentum_pass(self, tol: float = 1e-9) -> dict:
        """One calcMomentumEqs: assemble, solve the three components, update U, V, W."""
        self.assemble_momentum()
        sol = self.solve_momentum(tol)
        sol["norm"] = self.update_momentum(sol["x"])
        return sol

    def assemble_vof(self) -> None:
        """MSTACS face values + calcVolfracEq assembly: vof_A_*, vof_csr_*, vof_B, vof_face_vf{L,R}."""
        lib().orc_assemble_vof(self.h)

    def solve_vof(self, tol: float = 1e-9, maxiter: int = 1000) -> dict:
        x = np.empty(self.mesh.n_cells)
        rr = np.zeros(1)
        it = int(lib().orc_solve_vof(self.h, tol, maxiter, _p(x), _p(rr)))
        return {"x": x, "iters": it, "rel_res": float(rr[0])}

    def update_vof(self, x) -> float:
        xa = np.ascontiguousarray(x, dtype=np.float64)
        return float(lib().orc_update_vof(self.h, _p(xa)))

    def vof_pass(self, tol: float = 1e-9) -> dict:
        """One volume-fraction sub-iteration: reconstruct, assemble, solve, update VF."""
        self.assemble_vof()
        sol = self.solve_vof(tol)
        sol["norm"] = self.update_vof(sol["x"])
        return sol

    def pressure_pass(self, case, tol: float = 1e-8) -> dict:
        """One full calcPressureEq: assemble, solve, Gauss-Green, update."""
        self.set_case(case)
        self.assemble()
        sol = self.solve(False, tol)
        norm = self.update(sol["x"])
        sol["norm"] = norm
        return sol

    def surface_tension(self, sigma: float) -> None:
        """Curvature (kappa, ls) and the surface-tension source (src_sft, 4 per cell)."""
        lib().orc_surface_tension(self.h, float(sigma))

    # ---- compressible coupled 5x5 block system --------------------------------
    def set_coupled(self, case) -> None:
        """Fields, history, physics and boundary conditions of a CoupledCase."""
        prm = np.array([case.cv, case.gamma, case.mu, case.dt, case.dt_old, case.dt_old2,
                        case.gravity[0], case.gravity[1], case.gravity[2], case.urf], dtype=np.float64)
        bt = np.ascontiguousarray(case.bc_type, dtype=np.int32)
        bv = np.ascontiguousarray(case.bc_value, dtype=np.float64)
        lib().orc_set_coupled(self.h, _p(prm), _p(bt), _p(bv))
        for nm in ("P", "U", "V", "W", "T"):
            self.set("cpl_" + nm, getattr(case, nm))
        o, o2 = case.history()
        self.set("cpl_old", o)
        self.set("cpl_old2", o2)

    def assemble_coupled(self, terms: int = 7) -> None:
        """cpl_diag (25 per cell), cpl_LR / cpl_RL (25 per internal face), cpl_B (field-split).

        ``terms`` picks the parts added: 1 cell terms, 2 internal faces, 4
        boundary faces (tests take the system apart with it)."""
        lib().orc_coupled_terms(int(terms))
        try:
            lib().orc_assemble_coupled(self.h)
        finally:
            lib().orc_coupled_terms(7)

    def coupled_bsr(self):
        """(ptr, col, val[nnz, 5, 5]) on the scalar pattern, caller cell order."""
        ptr = self.get("CRS_ptr"); col = self.get("CRS_col")
        val = np.empty(25 * int(ptr[-1]))
        lib().orc_coupled_bsr(self.h, _p(val))
        return ptr, col, val.reshape(-1, 5, 5)

    def solve_coupled(self, tol: float = 1e-12, maxiter: int = 5000) -> dict:
        x = np.empty(5 * self.mesh.n_cells)
        rr = np.zeros(1)
        it = int(lib().orc_solve_coupled(self.h, tol, maxiter, _p(x), _p(rr)))
        return {"x": x, "iters": it, "rel_res": float(rr[0])}

    def update_coupled(self, x, limits) -> float:
        xa = np.ascontiguousarray(x, dtype=np.float64)
        la = np.ascontiguousarray(limits, dtype=np.float64)
        return float(lib().orc_update_coupled(self.h, _p(xa), _p(la)))

    @staticmethod
    def threads() -> int:
        return int(lib().orc_num_threads())
