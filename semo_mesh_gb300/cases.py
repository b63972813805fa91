"""Seeded synthetic cases for the pressure-correction hot path.

No public dataset is involved: the cases are the shapes and value
distributions of the workloads this library is measured on.

* ``box``      -- hex box, velocity i.i.d. uniform[-1,1] per component
                  (seed 1), one phase of density 1 and viscosity 1e-3, p = 0,
                  dt = 1, no gravity.
* ``vof``      -- jittered hex box with a water drop in air:
                  alpha = 0.5*(1 - tanh((|x - c| - 0.25)/0.01)), c the cube
                  centre; rho 1000 / 1.2, mu 1e-3 / 1.8e-5, g = (0,0,-9.81),
                  velocity i.i.d. uniform[-1,1] (seed 1), dt = 1e-4.

Boundary conditions in both: pressure fixedValue 0 on ``zmax`` and
zeroGradient elsewhere; velocity and volume fraction zeroGradient.  Pressure
and velocity under-relaxation are 0.3 (the reference's fvSolution defaults).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .meshgen import PolyMesh, hex_box, tet_box

# boundary-condition codes shared with the C-ABI (include/semo_gb300.h)
BC_ZERO_GRADIENT = 0
BC_FIXED_VALUE = 1
BC_NO_SLIP = 2
BC_SLIP = 3


@dataclass
class Case:
    name: str
    mesh: PolyMesh
    P: np.ndarray
    U: np.ndarray
    V: np.ndarray
    W: np.ndarray
    VF: np.ndarray
    # per patch: (type_p, type_u, type_vf), (val_p, val_u, val_v, val_w, val_vf)
    bc_type: np.ndarray = None      # (n_patches, 3) int32
    bc_value: np.ndarray = None     # (n_patches, 5) float64
    dt: float = 1.0
    rho: tuple = (1.0, 1.0)         # (phase 0 = VF[0], phase 1)
    mu: tuple = (1e-3, 1e-3)
    sigma: float = 0.0
    gravity: tuple = (0.0, 0.0, 0.0)
    use_gravity: bool = False
    pre_p_urf: float = 0.3
    pre_u_urf: float = 0.3
    mom_u_urf: float = 0.3          # momentumEq U relaxation (fvSolution default)
    vof_urf: float = 0.3            # speciesEq VF relaxation (fvSolution default)
    # BDF2 history for the momentum equation: (U, V, W) at steps n-1 and n-2;
    # None means "same as the current field" (the first step of a run)
    old: tuple = None
    old2: tuple = None
    old_vf: np.ndarray = None       # VF at steps n-1 and n-2 (None: the current VF)
    old2_vf: np.ndarray = None
    extra: dict = field(default_factory=dict)

    def vf_history(self):
        """(oldVF, old2VF), defaulting to the current VF."""
        o = self.old_vf if self.old_vf is not None else self.VF
        o2 = self.old2_vf if self.old2_vf is not None else self.VF
        return tuple(np.ascontiguousarray(a, dtype=np.float64) for a in (o, o2))

    def history(self):
        """(oldU, oldV, oldW, old2U, old2V, old2W), defaulting to the current velocity."""
        cur = (self.U, self.V, self.W)
        o = self.old if self.old is not None else cur
        o2 = self.old2 if self.old2 is not None else cur
        return tuple(np.ascontiguousarray(a, dtype=np.float64) for a in (*o, *o2))


def approx_cell_centres(mesh: PolyMesh) -> np.ndarray:
    """Mean of each cell's face-loop vertex means (used only to place fields)."""
    nf = mesh.n_faces
    cnt = np.diff(mesh.face_ptr).astype(np.int64)
    fid = np.repeat(np.arange(nf), cnt)
    fc = np.zeros((nf, 3))
    np.add.at(fc, fid, mesh.points[mesh.face_pts])
    fc /= cnt[:, None]
    cc = np.zeros((mesh.n_cells, 3))
    nc = np.zeros(mesh.n_cells)
    np.add.at(cc, mesh.owner, fc)
    np.add.at(nc, mesh.owner, 1.0)
    ni = mesh.n_internal
    np.add.at(cc, mesh.neighbour, fc[:ni])
    np.add.at(nc, mesh.neighbour, 1.0)
    return cc / nc[:, None]


def _default_bcs(mesh: PolyMesh):
    npatch = len(mesh.patch_names)
    bt = np.zeros((npatch, 3), dtype=np.int32)
    bv = np.zeros((npatch, 5), dtype=np.float64)
    bt[mesh.patch_names.index("zmax"), 0] = BC_FIXED_VALUE
    return bt, bv


def _velocity(n_cells: int, seed: int = 1):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1.0, 1.0, size=(3, n_cells))
    return u[0].copy(), u[1].copy(), u[2].copy()


def box_case(n: int, jitter: float = 0.0, mesh_seed: int = 1234) -> Case:
    mesh = hex_box(n, jitter=jitter, seed=mesh_seed)
    U, V, W = _velocity(mesh.n_cells, 1)
    bt, bv = _default_bcs(mesh)
    nc = mesh.n_cells
    return Case(name=f"box{n}" + ("j" if jitter else ""), mesh=mesh, P=np.zeros(nc), U=U, V=V, W=W,
                VF=np.ones(nc), bc_type=bt, bc_value=bv, dt=1.0, rho=(1.0, 1.0), mu=(1e-3, 1e-3))


def vof_case(n: int, jitter: float = 0.2, mesh_seed: int = 1234) -> Case:
    mesh = hex_box(n, jitter=jitter, seed=mesh_seed)
    U, V, W = _velocity(mesh.n_cells, 1)
    cc = approx_cell_centres(mesh)
    r = np.linalg.norm(cc - 0.5, axis=1)
    alpha = 0.5 * (1.0 - np.tanh((r - 0.25) / 0.01))
    bt, bv = _default_bcs(mesh)
    return Case(name=f"vof{n}", mesh=mesh, P=np.zeros(mesh.n_cells), U=U, V=V, W=W, VF=alpha,
                bc_type=bt, bc_value=bv, dt=1e-4, rho=(1000.0, 1.2), mu=(1e-3, 1.8e-5),
                gravity=(0.0, 0.0, -9.81), use_gravity=True)


def with_history(case: Case, seed: int, scale: float = 0.1) -> Case:
    """Seeded old / second-old velocities near the current one (exercises BDF2)."""
    rng = np.random.default_rng(seed)
    n = case.mesh.n_cells
    cur = (case.U, case.V, case.W)
    case.old = tuple(c + scale * rng.uniform(-1.0, 1.0, size=n) for c in cur)
    case.old2 = tuple(c + scale * rng.uniform(-1.0, 1.0, size=n) for c in cur)
    return case


def with_vf_history(case: Case, seed: int, scale: float = 0.05) -> Case:
    """Seeded old / second-old volume fractions near the current one, in [0, 1]."""
    rng = np.random.default_rng(seed)
    n = case.mesh.n_cells
    case.old_vf = np.clip(case.VF + scale * rng.uniform(-1.0, 1.0, size=n), 0.0, 1.0)
    case.old2_vf = np.clip(case.VF + scale * rng.uniform(-1.0, 1.0, size=n), 0.0, 1.0)
    return case


def with_fields(case: Case, seed: int, p_scale: float = 1.0) -> Case:
    """Same mesh, extra seeded randomness in P (exercises the pressure terms)."""
    rng = np.random.default_rng(seed)
    case.P = p_scale * rng.uniform(-1.0, 1.0, size=case.mesh.n_cells)
    return case


# ---------------------------------------------------------------------------
# compressible coupled (p, U, T) cases
# ---------------------------------------------------------------------------
@dataclass
class CoupledCase:
    """Ideal-gas fields for the 5x5 block-coupled system.

    ``bc_type`` per patch holds (type_p, type_u, type_T) with the codes above;
    ``bc_value`` per patch (p, u, v, w, T).  ``old`` / ``old2`` are the
    primitives (P, U, V, W, T) at steps n-1 and n-2, shape (5, n_cells).
    """
    name: str
    mesh: PolyMesh
    P: np.ndarray
    U: np.ndarray
    V: np.ndarray
    W: np.ndarray
    T: np.ndarray
    old: np.ndarray
    old2: np.ndarray
    bc_type: np.ndarray
    bc_value: np.ndarray
    cv: float = 717.5               # R / (gamma - 1) with R = 287
    gamma: float = 1.4
    mu: float = 1.8e-5
    dt: float = 1e-5
    dt_old: float = 1e-5
    dt_old2: float = 1e-5
    gravity: tuple = (0.0, 0.0, 0.0)
    urf: float = 1.0
    # update clamps (min, max) for P, U, V, W, T
    limits: np.ndarray = field(default_factory=lambda: np.array(
        [1.0, 1e12, -1e6, 1e6, -1e6, 1e6, -1e6, 1e6, 1.0, 1e5], dtype=np.float64))

    def history(self):
        return (np.ascontiguousarray(self.old, dtype=np.float64).reshape(-1),
                np.ascontiguousarray(self.old2, dtype=np.float64).reshape(-1))


def _face_smooth(mesh: PolyMesh, phi: np.ndarray, passes: int) -> np.ndarray:
    """``passes`` rounds of face-neighbour averaging: phi_i <- (phi_i + sum_j phi_j) / (1 + n_i)."""
    o = mesh.owner[:mesh.n_internal].astype(np.int64)
    q = mesh.neighbour.astype(np.int64)
    cnt = np.ones(mesh.n_cells)
    np.add.at(cnt, o, 1.0)
    np.add.at(cnt, q, 1.0)
    for _ in range(passes):
        s = phi.copy()
        np.add.at(s, o, phi[q])
        np.add.at(s, q, phi[o])
        phi = s / cnt
    return phi


def coupled_case(n: int, tets: bool = True, jitter: float = 0.2, mesh_seed: int = 1234,
                 history_scale: float = 1e-3) -> CoupledCase:
    """Ideal gas on a jittered box (6 tetrahedra per hex by default).

    p = 1e5 + 1e3 * (N(0,1), seed 2, smoothed by 3 face-neighbour averaging
    passes), T = 300 + uniform[-5, 5] (seed 4), velocity uniform[-50, 50] per
    component (seed 3), dt = 1e-5.  Walls all round: p and T zeroGradient,
    velocity noSlip.  The step n-1 and n-2 primitives are the current ones
    scaled by 1 +- ``history_scale`` (seeds 5, 6), which exercises the
    bounded BDF2.
    """
    mesh = tet_box(n, jitter=jitter, seed=mesh_seed) if tets else hex_box(n, jitter=jitter, seed=mesh_seed)
    nc = mesh.n_cells
    rng = np.random.default_rng(2)
    P = 1e5 + 1e3 * _face_smooth(mesh, rng.standard_normal(nc), 3)
    rng = np.random.default_rng(3)
    u = rng.uniform(-50.0, 50.0, size=(3, nc))
    rng = np.random.default_rng(4)
    T = 300.0 + rng.uniform(-5.0, 5.0, size=nc)
    cur = np.stack([P, u[0], u[1], u[2], T])
    hist = []
    for sd in (5, 6):
        r = np.random.default_rng(sd)
        hist.append(cur * (1.0 + history_scale * r.uniform(-1.0, 1.0, size=cur.shape)))
    npatch = len(mesh.patch_names)
    bt = np.zeros((npatch, 3), dtype=np.int32)
    bt[:, 1] = BC_NO_SLIP
    bv = np.zeros((npatch, 5), dtype=np.float64)
    return CoupledCase(name=("tet" if tets else "hex") + f"{n}c", mesh=mesh, P=P, U=u[0].copy(), V=u[1].copy(),
                       W=u[2].copy(), T=T, old=hist[0], old2=hist[1], bc_type=bt, bc_value=bv)
