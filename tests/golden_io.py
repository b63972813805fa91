"""Load the committed golden fixtures (made by tests/golden/make_golden.py)."""
import glob
import os

import numpy as np

from semo_mesh_gb300.cases import Case
from semo_mesh_gb300.meshgen import PATCH_NAMES, PolyMesh

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _all():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def names():
    """Fixtures of one pressure-correction pass."""
    return [n for n in _all() if not n.startswith(("outer_", "vofeq_", "foam_"))]


def outer_names():
    """Fixtures of a whole outer iteration: momentum equation, then pressure correction."""
    return [n for n in _all() if n.startswith("outer_")]


def vofeq_names():
    """Fixtures of one volume-fraction sub-iteration (MSTACS + calcVolfracEq)."""
    return [n for n in _all() if n.startswith("vofeq_")]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    mesh = PolyMesh(points=z["points"], face_ptr=z["face_ptr"], face_pts=z["face_pts"], owner=z["owner"],
                    neighbour=z["neighbour"], n_cells=int(z["n_cells"]), patch_names=list(PATCH_NAMES),
                    patch_start=z["patch_start"], patch_size=z["patch_size"])
    p = z["params"]
    case = Case(name=name, mesh=mesh, P=z["P"].copy(), U=z["U"].copy(), V=z["V"].copy(), W=z["W"].copy(),
                VF=z["VF"].copy(), bc_type=z["bc_type"].copy(), bc_value=z["bc_value"].copy(), dt=float(p[0]),
                rho=(float(p[1]), float(p[2])), mu=(float(p[3]), float(p[4])), sigma=float(p[5]),
                gravity=(float(p[6]), float(p[7]), float(p[8])), use_gravity=bool(p[11]),
                pre_p_urf=float(p[9]), pre_u_urf=float(p[10]))
    if p.size > 12:
        case.mom_u_urf = float(p[12])
    if p.size > 14:
        case.vof_urf = float(p[14])
    if "vf_history" in z.files:
        h = z["vf_history"]
        case.old_vf, case.old2_vf = h[0].copy(), h[1].copy()
    if "history" in z.files:
        h = z["history"]
        case.old = (h[0].copy(), h[1].copy(), h[2].copy())
        case.old2 = (h[3].copy(), h[4].copy(), h[5].copy())
    ref = {k[4:]: z[k] for k in z.files if k.startswith("ref_")}
    return case, ref
