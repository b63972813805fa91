"""Generate the golden fixtures in this folder from the reference's own code.

Builds oracle/_ref/semo_ref from the reference sources (oracle/ref/Makefile),
runs it on small seeded cases and stores inputs and every dumped intermediate
as .npz.  The fixtures are committed so the parity tests need neither the
reference tree nor its build.  Fixtures named outer_* hold a whole outer
iteration (momentum equation, then the pressure correction) with seeded old
and second-old velocities for the BDF2 term; fixtures named vofeq_* hold one
volume-fraction sub-iteration (MSTACS reconstruction + calcVolfracEq) with
seeded old and second-old volume fractions.  Names ending in "s" carry a
surface tension (sigma != 0): the reference then computes the curvature and
the surface-tension source first and every face velocity takes its terms.
foam_* are OpenFOAM polyMesh
directories written from seeded meshes, with foam_*_ref.npz holding what the
reference's own loader (SEMO_Mesh_Load::OpenFoam) read from them.

    python tests/golden/make_golden.py [REF_DIR] [--foam-only | --only NAME ...]
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from semo_mesh_gb300.cases import (box_case, vof_case, with_fields, with_history, with_vf_history,  # noqa: E402
                                   BC_FIXED_VALUE, BC_NO_SLIP, BC_SLIP)
from oracle.refcase import run_reference  # noqa: E402


def golden_cases():
    cs = []
    cs.append(("box4", box_case(4)))
    cs.append(("box5j", box_case(5, jitter=0.2)))
    cs.append(("vof6", vof_case(6)))
    c = with_fields(vof_case(5), seed=7, p_scale=50.0)
    c.name = "vof5p"
    # a second Dirichlet patch with a non-zero value exercises the boundary terms
    c.bc_type[c.mesh.patch_names.index("xmin"), 0] = BC_FIXED_VALUE
    c.bc_value[c.mesh.patch_names.index("xmin"), 0] = 3.0
    cs.append(("vof5p", c))
    c = box_case(7, jitter=0.3, mesh_seed=99)
    c.name = "box7j"
    c.P = np.random.default_rng(5).uniform(-2, 2, c.mesh.n_cells)
    cs.append(("box7j", c))
    # surface tension: curvature, source and the face-velocity terms
    c = with_fields(vof_case(6, jitter=0.2), seed=3, p_scale=50.0)
    c.sigma = 0.07
    c.name = "vof6js"
    cs.append(("vof6js", c))
    return cs


def outer_cases():
    cs = []
    c = with_history(with_fields(vof_case(6), seed=11, p_scale=80.0), seed=12)
    # walls of every supported velocity type exercise the momentum boundary loop
    c.bc_type[c.mesh.patch_names.index("xmin"), 1] = BC_NO_SLIP
    c.bc_type[c.mesh.patch_names.index("ymax"), 1] = BC_SLIP
    c.bc_type[c.mesh.patch_names.index("ymin"), 1] = BC_FIXED_VALUE
    c.bc_value[c.mesh.patch_names.index("ymin"), 1:4] = (0.5, -0.25, 0.125)
    c.name = "outer_vof6"
    cs.append(("outer_vof6", c))
    c = with_history(box_case(7, jitter=0.3, mesh_seed=77), seed=13, scale=0.3)
    c.dt = 0.01
    c.P = np.random.default_rng(14).uniform(-1, 1, c.mesh.n_cells)
    c.mom_u_urf = 0.7
    c.name = "outer_box7j"
    cs.append(("outer_box7j", c))
    c = with_history(with_fields(vof_case(6, jitter=0.2), seed=11, p_scale=80.0), seed=12)
    c.sigma = 0.07
    c.name = "outer_vof6js"
    cs.append(("outer_vof6js", c))
    return cs


def vofeq_cases():
    cs = []
    c = with_vf_history(with_fields(vof_case(8, jitter=0.25), seed=5, p_scale=100.0), seed=9)
    c.name = "vofeq_vof8"
    cs.append(("vofeq_vof8", c))
    c = with_vf_history(vof_case(7, jitter=0.2), seed=4)
    # an inflow patch with a fixed volume fraction exercises the boundary coefficient
    c.bc_type[c.mesh.patch_names.index("xmin"), 2] = BC_FIXED_VALUE
    c.bc_value[c.mesh.patch_names.index("xmin"), 4] = 0.7
    c.vof_urf = 0.5
    c.name = "vofeq_vof7"
    cs.append(("vofeq_vof7", c))
    c = with_vf_history(with_fields(vof_case(7, jitter=0.25), seed=5, p_scale=100.0), seed=9)
    c.sigma = 0.07
    c.name = "vofeq_vof7js"
    cs.append(("vofeq_vof7js", c))
    return cs


def save(name: str, case, ref: dict, momentum: bool = False, vof: bool = False) -> None:
    m = case.mesh
    out = {f"ref_{k}": v for k, v in ref.items()}
    if momentum:
        out["history"] = np.stack(case.history())
    if vof:
        out["vf_history"] = np.stack(case.vf_history())
    out.update(points=m.points, face_ptr=m.face_ptr, face_pts=m.face_pts, owner=m.owner,
               neighbour=m.neighbour, patch_start=m.patch_start, patch_size=m.patch_size,
               n_cells=np.int64(m.n_cells), P=case.P, U=case.U, V=case.V, W=case.W, VF=case.VF,
               bc_type=case.bc_type, bc_value=case.bc_value,
               params=np.array([case.dt, case.rho[0], case.rho[1], case.mu[0], case.mu[1], case.sigma,
                                case.gravity[0], case.gravity[1], case.gravity[2], case.pre_p_urf,
                                case.pre_u_urf, 1.0 if case.use_gravity else 0.0, case.mom_u_urf,
                                1.0 if momentum else 0.0, case.vof_urf]))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def foam_cases():
    """Meshes written as OpenFOAM polyMesh directories (tests/golden/foam_*)."""
    from semo_mesh_gb300.meshgen import hex_box, tet_box
    yield "foam_hex4j", hex_box(4, jitter=0.2, seed=7)
    yield "foam_tet2j", tet_box(2, jitter=0.2, seed=8)


def parse_foam_dump(path: str) -> dict:
    """The binary dump of `semo_ref foam` (oracle/ref/ref_driver.cpp)."""
    raw = open(path, "rb").read()
    pos = 0

    def i32(k=1):
        nonlocal pos
        v = np.frombuffer(raw, dtype=np.int32, count=k, offset=pos)
        pos += 4 * k
        return v

    np_ = int(i32()[0])
    pts = np.frombuffer(raw, dtype=np.float64, count=3 * np_, offset=pos).copy()
    pos += 24 * np_
    nf = int(i32()[0])
    fptr, fpts = [0], []
    for _ in range(nf):
        n = int(i32()[0])
        fpts.extend(i32(n).tolist())
        fptr.append(len(fpts))
    owner = i32(nf).copy()
    ni = int(i32()[0])
    neighbour = i32(ni).copy()
    npatch = int(i32()[0])
    names, start, size = [], [], []
    for _ in range(npatch):
        ln = int(i32()[0])
        names.append(raw[pos:pos + ln].decode())
        pos += ln
        start.append(int(i32()[0]))
        size.append(int(i32()[0]))
    return {"points": pts, "face_ptr": np.array(fptr, dtype=np.int32), "face_pts": np.array(fpts, dtype=np.int32),
            "owner": owner, "neighbour": neighbour, "patch_names": np.array(names),
            "patch_start": np.array(start, dtype=np.int32), "patch_size": np.array(size, dtype=np.int32)}


def make_foam() -> None:
    from semo_mesh_gb300.foam import write_polymesh
    exe = os.path.join(ROOT, "oracle", "_ref", "semo_ref")
    for name, mesh in foam_cases():
        d = os.path.join(HERE, name)
        write_polymesh(mesh, d)
        out = os.path.join(HERE, name + ".bin")
        subprocess.run([exe, "foam", d, out], check=True, stdout=subprocess.DEVNULL)
        np.savez_compressed(os.path.join(HERE, f"{name}_ref.npz"), **parse_foam_dump(out))
        os.remove(out)
        print(name, mesh.n_cells, "cells (OpenFOAM loader)")


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 and not sys.argv[1].startswith("--") else "/root/reference"
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={ref_dir}", "-j8"],
                   check=True, stdout=subprocess.DEVNULL)
    # --only NAME [NAME ...]: regenerate just those fixtures
    only = set(sys.argv[sys.argv.index("--only") + 1:]) if "--only" in sys.argv else None
    pick = (lambda n: only is None or n in only)
    if only is None or any(n.startswith("foam_") for n in only):
        make_foam()
    if "--foam-only" in sys.argv:
        return
    for name, case in golden_cases():
        if not pick(name):
            continue
        ref = run_reference(case, threads=1)
        save(name, case, ref)
        print(name, case.mesh.n_cells, "cells")
    for name, case in outer_cases():
        if not pick(name):
            continue
        ref = run_reference(case, threads=1, momentum=True)
        save(name, case, ref, momentum=True)
        print(name, case.mesh.n_cells, "cells (outer iteration)")
    for name, case in vofeq_cases():
        if not pick(name):
            continue
        ref = run_reference(case, threads=1, vof=True)
        save(name, case, ref, vof=True)
        print(name, case.mesh.n_cells, "cells (volume-fraction sub-iteration)")


if __name__ == "__main__":
    main()
