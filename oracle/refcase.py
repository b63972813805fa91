"""Case files for the reference driver (oracle/_ref/semo_ref) and its output.

Test infrastructure for the CPU checker: writes a mesh + fields + boundary
conditions in the binary layout oracle/ref/ref_driver.cpp reads, runs the
driver, and parses the named arrays it dumps.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(HERE, "_ref", "semo_ref")
MAGIC = 0x53454D4F


def write_case(case, path: str, flags: int | None = None, momentum: bool = False, vof: bool = False) -> None:
    """flags bit 0: gravity source; bit 1: whole outer iteration (momentum, then
    pressure); bit 2: one volume-fraction sub-iteration instead; bit 3:
    curvature and surface-tension source (set when the case has sigma != 0)."""
    m = case.mesh
    if flags is None:
        flags = ((1 if case.use_gravity else 0) | (2 if momentum else 0) | (4 if vof else 0)
                 | (8 if case.sigma != 0.0 else 0))
    with open(path, "wb") as f:
        f.write(struct.pack("<8i", MAGIC, m.n_points, m.n_faces, m.n_internal, m.n_cells,
                            len(m.patch_names), int(m.face_pts.shape[0]), flags))
        f.write(np.ascontiguousarray(m.points, dtype="<f8").tobytes())
        for a in (m.face_ptr, m.face_pts, m.owner, m.neighbour):
            f.write(np.ascontiguousarray(a, dtype="<i4").tobytes())
        for p in range(len(m.patch_names)):
            t = case.bc_type[p]
            v = case.bc_value[p]
            f.write(struct.pack("<6i", int(m.patch_start[p]), int(m.patch_size[p]), int(t[0]), int(t[1]), int(t[2]), 0))
            f.write(struct.pack("<6d", v[0], v[1], v[2], v[3], v[4], 0.0))
        for a in (case.P, case.U, case.V, case.W, case.VF):
            f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())
        prm = np.zeros(16)
        prm[:11] = [case.dt, case.rho[0], case.rho[1], case.mu[0], case.mu[1], case.sigma,
                    case.gravity[0], case.gravity[1], case.gravity[2], case.pre_p_urf, case.pre_u_urf]
        prm[12] = case.mom_u_urf
        prm[13] = case.vof_urf
        f.write(prm.astype("<f8").tobytes())
        if flags & 2:
            for a in case.history():
                f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())
        if flags & 4:
            for a in case.vf_history():
                f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())


def read_output(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        (ln,) = struct.unpack_from("<i", data, pos); pos += 4
        name = data[pos:pos + ln].decode(); pos += ln
        (dt,) = struct.unpack_from("<i", data, pos); pos += 4
        (cnt,) = struct.unpack_from("<q", data, pos); pos += 8
        if dt == 0:
            out[name] = np.frombuffer(data, dtype="<f8", count=cnt, offset=pos).copy(); pos += 8 * cnt
        else:
            out[name] = np.frombuffer(data, dtype="<i4", count=cnt, offset=pos).copy(); pos += 4 * cnt
    return out


def have_reference_binary() -> bool:
    return os.path.exists(REF_BIN)


def run_reference(case, threads: int = 1, timeout: float = 3600.0, momentum: bool = False,
                  vof: bool = False) -> dict:
    """Run the reference's own code on `case` and return its dumped arrays (one
    pressure pass; with `momentum` a momentum + pressure outer iteration; with
    `vof` one volume-fraction sub-iteration)."""
    if not have_reference_binary():
        raise FileNotFoundError(REF_BIN)
    with tempfile.TemporaryDirectory() as td:
        cp = os.path.join(td, "case.bin")
        op = os.path.join(td, "out.bin")
        write_case(case, cp, momentum=momentum, vof=vof)
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        subprocess.run([REF_BIN, cp, op], check=True, env=env, timeout=timeout,
                       stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
        return read_output(op)
