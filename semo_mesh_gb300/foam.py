"""OpenFOAM polyMesh directories (ASCII) to and from ``PolyMesh``.

``write_polymesh`` writes ``points``, ``faces``, ``owner``, ``neighbour`` and
``boundary`` in the ASCII layout SEMO's loader reads (one entry per line,
single spaces, coordinates with 17 significant digits so they read back
exactly).  ``read_polymesh`` parses such a directory through the library's
reader (``semo_foam_sizes`` / ``semo_foam_read``, the parsing of SEMO's
``SEMO_Mesh_Load::OpenFoam``); it needs no GPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .meshgen import PolyMesh

_HEADER = """FoamFile
{{
    version     2.0;
    format      ascii;
    class       {cls};
    location    "constant/polyMesh";
    object      {obj};
}}
"""


def _write_list(path: str, cls: str, obj: str, lines) -> None:
    with open(path, "w") as f:
        f.write(_HEADER.format(cls=cls, obj=obj))
        f.write("\n")
        f.write(f"{len(lines)}\n(\n")
        f.write("\n".join(lines))
        if lines:
            f.write("\n")
        f.write(")\n")


def write_polymesh(mesh: PolyMesh, directory: str) -> None:
    """Write ``mesh`` as an OpenFOAM polyMesh directory (created if needed)."""
    os.makedirs(directory, exist_ok=True)
    pts = [f"({x!r} {y!r} {z!r})" for x, y, z in mesh.points.tolist()]
    _write_list(os.path.join(directory, "points"), "vectorField", "points", pts)
    fp = mesh.face_ptr.tolist()
    idx = mesh.face_pts.tolist()
    faces = [f"{fp[i + 1] - fp[i]}(" + " ".join(str(q) for q in idx[fp[i]:fp[i + 1]]) + ")"
             for i in range(mesh.n_faces)]
    _write_list(os.path.join(directory, "faces"), "faceList", "faces", faces)
    _write_list(os.path.join(directory, "owner"), "labelList", "owner", [str(v) for v in mesh.owner.tolist()])
    _write_list(os.path.join(directory, "neighbour"), "labelList", "neighbour",
                [str(v) for v in mesh.neighbour.tolist()])
    with open(os.path.join(directory, "boundary"), "w") as f:
        f.write(_HEADER.format(cls="polyBoundaryMesh", obj="boundary"))
        f.write(f"\n{len(mesh.patch_names)}\n(\n")
        for name, start, size in zip(mesh.patch_names, mesh.patch_start.tolist(), mesh.patch_size.tolist()):
            f.write(f"    {name}\n    {{\n        type            patch;\n"
                    f"        nFaces          {size};\n        startFace       {start};\n    }}\n")
        f.write(")\n")


def read_polymesh(directory: str) -> PolyMesh:
    """Parse an OpenFOAM polyMesh directory with the library's reader."""
    from . import load_library
    L = load_library()
    d = directory.encode()
    sizes = (C.c_int64 * 6)()
    if L.semo_foam_sizes(d, sizes) != 0:
        raise RuntimeError(L.semo_foam_last_error().decode(errors="replace"))
    n_points, n_faces, n_internal, n_cells, n_fp, n_patches = (int(v) for v in sizes)
    pts = np.empty(3 * n_points)
    fptr = np.empty(n_faces + 1, dtype=np.int32)
    fpts = np.empty(n_fp, dtype=np.int32)
    own = np.empty(n_faces, dtype=np.int32)
    nei = np.empty(n_internal, dtype=np.int32)
    pstart = np.empty(n_patches, dtype=np.int32)
    psize = np.empty(n_patches, dtype=np.int32)
    names = C.create_string_buffer(64 * max(n_patches, 1))
    i32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
    if L.semo_foam_read(d, pts.ctypes.data_as(C.POINTER(C.c_double)), i32(fptr), i32(fpts), i32(own), i32(nei),
                        i32(pstart), i32(psize), names) != 0:
        raise RuntimeError(L.semo_foam_last_error().decode(errors="replace"))
    raw = names.raw
    pn = [raw[64 * p:64 * (p + 1)].split(b"\0", 1)[0].decode() for p in range(n_patches)]
    return PolyMesh(points=pts.reshape(-1, 3), face_ptr=fptr, face_pts=fpts, owner=own, neighbour=nei,
                    n_cells=n_cells, patch_names=pn, patch_start=pstart, patch_size=psize)
