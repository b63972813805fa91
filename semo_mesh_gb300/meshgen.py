"""Synthetic polyhedral meshes in OpenFOAM polyMesh order.

SEMO reads meshes as OpenFOAM ``points / faces / owner / neighbour / boundary``
lists (src/load/loadOpenFoam.cpp:8-383) and derives everything else from them
(src/mesh/build.cpp:480-705).  The generators here emit exactly that layout:

* internal faces first, in upper-triangular order (sorted by owner, then by
  neighbour), each with its point loop ordered so that the right-hand-rule
  normal points from owner to neighbour;
* then one contiguous block of boundary faces per patch, each ordered by owner
  cell, normals pointing out of the domain.

Hex boxes are n x n x n cells on the unit cube.  ``jitter`` moves every
interior vertex by i.i.d. uniform[-jitter, jitter] * h per coordinate (seeded);
vertices on the box surface are left in place so that each patch stays planar.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

PATCH_NAMES = ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")


@dataclass
class PolyMesh:
    points: np.ndarray          # (n_points, 3) float64
    face_ptr: np.ndarray        # (n_faces+1,) int32, CSR offsets into face_pts
    face_pts: np.ndarray        # int32 point indices of every face loop
    owner: np.ndarray           # (n_faces,) int32
    neighbour: np.ndarray       # (n_internal,) int32
    n_cells: int
    patch_names: list = field(default_factory=list)
    patch_start: np.ndarray = None   # (n_patches,) int32 first face of each patch
    patch_size: np.ndarray = None    # (n_patches,) int32

    @property
    def n_faces(self) -> int:
        return int(self.owner.shape[0])

    @property
    def n_internal(self) -> int:
        return int(self.neighbour.shape[0])

    @property
    def n_points(self) -> int:
        return int(self.points.shape[0])

    def patch_faces(self, name: str) -> np.ndarray:
        p = self.patch_names.index(name)
        s = int(self.patch_start[p])
        return np.arange(s, s + int(self.patch_size[p]), dtype=np.int64)

    def patch_cells(self, name: str) -> np.ndarray:
        return self.owner[self.patch_faces(name)]


def _quad_csr(quads: np.ndarray):
    nf = quads.shape[0]
    ptr = (np.arange(nf + 1, dtype=np.int64) * 4).astype(np.int32)
    return ptr, quads.reshape(-1).astype(np.int32)


def hex_box(n: int, jitter: float = 0.0, seed: int = 1234) -> PolyMesh:
    """n^3 hexahedra on [0,1]^3 (cell index i + n*j + n*n*k)."""
    n1 = n + 1
    h = 1.0 / n
    g = np.arange(n1, dtype=np.float64) * h
    # point index p(i,j,k) = i + n1*j + n1*n1*k
    pz, py, px = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([px.reshape(-1), py.reshape(-1), pz.reshape(-1)], axis=1).copy()
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter, jitter, size=pts.shape) * h
        ii = np.arange(n1)
        kk, jj, iq = np.meshgrid(ii, ii, ii, indexing="ij")
        interior = ((iq > 0) & (iq < n) & (jj > 0) & (jj < n) & (kk > 0) & (kk < n)).reshape(-1)
        pts[interior] += d[interior]

    def P(i, j, k):
        return i + n1 * j + n1 * n1 * k

    def C(i, j, k):
        return i + n * j + n * n * k

    # ---- internal faces in upper-triangular order ------------------------
    # owner c has up to three higher neighbours: c+1 (x), c+n (y), c+n*n (z);
    # in that order they are already sorted by neighbour index.
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    i = i.reshape(-1); j = j.reshape(-1); k = k.reshape(-1)
    c = C(i, j, k)
    slots = np.full((n * n * n, 3), -1, dtype=np.int64)
    quads = np.zeros((n * n * n, 3, 4), dtype=np.int64)
    nb = np.full((n * n * n, 3), -1, dtype=np.int64)
    mx = i < n - 1
    my = j < n - 1
    mz = k < n - 1
    # x-face at i+1: loop (j,k)->(j+1,k)->(j+1,k+1)->(j,k+1): normal +x
    quads[:, 0] = np.stack([P(i + 1, j, k), P(i + 1, j + 1, k), P(i + 1, j + 1, k + 1), P(i + 1, j, k + 1)], 1)
    # y-face at j+1: loop along z then x: normal +y
    quads[:, 1] = np.stack([P(i, j + 1, k), P(i, j + 1, k + 1), P(i + 1, j + 1, k + 1), P(i + 1, j + 1, k)], 1)
    # z-face at k+1: loop along x then y: normal +z
    quads[:, 2] = np.stack([P(i, j, k + 1), P(i + 1, j, k + 1), P(i + 1, j + 1, k + 1), P(i, j + 1, k + 1)], 1)
    nb[:, 0] = np.where(mx, c + 1, -1)
    nb[:, 1] = np.where(my, c + n, -1)
    nb[:, 2] = np.where(mz, c + n * n, -1)
    valid = nb >= 0
    own_i = np.repeat(c[:, None], 3, axis=1)[valid]
    nei_i = nb[valid]
    quad_i = quads[valid]

    # ---- boundary patches ------------------------------------------------
    t = np.arange(n)
    b2, b1 = np.meshgrid(t, t, indexing="ij")   # b2 slow, b1 fast -> owner order
    b1 = b1.reshape(-1); b2 = b2.reshape(-1)
    zero = np.zeros_like(b1)
    last = np.full_like(b1, n - 1)
    bq = []
    bo = []
    # xmin: cells (0,j,k), owner order k-major; outward normal -x
    bo.append(C(zero, b1, b2))
    bq.append(np.stack([P(0, b1, b2), P(0, b1, b2 + 1), P(0, b1 + 1, b2 + 1), P(0, b1 + 1, b2)], 1))
    # xmax: +x
    bo.append(C(last, b1, b2))
    bq.append(np.stack([P(n, b1, b2), P(n, b1 + 1, b2), P(n, b1 + 1, b2 + 1), P(n, b1, b2 + 1)], 1))
    # ymin: cells (i,0,k); -y
    bo.append(C(b1, zero, b2))
    bq.append(np.stack([P(b1, 0, b2), P(b1 + 1, 0, b2), P(b1 + 1, 0, b2 + 1), P(b1, 0, b2 + 1)], 1))
    # ymax: +y
    bo.append(C(b1, last, b2))
    bq.append(np.stack([P(b1, n, b2), P(b1, n, b2 + 1), P(b1 + 1, n, b2 + 1), P(b1 + 1, n, b2)], 1))
    # zmin: cells (i,j,0); -z
    bo.append(C(b1, b2, zero))
    bq.append(np.stack([P(b1, b2, 0), P(b1, b2 + 1, 0), P(b1 + 1, b2 + 1, 0), P(b1 + 1, b2, 0)], 1))
    # zmax: +z
    bo.append(C(b1, b2, last))
    bq.append(np.stack([P(b1, b2, n), P(b1 + 1, b2, n), P(b1 + 1, b2 + 1, n), P(b1, b2 + 1, n)], 1))

    n_int = own_i.shape[0]
    quads_all = np.concatenate([quad_i] + bq, axis=0)
    owner = np.concatenate([own_i] + bo).astype(np.int32)
    face_ptr, face_pts = _quad_csr(quads_all)
    sizes = np.array([n * n] * 6, dtype=np.int32)
    starts = (n_int + np.concatenate([[0], np.cumsum(sizes)[:-1]])).astype(np.int32)
    return PolyMesh(points=pts, face_ptr=face_ptr, face_pts=face_pts, owner=owner,
                    neighbour=nei_i.astype(np.int32), n_cells=n * n * n,
                    patch_names=list(PATCH_NAMES), patch_start=starts, patch_size=sizes)


def tet_box(n: int, jitter: float = 0.0, seed: int = 1234) -> PolyMesh:
    """Each hex of an n^3 box split into 6 tetrahedra (6 n^3 cells).

    Every hex uses the split along its (0,0,0)-(1,1,1) diagonal: for each
    ordering (a, b, c) of the axes, the tetrahedron v000, v000+e_a,
    v000+e_a+e_b, v111.  Neighbouring hexes then agree on the triangles of
    their shared quad, so the mesh is conforming.  Cell index 6*h + t for hex
    h = i + n*j + n*n*k and ordering t.  Vertices are placed (and jittered)
    exactly as in ``hex_box``; a jitter of 0.2 h moves two vertices of a
    tetrahedron towards each other by at most 0.57 h, below the smallest
    altitude (h / sqrt 2), so no tetrahedron inverts.
    """
    n1 = n + 1
    h = 1.0 / n
    g = np.arange(n1, dtype=np.float64) * h
    pz, py, px = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([px.reshape(-1), py.reshape(-1), pz.reshape(-1)], axis=1).copy()
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter, jitter, size=pts.shape) * h
        ii = np.arange(n1)
        kk, jj, iq = np.meshgrid(ii, ii, ii, indexing="ij")
        interior = ((iq > 0) & (iq < n) & (jj > 0) & (jj < n) & (kk > 0) & (kk < n)).reshape(-1)
        pts[interior] += d[interior]
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    i = i.reshape(-1).astype(np.int64); j = j.reshape(-1).astype(np.int64); k = k.reshape(-1).astype(np.int64)
    nh = n * n * n
    e = np.eye(3, dtype=np.int64)
    perms = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))
    lat = np.zeros((nh, 6, 4, 3), dtype=np.int64)      # lattice coordinates of each vertex
    ijk = np.stack([i, j, k], axis=1)
    for t, (a, b, _) in enumerate(perms):
        lat[:, t, 0] = ijk
        lat[:, t, 1] = ijk + e[a]
        lat[:, t, 2] = ijk + e[a] + e[b]
        lat[:, t, 3] = ijk + 1
    lat = lat.reshape(6 * nh, 4, 3)
    nc = 6 * nh
    pid = lat[..., 0] + n1 * lat[..., 1] + n1 * n1 * lat[..., 2]          # (nc, 4)
    # the four faces of each tetrahedron: drop vertex m, keep the other three
    drop = ((1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2))
    tri = np.stack([pid[:, list(d)] for d in drop], axis=1).reshape(-1, 3)          # (4 nc, 3)
    tri_lat = np.stack([lat[:, list(d)] for d in drop], axis=1).reshape(-1, 3, 3)
    opp_lat = lat.reshape(-1, 3)                                                     # the dropped vertex
    cell = np.repeat(np.arange(nc, dtype=np.int64), 4)
    # orient each triangle so that its right-hand normal leaves its tetrahedron
    a0 = tri_lat[:, 0]; a1 = tri_lat[:, 1]; a2 = tri_lat[:, 2]
    nrm = np.cross(a1 - a0, a2 - a0)
    inward = np.einsum("ij,ij->i", nrm, opp_lat - a0) > 0
    tri[inward] = tri[inward][:, [0, 2, 1]]
    # pair the triangles: sorted point triples as one key (points < 2^20 each)
    st = np.sort(tri, axis=1)
    key = (st[:, 0] << 40) | (st[:, 1] << 20) | st[:, 2]
    order = np.argsort(key, kind="stable")
    ks = key[order]
    same = np.flatnonzero(ks[1:] == ks[:-1])          # pairs (order[s], order[s+1])
    first = order[same]; second = order[same + 1]
    paired = np.zeros(key.shape[0], dtype=bool)
    paired[first] = True; paired[second] = True
    ca = cell[first]; cb = cell[second]
    own = np.minimum(ca, cb); nei = np.maximum(ca, cb)
    loops = np.where((ca <= cb)[:, None], tri[first], tri[second])                  # owner's outward loop
    o2 = np.lexsort((nei, own))
    own = own[o2]; nei = nei[o2]; loops = loops[o2]
    # boundary triangles: the patch whose plane holds all three vertices
    bidx = np.flatnonzero(~paired)
    bl = tri_lat[bidx]
    patch = np.full(bidx.shape[0], -1, dtype=np.int64)
    for p, (ax, val) in enumerate(((0, 0), (0, n), (1, 0), (1, n), (2, 0), (2, n))):
        on = np.all(bl[:, :, ax] == val, axis=1)
        patch[on & (patch < 0)] = p
    if np.any(patch < 0):
        raise RuntimeError("unpaired triangle off the box surface")
    bown = cell[bidx]
    ob = np.lexsort((bown, patch))
    bown = bown[ob]; bpatch = patch[ob]; bloops = tri[bidx][ob]
    sizes = np.bincount(bpatch, minlength=6).astype(np.int32)
    n_int = own.shape[0]
    starts = (n_int + np.concatenate([[0], np.cumsum(sizes)[:-1]])).astype(np.int32)
    allloops = np.concatenate([loops, bloops], axis=0)
    nf = allloops.shape[0]
    face_ptr = (np.arange(nf + 1, dtype=np.int64) * 3).astype(np.int32)
    return PolyMesh(points=pts, face_ptr=face_ptr, face_pts=allloops.reshape(-1).astype(np.int32),
                    owner=np.concatenate([own, bown]).astype(np.int32), neighbour=nei.astype(np.int32),
                    n_cells=nc, patch_names=list(PATCH_NAMES), patch_start=starts, patch_size=sizes)


def mesh_sizes(mesh: PolyMesh) -> dict:
    return {"cells": mesh.n_cells, "faces": mesh.n_faces, "internal_faces": mesh.n_internal,
            "boundary_faces": mesh.n_faces - mesh.n_internal, "points": mesh.n_points,
            "scalar_nnz": mesh.n_cells + 2 * mesh.n_internal}
