"""OpenFOAM polyMesh reading (SEMO_Mesh_Load::OpenFoam, src/load/loadOpenFoam.cpp).

The foam_* fixtures are polyMesh directories written from seeded meshes; the
matching foam_*_ref.npz hold what the reference's own loader read from them
(tests/golden/make_golden.py).  The library's reader must return the same
points (bit for bit), face point lists, owner, neighbour and patches.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
FOAM = sorted(d for d in os.listdir(GOLD) if d.startswith("foam_") and os.path.isdir(os.path.join(GOLD, d)))


def test_fixtures_present():
    assert len(FOAM) >= 2


@pytest.mark.parametrize("name", FOAM)
def test_reader_matches_reference_loader(name):
    from semo_mesh_gb300.foam import read_polymesh
    m = read_polymesh(os.path.join(GOLD, name))
    ref = np.load(os.path.join(GOLD, name + "_ref.npz"))
    assert np.array_equal(m.points.reshape(-1), ref["points"])
    assert np.array_equal(m.face_ptr, ref["face_ptr"])
    assert np.array_equal(m.face_pts, ref["face_pts"])
    assert np.array_equal(m.owner, ref["owner"])
    assert np.array_equal(m.neighbour, ref["neighbour"])
    assert m.patch_names == [str(x) for x in ref["patch_names"]]
    assert np.array_equal(m.patch_start, ref["patch_start"])
    assert np.array_equal(m.patch_size, ref["patch_size"])


@pytest.mark.parametrize("tets", [False, True])
def test_write_read_round_trip(tmp_path, tets):
    from semo_mesh_gb300.foam import read_polymesh, write_polymesh
    from semo_mesh_gb300.meshgen import hex_box, tet_box
    m = tet_box(3, jitter=0.2, seed=3) if tets else hex_box(5, jitter=0.2, seed=3)
    write_polymesh(m, str(tmp_path))
    r = read_polymesh(str(tmp_path))
    for k in ("points", "face_ptr", "face_pts", "owner", "neighbour", "patch_start", "patch_size"):
        assert np.array_equal(getattr(r, k), getattr(m, k)), k
    assert r.n_cells == m.n_cells and r.patch_names == list(m.patch_names)


def test_multiline_faces_and_missing_files(tmp_path):
    """A face written over several lines reads like a one-line face; a missing file is an error."""
    from semo_mesh_gb300.foam import read_polymesh, write_polymesh
    from semo_mesh_gb300.meshgen import hex_box
    m = hex_box(2)
    write_polymesh(m, str(tmp_path))
    faces = (tmp_path / "faces").read_text().split("\n")
    i = faces.index("(") + 1
    n, rest = faces[i].split("(", 1)
    faces[i] = n + "(" + rest.replace(" ", "\n", 1)
    (tmp_path / "faces").write_text("\n".join(faces))
    r = read_polymesh(str(tmp_path))
    assert np.array_equal(r.face_pts, m.face_pts)
    os.remove(tmp_path / "owner")
    with pytest.raises(RuntimeError, match="cannot open"):
        read_polymesh(str(tmp_path))


@pytest.mark.gpu
def test_load_foam_gives_the_same_pressure_system():
    """Uploading through the reader equals uploading the in-memory mesh."""
    import semo_mesh_gb300 as S
    from semo_mesh_gb300.cases import vof_case
    from semo_mesh_gb300.foam import write_polymesh
    import tempfile
    case = vof_case(6)
    d = tempfile.mkdtemp()
    write_polymesh(case.mesh, d)
    a = S.Context(precision="fp64", tol=1e-10)
    a.set_case(case)
    a.assemble()
    b = S.Context(precision="fp64", tol=1e-10)
    b.load_foam(d)
    case2 = vof_case(6)
    case2.mesh = b.mesh
    b.set_case(case2)
    b.assemble()
    sa, sb = a.system_rcm(), b.system_rcm()
    for k in ("ptr", "col", "val", "b"):
        assert np.array_equal(sa[k], sb[k]), k
