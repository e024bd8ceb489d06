"""OBJ ingestion (dr_obj_read) against the reference's own MeshReader::readObj + PolyMesh::bake
(built into oracle/_ref): the same objects, names, and triangle corners (positions, normals, texture
coordinates) bit for bit, on files covering the format's features and the reference's quirks.  CPU only."""
from pathlib import Path

import numpy as np
import pytest

import dumbray_gb300 as dr
from dumbray_gb300 import scenes
import _oracle as O

pytestmark = pytest.mark.skipif(not O.reference_available() or not hasattr(O.reference(), "dref_obj_read"),
                                reason="reference library with its OBJ reader not built here")

CUBE = """# a cube with normals and texture coordinates, two groups
v -1 -1 -1
v  1 -1 -1
v  1  1 -1
v -1  1 -1
v -1 -1  1
v  1 -1  1
v  1  1  1
v -1  1  1
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 -1
vn 0 0 1
vn 0 -1 0
vn 0 1 0
vn -1 0 0
vn 1 0 0
g Front Part
f 1/1/1 2/2/1 3/3/1 4/4/1
f 5/1/2 8/4/2 7/3/2 6/2/2
s off
g back
usemtl whatever
f 1/1/3 5/2/3 6/3/3 2/4/3
f 4/1/4 3/2/4 7/3/4 8/4/4   # trailing comment
f 1//5 4//5 8//5 5//5
f 2//6 6//6 7//6 3//6
"""

NO_NORMALS = "g poly\r\nv 0 0 0\r\nv 1 0 0\r\nv 1.5 1 0.25\r\nv 0.5 1.7 -0.5\r\nv -0.5 1 1e-3\r\n" \
             "o ignored_object_statement\r\nf 1 2 3 4 5\r\nv\t2 2 2\r\nf 1/ 3 6\r\ng   spaced name  \r\nf 2 3 6\r\n"


def _write(tmp_path, name, text):
    p = Path(tmp_path) / name
    p.write_bytes(text.encode() if isinstance(text, str) else text)
    return p


def _icosphere_obj(level=3):
    tris = scenes.icosphere(level, 0.7)
    lines = ["g sphere"]
    for t in tris:
        for v in t:
            lines.append("v %.9g %.9g %.9g" % tuple(v))
    for i in range(len(tris)):
        lines.append("f %d %d %d" % (3 * i + 1, 3 * i + 2, 3 * i + 3))
    return "\n".join(lines) + "\n"


def _same(path):
    ref = O.ref_read_obj(path)
    if ref is None or len(ref[0]) != len(ref[1]):
        with pytest.raises(dr.DumbRayError):
            dr.read_obj(path)
        return None
    ours = dr.read_obj(path)
    names, meshes = ref
    assert list(ours.keys()) == names
    for name, (xyz, nrm, uv) in zip(names, meshes):
        a = ours[name]
        for x, y in zip(a, (xyz, nrm, uv)):
            assert x.shape == y.shape
            assert np.array_equal(x.view(np.int32), y.view(np.int32)), name
    return ours


def test_cube_groups_normals_texcoords(tmp_path):
    ours = _same(_write(tmp_path, "cube.obj", CUBE))
    assert list(ours) == ["Front Part", "back"] and len(ours["back"][0]) == 8
    assert ours["Front Part"][0][0, 0, 0] == 1.0    # x mirrored


def test_generated_normals_crlf_ngons_and_partial_corners(tmp_path):
    ours = _same(_write(tmp_path, "poly.obj", NO_NORMALS))
    assert list(ours) == ["poly", "spaced name"]


def test_icosphere_floats(tmp_path):
    _same(_write(tmp_path, "ico.obj", _icosphere_obj(3)))


@pytest.mark.parametrize("text", [
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\ng late\nf 1 2 3\n",      # faces before the first group
    "g a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\ng b\ng c\nf 3 2 1\n",  # an empty group drops the names
    "g a\nv 0 0 0\nv 1 0 0\nf 1 2 3\n",                             # missing vertex
    "g a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1//4 2 3\n",                 # missing normal
    "g a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\ng trailing\n",        # names dropped at the end
])
def test_reference_failures_and_quirks(tmp_path, text):
    _same(_write(tmp_path, "q.obj", text))


def test_reference_example_mesh_if_present():
    # the reference's example mesh, copied next to the compiled reference by oracle/build_ref.sh
    p = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "example_scenes" / "0" / "files" / "cargo.obj"
    if not p.exists():
        pytest.skip("reference example scene not present")
    ours = _same(p)
    assert ours is not None and len(ours) > 1


def test_objects_build_a_scene_description(tmp_path):
    ours = dr.read_obj(_write(tmp_path, "cube.obj", CUBE))
    tris = np.concatenate([v[0] for v in ours.values()])
    nrm = np.concatenate([v[1] for v in ours.values()])
    assert tris.shape == nrm.shape == (12, 3, 3)
    st = dr.build_octree_host(tris)[0]
    assert st["refs"] >= 12
