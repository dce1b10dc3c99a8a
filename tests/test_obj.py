"""OBJ ingestion (CPU): fan triangulation, index forms and negative indices, degenerate
faces, usemtl material slots -- each checked against triangles written out by hand
from the file's own numbers."""
import numpy as np

from visionaray_gb300 import scenes
from visionaray_gb300.types import EMISSIVE, MATTE

OBJ = """# test mesh
mtllib test.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0 0 1
vt 0 0
vn 0 0 1
f 1 2 3
usemtl red
f 1/1 3/1 4/1
f 1//1 2//1 3//1 4//1
usemtl missing
f -5/1/1 -4/1/1 -1/1/1
usemtl light
f 1 2 2
f 2 3 5 4
"""

MTL = """newmtl red
Kd 0.9 0.1 0.1
newmtl light
Kd 0 0 0
Ke 5 5 4
"""


def tri(p1, p2, p3):
    p1, p2, p3 = (np.asarray(p, np.float32) for p in (p1, p2, p3))
    return p1, p2 - p1, p3 - p1


def test_obj_geometry_and_materials(tmp_path):
    (tmp_path / "test.obj").write_text(OBJ)
    (tmp_path / "test.mtl").write_text(MTL)
    tris, mats = scenes.load_obj(tmp_path / "test.obj")
    V = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1)]
    want = [
        (tri(V[0], V[1], V[2]), 0),
        (tri(V[0], V[2], V[3]), 0),          # after usemtl red: slot 0
        (tri(V[0], V[1], V[2]), 0),          # quad as a fan (0,1,2), (0,2,3)
        (tri(V[0], V[2], V[3]), 0),
        (tri(V[0], V[1], V[4]), 0),          # negative indices; unknown usemtl keeps slot 0
        # "f 1 2 2" is degenerate and dropped
        (tri(V[1], V[2], V[4]), 1),          # after usemtl light: slot 1; fan of 4
        (tri(V[1], V[4], V[3]), 1),
    ]
    assert len(tris) == len(want)
    for k, ((v1, e1, e2), g) in enumerate(want):
        assert tris[k]["prim_id"] == k
        assert tris[k]["geom_id"] == g
        assert np.array_equal(tris[k]["v1"], v1) and np.array_equal(tris[k]["e1"], e1)
        assert np.array_equal(tris[k]["e2"], e2)
    assert len(mats) == 2
    assert mats[0]["kind"] == MATTE and np.allclose(mats[0]["color"], (0.9, 0.1, 0.1))
    assert mats[1]["kind"] == EMISSIVE and np.allclose(mats[1]["color"], (5, 5, 4))


def test_obj_missing_file(tmp_path):
    import pytest
    with pytest.raises(FileNotFoundError):
        scenes.load_obj(tmp_path / "none.obj")


def test_obj_without_materials(tmp_path):
    (tmp_path / "a.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\nf 1 2 9\n")
    tris, mats = scenes.load_obj(tmp_path / "a.obj")
    assert len(tris) == 1 and tris[0]["geom_id"] == 0   # the out-of-range face is skipped
    assert len(mats) == 1 and mats[0]["kind"] == MATTE
