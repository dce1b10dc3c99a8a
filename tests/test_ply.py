"""PLY ingestion (the reference viewer's load_ply, src/common/ply_loader.cpp): the
reference reads PLY through tinyply, which is not vendored in the reference tree, so
these fixtures are written here and their triangles derived by hand: v1 = p[i0],
e1 = p[i1] - v1, e2 = p[i2] - v1 in float, prim_id in face order, geom_id 0, no
degenerate-face test; faces of more than three vertices as fans."""
import struct

import numpy as np
import pytest

from visionaray_gb300 import scenes

VERTS = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [1.0, 1.0, 0.0], [0.0, 1.0, 0.5], [0.25, 0.5, 2.0]],
                 np.float32)
FACES = [[0, 1, 2], [0, 2, 3], [4, 4, 4], [1, 2, 3, 4]]   # a degenerate face and a quad


def expected():
    tris = []
    for f in FACES:
        for last in range(2, len(f)):
            a, b, c = VERTS[f[0]], VERTS[f[last - 1]], VERTS[f[last]]
            tris.append((a, b - a, c - a))
    return tris


def check(tris):
    exp = expected()
    assert len(tris) == len(exp) == 5
    for k, (v1, e1, e2) in enumerate(exp):
        assert np.array_equal(tris["v1"][k], v1)
        assert np.array_equal(tris["e1"][k], e1)
        assert np.array_equal(tris["e2"][k], e2)
    assert list(tris["prim_id"]) == list(range(5))
    assert (tris["geom_id"] == 0).all()


def header(fmt, index_type="int", count_type="uchar", extra_vertex=(), extra_element=None):
    lines = ["ply", f"format {fmt} 1.0", "comment written by the test", f"element vertex {len(VERTS)}",
             "property float x", "property float y", "property float z"]
    lines += [f"property {t} {n}" for t, n in extra_vertex]
    if extra_element:
        lines += [f"element {extra_element[0]} {extra_element[1]}", "property int a", "property list uchar int b"]
    lines += [f"element face {len(FACES)}", "property uchar flags",
              f"property list {count_type} {index_type} vertex_indices", "end_header"]
    return ("\n".join(lines) + "\n").encode()


def test_ascii(tmp_path):
    body = "".join(f"{x} {y} {z} 7\n" for x, y, z in VERTS)
    body += "9 2 1 2\n"   # the extra element: a = 9, b = [1, 2]
    body += "".join(f"1 {len(f)} " + " ".join(str(i) for i in f) + "\n" for f in FACES)
    p = tmp_path / "mesh.ply"
    p.write_bytes(header("ascii", extra_vertex=[("uchar", "red")], extra_element=("edge", 1)) + body.encode())
    check(scenes.load_ply(p))


@pytest.mark.parametrize("order", ["<", ">"])
@pytest.mark.parametrize("index_type,code", [("int", "i"), ("uint", "I"), ("ushort", "H"), ("uchar", "B"),
                                             ("short", "h"), ("char", "b")])
def test_binary(tmp_path, order, index_type, code):
    fmt = "binary_little_endian" if order == "<" else "binary_big_endian"
    body = b"".join(struct.pack(order + "fffd", *v, 0.125) for v in VERTS)   # + a double property
    body += struct.pack(order + "iB", -5, 2) + struct.pack(order + "ii", 1, 2)   # the extra element
    for f in FACES:
        body += struct.pack(order + "BB", 0, len(f)) + struct.pack(order + code * len(f), *f)
    p = tmp_path / "mesh.ply"
    p.write_bytes(header(fmt, index_type, extra_vertex=[("double", "confidence")], extra_element=("edge", 1))
                  + body)
    check(scenes.load_ply(p))


def test_double_positions_and_int_counts(tmp_path):
    lines = ["ply", "format binary_little_endian 1.0", f"element vertex {len(VERTS)}", "property double x",
             "property double y", "property double z", f"element face {len(FACES)}",
             "property list int uint vertex_indices", "end_header"]
    body = b"".join(struct.pack("<ddd", *map(float, v)) for v in VERTS)
    for f in FACES:
        body += struct.pack("<i", len(f)) + struct.pack("<" + "I" * len(f), *f)
    p = tmp_path / "mesh.ply"
    p.write_bytes(("\n".join(lines) + "\n").encode() + body)
    check(scenes.load_ply(p))


def test_scene_of_a_loaded_mesh_matches_the_generator(tmp_path):
    """A heightfield written as PLY reads back as the generator's triangles (same
    vertices, faces in order), so ingestion and generation agree bit for bit."""
    tris = scenes.heightfield(grid=8, seed=3)
    v1, e1, e2 = tris["v1"], tris["e1"], tris["e2"]
    pts = np.concatenate([v1, v1 + e1, v1 + e2]).astype(np.float32)
    n = len(tris)
    faces = np.stack([np.arange(n), np.arange(n) + n, np.arange(n) + 2 * n], axis=1)
    lines = ["ply", "format binary_little_endian 1.0", f"element vertex {len(pts)}", "property float x",
             "property float y", "property float z", f"element face {n}", "property list uchar int vertex_indices",
             "end_header"]
    body = pts.astype("<f4").tobytes()
    body += b"".join(struct.pack("<B3i", 3, *map(int, f)) for f in faces)
    p = tmp_path / "hf.ply"
    p.write_bytes(("\n".join(lines) + "\n").encode() + body)
    got = scenes.load_ply(p)
    assert np.array_equal(got["v1"], v1)
    # e = (v1 + e) - v1 in float: equal to the generator's edge unless rounding moved it
    assert np.array_equal(got["e1"], (v1 + e1) - v1) and np.array_equal(got["e2"], (v1 + e2) - v1)
    assert np.array_equal(got["prim_id"], np.arange(n))


@pytest.mark.parametrize("case", ["index_out_of_range", "truncated", "no_vertex_indices", "two_index_face",
                                  "not_ply", "bad_format", "missing"])
def test_malformed_files_are_rejected(tmp_path, case):
    p = tmp_path / "bad.ply"
    good_body = b"".join(struct.pack("<fff", *v) for v in VERTS[:3]) + struct.pack("<B3i", 3, 0, 1, 2)
    head = ["ply", "format binary_little_endian 1.0", "element vertex 3", "property float x", "property float y",
            "property float z", "element face 1", "property list uchar int vertex_indices", "end_header"]
    if case == "index_out_of_range":
        data = ("\n".join(head) + "\n").encode() + good_body[:-4] + struct.pack("<i", 3)
    elif case == "truncated":
        data = ("\n".join(head) + "\n").encode() + good_body[:-3]
    elif case == "no_vertex_indices":
        data = ("\n".join(head).replace("vertex_indices", "vertex_index") + "\n").encode() + good_body
    elif case == "two_index_face":
        data = ("\n".join(head) + "\n").encode() + good_body[:-13] + struct.pack("<B2i", 2, 0, 1)
    elif case == "not_ply":
        data = b"obj\n" + good_body
    elif case == "bad_format":
        data = ("\n".join(head).replace("binary_little_endian", "binary_middle_endian") + "\n").encode() + good_body
    else:
        data = None
    if data is not None:
        p.write_bytes(data)
    with pytest.raises(ValueError):
        scenes.load_ply(p)
