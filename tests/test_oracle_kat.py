"""Known-answer tests of the oracle, re-derived from visionaray's own unit tests."""
import numpy as np
import pytest

from visionaray_gb300.types import RAY, TRIANGLE


def ray(o, d, tmin=0.0, tmax=3.4028234663852886e38):
    r = np.zeros(1, RAY)
    r["ori"], r["dir"], r["tmin"], r["tmax"] = o, d, tmin, tmax
    return r


def tri(v1, p2, p3, prim_id=0):
    t = np.zeros(1, TRIANGLE)
    v1 = np.asarray(v1, np.float32)
    t["v1"] = v1
    t["e1"] = np.asarray(p2, np.float32) - v1
    t["e2"] = np.asarray(p3, np.float32) - v1
    t["prim_id"] = prim_id
    return t


def four_tris():
    # test/unittests/math/intersect.cpp:60-121 (Ray1Tri4): planes x = -3, -2, -1, -0
    out = np.concatenate([tri((x, -1, -1), (x, -1, 1), (x, 1, 0), prim_id=i)
                          for i, x in enumerate((-3.0, -2.0, -1.0, -0.0))])
    return out


def test_morton_encode3d_kat(oracle):
    # test/unittests/morton.cpp:49-70 (morton_encode3D of the unit cube corners)
    # encoded through centroid quantisation is not directly reachable, so check the
    # interleave on Morton codes of a 2x2x2 lattice of tiny triangles instead.
    pts = [(x, y, z) for z in (0, 1) for y in (0, 1) for x in (0, 1)]
    tris = np.concatenate([tri((x, y, z), (x, y, z), (x, y, z), prim_id=i) for i, (x, y, z) in enumerate(pts)])
    codes = oracle.morton_codes(tris)
    # corner (1,1,1) quantises to 1023 on every axis, corner 0 to 0; bit i of x, y, z
    # lands on bit 3i, 3i+1, 3i+2: (1,0,0) -> 0b001001...001 = 0x09249249, etc.
    x_only = 0x09249249
    expect = [(x * x_only) | (y * (x_only << 1)) | (z * (x_only << 2)) for (x, y, z) in pts]
    assert list(codes) == expect
    # encode3D(1,1,1) == 7 (morton.cpp:68-69) is the lowest 3 bits of corner (1,1,1)
    assert codes[7] & 7 == 7 and codes[1] & 7 == 1 and codes[2] & 7 == 2 and codes[4] & 7 == 4


def test_ray_triangle_kat(oracle):
    r = ray((-2.0, 0.0, 0.0), (1.0, 0.0, 0.0))
    ts = four_tris()
    expect_t = {1: 0.0, 2: 1.0, 3: 2.0}
    for i in range(4):
        hit, rec = oracle.intersect(r, ts[i])
        assert hit
        if i in expect_t:
            assert rec["t"] == expect_t[i] and rec["prim_id"] == i
    # t = -1 for the triangle behind the origin: the raw test hits, traversal rejects it
    assert oracle.intersect(r, ts[0])[1]["t"] == -1.0


def test_ray_box_kat(oracle):
    # test/unittests/math/intersect.cpp:16-58 (Ray1AABB4)
    r = ray((-2.0, 0.0, 0.0), (1.0, 0.0, 0.0))
    boxes = [(-3.5, -2.5), (-2.5, -1.5), (-1.5, -0.5), (-0.5, 0.5)]
    res = [oracle.intersect_box(r, (lo, -0.5, -0.5), (hi, 0.5, 0.5)) for lo, hi in boxes]
    assert all(h for h, _, _ in res[1:])
    assert res[2][1] == 0.5 and res[3][1] == 1.5
    assert res[1][2] == 0.5 and res[2][2] == 1.5 and res[3][2] == 2.5


def test_closest_and_any_hit_on_kat_triangles(oracle):
    ts = four_tris()
    r = ray((-2.0, 0.0, 0.0), (1.0, 0.0, 0.0))
    tree = oracle.build_sah(ts)
    h = oracle.trace(tree, ts, r)
    assert h["prim_id"][0] == 1 and h["t"][0] == 0.0
    lin = oracle.trace_linear(ts, r)
    assert lin["prim_id"][0] == 1
    a = oracle.trace(tree, ts, r, any_hit=True)
    assert a["prim_id"][0] in (1, 2, 3)


def test_triangle_area_kat():
    # test/unittests/math/triangle.cpp:10-44: area = 0.5 * |e1 x e2|
    t = tri((0, 0, 0), (2, 0, 0), (0, 2, 0))
    area = 0.5 * np.linalg.norm(np.cross(t["e1"][0], t["e2"][0]))
    assert area == 2.0


def test_lbvh_cpu_rejects_max_leaf_one(oracle):
    # lbvh.h:505-508 + :633-645 recurse forever for max_leaf_size = 1 with equal codes
    with pytest.raises(ValueError):
        oracle.build_lbvh_cpu(four_tris(), max_leaf=1)


def test_karras_bounds_skip_non_finite(oracle):
    """The GPU builder's bounds are float atomicMin / atomicMax by compare-and-swap from
    (+FLT_MAX, -FLT_MAX) (detail/bvh/lbvh.h:63-91, 233-238, 332-372), which never store
    NaN, nor +Inf into a minimum or -Inf into a maximum: in the restated tree only the
    NaN triangles' own leaves carry NaN, no inner box does, and the closest hits over
    the tree are the brute-force ones."""
    from visionaray_gb300 import scenes

    from .parity import compare_closest, non_finite_soup
    tris = non_finite_soup(4000, seed=4)
    tree = oracle.build_karras(tris)
    inner = tree.nodes["num_prims"] == 0
    boxes = np.concatenate([tree.nodes["bbox_min"], tree.nodes["bbox_max"]], axis=1)
    assert not np.isnan(boxes[inner]).any()
    nan_leaves = np.isnan(boxes[~inner]).any(axis=1).sum()
    assert nan_leaves == 20
    assert (tree.nodes["bbox_min"][inner] < np.float32(np.inf)).all()
    rays = scenes.pinhole_rays(64, 64)
    compare_closest(oracle.trace(tree, tris, rays), oracle.trace_linear(tris, rays), rays, tris, oracle)
