"""GPU LBVH build against the oracle's restatement of visionaray's GPU builder.

Topology (children, leaf primitive ids) must be bit-exact and boxes equal, given
identical Morton codes -- which are compared first."""
import numpy as np
import pytest

import visionaray_gb300 as vg
from visionaray_gb300 import scenes

pytestmark = pytest.mark.gpu


def gpu_build(tris):
    return vg.lbvh_builder().build(vg.as_device_bytes(tris))


def assert_same_tree(got_nodes, got_idx, ref_tree):
    assert len(got_nodes) == len(ref_tree.nodes)
    for f in ("first", "num_prims"):
        assert np.array_equal(got_nodes[f], ref_tree.nodes[f]), f
    for f in ("bbox_min", "bbox_max"):
        assert (got_nodes[f] == ref_tree.nodes[f]).all(), f   # float ==: +0 equals -0
    assert np.array_equal(got_idx, ref_tree.indices)


CASES = [("soup", 2, 11), ("soup", 3, 12), ("soup", 17, 13), ("soup", 1000, 14), ("soup", 65536, 1),
         ("soup", 100003, 15), ("heightfield", 64, 1), ("heightfield", 256, 2)]


@pytest.mark.parametrize("kind,size,seed", CASES)
def test_lbvh_matches_restated_reference_builder(oracle, kind, size, seed):
    tris = scenes.soup(size, seed=seed) if kind == "soup" else scenes.heightfield(grid=size, seed=seed)
    bvh = gpu_build(tris)
    assert np.array_equal(bvh.morton_codes(), oracle.morton_codes(tris))
    nodes, idx = bvh.export_bvh2()
    ref = oracle.build_karras(tris)
    assert_same_tree(nodes, idx, ref)
    n, nn, height = bvh.counts
    assert n == len(tris) and nn == 2 * len(tris) - 1
    assert height + 1 == ref.depth   # inner levels on the longest path = depth - 1


def test_duplicate_centroids_order_by_index(oracle):
    base = scenes.soup(1, seed=1)
    tris = np.repeat(base, 300)
    tris["prim_id"] = np.arange(300)
    bvh = gpu_build(tris)
    nodes, idx = bvh.export_bvh2()
    assert_same_tree(nodes, idx, oracle.build_karras(tris))


def test_flat_scene_degenerate_axis(oracle):
    # all centroids on z = 0.5: size.z = 0 makes the quantised z NaN -> 1023 (lbvh.h:256-263)
    tris = scenes.soup(5000, seed=9)
    tris["v1"][:, 2] = 0.5
    tris["e1"][:, 2] = 0.0
    tris["e2"][:, 2] = 0.0
    bvh = gpu_build(tris)
    assert np.array_equal(bvh.morton_codes(), oracle.morton_codes(tris))
    nodes, idx = bvh.export_bvh2()
    assert_same_tree(nodes, idx, oracle.build_karras(tris))


def test_single_and_empty():
    one = scenes.soup(1, seed=2)
    bvh = gpu_build(one)
    nodes, idx = bvh.export_bvh2()
    assert len(nodes) == 1 and nodes["num_prims"][0] == 1 and nodes["first"][0] == 0
    empty = vg.lbvh_builder().build(np.zeros(0, vg.TRIANGLE))
    assert empty.counts == (0, 0, 0)


def test_host_and_device_builds_agree():
    tris = scenes.soup(4096, seed=21)
    a = vg.lbvh_builder().build(tris).export_bvh2()
    b = gpu_build(tris).export_bvh2()
    assert a[0].tobytes() == b[0].tobytes() and np.array_equal(a[1], b[1])


def test_rebuild_reuses_context_scratch():
    ctx = vg.default_context()
    before = ctx.launches
    for seed in (1, 2):
        gpu_build(scenes.soup(30000, seed=seed))
    assert ctx.launches > before
    ctx.synchronize()


@pytest.mark.parametrize("n", [1, 2, 777, 50000])
def test_refit_equals_reference_refitter(oracle, n):
    """gbrt_bvh_refit = bvh_refitter::refit on the exported tree (pinned to the
    reference by tests/test_oracle_reference.py), and queries on the refitted tree find
    the moved triangles."""
    from oracle import Tree
    from .parity import compare_closest
    tris = scenes.soup(n, seed=31, offset=0.02)
    moved = tris.copy()
    rng = np.random.default_rng(n)
    moved["v1"] += rng.uniform(-0.1, 0.1, size=(n, 3)).astype(np.float32)
    moved["e2"] *= np.float32(0.7)
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    nodes0, idx0 = bvh.export_bvh2()
    bvh.refit(vg.as_device_bytes(moved))
    nodes1, idx1 = bvh.export_bvh2()
    want = oracle.refit(Tree(nodes0, idx0), moved)
    assert nodes1.tobytes() == want.nodes.tobytes()
    assert np.array_equal(idx1, idx0)
    rays = scenes.pinhole_rays(64, 64)
    got = vg.hits_to_numpy(vg.closest_hit(vg.device_rays(rays), bvh))
    bvh.ctx.synchronize()
    compare_closest(got, oracle.trace(oracle.build_sah(moved), moved, rays), rays, moved, oracle)


def test_refit_rejects_other_counts():
    tris = scenes.soup(100, seed=2)
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    with pytest.raises(vg.GbrtError):
        bvh.refit(vg.as_device_bytes(tris[:99]))


@pytest.mark.parametrize("n", [1, 2, 3, 5000, 120000])
def test_rebuild_equals_fresh_build(oracle, n):
    """gbrt_bvh_rebuild_lbvh: a full rebuild of new positions of the same number of
    triangles, written into the tree's own arrays; the result equals a fresh build of
    those triangles and the oracle's restatement of visionaray's GPU builder, and a
    rebuild after the first allocates no device memory."""
    import torch
    a = scenes.soup(n, seed=50 + n)
    b = scenes.soup(n, seed=90 + n, offset=0.05)
    bvh = gpu_build(a)
    d_b = vg.as_device_bytes(b)
    bvh.rebuild(d_b)
    nodes, idx = bvh.export_bvh2()
    fresh = gpu_build(b).export_bvh2()
    assert nodes.tobytes() == fresh[0].tobytes() and np.array_equal(idx, fresh[1])
    assert_same_tree(nodes, idx, oracle.build_karras(b))
    d_a = vg.as_device_bytes(a)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    bvh.rebuild(d_a)
    bvh.ctx.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert_same_tree(*bvh.export_bvh2(), oracle.build_karras(a))


def test_rebuild_is_seen_by_a_path_tracing_scene():
    from visionaray_gb300.types import AREA_LIGHT, MATERIAL
    a, b = scenes.soup(3000, seed=61, offset=0.03), scenes.soup(3000, seed=62, offset=0.03)
    mats = np.zeros(1, MATERIAL)
    mats["color"], mats["scale"] = (0.6, 0.7, 0.8), 1.0
    cam = scenes.box_camera(eye=(0.5, 0.5, -1.0), center=(0.5, 0.5, 0.5), fovy_degrees=45.0)
    params = scenes.pt_params(40, 32, 2, num_bounces=3, ambient=(1.0, 1.0, 1.0))
    bvh = gpu_build(a)
    scene = vg.PTScene(bvh, mats, np.zeros(0, AREA_LIGHT))
    bvh.rebuild(vg.as_device_bytes(b))
    got = vg.pathtrace_frame(scene, cam, params).cpu().numpy()
    other = gpu_build(b)
    want = vg.pathtrace_frame(vg.PTScene(other, mats, np.zeros(0, AREA_LIGHT)), cam, params).cpu().numpy()
    assert got.tobytes() == want.tobytes()


def test_rebuild_rejects_other_counts_and_trees():
    tris = scenes.soup(100, seed=2)
    bvh = gpu_build(tris)
    with pytest.raises(vg.GbrtError):
        bvh.rebuild(vg.as_device_bytes(tris[:99]))
    ploc = vg.ploc_builder().build(vg.as_device_bytes(tris))
    with pytest.raises(vg.GbrtError):
        ploc.rebuild(vg.as_device_bytes(tris))
