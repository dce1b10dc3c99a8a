"""closest_hit / any_hit on the GPU against the oracle (visionaray's CPU traversal).

prim_id must match except for documented equal-t ties (re-verified with the oracle's
triangle test); t, u, v within 2 ulp where the triangle agrees (in practice
bit-exact: the device test rounds every operation as the reference does)."""
import numpy as np
import pytest
import torch

import visionaray_gb300 as vg
from visionaray_gb300 import scenes
from visionaray_gb300.types import NO_HIT, RAY, TRIANGLE

from .parity import compare_any, compare_closest, non_finite_soup

pytestmark = pytest.mark.gpu


def trace(bvh, rays, any_hit=False):
    d = vg.device_rays(rays)
    out = (vg.any_hit if any_hit else vg.closest_hit)(d, bvh)
    bvh.ctx.synchronize()
    return vg.hits_to_numpy(out)


@pytest.fixture(scope="module")
def soup_case(oracle):
    tris = scenes.soup(65536, seed=1)
    rays = scenes.pinhole_rays(1024, 1024)
    sah = oracle.build_sah(tris)
    ref_closest = oracle.trace(sah, tris, rays)
    ref_any = oracle.trace(sah, tris, rays, any_hit=True)
    return tris, rays, sah, ref_closest, ref_any


def test_soup_lbvh_closest_hit(oracle, soup_case):
    tris, rays, _, ref_closest, _ = soup_case
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    got = trace(bvh, rays)
    stats = compare_closest(got, ref_closest, rays, tris, oracle)
    assert stats["hits"] > 500000
    assert stats["exact_t"] == 1.0 and stats["exact_u"] == 1.0 and stats["exact_v"] == 1.0


def test_soup_lbvh_any_hit(oracle, soup_case):
    tris, rays, _, _, ref_any = soup_case
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    compare_any(trace(bvh, rays, any_hit=True), ref_any, rays, tris, oracle)


def test_uploaded_sah_tree(oracle, soup_case):
    tris, rays, sah, ref_closest, ref_any = soup_case
    bvh = vg.IndexBVH.upload(sah.nodes, sah.indices, tris)
    compare_closest(trace(bvh, rays), ref_closest, rays, tris, oracle)
    compare_any(trace(bvh, rays, any_hit=True), ref_any, rays, tris, oracle)


def test_host_buffer_path_equals_device_path(soup_case):
    tris, rays, _, _, _ = soup_case
    bvh = vg.lbvh_builder().build(tris)
    dev = trace(bvh, rays)
    host = vg.closest_hit(rays, bvh)
    assert host.tobytes() == dev.tobytes()
    host_any = vg.any_hit(rays, bvh)
    assert ((host_any["prim_id"] != NO_HIT) == (trace(bvh, rays, True)["prim_id"] != NO_HIT)).all()


@pytest.mark.parametrize("chunk", [1 << 16, 1 << 17])
def test_host_buffer_path_in_chunks(soup_case, chunk):
    """Small host chunks: the query runs as a quarter chunk, full chunks, the rest and
    a quarter chunk on alternating slots (a query of at most one chunk as a quarter, a
    half and a quarter of itself); hits equal the device path's bit for bit."""
    tris, rays, _, _, _ = soup_case
    ctx = vg.Context(0)
    ctx.set_host_chunk(chunk)
    bvh = vg.lbvh_builder(ctx).build(tris)
    dev = trace(bvh, rays)
    assert len(rays) > 4 * chunk
    host = vg.closest_hit(rays, bvh)
    assert host.tobytes() == dev.tobytes()
    odd = rays[: 2 * chunk + 12345]
    assert vg.closest_hit(odd, bvh).tobytes() == dev[: len(odd)].tobytes()
    small = rays[: chunk - 7]   # a quarter, a half and a quarter of itself
    assert vg.closest_hit(small, bvh).tobytes() == dev[: len(small)].tobytes()
    with pytest.raises(vg.runtime.GbrtError):
        ctx.set_host_chunk(1000)


@pytest.mark.parametrize("grid", [64, 512])
def test_heightfield_secondary_and_ao(oracle, grid):
    tris = scenes.heightfield(grid=grid, seed=1)
    closest, ao = scenes.surface_rays(tris, 65536, seed=7)
    tree = oracle.build_karras(tris)
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    compare_closest(trace(bvh, closest), oracle.trace(tree, tris, closest), closest, tris, oracle)
    compare_any(trace(bvh, ao, any_hit=True), oracle.trace(tree, tris, ao, any_hit=True), ao, tris, oracle)


def test_kat_triangles_on_gpu():
    # test/unittests/math/intersect.cpp:60-121: planes x = -3, -2, -1, -0
    tris = np.zeros(4, TRIANGLE)
    for i, x in enumerate((-3.0, -2.0, -1.0, -0.0)):
        v1 = np.array((x, -1, -1), np.float32)
        tris[i]["v1"] = v1
        tris[i]["e1"] = np.array((x, -1, 1), np.float32) - v1
        tris[i]["e2"] = np.array((x, 1, 0), np.float32) - v1
        tris[i]["prim_id"] = i
    r = np.zeros(3, RAY)
    r["ori"] = (-2.0, 0.0, 0.0)
    r["dir"] = (1.0, 0.0, 0.0)
    r["tmax"] = vg.FLT_MAX
    r["tmin"] = (0.0, 0.5, 3.0)
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    h = trace(bvh, r)
    assert list(h["prim_id"]) == [1, 2, NO_HIT]
    assert list(h["t"][:2]) == [0.0, 1.0]


def test_edge_case_rays(oracle):
    tris = scenes.soup(5000, seed=3, offset=0.05)
    rng = np.random.default_rng(1)
    n = 20000
    r = np.zeros(n, RAY)
    r["ori"] = rng.uniform(-0.2, 1.2, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[: n // 4, 0] = 0.0                  # axis-parallel components -> FLT_MAX reciprocal
    d[n // 4: n // 2, 1:] = 0.0
    d[n // 2: n // 2 + 100] = -0.0        # zero direction: no triangle can be hit
    r["dir"] = d
    r["tmax"] = vg.FLT_MAX
    r["tmin"][-100:] = 5.0                # tmin > tmax of anything inside
    r["tmax"][-100:] = 1.0
    tree = oracle.build_karras(tris)
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    compare_closest(trace(bvh, r), oracle.trace(tree, tris, r), r, tris, oracle)
    compare_any(trace(bvh, r, True), oracle.trace(tree, tris, r, any_hit=True), r, tris, oracle)


def test_empty_and_single_triangle_trees(oracle):
    rays = scenes.pinhole_rays(32, 32)
    empty = vg.lbvh_builder().build(np.zeros(0, TRIANGLE))
    h = trace(empty, rays)
    assert (h["prim_id"] == NO_HIT).all() and (h["t"] == vg.FLT_MAX).all()
    one = scenes.soup(1, seed=4, offset=0.4)
    one["v1"] = (0.1, 0.1, 0.5)
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(one))
    got = trace(bvh, rays)
    ref = oracle.trace_linear(one, rays)
    assert got.tobytes() == ref.tobytes()
    assert (got["prim_id"] == 0).sum() > 0


def test_zero_rays_and_status_clean():
    tris = scenes.soup(100, seed=5)
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    out = vg.closest_hit(torch.empty((0, 8), device="cuda"), bvh)
    assert out.shape[0] == 0
    bvh.ctx.synchronize()   # no stack overflow or bad index was flagged


def test_full_size_heightfield_sample(oracle):
    """The 2048x2048 heightfield (8,388,608 triangles) built on the GPU, traced with
    4M secondary rays; a fixed sample of rays is checked against the oracle's trace of
    the restated reference GPU tree, and the whole build against the restatement."""
    tris = scenes.heightfield(grid=2048, seed=1)
    closest, ao = scenes.surface_rays(tris, 1 << 22, seed=7)
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    nodes, idx = bvh.export_bvh2()
    ref = oracle.build_karras(tris)
    assert np.array_equal(nodes["first"], ref.nodes["first"])
    assert (nodes["bbox_min"] == ref.nodes["bbox_min"]).all()
    got_c = trace(bvh, closest)
    got_a = trace(bvh, ao, any_hit=True)
    sel = np.arange(0, len(closest), 97)
    compare_closest(got_c[sel], oracle.trace(ref, tris, closest[sel]), closest[sel], tris, oracle)
    sel_a = np.arange(0, len(ao), 389)
    compare_any(got_a[sel_a], oracle.trace(ref, tris, ao[sel_a], any_hit=True), ao[sel_a], tris, oracle)


def test_sorted_ray_order_gives_identical_hits():
    """GBRT_TRACE_SORT_RAYS changes only the order rays are traced in."""
    tris = scenes.heightfield(grid=512, seed=3)
    closest, ao = scenes.surface_rays(tris, 1 << 18, seed=9)
    ctx = vg.Context(0)
    bvh = vg.lbvh_builder(ctx).build(vg.as_device_bytes(tris))
    plain = [vg.hits_to_numpy(f(vg.device_rays(r), bvh)) for f, r in ((vg.closest_hit, closest), (vg.any_hit, ao))]
    ctx.set_trace_flags(ctx.TRACE_SORT_RAYS)
    srt = [vg.hits_to_numpy(f(vg.device_rays(r), bvh)) for f, r in ((vg.closest_hit, closest), (vg.any_hit, ao))]
    host = vg.closest_hit(closest, bvh)
    ctx.synchronize()
    assert plain[0].tobytes() == srt[0].tobytes()
    assert plain[1].tobytes() == srt[1].tobytes()
    assert host.tobytes() == plain[0].tobytes()


@pytest.mark.parametrize("refill", [1, 8, 32])
def test_persistent_traversal_gives_identical_hits(refill):
    """GBRT_TRACE_PERSISTENT (with and without the ray order) changes only which lane
    traces which ray and when; every hit is the one-thread-per-ray kernel's."""
    tris = scenes.heightfield(grid=512, seed=3)
    closest, ao = scenes.surface_rays(tris, 1 << 18, seed=9)
    ctx = vg.Context(0)
    bvh = vg.lbvh_builder(ctx).build(vg.as_device_bytes(tris))
    queries = ((vg.closest_hit, closest), (vg.any_hit, ao), (vg.closest_hit, closest[:1000]))
    plain = [vg.hits_to_numpy(f(vg.device_rays(r), bvh)) for f, r in queries]
    ctx.set_trace_refill(refill)
    for flags in (ctx.TRACE_PERSISTENT, ctx.TRACE_PERSISTENT | ctx.TRACE_SORT_RAYS):
        ctx.set_trace_flags(flags)
        got = [vg.hits_to_numpy(f(vg.device_rays(r), bvh)) for f, r in queries]
        host = vg.any_hit(ao, bvh)
        ctx.synchronize()
        for g, p in zip(got, plain):
            assert g.tobytes() == p.tobytes(), f"flags {flags}"
        assert host.tobytes() == plain[1].tobytes()


def test_wide_and_binary_nodes_agree(oracle):
    """The 4-wide collapse changes the traversal, not the answers."""
    tris = scenes.heightfield(grid=256, seed=5)
    closest, ao = scenes.surface_rays(tris, 1 << 16, seed=11)
    ctx = vg.Context(0)
    ctx.set_trace_flags(ctx.TRACE_WIDE_NODES)
    bvh = vg.lbvh_builder(ctx).build(vg.as_device_bytes(tris))
    wide_c, wide_a = trace(bvh, closest), trace(bvh, ao, any_hit=True)
    ctx.set_trace_flags(0)
    bin_c, bin_a = trace(bvh, closest), trace(bvh, ao, any_hit=True)
    compare_closest(wide_c, bin_c, closest, tris, oracle)
    assert ((wide_a["prim_id"] != NO_HIT) == (bin_a["prim_id"] != NO_HIT)).all()


@pytest.mark.parametrize("sort", [0, 1])
def test_eight_wide_nodes_agree(oracle, sort):
    """The 8-wide collapse (bvh_collapser's BVH8) changes the traversal, not the
    answers: closest hits as the node pairs' (equal-t ties aside) and every AO ray's
    occlusion; a soup against the oracle's SAH tree."""
    tris = scenes.heightfield(grid=256, seed=5)
    closest, ao = scenes.surface_rays(tris, 1 << 16, seed=11)
    ctx = vg.Context(0)
    ctx.set_trace_flags(ctx.TRACE_WIDE8_NODES | sort)
    bvh = vg.lbvh_builder(ctx).build(vg.as_device_bytes(tris))
    w_c, w_a = trace(bvh, closest), trace(bvh, ao, any_hit=True)
    ctx.set_trace_flags(sort)
    bin_c, bin_a = trace(bvh, closest), trace(bvh, ao, any_hit=True)
    compare_closest(w_c, bin_c, closest, tris, oracle)
    assert ((w_a["prim_id"] != NO_HIT) == (bin_a["prim_id"] != NO_HIT)).all()
    soup = scenes.soup(20000, seed=3)
    rays = scenes.pinhole_rays(256, 256)
    ctx.set_trace_flags(ctx.TRACE_WIDE8_NODES)
    bvh2 = vg.lbvh_builder(ctx).build(vg.as_device_bytes(soup))
    got = trace(bvh2, rays)
    compare_closest(got, oracle.trace(oracle.build_sah(soup), soup, rays), rays, soup, oracle)


@pytest.mark.parametrize("grid,sort", [(256, 0), (512, 1)])
def test_compressed_nodes_agree(oracle, grid, sort):
    """The quantised 4-wide nodes (bvh_compressed_node<4> layout, boxes rounded outward)
    change the traversal, not the answers: closest hits as the node pairs' (equal-t ties
    aside) and every AO ray's occlusion."""
    tris = scenes.heightfield(grid=grid, seed=5)
    closest, ao = scenes.surface_rays(tris, 1 << 16, seed=11)
    ctx = vg.Context(0)
    ctx.set_trace_flags(ctx.TRACE_COMPRESSED_NODES | sort)
    bvh = vg.lbvh_builder(ctx).build(vg.as_device_bytes(tris))
    q_c, q_a = trace(bvh, closest), trace(bvh, ao, any_hit=True)
    ctx.set_trace_flags(sort)
    bin_c, bin_a = trace(bvh, closest), trace(bvh, ao, any_hit=True)
    compare_closest(q_c, bin_c, closest, tris, oracle)
    assert ((q_a["prim_id"] != NO_HIT) == (bin_a["prim_id"] != NO_HIT)).all()
    soup = scenes.soup(20000, seed=3)
    rays = scenes.pinhole_rays(256, 256)
    ctx.set_trace_flags(ctx.TRACE_COMPRESSED_NODES)
    bvh2 = vg.lbvh_builder(ctx).build(vg.as_device_bytes(soup))
    got = trace(bvh2, rays)
    ref = oracle.trace(oracle.build_sah(soup), soup, rays)
    compare_closest(got, ref, rays, soup, oracle)


def test_degenerate_and_non_finite_triangles(oracle):
    """Zero-area, NaN and Inf triangles: the build and the queries complete without a
    flagged fault, no ray hits a bad triangle, and the tree is the reference GPU
    builder's for the same input (the oracle's restatement, traversed on the CPU): its
    atomic bottom-up bounds skip NaN, so every ray's closest hit is the brute-force one."""
    tris = non_finite_soup()
    rays = scenes.pinhole_rays(256, 256)
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    got = trace(bvh, rays)
    got_any = trace(bvh, rays, any_hit=True)
    ref = oracle.trace(oracle.build_karras(tris), tris, rays)
    compare_closest(got, ref, rays, tris, oracle)
    hit = got["prim_id"] != NO_HIT
    assert (got["prim_id"][hit] < 10000).sum() + (got["prim_id"][hit] >= 10060).sum() == hit.sum()
    assert ((got_any["prim_id"] != NO_HIT) == hit).all()
    lin = oracle.trace_linear(tris, rays)
    compare_closest(got, lin, rays, tris, oracle)
