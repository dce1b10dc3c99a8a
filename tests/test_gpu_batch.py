"""Batched build, ray queries and path tracing against the per-scene path.

A batch holds many scenes in one arena; its contract is that every scene comes out as
if it had been built and rendered alone: trees byte-identical to gbrt_bvh_build_lbvh's,
hits bit-identical to gbrt_trace_closest_hit's, images bit-identical to
gbrt_pathtrace_frame's.  A subset of scenes is also checked against the CPU oracle
(closest-hit parity as for the single-scene path)."""
import numpy as np
import pytest
import torch

import visionaray_gb300 as vg
from visionaray_gb300 import scenes
from visionaray_gb300.types import BATCH_ORDER_BLOCKS, BATCH_ORDER_ROWS, TRIANGLE

from .parity import compare_closest

pytestmark = pytest.mark.gpu

# uneven scenes, including an empty one and one- and two-triangle ones
COUNTS = [700, 0, 1, 2, 3, 17, 4096, 1, 250, 9000, 33, 1500]


def make_batch_inputs(counts, seed=5, sides=(32, 64, 48, 16)):
    offsets = np.zeros(len(counts) + 1, np.uint32)
    offsets[1:] = np.cumsum(counts)
    tris = np.empty(int(offsets[-1]), TRIANGLE)
    cams, params = [], []
    for s, n in enumerate(counts):
        if n:
            tris[offsets[s]:offsets[s + 1]] = scenes.soup(n, seed=seed * 100 + s, offset=0.5 / max(n, 1) ** (1 / 3))
        d = np.array([np.sin(1.3 * s + 0.4), 0.35, np.cos(1.3 * s + 0.4)])
        d = d / np.linalg.norm(d)
        cam = scenes.box_camera(eye=tuple(0.5 + 1.7 * d), center=(0.5, 0.5, 0.5), fovy_degrees=50.0)
        side = sides[s % len(sides)]
        cams.append(cam)
        params.append(scenes.pt_params(side, side + 8 * (s % 2), 2, num_bounces=3, frame_id=7 + s,
                                       ambient=(1.0, 0.9, 0.8), background=(0.1, 0.2, 0.3, 1.0)))
    mats = np.zeros(1, vg.types.MATERIAL)
    mats["kind"], mats["color"], mats["scale"] = 0, (0.7, 0.6, 0.5), 1.0
    return tris, offsets, np.array(cams), np.array(params), mats


@pytest.fixture(scope="module")
def batch_setup():
    tris, offsets, cams, params, mats = make_batch_inputs(COUNTS)
    d_tris = vg.as_device_bytes(tris)
    batch = vg.Batch(offsets)
    batch.build(d_tris)
    batch.set_frames(cams, params, mats)
    batch.ctx.synchronize()
    return tris, offsets, cams, params, mats, d_tris, batch


def scene_tris(tris, offsets, s):
    return tris[int(offsets[s]):int(offsets[s + 1])]


def test_batch_trees_equal_single_scene_builds(batch_setup):
    tris, offsets, _, _, _, _, batch = batch_setup
    for s in range(len(COUNTS)):
        t = scene_tris(tris, offsets, s)
        if len(t) == 0:
            continue
        nodes, idx = batch.export_bvh2(s)
        ref_nodes, ref_idx = vg.lbvh_builder().build(vg.as_device_bytes(t)).export_bvh2()
        assert nodes.tobytes() == ref_nodes.tobytes(), f"scene {s}: nodes differ"
        assert np.array_equal(idx, ref_idx), f"scene {s}: indices differ"


def test_batch_height_is_tallest_tree(batch_setup):
    tris, offsets, _, _, _, _, batch = batch_setup
    heights = []
    for s in range(len(COUNTS)):
        t = scene_tris(tris, offsets, s)
        if len(t):
            heights.append(vg.lbvh_builder().build(vg.as_device_bytes(t)).counts[2])
    assert batch.height() == max(heights)


def test_batch_closest_hit_bit_identical_and_oracle(batch_setup, oracle):
    tris, offsets, _, _, _, _, batch = batch_setup
    rays_per = []
    for s in range(len(COUNTS)):
        r = scenes.pinhole_rays(24 + s, 20, eye=(0.5, 0.5, -1.5 + 0.01 * s))
        rays_per.append(r)
    ray_offsets = np.zeros(len(COUNTS) + 1, np.uint32)
    ray_offsets[1:] = np.cumsum([len(r) for r in rays_per])
    all_rays = np.concatenate(rays_per)
    d_rays = vg.device_rays(all_rays)
    hits = vg.hits_to_numpy(batch.closest_hit(d_rays, ray_offsets))
    batch.ctx.synchronize()
    for s in range(len(COUNTS)):
        got = hits[ray_offsets[s]:ray_offsets[s + 1]]
        t = scene_tris(tris, offsets, s)
        bvh = vg.lbvh_builder().build(vg.as_device_bytes(t))
        ref = vg.hits_to_numpy(vg.closest_hit(vg.device_rays(rays_per[s]), bvh))
        assert got.tobytes() == ref.tobytes(), f"scene {s}: hits differ from the single-scene query"
        if s in (0, 6, 9) and len(t):
            orc = oracle.trace(oracle.build_sah(t), t, rays_per[s], any_hit=False)
            compare_closest(got, orc, rays_per[s], t, oracle)


def plain_images(tris, offsets, cams, params, mats):
    out = []
    for s in range(len(offsets) - 1):
        t = scene_tris(tris, offsets, s)
        bvh = vg.lbvh_builder().build(vg.as_device_bytes(t))
        sc = vg.PTScene(bvh, mats, np.zeros(0, vg.types.AREA_LIGHT))
        img = vg.pathtrace_frame(sc, cams[s], params[s])
        bvh.ctx.synchronize()
        out.append(img.cpu().numpy())
    return out


@pytest.fixture(scope="module")
def plain(batch_setup):
    tris, offsets, cams, params, mats, _, _ = batch_setup
    return plain_images(tris, offsets, cams, params, mats)


LAUNCHES = [(128, 32, 64, BATCH_ORDER_ROWS), (256, 64, 32, BATCH_ORDER_BLOCKS), (512, 32, 24, BATCH_ORDER_BLOCKS),
            (128, 64, 64, BATCH_ORDER_BLOCKS)]


@pytest.mark.parametrize("launch", LAUNCHES)
def test_batch_pathtrace_bit_identical(batch_setup, plain, launch):
    _, _, _, params, _, _, batch = batch_setup
    height = batch.height()
    if launch[2] < height:
        pytest.skip(f"stack {launch[2]} below the tallest tree ({height})")
    batch.launch = launch
    images = batch.pathtrace()
    batch.ctx.synchronize()
    for s in range(len(COUNTS)):
        got = batch.image(images, s, params).cpu().numpy()
        assert got.tobytes() == plain[s].tobytes(), f"scene {s}: image differs (launch {launch})"


@pytest.mark.parametrize("width,sort", [(2, 1), (4, 0), (4, 1), (8, 0), (8, 1)])
def test_batch_widths_and_sorted_order(batch_setup, plain, width, sort):
    """BVH width 4 and 8 (the arena's trees collapsed each frame) and the sorted pixel
    order (pixels grouped by their first primary hit): every scene's image equals its
    per-scene frame -- bit for bit through the node pairs; through the wide nodes the
    triangles of a leaf are visited in another order, so a pixel whose path met an
    equal-t tie may differ (the soups have none measurable: at most one pixel per scene
    is allowed).  Directly and replayed from a graph."""
    tris, offsets, cams, params, mats, d_tris, batch = batch_setup
    batch.launch = (256, 32, 64, BATCH_ORDER_BLOCKS, width, sort)
    assert (int(batch.launch["width"]), int(batch.launch["sort"])) == (width, sort)
    for run in ("direct", "graph"):
        images = batch.new_images()
        images.fill_(-1.0)
        if run == "direct":
            batch.pathtrace(images)
        else:
            batch.run_graph(d_tris, images)
        batch.ctx.synchronize()
        for s in range(len(COUNTS)):
            got = batch.image(images, s, params).cpu().numpy()
            if width == 2:
                assert got.tobytes() == plain[s].tobytes(), (run, s)
            else:
                differ = int((got != plain[s]).any(axis=2).sum())
                assert differ <= 1, (run, s, differ)
    batch.launch = (128, 32, 64, BATCH_ORDER_ROWS)


def test_batch_graph_replay_and_recapture(batch_setup, plain):
    tris, offsets, cams, params, mats, d_tris, batch = batch_setup
    batch.launch = (128, 32, 64, BATCH_ORDER_ROWS)
    images = batch.new_images()
    ctx = batch.ctx
    before = ctx.launches
    for _ in range(2):
        images.fill_(-1.0)
        batch.run_graph(d_tris, images)
        ctx.synchronize()
        for s in range(len(COUNTS)):
            assert batch.image(images, s, params).cpu().numpy().tobytes() == plain[s].tobytes()
    assert ctx.launches > before   # replays count their kernels
    # new triangles at another address: the graph is captured again
    moved = tris.copy()
    for f in ("v1",):
        moved[f] = moved[f] + np.float32(0.01)
    d_moved = vg.as_device_bytes(moved)
    batch.run_graph(d_moved, images)
    ctx.synchronize()
    ref = plain_images(moved, offsets, cams, params, mats)
    for s in range(len(COUNTS)):
        assert batch.image(images, s, params).cpu().numpy().tobytes() == ref[s].tobytes()
    batch.build(d_tris)   # leave the fixture's trees as they were
    ctx.synchronize()


def test_batch_autotune_picks_a_clean_shape(batch_setup, plain):
    _, _, _, params, _, _, batch = batch_setup
    images = batch.new_images()
    best, ms = batch.autotune(images, reps=1)
    assert ms > 0.0
    assert int(best["stack"]) >= batch.height()
    assert int(best["width"]) in (2, 4, 8) and int(best["sort"]) in (0, 1)
    assert tuple(int(x) for x in batch.launch) == tuple(int(x) for x in best)
    batch.launch = tuple(int(x) for x in best)[:4]   # the node pairs, unsorted: bit for bit
    images = batch.pathtrace()
    batch.ctx.synchronize()
    for s in range(len(COUNTS)):
        assert batch.image(images, s, params).cpu().numpy().tobytes() == plain[s].tobytes()


def test_batch_materials_bit_identical():
    """A shared material table with matte, mirror, glass and plastic slots (geom_id =
    prim_id mod 4): batched images equal the per-scene frames bit for bit."""
    from visionaray_gb300.types import GLASS, MATERIAL, MIRROR, PLASTIC
    counts = [900, 3, 2500, 0, 60]
    tris, offsets, cams, params, _ = make_batch_inputs(counts, seed=9)
    tris["geom_id"] = tris["prim_id"] % 4
    mats = np.zeros(4, MATERIAL)
    mats["kind"] = (0, MIRROR, GLASS, PLASTIC)
    mats["color"] = ((0.7, 0.6, 0.5), (0.9, 0.9, 0.8), (1.0, 1.0, 1.0), (0.2, 0.5, 0.7))
    mats["scale"] = 1.0
    mats["ior"] = ((1.0, 1.0, 1.0), (0.27, 0.42, 1.35), (1.5, 1.5, 1.5), (1.0, 1.0, 1.0))
    mats["absorption"][1] = (3.4, 2.3, 1.8)
    mats["color2"][2], mats["scale2"][2] = (1.0, 1.0, 1.0), 1.0
    mats["color2"][3], mats["scale2"][3], mats["exponent"][3] = (0.5, 0.5, 0.5), 1.0, 24.0
    params["num_bounces"] = 6
    d_tris = vg.as_device_bytes(tris)
    batch = vg.Batch(offsets)
    batch.build(d_tris)
    batch.set_frames(cams, params, mats)
    images = batch.pathtrace()
    batch.ctx.synchronize()
    ref = plain_images(tris, offsets, cams, params, mats)
    for s in range(len(counts)):
        assert batch.image(images, s, params).cpu().numpy().tobytes() == ref[s].tobytes(), s


def test_batch_short_stack_reports_overflow():
    # 140,000 copies of one tilted triangle: equal Morton codes give a balanced tree of
    # height 18 whose boxes all overlap, so the first descent pushes at every level
    n = 140000
    tris = np.zeros(n, TRIANGLE)
    tris["v1"] = (0.3, 0.3, 0.4)
    tris["e1"] = (0.4, 0.05, 0.1)
    tris["e2"] = (0.05, 0.4, 0.15)
    tris["prim_id"] = np.arange(n, dtype=np.uint32)
    offsets = np.array([0, n], np.uint32)
    cam = scenes.box_camera(eye=(0.5, 0.5, -1.5), center=(0.5, 0.5, 0.5), fovy_degrees=30.0)
    params = np.array([scenes.pt_params(16, 16, 1, num_bounces=1, ambient=(1.0, 1.0, 1.0))])
    mats = np.zeros(1, vg.types.MATERIAL)
    batch = vg.Batch(offsets)
    batch.build(vg.as_device_bytes(tris))
    batch.set_frames(np.array([cam]), params, mats)
    assert batch.height() > 16
    batch.launch = (128, 32, 16, BATCH_ORDER_ROWS)
    batch.pathtrace()
    with pytest.raises(vg.GbrtError) as e:
        batch.ctx.synchronize()
    assert e.value.status == 5
    batch.ctx.synchronize()   # the status was cleared
    batch.launch = (128, 32, 64, BATCH_ORDER_ROWS)
    batch.pathtrace()
    batch.ctx.synchronize()


def test_batch_rejects_bad_arguments():
    with pytest.raises(vg.GbrtError):
        vg.Batch(np.array([0, 5, 3], np.uint32))
    batch = vg.Batch(np.array([0, 4], np.uint32))
    with pytest.raises(vg.GbrtError):
        batch.launch = (100, 32, 64, 0)
    with pytest.raises(vg.GbrtError):
        batch.pathtrace(torch.empty((4, 4), dtype=torch.float32, device="cuda:0"))   # frames not set


def test_batch_rejects_unknown_material_kind():
    from visionaray_gb300.runtime import GbrtError
    tris, offsets, cams, params, mats = make_batch_inputs([50, 60])
    batch = vg.Batch(offsets)
    batch.build(vg.as_device_bytes(tris))
    mats["kind"][0] = 5
    with pytest.raises(GbrtError, match="unknown material kind"):
        batch.set_frames(cams, params, mats)


def test_lit_batch_equals_per_scene_frames():
    """Scenes with area lights: five box scenes of different seeds in one batch, one
    material table for all (each scene's geom_ids offset into it), scene s sampling its
    own two ceiling lights -- scene 3 has none and keeps the ambient light.  Each
    scene's batched image equals gbrt_pathtrace_frame's with that scene's lights, bit
    for bit, under two launch shapes."""
    parts, mat_parts, light_parts, light_offsets = [], [], [], [0]
    slot = 0
    for s in range(5):
        t, m, lights = scenes.box_scene(n_blobs=2 + s, subdiv=3, seed=10 + s)
        t = t.copy()
        t["geom_id"] += slot
        lights = lights.copy()
        lights["geometry"]["geom_id"] += slot
        if s == 3:
            lights = lights[:0]
        parts.append(t)
        mat_parts.append(m)
        light_parts.append(lights)
        light_offsets.append(light_offsets[-1] + len(lights))
        slot += len(m)
    tris = np.concatenate(parts)
    mats = np.concatenate(mat_parts)
    lights = np.concatenate(light_parts)
    offsets = np.zeros(len(parts) + 1, np.uint32)
    offsets[1:] = np.cumsum([len(p) for p in parts])
    cam = scenes.box_camera()
    cams = np.array([cam] * len(parts))
    params = np.array([scenes.pt_params(32 + 8 * s, 24 + 4 * s, 2, num_bounces=5, frame_id=3 + s,
                                        ambient=(0.2, 0.2, 0.2)) for s in range(len(parts))])
    batch = vg.Batch(offsets)
    batch.build(vg.as_device_bytes(tris))
    batch.set_frames(cams, params, mats)
    batch.set_lights(lights, light_offsets)
    want = []
    for s, t in enumerate(parts):
        bvh = vg.lbvh_builder().build(vg.as_device_bytes(t))
        img = vg.pathtrace_frame(vg.PTScene(bvh, mats, light_parts[s]), cam, params[s])
        bvh.ctx.synchronize()
        want.append(img.cpu().numpy())
    for launch in [(128, 32, 64, BATCH_ORDER_ROWS), (256, 64, 32, BATCH_ORDER_BLOCKS)]:
        batch.launch = launch
        images = batch.pathtrace()
        batch.ctx.synchronize()
        for s in range(len(parts)):
            got = batch.image(images, s, params).cpu().numpy()
            assert got.tobytes() == want[s].tobytes(), (launch, s)
    # the lights are sampled: scene 0 without its lights renders another image
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(parts[0]))
    dark = vg.pathtrace_frame(vg.PTScene(bvh, mats, light_parts[3]), cam, params[0]).cpu().numpy()
    assert dark.tobytes() != want[0].tobytes()
