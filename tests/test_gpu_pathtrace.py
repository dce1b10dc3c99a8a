"""The wavefront path tracer on the GPU against the oracle at matched random numbers
(gbrt_rng.h).  Reference mode (visionaray's shadow range, flags = 0) is compared with
the FP32 oracle computing cos/sin of the hemisphere sample in double, as the kernel
does (otherwise the two are the same float expressions); the corrected shadow range
is compared with the FP64 oracle.  Tolerances are stated per test."""
import numpy as np
import pytest
import torch

import visionaray_gb300 as vg
from oracle import Oracle
from visionaray_gb300 import scenes
from visionaray_gb300.types import PT_SHADOW_RANGE_FIX

pytestmark = pytest.mark.gpu


def render(tris, mats, lights, cam, params, accum=None):
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    scene = vg.PTScene(bvh, mats, lights)
    out = vg.pathtrace_frame(scene, cam, params, accum=accum)
    bvh.ctx.synchronize()
    return out.cpu().numpy().astype(np.float64), bvh, scene


@pytest.fixture(scope="module")
def small_box():
    tris, mats, lights = scenes.box_scene(n_blobs=8, subdiv=8, seed=1)
    return tris, mats, lights, scenes.box_camera()


def stats(a, b):
    d = np.abs(a - b)[..., :3]
    return {"exact": float((d.max(axis=2) == 0).mean()), "rmse": float(np.sqrt((d ** 2).mean())),
            "max": float(d.max()), "mean": float(b[..., :3].mean())}


def test_reference_mode_matches_fp32_oracle(oracle, small_box):
    tris, mats, lights, cam = small_box
    params = scenes.pt_params(96, 64, 8, num_bounces=8, frame_id=11)
    gpu, _, _ = render(tris, mats, lights, cam, params)
    ref, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params,
                              mode=Oracle.PT_FLOAT_TRIG_DOUBLE)
    s = stats(gpu, ref)
    # same float operations and random numbers: almost every pixel bit-exact; the
    # rest come from equal-t ties picked in a different traversal order
    assert s["exact"] >= 0.98, s
    assert s["rmse"] <= 0.01 * s["mean"], s


def test_shadow_range_fix_matches_fp64_oracle(oracle, small_box):
    tris, mats, lights, cam = small_box
    params = scenes.pt_params(96, 64, 8, num_bounces=8, frame_id=12, flags=PT_SHADOW_RANGE_FIX)
    gpu, _, _ = render(tris, mats, lights, cam, params)
    ref, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params, mode=Oracle.PT_DOUBLE)
    s = stats(gpu, ref)
    # FP32 against FP64 at matched random numbers: RMSE within 1% of the image mean
    assert s["rmse"] <= 0.01 * s["mean"], s


def test_progressive_blend(small_box):
    tris, mats, lights, cam = small_box
    p0 = scenes.pt_params(32, 16, 2, frame_id=1)
    a, bvh, scene = render(tris, mats, lights, cam, p0)
    acc = torch.from_numpy(a.astype(np.float32)).cuda()
    p1 = scenes.pt_params(32, 16, 2, frame_id=2, sfactor=0.5, dfactor=0.5)
    vg.pathtrace_frame(scene, cam, p1, accum=acc)
    f1 = vg.pathtrace_frame(scene, cam, scenes.pt_params(32, 16, 2, frame_id=2))
    bvh.ctx.synchronize()
    expect = f1.cpu().numpy() * np.float32(0.5) + a.astype(np.float32) * np.float32(0.5)
    assert np.array_equal(acc.cpu().numpy(), expect)


def test_background_and_no_lights(oracle, small_box):
    tris, mats, lights, _ = small_box
    blobs = tris[14:].copy()
    cam = scenes.box_camera(eye=(0.5, 0.5, -3.0), center=(0.5, 0.5, 0.0), fovy_degrees=20.0)
    params = scenes.pt_params(32, 16, 1, background=(0.25, 0.5, 1.0, 2.0), ambient=(0.1, 0.2, 0.3))
    gpu, _, _ = render(blobs, mats, lights[:0], cam, params)
    ref, _ = oracle.pathtrace(oracle.build_sah(blobs), blobs, mats, lights[:0], cam, params,
                              mode=Oracle.PT_FLOAT_TRIG_DOUBLE)
    assert (gpu.reshape(-1, 4) == np.array([0.5, 1.0, 2.0, 1.0])).all(axis=1).any()
    assert stats(gpu, ref)["exact"] >= 0.98


def test_full_box_scene_reduced_resolution(oracle):
    """The 256-blob box (2,478,094 triangles) at 192x108, 2 spp: the full geometry."""
    tris, mats, lights = scenes.box_scene()
    cam = scenes.box_camera()
    params = scenes.pt_params(192, 108, 2, num_bounces=8, frame_id=4)
    gpu, _, _ = render(tris, mats, lights, cam, params)
    ref, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params,
                              mode=Oracle.PT_FLOAT_TRIG_DOUBLE)
    s = stats(gpu, ref)
    assert s["exact"] >= 0.97, s
    assert s["rmse"] <= 0.02 * s["mean"], s


@pytest.mark.parametrize("flags", [0, PT_SHADOW_RANGE_FIX, PT_SHADOW_RANGE_FIX | 2])
def test_megakernel_equals_wavefront(small_box, flags):
    """GBRT_PT_MEGAKERNEL changes the scheduling only: same image bit for bit, including
    the progressive blend and the color output."""
    from visionaray_gb300.types import PT_MEGAKERNEL
    tris, mats, lights, cam = small_box
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    scene = vg.PTScene(bvh, mats, lights)
    out = []
    for mega in (0, PT_MEGAKERNEL):
        accum = torch.zeros((48, 80, 4), dtype=torch.float32, device="cuda:0")
        color = torch.zeros_like(accum)
        for f in range(3):
            p = scenes.pt_params(80, 48, 3, num_bounces=6, frame_id=20 + f, sfactor=1.0 / (f + 1),
                                 dfactor=1.0 - 1.0 / (f + 1), flags=flags | mega)
            vg.pathtrace_frame(scene, cam, p, accum=accum, color=color)
        bvh.ctx.synchronize()
        out.append((accum.cpu().numpy(), color.cpu().numpy()))
    assert out[0][0].tobytes() == out[1][0].tobytes()
    assert out[0][1].tobytes() == out[1][1].tobytes()


def test_megakernel_equals_wavefront_ambient_and_empty():
    from visionaray_gb300.types import AREA_LIGHT, MATERIAL, PT_MEGAKERNEL
    tris = scenes.soup(5000, seed=8, offset=0.03)
    mats = np.zeros(1, MATERIAL)
    mats["color"], mats["scale"] = (0.6, 0.7, 0.8), 1.0
    cam = scenes.box_camera(eye=(0.5, 0.5, -1.0), center=(0.5, 0.5, 0.5), fovy_degrees=45.0)
    for t in (tris, tris[:0]):
        bvh = vg.lbvh_builder().build(vg.as_device_bytes(t) if len(t) else t)
        scene = vg.PTScene(bvh, mats, np.zeros(0, AREA_LIGHT))
        imgs = [vg.pathtrace_frame(scene, cam, scenes.pt_params(33, 17, 4, num_bounces=4, ambient=(1.0, 0.5, 0.25),
                                                                background=(0.1, 0.2, 0.3, 0.5), flags=m)).cpu()
                for m in (0, PT_MEGAKERNEL)]
        assert imgs[0].numpy().tobytes() == imgs[1].numpy().tobytes()


@pytest.mark.parametrize("flags", [0, PT_SHADOW_RANGE_FIX])
def test_sorted_queues_equal_unsorted(small_box, flags):
    """GBRT_PT_SORT_QUEUES orders each bounce's ray and shadow queues by origin cell;
    the paths and the image are unchanged bit for bit."""
    from visionaray_gb300.types import PT_SORT_QUEUES
    tris, mats, lights, cam = small_box
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    scene = vg.PTScene(bvh, mats, lights)
    out = []
    for extra in (0, PT_SORT_QUEUES):
        p = scenes.pt_params(96, 64, 4, num_bounces=8, frame_id=5, flags=flags | extra)
        img = vg.pathtrace_frame(scene, cam, p)
        bvh.ctx.synchronize()
        out.append(img.cpu().numpy())
    assert out[0].tobytes() == out[1].tobytes()


@pytest.fixture(scope="module", params=["specular", "glossy", "lights"])
def material_box(request):
    """Mirror and glass blobs (conductor and dielectric Fresnel, refraction, total
    internal reflection); those plus plastic blobs and walls (lobe choice, Blinn
    sampling, glossy next-event estimation); or the latter lit by area, point and spot
    lights (generic lights, delta-light sampling)."""
    if request.param == "specular":
        tris, mats, lights = scenes.specular_box_scene(n_blobs=8, subdiv=8, seed=1)
    else:
        tris, mats, lights = scenes.glossy_box_scene(n_blobs=10, subdiv=8, seed=1)
        if request.param == "lights":
            lights = scenes.mixed_lights(lights)
    return tris, mats, lights, scenes.box_camera()


def test_unknown_light_kind_is_rejected():
    from visionaray_gb300.types import LIGHT
    tris, mats, area = scenes.box_scene(n_blobs=1, subdiv=4, seed=1)
    lights = scenes.mixed_lights(area)
    lights["kind"][2] = 7
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    from visionaray_gb300.runtime import GbrtError
    with pytest.raises(GbrtError, match="unknown light kind"):
        vg.PTScene(bvh, mats, lights)
    assert np.asarray(lights).dtype == LIGHT


def test_materials_reference_mode_matches_fp32_oracle(oracle, material_box):
    """Against the FP32 oracle (itself bit-exact against visionaray's kernel) at
    matched random numbers, pow / cos / sin in double on both sides."""
    tris, mats, lights, cam = material_box
    params = scenes.pt_params(96, 64, 8, num_bounces=8, frame_id=13)
    gpu, _, _ = render(tris, mats, lights, cam, params)
    ref, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params,
                              mode=Oracle.PT_FLOAT_TRIG_DOUBLE)
    s = stats(gpu, ref)
    assert s["exact"] >= 0.97, s
    assert s["rmse"] <= 0.01 * s["mean"], s


def test_materials_shadow_range_fix_matches_fp64_oracle(oracle, material_box):
    tris, mats, lights, cam = material_box
    params = scenes.pt_params(96, 64, 8, num_bounces=8, frame_id=14, flags=PT_SHADOW_RANGE_FIX)
    gpu, _, _ = render(tris, mats, lights, cam, params)
    ref, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params, mode=Oracle.PT_DOUBLE)
    s = stats(gpu, ref)
    # FP32 against FP64 at matched random numbers; a glass path whose Fresnel draw (or
    # a plastic path whose lobe draw) lands on the other side of its threshold in FP64
    # takes the other branch, hence 2%
    assert s["rmse"] <= 0.02 * s["mean"], s


def test_materials_megakernel_and_sorted_queues_equal_wavefront(material_box):
    from visionaray_gb300.types import PT_MEGAKERNEL, PT_SORT_QUEUES
    tris, mats, lights, cam = material_box
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    scene = vg.PTScene(bvh, mats, lights)
    out = []
    for extra in (0, PT_MEGAKERNEL, PT_SORT_QUEUES):
        p = scenes.pt_params(80, 48, 4, num_bounces=8, frame_id=6, flags=PT_SHADOW_RANGE_FIX | extra)
        img = vg.pathtrace_frame(scene, cam, p)
        bvh.ctx.synchronize()
        out.append(img.cpu().numpy())
    assert out[0].tobytes() == out[1].tobytes()
    assert out[0].tobytes() == out[2].tobytes()


def test_edge_materials_match_fp32_oracle(oracle):
    """Zero-reflectance and exponent-0 / 7.5 plastics, index-1 and index-2.4 glass, an
    index-1 mirror: the GPU against the FP32 oracle with its arithmetic."""
    from .materials import edge_material_box
    tris, mats, lights = edge_material_box()
    cam = scenes.box_camera()
    params = scenes.pt_params(96, 64, 4, num_bounces=8, frame_id=21)
    gpu, _, _ = render(tris, mats, lights, cam, params)
    ref, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params,
                              mode=Oracle.PT_FLOAT_TRIG_DOUBLE)
    s = stats(gpu, ref)
    assert np.isfinite(gpu).all()
    assert s["exact"] >= 0.97, s
    assert s["rmse"] <= 0.01 * s["mean"], s


def test_unknown_material_kind_is_rejected():
    from visionaray_gb300.runtime import GbrtError
    tris, mats, lights = scenes.box_scene(n_blobs=1, subdiv=4, seed=1)
    mats["kind"][20] = 9
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    with pytest.raises(GbrtError, match="unknown material kind"):
        vg.PTScene(bvh, mats, lights)
    with pytest.raises(GbrtError, match="unknown material kind"):
        vg.PTScene(bvh, mats, scenes.mixed_lights(lights))


@pytest.mark.parametrize("filt,address,transform", [("linear", "clamp", "identity"), ("linear", "wrap", "rotation"),
                                                    ("nearest", "mirror", "quarter_turn")])
def test_environment_light_matches_fp32_oracle(oracle, filt, address, transform):
    """gbrt_pt_scene_set_environment against the FP32 oracle (itself bit-exact against
    visionaray's kernel with environment_light).  atan2 / acos are CUDA's here and the
    C library's in the oracle, a few ulps apart: a lookup can land on a neighbouring
    texel (nearest) or weight (linear), so pixels are compared by error, not bits."""
    from oracle import env_light
    from visionaray_gb300 import types

    from .materials import ENV_TRANSFORMS, env_texels, open_blob_scene
    tris, mats, lights, cam = open_blob_scene()
    tex = env_texels()
    kw = dict(filter=getattr(types, "FILTER_" + filt.upper()), address=getattr(types, "ADDRESS_" + address.upper()),
              scale=(1.5, 1.0, 0.75), light_to_world=ENV_TRANSFORMS[transform])
    params = scenes.pt_params(96, 64, 4, num_bounces=6, frame_id=7)
    bvh = vg.lbvh_builder().build(vg.as_device_bytes(tris))
    scene = vg.PTScene(bvh, mats, lights)
    scene.set_environment(torch.from_numpy(tex).cuda(), **kw)
    gpu = vg.pathtrace_frame(scene, cam, params).cpu().numpy().astype(np.float64)
    ref, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params,
                              mode=Oracle.PT_FLOAT_TRIG_DOUBLE, env=env_light(tex, **kw))
    s = stats(gpu, ref)
    assert s["exact"] >= 0.5, s
    assert s["rmse"] <= 0.02 * s["mean"], s
    # removing it restores the ambient light
    scene.set_environment(None)
    plain = vg.pathtrace_frame(scene, cam, params).cpu().numpy()
    again, _, _ = render(tris, mats, lights, cam, params)
    assert np.array_equal(plain, again.astype(np.float32))


def test_environment_arguments_are_checked():
    from visionaray_gb300.runtime import GbrtError
    tris, mats, lights = scenes.box_scene(n_blobs=2, subdiv=2, seed=1)
    scene = vg.PTScene(vg.lbvh_builder().build(vg.as_device_bytes(tris)), mats, lights)
    tex = torch.ones((4, 8, 4), dtype=torch.float32, device="cuda:0")
    for kw in (dict(filter=2), dict(address=3), dict(light_to_world=np.zeros((4, 4), np.float32))):
        with pytest.raises(GbrtError):
            scene.set_environment(tex, **kw)
    with pytest.raises(ValueError):
        scene.set_environment(tex[..., :3])
