"""The path-tracing oracle against visionaray's own pathtracing::kernel (golden image
generated from the reference build, and direct comparison where it is built), and
the FP32 / FP64 agreement that the shadow-range fix restores."""
import hashlib

import numpy as np
import pytest

from oracle import Oracle, Reference
from visionaray_gb300 import scenes
from visionaray_gb300.types import PT_SHADOW_RANGE_FIX


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


@pytest.fixture(scope="module")
def small_box():
    tris, mats, lights = scenes.box_scene(n_blobs=8, subdiv=8, seed=1)
    return tris, mats, lights, scenes.box_camera()


def test_golden_image(oracle, small_box, golden):
    meta, samples = golden
    g = meta["pathtrace"]
    tris, mats, lights, cam = small_box
    assert digest(tris) == g["triangles_sha256"] and digest(mats) == g["materials_sha256"]
    pr = g["params"]
    params = scenes.pt_params(pr["width"], pr["height"], pr["spp"], num_bounces=pr["num_bounces"],
                              epsilon=pr["epsilon"], frame_id=pr["frame_id"])
    tree = oracle.build_sah(tris)
    img, _ = oracle.pathtrace(tree, tris, mats, lights, cam, params, mode=Oracle.PT_FLOAT)
    img = img.astype(np.float32)
    ref = samples["pt_image"]
    if Reference.available():
        # the same host and libm as the golden image: bit for bit
        assert np.array_equal(img, ref)
    else:
        # another host's cosf/sinf may round differently in the last bit, and the
        # reference's shadow test turns such differences into different light samples
        # for a few paths: the image statistics must still agree
        assert np.allclose(img.reshape(-1, 4).mean(0), ref.reshape(-1, 4).mean(0), rtol=0.03)
        assert (np.abs(img - ref).max(axis=2) == 0).mean() > 0.5


MATERIAL_SCENES = {
    # mirror (conductor Fresnel) and glass (dielectric Fresnel, refraction, total
    # internal reflection) blobs
    "specular": lambda: scenes.specular_box_scene(n_blobs=8, subdiv=8, seed=1),
    # plus plastic blobs and plastic walls (lobe choice, Blinn sampling and glossy NEE)
    "glossy": lambda: scenes.glossy_box_scene(n_blobs=10, subdiv=8, seed=1),
}


@pytest.mark.parametrize("name", sorted(MATERIAL_SCENES))
def test_golden_material_images(oracle, golden, name):
    """The material scenes against the reference kernel's images."""
    meta, samples = golden
    g = meta["pathtrace_" + name]
    tris, mats, lights = MATERIAL_SCENES[name]()
    assert digest(tris) == g["triangles_sha256"] and digest(mats) == g["materials_sha256"]
    pr = g["params"]
    params = scenes.pt_params(pr["width"], pr["height"], pr["spp"], num_bounces=pr["num_bounces"],
                              epsilon=pr["epsilon"], frame_id=pr["frame_id"])
    img, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, scenes.box_camera(), params,
                              mode=Oracle.PT_FLOAT)
    img = img.astype(np.float32)
    ref = samples["pt_%s_image" % name]
    if Reference.available():
        assert np.array_equal(img, ref)
    else:
        assert np.allclose(img.reshape(-1, 4).mean(0), ref.reshape(-1, 4).mean(0), rtol=0.03)
        assert (np.abs(img - ref).max(axis=2) == 0).mean() > 0.5


def test_golden_point_and_spot_lights(oracle, golden):
    """Area, point and spot lights (generic_light) against the reference kernel's image."""
    meta, samples = golden
    g = meta["pathtrace_lights"]
    tris, mats, area = scenes.glossy_box_scene(n_blobs=10, subdiv=8, seed=1)
    lights = scenes.mixed_lights(area)
    assert digest(lights) == g["lights_sha256"] and digest(mats) == g["materials_sha256"]
    pr = g["params"]
    params = scenes.pt_params(pr["width"], pr["height"], pr["spp"], num_bounces=pr["num_bounces"],
                              epsilon=pr["epsilon"], frame_id=pr["frame_id"])
    img, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, scenes.box_camera(), params,
                              mode=Oracle.PT_FLOAT)
    img = img.astype(np.float32)
    ref = samples["pt_lights_image"]
    if Reference.available():
        assert np.array_equal(img, ref)
    else:
        assert np.allclose(img.reshape(-1, 4).mean(0), ref.reshape(-1, 4).mean(0), rtol=0.03)
        assert (np.abs(img - ref).max(axis=2) == 0).mean() > 0.5


@pytest.mark.skipif(not Reference.available(), reason="visionaray sources not built here")
@pytest.mark.parametrize("frame,spp,bounces", [(0, 2, 8), (5, 3, 3), (9, 1, 1)])
def test_fp32_oracle_is_the_reference_kernel_lights(oracle, frame, spp, bounces):
    tris, mats, area = scenes.glossy_box_scene(n_blobs=10, subdiv=8, seed=1)
    lights = scenes.mixed_lights(area)
    cam = scenes.box_camera()
    params = scenes.pt_params(40, 24, spp, num_bounces=bounces, frame_id=frame)
    ref = Reference().pathtrace(tris, mats, lights, cam, params)
    img, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params, mode=Oracle.PT_FLOAT)
    assert np.array_equal(img.astype(np.float32), ref)


@pytest.mark.skipif(not Reference.available(), reason="visionaray sources not built here")
def test_reference_spot_light_adds_nothing(oracle):
    """spot_light::sample evaluates its cone at its own position (normalize(0) = NaN):
    the reference's image does not change with the spot light's power or position,
    and neither does the oracle's."""
    from visionaray_gb300.types import LIGHT_SPOT
    tris, mats, area = scenes.glossy_box_scene(n_blobs=10, subdiv=8, seed=1)
    lights = scenes.mixed_lights(area)
    other = lights.copy()
    spot = other["kind"] == LIGHT_SPOT
    other["kl"][spot] = 100.0
    other["position"][spot] = (0.5, 0.5, 0.5)
    params = scenes.pt_params(32, 16, 2, num_bounces=4, frame_id=3)
    cam = scenes.box_camera()
    a = Reference().pathtrace(tris, mats, lights, cam, params)
    assert np.array_equal(a, Reference().pathtrace(tris, mats, other, cam, params))
    tree = oracle.build_sah(tris)
    o1, _ = oracle.pathtrace(tree, tris, mats, lights, cam, params, mode=Oracle.PT_FLOAT)
    o2, _ = oracle.pathtrace(tree, tris, mats, other, cam, params, mode=Oracle.PT_FLOAT)
    assert np.array_equal(o1, o2)


@pytest.mark.skipif(not Reference.available(), reason="visionaray sources not built here")
@pytest.mark.parametrize("name", sorted(MATERIAL_SCENES))
@pytest.mark.parametrize("frame,spp,bounces", [(0, 2, 8), (5, 3, 3), (9, 1, 1)])
def test_fp32_oracle_is_the_reference_kernel_materials(oracle, name, frame, spp, bounces):
    tris, mats, lights = MATERIAL_SCENES[name]()
    cam = scenes.box_camera()
    params = scenes.pt_params(40, 24, spp, num_bounces=bounces, frame_id=frame)
    ref = Reference().pathtrace(tris, mats, lights, cam, params)
    img, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params, mode=Oracle.PT_FLOAT)
    assert np.array_equal(img.astype(np.float32), ref)
    # the materials change the image: the same geometry all matte differs
    _, matte, _ = scenes.box_scene(n_blobs=(len(tris) - 14) // (20 * 8 * 8), subdiv=8, seed=1)
    plain, _ = oracle.pathtrace(oracle.build_sah(tris), tris, matte, lights, cam, params, mode=Oracle.PT_FLOAT)
    changed = (np.abs(plain.astype(np.float32) - ref).max(axis=2) > 0).mean()
    assert changed > (0.05 if bounces > 1 else 0.0), changed


@pytest.mark.skipif(not Reference.available(), reason="visionaray sources not built here")
@pytest.mark.parametrize("frame,spp,bounces", [(0, 2, 8), (5, 3, 3), (9, 1, 1)])
def test_fp32_oracle_is_the_reference_kernel(oracle, small_box, frame, spp, bounces):
    tris, mats, lights, cam = small_box
    params = scenes.pt_params(40, 24, spp, num_bounces=bounces, frame_id=frame)
    ref = Reference().pathtrace(tris, mats, lights, cam, params)
    img, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params, mode=Oracle.PT_FLOAT)
    assert np.array_equal(img.astype(np.float32), ref)


@pytest.mark.skipif(not Reference.available(), reason="visionaray sources not built here")
def test_reference_blend_and_background(oracle, small_box):
    tris, mats, lights, cam = small_box
    ref = Reference()
    p0 = scenes.pt_params(16, 8, 2, frame_id=1)
    a = ref.pathtrace(tris, mats, lights, cam, p0)
    p1 = scenes.pt_params(16, 8, 2, frame_id=2, sfactor=0.5, dfactor=0.5)
    b = ref.pathtrace(tris, mats, lights, cam, p1, accum=a.copy())
    f2, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, p1, mode=Oracle.PT_FLOAT)
    assert np.array_equal(b, (f2.astype(np.float32) * np.float32(0.5) + a * np.float32(0.5)))
    # camera looking out of an open scene (blobs only): background pixels
    tris2, mats2, lights2 = tris[14:], mats, lights
    tris2 = tris2.copy()
    cam2 = scenes.box_camera(eye=(0.5, 0.5, -3.0), center=(0.5, 0.5, 0.0), fovy_degrees=20.0)
    pb = scenes.pt_params(16, 8, 1, background=(0.25, 0.5, 1.0, 2.0))
    c = ref.pathtrace(tris2, mats2, lights2, cam2, pb)
    o, _ = oracle.pathtrace(oracle.build_sah(tris2), tris2, mats2, lights2, cam2, pb, mode=Oracle.PT_FLOAT)
    assert np.array_equal(c, o.astype(np.float32))
    assert (c.reshape(-1, 4) == np.array([0.5, 1.0, 2.0, 1.0], np.float32)).all(axis=1).any()


@pytest.mark.skipif(not Reference.available(), reason="visionaray sources not built here")
@pytest.mark.parametrize("frame,spp,bounces", [(1, 2, 8), (4, 2, 3)])
def test_fp32_oracle_is_the_reference_kernel_edge_materials(oracle, frame, spp, bounces):
    from .materials import edge_material_box
    tris, mats, lights = edge_material_box()
    cam = scenes.box_camera()
    params = scenes.pt_params(40, 24, spp, num_bounces=bounces, frame_id=frame)
    ref = Reference().pathtrace(tris, mats, lights, cam, params)
    img, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params, mode=Oracle.PT_FLOAT)
    assert np.isfinite(ref).all()
    assert np.array_equal(img.astype(np.float32), ref)


def test_shadow_range_fix_makes_fp32_and_fp64_agree(oracle, small_box):
    tris, mats, lights, cam = small_box
    tree = oracle.build_sah(tris)
    fixed = scenes.pt_params(48, 32, 4, flags=PT_SHADOW_RANGE_FIX)
    f32, _ = oracle.pathtrace(tree, tris, mats, lights, cam, fixed, mode=Oracle.PT_FLOAT)
    f64, cnt = oracle.pathtrace(tree, tris, mats, lights, cam, fixed, mode=Oracle.PT_DOUBLE)
    rmse = np.sqrt(((f32 - f64)[..., :3] ** 2).mean())
    assert rmse < 2e-3 * f64[..., :3].mean() * 10, rmse
    # without the fix the light hides its own samples, rounding-dependent: the FP32
    # and FP64 images differ systematically
    plain = scenes.pt_params(48, 32, 4)
    g32, _ = oracle.pathtrace(tree, tris, mats, lights, cam, plain, mode=Oracle.PT_FLOAT)
    g64, _ = oracle.pathtrace(tree, tris, mats, lights, cam, plain, mode=Oracle.PT_DOUBLE)
    assert g32[..., :3].mean() > 1.1 * g64[..., :3].mean()
    assert f64[..., :3].mean() > 2.0 * g64[..., :3].mean()
    assert cnt[0] > 48 * 32 * 4 and cnt[1] > 0


@pytest.mark.parametrize("light_set", ["area", "mixed"])
def test_oracle_adjoint_through_specular_vertices(oracle, light_set):
    """The FP64 host adjoint on a box with mirror, glass and plastic blobs and plastic
    walls against central differences of the FP64 forward pass at common random
    numbers (roulette off, shadow range fixed, so the image is smooth in the albedos):
    specular and plastic vertices pass the adjoint through their fixed factor, and a
    plastic vertex's next-event term through its MIS weight and the light's emission."""
    from visionaray_gb300 import inverse
    tris, mats, lights = scenes.glossy_box_scene(n_blobs=5, subdiv=4, seed=1)
    if light_set == "mixed":
        lights = scenes.mixed_lights(lights)   # point and spot lights: no emission parameter
    cam = scenes.box_camera()
    params = scenes.pt_params(32, 24, 2, num_bounces=6, frame_id=7, flags=inverse.FLAGS)
    tree = oracle.build_sah(tris)
    albedo = np.ascontiguousarray(mats["color"], np.float32)
    emission = albedo.copy()
    adj = np.random.default_rng(0).normal(size=(24, 32, 4))
    adj[..., 3] = 0
    ga, ge, img = oracle.pathtrace_adjoint(tree, tris, mats, lights, cam, params, albedo, emission, adj)
    _, _, again = oracle.pathtrace_adjoint(tree, tris, mats, lights, cam, params, albedo, emission, adj)
    assert np.array_equal(img, again)

    def loss(a, e):
        return float((oracle.pathtrace_adjoint(tree, tris, mats, lights, cam, params, a, e, adj)[2] * adj).sum())

    matte = mats["kind"] == 0
    cand = np.argsort(-np.abs(ga[matte]).ravel())[:6]
    slots = np.flatnonzero(matte)
    cases = [("a", int(slots[i // 3]), int(i % 3)) for i in cand] + [("e", 12, 0)]
    for kind, slot, c in cases:
        base = albedo if kind == "a" else emission
        h = np.float32(1e-2 * max(1.0, float(base[slot, c])))
        plus, minus = base.copy(), base.copy()
        plus[slot, c] += h
        minus[slot, c] -= h
        step = float(plus[slot, c]) - float(minus[slot, c])
        if kind == "a":
            fd = (loss(plus, emission) - loss(minus, emission)) / step
        else:
            fd = (loss(albedo, plus) - loss(albedo, minus)) / step
        g = float((ga if kind == "a" else ge)[slot, c])
        # the image is a polynomial in the albedos (a slot met twice on a path enters
        # squared): central differences carry an O(h^2) term, 1e-4 relative bounds it
        assert abs(g - fd) <= 1e-4 * abs(fd) + 1e-9 * np.abs(ga).max(), (kind, slot, c, g, fd)


ENV_MODES = [("linear", "clamp", "identity"), ("linear", "wrap", "rotation"), ("nearest", "mirror", "quarter_turn"),
             ("nearest", "wrap", "rotation")]


@pytest.mark.skipif(not Reference.available(), reason="visionaray sources not built here")
@pytest.mark.parametrize("filt,address,transform", ENV_MODES)
def test_fp32_oracle_is_the_reference_kernel_environment(oracle, filt, address, transform):
    """environment_light<float, texture_ref<vec4, 2>> as the kernel's amb_light: the
    FP32 oracle's lat-long lookup, texture filters, address modes and float inverse
    transform are the reference's, bit for bit."""
    from oracle import env_light
    from visionaray_gb300 import types

    from .materials import ENV_TRANSFORMS, env_texels, open_blob_scene
    tris, mats, lights, cam = open_blob_scene()
    env = env_light(env_texels(), filter=getattr(types, "FILTER_" + filt.upper()),
                    address=getattr(types, "ADDRESS_" + address.upper()), scale=(1.5, 1.0, 0.75),
                    light_to_world=ENV_TRANSFORMS[transform])
    params = scenes.pt_params(40, 24, 2, num_bounces=4, frame_id=3)
    ref = Reference().pathtrace(tris, mats, lights, cam, params, env=env)
    img, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params, mode=Oracle.PT_FLOAT, env=env)
    assert np.array_equal(img.astype(np.float32), ref)
    plain = Reference().pathtrace(tris, mats, lights, cam, params)
    assert not np.array_equal(plain, ref)   # the environment is seen


def test_constant_nearest_environment_is_the_ambient_light(oracle):
    """A constant texture under the nearest filter and unit scale returns the texel
    itself, so the image equals the one with that ambient light (any transform)."""
    from oracle import env_light
    from visionaray_gb300 import types

    from .materials import ENV_TRANSFORMS, open_blob_scene
    tris, mats, lights, cam = open_blob_scene()
    c = np.array([0.3, 0.6, 0.9, 1.0], np.float32)
    env = env_light(np.broadcast_to(c, (8, 16, 4)), filter=types.FILTER_NEAREST, address=types.ADDRESS_WRAP,
                    light_to_world=ENV_TRANSFORMS["rotation"])
    tree = oracle.build_sah(tris)
    params = scenes.pt_params(24, 16, 2, num_bounces=3, frame_id=2)
    a, _ = oracle.pathtrace(tree, tris, mats, lights, cam, params, mode=Oracle.PT_FLOAT, env=env)
    b, _ = oracle.pathtrace(tree, tris, mats, lights, cam, scenes.pt_params(24, 16, 2, num_bounces=3, frame_id=2,
                                                                            ambient=tuple(c[:3])),
                            mode=Oracle.PT_FLOAT)
    assert np.array_equal(a, b)


def test_adjoint_with_an_environment_matches_finite_differences(oracle):
    """The path-replay adjoint carries the environment radiance of each escaped path
    (FP64 oracle, central differences of the albedo)."""
    from oracle import env_light

    from .materials import ENV_TRANSFORMS, env_texels, open_blob_scene
    tris, mats, lights, cam = open_blob_scene(n_blobs=4, subdiv=6)
    env = env_light(env_texels(32, 16), light_to_world=ENV_TRANSFORMS["rotation"])
    tree = oracle.build_sah(tris)
    params = scenes.pt_params(16, 12, 2, num_bounces=4, frame_id=1)
    albedo = np.ascontiguousarray(mats["color"], np.float32)
    adj = np.zeros((12, 16, 4))
    adj[..., :3] = 1.0
    ga, _, _ = oracle.pathtrace_adjoint(tree, tris, mats, lights, cam, params, albedo, None, adj, env=env)
    assert np.abs(ga).max() > 0
    g = int(np.argmax(np.abs(ga).max(axis=1)))
    h = 1e-3
    for ch in range(3):
        vals = []
        for sgn in (1, -1):
            a2 = albedo.copy()
            a2[g, ch] += sgn * h
            _, _, img = oracle.pathtrace_adjoint(tree, tris, mats, lights, cam, params, a2, None, adj, env=env)
            vals.append(img[..., :3].sum())
        fd = (vals[0] - vals[1]) / (2 * h)
        assert fd == pytest.approx(ga[g, ch], rel=1e-3, abs=1e-6 * np.abs(ga).max())


def test_golden_environment_image(oracle, golden):
    """The FP32 oracle against the reference kernel's image under an environment light
    (tests/golden, generated by visionaray's own CPU build): bit-exact where the host's C
    library is the generator's; elsewhere atan2 / acos / cos / sin may differ by ulps."""
    from oracle import env_light
    from visionaray_gb300 import types

    from .materials import ENV_TRANSFORMS, env_texels, open_blob_scene
    meta, samples = golden
    g = meta["pathtrace_environment"]
    tris, mats, lights, cam = open_blob_scene()
    tex = env_texels()
    assert digest(tex) == g["texels_sha256"] and digest(tris) == g["triangles_sha256"]
    env = env_light(tex, filter=types.FILTER_LINEAR, address=types.ADDRESS_WRAP, scale=(1.5, 1.0, 0.75),
                    light_to_world=ENV_TRANSFORMS["rotation"])
    params = scenes.pt_params(64, 48, 4, num_bounces=6, frame_id=8)
    img, _ = oracle.pathtrace(oracle.build_sah(tris), tris, mats, lights, cam, params, mode=Oracle.PT_FLOAT, env=env)
    img = img.astype(np.float32)
    ref = samples["pt_env_image"]
    if Reference.available():
        assert np.array_equal(img, ref)
    else:
        assert np.allclose(img.reshape(-1, 4).mean(0), ref.reshape(-1, 4).mean(0), rtol=0.03)
        assert (np.abs(img - ref).max(axis=2) == 0).mean() > 0.5
