"""The path-replay adjoint (gbrt_pathtrace_backward) against central finite differences
of the GPU forward pass at common random numbers, against the oracle's FP32 and FP64
host adjoints, and the forward pass against the plain frame.  Russian roulette is off
and the shadow range fixed (visionaray_gb300.inverse.FLAGS) so the image is smooth in
the albedos; tolerances are stated per test."""
import numpy as np
import pytest
import torch

import visionaray_gb300 as vg
from visionaray_gb300 import inverse, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    ctx = vg.Context(0)
    tris, mats, lights = scenes.box_scene(n_blobs=2, subdiv=4, seed=1)
    bvh = vg.lbvh_builder(ctx).build(vg.as_device_bytes(tris))
    scene = vg.PTScene(bvh, mats, lights)
    albedo = torch.from_numpy(np.ascontiguousarray(mats["color"], np.float32)).cuda()
    emission = albedo.clone()
    params = scenes.pt_params(48, 32, 4, num_bounces=6, frame_id=7, flags=inverse.FLAGS)
    cam = scenes.box_camera()
    adj = torch.from_numpy(np.random.default_rng(0).normal(size=(32, 48, 4)).astype(np.float32)).cuda()
    adj[..., 3] = 0
    return ctx, tris, mats, lights, scene, albedo, emission, params, cam, adj


def loss_of(scene, cam, params, albedo, emission, adj):
    img = vg.pathtrace_forward(scene, cam, params, albedo, emission)
    return float((img.double() * adj.double()).sum())


def test_forward_equals_plain_frame(setup):
    ctx, tris, mats, lights, scene, albedo, emission, params, cam, adj = setup
    img = vg.pathtrace_forward(scene, cam, params, albedo, emission)
    plain = vg.pathtrace_frame(scene, cam, params)
    ctx.synchronize()
    assert torch.equal(img, plain)


def test_adjoint_matches_central_differences(setup):
    ctx, tris, mats, lights, scene, albedo, emission, params, cam, adj = setup
    ga, ge = vg.pathtrace_backward(scene, cam, params, albedo, emission, adj)
    ctx.synchronize()
    ga, ge = ga.cpu().numpy(), ge.cpu().numpy()
    # 64 parameters: the 62 largest albedo gradients and two channels of the light
    order = np.argsort(-np.abs(ga).ravel())[:62]
    cases = [("a", int(i) // 3, int(i) % 3) for i in order] + [("e", 12, 0), ("e", 13, 1)]
    for kind, slot, c in cases:
        base = (albedo if kind == "a" else emission)
        h = 1e-3 * max(1.0, float(base[slot, c]))   # 1e-3 on albedos, relative on emission (15)
        plus, minus = base.clone(), base.clone()
        plus[slot, c] += h
        minus[slot, c] -= h
        step = float(plus[slot, c] - minus[slot, c])   # the float32 perturbation actually applied
        a_p, e_p = (plus, emission) if kind == "a" else (albedo, plus)
        a_m, e_m = (minus, emission) if kind == "a" else (albedo, minus)
        fd = (loss_of(scene, cam, params, a_p, e_p, adj) - loss_of(scene, cam, params, a_m, e_m, adj)) / step
        g = float((ga if kind == "a" else ge)[slot, c])
        # 1e-3 relative, plus an absolute floor for the FP32 forward's rounding: each
        # loss sums ~6,000 float32 pixel terms, whose rounding noise (~1e-7 relative
        # each) divided by the 2e-3 step is ~5e-4 in the quotient, i.e. 1e-4 of the
        # largest gradient (15) here
        assert abs(g - fd) <= 1e-3 * abs(fd) + 1e-4 * np.abs(ga).max(), (kind, slot, c, g, fd)


def test_adjoint_matches_host_adjoints(setup, oracle):
    ctx, tris, mats, lights, scene, albedo, emission, params, cam, adj = setup
    ga, ge = vg.pathtrace_backward(scene, cam, params, albedo, emission, adj)
    ctx.synchronize()
    ga, ge = ga.cpu().numpy().astype(np.float64), ge.cpu().numpy().astype(np.float64)
    tree = oracle.build_sah(tris)
    a_np, e_np, adj_np = albedo.cpu().numpy(), emission.cpu().numpy(), adj.cpu().numpy()
    for fp64, tol in ((False, 1e-4), (True, 2e-3)):
        ha, he, _ = oracle.pathtrace_adjoint(tree, tris, mats, lights, cam, params, a_np, e_np, adj_np, fp64=fp64)
        rel_a = np.linalg.norm(ga - ha) / np.linalg.norm(ha)
        rel_e = np.linalg.norm(ge - he) / np.linalg.norm(he)
        assert rel_a <= tol and rel_e <= tol, (fp64, rel_a, rel_e)


def test_inverse_albedo_recovers_the_seen_albedos():
    """A short run at reduced size: the albedo error of the slots the camera sees, on
    the same slots at the start and the end, falls (the decorrelated estimator)."""
    res = inverse.optimize(steps=40, width=128, height=128, spp=8, target_spp=64, min_pixels=16)
    start, end = res["errors_start"], res["errors_end"]
    assert end["coverage_weighted"] < 0.8 * start["coverage_weighted"], (start, end)
    assert res["losses"][-1] < res["losses"][0]
    assert res["bwd_ms"] > 0 and res["fwd_ms"] > 0


@pytest.mark.parametrize("light_set", ["area", "mixed"])
def test_adjoint_through_specular_and_plastic_vertices(oracle, light_set):
    """Mirror, glass and plastic blobs and plastic walls: the reverse sweep carries the
    adjoint through each specular or plastic vertex's fixed factor and a plastic
    vertex's next-event term; against the FP32 and FP64 host adjoints."""
    ctx = vg.Context(0)
    tris, mats, lights = scenes.glossy_box_scene(n_blobs=5, subdiv=4, seed=1)
    if light_set == "mixed":
        lights = scenes.mixed_lights(lights)
    bvh = vg.lbvh_builder(ctx).build(vg.as_device_bytes(tris))
    scene = vg.PTScene(bvh, mats, lights)
    albedo = torch.from_numpy(np.ascontiguousarray(mats["color"], np.float32)).cuda()
    emission = albedo.clone()
    cam = scenes.box_camera()
    adj = torch.from_numpy(np.random.default_rng(1).normal(size=(32, 48, 4)).astype(np.float32)).cuda()
    adj[..., 3] = 0
    params = scenes.pt_params(48, 32, 4, num_bounces=6, frame_id=9, flags=inverse.FLAGS)
    img = vg.pathtrace_forward(scene, cam, params, albedo, emission)
    assert torch.equal(img, vg.pathtrace_frame(scene, cam, params))
    ga, ge = vg.pathtrace_backward(scene, cam, params, albedo, emission, adj)
    ctx.synchronize()
    ga, ge = ga.cpu().numpy().astype(np.float64), ge.cpu().numpy().astype(np.float64)
    tree = oracle.build_sah(tris)
    a_np, e_np, adj_np = albedo.cpu().numpy(), emission.cpu().numpy(), adj.cpu().numpy()
    for fp64, tol in ((False, 1e-4), (True, 2e-3)):
        ha, he, _ = oracle.pathtrace_adjoint(tree, tris, mats, lights, cam, params, a_np, e_np, adj_np, fp64=fp64)
        rel_a = np.linalg.norm(ga - ha) / np.linalg.norm(ha)
        rel_e = np.linalg.norm(ge - he) / np.linalg.norm(he)
        assert rel_a <= tol and rel_e <= tol, (fp64, rel_a, rel_e)


def test_adjoint_with_an_environment_light(oracle):
    """Paths that leave into an environment light: the replay's miss vertex carries the
    lat-long lookup, against the FP32 and FP64 host adjoints (the lookup's atan2 / acos
    are CUDA's there and the C library's here: a few ulps apart)."""
    from oracle import env_light

    from .materials import ENV_TRANSFORMS, env_texels, open_blob_scene
    ctx = vg.Context(0)
    tris, mats, lights, cam = open_blob_scene(n_blobs=5, subdiv=4)
    bvh = vg.lbvh_builder(ctx).build(vg.as_device_bytes(tris))
    scene = vg.PTScene(bvh, mats, lights)
    tex = env_texels(32, 16)
    scene.set_environment(torch.from_numpy(tex).cuda(), light_to_world=ENV_TRANSFORMS["rotation"])
    albedo = torch.from_numpy(np.ascontiguousarray(mats["color"], np.float32)).cuda()
    emission = albedo.clone()
    adj = torch.from_numpy(np.random.default_rng(3).normal(size=(32, 48, 4)).astype(np.float32)).cuda()
    adj[..., 3] = 0
    params = scenes.pt_params(48, 32, 4, num_bounces=5, frame_id=4, flags=inverse.FLAGS)
    img = vg.pathtrace_forward(scene, cam, params, albedo, emission)
    assert torch.equal(img, vg.pathtrace_frame(scene, cam, params))
    ga, ge = vg.pathtrace_backward(scene, cam, params, albedo, emission, adj)
    ctx.synchronize()
    ga, ge = ga.cpu().numpy().astype(np.float64), ge.cpu().numpy().astype(np.float64)
    tree = oracle.build_sah(tris)
    env = env_light(tex, light_to_world=ENV_TRANSFORMS["rotation"])
    a_np, e_np, adj_np = albedo.cpu().numpy(), emission.cpu().numpy(), adj.cpu().numpy()
    for fp64, tol in ((False, 1e-3), (True, 3e-3)):
        ha, he, _ = oracle.pathtrace_adjoint(tree, tris, mats, lights, cam, params, a_np, e_np, adj_np, fp64=fp64,
                                             env=env)
        rel_a = np.linalg.norm(ga - ha) / np.linalg.norm(ha)
        rel_e = np.linalg.norm(ge - he) / np.linalg.norm(he)
        assert rel_a <= tol and rel_e <= tol, (fp64, rel_a, rel_e)
