"""The path-tracing workloads at their full sizes against the oracle.

- Box frame: the 256-blob box (2,478,094 triangles) at 1920x1080, 64 spp, depth 8,
  Russian roulette from depth 3, rendered whole on the GPU; a fixed sample of pixels
  (every 997th, 2,080 pixels) is rendered by the oracle at the same random numbers.
  visionaray's shadow range is compared with the FP32 oracle (the CUDA path's
  arithmetic); the corrected shadow range with the FP64 oracle.
- Inverse albedo: the 4,094-triangle box at 512x512, 16 spp, depth 6; the adjoint of the
  L2 image loss against central finite differences of the GPU forward pass (h = 1e-3,
  common random numbers) on 64 albedo parameters drawn by a seeded generator from all
  slots and on 64 drawn from the slots the camera sees, and against the FP64 host
  adjoint.
- Batch: 16 of the 512 full-size random-soup scenes (every 32nd) rendered in one
  persistent launch, against the oracle per scene.
Tolerances are stated per test, with the reason."""
import numpy as np
import pytest
import torch

import visionaray_gb300 as vg
from oracle import Oracle
from visionaray_gb300 import inverse, scenes
from visionaray_gb300.types import AREA_LIGHT, EMISSIVE, PT_SHADOW_RANGE_FIX

pytestmark = pytest.mark.gpu

W, H, SPP, DEPTH = 1920, 1080, 64, 8
PIXELS = np.arange(0, W * H, 997, dtype=np.uint32)


def pixel_stats(gpu, ref):
    """gpu, ref: (n, 4).  Fraction of pixels equal in RGB bit for bit, RMSE and the
    oracle's mean (RGB)."""
    d = np.abs(gpu[:, :3].astype(np.float64) - ref[:, :3])
    return {"pixels": len(gpu), "exact": float((d.max(axis=1) == 0).mean()), "rmse": float(np.sqrt((d ** 2).mean())),
            "mean": float(ref[:, :3].mean()), "max": float(d.max())}


@pytest.fixture(scope="module")
def box(oracle):
    tris, mats, lights = scenes.box_scene()
    return tris, mats, lights, scenes.box_camera(), oracle.build_sah(tris)


def gpu_frame(tris, mats, lights, cam, params, builder):
    make = vg.ploc_builder if builder == "ploc" else vg.lbvh_builder
    bvh = make().build(vg.as_device_bytes(tris))
    scene = vg.PTScene(bvh, mats, lights)
    img = vg.pathtrace_frame(scene, cam, params)
    bvh.ctx.synchronize()
    out = img.cpu().numpy().reshape(-1, 4)
    scene.close()
    bvh.close()
    return out


@pytest.mark.parametrize("builder", ["lbvh", "ploc"])
def test_box_frame_full_size_against_fp32_oracle(oracle, box, builder):
    tris, mats, lights, cam, tree = box
    params = scenes.pt_params(W, H, SPP, num_bounces=DEPTH, frame_id=1)
    gpu = gpu_frame(tris, mats, lights, cam, params, builder)[PIXELS]
    ref, cnt = oracle.pathtrace_pixels(tree, tris, mats, lights, cam, params, PIXELS, mode=Oracle.PT_FLOAT_TRIG_DOUBLE)
    s = pixel_stats(gpu, ref)
    print(builder, s, cnt)
    # Same float operations and random numbers: a pixel can differ only where one of its
    # 64 paths met an equal-t tie (a ray through a shared edge of two blob triangles)
    # that the GPU tree and the oracle's SAH tree resolve in another order (measured:
    # none in this sample)
    assert s["exact"] >= 0.99, s
    assert s["rmse"] <= 0.005 * s["mean"], s


def test_box_frame_full_size_shadow_range_fix_against_fp64_oracle(oracle, box):
    tris, mats, lights, cam, tree = box
    params = scenes.pt_params(W, H, SPP, num_bounces=DEPTH, frame_id=2, flags=PT_SHADOW_RANGE_FIX)
    gpu = gpu_frame(tris, mats, lights, cam, params, "lbvh")[PIXELS]
    ref, _ = oracle.pathtrace_pixels(tree, tris, mats, lights, cam, params, PIXELS, mode=Oracle.PT_DOUBLE)
    s = pixel_stats(gpu, ref)
    print("fp64", s)
    # FP32 against FP64 at matched random numbers: paths part only where rounding flips
    # a decision (roulette, a hit at an edge); RMSE within 1% of the image mean
    # (measured 0.46%)
    assert s["rmse"] <= 0.01 * s["mean"], s


def test_box_frame_full_size_reference_mode_against_fp64_oracle(oracle, box):
    """visionaray's own shadow range against the FP64 oracle.  Its light sample sits
    exactly at the shadow ray's tmax, so whether the light's own triangle occludes it is
    decided by rounding: FP32 keeps next-event estimation on more samples than FP64 and
    the FP32 image is brighter.  The GPU frame shows exactly the FP32 reference's gap to
    FP64 (it equals the FP32 oracle pixel for pixel), not a gap of its own."""
    tris, mats, lights, cam, tree = box
    params = scenes.pt_params(W, H, SPP, num_bounces=DEPTH, frame_id=3)
    gpu = gpu_frame(tris, mats, lights, cam, params, "lbvh")[PIXELS]
    f64, _ = oracle.pathtrace_pixels(tree, tris, mats, lights, cam, params, PIXELS, mode=Oracle.PT_DOUBLE)
    f32, _ = oracle.pathtrace_pixels(tree, tris, mats, lights, cam, params, PIXELS, mode=Oracle.PT_FLOAT_TRIG_DOUBLE)
    vs64, vs32 = pixel_stats(gpu, f64), pixel_stats(gpu, f32)
    gap_gpu = float(gpu[:, :3].mean()) / vs64["mean"] - 1.0
    gap_ref = vs32["mean"] / vs64["mean"] - 1.0
    print("reference mode: gpu vs fp64", vs64, "gpu vs fp32", vs32, f"mean gap to fp64: gpu {gap_gpu:.4f}, "
          f"fp32 reference {gap_ref:.4f}")
    assert vs32["exact"] >= 0.99, vs32
    assert abs(gap_gpu - gap_ref) <= 0.005, (gap_gpu, gap_ref)


@pytest.fixture(scope="module")
def inverse_setup():
    """The inverse-rendering state the gradients are checked at: albedos drawn from
    U[0.3, 0.7] per channel (seeded).  Not the optimisation's start (0.5 everywhere):
    there, with a grey light, every path throughput has three equal channels, and the
    next-event MIS weight's max(throughput) sits on a tie where it has no derivative --
    the adjoint takes the first maximal channel's, central differences average the two
    one-sided slopes."""
    ctx = vg.Context(0)
    scene, tris, mats, lights, hidden, emission = inverse.setup(ctx=ctx)
    cam = scenes.box_camera()
    tparams = scenes.pt_params(512, 512, 256, num_bounces=6, frame_id=inverse.TARGET_FRAME, flags=inverse.FLAGS)
    target = vg.pathtrace_forward(scene, cam, tparams, hidden, emission)
    state = np.random.default_rng(11).uniform(0.3, 0.7, size=tuple(hidden.shape)).astype(np.float32)
    albedo = torch.from_numpy(state).to(hidden.device)
    params = scenes.pt_params(512, 512, 16, num_bounces=6, frame_id=0, flags=inverse.FLAGS)
    img = vg.pathtrace_forward(scene, cam, params, albedo, emission)
    _, adj = inverse.l2_adjoint(img, target)
    ga, ge = vg.pathtrace_backward(scene, cam, params, albedo, emission, adj)
    ctx.synchronize()
    return ctx, scene, tris, mats, lights, cam, target, albedo, emission, params, adj, ga, ge


def central_differences(setup, picks, h=1e-3):
    """[(slot, channel, adjoint, fd, spread, cond)] for each (slot, channel) in picks:
    fd = (L(a + h) - L(a - h)) / (the float32 step actually applied) of the GPU forward
    at the forward frame's random numbers; spread = the largest difference of fd from
    the same quotient at 0.73 h and 1.37 h (the image is a polynomial in the albedos, so
    in exact arithmetic they agree to O(h^2), ~1e-6 relative: the spread measures the
    FP32 forward's rounding noise in the quotient); cond = the sum of the gradient's
    per-path terms by size (the replay with |dL/dI| as the image adjoint) over
    |adjoint|."""
    ctx, scene, tris, mats, lights, cam, target, albedo, emission, params, adj, ga, ge = setup
    ga_np = ga.cpu().numpy()
    gabs, _ = vg.pathtrace_backward(scene, cam, params, albedo, emission, adj.abs())
    gabs_np = gabs.cpu().numpy()

    def fd_at(slot, c, step):
        ap, am = albedo.clone(), albedo.clone()
        ap[slot, c] += step
        am[slot, c] -= step
        lp = inverse.l2_adjoint(vg.pathtrace_forward(scene, cam, params, ap, emission), target)[0]
        lm = inverse.l2_adjoint(vg.pathtrace_forward(scene, cam, params, am, emission), target)[0]
        return (lp - lm) / float(ap[slot, c] - am[slot, c])

    rows = []
    for slot, c in picks:
        fd = fd_at(slot, c, h)
        spread = max(abs(fd - fd_at(slot, c, 0.73 * h)), abs(fd - fd_at(slot, c, 1.37 * h)))
        g = float(ga_np[slot, c])
        cond = float(gabs_np[slot, c]) / abs(g) if g != 0.0 else (0.0 if gabs_np[slot, c] == 0 else np.inf)
        rows.append((slot, c, g, fd, spread, cond))
    ctx.synchronize()
    return rows


def check_rows(rows, label, min_resolved):
    """A gradient the central difference resolves -- its spread over step sizes below
    1e-4 of it, its terms not cancelling below 1 % of their summed size -- is held to
    1e-3 relative of that difference with no allowance; at least min_resolved of the
    64 are.  The others (a parameter that moves the image by less than the FP32
    forward's rounding in the pixels it touches) are held to 1e-3 plus four times the
    measured spread.  A slot no path reaches has no gradient either way (exact zeros)."""
    resolved = [r for r in rows if r[3] != 0.0 and r[4] <= 1e-4 * abs(r[3]) and r[5] <= 100.0]
    worst = max((abs(g - fd) / abs(fd) for _, _, g, fd, _, _ in resolved), default=0.0)
    print(f"{label}: {sum(1 for r in rows if r[3] != 0)} nonzero, {len(resolved)} resolved, worst relative error "
          f"of those {worst:.3g}")
    for r in rows:
        slot, c, g, fd, spread, cond = r
        if r in resolved:
            assert abs(g - fd) <= 1e-3 * abs(fd), (slot, c, g, fd, spread, cond)
        else:
            assert abs(g - fd) <= 1e-3 * abs(fd) + 4.0 * spread, (slot, c, g, fd, spread, cond)
    assert len(resolved) >= min_resolved


def test_inverse_albedo_adjoint_full_size_central_differences_seen_slots(inverse_setup):
    """64 parameters drawn from the slots the camera sees (450 of 4,092); on GB300 37
    of them are resolved (held to 1e-3 with no allowance), the floor is 32."""
    cov = inverse.pixel_coverage(inverse_setup[1], inverse_setup[2], inverse_setup[3], 512, 512)
    seen = np.flatnonzero(cov > 0)
    rng = np.random.default_rng(2024)
    picks = [(int(seen[k // 3]), int(k % 3)) for k in rng.choice(len(seen) * 3, 64, replace=False)]
    check_rows(central_differences(inverse_setup, picks), "seen slots", 32)


def test_inverse_albedo_adjoint_full_size_central_differences_all_slots(inverse_setup):
    """64 parameters drawn from all 4,092 matte slots (most reached by indirect light
    only); a slot that no path reaches has no gradient either way (exact zeros).  Most
    of these move the image by less than the FP32 forward's rounding: on GB300 4 of the
    61 nonzero ones are resolved, the floor is 3; the rest are held to 1e-3 plus four
    times their measured spread."""
    mats = inverse_setup[3]
    matte = np.flatnonzero(mats["kind"] != EMISSIVE)
    rng = np.random.default_rng(2025)
    picks = [(int(matte[k // 3]), int(k % 3)) for k in rng.choice(len(matte) * 3, 64, replace=False)]
    check_rows(central_differences(inverse_setup, picks), "all slots", 3)


def test_inverse_albedo_adjoint_full_size_against_fp64_host_adjoint(inverse_setup, oracle):
    ctx, scene, tris, mats, lights, cam, target, albedo, emission, params, adj, ga, ge = inverse_setup
    tree = oracle.build_sah(tris)
    ha, he, _ = oracle.pathtrace_adjoint(tree, tris, mats, lights, cam, params, albedo.cpu().numpy(),
                                         emission.cpu().numpy(), adj.cpu().numpy(), fp64=True)
    g = ga.cpu().numpy().astype(np.float64)
    ge_np = ge.cpu().numpy().astype(np.float64)
    rel_a = np.linalg.norm(g - ha) / np.linalg.norm(ha)
    rel_e = np.linalg.norm(ge_np - he) / np.linalg.norm(he)
    # per parameter: the slots the camera sees
    cov = inverse.pixel_coverage(scene, tris, mats, 512, 512)
    seen = cov > 0
    per = np.abs(g[seen] - ha[seen]) / np.maximum(np.abs(ha[seen]), 1e-30)
    print("fp64 host adjoint", rel_a, rel_e, "seen slots: median", float(np.median(per)), "p99",
          float(np.quantile(per, 0.99)))
    # the FP32 replay against the FP64 one: paths part where rounding flips a decision
    assert rel_a <= 2e-3 and rel_e <= 2e-3, (rel_a, rel_e)
    assert float(np.quantile(per, 0.95)) <= 1e-3


def test_batch_full_size_scenes_against_oracle(oracle):
    tris, offsets, cams, params, mats = scenes.batch_workload()
    ctx = vg.Context(0)
    d_tris = vg.as_device_bytes(tris)
    batch = vg.Batch(offsets, ctx)
    batch.set_frames(cams, params, mats)
    batch.build(d_tris)
    images = batch.pathtrace()
    ctx.synchronize()
    no_lights = np.zeros(0, AREA_LIGHT)
    worst = 1.0
    for s in range(0, 512, 32):
        t = tris[int(offsets[s]):int(offsets[s + 1])]
        img = batch.image(images, s, params).cpu().numpy().reshape(-1, 4)
        npix = len(img)
        pix = np.arange(0, npix, max(1, npix // 4096), dtype=np.uint32)
        ref, _ = oracle.pathtrace_pixels(oracle.build_sah(t), t, mats, no_lights, cams[s], params[s], pix,
                                         mode=Oracle.PT_FLOAT_TRIG_DOUBLE)
        st = pixel_stats(img[pix], ref)
        worst = min(worst, st["exact"])
        # 1 spp of 3 segments: a pixel differs only through an equal-t tie resolved in
        # another order by the GPU tree and the oracle's SAH tree
        assert st["exact"] >= 0.97, (s, len(t), st)
        assert st["rmse"] <= 0.02 * max(st["mean"], 1e-6), (s, len(t), st)
    print("worst exact fraction over 16 scenes", worst)
    batch.close()
