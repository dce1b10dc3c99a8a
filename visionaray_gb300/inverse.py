"""Inverse rendering of per-primitive albedo with the path-replay adjoint.

The workload: the path-tracing box scene reduced to 4,094 triangles (the box, the
ceiling light and 204 blobs of 20 triangles: icospheres at the lowest subdivision), a
target image rendered from hidden albedos, and Adam steps on the albedos from a uniform
start, each step a forward frame, the L2 image loss and the backward pass
(gbrt_pathtrace_forward / gbrt_pathtrace_backward).  At 512x512 the camera sees 450 of
the 4,092 matte slots directly (310 of them on 64 pixels or more); the other slots are
reached by indirect light only, or not at all, and their albedos are not identifiable
from the image.

Gradient estimator.  The L2 loss's image adjoint 2 (I - T) / npix comes from the
forward frame's noisy image I.  Replaying the backward pass with the forward frame's
random numbers multiplies that adjoint by dI/da of the *same* samples, and
E[(I - T) dI/da] = (E[I] - T) E[dI/da] + Cov(I, dI/da): the covariance term biases
every step (towards darker albedos wherever the image is noisy).  The backward pass
therefore replays an independent frame (frame id + GRAD_FRAME_OFFSET), whose dI/da is
independent of I, so the step's gradient is an unbiased estimate of the gradient of the
loss of the mean image (the decorrelated estimator of differentiable renderers such as
Mitsuba 3's separate primal and adjoint seeds).  `correlated=True` restores the
same-seed replay for comparison (`gradient_bias` measures both).
"""
import numpy as np

from . import runtime as rt
from . import scenes
from .types import PT_NO_RUSSIAN_ROULETTE, PT_SHADOW_RANGE_FIX

FLAGS = PT_SHADOW_RANGE_FIX | PT_NO_RUSSIAN_ROULETTE
GRAD_FRAME_OFFSET = 1 << 24      # backward frames: independent of every forward frame
TARGET_FRAME = (1 << 25) + 1000  # the target image's frame: independent of both


def setup(n_blobs=204, subdiv=1, seed=1, hidden_seed=5, ctx=None, builder="lbvh"):
    """(scene, tris, materials, lights, hidden albedo, emission) on the GPU."""
    import torch
    ctx = ctx or rt.default_context()
    tris, mats, lights = scenes.box_scene(n_blobs=n_blobs, subdiv=subdiv, seed=seed)
    make = rt.ploc_builder if builder == "ploc" else rt.lbvh_builder
    bvh = make(ctx).build(rt.as_device_bytes(tris, ctx.device))
    scene = rt.PTScene(bvh, mats, lights)
    rng = np.random.default_rng(hidden_seed)
    hidden = rng.uniform(0.1, 0.9, size=(len(mats), 3)).astype(np.float32)
    dev = f"cuda:{ctx.device}"
    emission = torch.from_numpy(np.ascontiguousarray(mats["color"], np.float32)).to(dev)
    return scene, tris, mats, lights, torch.from_numpy(hidden).to(dev), emission


def l2_adjoint(image, target):
    """L = mean over pixels of sum over RGB of (I - T)^2, and dL/dI (alpha zero)."""
    import torch
    d = image[..., :3] - target[..., :3]
    npix = image.shape[0] * image.shape[1]
    loss = (d.double() ** 2).sum() / npix
    adj = torch.zeros_like(image)
    adj[..., :3] = 2.0 * d / npix
    return float(loss), adj


def pixel_coverage(scene, tris, mats, width, height, camera=None):
    """Pixels per material slot whose pixel-centre primary ray hits a triangle of that
    slot (the box camera at width x height); emissive slots are reported as 0."""
    from .types import EMISSIVE
    cam = scenes.box_camera() if camera is None else camera
    rays = scenes.pinhole_rays(width, height, eye=tuple(cam["eye"]), center=tuple(cam["center"]),
                               up=tuple(cam["up"]), fovy_degrees=float(cam["fovy_degrees"]))
    hits = rt.hits_to_numpy(rt.closest_hit(rt.device_rays(rays, scene.ctx.device), scene.bvh))
    prim = hits["prim_id"]
    hit = prim != np.uint32(0xFFFFFFFF)
    slots = tris["geom_id"][prim[hit].astype(np.int64)]
    cov = np.bincount(slots.astype(np.int64), minlength=len(mats)).astype(np.int64)
    cov[mats["kind"] == EMISSIVE] = 0
    return cov


def albedo_errors(albedo, hidden, coverage, min_pixels=64):
    """Mean |albedo - hidden| over three fixed sets of slots: every slot seen by at least
    one pixel, the same weighted by pixel coverage, and the slots of >= min_pixels."""
    err = np.abs(albedo - hidden).mean(axis=1)
    seen = coverage > 0
    big = coverage >= min_pixels
    w = coverage.astype(np.float64)
    return {"seen": float(err[seen].mean()) if seen.any() else None,
            "coverage_weighted": float((err * w).sum() / w.sum()) if w.sum() > 0 else None,
            f"slots_ge_{min_pixels}px": float(err[big].mean()) if big.any() else None}


def optimize(steps=200, lr=0.02, width=512, height=512, spp=16, depth=6, target_spp=256, ctx=None, log=None,
             extra_flags=0, builder="lbvh", correlated=False, min_pixels=64):
    """Adam on the albedos.  Returns a dict with the loss history, the parameter errors
    at the start and the end on the same fixed sets of slots (albedo_errors), and the
    median forward / backward times (CUDA events).

    Under torch.distributed with N > 1 ranks (one GPU each) the step is data-parallel
    over samples: rank r renders its replicas.split_samples(spp, N)[r] samples per
    pixel with frame_id = step * N + r, the images are averaged by an all-reduce, every
    rank back-propagates the common loss through its own samples, and the gradients
    are summed by an all-reduce, so all ranks take the same Adam step.  With one rank
    this is the single-GPU step (frame_id = step)."""
    import torch
    import torch.distributed as dist

    from . import replicas
    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    rank = dist.get_rank() if world > 1 else 0
    my_spp = replicas.split_samples(spp, world)[rank]
    ctx = ctx or rt.default_context()
    scene, tris, mats, lights, hidden, emission = setup(ctx=ctx, builder=builder)
    cam = scenes.box_camera()
    coverage = pixel_coverage(scene, tris, mats, width, height, cam)
    tparams = scenes.pt_params(width, height, target_spp, num_bounces=depth, frame_id=TARGET_FRAME,
                               flags=FLAGS | extra_flags)
    target = rt.pathtrace_forward(scene, cam, tparams, hidden, emission)
    albedo = torch.full_like(hidden, 0.5)
    hidden_np = hidden.cpu().numpy()
    errors_start = albedo_errors(albedo.cpu().numpy(), hidden_np, coverage, min_pixels)
    m = torch.zeros_like(albedo)
    v = torch.zeros_like(albedo)
    b1, b2, eps = 0.9, 0.999, 1e-8
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fwd_ms, bwd_ms, losses = [], [], []
    image = None
    for it in range(steps):
        frame = it * world + rank
        params = scenes.pt_params(width, height, my_spp, num_bounces=depth, frame_id=frame,
                                  flags=FLAGS | extra_flags)
        gparams = params if correlated else scenes.pt_params(
            width, height, my_spp, num_bounces=depth, frame_id=frame + GRAD_FRAME_OFFSET, flags=FLAGS | extra_flags)
        ev[0].record(ctx.stream)
        image = rt.pathtrace_forward(scene, cam, params, albedo, emission, image=image)
        ev[1].record(ctx.stream)
        if world > 1:
            torch.cuda.synchronize()   # the collective runs on torch's stream
            replicas.mean_image_(image, my_spp, spp)
        loss, adj = l2_adjoint(image, target)
        if world > 1:
            adj.mul_(float(my_spp) / float(spp))   # this rank's share of the mean image
        grad_a = torch.zeros_like(albedo)
        grad_e = torch.zeros_like(emission)
        ev[2].record(ctx.stream)
        e3 = torch.cuda.Event(enable_timing=True)
        rt.pathtrace_backward(scene, cam, gparams, albedo, emission, adj, grad_a, grad_e)
        e3.record(ctx.stream)
        torch.cuda.synchronize()
        if world > 1:
            replicas.all_reduce_sum_(grad_a)
            replicas.all_reduce_sum_(grad_e)
        fwd_ms.append(ev[0].elapsed_time(ev[1]))
        bwd_ms.append(ev[2].elapsed_time(e3))
        losses.append(loss)
        # Adam (Kingma & Ba 2015), albedo kept in [0, 1]
        m.mul_(b1).add_(grad_a, alpha=1 - b1)
        v.mul_(b2).addcmul_(grad_a, grad_a, value=1 - b2)
        mh = m / (1 - b1 ** (it + 1))
        vh = v / (1 - b2 ** (it + 1))
        albedo.sub_(lr * mh / (vh.sqrt() + eps)).clamp_(0.0, 1.0)
        if log and (it % 20 == 0 or it == steps - 1):
            log(f"step {it} loss {loss:.6g}")
    ctx.synchronize()
    errors_end = albedo_errors(albedo.cpu().numpy(), hidden_np, coverage, min_pixels)
    return {"losses": losses, "fwd_ms": float(np.median(fwd_ms)), "bwd_ms": float(np.median(bwd_ms)),
            "errors_start": errors_start, "errors_end": errors_end, "triangles": int(len(tris)),
            "slots_seen": int((coverage > 0).sum()), f"slots_ge_{min_pixels}px": int((coverage >= min_pixels).sum()),
            "estimator": "correlated" if correlated else "decorrelated"}


def gradient_bias(rounds=(16, 64), width=512, height=512, spp=16, depth=6, ref_spp=1024, ctx=None, builder="lbvh",
                  min_pixels=64):
    """Bias of the per-step gradient estimator at one albedo state (0.5 everywhere), on
    the slots seen by at least min_pixels pixels: the mean of M independent 16-spp steps
    of (a) the same-seed replay and (b) the decorrelated replay, each against a
    reference gradient of the loss of the (nearly) noise-free image (its adjoint from a
    ref_spp forward frame, its dI/da from an independent ref_spp replay).  Returns the
    relative L2 distance to the reference after each M in `rounds`: an unbiased
    estimator's distance falls as 1/sqrt(M), a biased one levels off at its bias."""
    import torch
    ctx = ctx or rt.default_context()
    scene, tris, mats, lights, hidden, emission = setup(ctx=ctx, builder=builder)
    cam = scenes.box_camera()
    seen = torch.from_numpy(pixel_coverage(scene, tris, mats, width, height, cam) >= min_pixels).to(hidden.device)
    tparams = scenes.pt_params(width, height, 256, num_bounces=depth, frame_id=TARGET_FRAME, flags=FLAGS)
    target = rt.pathtrace_forward(scene, cam, tparams, hidden, emission)
    albedo = torch.full_like(hidden, 0.5)

    def grad(fwd_frame, bwd_frame, s):
        p = scenes.pt_params(width, height, s, num_bounces=depth, frame_id=fwd_frame, flags=FLAGS)
        q = scenes.pt_params(width, height, s, num_bounces=depth, frame_id=bwd_frame, flags=FLAGS)
        img = rt.pathtrace_forward(scene, cam, p, albedo, emission)
        _, adj = l2_adjoint(img, target)
        ga, _ = rt.pathtrace_backward(scene, cam, q, albedo, emission, adj)
        return ga.double()[seen]

    ref = grad(1 << 26, (1 << 26) + 1, ref_spp)
    n = float(ref.norm())
    same = torch.zeros_like(ref)
    dec = torch.zeros_like(ref)
    out = {"slots": int(seen.sum()), "spp": spp, "ref_spp": ref_spp, "rounds": list(rounds),
           "correlated_rel_l2": [], "decorrelated_rel_l2": []}
    for r in range(max(rounds)):
        same += grad(r, r, spp)
        dec += grad(r, r + GRAD_FRAME_OFFSET, spp)
        if r + 1 in rounds:
            out["correlated_rel_l2"].append(round(float((same / (r + 1) - ref).norm()) / n, 4))
            out["decorrelated_rel_l2"].append(round(float((dec / (r + 1) - ref).norm()) / n, 4))
    ctx.synchronize()
    return out
