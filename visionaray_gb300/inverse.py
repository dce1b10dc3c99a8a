"""Inverse rendering of per-primitive albedo with the path-replay adjoint.

The workload: the path-tracing box scene reduced to ~4k triangles (2 blobs of 2,000),
a target image rendered from hidden albedos, and Adam steps on the albedos from a
uniform start, each step a forward frame, the L2 image loss and the backward pass
(gbrt_pathtrace_forward / gbrt_pathtrace_backward).  Random numbers are common
(frame_id fixed) between the forward and backward pass of a step.
"""
import numpy as np

from . import runtime as rt
from . import scenes
from .types import PT_NO_RUSSIAN_ROULETTE, PT_SHADOW_RANGE_FIX

FLAGS = PT_SHADOW_RANGE_FIX | PT_NO_RUSSIAN_ROULETTE


def setup(n_blobs=2, subdiv=10, seed=1, hidden_seed=5, ctx=None, builder="lbvh"):
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


def optimize(steps=200, lr=0.02, width=512, height=512, spp=16, depth=6, target_spp=256, ctx=None, log=None,
             extra_flags=0, builder="lbvh"):
    """Adam on the albedos.  Returns a dict with the loss history, the parameter error
    and the mean forward / backward times (CUDA events).

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
    tparams = scenes.pt_params(width, height, target_spp, num_bounces=depth, frame_id=1000, flags=FLAGS | extra_flags)
    target = rt.pathtrace_forward(scene, cam, tparams, hidden, emission)
    albedo = torch.full_like(hidden, 0.5)
    m = torch.zeros_like(albedo)
    v = torch.zeros_like(albedo)
    b1, b2, eps = 0.9, 0.999, 1e-8
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fwd_ms, bwd_ms, losses = [], [], []
    image = None
    for it in range(steps):
        params = scenes.pt_params(width, height, my_spp, num_bounces=depth, frame_id=it * world + rank,
                                  flags=FLAGS | extra_flags)
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
        rt.pathtrace_backward(scene, cam, params, albedo, emission, adj, grad_a, grad_e)
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
    seen = (grad_a.abs().sum(1) > 0).cpu().numpy()
    err0 = float((0.5 - hidden).abs().mean())
    err = float((albedo - hidden).abs()[torch.from_numpy(seen).to(albedo.device)].mean()) if seen.any() else err0
    return {"losses": losses, "fwd_ms": float(np.median(fwd_ms)), "bwd_ms": float(np.median(bwd_ms)),
            "albedo_error_start": err0, "albedo_error_end_seen": err, "triangles": int(len(tris))}
