"""Times visionaray's own GPU kernels beside the product's on the same GB300.

BENCHMARK INFRASTRUCTURE (runs the reference's device code from
oracle/_ref/vsnray_ref_gpu.cubin through oracle/ref_gpu.py):

    python oracle/bench_reference_gpu.py [--reps 5] [--pt-spp 64]

Workloads are bench.py's: the 2048x2048 heightfield (8,388,608 triangles) with
4,194,304 closest-hit and 33,554,432 any-hit AO rays, traced by visionaray's
closest_hit / any_hit over the cuda_index_bvh that its GPU lbvh_builder produces for
these triangles (the product's export, byte-identical to it), one thread per ray, best
of 64/128/256-thread blocks; visionaray's GPU LBVH build of those triangles (its
kernels, CUB's merge sort), compared with the product's tree byte for byte; and the closed-box path-tracing scene at 1920x1080,
depth 8, through pathtracing::kernel one thread per pixel in cuda_sched's 16x16 blocks.
The product runs its default configuration on the same inputs.  Times are CUDA events
on the launching stream, median of `reps` after a warm-up; prints one JSON line.
"""
import argparse
import json
import os
import statistics
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def timed(fn, reps):
    import torch
    fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        out.append(a.elapsed_time(b))
    return statistics.median(out)


def traversal(ref, ctx, d_tris, bvh, d_c, d_a, reps):
    """visionaray's closest_hit / any_hit kernels (best of 64/128/256-thread blocks) and
    the product's queries on the same tree (the product's LBVH export, byte-identical to
    the reference GPU builder's) and rays."""
    import torch

    import visionaray_gb300 as vg
    from visionaray_gb300.types import NO_HIT
    n_c, n_a = d_c.shape[0], d_a.shape[0]
    tree = ref.tree(d_tris, bvh)
    h_c = torch.empty((n_c, 4), dtype=torch.float32, device=d_c.device)
    h_a = torch.empty((n_a, 4), dtype=torch.float32, device=d_c.device)
    r_c, r_a = torch.empty_like(h_c), torch.empty_like(h_a)
    ours_c = timed(lambda: vg.closest_hit(d_c, bvh, out=h_c), reps)
    ours_a = timed(lambda: vg.any_hit(d_a, bvh, out=h_a), reps)
    ref_c, ref_a = {}, {}
    for block in (64, 128, 256):
        ref_c[block] = timed(lambda: ref.trace(tree, d_c, r_c, any_hit=False, block=block), reps)
        ref_a[block] = timed(lambda: ref.trace(tree, d_a, r_a, any_hit=True, block=block), reps)
    bc, ba = min(ref_c, key=ref_c.get), min(ref_a, key=ref_a.get)
    ctx.synchronize()
    hc, rc = vg.hits_to_numpy(h_c), vg.hits_to_numpy(r_c)
    ha, ra = vg.hits_to_numpy(h_a), vg.hits_to_numpy(r_a)
    hit_o, hit_r = hc["prim_id"] != NO_HIT, rc["prim_id"] != NO_HIT
    return {"reps": reps, "tree_height": bvh.counts[2],
            "ours": {"closest_ms": round(ours_c, 3), "any_ms": round(ours_a, 3),
                     "closest_mrays_s": round(n_c / (ours_c * 1e-3) / 1e6, 1),
                     "any_mrays_s": round(n_a / (ours_a * 1e-3) / 1e6, 1)},
            "reference_gpu": {"closest_ms": round(ref_c[bc], 3), "any_ms": round(ref_a[ba], 3),
                              "closest_block": bc, "any_block": ba,
                              "closest_mrays_s": round(n_c / (ref_c[bc] * 1e-3) / 1e6, 1),
                              "any_mrays_s": round(n_a / (ref_a[ba] * 1e-3) / 1e6, 1)},
            "closest_speedup": round(ref_c[bc] / ours_c, 2), "any_speedup": round(ref_a[ba] / ours_a, 2),
            "agreement": {"closest_prim_equal": float((hc["prim_id"] == rc["prim_id"]).mean()),
                          "closest_hit_flag_equal": float((hit_o == hit_r).mean()),
                          "ao_occlusion_equal": float(((ha["prim_id"] != NO_HIT) == (ra["prim_id"] != NO_HIT)).mean())}}


def lbvh_build(ref, ctx, d_tris, reps):
    """visionaray's GPU LBVH build (lbvh_builder::build, detail/bvh/lbvh.h:681-844: its
    own kernels, CUB's stable merge sort, the primitive copy) against the product's
    build of the same triangles: the trees compared byte for byte (nodes and indices of
    the reference's cuda_index_bvh layout; the product's through gbrt_bvh_export_bvh2),
    then both timed.  The reference's device arrays are allocated once, outside its
    timed builds (its own build allocates them on every call); the product is timed
    both ways: the public build (allocates the tree) and the in-place rebuild (none)."""
    import torch

    import visionaray_gb300 as vg
    n = d_tris.numel() // 44
    b = ref.lbvh_buffers(n)
    nodes_r, idx_r = ref.lbvh_build(d_tris, b)
    bvh = vg.lbvh_builder(ctx).build(d_tris)
    nodes_o, idx_o = bvh.export_bvh2()
    torch.cuda.synchronize()
    same_nodes = bool(np.array_equal(nodes_r.cpu().numpy(), np.ascontiguousarray(nodes_o).view(np.uint8)))
    same_idx = bool(np.array_equal(idx_r.cpu().numpy(), np.ascontiguousarray(idx_o).view(np.uint8)))
    ms_r = timed(lambda: ref.lbvh_build(d_tris, b), reps)
    ms_o = timed(lambda: vg.lbvh_builder(ctx).build(d_tris), reps)
    ms_rebuild = timed(lambda: bvh.rebuild(d_tris), reps)
    ctx.synchronize()
    return {"triangles": int(n), "tree_nodes_identical": same_nodes, "tree_indices_identical": same_idx,
            "reference_gpu_ms": round(ms_r, 3), "ours_build_ms": round(ms_o, 3), "ours_rebuild_ms": round(ms_rebuild, 3),
            "speedup": round(ms_r / ms_o, 2), "speedup_rebuild": round(ms_r / ms_rebuild, 2),
            "note": "reference timed without its per-build allocations; sort = CUB DeviceMergeSort::StableSortKeys "
                    "as the reference calls it"}


def pathtrace(ref, ctx, spp, reps, builder="lbvh"):
    """visionaray's pathtracing::kernel (one thread per pixel, 16x16 blocks) and the
    product's frame on the box scene at 1920x1080, depth 8, through the same tree."""
    import torch

    import bench
    import visionaray_gb300 as vg
    from visionaray_gb300 import scenes
    tris, mats, lights = scenes.box_scene()
    d_tris = vg.as_device_bytes(tris, ctx.device)
    make = vg.ploc_builder if builder == "ploc" else vg.lbvh_builder
    bvh = make(ctx).build(d_tris)
    scene = vg.PTScene(bvh, mats, lights)
    cam = scenes.box_camera()
    params = scenes.pt_params(bench.PT_WIDTH, bench.PT_HEIGHT, spp, num_bounces=bench.PT_BOUNCES)
    img_o = torch.zeros((bench.PT_HEIGHT, bench.PT_WIDTH, 4), dtype=torch.float32, device=d_tris.device)
    ms_o = timed(lambda: vg.pathtrace_frame(scene, cam, params, accum=img_o), reps)
    rscene = ref.pt_scene(ref.tree(d_tris, bvh), mats, lights)
    img_r = torch.zeros_like(img_o)
    ms_r = timed(lambda: ref.pathtrace(rscene, cam, params, img_r), reps)
    ctx.synchronize()
    samples = bench.PT_WIDTH * bench.PT_HEIGHT * spp
    a, b = img_o[..., :3].double(), img_r[..., :3].double()
    return {"workload": bench.PT_WORKLOAD.replace("64 spp", f"{spp} spp"), "builder": builder,
            "ours_ms": round(ms_o, 2), "reference_gpu_ms": round(ms_r, 2),
            "ours_msamples_s": round(samples / (ms_o * 1e-3) / 1e6, 1),
            "reference_gpu_msamples_s": round(samples / (ms_r * 1e-3) / 1e6, 1),
            "speedup": round(ms_r / ms_o, 2),
            "image_mean": [round(float(a.mean()), 5), round(float(b.mean()), 5)]}


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--reps", type=int, default=5)
    p.add_argument("--pt-spp", type=int, default=64)
    p.add_argument("--grid", type=int, default=2048)
    p.add_argument("--origins", type=int, default=1 << 22)
    args = p.parse_args()

    import torch

    import bench
    import visionaray_gb300 as vg
    from oracle import build as oracle_build
    from oracle import ref_gpu
    from visionaray_gb300 import build, scenes

    build.build()
    oracle_build.build()
    ref = ref_gpu.ReferenceGPU(0)
    ctx = vg.default_context(0)
    ctx.set_trace_flags(ctx.TRACE_SORT_RAYS)
    tris, closest, ao = bench.workload(print, grid=args.grid, origins=args.origins)
    d_tris = vg.as_device_bytes(tris)
    bvh = vg.lbvh_builder(ctx).build(d_tris)
    res = {"workload": bench.WORKLOAD, "traversal": traversal(ref, ctx, d_tris, bvh, vg.device_rays(closest),
                                                               vg.device_rays(ao), args.reps),
           "lbvh_build": lbvh_build(ref, ctx, d_tris, args.reps)}
    del bvh, d_tris
    torch.cuda.empty_cache()
    res["pathtrace"] = pathtrace(ref, ctx, args.pt_spp, max(1, args.reps // 2))

    # path tracing with every material kind and generic lights: the box scene's 256
    # blobs cycling matte, plastic, mirror, plastic, glass, plastic walls, lit by
    # the ceiling light plus two point lights and a spot light
    tris, mats, area = scenes.glossy_box_scene(n_blobs=256, subdiv=22, seed=1)
    lights = scenes.mixed_lights(area)
    d_tris = vg.as_device_bytes(tris)
    bvh = vg.lbvh_builder(ctx).build(d_tris)
    scene = vg.PTScene(bvh, mats, lights)
    cam = scenes.box_camera()
    spp = max(1, args.pt_spp // 4)
    params = scenes.pt_params(bench.PT_WIDTH, bench.PT_HEIGHT, spp, num_bounces=bench.PT_BOUNCES)
    img_o = torch.zeros((bench.PT_HEIGHT, bench.PT_WIDTH, 4), dtype=torch.float32, device="cuda:0")
    ms_o = timed(lambda: vg.pathtrace_frame(scene, cam, params, accum=img_o), max(1, args.reps // 2))
    rscene = ref.pt_scene(ref.tree(d_tris, bvh), mats, lights)
    img_r = torch.zeros_like(img_o)
    ms_r = timed(lambda: ref.pathtrace(rscene, cam, params, img_r), max(1, args.reps // 2))
    ctx.synchronize()
    samples = bench.PT_WIDTH * bench.PT_HEIGHT * spp
    a, b = img_o[..., :3].double(), img_r[..., :3].double()
    res["pathtrace_materials"] = {
        "workload": f"glossy box (256 blobs cycling matte/plastic/mirror/plastic/glass, plastic walls, "
                    f"{len(tris):,} tris) + area, 2 point and 1 spot light, {bench.PT_WIDTH}x{bench.PT_HEIGHT}, "
                    f"{spp} spp, depth {bench.PT_BOUNCES}",
        "ours_ms": round(ms_o, 2), "reference_gpu_ms": round(ms_r, 2),
        "ours_msamples_s": round(samples / (ms_o * 1e-3) / 1e6, 1),
        "reference_gpu_msamples_s": round(samples / (ms_r * 1e-3) / 1e6, 1),
        "speedup": round(ms_r / ms_o, 2),
        "image_mean": [round(float(a.mean()), 5), round(float(b.mean()), 5)]}
    print(json.dumps(res), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
