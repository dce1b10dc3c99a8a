"""Benchmark of the ray-tracing hot path: LBVH build + incoherent traversal on the
2048x2048 sine heightfield (8,388,608 triangles), 4,194,304 secondary closest-hit rays
from surface points plus 8 ambient-occlusion any-hit rays per origin (tmax 0.05),
33,554,432 of them.  One step = closest_hit over the 4M rays + any_hit over the 32M
rays; the metric is rays traced per second over both kinds (Mrays/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times visionaray's own CPU path for the same workload (the
oracle's restatement, pinned to the reference's CPU code; its binned-SAH tree; all
host threads) on a bounded sample of each step.  For N > 1 (torchrun) every rank
traces its own replica (replicas only: the path has no exchange step) and the value is
the whole job's rays / the slowest rank's time.  Data are synthetic (seeded generators
of visionaray_gb300.scenes); inputs (1.2 GB of rays, 0.9 GB of BVH) exceed the 129 MB L2.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "incoherent closest-hit Mrays/s; PT Msamples/s batched vs plain; bwd/fwd time"
UNIT = "Mrays/s"
GRID, SCENE_SEED = 2048, 1
ORIGINS, RAY_SEED, AO_PER_ORIGIN, AO_TMAX, OFFSET = 1 << 22, 7, 8, 0.05, 1e-4
WORKLOAD = ("heightfield 2048x2048 (8,388,608 tris, 6 sine octaves) LBVH; one step = closest_hit over 4,194,304 "
            "incoherent secondary rays (cosine-weighted from surface points); the 33,554,432 any-hit AO rays "
            "(tmax 0.05) and the LBVH build are timed beside it")

# Algorithmic bytes per ray, B_ray = 32 (ray) + 16 (hit) + N_node*32 + N_tri*48, with
# N_node / N_tri the mean box / triangle tests per ray of visionaray's CPU traversal on
# its binned-SAH BVH2 of this heightfield, counted over all 4,194,304 closest rays and
# all 33,554,432 AO rays of this workload (oracle counters, equal to the reference's).
N_NODE_CLOSEST, N_TRI_CLOSEST = 76.92786217, 7.44575715   # B_ray = 2867.1 bytes
N_NODE_AO, N_TRI_AO = 65.19375747, 6.29761556             # B_ray = 2436.5 bytes


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum, mean of two
# launches each in one ncu capture of the full-size workload with the default ray
# order and the shipped kernel build).
TRAFFIC_CLOSEST, TRAFFIC_ANY = 2.705e9 + 0.201e9, 2.642e9 + 0.542e9
# L1 <-> L2 bytes per launch of the same kernels (lts__t_sectors_srcunit_tex_op_read.sum
# + lts__t_sectors_srcunit_tex_op_write.sum, 32-byte sectors; one single-pass ncu
# capture of the full-size workload).
L2_TRAFFIC_CLOSEST, L2_TRAFFIC_ANY = (336.27e6 + 45.39e6) * 32, (878.37e6 + 37.64e6) * 32


# Algorithmic bytes per path-traced sample, B_sample = sum of B_ray over the sample's
# path segments and shadow rays, counted on the oracle's FP32 run of each workload at
# the CUDA path's random numbers (python -m oracle.b_sample): the box frame (every 61st
# pixel, 64 spp: 6.75 segments per sample), the batch (every 8th scene, 1.77 segments)
# and the inverse-rendering frame (every 7th pixel, 16 spp: 11.9 segments).
B_SAMPLE_BOX, B_SAMPLE_BATCH, B_SAMPLE_INVERSE = 24726.4, 6132.6, 31621.4


def b_ray(n_node, n_tri):
    return 32 + 16 + n_node * 32 + n_tri * 48


def measured_l2_gbs(device):
    """L2 bandwidth measured here (no L2 peak is recorded for this GPU): the best of a
    device-to-device copy (read + write), an in-place add (read + write) and a sum
    (read) over buffers that stay resident in the 129 MB L2 (16 and 32 MB), in bytes
    moved over the CUDA-event time, best of 5 rounds of 50 operations each."""
    import torch
    best = 0.0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for mb in (16, 32):
        n = mb * 1024 * 1024 // 4
        a = torch.ones(n, dtype=torch.float32, device=device)
        b = torch.empty_like(a)
        for name, op, moved in (("copy", lambda: b.copy_(a), 8 * n), ("add", lambda: a.add_(1.0), 8 * n),
                                ("sum", lambda: a.sum(), 4 * n)):
            for _ in range(20):
                op()
            for _ in range(5):
                e0.record()
                for _ in range(50):
                    op()
                e1.record()
                torch.cuda.synchronize()
                best = max(best, moved * 50 / (e0.elapsed_time(e1) * 1e-3) / 1e9)
        del a, b
    return round(best, 1)


def roofline_of(samples, seconds, b_sample, peak, peak_source, scope, bound="hbm"):
    achieved = samples * b_sample / seconds / 1e9
    return {"bound": bound, "scope": scope, "b_sample": b_sample, "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_source}


def pt_cpu_baseline(tris, mats, lights, cam, params, pixel_step):
    """visionaray's pathtracing::kernel on the CPU (the oracle's FP32 mode, equal to the
    reference's kernel bit for bit; its binned-SAH tree, not timed; all host threads) on
    every pixel_step-th pixel of the frame: Msamples/s."""
    from oracle import Oracle
    o = Oracle()
    tree = o.build_sah(tris)
    npix = int(params["width"]) * int(params["height"])
    pix = np.arange(0, npix, pixel_step, dtype=np.uint32)
    t0 = time.perf_counter()
    o.pathtrace_pixels(tree, tris, mats, lights, cam, params, pix, mode=Oracle.PT_FLOAT)
    dt = time.perf_counter() - t0
    samples = len(pix) * int(params["spp"])
    return {"value": round(samples / dt / 1e6, 3), "unit": "Msamples/s", "cores": os.cpu_count() or 1,
            "kind": "port", "sample": f"every {pixel_step}th pixel ({len(pix)} pixels x {int(params['spp'])} spp, "
                                      f"{dt:.2f} s); binned-SAH tree not timed"}


def measured_hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload(rank_print=print, grid=GRID, origins=ORIGINS):
    from visionaray_gb300 import scenes
    t0 = time.time()
    tris = scenes.heightfield(grid=grid, seed=SCENE_SEED)
    closest, ao = scenes.surface_rays(tris, origins, seed=RAY_SEED, offset=OFFSET,
                                      ao_per_origin=AO_PER_ORIGIN, ao_tmax=AO_TMAX)
    rank_print(f"# workload generated in {time.time() - t0:.1f} s", file=sys.stderr)
    return tris, closest, ao


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 25 ms with timestamps from
    before the warm-up on, summarised over the samples inside the marked (timed) region
    (the nearest one if the region is shorter than the sampling period)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "25"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        import datetime
        rows = []
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                t = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((t, float(parts[2]), float(parts[3]), parts[6:10]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        t0 = self.t0 if self.t0 is not None else rows[0][0]
        t1 = self.t1 if self.t1 is not None else rows[-1][0]
        inside = [r for r in rows if t0 <= r[0] <= t1]
        nearest = not inside
        if nearest:
            mid = 0.5 * (t0 + t1)
            inside = [min(rows, key=lambda r: abs(r[0] - mid))]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = {n for r in inside for n, v in zip(names, r[3]) if v.lower() == "active"}
        out = {"sm_mhz": statistics.median(r[1] for r in inside), "sm_max_mhz": inside[-1][2],
               "reasons": sorted(reasons), "samples": len(inside)}
        if nearest:
            out["nearest_sample"] = True
        return out


def workload_config(grid, origins, n_closest, n_any, n_tris, builder="lbvh"):
    """The line's `config`: the workload alone, identical in both arms (what each run
    measured beside it goes elsewhere in the line)."""
    return {"workload": WORKLOAD if (grid, origins) == (GRID, ORIGINS) else
            f"REDUCED profiling case: heightfield {grid}x{grid}, {origins} origins",
            "rays_per_step": n_closest, "closest_rays": n_closest, "anyhit_rays": n_any, "triangles": n_tris,
            "builder": builder, "l2": "inputs larger than L2 (no flush)"}


def cpu_baseline(tris, closest, ao, rank_print=print, sample_every=4, repeats=1, any_repeats=1):
    """The reference's CPU path (oracle restatement, binned-SAH tree, all host threads)
    on every `sample_every`-th origin: its closest-hit ray `repeats` times, then its AO
    rays `any_repeats` times."""
    from oracle import Oracle, Reference
    kind = "reference" if Reference.available() else "port"
    nthreads = os.cpu_count() or 1
    t0 = time.time()
    if kind == "reference":
        ref = Reference()
        handle = ref.build_sah(tris)
        trace = lambda r, a: handle.trace(r, any_hit=a, nthreads=nthreads)  # noqa: E731
    else:
        o = Oracle()
        tree = o.build_sah(tris)
        trace = lambda r, a: o.trace(tree, tris, r, any_hit=a, nthreads=nthreads)  # noqa: E731
    build_s = time.time() - t0
    sel = np.arange(0, len(closest), sample_every)
    c_s = closest[sel]
    a_s = ao.reshape(len(closest), AO_PER_ORIGIN)[sel].reshape(-1)
    times_c, times_a = [], []
    for _ in range(repeats):
        t0 = time.perf_counter()
        trace(c_s, False)
        times_c.append(time.perf_counter() - t0)
    for _ in range(any_repeats):
        t0 = time.perf_counter()
        trace(a_s, True)
        times_a.append(time.perf_counter() - t0)
    return {"kind": kind, "cores": nthreads, "build_s": build_s, "closest_rays": len(c_s), "any_rays": len(a_s),
            "closest_times": times_c, "any_times": times_a,
            "sample": f"every {sample_every}th origin: {len(c_s)} closest-hit rays ({len(a_s)} AO rays for the "
                      f"any-hit figure); binned-SAH tree built in {build_s:.1f} s (not timed)"}


# The restatement against visionaray's own CPU code on the same tree and rays (x86-64, 8
# threads, heightfield 512x512, binned-SAH tree; identical hits): where the reference's
# CPU code cannot be built (the GPU host has no visionaray sources), the baseline is the
# restatement and runs at this fraction of the reference's speed.
PORT_VS_REFERENCE = {"closest": round(1.69 / 2.19, 3), "any": round(5.11 / 5.25, 3),
                     "measured": "x86-64, 8 threads, heightfield 512x512, binned-SAH tree, identical hits"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    tris, closest, ao = workload(grid=args.grid, origins=args.origins)
    res = cpu_baseline(tris, closest, ao, sample_every=4, repeats=args.warmup + args.steps)
    t = res["closest_times"][args.warmup:]
    ms = 1e3 * statistics.mean(t)
    value = res["closest_rays"] / statistics.mean(t) / 1e6
    any_value = res["any_rays"] / min(res["any_times"]) / 1e6
    base = {"value": round(value, 3), "unit": UNIT, "cores": res["cores"], "kind": res["kind"],
            "sample": res["sample"], "any_hit_mrays_s": round(any_value, 3)}
    if res["kind"] == "port":
        base["port_vs_reference"] = PORT_VS_REFERENCE
    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args.grid, args.origins, len(closest), len(ao), len(tris)),
            "run": {"sample": "each step a bounded sample of the workload (cpu_baseline.sample)",
                    "threads": res["cores"]},
            "cpu_baseline": base,
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


PT_WIDTH, PT_HEIGHT, PT_SPP, PT_BOUNCES = 1920, 1080, 64, 8
PT_WORKLOAD = ("path tracing: closed unit box + 0.25^2 ceiling light (emission 15) + 256 noisy icosphere "
               "blobs (2,478,094 tris, Lambertian albedo U[0.2,0.8]), 1920x1080, 64 spp, depth 8, "
               "Russian roulette from depth 3")


PT_GLOSSY_WORKLOAD = ("path tracing: the same box, its 256 blobs cycling matte / plastic / mirror / plastic / glass "
                      "and plastic walls, lit by the ceiling light, two point lights and a spot light, 1920x1080, "
                      "64 spp, depth 8, Russian roulette from depth 3")


def run_pathtrace(vg, ctx, frames, flags, rprint, builder="ploc", scene_kind="box", cpu=False):
    """Msamples/s of the path-tracing workload (one frame = 1920x1080 x 64 spp);
    scene_kind "glossy": the materials-and-lights variant of the same box."""
    import torch
    from visionaray_gb300 import scenes
    if scene_kind == "glossy":
        tris, mats, area = scenes.glossy_box_scene(n_blobs=256, subdiv=22, seed=1)
        lights = scenes.mixed_lights(area)
    else:
        tris, mats, lights = scenes.box_scene()
    make = vg.ploc_builder if builder == "ploc" else vg.lbvh_builder
    bvh = make(ctx).build(vg.as_device_bytes(tris, ctx.device))
    scene = vg.PTScene(bvh, mats, lights)
    cam = scenes.box_camera()
    dev = f"cuda:{ctx.device}"
    accum = torch.zeros((PT_HEIGHT, PT_WIDTH, 4), dtype=torch.float32, device=dev)
    params = scenes.pt_params(PT_WIDTH, PT_HEIGHT, PT_SPP, num_bounces=PT_BOUNCES, flags=flags)
    vg.pathtrace_frame(scene, cam, params, accum=accum)   # warm-up frame
    ctx.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    launches0 = ctx.launches
    ev[0].record(ctx.stream)
    for f in range(frames):
        p = scenes.pt_params(PT_WIDTH, PT_HEIGHT, PT_SPP, num_bounces=PT_BOUNCES, frame_id=f + 1,
                             sfactor=1.0 / (f + 2), dfactor=1.0 - 1.0 / (f + 2), flags=flags)
        vg.pathtrace_frame(scene, cam, p, accum=accum)
    ev[1].record(ctx.stream)
    torch.cuda.synchronize()
    ctx.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / frames
    samples = PT_WIDTH * PT_HEIGHT * PT_SPP
    mean = accum[..., :3].mean().item()
    res = {"workload": PT_GLOSSY_WORKLOAD if scene_kind == "glossy" else PT_WORKLOAD, "flags": flags,
           "builder": builder, "frames": frames, "ms_per_frame": round(ms, 2),
           "msamples_s": round(samples / (ms * 1e-3) / 1e6, 2), "image_mean": round(mean, 5),
           "gpu_launches_per_frame": (ctx.launches - launches0) // frames}
    if scene_kind == "box" and flags == 0:
        peak, kind = measured_hbm_peak()
        res["roofline"] = roofline_of(samples, ms * 1e-3, B_SAMPLE_BOX, peak, f"{kind} hbm_gbs",
                                      "frame: every kernel of the wavefront frame (extend, shade, shadow)")
    if scene_kind == "box" and flags == 0:
        res["instanced"] = run_pathtrace_instanced(vg, ctx, frames, builder)
    if cpu:
        res["cpu_baseline"] = pt_cpu_baseline(tris, mats, lights, cam,
                                              scenes.pt_params(PT_WIDTH, PT_HEIGHT, PT_SPP, num_bounces=PT_BOUNCES,
                                                               frame_id=1, flags=flags), 61)
    return res


def run_pathtrace_instanced(vg, ctx, frames, builder):
    """The box frame with its 256 blobs as instances of one 9,680-triangle blob
    (gbrt_pt_scene_create_instanced: a two-level tree, the room and the blob trees),
    against the same geometry flattened into one tree: Msamples/s and tree bytes."""
    import torch
    from visionaray_gb300 import scenes
    d = scenes.instanced_box_scene(n_blobs=256, subdiv=22, seed=1)
    make = vg.ploc_builder if builder == "ploc" else vg.lbvh_builder
    room = make(ctx).build(vg.as_device_bytes(d["room"], ctx.device))
    blob = make(ctx).build(vg.as_device_bytes(d["blob"], ctx.device))
    ident = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0]
    tlas = vg.TLAS([(room, ident)] + [(blob, xf) for xf in d["transforms"]], ctx)
    scene_i = vg.PTScene.over_instances(tlas, d["materials"], d["lights"], d["inst_geom"])
    flat = make(ctx).build(vg.as_device_bytes(d["flat"], ctx.device))
    scene_f = vg.PTScene(flat, d["materials"], d["lights"])
    cam = scenes.box_camera()
    dev = f"cuda:{ctx.device}"
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    out = {"workload": f"{PT_WIDTH}x{PT_HEIGHT}, {PT_SPP} spp, depth {PT_BOUNCES}: the box room + 256 instances of one "
                       f"{len(d['blob'])}-triangle blob (radii U[0.03, 0.08]), per-instance-triangle albedo",
           "builder": builder}

    def tree_bytes(n):   # node pairs + leaf triangles
        return max(n - 1, 0) * 64 + n * 48

    for name, sc in (("instanced", scene_i), ("flattened", scene_f)):
        accum = torch.zeros((PT_HEIGHT, PT_WIDTH, 4), dtype=torch.float32, device=dev)
        vg.pathtrace_frame(sc, cam, scenes.pt_params(PT_WIDTH, PT_HEIGHT, PT_SPP, num_bounces=PT_BOUNCES), accum=accum)
        ctx.synchronize()
        ev[0].record(ctx.stream)
        for f in range(frames):
            vg.pathtrace_frame(sc, cam, scenes.pt_params(PT_WIDTH, PT_HEIGHT, PT_SPP, num_bounces=PT_BOUNCES,
                                                         frame_id=f + 1), accum=accum)
        ev[1].record(ctx.stream)
        torch.cuda.synchronize()
        ctx.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / frames
        out[name] = {"ms_per_frame": round(ms, 2),
                     "msamples_s": round(PT_WIDTH * PT_HEIGHT * PT_SPP / (ms * 1e-3) / 1e6, 2),
                     "image_mean": round(float(accum[..., :3].mean().item()), 5)}
    out["instanced"]["tree_bytes"] = tree_bytes(len(d["room"])) + tree_bytes(len(d["blob"])) + 64 * 256
    out["flattened"]["tree_bytes"] = tree_bytes(len(d["flat"]))
    for x in (scene_i, scene_f):
        x.close()
    tlas.close()
    return out


BATCH_WORKLOAD = ("512 random-soup scenes (triangle counts log-uniform in [1k, 1M], vertex offsets 0.5/cbrt(n)), "
                  "seeded cameras, square resolutions from {64,128,256,512}, 1 spp of 1 primary ray + 2 diffuse "
                  "bounces, matte 0.7 under white ambient light; one step = build every scene + render one frame "
                  "of every scene")


def run_batch(vg, ctx, steps, plain_steps, rprint, num_scenes=512, max_tris=1_000_000, cpu=False):
    """The batched graph (build + frame of 512 scenes in one CUDA graph, autotuned
    persistent launch) against two plain per-scene loops on the same GPU -- one that
    creates a tree and a scene per scene and step (gbrt_bvh_build_lbvh +
    gbrt_pt_scene_create + gbrt_pathtrace_frame), one that rebuilds trees made once
    into their own arrays (gbrt_bvh_rebuild_lbvh + gbrt_pathtrace_frame) -- Msamples/s
    of each and whether their images are bit-identical."""
    import torch
    from visionaray_gb300 import replicas, scenes
    from visionaray_gb300.types import AREA_LIGHT
    t0 = time.time()
    tris, offsets, cams, params, mats = scenes.batch_workload(num_scenes=num_scenes, n_max=max_tris)
    gen_s = time.time() - t0
    world, rank, _ = replicas.world_from_env()
    if world > 1:
        # whole scenes per rank, balanced by cost; every rank computes the same partition
        mine = replicas.partition(replicas.scene_costs(offsets, params), world)[rank]
        tris = np.concatenate([tris[int(offsets[s]):int(offsets[s + 1])] for s in mine])
        sizes = [int(offsets[s + 1] - offsets[s]) for s in mine]
        offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
        cams, params = cams[mine], params[mine]
    ns = len(offsets) - 1
    d_tris = vg.as_device_bytes(tris, ctx.device)
    tris_host = tris if cpu else None
    del tris
    batch = vg.Batch(offsets, ctx)
    batch.set_frames(cams, params, mats)
    batch.build(d_tris)
    images = batch.new_images()
    t0 = time.time()
    best, tune_ms = batch.autotune(images, reps=1)
    tune_s = time.time() - t0
    height = batch.height()
    # the whole job's samples (every rank renders its own scenes)
    samples = int(replicas.reduce_over_ranks(int(batch.pixel_offsets[-1]) * int(params["spp"][0]), "sum",
                                             f"cuda:{ctx.device}"))
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    for _ in range(3):
        batch.run_graph(d_tris, images)
    ctx.synchronize()
    launches0 = ctx.launches
    ev[0].record(ctx.stream)
    for _ in range(steps):
        batch.run_graph(d_tris, images)
    ev[1].record(ctx.stream)
    torch.cuda.synchronize()
    ctx.synchronize()
    batch_ms = replicas.reduce_over_ranks(ev[0].elapsed_time(ev[1]) / steps, "max", f"cuda:{ctx.device}")
    batch_launches = (ctx.launches - launches0) // steps
    # the frame alone (persistent kernel), for the breakdown
    ev[0].record(ctx.stream)
    batch.pathtrace(images)
    ev[1].record(ctx.stream)
    torch.cuda.synchronize()
    frame_ms = ev[0].elapsed_time(ev[1])

    # every BVH width x ray order at the tuner's block, tile, stack and pixel order: one
    # graph step each (build, the collapse and the pixel sort where the shape has them,
    # the frame), after a replay that captures it
    tuned = tuple(int(best[k]) for k in best.dtype.names)
    width_sort_ms = {}
    for w, srt in ((2, 0), (2, 1), (4, 0), (4, 1), (8, 0), (8, 1)):
        batch.launch = tuned[:4] + (w, srt)
        batch.run_graph(d_tris, images)
        ctx.synchronize()
        ev[0].record(ctx.stream)
        batch.run_graph(d_tris, images)
        ev[1].record(ctx.stream)
        torch.cuda.synchronize()
        ctx.synchronize()
        width_sort_ms[f"width{w}_sort{srt}"] = round(ev[0].elapsed_time(ev[1]), 2)
    batch.launch = tuned
    batch.run_graph(d_tris, images)
    ctx.synchronize()

    plain_images = torch.full_like(images, -1.0)
    no_lights = np.zeros(0, AREA_LIGHT)
    views = []
    for s in range(ns):
        a, b = int(batch.pixel_offsets[s]), int(batch.pixel_offsets[s + 1])
        views.append(plain_images[a:b].view(int(params["height"][s]), int(params["width"][s]), 4))

    def plain_step():
        builder = vg.lbvh_builder(ctx)
        for s in range(ns):
            bvh = builder.build(d_tris[int(offsets[s]) * 44:int(offsets[s + 1]) * 44])
            sc = vg.PTScene(bvh, mats, no_lights)
            vg.pathtrace_frame(sc, cams[s], params[s], accum=views[s])
            sc.close()
            bvh.close()

    kept = []   # (tree, scene) per scene, made once for the preallocated loop

    def preallocated_step():
        for s in range(ns):
            bvh, sc = kept[s]
            bvh.rebuild(d_tris[int(offsets[s]) * 44:int(offsets[s + 1]) * 44])
            vg.pathtrace_frame(sc, cams[s], params[s], accum=views[s])

    def time_plain(step_fn):
        plain_images.fill_(-1.0)
        step_fn()   # warm-up (grows the context scratch to the largest scene)
        ctx.synchronize()
        launches0 = ctx.launches
        torch.cuda.synchronize()
        ev[0].record(ctx.stream)
        for _ in range(plain_steps):
            step_fn()
        ev[1].record(ctx.stream)
        torch.cuda.synchronize()
        ctx.synchronize()
        plain_ms = replicas.reduce_over_ranks(ev[0].elapsed_time(ev[1]) / plain_steps, "max", f"cuda:{ctx.device}")
        plain_launches = (ctx.launches - launches0) // plain_steps
        differ = 0.0 if torch.equal(images.view(torch.int32), plain_images.view(torch.int32)) else 1.0
        identical = replicas.reduce_over_ranks(differ, "sum", f"cuda:{ctx.device}") == 0.0
        return ({"ms_per_step": round(plain_ms, 2), "msamples_s": round(samples / (plain_ms * 1e-3) / 1e6, 2),
                 "gpu_launches_per_step": int(plain_launches), "steps": plain_steps,
                 "images_bit_identical": identical, "speedup_of_batched": round(plain_ms / batch_ms, 2)},
                round(plain_ms / batch_ms, 2), identical)

    if plain_steps <= 0:
        res_plain, speedup, identical, res_pre = None, None, None, None
    else:
        res_plain, speedup, identical = time_plain(plain_step)
        builder = vg.lbvh_builder(ctx)
        for s in range(ns):
            bvh = builder.build(d_tris[int(offsets[s]) * 44:int(offsets[s + 1]) * 44])
            kept.append((bvh, vg.PTScene(bvh, mats, no_lights)))
        res_pre, _, identical_pre = time_plain(preallocated_step)
        identical = identical and identical_pre
        for bvh, sc in kept:
            sc.close()
            bvh.close()
        kept.clear()
    mean = float(images[:, :3].mean().item())
    workload = BATCH_WORKLOAD if (num_scenes, max_tris) == (512, 1_000_000) else (
        f"REDUCED profiling case: {num_scenes} scenes, triangle counts log-uniform in [1k, {max_tris}]")
    res = {"workload": workload, "scenes": int(replicas.reduce_over_ranks(ns, "sum", f"cuda:{ctx.device}")),
           "parallelism": f"scenes partitioned over {world} GPU(s)" if world > 1 else "one GPU",
           "triangles": int(replicas.reduce_over_ranks(int(offsets[-1]), "sum", f"cuda:{ctx.device}")),
           "samples_per_step": samples, "generate_s": round(gen_s, 1), "tallest_tree": height,
           "batched": {"ms_per_step": round(batch_ms, 2), "msamples_s": round(samples / (batch_ms * 1e-3) / 1e6, 2),
                       "frame_kernel_ms": round(frame_ms, 2), "gpu_launches_per_step": int(batch_launches),
                       "steps": steps, "launch": {k: int(best[k]) for k in best.dtype.names},
                       "autotune_frame_ms": round(float(tune_ms), 2), "autotune_s": round(tune_s, 1),
                       "graph_step_ms_by_width_and_sort": width_sort_ms},
           "plain": res_plain, "plain_preallocated": res_pre, "speedup": speedup,
           "images_bit_identical": identical, "image_mean": round(mean, 5)}
    peak, kind = measured_hbm_peak()
    res["roofline"] = roofline_of(samples, frame_ms * 1e-3, B_SAMPLE_BATCH, peak, f"{kind} hbm_gbs",
                                  "the persistent frame kernel (batch_pt) alone")
    if cpu and world == 1 and (num_scenes, max_tris) == (512, 1_000_000):
        res["cpu_baseline"] = batch_cpu_baseline(tris_host, offsets, cams, params, mats)
    batch.close()
    del d_tris, images, plain_images, views
    torch.cuda.empty_cache()
    return res


def batch_cpu_baseline(tris, offsets, cams, params, mats, scene_step=32):
    """The plain per-scene loop on the CPU with visionaray's CPU path (the oracle's
    restatement: binned-SAH build + pathtracing::kernel in FP32, all host threads) on
    every scene_step-th scene: Msamples/s over build + render time."""
    from oracle import Oracle

    from visionaray_gb300.types import AREA_LIGHT
    o = Oracle()
    build_s = render_s = 0.0
    samples = 0
    chosen = range(0, len(offsets) - 1, scene_step)
    for s in chosen:
        t = tris[int(offsets[s]):int(offsets[s + 1])]
        t0 = time.perf_counter()
        tree = o.build_sah(t)
        t1 = time.perf_counter()
        o.pathtrace(tree, t, mats, np.zeros(0, AREA_LIGHT), cams[s], params[s], mode=Oracle.PT_FLOAT)
        t2 = time.perf_counter()
        build_s += t1 - t0
        render_s += t2 - t1
        samples += int(params["width"][s]) * int(params["height"][s]) * int(params["spp"][s])
    return {"value": round(samples / (build_s + render_s) / 1e6, 3), "unit": "Msamples/s",
            "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"every {scene_step}th scene ({len(chosen)} scenes, {samples} samples): binned-SAH build "
                      f"{build_s:.2f} s + render {render_s:.2f} s"}


def run_adjoint(ctx, steps, rprint, flags=0, builder="ploc", cpu=False):
    """The inverse-albedo workload: `steps` Adam steps of forward frame + L2 loss +
    path-replay adjoint; median forward / backward times and their ratio, the albedo
    errors at the start and the end on the same sets of slots, and the bias of the
    gradient estimator (same-seed against decorrelated replay)."""
    from visionaray_gb300 import inverse
    r = inverse.optimize(steps=steps, ctx=ctx, extra_flags=flags, builder=builder)
    rnd = lambda d: {k: (round(v, 4) if v is not None else None) for k, v in d.items()}  # noqa: E731
    res = {"workload": "inverse albedo on the box scene reduced to 4,094 triangles (204 blobs of 20 triangles): "
                        "512x512, 16 spp, depth 6 forward + L2 loss + adjoint per step, target 256 spp",
            "steps": steps, "flags": int(inverse.FLAGS | flags), "builder": builder, "fwd_ms": round(r["fwd_ms"], 3),
            "bwd_ms": round(r["bwd_ms"], 3), "bwd_over_fwd": round(r["bwd_ms"] / r["fwd_ms"], 3),
            "loss_start": round(r["losses"][0], 6), "loss_end": round(r["losses"][-1], 6),
            "estimator": r["estimator"], "slots_seen": r["slots_seen"], "slots_ge_64px": r["slots_ge_64px"],
            "albedo_error_start": rnd(r["errors_start"]), "albedo_error_end": rnd(r["errors_end"]),
            "gradient_bias": inverse.gradient_bias(ctx=ctx, builder=builder)}
    # the 4,094-triangle scene (~200 KB of tree and triangles) is L2-resident: its
    # traversal bytes are served by L2, so the roofline is L2's (measured copy peak)
    l2 = measured_l2_gbs(f"cuda:{ctx.device}")
    samples = 512 * 512 * 16
    res["roofline"] = {
        "forward": roofline_of(samples, r["fwd_ms"] * 1e-3, B_SAMPLE_INVERSE, l2, "L2 measured in this run (best of copy, in-place add, sum)",
                               "forward frame (gbrt_pathtrace_forward)", bound="l2"),
        "backward": roofline_of(samples, r["bwd_ms"] * 1e-3, B_SAMPLE_INVERSE, l2, "L2 measured in this run (best of copy, in-place add, sum)",
                                "path-replay kernel (replays the forward's segments)", bound="l2")}
    if cpu:
        from visionaray_gb300 import scenes
        tris, mats, lights = scenes.box_scene(n_blobs=204, subdiv=1, seed=1)
        p = scenes.pt_params(512, 512, 16, num_bounces=6, frame_id=0, flags=inverse.FLAGS | flags)
        res["cpu_baseline"] = pt_cpu_baseline(tris, mats, lights, scenes.box_camera(), p, 7)
        res["cpu_baseline"]["note"] = "forward frame only: the reference has no adjoint"
    return res


def run_ours(args):
    import torch
    import torch.distributed as dist

    import visionaray_gb300 as vg
    from visionaray_gb300.types import HIT

    from visionaray_gb300 import replicas
    world, rank, local = replicas.init("nccl")
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"

    def rprint(*a, **k):
        if rank == 0:
            print(*a, **k)

    tris, closest, ao = workload(rprint, grid=args.grid, origins=args.origins)
    n_c, n_a = len(closest), len(ao)
    rays_per_step = n_c + n_a

    ctx = vg.Context(local)
    ctx.set_trace_flags(args.trace_flags)
    ctx.set_trace_refill(args.trace_refill)
    stream = ctx.stream

    # LBVH build, timed separately (build is not part of the traversal metric)
    d_tris = vg.as_device_bytes(tris, local)
    torch.cuda.synchronize()
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    builder = vg.ploc_builder(ctx) if args.builder == "ploc" else vg.lbvh_builder(ctx)
    bvh = builder.build(d_tris)   # warm (allocates the context scratch)
    del bvh
    b0.record(stream)
    bvh = builder.build(d_tris)
    b1.record(stream)
    torch.cuda.synchronize()
    build_ms = b0.elapsed_time(b1)

    d_closest = vg.device_rays(closest, local)
    d_ao = vg.device_rays(ao, local)
    h_closest = torch.empty((n_c, 4), dtype=torch.float32, device=dev)
    h_ao = torch.empty((n_a, 4), dtype=torch.float32, device=dev)

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        vg.closest_hit(d_closest, bvh, out=h_closest)
        if ev:
            ev[1].record(stream)
        vg.any_hit(d_ao, bvh, out=h_ao)
        if ev:
            ev[2].record(stream)

    # The headline step is closest_hit over the 4,194,304 secondary rays (the metric is
    # closest-hit Mrays/s); the AO any-hit rays and the build-inclusive step (LBVH build
    # + closest + any hit) are timed beside it.  The clock sampler runs from before the
    # warm-up (nvidia-smi takes a moment to start); only its samples inside the timed
    # region count.  Kernel timing records CUDA events around each query's traversal
    # kernel on the context stream (after the query's ray ordering).
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        # warm-up: at least W steps and at least 1.5 s of them (a GPU fresh out of idle
        # runs its first second slower while its clocks and power state settle)
        t_warm = time.perf_counter()
        done = 0
        while done < args.warmup or time.perf_counter() - t_warm < 1.5:
            vg.closest_hit(d_closest, bvh, out=h_closest)
            vg.any_hit(d_ao, bvh, out=h_ao)
            done += 1
            if done % 8 == 0:
                ctx.synchronize()
        ctx.synchronize()
        launches0 = ctx.launches
        ctx.set_kernel_timing(True)
        replicas.barrier()
        torch.cuda.synchronize()
        clocks.mark_start()
        start.record(stream)
        for _ in range(args.steps):
            vg.closest_hit(d_closest, bvh, out=h_closest)
        stop.record(stream)
        torch.cuda.synchronize()
        clocks.mark_end()
    replicas.barrier()
    gpu_launches = ctx.launches - launches0
    closest_kernel_ms = ctx.kernel_times()
    ctx.synchronize()   # raises on a flagged stack overflow / bad index
    total_ms = replicas.reduce_over_ranks(start.elapsed_time(stop), "max", dev)   # the slowest rank
    ms_per_step = total_ms / args.steps
    value = world * n_c * args.steps / (total_ms * 1e-3) / 1e6

    # the AO any-hit rays, timed the same way
    ctx.set_kernel_timing(True)
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(args.steps):
        vg.any_hit(d_ao, bvh, out=h_ao)
    stop.record(stream)
    torch.cuda.synchronize()
    any_ms = start.elapsed_time(stop) / args.steps
    any_kernel_ms = ctx.kernel_times()
    ctx.set_kernel_timing(False)

    # the whole configuration per step: LBVH build (a new tree each step, through the
    # public build call) + closest hit + any hit
    bi_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(bi_steps):
        step_bvh = builder.build(d_tris)
        vg.closest_hit(d_closest, step_bvh, out=h_closest)
        vg.any_hit(d_ao, step_bvh, out=h_ao)
        del step_bvh
    stop.record(stream)
    torch.cuda.synchronize()
    ctx.synchronize()
    bi_ms = start.elapsed_time(stop) / bi_steps

    # end to end through the host-buffer C ABI: pinned host rays in, hits out, per step
    # (host wall time, median of up to 10 steps: host-side jitter in the pinned copies
    # makes single steps vary by ~10 %)
    pin_c = torch.from_numpy(closest.view(np.float32).reshape(-1, 8)).pin_memory()
    pin_a = torch.from_numpy(ao.view(np.float32).reshape(-1, 8)).pin_memory()
    out_c = torch.empty((n_c, 4), dtype=torch.float32).pin_memory()
    out_a = torch.empty((n_a, 4), dtype=torch.float32).pin_memory()
    np_c, np_a = pin_c.numpy().view(closest.dtype).reshape(-1), pin_a.numpy().view(ao.dtype).reshape(-1)
    np_oc, np_oa = out_c.numpy().view(HIT).reshape(-1), out_a.numpy().view(HIT).reshape(-1)
    e2e_steps = max(3, min(args.steps, 10))
    vg.closest_hit(np_c, bvh, out=np_oc)
    vg.any_hit(np_a, bvh, out=np_oa)
    replicas.barrier()
    e2e_c, e2e_both = [], []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        vg.closest_hit(np_c, bvh, out=np_oc)
        t1 = time.perf_counter()
        vg.any_hit(np_a, bvh, out=np_oa)
        e2e_c.append(t1 - t0)
        e2e_both.append(time.perf_counter() - t0)
    e2e_s = replicas.reduce_over_ranks(statistics.median(e2e_c), "max", dev)
    e2e_value = world * n_c / e2e_s / 1e6
    e2e_both_s = replicas.reduce_over_ranks(statistics.median(e2e_both), "max", dev)
    # the host path must give the device path's answers
    same = bool((np_oc.view(np.uint8) == h_closest.cpu().numpy().view(np.uint8).reshape(-1)).all() and
                (np_oa.view(np.uint8) == h_ao.cpu().numpy().view(np.uint8).reshape(-1)).all())

    # roofline of the dominant kernel of the step (closest hit's traversal kernel), per
    # launch: the rays x B_ray over the kernel's own CUDA-event duration
    peak, peak_kind = measured_hbm_peak()
    per = {}
    for name, kms, qms, n, nn, nt in (("closest", closest_kernel_ms, ms_per_step, n_c, N_NODE_CLOSEST, N_TRI_CLOSEST),
                                      ("any", any_kernel_ms, any_ms, n_a, N_NODE_AO, N_TRI_AO)):
        ms = statistics.mean(kms) if kms else qms
        algo = n * b_ray(nn, nt)
        per[name] = {"kernel_ms_per_launch": round(ms, 4), "query_ms": round(qms, 4), "rays": n,
                     "mrays_s": round(n / (qms * 1e-3) / 1e6, 2), "kernel_mrays_s": round(n / (ms * 1e-3) / 1e6, 2),
                     "algorithmic_bytes": int(algo), "achieved_gbs": round(algo / (ms * 1e-3) / 1e9, 1),
                     "launches_timed": len(kms)}
    d = per["closest"]
    default_cfg = (args.grid, args.origins, args.trace_flags) == (GRID, ORIGINS, 1)
    roofline = {"bound": "hbm", "kernel": ("trace_rays_permuted<0, 0>" if args.trace_flags & 1 else "trace_rays<0, 0>"),
                "achieved": d["achieved_gbs"], "peak": peak, "unit": "GB/s",
                "frac": round(d["achieved_gbs"] / peak, 4),
                "traffic": TRAFFIC_CLOSEST if default_cfg else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, full-size capture",
                "peak_source": f"{peak_kind} hbm_gbs",
                "b_ray": round(b_ray(N_NODE_CLOSEST, N_TRI_CLOSEST), 1),
                "timing": "CUDA events around the traversal kernel on its stream, mean over the timed launches",
                "limiter": "latency of dependent node fetches under divergence (ncu: DRAM ~14 % of peak at full size)"}
    # the pure-I/O floor (48 B per ray: the ray in, the hit out) and the DRAM bandwidth
    # the launch actually drew (its ncu traffic over its event time)
    io_gbs = d["rays"] * 48 / (d["kernel_ms_per_launch"] * 1e-3) / 1e9
    roofline["io_floor"] = {"bytes_per_ray": 48, "achieved_gbs": round(io_gbs, 1), "frac": round(io_gbs / peak, 4)}
    if roofline["traffic"]:
        roofline["dram_gbs"] = round(roofline["traffic"] / (d["kernel_ms_per_launch"] * 1e-3) / 1e9, 1)
        # the L2 side of the same launch: its L1 <-> L2 bytes over its time, against the
        # L2 bandwidth measured in this run
        l2_peak = measured_l2_gbs(dev)
        l2_gbs = L2_TRAFFIC_CLOSEST / (d["kernel_ms_per_launch"] * 1e-3) / 1e9
        roofline["l2"] = {"traffic": L2_TRAFFIC_CLOSEST, "achieved_gbs": round(l2_gbs, 1), "peak": l2_peak,
                          "frac": round(l2_gbs / l2_peak, 4),
                          "traffic_source": "ncu lts__t_sectors_srcunit_tex_op_read.sum + _write.sum x 32 B "
                                            "per launch, full-size capture",
                          "peak_source": "L2 measured in this run (best of copy, in-place add, sum)"}

    # the same rays through the PLOC tree (a higher-quality GPU build; the workload's
    # builder is the LBVH, so this is reported beside the line's value, not as it)
    alt = None
    if args.builder == "lbvh" and not args.no_ploc:
        b0.record(stream)
        pbvh = vg.ploc_builder(ctx).build(d_tris)
        b1.record(stream)
        torch.cuda.synchronize()
        p_build = b0.elapsed_time(b1)
        saved, bvh = bvh, pbvh
        for _ in range(max(3, args.warmup)):
            vg.closest_hit(d_closest, bvh, out=h_closest)
            vg.any_hit(d_ao, bvh, out=h_ao)
        torch.cuda.synchronize()
        pts = []
        for fn in (lambda: vg.closest_hit(d_closest, bvh, out=h_closest), lambda: vg.any_hit(d_ao, bvh, out=h_ao)):
            start.record(stream)
            for _ in range(args.steps):
                fn()
            stop.record(stream)
            torch.cuda.synchronize()
            pts.append(start.elapsed_time(stop) / args.steps)
        ctx.synchronize()
        pc, pa = pts
        alt = {"builder": "ploc", "build_ms": round(p_build, 3),
               "closest_mrays_s": round(n_c / (pc * 1e-3) / 1e6, 2), "any_mrays_s": round(n_a / (pa * 1e-3) / 1e6, 2),
               "closest_plus_anyhit_mrays_s": round(rays_per_step / ((pc + pa) * 1e-3) / 1e6, 2),
               "note": "same rays and hits (ties aside) through a PLOC tree; not the workload's LBVH"}
        bvh = saved
        del pbvh

    cpu_legs = rank == 0 and world == 1 and not args.no_cpu_baseline
    # visionaray's own GPU kernels (oracle/_ref/vsnray_ref_gpu.cubin, device code built
    # from its headers) on the same GPU, tree and rays, and its path tracer on the box
    # frame at 16 spp: a baseline beside the line, outside its timed region
    reference_gpu = None
    if cpu_legs and not args.no_reference_gpu:
        from oracle import bench_reference_gpu, ref_gpu
        if ref_gpu.available():
            rg = ref_gpu.ReferenceGPU(local)
            reference_gpu = {"traversal": bench_reference_gpu.traversal(rg, ctx, d_tris, bvh, d_closest, d_ao, 3),
                             "lbvh_build": bench_reference_gpu.lbvh_build(rg, ctx, d_tris, 3)}
            if args.pt_frames > 0:
                reference_gpu["pathtrace"] = bench_reference_gpu.pathtrace(rg, ctx, 16, 1)
            del rg
        else:
            reference_gpu = {"unavailable": "the reference's GPU kernels were not built (visionaray's headers were "
                                            "absent where this tree was built)"}
    pt = None
    if args.pt_frames > 0:
        pt = run_pathtrace(vg, ctx, args.pt_frames, args.pt_flags, rprint, args.pt_builder, args.pt_scene,
                           cpu=cpu_legs)

    batched = None
    if args.batch_steps > 0:
        batched = run_batch(vg, ctx, args.batch_steps, args.batch_plain_steps, rprint, args.batch_scenes,
                            args.batch_max_tris, cpu=cpu_legs)

    adjoint = None
    if args.adjoint_steps > 0:
        adjoint = run_adjoint(ctx, args.adjoint_steps, rprint, args.pt_flags, args.pt_builder, cpu=cpu_legs)

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        res = cpu_baseline(tris, closest, ao, rank_print=rprint, sample_every=4, repeats=2)
        base = {"value": round(res["closest_rays"] / min(res["closest_times"]) / 1e6, 3), "unit": UNIT,
                "cores": res["cores"], "kind": res["kind"], "sample": res["sample"],
                "any_hit_mrays_s": round(res["any_rays"] / min(res["any_times"]) / 1e6, 3)}
        if res["kind"] == "port":
            base["port_vs_reference"] = PORT_VS_REFERENCE

    line = {"metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args.grid, args.origins, n_c, n_a, int(len(tris)), args.builder),
            "run": {"parallelism": f"replicas x{world}", "build_ms": round(build_ms, 3),
                    "trace_flags": args.trace_flags, "trace_refill": args.trace_refill, "warmup_steps_run": done},
            "kernels": per, "roofline": roofline,
            "e2e": {"value": round(e2e_value, 2), "unit": UNIT, "h2d_bytes_per_step": int(n_c * 32),
                    "d2h_bytes_per_step": int(n_c * 16), "matches_device_path": same,
                    "steps": e2e_steps, "statistic": "median host wall time per step"},
            "anyhit": {"rays": n_a, "ms_per_step": round(any_ms, 3),
                       "mrays_s": round(world * n_a / (any_ms * 1e-3) / 1e6, 2)},
            "closest_plus_anyhit": {
                "rays_per_step": rays_per_step, "ms_per_step": round(ms_per_step + any_ms, 3),
                "mrays_s": round(world * rays_per_step / ((ms_per_step + any_ms) * 1e-3) / 1e6, 2),
                "e2e_mrays_s": round(world * rays_per_step / e2e_both_s / 1e6, 2)},
            "build_inclusive": {"ms_per_step": round(bi_ms, 3), "steps": bi_steps,
                                "mrays_s": round(world * rays_per_step / (bi_ms * 1e-3) / 1e6, 2),
                                "step": "gbrt_bvh_build_lbvh (new tree) + closest hit + any hit"},
            "gpu_launches": int(gpu_launches), "clocks": clocks.summary(), "cpu_baseline": base,
            "ploc_tree": alt, "reference_gpu": reference_gpu, "pathtrace": pt, "batched_pathtrace": batched,
            "adjoint": adjoint}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--pt-frames", type=int, default=2, help="timed path-tracing frames (0: skip)")
    p.add_argument("--pt-scene", choices=("box", "glossy"), default="box",
                   help="path-tracing scene: the matte box of the workload, or its materials-and-lights variant")
    p.add_argument("--no-ploc", action="store_true", help="skip the traversal through the PLOC tree")
    p.add_argument("--no-reference-gpu", action="store_true",
                   help="skip the comparison with visionaray's own GPU kernels")
    p.add_argument("--builder", choices=["lbvh", "ploc"], default="lbvh",
                   help="tree of the traversal leg: the LBVH (the workload's builder) or the PLOC build")
    p.add_argument("--pt-builder", choices=["lbvh", "ploc"], default="ploc",
                   help="tree of the path-tracing and adjoint legs (their workloads name no builder)")
    p.add_argument("--pt-flags", type=int, default=0,
                   help="GBRT_PT_* scheduling bits of the path-tracing and adjoint legs (4: megakernel)")
    p.add_argument("--batch-steps", type=int, default=3, help="timed batched-graph steps (0: skip)")
    p.add_argument("--batch-plain-steps", type=int, default=1, help="timed plain per-scene loop steps")
    p.add_argument("--adjoint-steps", type=int, default=200, help="inverse-albedo Adam steps (0: skip)")
    p.add_argument("--batch-scenes", type=int, default=512, help="(profiling only) scenes of the batch leg")
    p.add_argument("--batch-max-tris", type=int, default=1_000_000, help="(profiling only) largest batch scene")
    p.add_argument("--trace-flags", type=int, default=1,
                   help="GBRT_TRACE_* bits of the ray queries (1: coherent ray order, 2: 4-wide nodes, "
                        "4: persistent traversal)")
    p.add_argument("--trace-refill", type=int, default=8,
                   help="persistent traversal (flag 4): idle lanes of a warp that trigger a refill")
    # smaller cases for profiling captures only; the benchmark is the default size
    p.add_argument("--grid", type=int, default=GRID)
    p.add_argument("--origins", type=int, default=ORIGINS)
    args = p.parse_args()
    if args.warmup < 3:
        print("# warmup raised to 3 (timing rule)", file=sys.stderr)
        args.warmup = 3
    if args.impl == "reference":
        from oracle import build as oracle_build
        oracle_build.build()
        return run_reference(args)
    from visionaray_gb300 import build
    build.build()
    if not args.no_cpu_baseline:
        from oracle import build as oracle_build
        oracle_build.build()   # the CPU-baseline leg's checker build
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
