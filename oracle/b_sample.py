"""Algorithmic bytes per path-traced sample (MEASUREMENT INFRASTRUCTURE; the values it
prints are frozen in bench.py).

B_sample = sum over the sample's path segments and shadow rays of B_ray, with
B_ray = 32 (ray in) + 16 (hit out) + N_node * 32 + N_tri * 48, where N_node / N_tri are
the box and triangle tests of visionaray's CPU traversal on its binned-SAH BVH2 (the
oracle's counters, equal to the reference's).  Counted on the oracle's FP32 run of each
workload at the CUDA path's random numbers, over a fixed subset of pixels:

    python -m oracle.b_sample [box|batch|inverse ...]

  box      1920x1080, 64 spp, depth 8 box scene (2,478,094 triangles), every 61st pixel
  batch    the 512-scene batch (1 spp, 3 segments, ambient light), every 8th scene,
           every pixel
  inverse  the 4,094-triangle inverse-rendering box at 512x512, 16 spp, depth 6 with the
           corrected shadow range and no roulette, every 7th pixel
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def b_sample(counters, samples):
    closest, shadow, boxes, tris = (int(c) for c in counters)
    total = (closest + shadow) * 48 + boxes * 32 + tris * 48
    return {"samples": int(samples), "closest_rays": closest, "shadow_rays": shadow, "box_tests": boxes,
            "tri_tests": tris, "bytes_per_sample": total / samples,
            "segments_per_sample": (closest + shadow) / samples}


def box(oracle):
    from visionaray_gb300 import scenes
    tris, mats, lights = scenes.box_scene()
    params = scenes.pt_params(1920, 1080, 64, num_bounces=8, frame_id=1)
    pix = np.arange(0, 1920 * 1080, 61, dtype=np.uint32)
    _, cnt = oracle.pathtrace_pixels(oracle.build_sah(tris), tris, mats, lights, scenes.box_camera(), params, pix,
                                     mode=oracle.PT_FLOAT_TRIG_DOUBLE)
    return b_sample(cnt, len(pix) * 64)


def batch(oracle):
    from visionaray_gb300 import scenes
    from visionaray_gb300.types import AREA_LIGHT
    tris, offsets, cams, params, mats = scenes.batch_workload()
    total = np.zeros(4, np.uint64)
    samples = 0
    for s in range(0, len(offsets) - 1, 8):
        t = tris[int(offsets[s]):int(offsets[s + 1])]
        npix = int(params["width"][s]) * int(params["height"][s])
        pix = np.arange(npix, dtype=np.uint32)
        _, cnt = oracle.pathtrace_pixels(oracle.build_sah(t), t, mats, np.zeros(0, AREA_LIGHT), cams[s], params[s],
                                         pix, mode=oracle.PT_FLOAT_TRIG_DOUBLE)
        total += cnt
        samples += npix * int(params["spp"][s])
    return b_sample(total, samples)


def inverse(oracle):
    from visionaray_gb300 import scenes
    from visionaray_gb300.types import PT_NO_RUSSIAN_ROULETTE, PT_SHADOW_RANGE_FIX
    tris, mats, lights = scenes.box_scene(n_blobs=204, subdiv=1, seed=1)
    params = scenes.pt_params(512, 512, 16, num_bounces=6, frame_id=0,
                              flags=PT_SHADOW_RANGE_FIX | PT_NO_RUSSIAN_ROULETTE)
    pix = np.arange(0, 512 * 512, 7, dtype=np.uint32)
    _, cnt = oracle.pathtrace_pixels(oracle.build_sah(tris), tris, mats, lights, scenes.box_camera(), params, pix,
                                     mode=oracle.PT_FLOAT_TRIG_DOUBLE)
    return b_sample(cnt, len(pix) * 16)


def main(names):
    from oracle import Oracle
    from oracle import build as oracle_build
    from visionaray_gb300 import build
    build.build()
    oracle_build.build()
    o = Oracle()
    for name in names:
        print(json.dumps({name: globals()[name](o)}), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or ["box", "batch", "inverse"])
