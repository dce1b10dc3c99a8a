"""Generates the golden vectors in this directory from visionaray's OWN CPU code.

Run where the visionaray sources are present (they are compiled from their headers
into oracle/_ref/libvsnray_ref.so by oracle/Makefile):

    python -m visionaray_gb300.build && python tests/golden/make_golden.py

Every number here comes from the reference build (oracle.Reference), never from the
oracle restatement, so the tests that compare the restatement (and through it the
CUDA path) against these files pin parity to the reference itself.  Inputs are the
deterministic scenes of visionaray_gb300.scenes (bit-identical on x86-64 and
AArch64), so only digests and small samples are stored.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import Reference  # noqa: E402
from visionaray_gb300 import scenes  # noqa: E402

SAMPLE_STRIDE = 251   # every 251st ray's full hit record is stored


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def tree_record(handle):
    t = handle.tree()
    return {"num_nodes": int(len(t.nodes)), "num_indices": int(len(t.indices)),
            "depth": int(t.depth), "sha256": digest(t.nodes, t.indices),
            "sah_cost": float(handle.sah_cost())}


def trace_record(handle, rays, any_hit, name, samples):
    hits, cnt = handle.trace(rays, any_hit=any_hit, counters=True)
    samples[name] = hits[::SAMPLE_STRIDE]
    return {"sha256": digest(hits), "num_hits": int((hits["prim_id"] != 0xFFFFFFFF).sum()),
            "box_tests": int(cnt[0]), "tri_tests": int(cnt[1]), "num_rays": int(len(rays))}


def soup_case(ref, samples):
    tris = scenes.soup(65536, seed=1, offset=0.02)
    rays = scenes.pinhole_rays(1024, 1024)
    sah = ref.build_sah(tris)
    lbvh = ref.build_lbvh_cpu(tris)
    ids, codes = ref.lbvh_sorted_refs(tris)
    left, right = ref.karras_children(codes)
    rec = {
        "scene": {"kind": "soup", "n": 65536, "seed": 1, "offset": 0.02},
        "rays": {"kind": "pinhole", "width": 1024, "height": 1024, "eye": [0.5, 0.5, -1.5],
                 "center": [0.5, 0.5, 0.0], "up": [0.0, 1.0, 0.0], "fovy": 45.0},
        "triangles_sha256": digest(tris),
        "rays_sha256": digest(rays),
        "sah": tree_record(sah),
        "lbvh_cpu": tree_record(lbvh),
        "morton_sorted_sha256": digest(ids, codes),
        "karras_children_sha256": digest(left, right),
        "sah_closest": trace_record(sah, rays, False, "soup_sah_closest", samples),
        "sah_any": trace_record(sah, rays, True, "soup_sah_any", samples),
        "lbvh_cpu_closest": trace_record(lbvh, rays, False, "soup_lbvh_closest", samples),
    }
    samples["soup_morton_ids"] = ids[::SAMPLE_STRIDE]
    samples["soup_morton_codes"] = codes[::SAMPLE_STRIDE]
    return rec


def heightfield_case(ref, samples):
    tris = scenes.heightfield(grid=128, seed=1)
    closest, ao = scenes.surface_rays(tris, 16384, seed=7, offset=1e-4, ao_per_origin=8, ao_tmax=0.05)
    sah = ref.build_sah(tris)
    ids, codes = ref.lbvh_sorted_refs(tris)
    left, right = ref.karras_children(codes)
    return {
        "scene": {"kind": "heightfield", "grid": 128, "seed": 1, "base_amplitude": 0.05,
                  "base_frequency": 2.0, "octaves": 6},
        "rays": {"kind": "surface", "origins": 16384, "seed": 7, "offset": 1e-4, "ao_per_origin": 8,
                 "ao_tmax": 0.05},
        "triangles_sha256": digest(tris),
        "closest_rays_sha256": digest(closest),
        "ao_rays_sha256": digest(ao),
        "sah": tree_record(sah),
        "morton_sorted_sha256": digest(ids, codes),
        "karras_children_sha256": digest(left, right),
        "sah_closest": trace_record(sah, closest, False, "hf_sah_closest", samples),
        "sah_ao_any": trace_record(sah, ao, True, "hf_sah_ao_any", samples),
    }


def pathtrace_case(ref, samples):
    tris, mats, lights = scenes.box_scene(n_blobs=8, subdiv=8, seed=1)
    cam = scenes.box_camera()
    params = scenes.pt_params(64, 48, 4, num_bounces=8, epsilon=1e-4, frame_id=3)
    img = ref.pathtrace(tris, mats, lights, cam, params)
    samples["pt_image"] = img
    return {"scene": {"kind": "box", "n_blobs": 8, "subdiv": 8, "seed": 1},
            "camera": "scenes.box_camera()", "params": {"width": 64, "height": 48, "spp": 4, "num_bounces": 8,
                                                        "epsilon": 1e-4, "frame_id": 3, "flags": 0},
            "triangles_sha256": digest(tris), "materials_sha256": digest(mats),
            "image_sha256": digest(img), "mean_rgb": [float(v) for v in img.reshape(-1, 4).mean(0)[:3]]}


def material_pathtrace_case(ref, samples, kind, frame_id):
    """scenes.specular_box_scene (mirror, glass) or scenes.glossy_box_scene (plus
    plastic) at 64 x 48, 4 spp."""
    if kind == "specular_box":
        tris, mats, lights = scenes.specular_box_scene(n_blobs=8, subdiv=8, seed=1)
        scene = {"kind": kind, "n_blobs": 8, "subdiv": 8, "seed": 1}
    else:
        tris, mats, lights = scenes.glossy_box_scene(n_blobs=10, subdiv=8, seed=1)
        scene = {"kind": kind, "n_blobs": 10, "subdiv": 8, "seed": 1}
    cam = scenes.box_camera()
    params = scenes.pt_params(64, 48, 4, num_bounces=8, epsilon=1e-4, frame_id=frame_id)
    img = ref.pathtrace(tris, mats, lights, cam, params)
    samples["pt_%s_image" % kind.split("_")[0]] = img
    return {"scene": scene,
            "camera": "scenes.box_camera()", "params": {"width": 64, "height": 48, "spp": 4, "num_bounces": 8,
                                                        "epsilon": 1e-4, "frame_id": frame_id, "flags": 0},
            "triangles_sha256": digest(tris), "materials_sha256": digest(mats),
            "image_sha256": digest(img), "mean_rgb": [float(v) for v in img.reshape(-1, 4).mean(0)[:3]]}


def lights_pathtrace_case(ref, samples):
    """scenes.glossy_box_scene lit by scenes.mixed_lights (area, point and spot lights)."""
    tris, mats, area = scenes.glossy_box_scene(n_blobs=10, subdiv=8, seed=1)
    lights = scenes.mixed_lights(area)
    cam = scenes.box_camera()
    params = scenes.pt_params(64, 48, 4, num_bounces=8, epsilon=1e-4, frame_id=7)
    img = ref.pathtrace(tris, mats, lights, cam, params)
    samples["pt_lights_image"] = img
    return {"scene": {"kind": "glossy_box", "n_blobs": 10, "subdiv": 8, "seed": 1, "lights": "mixed_lights"},
            "camera": "scenes.box_camera()", "params": {"width": 64, "height": 48, "spp": 4, "num_bounces": 8,
                                                        "epsilon": 1e-4, "frame_id": 7, "flags": 0},
            "triangles_sha256": digest(tris), "materials_sha256": digest(mats), "lights_sha256": digest(lights),
            "image_sha256": digest(img), "mean_rgb": [float(v) for v in img.reshape(-1, 4).mean(0)[:3]]}


def environment_pathtrace_case(ref, samples):
    """The open blob scene (box walls removed) under an environment light: the seeded
    lat-long map of tests/materials.py, bilinear, Wrap, rotated."""
    from oracle import env_light
    from tests.materials import ENV_TRANSFORMS, env_texels, open_blob_scene
    from visionaray_gb300 import types
    tris, mats, lights, cam = open_blob_scene()
    tex = env_texels()
    env = env_light(tex, filter=types.FILTER_LINEAR, address=types.ADDRESS_WRAP, scale=(1.5, 1.0, 0.75),
                    light_to_world=ENV_TRANSFORMS["rotation"])
    params = scenes.pt_params(64, 48, 4, num_bounces=6, frame_id=8)
    img = ref.pathtrace(tris, mats, lights, cam, params, env=env)
    samples["pt_env_image"] = img
    return {"scene": "tests.materials.open_blob_scene()", "environment": {"texels": "env_texels()",
            "filter": "linear", "address": "wrap", "scale": [1.5, 1.0, 0.75], "light_to_world": "rotation"},
            "params": {"width": 64, "height": 48, "spp": 4, "num_bounces": 6, "frame_id": 8},
            "texels_sha256": digest(tex), "triangles_sha256": digest(tris), "image_sha256": digest(img),
            "mean_rgb": [float(v) for v in img.reshape(-1, 4).mean(0)[:3]]}


def main():
    if not Reference.available():
        raise SystemExit("oracle/_ref/libvsnray_ref.so is missing: build it where the visionaray "
                         "sources are present (make -C oracle ref)")
    ref = Reference()
    samples = {}
    out = {"generator": "visionaray CPU path compiled from its headers (oracle/ref_driver.cpp)",
           "sample_stride": SAMPLE_STRIDE,
           "soup": soup_case(ref, samples),
           "heightfield": heightfield_case(ref, samples),
           "pathtrace": pathtrace_case(ref, samples),
           "pathtrace_specular": material_pathtrace_case(ref, samples, "specular_box", 5),
           "pathtrace_glossy": material_pathtrace_case(ref, samples, "glossy_box", 6),
           "pathtrace_lights": lights_pathtrace_case(ref, samples),
           "pathtrace_environment": environment_pathtrace_case(ref, samples)}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "golden_samples.npz"), **samples)
    print("wrote golden.json and golden_samples.npz")


if __name__ == "__main__":
    main()
