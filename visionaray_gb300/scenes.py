"""Deterministic synthetic workloads (ctypes over libgbrt_scenes.so, see csrc/scenes.h).

The scenes stand in for the benchmark inputs: a random triangle soup (65,536
triangles for the soup case), a 2048x2048 sine heightfield (8,388,608 triangles),
pinhole primary rays and surface-sampled secondary / ambient-occlusion rays.  All
values are bit-identical on x86-64 and AArch64 hosts.
"""
import ctypes
import os

import numpy as np

from .types import RAY, TRIANGLE

_LIB = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libgbrt_scenes.so")
_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            raise RuntimeError(f"{_LIB} is missing: run visionaray_gb300.build.build() first")
        lib = ctypes.CDLL(_LIB)
        vp, u32, u64, f32, f64 = (ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64,
                                  ctypes.c_float, ctypes.c_double)
        lib.gbrt_scene_soup.argtypes = [u32, u64, f32, vp]
        lib.gbrt_scene_heightfield.argtypes = [u32, u64, f64, f64, ctypes.c_int, vp]
        lib.gbrt_rays_pinhole.argtypes = [vp, vp, vp, f32, u32, u32, vp]
        lib.gbrt_rays_surface.argtypes = [vp, u32, u32, u64, f32, u32, f32, vp, vp]
        lib.gbrt_scene_u01.argtypes = [u64, u64, u64]
        lib.gbrt_scene_u01.restype = f32
        _lib = lib
    return _lib


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def soup(n, seed=1, offset=0.02):
    """Random soup: centres U[0,1]^3, vertex offsets U[-offset, offset]^3."""
    out = np.empty(n, TRIANGLE)
    _load().gbrt_scene_soup(n, seed, offset, _ptr(out))
    return out


def heightfield(grid=2048, seed=1, base_amplitude=0.05, base_frequency=2.0, octaves=6):
    """2*grid^2 triangles over [0,1]^2, z = sum of `octaves` sines."""
    out = np.empty(2 * grid * grid, TRIANGLE)
    _load().gbrt_scene_heightfield(grid, seed, base_amplitude, base_frequency, octaves, _ptr(out))
    return out


def pinhole_rays(width, height, eye=(0.5, 0.5, -1.5), center=(0.5, 0.5, 0.0), up=(0.0, 1.0, 0.0),
                 fovy_degrees=45.0):
    out = np.empty(width * height, RAY)
    e, c, u = (np.asarray(v, np.float32) for v in (eye, center, up))
    _load().gbrt_rays_pinhole(_ptr(e), _ptr(c), _ptr(u), fovy_degrees, width, height, _ptr(out))
    return out


def surface_rays(tris, n_origins, seed=7, offset=1e-4, ao_per_origin=8, ao_tmax=0.05,
                 closest=True, ao=True):
    """(closest_rays, ao_rays) from uniformly sampled surface points."""
    tris = np.ascontiguousarray(tris)
    c = np.empty(n_origins, RAY) if closest else None
    a = np.empty(n_origins * ao_per_origin, RAY) if ao else None
    _load().gbrt_rays_surface(_ptr(tris), len(tris), n_origins, seed, offset, ao_per_origin,
                              ao_tmax, _ptr(c), _ptr(a))
    return c, a


def u01(seed, stream, index):
    return _load().gbrt_scene_u01(seed, stream, index)


def box_scene(n_blobs=256, subdiv=22, seed=1, light_y=0.999, emission=15.0):
    """The path-tracing scene: unit box (12 triangles), a 0.25 x 0.25 ceiling quad light
    (2 triangles, emission `emission`), `n_blobs` noisy icospheres of 20*subdiv^2
    triangles.  Returns (triangles, materials per geom_id, area lights)."""
    from .types import AREA_LIGHT, EMISSIVE, MATERIAL, MATTE
    lib = _load()
    if not hasattr(lib.gbrt_scene_box, "_typed"):
        lib.gbrt_scene_box_count.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        lib.gbrt_scene_box_count.restype = ctypes.c_uint64
        lib.gbrt_scene_box.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float,
                                       ctypes.c_void_p, ctypes.c_void_p]
        lib.gbrt_scene_box._typed = True
    n = lib.gbrt_scene_box_count(n_blobs, subdiv)
    tris = np.empty(n, TRIANGLE)
    albedo = np.empty((n, 3), np.float32)
    lib.gbrt_scene_box(n_blobs, subdiv, seed, light_y, _ptr(tris), _ptr(albedo))
    mats = np.zeros(n, MATERIAL)
    mats["kind"] = MATTE
    mats["color"] = albedo
    mats["scale"] = 1.0
    mats["kind"][12:14] = EMISSIVE
    mats["color"][12:14] = emission
    lights = np.zeros(2, AREA_LIGHT)
    lights["geometry"] = tris[12:14]
    lights["cl"] = emission
    lights["kl"] = 1.0
    return tris, mats, lights


def instanced_box_scene(n_blobs=256, subdiv=22, seed=1, light_y=0.999, emission=15.0, albedo_seed=9):
    """box_scene's room with its blobs as instances of ONE noisy icosphere (visionaray's
    index_bvh_inst_t use): the room (12 wall triangles + the 2-triangle ceiling light)
    is one tree, the unit blob (20*subdiv^2 triangles, centred at the origin, radius
    ~1) another; blob k is the unit blob scaled by a radius U[0.03, 0.08] and moved to a
    centre inside the box (seeded).  Material slots: the room's 14, then one per
    triangle of every blob instance (Lambertian albedo U[0.2, 0.8]).  Returns a dict:
    room, blob (triangles), transforms (n_blobs x 12: visionaray's mat4x3, columns),
    materials, lights, inst_geom (the first material slot of the room and of each
    blob), flat (the same scene flattened into one triangle array: each blob's
    triangles carried to world space in float32, geom_id = its material slot)."""
    room, mats, lights = box_scene(n_blobs=0, subdiv=subdiv, seed=seed, light_y=light_y, emission=emission)
    one, _, _ = box_scene(n_blobs=1, subdiv=subdiv, seed=seed, light_y=light_y, emission=emission)
    blob = one[14:].copy()
    v = np.concatenate([blob["v1"], blob["v1"] + blob["e1"], blob["v1"] + blob["e2"]]).astype(np.float64)
    c0 = v.mean(axis=0)
    r0 = float(np.sqrt(((v - c0) ** 2).sum(axis=1)).max())
    blob["v1"] = ((blob["v1"].astype(np.float64) - c0) / r0).astype(np.float32)
    blob["e1"] = (blob["e1"].astype(np.float64) / r0).astype(np.float32)
    blob["e2"] = (blob["e2"].astype(np.float64) / r0).astype(np.float32)
    nb = len(blob)
    blob["geom_id"] = np.arange(nb, dtype=np.uint32)
    blob["prim_id"] = np.arange(nb, dtype=np.uint32)
    transforms = np.zeros((n_blobs, 12), np.float32)
    radius = np.array([0.03 + 0.05 * u01(seed, 500, k) for k in range(n_blobs)], np.float32)
    centre = np.array([[(radius[k] * 1.2) + (1.0 - 2.4 * radius[k]) * u01(seed, 501 + a, k) for a in range(3)]
                       for k in range(n_blobs)], np.float32)
    transforms[:, 0] = transforms[:, 4] = transforms[:, 8] = radius
    transforms[:, 9:12] = centre
    from .types import MATERIAL, MATTE
    rng = np.random.default_rng(albedo_seed)
    blob_mats = np.zeros(n_blobs * nb, MATERIAL)
    blob_mats["kind"] = MATTE
    blob_mats["color"] = rng.uniform(0.2, 0.8, size=(n_blobs * nb, 3)).astype(np.float32)
    blob_mats["scale"] = 1.0
    materials = np.concatenate([mats, blob_mats])
    inst_geom = np.concatenate([[0], 14 + nb * np.arange(n_blobs)]).astype(np.uint32)
    flat = np.empty(14 + n_blobs * nb, TRIANGLE)
    flat[:14] = room
    for k in range(n_blobs):
        t = flat[14 + k * nb:14 + (k + 1) * nb]
        t["v1"] = blob["v1"] * radius[k] + centre[k]
        t["e1"] = blob["e1"] * radius[k]
        t["e2"] = blob["e2"] * radius[k]
        t["geom_id"] = 14 + k * nb + blob["geom_id"]
        t["prim_id"] = 14 + k * nb + blob["prim_id"]
    return {"room": room, "blob": blob, "transforms": transforms, "materials": materials, "lights": lights,
            "inst_geom": inst_geom, "flat": flat}


def specular_box_scene(n_blobs=256, subdiv=22, seed=1, light_y=0.999, emission=15.0, cycle=None):
    """box_scene whose blobs take their material kinds from `cycle` in turn (default
    matte, mirror, glass): a gold-like mirror (conductor Fresnel: ior (0.27, 0.42, 1.35),
    absorption (3.4, 2.3, 1.8)), clear glass (ior 1.5, transmission and reflection
    colors 1), a red plastic (cd (0.7, 0.2, 0.15), cs 0.4 white, exponent 32) or the blob's
    matte albedo: the specular and glossy materials on closed, noisy surfaces, so paths
    refract in and out and meet total internal reflection.  Returns (triangles,
    materials per geom_id, area lights)."""
    from .types import GLASS, MATTE, MIRROR, PLASTIC
    cycle = (MATTE, MIRROR, GLASS) if cycle is None else tuple(cycle)
    tris, mats, lights = box_scene(n_blobs, subdiv, seed, light_y, emission)
    per = 20 * subdiv * subdiv
    for b in range(n_blobs):
        sl = slice(14 + b * per, 14 + (b + 1) * per)
        kind = cycle[b % len(cycle)]
        if kind == PLASTIC:
            mats["kind"][sl] = PLASTIC
            mats["color"][sl] = (0.7, 0.2, 0.15)
            mats["scale"][sl] = 1.0
            mats["color2"][sl] = (0.4, 0.4, 0.4)
            mats["scale2"][sl] = 1.0
            mats["exponent"][sl] = 32.0
        elif kind == MIRROR:
            mats["kind"][sl] = MIRROR
            mats["color"][sl] = (0.95, 0.9, 0.8)
            mats["scale"][sl] = 1.0
            mats["ior"][sl] = (0.27, 0.42, 1.35)
            mats["absorption"][sl] = (3.4, 2.3, 1.8)
        elif kind == GLASS:
            mats["kind"][sl] = GLASS
            mats["color"][sl] = (1.0, 1.0, 1.0)
            mats["scale"][sl] = 1.0
            mats["color2"][sl] = (1.0, 1.0, 1.0)
            mats["scale2"][sl] = 1.0
            mats["ior"][sl] = (1.5, 1.5, 1.5)
    return tris, mats, lights


def glossy_box_scene(n_blobs=10, subdiv=8, seed=1, light_y=0.999, emission=15.0):
    """specular_box_scene with blobs cycling matte, plastic, mirror, plastic, glass and
    the box's walls (its first 12 triangles) a white plastic (cd 0.8, cs 0.25, exponent
    16): glossy next-event estimation and Blinn sampling over most of the image."""
    from .types import GLASS, MATTE, MIRROR, PLASTIC
    tris, mats, lights = specular_box_scene(n_blobs, subdiv, seed, light_y, emission,
                                            cycle=(MATTE, PLASTIC, MIRROR, PLASTIC, GLASS))
    walls = slice(0, 12)
    mats["kind"][walls] = PLASTIC
    mats["color"][walls] = (0.8, 0.8, 0.8)
    mats["scale"][walls] = 1.0
    mats["color2"][walls] = (0.25, 0.25, 0.25)
    mats["scale2"][walls] = 1.0
    mats["exponent"][walls] = 16.0
    return tris, mats, lights


def mixed_lights(area_lights):
    """The box's area lights plus two point lights and a spot light (LIGHT records):
    a warm point light at (0.3, 0.7, 0.5) with attenuation (1, 0.5, 0.25), a green one
    at (0.6, 0.3, 0.7) with (2, 0, 1), and a blue spot at (0.7, 0.6, 0.4) aimed down
    (cutoff 0.8 rad, exponent 4), which the reference's sampling leaves dark."""
    from .types import LIGHT, LIGHT_POINT, LIGHT_SPOT, lights_of_area_lights
    area = lights_of_area_lights(area_lights)
    out = np.zeros(len(area) + 3, LIGHT)
    out[:len(area)] = area
    pt, sp, pt2 = out[len(area)], out[len(area) + 1], out[len(area) + 2]
    pt["kind"], pt["cl"], pt["kl"], pt["position"], pt["attenuation"] = (
        LIGHT_POINT, (1.0, 0.8, 0.6), 0.4, (0.3, 0.7, 0.5), (1.0, 0.5, 0.25))
    sp["kind"], sp["cl"], sp["kl"], sp["position"], sp["attenuation"] = (
        LIGHT_SPOT, (0.5, 0.5, 1.0), 2.0, (0.7, 0.6, 0.4), (1.0, 0.0, 0.0))
    sp["spot_direction"], sp["spot_cutoff"], sp["spot_exponent"] = (0.0, -1.0, 0.0), 0.8, 4.0
    pt2["kind"], pt2["cl"], pt2["kl"], pt2["position"], pt2["attenuation"] = (
        LIGHT_POINT, (0.2, 1.0, 0.3), 1.0, (0.6, 0.3, 0.7), (2.0, 0.0, 1.0))
    return out


def box_camera(eye=(0.5, 0.5, 0.02), center=(0.5, 0.5, 1.0), up=(0.0, 1.0, 0.0), fovy_degrees=60.0):
    """Camera inside the closed box, near the front wall, looking at the back wall."""
    from .types import CAMERA
    c = np.zeros(1, CAMERA)
    c["eye"], c["center"], c["up"], c["fovy_degrees"] = eye, center, up, fovy_degrees
    return c[0]


def pt_params(width, height, spp, num_bounces=8, epsilon=1e-4, frame_id=0, sfactor=1.0, dfactor=0.0,
              background=(0.0, 0.0, 0.0, 1.0), ambient=(0.0, 0.0, 0.0), flags=0):
    from .types import PT_PARAMS
    p = np.zeros(1, PT_PARAMS)
    p["width"], p["height"], p["spp"], p["num_bounces"] = width, height, spp, num_bounces
    p["epsilon"], p["frame_id"], p["sfactor"], p["dfactor"] = epsilon, frame_id, sfactor, dfactor
    p["background"], p["ambient"], p["flags"] = background, ambient, flags
    return p[0]


BATCH_SIDES = (64, 128, 256, 512)


def batch_workload(num_scenes=512, seed=3, n_min=1000, n_max=1_000_000, spp=1, num_bounces=3, frame_id=0):
    """The batched workload: `num_scenes` random soups (the soup generator with the
    offset scale 0.5 / cbrt(n)) whose triangle counts are log-uniform in
    [n_min, n_max], each with a seeded camera on a sphere around the soup looking at its
    centre and a square resolution drawn from BATCH_SIDES; one matte material of
    albedo 0.7, white ambient light, `spp` samples of 1 primary ray + (num_bounces - 1)
    diffuse bounces.  Returns (triangles, offsets, cameras, params, materials)."""
    import math

    from .types import CAMERA, MATERIAL, MATTE, PT_PARAMS
    lib = _load()
    counts = np.empty(num_scenes, np.int64)
    lo, hi = math.log(n_min), math.log(n_max)
    for s in range(num_scenes):
        counts[s] = int(round(math.exp(lo + u01(seed, 1, s) * (hi - lo))))
    offsets = np.zeros(num_scenes + 1, np.uint32)
    offsets[1:] = np.cumsum(counts)
    tris = np.empty(int(offsets[-1]), TRIANGLE)
    cams = np.zeros(num_scenes, CAMERA)
    params = np.zeros(num_scenes, PT_PARAMS)
    for s in range(num_scenes):
        n = int(counts[s])
        view = tris[int(offsets[s]):int(offsets[s + 1])]
        lib.gbrt_scene_soup(n, seed * 1000003 + s, 0.5 / n ** (1.0 / 3.0), _ptr(view))
        z = 2.0 * u01(seed, 2, s) - 1.0
        phi = 2.0 * math.pi * u01(seed, 4, s)
        r = math.sqrt(max(0.0, 1.0 - z * z))
        d = (r * math.cos(phi), r * math.sin(phi), z)
        cams[s]["eye"] = (0.5 + 1.6 * d[0], 0.5 + 1.6 * d[1], 0.5 + 1.6 * d[2])
        cams[s]["center"] = (0.5, 0.5, 0.5)
        cams[s]["up"] = (0.0, 0.0, 1.0) if abs(d[1]) > 0.9 else (0.0, 1.0, 0.0)
        cams[s]["fovy_degrees"] = 50.0
        side = BATCH_SIDES[min(int(u01(seed, 3, s) * len(BATCH_SIDES)), len(BATCH_SIDES) - 1)]
        params[s] = pt_params(side, side, spp, num_bounces=num_bounces, frame_id=frame_id,
                              ambient=(1.0, 1.0, 1.0))
    mats = np.zeros(1, MATERIAL)
    mats["kind"], mats["color"], mats["scale"] = MATTE, 0.7, 1.0
    return tris, offsets, cams, params, mats


def load_ply(path):
    """Triangles of a Stanford PLY file (ascii or binary), as the reference viewer's
    loader reads them: the vertex element's x, y, z and the face element's
    vertex_indices, geom_id 0, faces of more than three vertices as fans.  Raises
    ValueError for an unreadable or malformed file."""
    lib = _load()
    if not hasattr(lib.gbrt_ply_load, "_typed"):
        lib.gbrt_ply_load.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint64]
        lib.gbrt_ply_load.restype = ctypes.c_int64
        lib.gbrt_ply_load._typed = True
    p = str(path).encode()
    n = lib.gbrt_ply_load(p, None, 0)
    if n < 0:
        raise ValueError(f"cannot read PLY file {path}")
    tris = np.empty(n, TRIANGLE)
    lib.gbrt_ply_load(p, _ptr(tris), n)
    return tris


def load_obj(path):
    """(triangles, materials) of a Wavefront OBJ file, as the reference viewer's loader
    reads its geometry (fans, negative indices, degenerate faces dropped, geom_id per
    usemtl slot); materials are matte (Kd) or emissive (Ke) per slot."""
    from .types import MATERIAL
    lib = _load()
    if not hasattr(lib.gbrt_obj_load, "_typed"):
        lib.gbrt_obj_load.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint64]
        lib.gbrt_obj_load.restype = ctypes.c_int64
        lib.gbrt_obj_materials.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint64]
        lib.gbrt_obj_materials.restype = ctypes.c_int64
        lib.gbrt_obj_load._typed = True
    p = str(path).encode()
    n = lib.gbrt_obj_load(p, None, 0)
    if n < 0:
        raise FileNotFoundError(path)
    tris = np.empty(n, TRIANGLE)
    lib.gbrt_obj_load(p, _ptr(tris), n)
    m = lib.gbrt_obj_materials(p, None, 0)
    mats = np.zeros(m, MATERIAL)
    lib.gbrt_obj_materials(p, _ptr(mats), m)
    return tris, mats
