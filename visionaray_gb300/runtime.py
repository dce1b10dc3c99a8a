"""Python host side over the C ABI (include/visionaray_gb300/gbrt.h).

Mirrors the reference's interface for the hot path:
  visionaray                                      here
  lbvh_builder{}.build(cuda_index_bvh<P>{}, p, n)  lbvh_builder().build(tris)        -> IndexBVH
  (cuda_index_bvh from a host index_bvh)           IndexBVH.upload(nodes, indices, tris)
  closest_hit(ray, refs, refs + 1)                 closest_hit(rays, bvh)            -> hits
  any_hit(ray, refs, refs + 1)                     any_hit(rays, bvh)                -> hits
Rays/hits are batched (a C ABI cannot take per-ray device functors).  Device buffers
are torch CUDA tensors used as plain memory; host buffers are numpy arrays.  There is
no CPU fallback: without libgbrt.so or a GPU every call raises.
"""
import ctypes
import os

import numpy as np

from .types import (ADDRESS_CLAMP, AREA_LIGHT, BATCH_LAUNCH, BVH_NODE, CAMERA, FILTER_LINEAR, HIT, HIT_INST, INSTANCE,
                    LIGHT, MATERIAL, PT_PARAMS, RAY, TRIANGLE, environment)

LIBGBRT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libgbrt.so")

STATUS = {0: "GBRT_OK", 1: "GBRT_ERR_INVALID_ARG", 2: "GBRT_ERR_OUT_OF_MEMORY", 3: "GBRT_ERR_CUDA",
          4: "GBRT_ERR_WATCHDOG", 5: "GBRT_ERR_STACK_OVERFLOW", 6: "GBRT_ERR_TOO_LARGE"}

# Every function the C ABI exports, with its ctypes signature (restype, argtypes).
_vp, _u32, _u64, _i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
_pp = ctypes.POINTER(ctypes.c_void_p)
SIGNATURES = {
    "gbrt_abi_version": (_i32, []),
    "gbrt_context_create": (_i32, [_i32, _vp, _pp]),
    "gbrt_context_destroy": (_i32, [_vp]),
    "gbrt_context_set_stream": (_i32, [_vp, _vp]),
    "gbrt_context_synchronize": (_i32, [_vp]),
    "gbrt_last_error": (ctypes.c_char_p, [_vp]),
    "gbrt_kernel_launch_count": (_u64, [_vp]),
    "gbrt_context_set_kernel_timing": (_i32, [_vp, _i32]),
    "gbrt_bvh_rebuild_lbvh": (_i32, [_vp, _vp, _vp, _u32]),
    "gbrt_pt_scene_create_instanced": (_i32, [_vp, _vp, _vp, _u32, _vp, _u32, _vp, _pp]),
    "gbrt_context_kernel_times": (_i32, [_vp, _vp, _u32, _vp]),
    "gbrt_context_set_trace_flags": (_i32, [_vp, _u32]),
    "gbrt_context_set_trace_refill": (_i32, [_vp, _u32]),
    "gbrt_context_set_host_chunk": (_i32, [_vp, _u32]),
    "gbrt_bvh_build_lbvh": (_i32, [_vp, _vp, _u32, _pp]),
    "gbrt_bvh_build_lbvh_host": (_i32, [_vp, _vp, _u32, _pp]),
    "gbrt_bvh_build_ploc": (_i32, [_vp, _vp, _u32, _pp]),
    "gbrt_bvh_upload_bvh2_host": (_i32, [_vp, _vp, _u32, _vp, _u32, _vp, _u32, _pp]),
    "gbrt_bvh_destroy": (_i32, [_vp]),
    "gbrt_bvh_counts": (_i32, [_vp, _vp, _vp, _vp]),
    "gbrt_bvh_export_bvh2": (_i32, [_vp, _vp, _vp, _vp]),
    "gbrt_bvh_refit": (_i32, [_vp, _vp, _vp, _u32]),
    "gbrt_bvh_morton_codes": (_i32, [_vp, _vp, _vp]),
    "gbrt_bvh_build_lbvh_noalloc": (_i32, [_vp, _vp, _u32, _vp, _vp]),
    "gbrt_trace_closest_hit": (_i32, [_vp, _vp, _vp, _u32, _vp]),
    "gbrt_trace_any_hit": (_i32, [_vp, _vp, _vp, _u32, _vp]),
    "gbrt_trace_closest_hit_host": (_i32, [_vp, _vp, _vp, _u32, _vp]),
    "gbrt_trace_any_hit_host": (_i32, [_vp, _vp, _vp, _u32, _vp]),
    "gbrt_pt_scene_create": (_i32, [_vp, _vp, _vp, _u32, _vp, _u32, _pp]),
    "gbrt_pt_scene_create_lights": (_i32, [_vp, _vp, _vp, _u32, _vp, _u32, _pp]),
    "gbrt_pt_scene_destroy": (_i32, [_vp]),
    "gbrt_pt_scene_set_environment": (_i32, [_vp, _vp, _vp]),
    "gbrt_pinhole_camera_basis": (_i32, [_vp, _u32, _u32, _vp]),
    "gbrt_pathtrace_frame": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "gbrt_pathtrace_forward": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbrt_pathtrace_backward": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbrt_tlas_build": (_i32, [_vp, _vp, _u32, _pp]),
    "gbrt_tlas_destroy": (_i32, [_vp]),
    "gbrt_tlas_trace_closest_hit": (_i32, [_vp, _vp, _vp, _u32, _vp]),
    "gbrt_tlas_trace_any_hit": (_i32, [_vp, _vp, _vp, _u32, _vp]),
    "gbrt_batch_create": (_i32, [_vp, _vp, _u32, _pp]),
    "gbrt_batch_destroy": (_i32, [_vp]),
    "gbrt_batch_build": (_i32, [_vp, _vp, _vp]),
    "gbrt_batch_export_bvh2": (_i32, [_vp, _vp, _u32, _vp, _vp]),
    "gbrt_batch_trace_closest_hit": (_i32, [_vp, _vp, _vp, _vp, _vp]),
    "gbrt_batch_set_frames": (_i32, [_vp, _vp, _vp, _vp, _vp, _u32]),
    "gbrt_batch_set_launch": (_i32, [_vp, _vp]),
    "gbrt_batch_set_lights": (_i32, [_vp, _vp, _vp, _u32, _vp]),
    "gbrt_batch_get_launch": (_i32, [_vp, _vp]),
    "gbrt_batch_height": (_i32, [_vp, _vp, _vp]),
    "gbrt_batch_pathtrace": (_i32, [_vp, _vp, _vp]),
    "gbrt_batch_run_graph": (_i32, [_vp, _vp, _vp, _vp]),
    "gbrt_batch_autotune": (_i32, [_vp, _vp, _vp, _u32, _vp, _vp]),
}

_lib = None


class GbrtError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


def load_library(path=LIBGBRT):
    """Loads libgbrt.so (no GPU needed to load).  Raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run visionaray_gb300.build.build() "
                               "(the CUDA path has no fallback)")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        _lib = lib
    return _lib


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("visionaray_gb300 needs a CUDA GPU (there is no CPU path)")
    return torch


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _hptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class Context:
    """A gbrt_context bound to one device and (by default) torch's current stream."""

    def __init__(self, device=0, stream=None):
        torch = _torch()
        self.lib = load_library()
        self.device = device
        if stream is None:
            stream = torch.cuda.current_stream(device)
        self.stream = stream
        h = ctypes.c_void_p()
        st = self.lib.gbrt_context_create(device, ctypes.c_void_p(stream.cuda_stream), ctypes.byref(h))
        if st != 0:
            raise GbrtError(st, "gbrt_context_create failed")
        self.h = h

    def check(self, st):
        if st != 0:
            raise GbrtError(st, self.lib.gbrt_last_error(self.h).decode())

    def synchronize(self):
        self.check(self.lib.gbrt_context_synchronize(self.h))

    TRACE_SORT_RAYS = 1
    TRACE_WIDE_NODES = 2
    TRACE_PERSISTENT = 4
    TRACE_COMPRESSED_NODES = 8
    TRACE_WIDE8_NODES = 16

    def set_trace_flags(self, flags):
        """GBRT_TRACE_* options of the ray queries (TRACE_SORT_RAYS: coherent order)."""
        self.check(self.lib.gbrt_context_set_trace_flags(self.h, int(flags)))

    def set_trace_refill(self, min_idle_lanes):
        """Persistent traversal: idle lanes of a warp that trigger a refill (1..32)."""
        self.check(self.lib.gbrt_context_set_trace_refill(self.h, int(min_idle_lanes)))

    def set_host_chunk(self, rays):
        """Rays per chunk of the host-buffer queries (2^16 .. 2^26, default 2^23)."""
        self.check(self.lib.gbrt_context_set_host_chunk(self.h, int(rays)))

    @property
    def launches(self):
        return int(self.lib.gbrt_kernel_launch_count(self.h))

    def set_kernel_timing(self, enable):
        """Records CUDA events around the traversal kernel of every ray query (see
        gbrt_context_set_kernel_timing); enabling clears the record."""
        self.check(self.lib.gbrt_context_set_kernel_timing(self.h, 1 if enable else 0))

    def kernel_times(self, max_queries=256):
        """Traversal-kernel durations (ms) of the queries recorded since the last call,
        oldest first (at most the 256 most recent); waits for them."""
        out = np.zeros(max_queries, np.float32)
        count = ctypes.c_uint32()
        self.check(self.lib.gbrt_context_kernel_times(self.h, _hptr(out), max_queries, ctypes.byref(count)))
        return [float(x) for x in out[:count.value]]

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbrt_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = {}


def default_context(device=0):
    if device not in _default:
        _default[device] = Context(device)
    return _default[device]


def as_device_bytes(arr, device=0):
    """numpy structured array -> torch uint8 CUDA tensor holding the same bytes."""
    torch = _torch()
    a = np.ascontiguousarray(arr)
    return torch.from_numpy(a.view(np.uint8).reshape(-1)).to(f"cuda:{device}")


def device_rays(rays, device=0):
    """Rays as an (n, 8) float32 CUDA tensor (16-byte aligned, 32 bytes per ray)."""
    torch = _torch()
    a = np.ascontiguousarray(rays)
    return torch.from_numpy(a.view(np.float32).reshape(-1, 8)).to(f"cuda:{device}")


def hits_to_numpy(t):
    return t.detach().cpu().numpy().reshape(-1).view(HIT)


class IndexBVH:
    """cuda_index_bvh<basic_triangle<3, float>> counterpart: an opaque device BVH."""

    def __init__(self, ctx, handle):
        self.ctx, self.h = ctx, handle

    @property
    def counts(self):
        p, nn, d = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        self.ctx.check(self.ctx.lib.gbrt_bvh_counts(self.h, ctypes.byref(p), ctypes.byref(nn), ctypes.byref(d)))
        return p.value, nn.value, d.value

    @classmethod
    def upload(cls, nodes, indices, tris, ctx=None):
        """Host visionaray index_bvh (BVH_NODE nodes, uint32 indices, TRIANGLE prims)."""
        ctx = ctx or default_context()
        nodes = np.ascontiguousarray(nodes, BVH_NODE)
        indices = np.ascontiguousarray(indices, np.uint32)
        tris = np.ascontiguousarray(tris, TRIANGLE)
        h = ctypes.c_void_p()
        ctx.check(ctx.lib.gbrt_bvh_upload_bvh2_host(ctx.h, _hptr(nodes), len(nodes), _hptr(indices), len(indices),
                                                    _hptr(tris), len(tris), ctypes.byref(h)))
        return cls(ctx, h)

    def export_bvh2(self):
        """(nodes, indices) in the reference GPU builder's cuda_index_bvh layout."""
        torch = _torch()
        n, nn, _ = self.counts
        nodes = torch.empty(max(nn, 1) * 32, dtype=torch.uint8, device=f"cuda:{self.ctx.device}")
        idx = torch.empty(max(n, 1), dtype=torch.int32, device=f"cuda:{self.ctx.device}")
        self.ctx.check(self.ctx.lib.gbrt_bvh_export_bvh2(self.ctx.h, self.h, _dptr(nodes), _dptr(idx)))
        self.ctx.synchronize()
        return (nodes.cpu().numpy()[: nn * 32].view(BVH_NODE),
                idx.cpu().numpy()[:n].view(np.uint32))

    def refit(self, tris):
        """bvh_refitter::refit: new positions of the same triangles (torch uint8 CUDA tensor,
        n x 44 bytes, the build's input order); topology kept, boxes recomputed."""
        n = tris.numel() * tris.element_size() // TRIANGLE.itemsize
        self.ctx.check(self.ctx.lib.gbrt_bvh_refit(self.ctx.h, self.h, _dptr(tris), n))
        return self

    def rebuild(self, tris):
        """lbvh_builder::build into this tree's arrays (gbrt_bvh_rebuild_lbvh): the same
        number of triangles at any positions (torch uint8 CUDA tensor, n x 44 bytes); no
        device allocation."""
        n = tris.numel() * tris.element_size() // TRIANGLE.itemsize
        self.ctx.check(self.ctx.lib.gbrt_bvh_rebuild_lbvh(self.ctx.h, self.h, _dptr(tris), n))
        return self

    def morton_codes(self):
        torch = _torch()
        n, _, _ = self.counts
        out = torch.empty(max(n, 1), dtype=torch.int32, device=f"cuda:{self.ctx.device}")
        self.ctx.check(self.ctx.lib.gbrt_bvh_morton_codes(self.ctx.h, self.h, _dptr(out)))
        self.ctx.synchronize()
        return out.cpu().numpy()[:n].view(np.uint32)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gbrt_bvh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class lbvh_builder:
    """lbvh_builder (detail/bvh/lbvh.h:473-851), GPU build only."""

    def __init__(self, ctx=None):
        self.ctx = ctx or default_context()

    def build(self, tris):
        """tris: torch uint8 CUDA tensor of n*44 bytes (device path) or a numpy
        TRIANGLE array (host path, copied in)."""
        ctx = self.ctx
        h = ctypes.c_void_p()
        if isinstance(tris, np.ndarray):
            tris = np.ascontiguousarray(tris, TRIANGLE)
            ctx.check(ctx.lib.gbrt_bvh_build_lbvh_host(ctx.h, _hptr(tris), len(tris), ctypes.byref(h)))
        else:
            n = tris.numel() * tris.element_size() // TRIANGLE.itemsize
            ctx.check(ctx.lib.gbrt_bvh_build_lbvh(ctx.h, _dptr(tris), n, ctypes.byref(h)))
        return IndexBVH(ctx, h)


class ploc_builder:
    """High-quality GPU build (parallel locally-ordered clustering); no visionaray
    counterpart.  Same IndexBVH handle as lbvh_builder."""

    def __init__(self, ctx=None):
        self.ctx = ctx or default_context()

    def build(self, tris):
        """tris: torch uint8 CUDA tensor of n*44 bytes."""
        ctx = self.ctx
        h = ctypes.c_void_p()
        n = tris.numel() * tris.element_size() // TRIANGLE.itemsize
        ctx.check(ctx.lib.gbrt_bvh_build_ploc(ctx.h, _dptr(tris), n, ctypes.byref(h)))
        return IndexBVH(ctx, h)


def _trace(rays, bvh, out, any_hit):
    ctx = bvh.ctx
    lib = ctx.lib
    if isinstance(rays, np.ndarray):
        rays = np.ascontiguousarray(rays, RAY)
        hits = out if out is not None else np.empty(len(rays), HIT)
        fn = lib.gbrt_trace_any_hit_host if any_hit else lib.gbrt_trace_closest_hit_host
        ctx.check(fn(ctx.h, bvh.h, _hptr(rays), len(rays), _hptr(hits)))
        return hits
    torch = _torch()
    n = rays.numel() * rays.element_size() // RAY.itemsize
    hits = out if out is not None else torch.empty((n, 4), dtype=torch.float32, device=rays.device)
    fn = lib.gbrt_trace_any_hit if any_hit else lib.gbrt_trace_closest_hit
    ctx.check(fn(ctx.h, bvh.h, _dptr(rays), n, _dptr(hits)))
    return hits


def closest_hit(rays, bvh, out=None):
    """closest_hit over one BVH for a batch of rays (device tensor or host array)."""
    return _trace(rays, bvh, out, False)


def any_hit(rays, bvh, out=None):
    """any_hit over one BVH for a batch of rays (device tensor or host array)."""
    return _trace(rays, bvh, out, True)


class PTScene:
    """make_kernel_params(prims, materials, lights, ...) counterpart: a BVH with its
    materials (one per geom_id) and lights -- AREA_LIGHT records, or LIGHT records
    (area, point and spot lights) -- ready for pathtrace_frame."""

    def __init__(self, bvh, materials, lights):
        self.bvh, self.ctx = bvh, bvh.ctx
        mats = np.ascontiguousarray(materials, MATERIAL)
        h = ctypes.c_void_p()
        if np.asarray(lights).dtype == LIGHT:
            lts = np.ascontiguousarray(lights, LIGHT)
            create = self.ctx.lib.gbrt_pt_scene_create_lights
        else:
            lts = np.ascontiguousarray(lights, AREA_LIGHT)
            create = self.ctx.lib.gbrt_pt_scene_create
        self.ctx.check(create(self.ctx.h, bvh.h, _hptr(mats), len(mats), _hptr(lts), len(lts), ctypes.byref(h)))
        self.h = h
        self._env = None

    @classmethod
    def over_instances(cls, tlas, materials, lights, inst_geom):
        """make_kernel_params over a two-level tree (gbrt_pt_scene_create_instanced):
        rays traced through the TLAS's instances, a hit shaded with its instance's
        triangle in world space and material slot inst_geom[instance] + geom_id."""
        from .types import lights_of_area_lights
        self = cls.__new__(cls)
        self.bvh, self.tlas, self.ctx = None, tlas, tlas.ctx
        mats = np.ascontiguousarray(materials, MATERIAL)
        lts = (np.ascontiguousarray(lights, LIGHT) if np.asarray(lights).dtype == LIGHT
               else lights_of_area_lights(lights))
        geom = np.ascontiguousarray(inst_geom, np.uint32)
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.gbrt_pt_scene_create_instanced(self.ctx.h, tlas.h, _hptr(mats), len(mats),
                                                                   _hptr(lts), len(lts), _hptr(geom), ctypes.byref(h)))
        self.h = h
        self._env = None
        return self

    def set_environment(self, texels, filter=FILTER_LINEAR, address=ADDRESS_CLAMP, scale=(1.0, 1.0, 1.0),
                        light_to_world=None):
        """environment_light in place of the ambient light: texels is an (h, w, 4)
        float32 CUDA tensor (texel (x, y) at [y, x]), kept alive by the scene; None
        removes it."""
        if texels is None:
            self.ctx.check(self.ctx.lib.gbrt_pt_scene_set_environment(self.ctx.h, self.h, None))
            self._env = None
            return
        t = texels.contiguous()
        if t.dim() != 3 or t.shape[2] != 4 or t.dtype != _torch().float32 or not t.is_cuda:
            raise ValueError("texels must be an (h, w, 4) float32 CUDA tensor")
        e = environment(t.data_ptr(), t.shape[1], t.shape[0], filter, address, scale, light_to_world)
        self.ctx.check(self.ctx.lib.gbrt_pt_scene_set_environment(self.ctx.h, self.h, _hptr(e)))
        self._env = t

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gbrt_pt_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pinhole_camera_basis(camera, width, height):
    """pinhole_camera::begin_frame: (eye, U, V, W) as a (4, 3) float32 array."""
    cam = np.ascontiguousarray(np.asarray(camera, CAMERA).reshape(1))
    out = np.zeros((4, 3), np.float32)
    st = load_library().gbrt_pinhole_camera_basis(_hptr(cam), int(width), int(height), _hptr(out))
    if st != 0:
        raise GbrtError(st, "gbrt_pinhole_camera_basis: bad camera or size")
    return out


def pathtrace_frame(scene, camera, params, accum=None, color=None):
    """One frame of the jittered-blend sampler around the path tracer
    (cuda_sched::frame(pathtracing::kernel, sparams)).  accum / color are (h, w, 4)
    float32 CUDA tensors (accum is read and written); returns accum."""
    torch = _torch()
    ctx = scene.ctx
    cam = np.ascontiguousarray(np.asarray(camera, CAMERA).reshape(1))
    par = np.ascontiguousarray(np.asarray(params, PT_PARAMS).reshape(1))
    w, h = int(par["width"][0]), int(par["height"][0])
    dev = f"cuda:{ctx.device}"
    if accum is None:
        accum = torch.zeros((h, w, 4), dtype=torch.float32, device=dev)
    cptr = _dptr(color) if color is not None else None
    ctx.check(ctx.lib.gbrt_pathtrace_frame(ctx.h, scene.h, _hptr(cam), _hptr(par), _dptr(accum), cptr))
    return accum


def pathtrace_forward(scene, camera, params, albedo, emission, image=None):
    """Differentiable renderer, forward: image (h, w, 4) of one frame with per-slot
    albedo / emission parameters ((num_materials, 3) float32 CUDA tensors)."""
    torch = _torch()
    ctx = scene.ctx
    cam = np.ascontiguousarray(np.asarray(camera, CAMERA).reshape(1))
    par = np.ascontiguousarray(np.asarray(params, PT_PARAMS).reshape(1))
    w, h = int(par["width"][0]), int(par["height"][0])
    if image is None:
        image = torch.empty((h, w, 4), dtype=torch.float32, device=f"cuda:{ctx.device}")
    ctx.check(ctx.lib.gbrt_pathtrace_forward(ctx.h, scene.h, _hptr(cam), _hptr(par), _dptr(albedo),
                                             _dptr(emission), _dptr(image)))
    return image


def pathtrace_backward(scene, camera, params, albedo, emission, image_adjoint, grad_albedo=None,
                       grad_emission=None):
    """Differentiable renderer, backward (path replay): gradients of sum(I * image_adjoint)
    w.r.t. albedo and emission, added to grad_albedo / grad_emission (zeros if None)."""
    torch = _torch()
    ctx = scene.ctx
    cam = np.ascontiguousarray(np.asarray(camera, CAMERA).reshape(1))
    par = np.ascontiguousarray(np.asarray(params, PT_PARAMS).reshape(1))
    if grad_albedo is None:
        grad_albedo = torch.zeros_like(albedo)
    if grad_emission is None:
        grad_emission = torch.zeros_like(emission)
    adj = image_adjoint.contiguous()
    ctx.check(ctx.lib.gbrt_pathtrace_backward(ctx.h, scene.h, _hptr(cam), _hptr(par), _dptr(albedo),
                                              _dptr(emission), _dptr(adj), _dptr(grad_albedo),
                                              _dptr(grad_emission)))
    return grad_albedo, grad_emission


class Batch:
    """Many scenes in one BVH arena (gbrt_batch): scene s owns the triangles
    [offsets[s], offsets[s + 1]) of one concatenated TRIANGLE array.  No visionaray
    counterpart: the reference builds and renders one scene per call."""

    def __init__(self, offsets, ctx=None):
        self.ctx = ctx or default_context()
        self.offsets = np.ascontiguousarray(offsets, np.uint32)
        self.num_scenes = len(self.offsets) - 1
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.gbrt_batch_create(self.ctx.h, _hptr(self.offsets), self.num_scenes,
                                                      ctypes.byref(h)))
        self.h = h
        self.pixel_offsets = None

    def build(self, tris):
        """tris: torch uint8 CUDA tensor of the concatenated triangles (44 bytes each)."""
        self.ctx.check(self.ctx.lib.gbrt_batch_build(self.ctx.h, self.h, _dptr(tris)))

    def export_bvh2(self, scene):
        """(nodes, indices) of one scene in the cuda_index_bvh layout."""
        torch = _torch()
        n = int(self.offsets[scene + 1] - self.offsets[scene])
        nn = 2 * n - 1 if n else 0
        dev = f"cuda:{self.ctx.device}"
        nodes = torch.empty(max(nn, 1) * 32, dtype=torch.uint8, device=dev)
        idx = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        self.ctx.check(self.ctx.lib.gbrt_batch_export_bvh2(self.ctx.h, self.h, scene, _dptr(nodes), _dptr(idx)))
        self.ctx.synchronize()
        return (nodes.cpu().numpy()[: nn * 32].view(BVH_NODE), idx.cpu().numpy()[:n].view(np.uint32))

    def closest_hit(self, rays, ray_offsets, out=None):
        """closest_hit of every scene's rays in one launch: scene s traces rays
        [ray_offsets[s], ray_offsets[s + 1]) of the (n, 8) float32 device tensor."""
        torch = _torch()
        ro = np.ascontiguousarray(ray_offsets, np.uint32)
        n = int(ro[-1])
        hits = out if out is not None else torch.empty((max(n, 1), 4), dtype=torch.float32, device=rays.device)
        self.ctx.check(self.ctx.lib.gbrt_batch_trace_closest_hit(self.ctx.h, self.h, _dptr(rays), _hptr(ro),
                                                                 _dptr(hits)))
        return hits

    def set_frames(self, cameras, params, materials):
        cams = np.ascontiguousarray(cameras, CAMERA)
        pars = np.ascontiguousarray(params, PT_PARAMS)
        mats = np.ascontiguousarray(materials, MATERIAL)
        self.ctx.check(self.ctx.lib.gbrt_batch_set_frames(self.ctx.h, self.h, _hptr(cams), _hptr(pars),
                                                          _hptr(mats), len(mats)))
        px = pars["width"].astype(np.uint64) * pars["height"].astype(np.uint64)
        self.pixel_offsets = np.concatenate([[0], np.cumsum(px)]).astype(np.uint64)

    def set_lights(self, lights, light_offsets):
        """Scene s samples lights[light_offsets[s]:light_offsets[s + 1]] (LIGHT records,
        or AREA_LIGHT records, which are converted)."""
        from .types import lights_of_area_lights
        lts = (np.ascontiguousarray(lights, LIGHT) if np.asarray(lights).dtype == LIGHT
               else lights_of_area_lights(lights))
        offs = np.ascontiguousarray(light_offsets, np.uint32)
        self.ctx.check(self.ctx.lib.gbrt_batch_set_lights(self.ctx.h, self.h, _hptr(lts), len(lts),
                                                          _hptr(offs) if len(lts) else None))

    @property
    def launch(self):
        out = np.zeros(1, BATCH_LAUNCH)
        self.ctx.check(self.ctx.lib.gbrt_batch_get_launch(self.h, _hptr(out)))
        return out[0]

    @launch.setter
    def launch(self, value):
        """(block, tile, stack, order[, width[, sort]]): width defaults to 2 (node
        pairs), sort to 0."""
        v = [int(x) for x in (tuple(value) if not isinstance(value, np.void) else value.tolist())]
        v += [2, 0][len(v) - 4:] if len(v) < 6 else []
        arr = np.asarray([tuple(v)], BATCH_LAUNCH)
        self.ctx.check(self.ctx.lib.gbrt_batch_set_launch(self.h, _hptr(arr)))

    def height(self):
        out = ctypes.c_uint32()
        self.ctx.check(self.ctx.lib.gbrt_batch_height(self.ctx.h, self.h, ctypes.byref(out)))
        return out.value

    def new_images(self):
        torch = _torch()
        return torch.empty((max(int(self.pixel_offsets[-1]), 1), 4), dtype=torch.float32,
                           device=f"cuda:{self.ctx.device}")

    def pathtrace(self, images=None):
        """One frame of every scene in one persistent launch -> (total_pixels, 4) images."""
        images = images if images is not None else self.new_images()
        self.ctx.check(self.ctx.lib.gbrt_batch_pathtrace(self.ctx.h, self.h, _dptr(images)))
        return images

    def run_graph(self, tris, images):
        """build + pathtrace replayed from one CUDA graph."""
        self.ctx.check(self.ctx.lib.gbrt_batch_run_graph(self.ctx.h, self.h, _dptr(tris), _dptr(images)))
        return images

    def autotune(self, images, reps=2):
        """Picks the fastest launch shape; returns (launch record, ms per frame)."""
        best = np.zeros(1, BATCH_LAUNCH)
        ms = ctypes.c_float()
        self.ctx.check(self.ctx.lib.gbrt_batch_autotune(self.ctx.h, self.h, _dptr(images), reps, _hptr(best),
                                                        ctypes.byref(ms)))
        return best[0], ms.value

    def image(self, images, scene, params):
        """Scene s's (h, w, 4) view of the batch images."""
        p = np.asarray(params, PT_PARAMS).reshape(-1)[scene]
        a, b = int(self.pixel_offsets[scene]), int(self.pixel_offsets[scene + 1])
        return images[a:b].reshape(int(p["height"]), int(p["width"]), 4)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gbrt_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TLAS:
    """The top-level tree over instances (index_bvh<index_bvh_inst_t>): instances is a
    list of (IndexBVH, transform) with transform visionaray's mat4x3 as 12 floats
    (columns 0..3; the linear map's row i is column i, the translation column 3).
    Keeps the bottom-level trees alive."""

    def __init__(self, instances, ctx=None):
        self.ctx = ctx or default_context()
        self.blas = [b for b, _ in instances]
        arr = np.zeros(len(instances), INSTANCE)
        for k, (b, xf) in enumerate(instances):
            arr[k]["blas"] = b.h.value or 0
            arr[k]["transform"] = np.asarray(xf, np.float32).reshape(12)
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.gbrt_tlas_build(self.ctx.h, _hptr(arr), len(arr), ctypes.byref(h)))
        self.h = h

    def _trace(self, rays, any_hit, out):
        torch = _torch()
        n = rays.numel() * rays.element_size() // RAY.itemsize
        hits = out if out is not None else torch.empty((max(n, 1), 8), dtype=torch.float32, device=rays.device)
        fn = self.ctx.lib.gbrt_tlas_trace_any_hit if any_hit else self.ctx.lib.gbrt_tlas_trace_closest_hit
        self.ctx.check(fn(self.ctx.h, self.h, _dptr(rays), n, _dptr(hits)))
        return hits

    def closest_hit(self, rays, out=None):
        """Device rays (n, 8) float32 -> (n, 8) hit records (HIT_INST bytes)."""
        return self._trace(rays, False, out)

    def any_hit(self, rays, out=None):
        return self._trace(rays, True, out)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gbrt_tlas_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def hits_inst_to_numpy(t, n=None):
    a = t.detach().cpu().numpy().reshape(-1).view(HIT_INST)
    return a if n is None else a[:n]
