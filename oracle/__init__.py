"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py, always as the checker or the timed CPU baseline, never as the product.
`Oracle` wraps oracle/_build/liboracle.so (the restatement, oracle.cpp);
`Reference` wraps oracle/_ref/libvsnray_ref.so (visionaray's own CPU code compiled
from its headers), which exists only where the visionaray sources were present.
"""
import ctypes
import os

import numpy as np

from visionaray_gb300.types import (ADDRESS_CLAMP, BVH_NODE, CAMERA, FILTER_LINEAR, HIT, LIGHT, MATERIAL, PT_PARAMS,
                                    environment, lights_of_area_lights)

HERE = os.path.dirname(os.path.abspath(__file__))
LIBORACLE = os.path.join(HERE, "_build", "liboracle.so")
LIBREF = os.path.join(HERE, "_ref", "libvsnray_ref.so")

_vp, _u32, _u64, _i32, _f32 = (ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64,
                               ctypes.c_int, ctypes.c_float)


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class Tree:
    """Host BVH in visionaray's index_bvh layout: nodes (BVH_NODE) and indices."""

    def __init__(self, nodes, indices):
        self.nodes = nodes
        self.indices = indices

    @property
    def depth(self):
        if len(self.nodes) == 0:
            return 0
        best, st = 0, [(0, 1)]
        while st:
            i, d = st.pop()
            best = max(best, d)
            if self.nodes["num_prims"][i] == 0:
                f = int(self.nodes["first"][i])
                st += [(f, d + 1), (f + 1, d + 1)]
        return best


class env_light:
    """An environment light for the host renderers: texels (h, w, 4) float32 (texel
    (x, y) at [y, x]), FILTER_* / ADDRESS_* modes, scale and a 4x4 light_to_world."""

    def __init__(self, texels, filter=FILTER_LINEAR, address=ADDRESS_CLAMP, scale=(1.0, 1.0, 1.0),
                 light_to_world=None):
        self.texels = np.ascontiguousarray(texels, np.float32)
        h, w = self.texels.shape[:2]
        self.record = environment(self.texels.ctypes.data, w, h, filter, address, scale, light_to_world)


def _env_p(env):
    return None if env is None else env.record.ctypes.data


def _as_lights(lights):
    """LIGHT records (area, point, spot); AREA_LIGHT records are converted."""
    if np.asarray(lights).dtype == LIGHT:
        return np.ascontiguousarray(lights, LIGHT)
    return lights_of_area_lights(lights)


class Oracle:
    def __init__(self, path=LIBORACLE):
        if not os.path.exists(path):
            raise RuntimeError(f"{path} missing: build the oracle (make -C oracle)")
        L = ctypes.CDLL(path)
        for name in ("orc_build_sah", "orc_build_lbvh_cpu"):
            getattr(L, name).argtypes = [_vp, _u32, _i32]
            getattr(L, name).restype = _vp
        L.orc_build_karras.argtypes = [_vp, _u32]
        L.orc_build_karras.restype = _vp
        for name in ("orc_bvh_num_nodes", "orc_bvh_num_indices", "orc_bvh_depth"):
            getattr(L, name).argtypes = [_vp]
            getattr(L, name).restype = _u32
        L.orc_bvh_copy.argtypes = [_vp, _vp, _vp]
        L.orc_bvh_free.argtypes = [_vp]
        L.orc_morton_codes.argtypes = [_vp, _u32, _vp]
        L.orc_karras_children.argtypes = [_vp, _u32, _vp, _vp]
        L.orc_sah_cost.argtypes = [_vp, _u32, _f32, _f32, _f32]
        L.orc_refit.argtypes = [_vp, _u32, _vp, _vp, _vp]
        L.orc_trace_instances.argtypes = [_vp, _u32, _vp, _u64, _i32, _i32, _vp]
        L.orc_sah_cost.restype = _f32
        L.orc_intersect_triangle.argtypes = [_vp, _vp, _vp]
        L.orc_intersect_triangle.restype = _i32
        L.orc_intersect_box.argtypes = [_vp, _vp, _vp, _vp, _vp]
        L.orc_intersect_box.restype = _i32
        L.orc_trace.argtypes = [_vp, _u32, _vp, _vp, _vp, _u64, _i32, _i32, _vp, _vp]
        L.orc_trace.restype = _i32
        L.orc_trace_linear.argtypes = [_vp, _u32, _vp, _u64, _i32, _i32, _vp]
        L.orc_pathtrace.argtypes = [_vp, _vp, _u32, _vp, _vp, _u32, _vp, _u32, _vp, _vp, _i32, _i32, _vp, _vp, _vp]
        L.orc_pathtrace_pixels.argtypes = [_vp, _vp, _u32, _vp, _vp, _u32, _vp, _u32, _vp, _vp, _i32, _i32, _vp,
                                           _u64, _vp, _vp, _vp]
        L.orc_pathtrace_adjoint.argtypes = [_vp, _vp, _u32, _vp, _vp, _u32, _vp, _u32, _vp, _vp, _vp, _vp, _vp,
                                            _i32, _i32, _vp, _vp, _vp, _vp]
        self.L = L

    def _tree(self, h):
        if not h:
            raise ValueError("oracle refused the build")
        try:
            nodes = np.zeros(self.L.orc_bvh_num_nodes(h), BVH_NODE)
            idx = np.zeros(self.L.orc_bvh_num_indices(h), np.uint32)
            self.L.orc_bvh_copy(h, _p(nodes), _p(idx))
            return Tree(nodes, idx)
        finally:
            self.L.orc_bvh_free(h)

    def build_sah(self, tris, max_leaf=4):
        tris = np.ascontiguousarray(tris)
        return self._tree(self.L.orc_build_sah(_p(tris), len(tris), max_leaf))

    def build_lbvh_cpu(self, tris, max_leaf=4):
        tris = np.ascontiguousarray(tris)
        return self._tree(self.L.orc_build_lbvh_cpu(_p(tris), len(tris), max_leaf))

    def build_karras(self, tris):
        tris = np.ascontiguousarray(tris)
        return self._tree(self.L.orc_build_karras(_p(tris), len(tris)))

    def morton_codes(self, tris):
        tris = np.ascontiguousarray(tris)
        out = np.empty(len(tris), np.uint32)
        self.L.orc_morton_codes(_p(tris), len(tris), _p(out))
        return out

    def karras_children(self, sorted_codes):
        c = np.ascontiguousarray(sorted_codes, np.uint32)
        n = len(c)
        left = np.empty(max(n - 1, 0), np.int32)
        right = np.empty(max(n - 1, 0), np.int32)
        self.L.orc_karras_children(_p(c), n, _p(left), _p(right))
        return left, right

    def sah_cost(self, tree, ci=1.2, cl=0.0, cp=1.0):
        return self.L.orc_sah_cost(_p(tree.nodes), len(tree.nodes), ci, cl, cp)

    def trace(self, tree, tris, rays, any_hit=False, nthreads=0, counters=False):
        tris = np.ascontiguousarray(tris)
        rays = np.ascontiguousarray(rays)
        hits = np.empty(len(rays), HIT)
        cnt = np.zeros(2, np.uint64)
        rc = self.L.orc_trace(_p(tree.nodes), len(tree.nodes), _p(tree.indices), _p(tris),
                              _p(rays), len(rays), int(any_hit), nthreads, _p(hits), _p(cnt))
        if rc != 0:
            raise RuntimeError("oracle traversal stack (32 entries) overflowed")
        return (hits, cnt) if counters else hits

    def trace_linear(self, tris, rays, any_hit=False, nthreads=0):
        tris = np.ascontiguousarray(tris)
        rays = np.ascontiguousarray(rays)
        hits = np.empty(len(rays), HIT)
        self.L.orc_trace_linear(_p(tris), len(tris), _p(rays), len(rays), int(any_hit), nthreads,
                                _p(hits))
        return hits

    PT_FLOAT, PT_DOUBLE, PT_FLOAT_TRIG_DOUBLE = 0, 1, 2
    # or-ed into a mode: the hemisphere sample's two draws in argument order, as
    # visionaray's device build evaluates them (its CPU build draws the second first)
    PT_DRAWS_IN_ORDER = 4

    def pathtrace(self, tree, tris, materials, lights, camera, params, mode=1, nthreads=0, env=None):
        """Per-pixel average RGBA (height, width, 4) of one frame, and the counters
        {closest, shadow, boxes, tris}.  mode: PT_FLOAT (the reference's arithmetic),
        PT_DOUBLE (the FP64 oracle), PT_FLOAT_TRIG_DOUBLE (the CUDA path's).  env: an
        environment light (env_light()) in place of the ambient light."""
        tris = np.ascontiguousarray(tris)
        materials = np.ascontiguousarray(materials, MATERIAL)
        lights = _as_lights(lights)
        camera = np.ascontiguousarray(np.asarray(camera, CAMERA).reshape(1))
        params = np.ascontiguousarray(np.asarray(params, PT_PARAMS).reshape(1))
        w, h = int(params["width"][0]), int(params["height"][0])
        out = np.zeros((h, w, 4), np.float64)
        cnt = np.zeros(4, np.uint64)
        self.L.orc_pathtrace(_p(tris), _p(tree.nodes), len(tree.nodes), _p(tree.indices), _p(materials),
                             len(materials), _p(lights), len(lights), _p(camera), _p(params), int(mode), nthreads,
                             _p(out), _p(cnt), _env_p(env))
        return out, cnt

    def pathtrace_pixels(self, tree, tris, materials, lights, camera, params, pixels, mode=1, nthreads=0, env=None):
        """`pathtrace` on the listed pixels only (row-major indices < width * height):
        RGBA (len(pixels), 4) and the counters {closest, shadow, boxes, tris} of those
        pixels' paths."""
        tris = np.ascontiguousarray(tris)
        materials = np.ascontiguousarray(materials, MATERIAL)
        lights = _as_lights(lights)
        camera = np.ascontiguousarray(np.asarray(camera, CAMERA).reshape(1))
        params = np.ascontiguousarray(np.asarray(params, PT_PARAMS).reshape(1))
        pix = np.ascontiguousarray(pixels, np.uint32)
        npix = int(params["width"][0]) * int(params["height"][0])
        if len(pix) and int(pix.max()) >= npix:
            raise ValueError("pixel index outside the frame")
        out = np.zeros((len(pix), 4), np.float64)
        cnt = np.zeros(4, np.uint64)
        self.L.orc_pathtrace_pixels(_p(tris), _p(tree.nodes), len(tree.nodes), _p(tree.indices), _p(materials),
                                    len(materials), _p(lights), len(lights), _p(camera), _p(params), int(mode),
                                    nthreads, _p(pix), len(pix), _p(out), _p(cnt), _env_p(env))
        return out, cnt

    def pathtrace_adjoint(self, tree, tris, materials, lights, camera, params, albedo, emission, img_adj,
                          fp64=True, nthreads=0, env=None):
        """(grad_albedo, grad_emission, image): the path-replay adjoint of sum(I * img_adj)
        (img_adj (h, w, 4)) at the gbrt_rng.h stream, in double (fp64) or float."""
        tris = np.ascontiguousarray(tris)
        materials = np.ascontiguousarray(materials, MATERIAL)
        lights = _as_lights(lights)
        camera = np.ascontiguousarray(np.asarray(camera, CAMERA).reshape(1))
        params = np.ascontiguousarray(np.asarray(params, PT_PARAMS).reshape(1))
        w, h = int(params["width"][0]), int(params["height"][0])
        a = np.ascontiguousarray(albedo, np.float32) if albedo is not None else None
        e = np.ascontiguousarray(emission, np.float32) if emission is not None else None
        adj = np.ascontiguousarray(img_adj, np.float64)
        ga = np.zeros((len(materials), 3), np.float64)
        ge = np.zeros((len(materials), 3), np.float64)
        img = np.zeros((h, w, 4), np.float64)
        self.L.orc_pathtrace_adjoint(_p(tris), _p(tree.nodes), len(tree.nodes), _p(tree.indices), _p(materials),
                                     len(materials), _p(lights), len(lights), _p(camera), _p(params), _p(a), _p(e),
                                     _p(adj), int(fp64), nthreads, _p(ga), _p(ge), _p(img), _env_p(env))
        return ga, ge, img

    def refit(self, tree, tris):
        """bvh_refitter::refit: the tree's nodes with boxes recomputed from `tris`."""
        nodes = np.ascontiguousarray(tree.nodes, BVH_NODE)
        out = np.empty_like(nodes)
        tris = np.ascontiguousarray(tris)
        self.L.orc_refit(_p(nodes), len(nodes), _p(np.ascontiguousarray(tree.indices, np.uint32)), _p(tris), _p(out))
        return Tree(out, tree.indices)

    def trace_instances(self, instances, rays, any_hit=False, nthreads=0):
        """Two-level query, brute force over instances = [(tree, tris, transform12)]."""
        from visionaray_gb300.types import HIT_INST

        class Inst(ctypes.Structure):
            _fields_ = [("nodes", _vp), ("num_nodes", _u32), ("indices", _vp), ("tris", _vp),
                        ("transform", ctypes.c_float * 12)]
        keep = []
        arr = (Inst * max(len(instances), 1))()
        for k, (tree, tris, xf) in enumerate(instances):
            nodes = np.ascontiguousarray(tree.nodes, BVH_NODE)
            idx = np.ascontiguousarray(tree.indices, np.uint32)
            tr = np.ascontiguousarray(tris)
            keep += [nodes, idx, tr]
            arr[k].nodes, arr[k].num_nodes = nodes.ctypes.data, len(nodes)
            arr[k].indices, arr[k].tris = idx.ctypes.data, tr.ctypes.data
            arr[k].transform[:] = [float(x) for x in np.asarray(xf, np.float32).reshape(12)]
        rays = np.ascontiguousarray(rays)
        out = np.zeros(len(rays), HIT_INST)
        self.L.orc_trace_instances(ctypes.addressof(arr), len(instances), _p(rays), len(rays), int(any_hit),
                                   nthreads, _p(out))
        return out

    def intersect_box(self, ray, bmin, bmax):
        ray = np.ascontiguousarray(np.asarray(ray).reshape(1))
        lo = np.ascontiguousarray(bmin, np.float32)
        hi = np.ascontiguousarray(bmax, np.float32)
        tn, tf = ctypes.c_float(), ctypes.c_float()
        hit = self.L.orc_intersect_box(_p(ray), _p(lo), _p(hi), ctypes.byref(tn), ctypes.byref(tf))
        return bool(hit), tn.value, tf.value

    def intersect(self, ray, tri):
        ray = np.ascontiguousarray(np.asarray(ray).reshape(1))
        tri = np.ascontiguousarray(np.asarray(tri).reshape(1))
        out = np.empty(1, HIT)
        hit = self.L.orc_intersect_triangle(_p(ray), _p(tri), _p(out))
        return bool(hit), out[0]


class Reference:
    """visionaray's own CPU code (oracle/_ref); only where it was built."""

    @staticmethod
    def available():
        return os.path.exists(LIBREF)

    def __init__(self, path=LIBREF):
        L = ctypes.CDLL(path)
        for name in ("ref_build_sah", "ref_build_lbvh_cpu"):
            getattr(L, name).argtypes = [_vp, _u32, _i32]
            getattr(L, name).restype = _vp
        for name in ("ref_num_nodes", "ref_num_indices"):
            getattr(L, name).argtypes = [_vp]
            getattr(L, name).restype = _u32
        L.ref_copy.argtypes = [_vp, _vp, _vp]
        L.ref_free.argtypes = [_vp]
        L.ref_sah_cost.argtypes = [_vp]
        L.ref_sah_cost.restype = _f32
        L.ref_lbvh_sorted_refs.argtypes = [_vp, _u32, _vp, _vp]
        L.ref_karras_children.argtypes = [_vp, _u32, _vp, _vp]
        L.ref_trace.argtypes = [_vp, _vp, _u64, _i32, _i32, _vp, _vp]
        L.ref_trace.restype = _i32
        L.ref_pathtrace.argtypes = [_vp, _u32, _vp, _u32, _vp, _u32, _vp, _vp, _vp, _i32, _vp]
        L.ref_refit.argtypes = [_vp, _vp, _u32]
        L.ref_trace_instances.argtypes = [_u32, _vp, _vp, _u32, _vp, _vp, _vp, _u64, _i32, _vp]
        self.L = L

    class Handle:
        def __init__(self, L, h):
            self.L, self.h = L, h

        def __del__(self):
            if self.h:
                self.L.ref_free(self.h)
                self.h = None

        def tree(self):
            nodes = np.zeros(self.L.ref_num_nodes(self.h), BVH_NODE)
            idx = np.zeros(self.L.ref_num_indices(self.h), np.uint32)
            self.L.ref_copy(self.h, _p(nodes), _p(idx))
            return Tree(nodes, idx)

        def sah_cost(self):
            return self.L.ref_sah_cost(self.h)

        def refit(self, tris):
            """bvh_refitter::refit to new positions of the same triangles."""
            tris = np.ascontiguousarray(tris)
            self.L.ref_refit(self.h, _p(tris), len(tris))

        def trace(self, rays, any_hit=False, nthreads=0, counters=False):
            rays = np.ascontiguousarray(rays)
            hits = np.empty(len(rays), HIT)
            cnt = np.zeros(2, np.uint64)
            self.L.ref_trace(self.h, _p(rays), len(rays), int(any_hit), nthreads, _p(hits), _p(cnt))
            return (hits, cnt) if counters else hits

    def build_sah(self, tris, max_leaf=4):
        tris = np.ascontiguousarray(tris)
        return Reference.Handle(self.L, self.L.ref_build_sah(_p(tris), len(tris), max_leaf))

    def build_lbvh_cpu(self, tris, max_leaf=4):
        tris = np.ascontiguousarray(tris)
        return Reference.Handle(self.L, self.L.ref_build_lbvh_cpu(_p(tris), len(tris), max_leaf))

    def trace_instances(self, meshes, inst_mesh, transforms, rays, any_hit=False):
        """visionaray's own two-level query: meshes = [tris], instance k = mesh
        inst_mesh[k] with the mat4x3 transforms[k] (12 floats)."""
        from visionaray_gb300.types import HIT_INST
        meshes = [np.ascontiguousarray(m) for m in meshes]
        ptrs = (ctypes.c_void_p * len(meshes))(*[m.ctypes.data for m in meshes])
        sizes = np.array([len(m) for m in meshes], np.uint32)
        im = np.ascontiguousarray(inst_mesh, np.uint32)
        xf = np.ascontiguousarray(transforms, np.float32).reshape(-1)
        rays = np.ascontiguousarray(rays)
        out = np.zeros(len(rays), HIT_INST)
        self.L.ref_trace_instances(len(meshes), ctypes.addressof(ptrs), _p(sizes), len(im), _p(im), _p(xf), _p(rays),
                                   len(rays), int(any_hit), _p(out))
        return out

    def lbvh_sorted_refs(self, tris):
        tris = np.ascontiguousarray(tris)
        ids = np.empty(len(tris), np.int32)
        codes = np.empty(len(tris), np.uint32)
        self.L.ref_lbvh_sorted_refs(_p(tris), len(tris), _p(ids), _p(codes))
        return ids, codes

    def karras_children(self, sorted_codes):
        c = np.ascontiguousarray(sorted_codes, np.uint32)
        n = len(c)
        left = np.empty(max(n - 1, 0), np.int32)
        right = np.empty(max(n - 1, 0), np.int32)
        self.L.ref_karras_children(_p(c), n, _p(left), _p(right))
        return left, right

    def pathtrace(self, tris, materials, lights, camera, params, accum=None, nthreads=0, env=None):
        """visionaray's pathtracing::kernel (its SAH tree), one frame blended into accum
        (height, width, 4) float32; env (env_light): environment_light as amb_light."""
        tris = np.ascontiguousarray(tris)
        materials = np.ascontiguousarray(materials, MATERIAL)
        lights = _as_lights(lights)
        camera = np.ascontiguousarray(np.asarray(camera, CAMERA).reshape(1))
        params = np.ascontiguousarray(np.asarray(params, PT_PARAMS).reshape(1))
        w, h = int(params["width"][0]), int(params["height"][0])
        acc = np.zeros((h, w, 4), np.float32) if accum is None else np.ascontiguousarray(accum, np.float32)
        self.L.ref_pathtrace(_p(tris), len(tris), _p(materials), len(materials), _p(lights), len(lights),
                             _p(camera), _p(params), _p(acc), nthreads, _env_p(env))
        return acc
