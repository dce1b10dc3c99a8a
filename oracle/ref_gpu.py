"""visionaray's own GPU traversal and path-tracing kernel, run on the GPU host.

BENCHMARK AND TEST INFRASTRUCTURE ONLY.  oracle/ref_gpu.cu drives visionaray's
closest_hit / any_hit (device branch: detail/bvh/intersect.inl:166-356) and
pathtracing::kernel (detail/pathtracing.inl:42-233) from a few extern "C" kernels; the
build compiles it from the unmodified visionaray headers into
oracle/_ref/vsnray_ref_gpu.cubin (device code for sm_103a, independent of the host
CPU).  This module loads that cubin with the CUDA driver API into torch's context and
launches its kernels on torch device buffers, so the reference's GPU path is timed on
the same GPU, trees, rays and random numbers as the product's kernels.  Nothing in
the product imports it.
"""
import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "vsnray_ref_gpu.cubin")               # nvcc defaults
CUBIN_EXACT = os.path.join(HERE, "_ref", "vsnray_ref_gpu_exact.cubin")   # --fmad=false
KERNELS = ("vsnray_ref_closest_hit", "vsnray_ref_any_hit", "vsnray_ref_pt_setup", "vsnray_ref_pathtrace",
           "vsnray_ref_pt_setup_ext", "vsnray_ref_pathtrace_ext", "vsnray_ref_sizes")
# visionaray's GPU LBVH build kernels (detail/bvh/lbvh.h:215-466), by their own names
LBVH_KERNELS = ("compute_bounds_and_centroids", "assign_morton_codes", "init_nodes", "build_hierarchy",
                "assign_node_bounds", "collapse", "sequence")
LIBSORT = os.path.join(HERE, "_build", "libref_sort.so")


def available(exact=False):
    return os.path.exists(CUBIN_EXACT if exact else CUBIN)


class _RefPtrs(ctypes.Structure):
    # index_bvh_ref_t: primitives, nodes, indices, each [first, last)
    _fields_ = [("p", ctypes.c_void_p * 6)]


def camera_basis(camera, width, height):
    """pinhole_camera::begin_frame's eye, U, V, W as the product computes them (12 float32)."""
    from visionaray_gb300.runtime import pinhole_camera_basis
    return pinhole_camera_basis(camera, width, height).reshape(-1)


class _Tree:
    """Device arrays of one tree and the index_bvh_ref_t over them (kept together so
    the arrays live as long as the pointers are used)."""

    def __init__(self, tris, nodes, indices):
        self.tensors = (tris, nodes, indices)
        n = tris.numel() * tris.element_size() // 44
        nn = nodes.numel() * nodes.element_size() // 32
        ni = indices.numel() * indices.element_size() // 4
        self.ptrs = _RefPtrs()
        t0, n0, i0 = tris.data_ptr(), nodes.data_ptr(), indices.data_ptr()
        self.ptrs.p[:] = [t0, t0 + 44 * n, n0, n0 + 32 * nn, i0, i0 + 4 * ni]


class ReferenceGPU:
    """The cubin's kernels on one device (torch's primary context).  exact: the build
    without fused multiply-adds (the CPU reference's arithmetic) instead of the one with
    nvcc's default contraction (visionaray's own GPU build)."""

    def __init__(self, device=0, exact=False):
        import torch
        path = CUBIN_EXACT if exact else CUBIN
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing (it is built where the visionaray headers are)")
        self.torch = torch
        self.dev = f"cuda:{device}"
        torch.cuda.set_device(device)
        torch.zeros(1, device=self.dev)   # makes the primary context current
        cu = ctypes.CDLL("libcuda.so.1")
        vp = ctypes.c_void_p
        cu.cuModuleLoad.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p]
        cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
        cu.cuLaunchKernel.argtypes = [vp] + [ctypes.c_uint] * 7 + [vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
        cu.cuGetErrorName.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        self.cu = cu
        self.mod = vp()
        self._check(cu.cuModuleLoad(ctypes.byref(self.mod), path.encode()), "cuModuleLoad")
        self.fn = {}
        for name in KERNELS:
            f = vp()
            self._check(cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()), name)
            self.fn[name] = f
        sizes = torch.zeros(8, dtype=torch.int32, device=self.dev)
        self._launch("vsnray_ref_sizes", (1, 1, 1), (1, 1, 1), [vp(sizes.data_ptr())])
        torch.cuda.synchronize()
        (self.size_ref, self.size_mat, self.size_light, self.size_mat_ext, self.size_light_ext, self.size_node,
         self.size_prim_ref, self.size_aabb) = (int(x) for x in sizes.tolist())
        self.lbvh = None

    def _check(self, err, what):
        if err != 0:
            name = ctypes.c_char_p()
            self.cu.cuGetErrorName(err, ctypes.byref(name))
            raise RuntimeError(f"{what}: CUDA driver error {err} ({name.value})")

    def _launch(self, name, grid, block, args):
        ptrs = (ctypes.c_void_p * len(args))(*[ctypes.addressof(a) for a in args])
        stream = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        self._check(self.cu.cuLaunchKernel(self.fn[name], *grid, *block, 0, stream, ptrs, None), name)

    def tree(self, tris, bvh):
        """index_bvh_ref_t of a product BVH built from the device triangles `tris` (n x 44 B,
        input order): its export in the reference GPU builder's cuda_index_bvh layout.
        The returned object owns the device copies the pointers refer to."""
        _, _, height = bvh.counts
        # the reference's device traversal encodes its restart trail in 64 bits
        # (detail/bvh/intersect.inl:166-356): deeper trees are outside its domain
        if height >= 63:
            raise ValueError(f"tree height {height}: beyond the reference traversal's 64-level trail")
        from visionaray_gb300.runtime import as_device_bytes
        nodes, idx = bvh.export_bvh2()
        return _Tree(tris, as_device_bytes(nodes), self.torch.from_numpy(idx.view(np.int32)).to(self.dev))

    def trace(self, tree, rays, hits, any_hit=False, block=128):
        """closest_hit / any_hit of every ray (rays: (n, 8) float32, hits: (n, 4))."""
        n = rays.shape[0]
        if n == 0:
            return hits
        name = "vsnray_ref_any_hit" if any_hit else "vsnray_ref_closest_hit"
        self._launch(name, ((n + block - 1) // block, 1, 1), (block, 1, 1),
                     [tree.ptrs, ctypes.c_void_p(rays.data_ptr()), ctypes.c_uint(n),
                      ctypes.c_void_p(hits.data_ptr())])
        return hits

    def pt_scene(self, tree, materials, lights):
        """Device arrays of visionaray objects for pathtrace(): the tree ref, one
        material per slot and the lights.  Matte / emissive slots with area lights
        (AREA_LIGHT records) use generic_material<matte, emissive> and area_light;
        otherwise (a mirror, glass or plastic slot, or LIGHT records) the extended
        instantiation: generic_material<matte, emissive, mirror, glass, plastic> and
        generic_light<area_light, point_light, spot_light>."""
        torch = self.torch
        from visionaray_gb300.runtime import as_device_bytes
        from visionaray_gb300.types import LIGHT, MATTE, EMISSIVE, lights_of_area_lights
        materials = np.ascontiguousarray(materials)
        ext = np.asarray(lights).dtype == LIGHT or bool(np.isin(materials["kind"], (MATTE, EMISSIVE), invert=True).any())
        if ext and np.asarray(lights).dtype != LIGHT:
            lights = lights_of_area_lights(lights)
        m = as_device_bytes(materials)
        l_ = as_device_bytes(np.ascontiguousarray(lights)) if len(lights) else torch.zeros(128, dtype=torch.uint8,
                                                                                         device=self.dev)
        nm, nl = len(materials), len(lights)
        size_mat = self.size_mat_ext if ext else self.size_mat
        size_light = self.size_light_ext if ext else self.size_light
        refs = torch.zeros(self.size_ref, dtype=torch.uint8, device=self.dev)
        mats = torch.zeros(max(nm, 1) * size_mat, dtype=torch.uint8, device=self.dev)
        lts = torch.zeros(max(nl, 1) * size_light, dtype=torch.uint8, device=self.dev)
        items = max(nm, nl, 1)
        vp = ctypes.c_void_p
        self._launch("vsnray_ref_pt_setup_ext" if ext else "vsnray_ref_pt_setup", ((items + 127) // 128, 1, 1),
                     (128, 1, 1), [tree.ptrs, vp(refs.data_ptr()), vp(m.data_ptr()), ctypes.c_uint(nm),
                                   vp(mats.data_ptr()), vp(l_.data_ptr()), ctypes.c_uint(nl), vp(lts.data_ptr())])
        return {"refs": refs, "mats": mats, "lights": lts, "nl": nl, "ext": ext, "keep": (m, l_, tree)}

    def pathtrace(self, scene, camera, params, accum, block=(16, 16)):
        """One frame of pathtracing::kernel, one thread per pixel (cuda_sched's 16 x 16
        blocks by default), blended into accum ((h, w, 4) float32) like
        gbrt_pathtrace_frame."""
        p = np.ascontiguousarray(np.asarray(params).reshape(1))
        w, h = int(p["width"][0]), int(p["height"][0])
        cam = (ctypes.c_float * 12)(*camera_basis(camera, w, h).tolist())
        par = (ctypes.c_char * p.dtype.itemsize).from_buffer_copy(p.tobytes())
        vp = ctypes.c_void_p
        grid = ((w + block[0] - 1) // block[0], (h + block[1] - 1) // block[1], 1)
        self._launch("vsnray_ref_pathtrace_ext" if scene["ext"] else "vsnray_ref_pathtrace", grid,
                     (block[0], block[1], 1),
                     [vp(scene["refs"].data_ptr()), vp(scene["mats"].data_ptr()), vp(scene["lights"].data_ptr()),
                      ctypes.c_uint(scene["nl"]), cam, par, vp(accum.data_ptr())])
        return accum

    # -- visionaray's GPU LBVH build (lbvh_builder::build, detail/bvh/lbvh.h:681-844) --

    def _lbvh_kernels(self):
        """The build's kernels of the cubin, found by enumerating the module (they keep
        the reference's internal-linkage names)."""
        if self.lbvh is not None:
            return self.lbvh
        cu, vp = self.cu, ctypes.c_void_p
        cu.cuModuleGetFunctionCount.argtypes = [ctypes.POINTER(ctypes.c_uint), vp]
        cu.cuModuleEnumerateFunctions.argtypes = [ctypes.POINTER(vp), ctypes.c_uint, vp]
        cu.cuFuncGetName.argtypes = [ctypes.POINTER(ctypes.c_char_p), vp]
        count = ctypes.c_uint()
        self._check(cu.cuModuleGetFunctionCount(ctypes.byref(count), self.mod), "cuModuleGetFunctionCount")
        funcs = (vp * count.value)()
        self._check(cu.cuModuleEnumerateFunctions(funcs, count, self.mod), "cuModuleEnumerateFunctions")
        names = {}
        for f in funcs:
            nm = ctypes.c_char_p()
            self._check(cu.cuFuncGetName(ctypes.byref(nm), f), "cuFuncGetName")
            names[nm.value.decode()] = vp(f)
        found = {}
        for k in LBVH_KERNELS:
            pat = re.compile(r"4lbvhL?%d%s[EI]" % (len(k), k))
            hits = [n for n in names if pat.search(n)]
            if len(hits) != 1:
                raise RuntimeError(f"LBVH kernel {k}: {len(hits)} matches in the cubin")
            found[k] = names[hits[0]]
        sort = ctypes.CDLL(LIBSORT)
        sort.vsnray_ref_sort_bytes.argtypes = [ctypes.c_uint32]
        sort.vsnray_ref_sort_bytes.restype = ctypes.c_size_t
        sort.vsnray_ref_sort.argtypes = [vp, ctypes.c_size_t, vp, ctypes.c_uint32, vp]
        sort.vsnray_ref_sort.restype = ctypes.c_int
        self.lbvh = (found, sort)
        return self.lbvh

    def _launch_fn(self, fn, count, args, what):
        block = 1024   # the build's num_threads
        ptrs = (ctypes.c_void_p * len(args))(*[ctypes.addressof(a) for a in args])
        stream = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        self._check(self.cu.cuLaunchKernel(fn, (count + block - 1) // block, 1, 1, block, 1, 1, 0, stream, ptrs, None),
                    what)

    def lbvh_buffers(self, n):
        """Device buffers of one build of n >= 2 triangles: the build's own arrays
        (bounds, centroids, prim refs, construction nodes), the output tree (2n - 1
        nodes, n triangles, n indices) and the sort's temporary storage.  Allocated once,
        outside the timed build (the reference allocates them on every build)."""
        if n < 2:
            raise ValueError("the timed build takes at least two triangles")
        torch = self.torch
        _, sort = self._lbvh_kernels()
        temp_bytes = int(sort.vsnray_ref_sort_bytes(n))
        if temp_bytes == 0:
            raise RuntimeError("cub::DeviceMergeSort::StableSortKeys: no temporary storage size")

        def buf(nbytes):
            return torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device=self.dev)

        flt = np.finfo(np.float32).max
        invalid = np.tile(np.array([flt, flt, flt, -flt, -flt, -flt], np.float32), 2)   # aabb::invalidate
        assert self.size_aabb == 24 and self.size_prim_ref == 8
        return {"n": n, "invalid": torch.from_numpy(invalid.view(np.uint8)).to(self.dev),
                "bounds": buf(2 * self.size_aabb), "prim_bounds": buf(n * self.size_aabb),
                "centroids": buf(n * 12), "prim_refs": buf(n * self.size_prim_ref),
                "inner": buf((n - 1) * self.size_node), "leaves": buf(n * self.size_node),
                "nodes": buf((2 * n - 1) * 32), "prims": buf(n * 44), "indices": buf(n * 4),
                "temp": buf(temp_bytes), "temp_bytes": temp_bytes}

    def lbvh_build(self, tris, b):
        """lbvh_builder::build(cuda_index_bvh<basic_triangle<3, float>>{}, tris, n) on the
        current stream: the reference's kernels in its order with its launch shape
        (1024-thread blocks), CUB's stable merge sort of the prim refs, the zero fill of
        the node array its resize does, the device copy of the primitives and the index
        sequence; into the buffers of lbvh_buffers(n)."""
        fns, sort = self._lbvh_kernels()
        vp, n = ctypes.c_void_p, b["n"]

        def p(name):
            return vp(b[name].data_ptr())

        bounds = b["bounds"]
        bounds.copy_(b["invalid"])
        scene_b, centroid_b = vp(bounds.data_ptr()), vp(bounds.data_ptr() + self.size_aabb)
        self._launch_fn(fns["compute_bounds_and_centroids"], n,
                        [p("prim_bounds"), p("centroids"), scene_b, centroid_b, vp(tris.data_ptr()), ctypes.c_int(n)],
                        "compute_bounds_and_centroids")
        self._launch_fn(fns["assign_morton_codes"], n, [p("prim_refs"), p("centroids"), centroid_b, ctypes.c_int(n)],
                        "assign_morton_codes")
        stream = vp(self.torch.cuda.current_stream().cuda_stream)
        err = sort.vsnray_ref_sort(p("temp"), b["temp_bytes"], p("prim_refs"), n, stream)
        if err != 0:
            raise RuntimeError(f"cub::DeviceMergeSort::StableSortKeys: cudaError {err}")
        self._launch_fn(fns["init_nodes"], n - 1, [p("inner"), ctypes.c_size_t(n - 1)], "init_nodes")
        self._launch_fn(fns["init_nodes"], n, [p("leaves"), ctypes.c_size_t(n)], "init_nodes")
        self._launch_fn(fns["build_hierarchy"], n, [p("inner"), p("leaves"), p("prim_refs"), ctypes.c_int(n)],
                        "build_hierarchy")
        # tree.nodes().resize(2n - 1) value-initialises the nodes (zeros); set_leaf leaves
        # a leaf's two ordered-traversal bytes as they were, so they stay zero
        b["nodes"].zero_()
        self._launch_fn(fns["assign_node_bounds"], n,
                        [p("inner"), p("leaves"), p("prim_bounds"), p("prim_refs"), ctypes.c_int(n)],
                        "assign_node_bounds")
        self._launch_fn(fns["collapse"], n, [p("nodes"), p("inner"), p("leaves"), p("prim_refs"), ctypes.c_int(n)],
                        "collapse")
        b["prims"][:n * 44].copy_(tris.reshape(-1)[:n * 44])
        self._launch_fn(fns["sequence"], n, [p("indices"), ctypes.c_uint(n)], "sequence")
        return b["nodes"][:(2 * n - 1) * 32], b["indices"][:n * 4]
