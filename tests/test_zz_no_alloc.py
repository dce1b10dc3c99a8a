"""gbrt_bvh_build_lbvh_noalloc: the LBVH build for callers that cannot allocate device
memory (hosts that own the whole device-memory budget and give a library only its
output buffers; per-frame rebuild loops where cudaMalloc/cudaFree would synchronise
the device).  Its temporaries live in a fixed device array inside the library, so it
must produce exactly the tree of the allocating entry point
(gbrt_bvh_build_lbvh + gbrt_bvh_export_bvh2) -- checked here through the C ABI on two
calls in a row, the second on a smaller, different scene so that anything the first
call left in the shared array would show.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

import visionaray_gb300 as vg
from visionaray_gb300 import runtime, scenes
from visionaray_gb300.types import BVH_NODE

pytestmark = pytest.mark.gpu

MAX_PRIMS = 65536   # the array's documented limit


def noalloc_build(ctx, tris, free_bytes=None):
    """Calls the C ABI directly: caller-owned input and output device buffers only.
    With `free_bytes` (a list), appends the device's free memory just before and just
    after the call, with every buffer already allocated."""
    n = len(tris)
    d_tris = vg.as_device_bytes(tris)
    d_nodes = torch.empty((2 * n - 1) * 32, dtype=torch.uint8, device="cuda")
    d_idx = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    if free_bytes is not None:
        free_bytes.append(torch.cuda.mem_get_info()[0])
    st = ctx.lib.gbrt_bvh_build_lbvh_noalloc(ctx.h, ctypes.c_void_p(d_tris.data_ptr()), n,
                                             ctypes.c_void_p(d_nodes.data_ptr()), ctypes.c_void_p(d_idx.data_ptr()))
    ctx.check(st)
    ctx.synchronize()
    if free_bytes is not None:
        free_bytes.append(torch.cuda.mem_get_info()[0])
    return d_nodes.cpu().numpy().view(BVH_NODE), d_idx.cpu().numpy().view(np.uint32)


def allocating_build(ctx, tris):
    bvh = vg.lbvh_builder(ctx).build(vg.as_device_bytes(tris))
    return bvh.export_bvh2()


def assert_same(a, b):
    (na, ia), (nb, ib) = a, b
    assert len(na) == len(nb)
    assert np.array_equal(na["first"], nb["first"]) and np.array_equal(na["num_prims"], nb["num_prims"])
    assert (na["bbox_min"] == nb["bbox_min"]).all() and (na["bbox_max"] == nb["bbox_max"]).all()
    assert np.array_equal(ia, ib)


def test_noalloc_build_matches_allocating_build_twice():
    ctx = vg.Context(0)
    first = scenes.soup(MAX_PRIMS, seed=31)              # the largest accepted input
    second = scenes.heightfield(grid=64, seed=5)          # 8,192 triangles, other scene
    for tris in (first, second):
        assert_same(noalloc_build(ctx, tris), allocating_build(ctx, tris))


@pytest.mark.parametrize("n", [1, 2, 3])
def test_noalloc_build_of_the_smallest_scenes(n):
    """One triangle (a single leaf: its own code path), two and three triangles."""
    ctx = vg.Context(0)
    tris = scenes.soup(n, seed=40 + n)
    for _ in range(2):
        assert_same(noalloc_build(ctx, tris), allocating_build(ctx, tris))


def test_noalloc_build_allocates_no_device_memory():
    """On a context that has already built trees (and after the array's device address
    was looked up), a call leaves the device's free memory unchanged."""
    ctx = vg.Context(0)
    tris = scenes.soup(20000, seed=44)
    expect = allocating_build(ctx, tris)
    assert_same(noalloc_build(ctx, tris), expect)      # first call: the set-up
    free = []
    for _ in range(2):
        assert_same(noalloc_build(ctx, tris, free_bytes=free), expect)
    assert free[0] == free[1] and free[2] == free[3], free


def test_noalloc_rejects_inputs_above_the_limit():
    ctx = vg.Context(0)
    st = ctx.lib.gbrt_bvh_build_lbvh_noalloc(ctx.h, ctypes.c_void_p(16), MAX_PRIMS + 1, ctypes.c_void_p(16),
                                             ctypes.c_void_p(16))
    assert st == 6   # GBRT_ERR_TOO_LARGE, before any GPU work
    assert b"65536" in ctx.lib.gbrt_last_error(ctx.h)
    assert runtime.STATUS[st] == "GBRT_ERR_TOO_LARGE"
