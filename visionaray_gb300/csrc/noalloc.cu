// gbrt_bvh_build_lbvh_noalloc: the GPU LBVH build for callers that cannot allocate
// device memory.
//
// Who cannot allocate: a host application that owns the whole device-memory budget
// and hands libraries only the buffers they return results in (a renderer or game
// engine with its own pre-reserved VRAM pool, a plugin inside such a host), and
// per-frame rebuild loops where a cudaMalloc/cudaFree pair would implicitly
// synchronise the device and stall the frame.  gbrt_bvh_build_lbvh allocates the tree
// and grows a context scratch buffer; this entry point does neither.  The caller
// passes the triangles and the two output arrays (the reference's cuda_index_bvh node
// layout); every temporary lives in one file-scope __device__ array of fixed size,
// which each GPU that loads this library holds until the process exits.
//
// Limits and sharing:
//   - at most kNoAllocMaxPrims (65,536) triangles; larger inputs are rejected with
//     GBRT_ERR_TOO_LARGE before any GPU work;
//   - the array holds about 10 MB per device;
//   - every call on a device uses the same array and leaves its contents behind; the
//     build clears what must start at zero (node records, arrival counters, parent
//     links, bounds words) itself, so calls that follow one another on a stream are
//     independent, but calls whose executions overlap on the GPU (two streams, two
//     host threads) race on the array and give wrong trees;
//   - the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, which may load the module on that device); make that
//     first call before any stream capture begins.

#include "api_internal.h"

#include <mutex>

namespace gbrt {
namespace {

constexpr uint32_t kNoAllocMaxPrims = 65536;
constexpr size_t kNoAllocScratchBytes = lbvh_scratch_layout_for(kNoAllocMaxPrims).total;
constexpr int kMaxDevices = 64;

// Every temporary of a build of up to kNoAllocMaxPrims triangles.  Host code only
// sees a stand-in symbol: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_address[kMaxDevices] = {};

// Makes ctx->device current for its lifetime and restores the caller's device; both
// switches are checked, so a failure is reported instead of running on another device.
struct checked_device
{
    int prev = -1;
    bool switched = false;
    cudaError_t error = cudaSuccess;

    explicit checked_device(int dev)
    {
        error = cudaGetDevice(&prev);
        if (error == cudaSuccess && prev != dev)
        {
            error = cudaSetDevice(dev);
            switched = error == cudaSuccess;
        }
    }
    // Restores the caller's device; the status of that switch back.
    cudaError_t restore()
    {
        if (!switched) return cudaSuccess;
        switched = false;
        return cudaSetDevice(prev);
    }
    ~checked_device() { restore(); }
};

// Once per device, with that device current: the array's device address.
gbrt_status scratch_address(gbrt_context* ctx, void** out)
{
    if (ctx->device < 0 || ctx->device >= kMaxDevices)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "build_lbvh_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_address[ctx->device])
    {
        checked_device dev(ctx->device);
        if (dev.error != cudaSuccess) return check_cuda(ctx, dev.error, "build_lbvh_noalloc: selecting the device");
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return check_cuda(ctx, e, "build_lbvh_noalloc: cudaGetSymbolAddress");
        e = dev.restore();
        if (e != cudaSuccess) return check_cuda(ctx, e, "build_lbvh_noalloc: restoring the caller's device");
        g_scratch_address[ctx->device] = p;
    }
    *out = g_scratch_address[ctx->device];
    return GBRT_OK;
}

} // namespace
} // namespace gbrt

extern "C" gbrt_status gbrt_bvh_build_lbvh_noalloc(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n,
                                                   gbrt_bvh_node* d_nodes, uint32_t* d_indices)
{
    using namespace gbrt;
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (n > kNoAllocMaxPrims)
        return fail(ctx, GBRT_ERR_TOO_LARGE,
                    "build_lbvh_noalloc: " + std::to_string(n) + " triangles exceed the fixed scratch limit of " +
                        std::to_string(kNoAllocMaxPrims) + "; use gbrt_bvh_build_lbvh");
    if (n == 0) return GBRT_OK;
    if (!d_tris || !d_nodes || !d_indices)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "build_lbvh_noalloc: null triangle, node or index buffer");
    if ((reinterpret_cast<uintptr_t>(d_tris) & 3u) != 0 || (reinterpret_cast<uintptr_t>(d_nodes) & 15u) != 0 ||
        (reinterpret_cast<uintptr_t>(d_indices) & 3u) != 0)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "build_lbvh_noalloc: misaligned buffer");
    void* scratch = nullptr;
    gbrt_status st = scratch_address(ctx, &scratch);
    if (st != GBRT_OK) return st;
    checked_device dev(ctx->device);
    if (dev.error != cudaSuccess) return check_cuda(ctx, dev.error, "build_lbvh_noalloc: selecting the device");
    st = build_lbvh_in_scratch(ctx, d_tris, n, scratch, kNoAllocScratchBytes, d_nodes, d_indices);
    cudaError_t e = dev.restore();
    if (st == GBRT_OK && e != cudaSuccess)
        return check_cuda(ctx, e, "build_lbvh_noalloc: restoring the caller's device");
    return st;
}
