// C ABI of include/visionaray_gb300/gbrt.h: argument checks, ownership, streams.

#include "api_internal.h"

#include <algorithm>
#include <new>
#include <vector>

namespace gbrt {

constexpr uint32_t kMaxPrims = 1u << 29;   // keeps every Karras index computation in int range

gbrt_status fail(gbrt_context* ctx, gbrt_status st, std::string const& what)
{
    if (ctx) ctx->last_error = what;
    return st;
}

gbrt_status check_cuda(gbrt_context* ctx, cudaError_t err, const char* where)
{
    std::string msg = std::string(where) + ": " + cudaGetErrorName(err) + " (" + cudaGetErrorString(err) + ")";
    return fail(ctx, err == cudaErrorMemoryAllocation ? GBRT_ERR_OUT_OF_MEMORY : GBRT_ERR_CUDA, msg);
}

gbrt_status ensure_scratch(gbrt_context* ctx, size_t bytes)
{
    if (ctx->scratch_bytes >= bytes) return GBRT_OK;
    if (ctx->scratch)
    {
        // the old scratch may still be read by queued work
        GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        GBRT_CUDA(ctx, cudaFree(ctx->scratch));
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
    }
    size_t grow = std::max(bytes, size_t(1) << 20);
    GBRT_CUDA(ctx, cudaMalloc(&ctx->scratch, grow));
    ctx->scratch_bytes = grow;
    return GBRT_OK;
}

namespace {

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

void free_bvh_arrays(gbrt_bvh* b)
{
    free_wide_nodes(b);
    cudaFree(b->nodes);
    cudaFree(b->tris);
    cudaFree(b->sorted_codes);
    cudaFree(b->sorted_ids);
    b->nodes = nullptr;
    b->tris = nullptr;
    b->sorted_codes = nullptr;
    b->sorted_ids = nullptr;
}

gbrt_status ensure_trace_scratch(gbrt_context* ctx, uint32_t n)
{
    size_t bytes = trace_scratch_bytes(n);
    if (ctx->trace_scratch_bytes >= bytes) return GBRT_OK;
    if (ctx->trace_scratch)
    {
        GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        GBRT_CUDA(ctx, cudaFree(ctx->trace_scratch));
        ctx->trace_scratch = nullptr;
        ctx->trace_scratch_bytes = 0;
    }
    GBRT_CUDA(ctx, cudaMalloc(&ctx->trace_scratch, bytes));
    ctx->trace_scratch_bytes = bytes;
    return GBRT_OK;
}

gbrt_status ensure_slots(gbrt_context* ctx, size_t rays_per_slot)
{
    if (ctx->slot_capacity >= rays_per_slot) return GBRT_OK;
    for (int k = 0; k < gbrt_context::kSlots; ++k)
    {
        if (ctx->slot_stream[k]) GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->slot_stream[k]));
        cudaFree(ctx->slot_rays[k]);
        cudaFree(ctx->slot_hits[k]);
        cudaFree(ctx->slot_trace_scratch[k]);
        ctx->slot_rays[k] = ctx->slot_hits[k] = ctx->slot_trace_scratch[k] = nullptr;
    }
    ctx->slot_capacity = 0;
    ctx->slot_trace_scratch_bytes = 0;
    for (int k = 0; k < gbrt_context::kSlots; ++k)
    {
        if (!ctx->slot_stream[k]) GBRT_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->slot_stream[k], cudaStreamNonBlocking));
        if (!ctx->slot_done[k]) GBRT_CUDA(ctx, cudaEventCreateWithFlags(&ctx->slot_done[k], cudaEventDisableTiming));
        GBRT_CUDA(ctx, cudaMalloc(&ctx->slot_rays[k], rays_per_slot * sizeof(gbrt_ray)));
        GBRT_CUDA(ctx, cudaMalloc(&ctx->slot_hits[k], rays_per_slot * sizeof(gbrt_hit)));
        GBRT_CUDA(ctx, cudaMalloc(&ctx->slot_trace_scratch[k], trace_scratch_bytes(uint32_t(rays_per_slot))));
    }
    ctx->slot_capacity = rays_per_slot;
    ctx->slot_trace_scratch_bytes = trace_scratch_bytes(uint32_t(rays_per_slot));
    return GBRT_OK;
}

// The chunk sizes of a host-buffer query of n rays with full chunks of c: a quarter
// chunk first and last (the copy-in before the first traversal and the copy-out after
// the last one overlap nothing), full chunks between.  Queries of at most c rays are
// split into a quarter, a half and a quarter of themselves; at most c / 4 rays, one
// chunk.
std::vector<size_t> host_chunks(size_t n, size_t c)
{
    std::vector<size_t> out;
    const size_t q = c / 4;
    if (n <= q)
    {
        out.push_back(n);
        return out;
    }
    if (n <= c)
    {
        const size_t a = n / 4;
        out.push_back(a);
        out.push_back(n - 2 * a);
        out.push_back(a);
        return out;
    }
    out.push_back(q);
    size_t rest = n - q;
    while (rest > c + q)
    {
        out.push_back(c);
        rest -= c;
    }
    if (rest > q)
    {
        out.push_back(rest - q);
        out.push_back(q);
    }
    else
    {
        out.push_back(rest);
    }
    return out;
}

// Host-buffer trace: chunks alternate between the slots, each on its own stream, so
// the copy-in of one chunk overlaps the traversal and copy-out of the others.
gbrt_status trace_host(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_ray const* h_rays, uint32_t n, gbrt_hit* h_hits,
                       bool any_hit)
{
    if (n == 0) return GBRT_OK;
    const std::vector<size_t> sizes = host_chunks(n, ctx->host_chunk);
    const size_t chunk = *std::max_element(sizes.begin(), sizes.end());   // rays per slot
    gbrt_status st = ensure_slots(ctx, chunk);
    if (st != GBRT_OK) return st;
    // work queued on the context stream (e.g. the build) must finish first
    cudaEvent_t ready;
    GBRT_CUDA(ctx, cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    GBRT_CUDA(ctx, cudaEventRecord(ready, ctx->stream));
    for (int k = 0; k < gbrt_context::kSlots; ++k) GBRT_CUDA(ctx, cudaStreamWaitEvent(ctx->slot_stream[k], ready, 0));
    size_t b = 0;
    for (size_t c = 0; c < sizes.size(); b += sizes[c], ++c)
    {
        int k = int(c % gbrt_context::kSlots);
        cudaStream_t s = ctx->slot_stream[k];
        uint32_t m = uint32_t(sizes[c]);
        GBRT_CUDA(ctx, cudaMemcpyAsync(ctx->slot_rays[k], h_rays + b, size_t(m) * sizeof(gbrt_ray),
                                       cudaMemcpyHostToDevice, s));
        st = trace(ctx, bvh, static_cast<gbrt_ray*>(ctx->slot_rays[k]), m, static_cast<gbrt_hit*>(ctx->slot_hits[k]),
                   any_hit, s, ctx->slot_trace_scratch[k], ctx->slot_trace_scratch_bytes);
        if (st != GBRT_OK) return st;
        GBRT_CUDA(ctx, cudaMemcpyAsync(h_hits + b, ctx->slot_hits[k], size_t(m) * sizeof(gbrt_hit),
                                       cudaMemcpyDeviceToHost, s));
    }
    for (int k = 0; k < gbrt_context::kSlots; ++k) GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->slot_stream[k]));
    cudaEventDestroy(ready);
    return GBRT_OK;
}

gbrt_status check_trace_args(gbrt_context* ctx, gbrt_bvh const* bvh, const void* rays, uint32_t n, const void* hits)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!bvh) return fail(ctx, GBRT_ERR_INVALID_ARG, "trace: null bvh");
    if (n > 0 && (!rays || !hits)) return fail(ctx, GBRT_ERR_INVALID_ARG, "trace: null ray or hit buffer");
    return GBRT_OK;
}

} // namespace
} // namespace gbrt

using namespace gbrt;

extern "C" {

int gbrt_abi_version(void) { return GBRT_ABI_VERSION; }

gbrt_status gbrt_context_create(int device, void* stream, gbrt_context** out)
{
    if (!out) return GBRT_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return GBRT_ERR_INVALID_ARG;
    auto* ctx = new (std::nothrow) gbrt_context;
    if (!ctx) return GBRT_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    ctx->stream = static_cast<cudaStream_t>(stream);
    device_guard g(device);
    if (cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaMalloc(&ctx->d_status, sizeof(uint32_t)) != cudaSuccess ||
        cudaMemset(ctx->d_status, 0, sizeof(uint32_t)) != cudaSuccess)
    {
        cudaFree(ctx->d_status);
        delete ctx;
        return GBRT_ERR_CUDA;
    }
    *out = ctx;
    return GBRT_OK;
}

gbrt_status gbrt_context_destroy(gbrt_context* ctx)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    {
        device_guard g(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        for (int k = 0; k < gbrt_context::kSlots; ++k)
        {
            if (ctx->slot_stream[k])
            {
                cudaStreamSynchronize(ctx->slot_stream[k]);
                cudaStreamDestroy(ctx->slot_stream[k]);
            }
            if (ctx->slot_done[k]) cudaEventDestroy(ctx->slot_done[k]);
            cudaFree(ctx->slot_rays[k]);
            cudaFree(ctx->slot_hits[k]);
            cudaFree(ctx->slot_trace_scratch[k]);
        }
        for (cudaEvent_t& e : ctx->timing_events)
            if (e) cudaEventDestroy(e);
        cudaFree(ctx->trace_scratch);
        cudaFree(ctx->scratch);
        cudaFree(ctx->pt_scratch);
        cudaFree(ctx->d_trig);
        cudaFree(ctx->d_status);
    }
    delete ctx;
    return GBRT_OK;
}

gbrt_status gbrt_context_set_trace_flags(gbrt_context* ctx, uint32_t flags)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (flags & ~(GBRT_TRACE_SORT_RAYS | GBRT_TRACE_WIDE_NODES | GBRT_TRACE_PERSISTENT | GBRT_TRACE_COMPRESSED_NODES |
                  GBRT_TRACE_WIDE8_NODES))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "set_trace_flags: unknown flag");
    ctx->trace_flags = flags;
    return GBRT_OK;
}

gbrt_status gbrt_context_set_trace_refill(gbrt_context* ctx, uint32_t min_idle_lanes)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (min_idle_lanes < 1 || min_idle_lanes > 32)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "set_trace_refill: 1 to 32 lanes");
    ctx->trace_refill = min_idle_lanes;
    return GBRT_OK;
}

gbrt_status gbrt_context_set_host_chunk(gbrt_context* ctx, uint32_t rays)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (rays < (1u << 16) || rays > (1u << 26))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "set_host_chunk: 2^16 to 2^26 rays");
    ctx->host_chunk = rays;
    return GBRT_OK;
}

gbrt_status gbrt_context_set_stream(gbrt_context* ctx, void* stream)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    ctx->stream = static_cast<cudaStream_t>(stream);
    return GBRT_OK;
}

gbrt_status gbrt_context_synchronize(gbrt_context* ctx)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    device_guard g(ctx->device);
    uint32_t status = 0;
    GBRT_CUDA(ctx, cudaMemcpyAsync(&status, ctx->d_status, 4, cudaMemcpyDeviceToHost, ctx->stream));
    GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (status != 0)
    {
        GBRT_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, 4, ctx->stream));
        GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (status & kStatusStackOverflow)
            return fail(ctx, GBRT_ERR_STACK_OVERFLOW, "a traversal stack overflowed; results are incomplete");
        if (status & kStatusBadIndex)
            return fail(ctx, GBRT_ERR_CUDA, "a kernel met an out-of-range node or triangle index and skipped it");
        return fail(ctx, GBRT_ERR_CUDA, "a kernel reported unknown status bits " + std::to_string(status));
    }
    return GBRT_OK;
}

gbrt_status gbrt_context_set_kernel_timing(gbrt_context* ctx, int enable)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    device_guard g(ctx->device);
    if (enable && !ctx->timing_events[0])
        for (cudaEvent_t& e : ctx->timing_events)
            GBRT_CUDA(ctx, cudaEventCreate(&e));
    ctx->kernel_timing = enable != 0;
    ctx->timing_count = 0;
    return GBRT_OK;
}

gbrt_status gbrt_context_kernel_times(gbrt_context* ctx, float* out_ms, uint32_t max, uint32_t* count)
{
    if (!ctx || !count || (max > 0 && !out_ms)) return GBRT_ERR_INVALID_ARG;
    device_guard g(ctx->device);
    const uint32_t ring = gbrt_context::kTimingRing;
    uint32_t m = ctx->timing_count < ring ? ctx->timing_count : ring;
    if (m > max) m = max;
    for (uint32_t j = 0; j < m; ++j)
    {
        const uint32_t k = (ctx->timing_count - m + j) % ring;
        GBRT_CUDA(ctx, cudaEventSynchronize(ctx->timing_events[2 * k + 1]));
        GBRT_CUDA(ctx, cudaEventElapsedTime(&out_ms[j], ctx->timing_events[2 * k], ctx->timing_events[2 * k + 1]));
    }
    *count = m;
    ctx->timing_count = 0;
    return GBRT_OK;
}

const char* gbrt_last_error(gbrt_context const* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

uint64_t gbrt_kernel_launch_count(gbrt_context const* ctx) { return ctx ? ctx->launches : 0; }

gbrt_status gbrt_bvh_build_lbvh(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n, gbrt_bvh** out)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!out) return fail(ctx, GBRT_ERR_INVALID_ARG, "build_lbvh: null output");
    *out = nullptr;
    if (n > 0 && !d_tris) return fail(ctx, GBRT_ERR_INVALID_ARG, "build_lbvh: null triangles");
    if (n > kMaxPrims) return fail(ctx, GBRT_ERR_TOO_LARGE, "build_lbvh: more than 2^29 triangles");
    if ((reinterpret_cast<uintptr_t>(d_tris) & 3u) != 0)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "build_lbvh: triangles not 4-byte aligned");
    device_guard g(ctx->device);
    auto* bvh = new (std::nothrow) gbrt_bvh;
    if (!bvh) return fail(ctx, GBRT_ERR_OUT_OF_MEMORY, "build_lbvh: host allocation");
    bvh->device = ctx->device;
    gbrt_status st = build_lbvh(ctx, d_tris, n, bvh);
    if (st != GBRT_OK)
    {
        cudaStreamSynchronize(ctx->stream);
        free_bvh_arrays(bvh);
        delete bvh;
        return st;
    }
    *out = bvh;
    return GBRT_OK;
}

gbrt_status gbrt_bvh_build_ploc(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n, gbrt_bvh** out)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!out) return fail(ctx, GBRT_ERR_INVALID_ARG, "build_ploc: null output");
    *out = nullptr;
    if (n > 0 && !d_tris) return fail(ctx, GBRT_ERR_INVALID_ARG, "build_ploc: null triangles");
    if (n > kMaxPrims) return fail(ctx, GBRT_ERR_TOO_LARGE, "build_ploc: more than 2^29 triangles");
    if ((reinterpret_cast<uintptr_t>(d_tris) & 3u) != 0)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "build_ploc: triangles not 4-byte aligned");
    device_guard g(ctx->device);
    auto* bvh = new (std::nothrow) gbrt_bvh;
    if (!bvh) return fail(ctx, GBRT_ERR_OUT_OF_MEMORY, "build_ploc: host allocation");
    bvh->device = ctx->device;
    gbrt_status st = build_ploc(ctx, d_tris, n, bvh);
    if (st != GBRT_OK)
    {
        cudaStreamSynchronize(ctx->stream);
        free_bvh_arrays(bvh);
        delete bvh;
        return st;
    }
    *out = bvh;
    return GBRT_OK;
}

gbrt_status gbrt_bvh_build_lbvh_host(gbrt_context* ctx, gbrt_triangle const* h_tris, uint32_t n, gbrt_bvh** out)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!out) return fail(ctx, GBRT_ERR_INVALID_ARG, "build_lbvh_host: null output");
    if (n > 0 && !h_tris) return fail(ctx, GBRT_ERR_INVALID_ARG, "build_lbvh_host: null triangles");
    if (n > kMaxPrims) return fail(ctx, GBRT_ERR_TOO_LARGE, "build_lbvh_host: more than 2^29 triangles");
    device_guard g(ctx->device);
    gbrt_triangle* d = nullptr;
    if (n > 0)
    {
        GBRT_CUDA(ctx, cudaMalloc(&d, size_t(n) * sizeof(gbrt_triangle)));
        cudaError_t e = cudaMemcpyAsync(d, h_tris, size_t(n) * sizeof(gbrt_triangle), cudaMemcpyHostToDevice,
                                        ctx->stream);
        if (e != cudaSuccess)
        {
            cudaFree(d);
            return check_cuda(ctx, e, "build_lbvh_host: copy");
        }
    }
    gbrt_status st = gbrt_bvh_build_lbvh(ctx, d, n, out);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(d);
    return st;
}

gbrt_status gbrt_bvh_upload_bvh2_host(gbrt_context* ctx, gbrt_bvh_node const* nodes, uint32_t num_nodes,
                                      uint32_t const* indices, uint32_t num_indices, gbrt_triangle const* tris,
                                      uint32_t num_tris, gbrt_bvh** out)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!out) return fail(ctx, GBRT_ERR_INVALID_ARG, "upload_bvh2: null output");
    *out = nullptr;
    if ((num_nodes && !nodes) || (num_indices && !indices) || (num_tris && !tris))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "upload_bvh2: null array");
    if (num_tris > kMaxPrims || num_indices > kMaxPrims)
        return fail(ctx, GBRT_ERR_TOO_LARGE, "upload_bvh2: more than 2^29 primitives");
    device_guard g(ctx->device);
    auto* bvh = new (std::nothrow) gbrt_bvh;
    if (!bvh) return fail(ctx, GBRT_ERR_OUT_OF_MEMORY, "upload_bvh2: host allocation");
    bvh->device = ctx->device;
    gbrt_status st = upload_bvh2(ctx, nodes, num_nodes, indices, num_indices, tris, num_tris, bvh);
    if (st != GBRT_OK)
    {
        free_bvh_arrays(bvh);
        delete bvh;
        return st;
    }
    *out = bvh;
    return GBRT_OK;
}

gbrt_status gbrt_bvh_destroy(gbrt_bvh* bvh)
{
    if (!bvh) return GBRT_ERR_INVALID_ARG;
    device_guard g(bvh->device);
    free_bvh_arrays(bvh);
    delete bvh;
    return GBRT_OK;
}

gbrt_status gbrt_bvh_counts(gbrt_bvh const* bvh, uint32_t* num_prims, uint32_t* num_bvh2_nodes, uint32_t* depth_bound)
{
    if (!bvh) return GBRT_ERR_INVALID_ARG;
    if (num_prims) *num_prims = bvh->num_prims;
    if (num_bvh2_nodes) *num_bvh2_nodes = bvh->num_prims > 0 ? 2 * bvh->num_prims - 1 : 0;
    if (depth_bound) *depth_bound = bvh->height;
    return GBRT_OK;
}

gbrt_status gbrt_bvh_rebuild_lbvh(gbrt_context* ctx, gbrt_bvh* bvh, gbrt_triangle const* d_tris, uint32_t n)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!bvh || (n > 0 && !d_tris)) return fail(ctx, GBRT_ERR_INVALID_ARG, "rebuild_lbvh: null argument");
    if (bvh->kind != bvh_kind::lbvh) return fail(ctx, GBRT_ERR_INVALID_ARG, "rebuild_lbvh: not an LBVH");
    if (n != bvh->num_prims)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "rebuild_lbvh: triangle count differs from the tree's");
    if (bvh->device != ctx->device) return fail(ctx, GBRT_ERR_INVALID_ARG, "rebuild_lbvh: tree on another device");
    if ((reinterpret_cast<uintptr_t>(d_tris) & 3u) != 0)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "rebuild_lbvh: triangles not 4-byte aligned");
    device_guard g(ctx->device);
    return build_lbvh(ctx, d_tris, n, bvh);
}

gbrt_status gbrt_bvh_refit(gbrt_context* ctx, gbrt_bvh* bvh, gbrt_triangle const* d_tris, uint32_t n)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!bvh || (n > 0 && !d_tris)) return fail(ctx, GBRT_ERR_INVALID_ARG, "refit: null argument");
    if (bvh->kind != bvh_kind::lbvh && bvh->kind != bvh_kind::ploc)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "refit: not a GPU-built tree");
    if (n != bvh->num_prims) return fail(ctx, GBRT_ERR_INVALID_ARG, "refit: triangle count differs from the build");
    device_guard g(ctx->device);
    return refit_lbvh(ctx, bvh, d_tris);
}

gbrt_status gbrt_bvh_export_bvh2(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_bvh_node* d_nodes, uint32_t* d_indices)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!bvh || (bvh->num_prims > 0 && (!d_nodes || !d_indices)))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "export_bvh2: null argument");
    if (!aligned16(d_nodes)) return fail(ctx, GBRT_ERR_INVALID_ARG, "export_bvh2: nodes not 16-byte aligned");
    device_guard g(ctx->device);
    return export_bvh2(ctx, bvh, d_nodes, d_indices);
}

gbrt_status gbrt_bvh_morton_codes(gbrt_context* ctx, gbrt_bvh const* bvh, uint32_t* d_codes)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!bvh || (bvh->num_prims > 0 && !d_codes)) return fail(ctx, GBRT_ERR_INVALID_ARG, "morton_codes: null argument");
    device_guard g(ctx->device);
    return morton_codes_input_order(ctx, bvh, d_codes);
}

static gbrt_status trace_device(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_ray const* d_rays, uint32_t n,
                                gbrt_hit* d_hits, bool any_hit)
{
    gbrt_status st = check_trace_args(ctx, bvh, d_rays, n, d_hits);
    if (st != GBRT_OK) return st;
    if (!aligned16(d_rays) || !aligned16(d_hits))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "trace: ray and hit buffers must be 16-byte aligned");
    device_guard g(ctx->device);
    if (ctx->trace_flags & (GBRT_TRACE_SORT_RAYS | GBRT_TRACE_PERSISTENT))
    {
        gbrt_status s2 = ensure_trace_scratch(ctx, n);
        if (s2 != GBRT_OK) return s2;
    }
    return trace(ctx, bvh, d_rays, n, d_hits, any_hit, ctx->stream, ctx->trace_scratch, ctx->trace_scratch_bytes);
}

gbrt_status gbrt_trace_closest_hit(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_ray const* d_rays, uint32_t n,
                                   gbrt_hit* d_hits)
{
    return trace_device(ctx, bvh, d_rays, n, d_hits, false);
}

gbrt_status gbrt_trace_any_hit(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_ray const* d_rays, uint32_t n,
                               gbrt_hit* d_hits)
{
    return trace_device(ctx, bvh, d_rays, n, d_hits, true);
}

gbrt_status gbrt_trace_closest_hit_host(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_ray const* h_rays, uint32_t n,
                                        gbrt_hit* h_hits)
{
    gbrt_status st = check_trace_args(ctx, bvh, h_rays, n, h_hits);
    if (st != GBRT_OK) return st;
    device_guard g(ctx->device);
    return trace_host(ctx, bvh, h_rays, n, h_hits, false);
}

gbrt_status gbrt_trace_any_hit_host(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_ray const* h_rays, uint32_t n,
                                    gbrt_hit* h_hits)
{
    gbrt_status st = check_trace_args(ctx, bvh, h_rays, n, h_hits);
    if (st != GBRT_OK) return st;
    device_guard g(ctx->device);
    return trace_host(ctx, bvh, h_rays, n, h_hits, true);
}

} // extern "C"
