// closest_hit / any_hit ray queries over the node-pair BVH: one thread per ray over
// the shared traversal core (traverse_core.cuh), 128-bit ray loads and hit stores.

#include "traverse_core.cuh"

namespace gbrt {
namespace {

constexpr int kTraceBlock = 128;

template <bool AnyHit>
__global__ void __launch_bounds__(kTraceBlock) trace_rays(const bvh2_node* __restrict__ nodes,
                                                          const tri48* __restrict__ tris, int32_t root,
                                                          int32_t num_inner, int32_t num_tris,
                                                          const gbrt_ray* __restrict__ rays, uint32_t n,
                                                          gbrt_hit* __restrict__ hits,
                                                          uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kTraceBlock + threadIdx.x;
    if (i >= n) return;

    float4 r0 = ldg4(&rays[i]);
    float4 r1 = ldg4(reinterpret_cast<const float4*>(&rays[i]) + 1);
    trace_result h = traverse_bvh<AnyHit>(nodes, tris, root, num_inner, num_tris, { r0.x, r0.y, r0.z },
                                          { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    uint32_t prim = h.tri >= 0 ? __float_as_uint(ldg4(&tris[h.tri].t0).w) : GBRT_NO_HIT;
    reinterpret_cast<uint4*>(hits)[i] =
        make_uint4(prim, __float_as_uint(h.t), __float_as_uint(h.u), __float_as_uint(h.v));
}

__global__ void __launch_bounds__(kTraceBlock) write_misses(gbrt_hit* __restrict__ hits, uint32_t n)
{
    uint32_t i = blockIdx.x * kTraceBlock + threadIdx.x;
    if (i < n) reinterpret_cast<uint4*>(hits)[i] = make_uint4(GBRT_NO_HIT, __float_as_uint(FLT_MAX), 0u, 0u);
}

} // namespace

gbrt_status trace(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_ray const* d_rays, uint32_t n, gbrt_hit* d_hits,
                  bool any_hit, cudaStream_t stream)
{
    if (n == 0) return GBRT_OK;
    uint32_t blocks = (n + kTraceBlock - 1) / kTraceBlock;
    if (bvh->num_prims == 0)
    {
        write_misses<<<blocks, kTraceBlock, 0, stream>>>(d_hits, n);
        GBRT_LAUNCH_CHECK(ctx, "write_misses");
        return GBRT_OK;
    }
    if (any_hit)
        trace_rays<true><<<blocks, kTraceBlock, 0, stream>>>(bvh->nodes, bvh->tris, bvh->root, int32_t(bvh->num_inner),
                                                             int32_t(bvh->num_prims), d_rays, n, d_hits, ctx->d_status);
    else
        trace_rays<false><<<blocks, kTraceBlock, 0, stream>>>(bvh->nodes, bvh->tris, bvh->root,
                                                              int32_t(bvh->num_inner), int32_t(bvh->num_prims), d_rays,
                                                              n, d_hits, ctx->d_status);
    GBRT_LAUNCH_CHECK(ctx, "trace_rays");
    return GBRT_OK;
}

} // namespace gbrt
