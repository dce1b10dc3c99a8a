// closest_hit / any_hit ray queries over the node-pair BVH: one thread per ray over
// the shared traversal core (traverse_core.cuh), 128-bit ray loads and hit stores.
//
// With GBRT_TRACE_SORT_RAYS, a call first orders its rays by the Morton cell of their
// origin (24-bit key, 256 cells per axis of the scene box; a stable radix sort keeps
// rays of one cell in input order) and traces them through that permutation, so the
// 32 rays of a warp start in one region of the scene and share its upper tree path.
// Each ray is still traced independently: the hits are identical bit for bit.

#include "traverse_core.cuh"

namespace gbrt {
namespace {

constexpr int kTraceBlock = 128;

template <bool AnyHit, bool Wide>
__global__ void __launch_bounds__(kTraceBlock) trace_rays(bvh_view v, const gbrt_ray* __restrict__ rays, uint32_t n,
                                                          gbrt_hit* __restrict__ hits,
                                                          uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kTraceBlock + threadIdx.x;
    if (i >= n) return;

    float4 r0 = ldg4(&rays[i]);
    float4 r1 = ldg4(reinterpret_cast<const float4*>(&rays[i]) + 1);
    trace_result h = traverse_view<AnyHit, Wide>(v, { r0.x, r0.y, r0.z }, { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    uint32_t prim = h.tri >= 0 ? __float_as_uint(ldg4(&v.tris[h.tri].t0).w) : GBRT_NO_HIT;
    reinterpret_cast<uint4*>(hits)[i] =
        make_uint4(prim, __float_as_uint(h.t), __float_as_uint(h.u), __float_as_uint(h.v));
}

// Rays in the order perm[0..n): ray j = perm[i] writes hit j.
template <bool AnyHit, bool Wide>
__global__ void __launch_bounds__(kTraceBlock) trace_rays_permuted(bvh_view v, const gbrt_ray* __restrict__ rays,
                                                                   uint32_t n, const uint32_t* __restrict__ perm,
                                                                   gbrt_hit* __restrict__ hits,
                                                                   uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kTraceBlock + threadIdx.x;
    if (i >= n) return;
    uint32_t j = __ldg(&perm[i]);
    if (j >= n)
    {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    float4 r0 = ldg4(&rays[j]);
    float4 r1 = ldg4(reinterpret_cast<const float4*>(&rays[j]) + 1);
    trace_result h = traverse_view<AnyHit, Wide>(v, { r0.x, r0.y, r0.z }, { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    uint32_t prim = h.tri >= 0 ? __float_as_uint(ldg4(&v.tris[h.tri].t0).w) : GBRT_NO_HIT;
    reinterpret_cast<uint4*>(hits)[j] =
        make_uint4(prim, __float_as_uint(h.t), __float_as_uint(h.u), __float_as_uint(h.v));
}

// 24-bit Morton key of each ray's origin cell (8 bits per axis of the scene box).
__global__ void __launch_bounds__(kTraceBlock) ray_origin_keys(const gbrt_ray* __restrict__ rays, uint32_t n,
                                                               float3 lo, float3 scale, uint32_t* __restrict__ keys,
                                                               uint32_t* __restrict__ values)
{
    uint32_t i = blockIdx.x * kTraceBlock + threadIdx.x;
    if (i >= n) return;
    float4 r0 = ldg4(&rays[i]);
    float q[3] = { (r0.x - lo.x) * scale.x, (r0.y - lo.y) * scale.y, (r0.z - lo.z) * scale.z };
    uint32_t c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        float v = fminf(fmaxf(q[a], 0.0f), 255.0f);   // NaN (degenerate ray) lands in cell 0
        c[a] = uint32_t(v);
    }
    keys[i] = morton3(c[0], c[1], c[2]);
    values[i] = i;
}

__global__ void __launch_bounds__(kTraceBlock) write_misses(gbrt_hit* __restrict__ hits, uint32_t n)
{
    uint32_t i = blockIdx.x * kTraceBlock + threadIdx.x;
    if (i < n) reinterpret_cast<uint4*>(hits)[i] = make_uint4(GBRT_NO_HIT, __float_as_uint(FLT_MAX), 0u, 0u);
}

constexpr uint32_t kSortMinRays = 1u << 16;   // below this the order costs more than it saves
constexpr int kOriginKeyBits = 24;

inline size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

} // namespace

size_t trace_scratch_bytes(uint32_t n)
{
    return 4 * align256(size_t(n) * 4) + align256(radix_sort_scratch_bytes(n));
}

gbrt_status trace(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_ray const* d_rays, uint32_t n, gbrt_hit* d_hits,
                  bool any_hit, cudaStream_t stream, void* scratch, size_t scratch_bytes)
{
    if (n == 0) return GBRT_OK;
    uint32_t blocks = (n + kTraceBlock - 1) / kTraceBlock;
    if (bvh->num_prims == 0)
    {
        write_misses<<<blocks, kTraceBlock, 0, stream>>>(d_hits, n);
        GBRT_LAUNCH_CHECK(ctx, "write_misses");
        return GBRT_OK;
    }
    const bvh_view v = view_of(bvh);
    const bool wide = bvh->nodes4 != nullptr && (ctx->trace_flags & GBRT_TRACE_WIDE_NODES);
    if ((ctx->trace_flags & GBRT_TRACE_SORT_RAYS) && n >= kSortMinRays && scratch &&
        scratch_bytes >= trace_scratch_bytes(n))
    {
        char* base = static_cast<char*>(scratch);
        size_t w = align256(size_t(n) * 4);
        uint32_t* keys = reinterpret_cast<uint32_t*>(base);
        uint32_t* vals = reinterpret_cast<uint32_t*>(base + w);
        uint32_t* keys_alt = reinterpret_cast<uint32_t*>(base + 2 * w);
        uint32_t* vals_alt = reinterpret_cast<uint32_t*>(base + 3 * w);
        float3 lo = make_float3(bvh->lo[0], bvh->lo[1], bvh->lo[2]);
        float ext[3] = { bvh->hi[0] - bvh->lo[0], bvh->hi[1] - bvh->lo[1], bvh->hi[2] - bvh->lo[2] };
        float3 scale = make_float3(ext[0] > 0.0f ? 256.0f / ext[0] : 0.0f, ext[1] > 0.0f ? 256.0f / ext[1] : 0.0f,
                                   ext[2] > 0.0f ? 256.0f / ext[2] : 0.0f);
        ray_origin_keys<<<blocks, kTraceBlock, 0, stream>>>(d_rays, n, lo, scale, keys, vals);
        GBRT_LAUNCH_CHECK(ctx, "ray_origin_keys");
        gbrt_status st = radix_sort_pairs(ctx, keys, vals, keys_alt, vals_alt, n, kOriginKeyBits, base + 4 * w,
                                          stream);
        if (st != GBRT_OK) return st;
        const uint32_t* perm = vals;   // radix_sort_pairs leaves the result in (keys, values)
        auto launch = [&](auto kernel) { kernel<<<blocks, kTraceBlock, 0, stream>>>(v, d_rays, n, perm, d_hits,
                                                                                    ctx->d_status); };
        if (wide)
            any_hit ? launch(trace_rays_permuted<true, true>) : launch(trace_rays_permuted<false, true>);
        else
            any_hit ? launch(trace_rays_permuted<true, false>) : launch(trace_rays_permuted<false, false>);
        GBRT_LAUNCH_CHECK(ctx, "trace_rays_permuted");
        return GBRT_OK;
    }
    auto launch = [&](auto kernel) { kernel<<<blocks, kTraceBlock, 0, stream>>>(v, d_rays, n, d_hits, ctx->d_status); };
    if (wide)
        any_hit ? launch(trace_rays<true, true>) : launch(trace_rays<false, true>);
    else
        any_hit ? launch(trace_rays<true, false>) : launch(trace_rays<false, false>);
    GBRT_LAUNCH_CHECK(ctx, "trace_rays");
    return GBRT_OK;
}

} // namespace gbrt
