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
// Entries of the traversal stack held in shared memory (the rest in local memory):
// 8 x 128 threads x 4 B = 4 KB per block.
constexpr int kSharedStack = 8;
// Resident blocks the register allocation must allow (launch bounds): any hit 12 blocks
// of 128 threads = 48 warps per SM at <= 40 registers; closest hit 16 blocks = 64 warps
// at <= 32 registers.  Measured on the heightfield workload (kernel alone, hits
// identical): closest 3.412 ms at 16 shared entries and 12 blocks, 3.389 / 3.386 at
// 14 / 16 blocks, 3.297 at 8 shared entries and 16 blocks; 24 shared entries 3.662.
// Any hit (AO rays, the unordered loop): 13.86 ms at 12 blocks, 14.44 at 10, 14.51 at 16.
constexpr int kMinBlocksAny = 12, kMinBlocksClosest = 16;

// One ray through the node pairs (stack top in shared memory) or the 4-wide nodes.
// Node layouts of the ray queries: the node pairs, the 4-wide nodes, the quantised
// 4-wide nodes.
enum : int
{
    kNodesPairs = 0,
    kNodesWide = 1,
    kNodesCompressed = 2,
    kNodesWide8 = 3,
};

template <bool AnyHit, int Nodes>
__device__ __forceinline__ trace_result trace_one(bvh_view const& v, f3 o, f3 d, float tmin, float tmax,
                                                  uint32_t* __restrict__ status)
{
    if constexpr (Nodes == kNodesCompressed)
        return traverse_bvh4<AnyHit>(v.nodes4q, v.num_nodes4, v.tris, v.num_tris, o, d, tmin, tmax, status);
    else if constexpr (Nodes == kNodesWide8)
        return traverse_bvhw<AnyHit, 8>(v.nodes8, v.num_nodes8, v.tris, v.num_tris, o, d, tmin, tmax, status);
    else
        // any-hit ray queries unordered (traverse_bvh_with)
        return traverse_view_shared<AnyHit, Nodes == kNodesWide, kTraceBlock, kSharedStack, !AnyHit>(v, o, d, tmin,
                                                                                                       tmax, status);
}

template <bool AnyHit, int Nodes>
__global__ void __launch_bounds__(kTraceBlock, AnyHit ? kMinBlocksAny : kMinBlocksClosest) trace_rays(bvh_view v, const gbrt_ray* __restrict__ rays, uint32_t n,
                                                          gbrt_hit* __restrict__ hits,
                                                          uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kTraceBlock + threadIdx.x;
    if (i >= n) return;

    float4 r0 = ldg4(&rays[i]);
    float4 r1 = ldg4(reinterpret_cast<const float4*>(&rays[i]) + 1);
    trace_result h = trace_one<AnyHit, Nodes>(v, { r0.x, r0.y, r0.z }, { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    uint32_t prim = h.tri >= 0 ? __float_as_uint(ldg4(&v.tris[h.tri].t0).w) : GBRT_NO_HIT;
    reinterpret_cast<uint4*>(hits)[i] =
        make_uint4(prim, __float_as_uint(h.t), __float_as_uint(h.u), __float_as_uint(h.v));
}

// Rays in the order perm[0..n): ray j = perm[i] writes hit j.
template <bool AnyHit, int Nodes>
__global__ void __launch_bounds__(kTraceBlock, AnyHit ? kMinBlocksAny : kMinBlocksClosest) trace_rays_permuted(bvh_view v, const gbrt_ray* __restrict__ rays,
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
    trace_result h = trace_one<AnyHit, Nodes>(v, { r0.x, r0.y, r0.z }, { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    uint32_t prim = h.tri >= 0 ? __float_as_uint(ldg4(&v.tris[h.tri].t0).w) : GBRT_NO_HIT;
    reinterpret_cast<uint4*>(hits)[j] =
        make_uint4(prim, __float_as_uint(h.t), __float_as_uint(h.u), __float_as_uint(h.v));
}

// Persistent traversal with per-lane refill (Aila & Laine 2009, "persistent
// while-while" with dynamic ray fetch): a grid that just fills the GPU; each warp takes
// ray indices off one atomic counter for its idle lanes, one warp-aggregated atomic per
// refill, once at least `refill_min` lanes are idle (or all are).  An iteration walks
// every busy lane to its next leaf, tests that leaf and pops the stack; a lane whose
// traversal ends stores its hit and is refilled, so lanes no longer idle until the
// slowest ray of their warp finishes.  The visit order of each ray is traverse_bvh's,
// so the hits are identical bit for bit.  perm (may be null): lane k traces ray
// perm[k].
template <bool AnyHit>
__global__ void __launch_bounds__(kTraceBlock) trace_rays_dynamic(bvh_view v, const gbrt_ray* __restrict__ rays,
                                                                  uint32_t n, const uint32_t* __restrict__ perm,
                                                                  gbrt_hit* __restrict__ hits,
                                                                  uint32_t* __restrict__ next_ray, uint32_t refill_min,
                                                                  uint32_t* __restrict__ status)
{
    const uint32_t full = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lanes_below = (1u << lane) - 1u;
    int stack[kStackSize];
    int sp = 0;
    int node = kEmptyLink;
    uint32_t ray = 0;
    bool have = false;
    bool drained = false;   // warp-uniform: the counter has passed n
    f3 o = { 0.0f, 0.0f, 0.0f }, d = { 0.0f, 0.0f, 0.0f };
    float ix = 0.0f, iy = 0.0f, iz = 0.0f, tmin = 0.0f, tmax = 0.0f;
    trace_result best{ -1, FLT_MAX, 0.0f, 0.0f };

    for (;;)
    {
        const uint32_t idle = __ballot_sync(full, !have);
        const uint32_t nidle = __popc(idle);
        if (!drained && nidle != 0 && (nidle >= refill_min || idle == full))
        {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (int(lane) == leader) base = atomicAdd(next_ray, nidle);
            base = __shfl_sync(full, base, leader);
            drained = uint64_t(base) + nidle >= uint64_t(n);
            if (!have)
            {
                const uint64_t k = uint64_t(base) + __popc(idle & lanes_below);
                if (k < n)
                {
                    const uint32_t j = perm ? __ldg(&perm[k]) : uint32_t(k);
                    if (j < n)
                    {
                        float4 r0 = ldg4(&rays[j]);
                        float4 r1 = ldg4(reinterpret_cast<const float4*>(&rays[j]) + 1);
                        o = { r0.x, r0.y, r0.z };
                        d = { r0.w, r1.x, r1.y };
                        tmin = r1.z;
                        tmax = r1.w;
                        ix = safe_rcp(d.x);
                        iy = safe_rcp(d.y);
                        iz = safe_rcp(d.z);
                        best = { -1, FLT_MAX, 0.0f, 0.0f };
                        sp = 0;
                        node = v.root;
                        ray = j;
                        have = true;
                    }
                    else
                    {
                        atomicOr(status, kStatusBadIndex);
                    }
                }
            }
        }
        if (!__any_sync(full, have)) break;
        if (!have) continue;

        // inner nodes until a leaf or the end of the traversal (traverse_bvh's loop)
        while (node >= 0)
        {
            if (node >= v.num_inner)
            {
                atomicOr(status, kStatusBadIndex);
                node = kEmptyLink;
                break;
            }
            float4 a, b, z;
            int4 link;
            load_pair(v.nodes + node, a, b, z, link);
            float lx0 = (a.x - o.x) * ix, hx0 = (a.y - o.x) * ix;
            float ly0 = (a.z - o.y) * iy, hy0 = (a.w - o.y) * iy;
            float lz0 = (z.x - o.z) * iz, hz0 = (z.y - o.z) * iz;
            float lx1 = (b.x - o.x) * ix, hx1 = (b.y - o.x) * ix;
            float ly1 = (b.z - o.y) * iy, hy1 = (b.w - o.y) * iy;
            float lz1 = (z.z - o.z) * iz, hz1 = (z.w - o.z) * iz;
            float tn0 = fmaxf(tmin, fmaxf(fminf(lx0, hx0), fmaxf(fminf(ly0, hy0), fminf(lz0, hz0))));
            float tf0 = fminf(tmax, fminf(fmaxf(lx0, hx0), fminf(fmaxf(ly0, hy0), fmaxf(lz0, hz0))));
            float tn1 = fmaxf(tmin, fmaxf(fminf(lx1, hx1), fmaxf(fminf(ly1, hy1), fminf(lz1, hz1))));
            float tf1 = fminf(tmax, fminf(fmaxf(lx1, hx1), fminf(fmaxf(ly1, hy1), fmaxf(lz1, hz1))));
            bool h0 = tf0 >= tn0 && (AnyHit || tn0 < best.t);   // as traverse_bvh_with
            bool h1 = tf1 >= tn1 && (AnyHit || tn1 < best.t);
            if (h0 && h1)
            {
                bool first0 = AnyHit || tn0 < tn1;   // the ray queries' order (trace_one)
                int near_child = first0 ? link.x : link.y;
                int far_child = first0 ? link.y : link.x;
                if (sp < kStackSize)
                    stack[sp++] = far_child;
                else
                    atomicOr(status, kStatusStackOverflow);
                node = near_child;
            }
            else if (h0 || h1)
            {
                node = h0 ? link.x : link.y;
            }
            else
            {
                node = sp > 0 ? stack[--sp] : kEmptyLink;
            }
        }
        bool done = node == kEmptyLink;
        if (!done)
        {
            for (int t = ~node;; ++t)
            {
                if (t >= v.num_tris)
                {
                    atomicOr(status, kStatusBadIndex);
                    break;
                }
                const tri48* tp = v.tris + t;
                float4 t0 = ldg4(&tp->t0);
                float4 t1 = ldg4(&tp->t1);
                float4 t2 = ldg4(&tp->t2);
                tri_hit h = intersect_triangle(o, d, { t0.x, t0.y, t0.z }, { t1.x, t1.y, t1.z }, { t2.x, t2.y, t2.z });
                if (h.hit && h.t < best.t && h.t >= tmin && h.t <= tmax)
                {
                    best = { t, h.t, h.u, h.v };
                    if (AnyHit)
                    {
                        done = true;
                        break;
                    }
                }
                if (__float_as_uint(t2.w) & kLastInLeaf) break;
            }
            if (!done)
            {
                node = sp > 0 ? stack[--sp] : kEmptyLink;
                done = node == kEmptyLink;
            }
        }
        if (done)
        {
            uint32_t prim = best.tri >= 0 ? __float_as_uint(ldg4(&v.tris[best.tri].t0).w) : GBRT_NO_HIT;
            reinterpret_cast<uint4*>(hits)[ray] =
                make_uint4(prim, __float_as_uint(best.t), __float_as_uint(best.u), __float_as_uint(best.v));
            have = false;
            node = kEmptyLink;
        }
    }
}

// Ray order.  Closest-hit queries: the Morton key of the origin's cell, 8 bits per
// axis of the scene box (24 bits).  Any-hit queries: 6 bits per axis followed by the
// direction's octant (21 bits), so a warp's rays also share their near/far child order.
// Measured on the heightfield workload (kernel alone, same rays): AO any hit 16.58 ->
// 16.24 ms with the octant; closest hit 3.56 -> 3.74 ms with it, hence per query kind.
constexpr int kCellBitsClosest = 8;
constexpr int kCellBitsAny = 6;

// The sort key of each ray (above): cell_bits per axis, then the octant if asked.
__global__ void __launch_bounds__(kTraceBlock) ray_origin_keys(const gbrt_ray* __restrict__ rays, uint32_t n,
                                                               float3 lo, float3 scale, int cell_bits, bool octant,
                                                               uint32_t* __restrict__ keys,
                                                               uint32_t* __restrict__ values)
{
    uint32_t i = blockIdx.x * kTraceBlock + threadIdx.x;
    if (i >= n) return;
    float4 r0 = ldg4(&rays[i]);
    float q[3] = { (r0.x - lo.x) * scale.x, (r0.y - lo.y) * scale.y, (r0.z - lo.z) * scale.z };
    const float top = float((1 << cell_bits) - 1);
    uint32_t c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        float v = fminf(fmaxf(q[a], 0.0f), top);   // NaN (degenerate ray) lands in cell 0
        c[a] = uint32_t(v);
    }
    uint32_t key = morton3(c[0], c[1], c[2]);
    if (octant)
    {
        float4 r1 = ldg4(reinterpret_cast<const float4*>(&rays[i]) + 1);
        // direction = (r0.w, r1.x, r1.y): one bit per negative component
        key = (key << 3) | (r0.w < 0.0f ? 1u : 0u) | (r1.x < 0.0f ? 2u : 0u) | (r1.y < 0.0f ? 4u : 0u);
    }
    keys[i] = key;
    values[i] = i;
}

__global__ void __launch_bounds__(kTraceBlock) write_misses(gbrt_hit* __restrict__ hits, uint32_t n)
{
    uint32_t i = blockIdx.x * kTraceBlock + threadIdx.x;
    if (i < n) reinterpret_cast<uint4*>(hits)[i] = make_uint4(GBRT_NO_HIT, __float_as_uint(FLT_MAX), 0u, 0u);
}

constexpr uint32_t kSortMinRays = 1u << 16;   // below this the order costs more than it saves

inline size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

} // namespace

// Scratch of one trace call: the persistent kernel's ray counter, then the ray order's
// keys / values (double-buffered) and the sort's own scratch.
constexpr size_t kCounterBytes = 256;

size_t trace_scratch_bytes(uint32_t n)
{
    return kCounterBytes + 4 * align256(size_t(n) * 4) + align256(radix_sort_scratch_bytes(n));
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
    const bool wide8 = bvh->nodes8 != nullptr && (ctx->trace_flags & GBRT_TRACE_WIDE8_NODES);
    const bool compressed = !wide8 && bvh->nodes4q != nullptr && (ctx->trace_flags & GBRT_TRACE_COMPRESSED_NODES);
    const bool wide = !wide8 && !compressed && bvh->nodes4 != nullptr && (ctx->trace_flags & GBRT_TRACE_WIDE_NODES);
    const bool have_scratch = scratch && scratch_bytes >= trace_scratch_bytes(n);
    const bool persistent = (ctx->trace_flags & GBRT_TRACE_PERSISTENT) && !wide && !compressed && !wide8 && have_scratch;
    const uint32_t* perm = nullptr;
    if ((ctx->trace_flags & GBRT_TRACE_SORT_RAYS) && n >= kSortMinRays && have_scratch)
    {
        char* base = static_cast<char*>(scratch) + kCounterBytes;
        size_t w = align256(size_t(n) * 4);
        uint32_t* keys = reinterpret_cast<uint32_t*>(base);
        uint32_t* vals = reinterpret_cast<uint32_t*>(base + w);
        uint32_t* keys_alt = reinterpret_cast<uint32_t*>(base + 2 * w);
        uint32_t* vals_alt = reinterpret_cast<uint32_t*>(base + 3 * w);
        float3 lo = make_float3(bvh->lo[0], bvh->lo[1], bvh->lo[2]);
        float ext[3] = { bvh->hi[0] - bvh->lo[0], bvh->hi[1] - bvh->lo[1], bvh->hi[2] - bvh->lo[2] };
        const int cell_bits = any_hit ? kCellBitsAny : kCellBitsClosest;
        const float cells = float(1 << cell_bits);
        float3 scale = make_float3(ext[0] > 0.0f ? cells / ext[0] : 0.0f, ext[1] > 0.0f ? cells / ext[1] : 0.0f,
                                   ext[2] > 0.0f ? cells / ext[2] : 0.0f);
        ray_origin_keys<<<blocks, kTraceBlock, 0, stream>>>(d_rays, n, lo, scale, cell_bits, any_hit, keys, vals);
        GBRT_LAUNCH_CHECK(ctx, "ray_origin_keys");
        const int key_bits = 3 * cell_bits + (any_hit ? 3 : 0);
        uint32_t* sorted = nullptr;
        gbrt_status st = radix_sort_pairs(ctx, keys, vals, keys_alt, vals_alt, n, key_bits, base + 4 * w, stream,
                                          &sorted);
        if (st != GBRT_OK) return st;
        perm = sorted;   // vals or vals_alt, wherever the last pass left the order
        if (!persistent)
        {
            kernel_timer timer(ctx, stream);
            auto launch = [&](auto kernel) { kernel<<<blocks, kTraceBlock, 0, stream>>>(v, d_rays, n, perm, d_hits,
                                                                                        ctx->d_status); };
            if (wide8)
                any_hit ? launch(trace_rays_permuted<true, kNodesWide8>) : launch(trace_rays_permuted<false, kNodesWide8>);
            else if (compressed)
                any_hit ? launch(trace_rays_permuted<true, kNodesCompressed>)
                        : launch(trace_rays_permuted<false, kNodesCompressed>);
            else if (wide)
                any_hit ? launch(trace_rays_permuted<true, kNodesWide>) : launch(trace_rays_permuted<false, kNodesWide>);
            else
                any_hit ? launch(trace_rays_permuted<true, kNodesPairs>)
                        : launch(trace_rays_permuted<false, kNodesPairs>);
            GBRT_LAUNCH_CHECK(ctx, "trace_rays_permuted");
            return GBRT_OK;
        }
    }
    if (persistent)
    {
        uint32_t* counter = static_cast<uint32_t*>(scratch);
        auto kernel = any_hit ? trace_rays_dynamic<true> : trace_rays_dynamic<false>;
        int per_sm = 0;
        GBRT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTraceBlock, 0));
        uint32_t grid = uint32_t(ctx->num_sms) * uint32_t(per_sm > 0 ? per_sm : 1);
        if (grid > blocks) grid = blocks;
        GBRT_CUDA(ctx, cudaMemsetAsync(counter, 0, 4, stream));
        kernel_timer timer(ctx, stream);
        kernel<<<grid, kTraceBlock, 0, stream>>>(v, d_rays, n, perm, d_hits, counter, ctx->trace_refill,
                                                 ctx->d_status);
        GBRT_LAUNCH_CHECK(ctx, "trace_rays_dynamic");
        return GBRT_OK;
    }
    kernel_timer timer(ctx, stream);
    auto launch = [&](auto kernel) { kernel<<<blocks, kTraceBlock, 0, stream>>>(v, d_rays, n, d_hits, ctx->d_status); };
    if (wide8)
        any_hit ? launch(trace_rays<true, kNodesWide8>) : launch(trace_rays<false, kNodesWide8>);
    else if (compressed)
        any_hit ? launch(trace_rays<true, kNodesCompressed>) : launch(trace_rays<false, kNodesCompressed>);
    else if (wide)
        any_hit ? launch(trace_rays<true, kNodesWide>) : launch(trace_rays<false, kNodesWide>);
    else
        any_hit ? launch(trace_rays<true, kNodesPairs>) : launch(trace_rays<false, kNodesPairs>);
    GBRT_LAUNCH_CHECK(ctx, "trace_rays");
    return GBRT_OK;
}

} // namespace gbrt
