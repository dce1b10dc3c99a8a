// Batched LBVH build and ray queries over many scenes in one arena.
//
// visionaray builds and renders one scene per call (lbvh.h:681-844, cuda_sched.inl:
// 226-246); hundreds of small scenes then cost hundreds of launches, allocations and
// synchronisations each.  Here all scenes' triangles are one array and every stage is
// one launch over all of them:
//   batch_centroids : per-triangle bounds and centroid, per-scene centroid bounds (lanes
//                     of one scene reduced in the warp, one set of atomics per scene
//                     and warp)
//   batch_morton    : each scene's codes against its own bounds -- the codes a single-
//                     scene build computes
//   two stable radix sorts: by code, then by scene, giving (scene, code, index) order,
//                     i.e. every scene's segment sorted as its own build sorts it
//   batch_hierarchy : Karras splits inside each segment, links in arena indices
//   batch_refit     : the bottom-up refit of refit_and_emit over all segments
// so each scene's tree equals gbrt_bvh_build_lbvh's for that scene: same codes, same
// order, same topology and boxes, hence bit-identical hits.  No stage allocates or
// synchronises: a build can be captured in a CUDA graph.

#include "collapse.cuh"
#include "lbvh_device.cuh"
#include "traverse_core.cuh"

#include <algorithm>
#include <new>

namespace gbrt {
namespace {

constexpr int kBlock = 256;

__global__ void __launch_bounds__(kBlock) batch_init_bounds(int* __restrict__ bounds, uint32_t num_scenes)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= num_scenes * 6) return;
    bounds[i] = (i % 6) < 3 ? float_to_ordered(FLT_MAX) : float_to_ordered(-FLT_MAX);
}

__global__ void __launch_bounds__(kBlock) batch_centroids(gbrt_triangle const* __restrict__ tris, uint32_t total,
                                                          const uint32_t* __restrict__ offsets, uint32_t num_scenes,
                                                          float4* __restrict__ centroids,
                                                          uint32_t* __restrict__ prim_scene, int* __restrict__ bounds)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    bool active = i < total;
    uint32_t s = 0;
    f3 c = { 0.0f, 0.0f, 0.0f };
    if (active)
    {
        s = upper_segment(offsets, num_scenes, i);
        c = box_center(tri_box(load_tri(tris, i)));
        centroids[i] = make_float4(c.x, c.y, c.z, 0.0f);
        prim_scene[i] = s;
    }
    uint32_t mask = __ballot_sync(0xFFFFFFFFu, active);
    if (!active) return;
    uint32_t peers = __match_any_sync(mask, s);
    // the reference's atomic fold (lbvh.h:233-238) skips NaN and outward infinities
    float mn[3] = { cas_lo(c.x), cas_lo(c.y), cas_lo(c.z) }, mx[3] = { cas_hi(c.x), cas_hi(c.y), cas_hi(c.z) };
    for (uint32_t m = peers; m; m &= m - 1)
    {
        int src = __ffs(m) - 1;
        for (int a = 0; a < 3; ++a)
        {
            float v = __shfl_sync(peers, a == 0 ? c.x : (a == 1 ? c.y : c.z), src);
            mn[a] = ref_min(mn[a], cas_lo(v));
            mx[a] = ref_max(mx[a], cas_hi(v));
        }
    }
    if ((threadIdx.x & 31) == __ffs(peers) - 1)
    {
        for (int a = 0; a < 3; ++a)
        {
            atomicMin(&bounds[6 * s + a], float_to_ordered(mn[a]));
            atomicMax(&bounds[6 * s + 3 + a], float_to_ordered(mx[a]));
        }
    }
}

// lbvh.h:253-267 against the triangle's own scene's centroid bounds.
__global__ void __launch_bounds__(kBlock) batch_morton(const float4* __restrict__ centroids,
                                                       const uint32_t* __restrict__ prim_scene, uint32_t total,
                                                       const int* __restrict__ bounds, uint32_t* __restrict__ codes_in,
                                                       uint32_t* __restrict__ keys, uint32_t* __restrict__ values)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= total) return;
    const int* cbo = bounds + 6 * prim_scene[i];
    box3 cb;
    cb.lo = { ordered_to_float(cbo[0]), ordered_to_float(cbo[1]), ordered_to_float(cbo[2]) };
    cb.hi = { ordered_to_float(cbo[3]), ordered_to_float(cbo[4]), ordered_to_float(cbo[5]) };
    f3 center = box_center(cb);
    f3 size = { __fsub_rn(cb.hi.x, cb.lo.x), __fsub_rn(cb.hi.y, cb.lo.y), __fsub_rn(cb.hi.z, cb.lo.z) };
    float4 c4 = centroids[i];
    float c[3] = { c4.x, c4.y, c4.z };
    float cc[3] = { center.x, center.y, center.z };
    float cs[3] = { size.x, size.y, size.z };
    uint32_t q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        float v = __fsub_rn(c[a], cc[a]);
        v = __fdiv_rn(__fadd_rn(v, __fmul_rn(cs[a], 0.5f)), cs[a]);
        v = __fmul_rn(v, 1024.0f);
        v = ref_min(ref_max(v, 0.0f), 1023.0f);
        q[a] = static_cast<uint32_t>(v);
    }
    uint32_t code = morton3(q[0], q[1], q[2]);
    codes_in[i] = code;
    keys[i] = code;
    values[i] = i;
}

__global__ void __launch_bounds__(kBlock) gather_scene_keys(const uint32_t* __restrict__ values,
                                                            const uint32_t* __restrict__ prim_scene, uint32_t total,
                                                            uint32_t* __restrict__ keys)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < total) keys[i] = prim_scene[values[i]];
}

__global__ void __launch_bounds__(kBlock) gather_codes(const uint32_t* __restrict__ values,
                                                       const uint32_t* __restrict__ codes_in, uint32_t total,
                                                       uint32_t* __restrict__ sorted_codes)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < total) sorted_codes[i] = codes_in[values[i]];
}

// Inner node g of the arena: Karras split inside its scene's segment, links translated
// to arena indices (inner: inner_offsets[s] + c, leaf: ~(offsets[s] + j)).
__global__ void __launch_bounds__(kBlock) batch_hierarchy(const uint32_t* __restrict__ sorted_codes,
                                                          const uint32_t* __restrict__ offsets,
                                                          const uint32_t* __restrict__ inner_offsets,
                                                          uint32_t num_scenes, uint32_t total_inner,
                                                          bvh2_node* __restrict__ nodes, int* __restrict__ leaf_parent,
                                                          int2* __restrict__ ranges)
{
    uint32_t g = blockIdx.x * kBlock + threadIdx.x;
    if (g >= total_inner) return;
    uint32_t s = upper_segment(inner_offsets, num_scenes, g);
    int base_leaf = int(offsets[s]);
    int base_inner = int(inner_offsets[s]);
    int n = int(offsets[s + 1]) - base_leaf;
    int i = int(g) - base_inner;
    int first, last, split;
    karras_node(sorted_codes + base_leaf, n, i, first, last, split);
    int left = split, right = split + 1;
    int cl, cr;
    int gi = int(g);
    if (left == first)
    {
        cl = ~(base_leaf + left);
        leaf_parent[base_leaf + left] = (gi << 1) | 0;
    }
    else
    {
        cl = base_inner + left;
        nodes[base_inner + left].link.w = (gi << 1) | 0;
    }
    if (right == last)
    {
        cr = ~(base_leaf + right);
        leaf_parent[base_leaf + right] = (gi << 1) | 1;
    }
    else
    {
        cr = base_inner + right;
        nodes[base_inner + right].link.w = (gi << 1) | 1;
    }
    nodes[g].link.x = cl;
    nodes[g].link.y = cr;
    if (i == 0) nodes[g].link.w = -1;
    ranges[g] = make_int2(base_leaf + first, base_leaf + last);
}

// Level 0 of the arena's wide collapse: scene s with an inner root gets wide node s.
__global__ void __launch_bounds__(kBlock) batch_collapse_seed(const int32_t* __restrict__ roots, uint32_t num_scenes,
                                                              int2* __restrict__ q, uint32_t* __restrict__ count,
                                                              uint32_t* __restrict__ node_counter)
{
    uint32_t s = blockIdx.x * kBlock + threadIdx.x;
    if (s == 0) *node_counter = num_scenes;
    if (s >= num_scenes || roots[s] < 0) return;
    q[atomicAdd(count, 1u)] = make_int2(roots[s], int(s));
}

// refit_and_emit over all segments: a leaf without a parent (a one-triangle scene) only
// emits its triangle; every root records its height into *height (max over scenes).
__global__ void __launch_bounds__(kBlock) batch_refit(gbrt_triangle const* __restrict__ tris_in,
                                                      const uint32_t* __restrict__ sorted_ids, uint32_t total,
                                                      uint32_t total_inner, const int* __restrict__ leaf_parent,
                                                      bvh2_node* __restrict__ nodes, uint32_t* __restrict__ arrivals,
                                                      tri48* __restrict__ tris_out, uint32_t* __restrict__ height_out,
                                                      uint32_t* __restrict__ status)
{
    uint32_t j = blockIdx.x * kBlock + threadIdx.x;
    if (j >= total) return;
    uint32_t id = __ldg(&sorted_ids[j]);
    if (id >= total)
    {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    tri_in t = load_tri(tris_in, id);
    tri48 o;
    o.t0 = make_float4(t.v1.x, t.v1.y, t.v1.z, __uint_as_float(t.prim_id));
    o.t1 = make_float4(t.e1.x, t.e1.y, t.e1.z, __uint_as_float(t.geom_id));
    o.t2 = make_float4(t.e2.x, t.e2.y, t.e2.z, __uint_as_float(kLastInLeaf));
    tris_out[j] = o;
    int link = leaf_parent[j];
    if (link == -1) return;   // one-triangle scene: the leaf is the root
    box3 b = tri_box(t);
    int height = 0;
    for (uint32_t step = 0; step < total; ++step)
    {
        if (link < 0 || uint32_t(link >> 1) >= total_inner)
        {
            atomicOr(status, kStatusBadIndex);
            return;
        }
        int node = link >> 1, side = link & 1;
        bvh2_node* nd = &nodes[node];
        store_child_box(nd, side, b);
        atomicMax(&nd->link.z, height + 1);
        __threadfence();
        if (atomicAdd(&arrivals[node], 1u) == 0) return;
        __threadfence();
        b = load_union_cg(nd);
        height = __ldcg(&nd->link.z);
        int up = __ldcg(&nd->link.w);
        if (up < 0)
        {
            atomicMax(height_out, uint32_t(height));
            return;
        }
        link = up;
    }
    atomicOr(status, kStatusBadIndex);
}

// closest_hit of every scene's rays: ray r belongs to the scene whose ray range holds it.
__global__ void __launch_bounds__(128) batch_trace(const bvh2_node* __restrict__ nodes, const tri48* __restrict__ tris,
                                                   const int32_t* __restrict__ roots,
                                                   const uint32_t* __restrict__ ray_offsets, uint32_t num_scenes,
                                                   int32_t total_inner, int32_t total_tris,
                                                   const gbrt_ray* __restrict__ rays, uint32_t n,
                                                   gbrt_hit* __restrict__ hits, uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * 128 + threadIdx.x;
    if (i >= n) return;
    uint32_t s = upper_segment(ray_offsets, num_scenes, i);
    float4 r0 = ldg4(&rays[i]);
    float4 r1 = ldg4(reinterpret_cast<const float4*>(&rays[i]) + 1);
    trace_result h = traverse_bvh<false>(nodes, tris, __ldg(&roots[s]), total_inner, total_tris, { r0.x, r0.y, r0.z },
                                         { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    uint32_t prim = h.tri >= 0 ? __float_as_uint(ldg4(&tris[h.tri].t0).w) : GBRT_NO_HIT;
    reinterpret_cast<uint4*>(hits)[i] =
        make_uint4(prim, __float_as_uint(h.t), __float_as_uint(h.u), __float_as_uint(h.v));
}

// Reference-layout export of one scene (lbvh::collapse, lbvh.h:374-451): arena indices
// are made scene-local again.
__global__ void __launch_bounds__(kBlock) batch_export(const bvh2_node* __restrict__ nodes, int base_inner,
                                                       int num_inner, int base_leaf,
                                                       const uint32_t* __restrict__ sorted_ids,
                                                       gbrt_bvh_node* __restrict__ out)
{
    int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= num_inner) return;
    bvh2_node nd = nodes[base_inner + i];
    box3 cbox[2];
    cbox[0].lo = { nd.xy0.x, nd.xy0.z, nd.z01.x };
    cbox[0].hi = { nd.xy0.y, nd.xy0.w, nd.z01.y };
    cbox[1].lo = { nd.xy1.x, nd.xy1.z, nd.z01.z };
    cbox[1].hi = { nd.xy1.y, nd.xy1.w, nd.z01.w };
    int child[2] = { nd.link.x, nd.link.y };
    auto put = [&](gbrt_bvh_node& d, box3 const& b, uint32_t first, uint16_t count) {
        d.bbox_min[0] = b.lo.x;
        d.bbox_min[1] = b.lo.y;
        d.bbox_min[2] = b.lo.z;
        d.bbox_max[0] = b.hi.x;
        d.bbox_max[1] = b.hi.y;
        d.bbox_max[2] = b.hi.z;
        d.first_child_or_prim = first;
        d.num_prims = count;
        d.ordered_traversal_axis = 0;
        d.ordered_traversal_sign = 0;
    };
    for (int s = 0; s < 2; ++s)
    {
        gbrt_bvh_node& d = out[1 + 2 * i + s];
        if (child[s] < 0)
            put(d, cbox[s], __ldg(&sorted_ids[~child[s]]) - uint32_t(base_leaf), 1);
        else
            put(d, cbox[s], uint32_t(1 + 2 * (child[s] - base_inner)), 0);
    }
    if (i == 0)
    {
        put(out[0], box_union_cas(cbox[0], cbox[1]), 1u, 0);
    }
}

__global__ void __launch_bounds__(kBlock) iota_from(uint32_t* __restrict__ out, uint32_t n)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < n) out[i] = i;
}

inline uint32_t blocks_for(uint64_t n) { return uint32_t((n + kBlock - 1) / kBlock); }
inline size_t align_up(size_t v) { return (v + 255) & ~size_t(255); }

struct batch_scratch
{
    size_t centroids, prim_scene, bounds, codes_in, keys_alt, vals_alt, scene_keys, leaf_parent, arrivals, sort, total;
};

batch_scratch scratch_layout(uint32_t total, uint32_t num_scenes)
{
    batch_scratch l{};
    size_t o = 0;
    l.centroids = o;   o = align_up(o + size_t(total) * 16);
    l.prim_scene = o;  o = align_up(o + size_t(total) * 4);
    l.bounds = o;      o = align_up(o + size_t(num_scenes) * 24);
    l.codes_in = o;    o = align_up(o + size_t(total) * 4);
    l.keys_alt = o;    o = align_up(o + size_t(total) * 4);
    l.vals_alt = o;    o = align_up(o + size_t(total) * 4);
    l.scene_keys = o;  o = align_up(o + size_t(total) * 4);
    l.leaf_parent = o; o = align_up(o + size_t(total) * 4);
    l.arrivals = o;    o = align_up(o + size_t(total) * 4);
    l.sort = o;        o = align_up(o + radix_sort_scratch_bytes(total));
    l.total = o;
    return l;
}

void free_batch(gbrt_batch* b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
    cudaFree(b->d_offsets);
    cudaFree(b->d_inner_offsets);
    cudaFree(b->d_roots);
    cudaFree(b->nodes);
    cudaFree(b->tris);
    cudaFree(b->sorted_codes);
    cudaFree(b->sorted_ids);
    cudaFree(b->d_height);
    cudaFree(b->scratch);
    cudaFree(b->d_frames);
    cudaFree(b->d_pixel_offsets);
    cudaFree(b->d_materials);
    cudaFree(b->d_work);
    cudaFree(b->d_lights);
    cudaFree(b->d_light_offsets);
    cudaFree(b->ranges);
    cudaFree(b->wide_nodes);
    cudaFree(b->wide_queue[0]);
    cudaFree(b->wide_queue[1]);
    cudaFree(b->wide_counts);
    cudaFree(b->sort_buf);
    cudaFree(b->sort_scratch);
}

} // namespace

gbrt_status batch_build(gbrt_context* ctx, gbrt_batch* b, gbrt_triangle const* d_tris, cudaStream_t s)
{
    if (b->total == 0) return GBRT_OK;
    const batch_scratch l = scratch_layout(b->total, b->num_scenes);
    char* base = static_cast<char*>(b->scratch);
    float4* centroids = reinterpret_cast<float4*>(base + l.centroids);
    uint32_t* prim_scene = reinterpret_cast<uint32_t*>(base + l.prim_scene);
    int* bounds = reinterpret_cast<int*>(base + l.bounds);
    uint32_t* codes_in = reinterpret_cast<uint32_t*>(base + l.codes_in);
    uint32_t* keys_alt = reinterpret_cast<uint32_t*>(base + l.keys_alt);
    uint32_t* vals_alt = reinterpret_cast<uint32_t*>(base + l.vals_alt);
    uint32_t* scene_keys = reinterpret_cast<uint32_t*>(base + l.scene_keys);
    int* leaf_parent = reinterpret_cast<int*>(base + l.leaf_parent);
    uint32_t* arrivals = reinterpret_cast<uint32_t*>(base + l.arrivals);
    const uint32_t n = b->total;

    batch_init_bounds<<<blocks_for(uint64_t(b->num_scenes) * 6), kBlock, 0, s>>>(bounds, b->num_scenes);
    GBRT_LAUNCH_CHECK(ctx, "batch_init_bounds");
    batch_centroids<<<blocks_for(n), kBlock, 0, s>>>(d_tris, n, b->d_offsets, b->num_scenes, centroids, prim_scene,
                                                      bounds);
    GBRT_LAUNCH_CHECK(ctx, "batch_centroids");
    batch_morton<<<blocks_for(n), kBlock, 0, s>>>(centroids, prim_scene, n, bounds, codes_in, b->sorted_codes,
                                                   b->sorted_ids);
    GBRT_LAUNCH_CHECK(ctx, "batch_morton");
    gbrt_status st = radix_sort_pairs(ctx, b->sorted_codes, b->sorted_ids, keys_alt, vals_alt, n, 30, base + l.sort, s);
    if (st != GBRT_OK) return st;
    if (b->num_scenes > 1)
    {
        int scene_bits = 1;
        while ((1u << scene_bits) < b->num_scenes) ++scene_bits;
        gather_scene_keys<<<blocks_for(n), kBlock, 0, s>>>(b->sorted_ids, prim_scene, n, scene_keys);
        GBRT_LAUNCH_CHECK(ctx, "gather_scene_keys");
        st = radix_sort_pairs(ctx, scene_keys, b->sorted_ids, keys_alt, vals_alt, n, scene_bits, base + l.sort, s);
        if (st != GBRT_OK) return st;
        gather_codes<<<blocks_for(n), kBlock, 0, s>>>(b->sorted_ids, codes_in, n, b->sorted_codes);
        GBRT_LAUNCH_CHECK(ctx, "gather_codes");
    }
    GBRT_CUDA(ctx, cudaMemsetAsync(leaf_parent, 0xFF, size_t(n) * 4, s));
    GBRT_CUDA(ctx, cudaMemsetAsync(arrivals, 0, size_t(n) * 4, s));
    GBRT_CUDA(ctx, cudaMemsetAsync(b->d_height, 0, 4, s));
    if (b->total_inner > 0)
    {
        GBRT_CUDA(ctx, cudaMemsetAsync(b->nodes, 0, size_t(b->total_inner) * sizeof(bvh2_node), s));
        batch_hierarchy<<<blocks_for(b->total_inner), kBlock, 0, s>>>(b->sorted_codes, b->d_offsets, b->d_inner_offsets,
                                                                      b->num_scenes, b->total_inner, b->nodes,
                                                                      leaf_parent, b->ranges);
        GBRT_LAUNCH_CHECK(ctx, "batch_hierarchy");
    }
    batch_refit<<<blocks_for(n), kBlock, 0, s>>>(d_tris, b->sorted_ids, n, b->total_inner, leaf_parent, b->nodes,
                                                 arrivals, b->tris, b->d_height, ctx->d_status);
    GBRT_LAUNCH_CHECK(ctx, "batch_refit");
    ++b->build_gen;
    return GBRT_OK;
}

gbrt_status ensure_batch_wide(gbrt_context* ctx, gbrt_batch* b)
{
    if (b->wide_nodes || b->total_inner == 0) return GBRT_OK;
    // a scene of n triangles has at most 2n / (L + 1) wide nodes above leaves of L
    uint64_t cap = b->num_scenes;
    for (uint32_t s = 0; s < b->num_scenes; ++s)
        cap += 2ull * (b->offsets[s + 1] - b->offsets[s]) / (kLeafMax4 + 1) + 2;
    if (cap > (1ull << 31)) return fail(ctx, GBRT_ERR_TOO_LARGE, "batch: wide collapse too large");
    GBRT_CUDA(ctx, cudaMalloc(&b->wide_nodes, size_t(cap) * sizeof(bvh8_node)));
    GBRT_CUDA(ctx, cudaMalloc(&b->wide_queue[0], size_t(cap) * sizeof(int2)));
    GBRT_CUDA(ctx, cudaMalloc(&b->wide_queue[1], size_t(cap) * sizeof(int2)));
    GBRT_CUDA(ctx, cudaMalloc(&b->wide_counts, (kBatchCollapseLevels + 2) * sizeof(uint32_t)));
    b->wide_cap = uint32_t(cap);
    return GBRT_OK;
}

gbrt_status batch_collapse(gbrt_context* ctx, gbrt_batch* b, uint32_t width, cudaStream_t s)
{
    if (b->total_inner == 0)
    {
        b->collapsed_width = width;
        b->collapsed_gen = b->build_gen;
        return GBRT_OK;
    }
    if (!b->wide_nodes) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch: wide nodes not allocated");
    uint32_t* counts = b->wide_counts;                    // [level], node counter last
    uint32_t* node_counter = counts + kBatchCollapseLevels + 1;
    GBRT_CUDA(ctx, cudaMemsetAsync(counts, 0, (kBatchCollapseLevels + 2) * sizeof(uint32_t), s));
    batch_collapse_seed<<<blocks_for(b->num_scenes), kBlock, 0, s>>>(b->d_roots, b->num_scenes, b->wide_queue[0],
                                                                     counts, node_counter);
    GBRT_LAUNCH_CHECK(ctx, "batch_collapse_seed");
    // every level on a fixed grid (the kernel walks its queue): no host synchronisation
    const uint32_t grid = uint32_t(ctx->num_sms) * 8u;
    for (uint32_t level = 0; level < kBatchCollapseLevels; ++level)
    {
        int2* q_in = b->wide_queue[level & 1];
        int2* q_out = b->wide_queue[(level + 1) & 1];
        if (width == 4)
            collapse_wide<4><<<grid, 256, 0, s>>>(b->nodes, b->ranges, q_in, counts + level, q_out, counts + level + 1,
                                                  static_cast<bvh4_node*>(b->wide_nodes), node_counter, b->wide_cap,
                                                  kLeafMax4, int(b->total_inner), ctx->d_status);
        else
            collapse_wide<8><<<grid, 256, 0, s>>>(b->nodes, b->ranges, q_in, counts + level, q_out, counts + level + 1,
                                                  static_cast<bvh8_node*>(b->wide_nodes), node_counter, b->wide_cap,
                                                  kLeafMax4, int(b->total_inner), ctx->d_status);
        GBRT_LAUNCH_CHECK(ctx, "collapse_wide");
    }
    b->collapsed_width = width;
    b->collapsed_gen = b->build_gen;
    return GBRT_OK;
}

} // namespace gbrt

using namespace gbrt;

extern "C" gbrt_status gbrt_batch_create(gbrt_context* ctx, uint32_t const* h_offsets, uint32_t num_scenes,
                                         gbrt_batch** out)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!out || !h_offsets || num_scenes == 0) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_create: bad argument");
    *out = nullptr;
    if (num_scenes > (1u << 24)) return fail(ctx, GBRT_ERR_TOO_LARGE, "batch_create: more than 2^24 scenes");
    if (h_offsets[0] != 0) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_create: offsets[0] must be 0");
    for (uint32_t k = 0; k < num_scenes; ++k)
        if (h_offsets[k + 1] < h_offsets[k]) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_create: offsets decrease");
    if (h_offsets[num_scenes] > (1u << 29)) return fail(ctx, GBRT_ERR_TOO_LARGE, "batch_create: more than 2^29 triangles");
    device_guard g(ctx->device);
    auto* b = new (std::nothrow) gbrt_batch;
    if (!b) return fail(ctx, GBRT_ERR_OUT_OF_MEMORY, "batch_create: host allocation");
    b->device = ctx->device;
    b->num_scenes = num_scenes;
    b->total = h_offsets[num_scenes];
    b->offsets.assign(h_offsets, h_offsets + num_scenes + 1);
    b->inner_offsets.resize(num_scenes + 1);
    b->roots.resize(num_scenes);
    uint32_t inner = 0;
    for (uint32_t k = 0; k < num_scenes; ++k)
    {
        uint32_t nk = h_offsets[k + 1] - h_offsets[k];
        b->inner_offsets[k] = inner;
        b->roots[k] = nk >= 2 ? int32_t(inner) : (nk == 1 ? ~int32_t(h_offsets[k]) : INT32_MIN);
        inner += nk >= 1 ? nk - 1 : 0;
    }
    b->inner_offsets[num_scenes] = inner;
    b->total_inner = inner;
    auto bail = [&](cudaError_t e, const char* what) {
        free_batch(b);
        delete b;
        return check_cuda(ctx, e, what);
    };
    cudaError_t e = cudaSuccess;
    size_t n = b->total;
    if ((e = cudaMalloc(&b->d_offsets, (num_scenes + 1) * 4)) != cudaSuccess) return bail(e, "batch_create");
    if ((e = cudaMalloc(&b->d_inner_offsets, (num_scenes + 1) * 4)) != cudaSuccess) return bail(e, "batch_create");
    if ((e = cudaMalloc(&b->d_roots, num_scenes * 4)) != cudaSuccess) return bail(e, "batch_create");
    if ((e = cudaMalloc(&b->d_height, 4)) != cudaSuccess) return bail(e, "batch_create");
    if ((e = cudaMalloc(&b->d_work, 4)) != cudaSuccess) return bail(e, "batch_create");
    if (n > 0)
    {
        if ((e = cudaMalloc(&b->tris, n * sizeof(tri48))) != cudaSuccess) return bail(e, "batch_create: triangles");
        if ((e = cudaMalloc(&b->sorted_codes, n * 4)) != cudaSuccess) return bail(e, "batch_create");
        if ((e = cudaMalloc(&b->sorted_ids, n * 4)) != cudaSuccess) return bail(e, "batch_create");
        if (inner > 0 && (e = cudaMalloc(&b->nodes, size_t(inner) * sizeof(bvh2_node))) != cudaSuccess)
            return bail(e, "batch_create: nodes");
        if (inner > 0 && (e = cudaMalloc(&b->ranges, size_t(inner) * sizeof(int2))) != cudaSuccess)
            return bail(e, "batch_create: ranges");
        b->scratch_bytes = scratch_layout(b->total, num_scenes).total;
        if ((e = cudaMalloc(&b->scratch, b->scratch_bytes)) != cudaSuccess) return bail(e, "batch_create: scratch");
    }
    if ((e = cudaMemcpy(b->d_offsets, b->offsets.data(), (num_scenes + 1) * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b->d_inner_offsets, b->inner_offsets.data(), (num_scenes + 1) * 4, cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (e = cudaMemcpy(b->d_roots, b->roots.data(), num_scenes * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(e, "batch_create: copies");
    *out = b;
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_batch_destroy(gbrt_batch* batch)
{
    if (!batch) return GBRT_ERR_INVALID_ARG;
    device_guard g(batch->device);
    free_batch(batch);
    delete batch;
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_batch_build(gbrt_context* ctx, gbrt_batch* batch, gbrt_triangle const* d_tris)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!batch || (batch->total && !d_tris)) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_build: null argument");
    device_guard g(ctx->device);
    return batch_build(ctx, batch, d_tris, ctx->stream);
}

extern "C" gbrt_status gbrt_batch_export_bvh2(gbrt_context* ctx, gbrt_batch const* batch, uint32_t scene,
                                              gbrt_bvh_node* d_nodes, uint32_t* d_indices)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!batch || scene >= batch->num_scenes) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_export_bvh2: bad scene");
    uint32_t n = batch->offsets[scene + 1] - batch->offsets[scene];
    if (n == 0) return GBRT_OK;
    if (!d_nodes || !d_indices) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_export_bvh2: null output");
    device_guard g(ctx->device);
    cudaStream_t s = ctx->stream;
    if (n == 1)
    {
        // the single leaf: its box from the emitted triangle, first_prim 0
        gbrt_bvh_node leaf{};
        tri48 t;
        GBRT_CUDA(ctx, cudaMemcpy(&t, batch->tris + batch->offsets[scene], sizeof(t), cudaMemcpyDeviceToHost));
        float v[3][3] = { { t.t0.x, t.t0.y, t.t0.z },
                          { t.t0.x + t.t1.x, t.t0.y + t.t1.y, t.t0.z + t.t1.z },
                          { t.t0.x + t.t2.x, t.t0.y + t.t2.y, t.t0.z + t.t2.z } };
        for (int a = 0; a < 3; ++a)
        {
            leaf.bbox_min[a] = std::min(std::min(v[0][a], v[1][a]), v[2][a]);
            leaf.bbox_max[a] = std::max(std::max(v[0][a], v[1][a]), v[2][a]);
        }
        leaf.num_prims = 1;
        uint32_t zero = 0;
        GBRT_CUDA(ctx, cudaMemcpyAsync(d_nodes, &leaf, sizeof(leaf), cudaMemcpyHostToDevice, s));
        GBRT_CUDA(ctx, cudaMemcpyAsync(d_indices, &zero, 4, cudaMemcpyHostToDevice, s));
        GBRT_CUDA(ctx, cudaStreamSynchronize(s));
        return GBRT_OK;
    }
    batch_export<<<blocks_for(n - 1), kBlock, 0, s>>>(batch->nodes, int(batch->inner_offsets[scene]), int(n - 1),
                                                      int(batch->offsets[scene]), batch->sorted_ids, d_nodes);
    GBRT_LAUNCH_CHECK(ctx, "batch_export");
    iota_from<<<blocks_for(n), kBlock, 0, s>>>(d_indices, n);
    GBRT_LAUNCH_CHECK(ctx, "iota_from");
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_batch_trace_closest_hit(gbrt_context* ctx, gbrt_batch const* batch, gbrt_ray const* d_rays,
                                                    uint32_t const* h_ray_offsets, gbrt_hit* d_hits)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!batch || !h_ray_offsets) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_trace: null argument");
    uint32_t n = h_ray_offsets[batch->num_scenes];
    if (h_ray_offsets[0] != 0) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_trace: offsets[0] must be 0");
    for (uint32_t k = 0; k < batch->num_scenes; ++k)
        if (h_ray_offsets[k + 1] < h_ray_offsets[k]) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_trace: offsets decrease");
    if (n == 0) return GBRT_OK;
    if (!d_rays || !d_hits || (reinterpret_cast<uintptr_t>(d_rays) & 15u) || (reinterpret_cast<uintptr_t>(d_hits) & 15u))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_trace: null or misaligned buffers");
    device_guard g(ctx->device);
    // the ray offsets travel through the context scratch (enqueue-ordered copy)
    gbrt_status st = ensure_scratch(ctx, size_t(batch->num_scenes + 1) * 4);
    if (st != GBRT_OK) return st;
    uint32_t* d_ro = static_cast<uint32_t*>(ctx->scratch);
    GBRT_CUDA(ctx, cudaMemcpyAsync(d_ro, h_ray_offsets, size_t(batch->num_scenes + 1) * 4, cudaMemcpyHostToDevice,
                                   ctx->stream));
    batch_trace<<<(n + 127) / 128, 128, 0, ctx->stream>>>(batch->nodes, batch->tris, batch->d_roots, d_ro,
                                                          batch->num_scenes, int32_t(batch->total_inner),
                                                          int32_t(batch->total), d_rays, n, d_hits, ctx->d_status);
    GBRT_LAUNCH_CHECK(ctx, "batch_trace");
    GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // the host offsets may go away
    return GBRT_OK;
}
