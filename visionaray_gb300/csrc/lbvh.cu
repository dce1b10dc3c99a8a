// GPU LBVH construction (Karras, "Maximizing Parallelism in the Construction of BVHs,
// Octrees, and k-d Trees", HPG 2012) -- replaces lbvh_builder::build(cuda_index_bvh<P>{},
// prims, n) of visionaray detail/bvh/lbvh.h:681-844.
//
// Pipeline (all on the context stream, one synchronisation at the end):
//   1. centroid_bounds  : per-triangle bounds and centroid (lbvh.h:215-240), block
//                         min/max reduction, 6 atomics per block on order-preserving
//                         ints (the reference does 6 CAS loops per triangle on one
//                         address).
//   2. morton_codes     : centroid quantised op-for-op as lbvh.h:253-267.
//   3. radix sort       : stable, by the 30-bit code (radix_sort.cu).
//   4. build_hierarchy  : Karras split per inner node (lbvh.h:120-185, 281-330).
//   5. refit_and_emit   : one thread per leaf writes the triangle in leaf order and its
//                         box into the parent's child slot, then climbs; at each node
//                         the SECOND arriving thread continues (an atomic counter per
//                         node) so every node is combined once -- the reference walks
//                         every leaf to the root with 6 CAS loops per level
//                         (lbvh.h:332-372).
// Topology and boxes equal the reference's for identical Morton codes; the node-pair
// layout is gbrt::bvh2_node (bvh_layout.cuh).

#include "collapse.cuh"
#include "lbvh_device.cuh"

#include <algorithm>
#include <vector>

namespace gbrt {
namespace {

constexpr int kBlock = 256;

// cb_ordered: {min.x, min.y, min.z, max.x, max.y, max.z} as order-preserving ints,
// initialised to (+FLT_MAX, -FLT_MAX).
__global__ void __launch_bounds__(kBlock) centroid_bounds(gbrt_triangle const* __restrict__ tris, uint32_t n,
                                                          float4* __restrict__ centroids,
                                                          int* __restrict__ cb_ordered)
{
    float mn[3] = { FLT_MAX, FLT_MAX, FLT_MAX };
    float mx[3] = { -FLT_MAX, -FLT_MAX, -FLT_MAX };
    for (uint64_t i = uint64_t(blockIdx.x) * kBlock + threadIdx.x; i < n; i += uint64_t(gridDim.x) * kBlock)
    {
        box3 b = tri_box(load_tri(tris, i));
        f3 c = box_center(b);
        centroids[i] = make_float4(c.x, c.y, c.z, 0.0f);
        // the reference's atomic fold (lbvh.h:233-238) skips NaN and outward infinities
        mn[0] = ref_min(mn[0], cas_lo(c.x));
        mn[1] = ref_min(mn[1], cas_lo(c.y));
        mn[2] = ref_min(mn[2], cas_lo(c.z));
        mx[0] = ref_max(mx[0], cas_hi(c.x));
        mx[1] = ref_max(mx[1], cas_hi(c.y));
        mx[2] = ref_max(mx[2], cas_hi(c.z));
    }
    __shared__ float red[kBlock / 32][6];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int a = 0; a < 3; ++a)
    {
        mn[a] = warp_min(mn[a]);
        mx[a] = warp_max(mx[a]);
    }
    if (lane == 0)
    {
        for (int a = 0; a < 3; ++a)
        {
            red[warp][a] = mn[a];
            red[warp][3 + a] = mx[a];
        }
    }
    __syncthreads();
    if (threadIdx.x < 6)
    {
        int a = threadIdx.x;
        float v = red[0][a];
        for (int w = 1; w < kBlock / 32; ++w) v = a < 3 ? ref_min(v, red[w][a]) : ref_max(v, red[w][a]);
        if (a < 3)
            atomicMin(&cb_ordered[a], float_to_ordered(v));
        else
            atomicMax(&cb_ordered[a], float_to_ordered(v));
    }
}

__global__ void __launch_bounds__(kBlock) morton_codes(const float4* __restrict__ centroids, uint32_t n,
                                                       const int* __restrict__ cb_ordered,
                                                       uint32_t* __restrict__ keys,
                                                       uint32_t* __restrict__ values)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    box3 cb;
    cb.lo = { ordered_to_float(cb_ordered[0]), ordered_to_float(cb_ordered[1]), ordered_to_float(cb_ordered[2]) };
    cb.hi = { ordered_to_float(cb_ordered[3]), ordered_to_float(cb_ordered[4]), ordered_to_float(cb_ordered[5]) };
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
        // centroid -= center; centroid = (centroid + size * 0.5) / size;
        // centroid = min(max(centroid * 1024, 0), 1023)       (lbvh.h:256-263)
        float v = __fsub_rn(c[a], cc[a]);
        v = __fdiv_rn(__fadd_rn(v, __fmul_rn(cs[a], 0.5f)), cs[a]);
        v = __fmul_rn(v, 1024.0f);
        v = ref_min(ref_max(v, 0.0f), 1023.0f);
        q[a] = static_cast<uint32_t>(v);
    }
    keys[i] = morton3(q[0], q[1], q[2]);
    values[i] = i;
}

// Inner node i of n-1: children into nodes[i].link.{x,y} (inner index, or ~leaf for a
// leaf), parent links for inner children in nodes[c].link.w = (i << 1) | side, for
// leaves in leaf_parent[j].
__global__ void __launch_bounds__(kBlock) build_hierarchy(const uint32_t* __restrict__ codes, int n,
                                                          bvh2_node* __restrict__ nodes,
                                                          int* __restrict__ leaf_parent,
                                                          int2* __restrict__ ranges)
{
    int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n - 1) return;
    int first, last, split;
    karras_node(codes, n, i, first, last, split);
    if (ranges) ranges[i] = make_int2(first, last);   // the sorted primitives under node i

    int left = split, right = split + 1;
    int cl, cr;
    if (left == first)
    {
        cl = ~left;
        leaf_parent[left] = (i << 1) | 0;
    }
    else
    {
        cl = left;
        nodes[left].link.w = (i << 1) | 0;
    }
    if (right == last)
    {
        cr = ~right;
        leaf_parent[right] = (i << 1) | 1;
    }
    else
    {
        cr = right;
        nodes[right].link.w = (i << 1) | 1;
    }
    nodes[i].link.x = cl;
    nodes[i].link.y = cr;
    if (i == 0) nodes[0].link.w = -1;
}

__global__ void __launch_bounds__(kBlock) refit_and_emit(gbrt_triangle const* __restrict__ tris_in,
                                                         const uint32_t* __restrict__ sorted_ids, int n,
                                                         const int* __restrict__ leaf_parent,
                                                         bvh2_node* __restrict__ nodes,
                                                         uint32_t* __restrict__ arrivals,
                                                         tri48* __restrict__ tris_out,
                                                         uint32_t* __restrict__ root_height,
                                                         uint32_t* __restrict__ status)
{
    int j = blockIdx.x * kBlock + threadIdx.x;
    if (j >= n) return;
    tri_in t = load_tri(tris_in, __ldg(&sorted_ids[j]));
    tri48 o;
    o.t0 = make_float4(t.v1.x, t.v1.y, t.v1.z, __uint_as_float(t.prim_id));
    o.t1 = make_float4(t.e1.x, t.e1.y, t.e1.z, __uint_as_float(t.geom_id));
    o.t2 = make_float4(t.e2.x, t.e2.y, t.e2.z, __uint_as_float(kLastInLeaf));
    tris_out[j] = o;

    box3 b = tri_box(t);
    int link = leaf_parent[j];
    int height = 0;   // height of the subtree whose box is `b`
    // a valid tree has at most n-1 levels; the bound only guards against a corrupt link
    for (int step = 0; step < n; ++step)
    {
        if (link < 0 || (link >> 1) >= n - 1)
        {
            atomicOr(status, kStatusBadIndex);
            return;
        }
        int node = link >> 1, side = link & 1;
        bvh2_node* nd = &nodes[node];
        store_child_box(nd, side, b);
        // the subtree height travels in the node's link.z as max over arrivals
        atomicMax(&nd->link.z, height + 1);
        __threadfence();
        if (atomicAdd(&arrivals[node], 1u) == 0) return;   // first arrival stops
        __threadfence();
        b = load_union_cg(nd);
        height = __ldcg(&nd->link.z);
        int up = __ldcg(&nd->link.w);
        if (up < 0)
        {
            *root_height = uint32_t(height);
            return;
        }
        link = up;
    }
    atomicOr(status, kStatusBadIndex);
}

// bvh_compressed_node<4>::init (bvh.h:350-393) on the GPU, rounding outward: origin =
// the node box's low corner, per axis the exponent e of the smallest power of two with
// 255 * 2^e >= the box's extent (rounded up), and per child
// lo = floor(round_down(lo - origin) / 2^e), hi = ceil(round_up(hi - origin) / 2^e);
// the division by 2^e is exact.  Decoding origin + q * 2^e rounded down (lo) or up (hi)
// then never shrinks a box.
__device__ __forceinline__ int quant_exponent(float extent)
{
    float t = __fdiv_ru(extent, 255.0f);
    if (!(t > 0.0f)) return -126;   // flat (or degenerate) axis: every offset is 0
    int ex;
    float m = frexpf(t, &ex);       // t = m * 2^ex, m in [0.5, 1)
    int e = m == 0.5f ? ex - 1 : ex;
    return e < -126 ? -126 : (e > 126 ? 126 : e);
}

__global__ void __launch_bounds__(kBlock) quantize_nodes4(const bvh4_node* __restrict__ nodes4, uint32_t count,
                                                          bvh4q_node* __restrict__ out)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= count) return;
    bvh4_node nd = nodes4[i];
    const float lo[3][4] = { { nd.lox.x, nd.lox.y, nd.lox.z, nd.lox.w },
                             { nd.loy.x, nd.loy.y, nd.loy.z, nd.loy.w },
                             { nd.loz.x, nd.loz.y, nd.loz.z, nd.loz.w } };
    const float hi[3][4] = { { nd.hix.x, nd.hix.y, nd.hix.z, nd.hix.w },
                             { nd.hiy.x, nd.hiy.y, nd.hiy.z, nd.hiy.w },
                             { nd.hiz.x, nd.hiz.y, nd.hiz.z, nd.hiz.w } };
    const int ch[4] = { nd.child.x, nd.child.y, nd.child.z, nd.child.w };
    const int ct[4] = { nd.count.x, nd.count.y, nd.count.z, nd.count.w };
    bvh4q_node q;
    for (int a = 0; a < 3; ++a)
    {
        float mn = FLT_MAX, mx = -FLT_MAX;
        for (int k = 0; k < 4; ++k)
        {
            if (ct[k] < 0) continue;
            mn = fminf(mn, lo[a][k]);
            mx = fmaxf(mx, hi[a][k]);
        }
        if (mn > mx) mn = mx = 0.0f;   // no child (cannot happen for an emitted node)
        const int e = quant_exponent(__fsub_ru(mx, mn));
        const float inv = __int_as_float((127 - e) << 23);   // 2^-e, e in [-126, 126]
        q.origin[a] = mn;
        q.e[a] = (signed char)e;
        for (int k = 0; k < 4; ++k)
        {
            float ql = 0.0f, qh = 0.0f;
            if (ct[k] >= 0)
            {
                ql = floorf(__fsub_rd(lo[a][k], mn) * inv);
                qh = ceilf(__fsub_ru(hi[a][k], mn) * inv);
            }
            q.q[a * 4 + k] = (unsigned char)fminf(fmaxf(ql, 0.0f), 255.0f);
            q.q[12 + a * 4 + k] = (unsigned char)fminf(fmaxf(qh, 0.0f), 255.0f);
        }
    }
    for (int k = 0; k < 4; ++k)
    {
        int32_t id = ct[k] < 0 ? -1 : ch[k];
        int16_t c = ct[k] < 0 ? int16_t(-1) : int16_t(ct[k]);
        memcpy(&q.children[6 * k], &id, 4);
        memcpy(&q.children[6 * k + 4], &c, 2);
    }
    q.pad = 0;
    out[i] = q;
}

__global__ void collapse_root(int2* __restrict__ q, uint32_t* __restrict__ counts, uint32_t* __restrict__ node4_counter)
{
    q[0] = make_int2(0, 0);
    counts[0] = 1;
    *node4_counter = 1;
}

// lbvh::collapse (lbvh.h:374-451): nodes of the cuda_index_bvh layout -- root at 0, the
// children of inner node i at 1+2i and 2+2i, one primitive per leaf with first_prim =
// the original index.
__global__ void __launch_bounds__(kBlock) export_collapse(const bvh2_node* __restrict__ nodes, int num_inner,
                                                          const uint32_t* __restrict__ sorted_ids,
                                                          gbrt_bvh_node* __restrict__ out)
{
    int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= num_inner) return;
    bvh2_node nd = nodes[i];
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
            put(d, cbox[s], __ldg(&sorted_ids[~child[s]]), 1);
        else
            put(d, cbox[s], uint32_t(1 + 2 * child[s]), 0);
    }
    if (i == 0)
    {
        put(out[0], box_union_cas(cbox[0], cbox[1]), 1u, 0);
    }
}

// Single-triangle tree: the root is the leaf (lbvh.h:428-433).
__global__ void export_single_leaf(const tri48* __restrict__ tris, const uint32_t* __restrict__ sorted_ids,
                                   gbrt_bvh_node* __restrict__ out, uint32_t* __restrict__ indices)
{
    tri48 t = tris[0];
    tri_in ti;
    ti.v1 = { t.t0.x, t.t0.y, t.t0.z };
    ti.e1 = { t.t1.x, t.t1.y, t.t1.z };
    ti.e2 = { t.t2.x, t.t2.y, t.t2.z };
    box3 b = tri_box(ti);
    gbrt_bvh_node& d = out[0];
    d.bbox_min[0] = b.lo.x;
    d.bbox_min[1] = b.lo.y;
    d.bbox_min[2] = b.lo.z;
    d.bbox_max[0] = b.hi.x;
    d.bbox_max[1] = b.hi.y;
    d.bbox_max[2] = b.hi.z;
    d.first_child_or_prim = sorted_ids[0];
    d.num_prims = 1;
    d.ordered_traversal_axis = 0;
    d.ordered_traversal_sign = 0;
    indices[0] = 0;
}

// Leaf parents of a built tree, for a refit: inner node i writes (i << 1) | side for
// each leaf child.
__global__ void __launch_bounds__(kBlock) leaf_parents_of(const bvh2_node* __restrict__ nodes, int num_inner,
                                                          int num_leaves, int* __restrict__ leaf_parent,
                                                          uint32_t* __restrict__ status)
{
    int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= num_inner) return;
    int4 link = __ldg(&nodes[i].link);
    const int child[2] = { link.x, link.y };
    for (int side = 0; side < 2; ++side)
    {
        if (child[side] >= 0) continue;
        int j = ~child[side];
        if (j < num_leaves)
            leaf_parent[j] = (i << 1) | side;
        else
            atomicOr(status, kStatusBadIndex);
    }
}

__global__ void emit_single(gbrt_triangle const* __restrict__ tris_in, tri48* __restrict__ tris_out)
{
    tri_in t = load_tri(tris_in, 0);
    tri48 o;
    o.t0 = make_float4(t.v1.x, t.v1.y, t.v1.z, __uint_as_float(t.prim_id));
    o.t1 = make_float4(t.e1.x, t.e1.y, t.e1.z, __uint_as_float(t.geom_id));
    o.t2 = make_float4(t.e2.x, t.e2.y, t.e2.z, __uint_as_float(kLastInLeaf));
    tris_out[0] = o;
}

__global__ void __launch_bounds__(kBlock) iota(uint32_t* __restrict__ out, uint32_t n)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < n) out[i] = i;
}

__global__ void __launch_bounds__(kBlock) scatter_codes(const uint32_t* __restrict__ sorted_codes,
                                                        const uint32_t* __restrict__ sorted_ids, uint32_t n,
                                                        uint32_t* __restrict__ out)
{
    uint32_t j = blockIdx.x * kBlock + threadIdx.x;
    if (j < n) out[sorted_ids[j]] = sorted_codes[j];
}

// Centroid-bounds words (+FLT_MAX x3, -FLT_MAX x3 as ordered ints) and the root
// height word, set on the device so a build needs no host-side staging.
__global__ void init_build_words(int* __restrict__ words)
{
    int t = threadIdx.x;
    if (t < 3) words[t] = float_to_ordered(FLT_MAX);
    else if (t < 6) words[t] = float_to_ordered(-FLT_MAX);
    else if (t < 8) words[t] = t == 6 ? 1 : 0;
}

inline uint32_t blocks_for(uint64_t n) { return uint32_t((n + kBlock - 1) / kBlock); }

inline size_t align_up(size_t v) { return (v + 255) & ~size_t(255); }

} // namespace

// The box of a one-triangle tree: get_bounds(triangle) (math/detail/triangle.inl:43-52)
// on the host, from the device triangle.
gbrt_status set_single_box(gbrt_context* ctx, gbrt_bvh* bvh, gbrt_triangle const* d_tris)
{
    gbrt_triangle t;
    GBRT_CUDA(ctx, cudaMemcpyAsync(&t, d_tris, sizeof(t), cudaMemcpyDeviceToHost, ctx->stream));
    GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    auto mn = [](float a, float b) { return a < b ? a : b; };
    auto mx = [](float a, float b) { return a < b ? b : a; };
    for (int a = 0; a < 3; ++a)
    {
        float p1 = t.v1[a] + t.e1[a], p2 = t.v1[a] + t.e2[a];
        bvh->lo[a] = mn(mn(mn(FLT_MAX, t.v1[a]), p1), p2);
        bvh->hi[a] = mx(mx(mx(-FLT_MAX, t.v1[a]), p1), p2);
    }
    return GBRT_OK;
}

// The scene box: the union of the root's two child boxes with the reference's min / max
// (x < y ? x : y), as the exported root node holds it.
void set_scene_box(gbrt_bvh* bvh, bvh2_node const& root)
{
    auto mn = [](float a, float b) { return a < b ? a : b; };
    auto mx = [](float a, float b) { return a < b ? b : a; };
    bvh->lo[0] = mn(root.xy0.x, root.xy1.x);
    bvh->hi[0] = mx(root.xy0.y, root.xy1.y);
    bvh->lo[1] = mn(root.xy0.z, root.xy1.z);
    bvh->hi[1] = mx(root.xy0.w, root.xy1.w);
    bvh->lo[2] = mn(root.z01.x, root.z01.z);
    bvh->hi[2] = mx(root.z01.y, root.z01.w);
}

gbrt_status build_lbvh(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n, gbrt_bvh* bvh)
{
    bvh->kind = bvh_kind::lbvh;
    bvh->num_prims = n;
    bvh->num_inner = n > 0 ? n - 1 : 0;
    bvh->root = n > 1 ? 0 : ~0;
    bvh->height = n > 1 ? 1 : 0;
    if (n == 0) return GBRT_OK;

    cudaStream_t s = ctx->stream;
    // a rebuild (gbrt_bvh_rebuild_lbvh) of a tree of the same size writes into its arrays
    if (!bvh->tris) GBRT_CUDA(ctx, cudaMalloc(&bvh->tris, size_t(n) * sizeof(tri48)));
    if (!bvh->sorted_codes) GBRT_CUDA(ctx, cudaMalloc(&bvh->sorted_codes, size_t(n) * 4));
    if (!bvh->sorted_ids) GBRT_CUDA(ctx, cudaMalloc(&bvh->sorted_ids, size_t(n) * 4));
    if (bvh->num_inner > 0 && !bvh->nodes)
        GBRT_CUDA(ctx, cudaMalloc(&bvh->nodes, size_t(bvh->num_inner) * sizeof(bvh2_node)));
    if (bvh->nodes4 || bvh->nodes8)
    {
        // a rebuild with a wide collapse from the previous build: its size may change
        GBRT_CUDA(ctx, cudaStreamSynchronize(s));
        free_wide_nodes(bvh);
    }

    // scratch: centroids | keys_alt | vals_alt | leaf_parent | arrivals | cb(6) | height | sort
    size_t off_centroids = 0;
    size_t off_keys_alt = align_up(off_centroids + size_t(n) * 16);
    size_t off_vals_alt = align_up(off_keys_alt + size_t(n) * 4);
    size_t off_parent = align_up(off_vals_alt + size_t(n) * 4);
    size_t off_arrivals = align_up(off_parent + size_t(n) * 4);
    size_t off_cb = align_up(off_arrivals + size_t(n) * 4);
    size_t off_sort = align_up(off_cb + 8 * 4);
    // wide collapse: node ranges, two level queues, per-level counts, node counter and
    // the nodes themselves (a tree with n leaves has at most 2n / (L + 1) nodes above L
    // leaves, the bound on the wide node count for leaves of at most L triangles)
    const int leaf_max = kLeafMax4;
    const uint32_t cap4 = uint32_t(2ull * n / (leaf_max + 1) + 2);
    const size_t wide_bytes = (ctx->trace_flags & GBRT_TRACE_WIDE8_NODES) ? sizeof(bvh8_node) : sizeof(bvh4_node);
    size_t off_ranges = align_up(off_sort + radix_sort_scratch_bytes(n));
    size_t off_q0 = align_up(off_ranges + size_t(n) * 8);
    size_t off_q1 = align_up(off_q0 + size_t(cap4) * 8);
    size_t off_counts = align_up(off_q1 + size_t(cap4) * 8);
    size_t off_nodes4 = align_up(off_counts + 256 * 4);
    size_t total = off_nodes4 + size_t(cap4) * wide_bytes;
    gbrt_status st = ensure_scratch(ctx, total);
    if (st != GBRT_OK) return st;
    char* base = static_cast<char*>(ctx->scratch);
    float4* centroids = reinterpret_cast<float4*>(base + off_centroids);
    uint32_t* keys_alt = reinterpret_cast<uint32_t*>(base + off_keys_alt);
    uint32_t* vals_alt = reinterpret_cast<uint32_t*>(base + off_vals_alt);
    int* leaf_parent = reinterpret_cast<int*>(base + off_parent);
    uint32_t* arrivals = reinterpret_cast<uint32_t*>(base + off_arrivals);
    int* cb = reinterpret_cast<int*>(base + off_cb);
    uint32_t* root_height = reinterpret_cast<uint32_t*>(cb + 6);
    int2* ranges = reinterpret_cast<int2*>(base + off_ranges);
    int2* queue[2] = { reinterpret_cast<int2*>(base + off_q0), reinterpret_cast<int2*>(base + off_q1) };
    uint32_t* level_counts = reinterpret_cast<uint32_t*>(base + off_counts);   // [0..254]
    uint32_t* node4_counter = level_counts + 255;
    void* wide_tmp = base + off_nodes4;

    // cb = (+FLT_MAX x3, -FLT_MAX x3) as ordered ints; root height 1 by default
    int init[8];
    {
        float lo = FLT_MAX, hi = -FLT_MAX;
        int li, hi_i;
        memcpy(&li, &lo, 4);
        memcpy(&hi_i, &hi, 4);
        hi_i = hi_i ^ 0x7FFFFFFF;   // negative float -> ordered int
        for (int a = 0; a < 3; ++a)
        {
            init[a] = li;
            init[3 + a] = hi_i;
        }
        init[6] = 1;
        init[7] = 0;
    }
    GBRT_CUDA(ctx, cudaMemcpyAsync(cb, init, sizeof(init), cudaMemcpyHostToDevice, s));

    uint32_t grid = std::min<uint32_t>(blocks_for(n), uint32_t(ctx->num_sms) * 8);
    centroid_bounds<<<grid, kBlock, 0, s>>>(d_tris, n, centroids, cb);
    GBRT_LAUNCH_CHECK(ctx, "centroid_bounds");
    morton_codes<<<blocks_for(n), kBlock, 0, s>>>(centroids, n, cb, bvh->sorted_codes, bvh->sorted_ids);
    GBRT_LAUNCH_CHECK(ctx, "morton_codes");
    st = radix_sort_pairs(ctx, bvh->sorted_codes, bvh->sorted_ids, keys_alt, vals_alt, n, 30,
                          base + off_sort);
    if (st != GBRT_OK) return st;

    if (n > 1)
    {
        GBRT_CUDA(ctx, cudaMemsetAsync(bvh->nodes, 0, size_t(bvh->num_inner) * sizeof(bvh2_node), s));
        GBRT_CUDA(ctx, cudaMemsetAsync(arrivals, 0, size_t(n) * 4, s));
        GBRT_CUDA(ctx, cudaMemsetAsync(leaf_parent, 0xFF, size_t(n) * 4, s));
        build_hierarchy<<<blocks_for(n - 1), kBlock, 0, s>>>(bvh->sorted_codes, int(n), bvh->nodes, leaf_parent,
                                                             ranges);
        GBRT_LAUNCH_CHECK(ctx, "build_hierarchy");
        refit_and_emit<<<blocks_for(n), kBlock, 0, s>>>(d_tris, bvh->sorted_ids, int(n), leaf_parent, bvh->nodes,
                                                        arrivals, bvh->tris, root_height, ctx->d_status);
        GBRT_LAUNCH_CHECK(ctx, "refit_and_emit");
        uint32_t h = 0;
        bvh2_node root;
        GBRT_CUDA(ctx, cudaMemcpyAsync(&h, root_height, 4, cudaMemcpyDeviceToHost, s));
        GBRT_CUDA(ctx, cudaMemcpyAsync(&root, bvh->nodes, sizeof(root), cudaMemcpyDeviceToHost, s));
        GBRT_CUDA(ctx, cudaStreamSynchronize(s));
        bvh->height = h;
        // scene bounds: the union of the root's two child boxes
        set_scene_box(bvh, root);

        // collapse into wide nodes (on request), one level per launch; the pair tree has
        // h inner levels, so h levels drain every queue
        auto collapse = [&](auto width_tag, uint32_t* out_count) -> gbrt_status {
            constexpr int W = decltype(width_tag)::value;
            if (h + 1 > 254) return fail(ctx, GBRT_ERR_STACK_OVERFLOW, "LBVH height exceeds the collapse levels");
            GBRT_CUDA(ctx, cudaMemsetAsync(level_counts, 0, 256 * 4, s));
            collapse_root<<<1, 1, 0, s>>>(queue[0], level_counts, node4_counter);
            GBRT_LAUNCH_CHECK(ctx, "collapse_root");
            auto* nodes_tmp = static_cast<typename wide_node<W>::type*>(wide_tmp);
            uint64_t width = 1;
            for (uint32_t level = 0; level < h; ++level)
            {
                uint32_t items = uint32_t(std::max<uint64_t>(1, std::min<uint64_t>(width, cap4)));
                collapse_wide<W><<<blocks_for(items), kBlock, 0, s>>>(
                    bvh->nodes, ranges, queue[level & 1], level_counts + level, queue[(level + 1) & 1],
                    level_counts + level + 1, nodes_tmp, node4_counter, cap4, leaf_max, int(n - 1), ctx->d_status);
                GBRT_LAUNCH_CHECK(ctx, "collapse_wide");
                if (width < cap4) width *= W;   // saturates: W^level overflows past a few dozen levels
            }
            uint32_t tail[2] = { 0, 0 };
            GBRT_CUDA(ctx, cudaMemcpyAsync(&tail[0], level_counts + h, 4, cudaMemcpyDeviceToHost, s));
            GBRT_CUDA(ctx, cudaMemcpyAsync(&tail[1], node4_counter, 4, cudaMemcpyDeviceToHost, s));
            GBRT_CUDA(ctx, cudaStreamSynchronize(s));
            if (tail[0] != 0 || tail[1] == 0 || tail[1] > cap4)
                return fail(ctx, GBRT_ERR_CUDA, "wide collapse did not complete");
            *out_count = tail[1];
            return GBRT_OK;
        };
        if (ctx->trace_flags & (GBRT_TRACE_WIDE_NODES | GBRT_TRACE_COMPRESSED_NODES))
        {
            uint32_t count = 0;
            st = collapse(std::integral_constant<int, 4>{}, &count);
            if (st != GBRT_OK) return st;
            bvh->num_nodes4 = count;
            bvh->leaf_max4 = uint32_t(leaf_max);
            GBRT_CUDA(ctx, cudaMalloc(&bvh->nodes4, size_t(count) * sizeof(bvh4_node)));
            GBRT_CUDA(ctx, cudaMemcpyAsync(bvh->nodes4, wide_tmp, size_t(count) * sizeof(bvh4_node),
                                           cudaMemcpyDeviceToDevice, s));
            if (ctx->trace_flags & GBRT_TRACE_COMPRESSED_NODES)
            {
                GBRT_CUDA(ctx, cudaMalloc(&bvh->nodes4q, size_t(count) * sizeof(bvh4q_node)));
                quantize_nodes4<<<blocks_for(count), kBlock, 0, s>>>(bvh->nodes4, count, bvh->nodes4q);
                GBRT_LAUNCH_CHECK(ctx, "quantize_nodes4");
            }
        }
        if (ctx->trace_flags & GBRT_TRACE_WIDE8_NODES)
        {
            uint32_t count = 0;
            st = collapse(std::integral_constant<int, 8>{}, &count);
            if (st != GBRT_OK) return st;
            bvh->num_nodes8 = count;
            GBRT_CUDA(ctx, cudaMalloc(&bvh->nodes8, size_t(count) * sizeof(bvh8_node)));
            GBRT_CUDA(ctx, cudaMemcpyAsync(bvh->nodes8, wide_tmp, size_t(count) * sizeof(bvh8_node),
                                           cudaMemcpyDeviceToDevice, s));
        }
    }
    else
    {
        // one triangle: it is the root leaf (lbvh.h:428-433)
        emit_single<<<1, 1, 0, s>>>(d_tris, bvh->tris);
        GBRT_LAUNCH_CHECK(ctx, "emit_single");
        st = set_single_box(ctx, bvh, d_tris);
        if (st != GBRT_OK) return st;
    }
    if (bvh->height + 1 > uint32_t(kStackSize))
        return fail(ctx, GBRT_ERR_STACK_OVERFLOW, "LBVH height exceeds the traversal stack");
    return GBRT_OK;
}

// bvh_refitter::refit (detail/bvh/refit.h:25-117) on the GPU: the tree keeps its
// topology and leaf order; the leaf triangles are re-emitted from the new positions and
// every node's boxes recomputed bottom-up by the build's refit kernel (second arrival
// continues).  The 4-wide collapse, if any, is dropped (queries fall back to the pairs).
gbrt_status refit_lbvh(gbrt_context* ctx, gbrt_bvh* bvh, gbrt_triangle const* d_tris)
{
    const uint32_t n = bvh->num_prims;
    if (n == 0) return GBRT_OK;
    cudaStream_t s = ctx->stream;
    if (bvh->nodes4 || bvh->nodes8)
    {
        GBRT_CUDA(ctx, cudaStreamSynchronize(s));
        free_wide_nodes(bvh);
    }
    if (n == 1)
    {
        emit_single<<<1, 1, 0, s>>>(d_tris, bvh->tris);
        GBRT_LAUNCH_CHECK(ctx, "emit_single");
        return set_single_box(ctx, bvh, d_tris);
    }
    const size_t off_parent = 0, off_arrivals = align_up(size_t(n) * 4), off_height = align_up(off_arrivals + size_t(n) * 4);
    gbrt_status st = ensure_scratch(ctx, off_height + 256);
    if (st != GBRT_OK) return st;
    char* base = static_cast<char*>(ctx->scratch);
    int* leaf_parent = reinterpret_cast<int*>(base + off_parent);
    uint32_t* arrivals = reinterpret_cast<uint32_t*>(base + off_arrivals);
    uint32_t* root_height = reinterpret_cast<uint32_t*>(base + off_height);
    GBRT_CUDA(ctx, cudaMemsetAsync(leaf_parent, 0xFF, size_t(n) * 4, s));
    GBRT_CUDA(ctx, cudaMemsetAsync(arrivals, 0, size_t(n) * 4, s));
    leaf_parents_of<<<blocks_for(bvh->num_inner), kBlock, 0, s>>>(bvh->nodes, int(bvh->num_inner), int(n),
                                                                  leaf_parent, ctx->d_status);
    GBRT_LAUNCH_CHECK(ctx, "leaf_parents_of");
    refit_and_emit<<<blocks_for(n), kBlock, 0, s>>>(d_tris, bvh->sorted_ids, int(n), leaf_parent, bvh->nodes, arrivals,
                                                    bvh->tris, root_height, ctx->d_status);
    GBRT_LAUNCH_CHECK(ctx, "refit_and_emit");
    bvh2_node root;
    GBRT_CUDA(ctx, cudaMemcpyAsync(&root, bvh->nodes + (bvh->root > 0 ? bvh->root : 0), sizeof(root),
                                   cudaMemcpyDeviceToHost, s));
    GBRT_CUDA(ctx, cudaStreamSynchronize(s));
    set_scene_box(bvh, root);
    return GBRT_OK;
}

// Morton order of n triangles (the LBVH build's first three stages): codes_out[j] /
// ids_out[j] = the code and the input index of the j-th triangle in order.  Uses the
// context scratch; stream-ordered, no synchronisation.
gbrt_status morton_order(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n, uint32_t* codes_out,
                         uint32_t* ids_out)
{
    if (n == 0) return GBRT_OK;
    cudaStream_t s = ctx->stream;
    size_t off_centroids = 0;
    size_t off_keys_alt = align_up(off_centroids + size_t(n) * 16);
    size_t off_vals_alt = align_up(off_keys_alt + size_t(n) * 4);
    size_t off_cb = align_up(off_vals_alt + size_t(n) * 4);
    size_t off_sort = align_up(off_cb + 8 * 4);
    gbrt_status st = ensure_scratch(ctx, off_sort + radix_sort_scratch_bytes(n));
    if (st != GBRT_OK) return st;
    char* base = static_cast<char*>(ctx->scratch);
    float4* centroids = reinterpret_cast<float4*>(base + off_centroids);
    int* cb = reinterpret_cast<int*>(base + off_cb);
    init_build_words<<<1, 8, 0, s>>>(cb);
    GBRT_LAUNCH_CHECK(ctx, "init_build_words");
    uint32_t grid = std::min<uint32_t>(blocks_for(n), uint32_t(ctx->num_sms) * 8);
    centroid_bounds<<<grid, kBlock, 0, s>>>(d_tris, n, centroids, cb);
    GBRT_LAUNCH_CHECK(ctx, "centroid_bounds");
    morton_codes<<<blocks_for(n), kBlock, 0, s>>>(centroids, n, cb, codes_out, ids_out);
    GBRT_LAUNCH_CHECK(ctx, "morton_codes");
    return radix_sort_pairs(ctx, codes_out, ids_out, reinterpret_cast<uint32_t*>(base + off_keys_alt),
                            reinterpret_cast<uint32_t*>(base + off_vals_alt), n, 30, base + off_sort);
}

gbrt_status export_bvh2(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_bvh_node* d_nodes, uint32_t* d_indices)
{
    if (bvh->kind == bvh_kind::ploc) return export_generic(ctx, bvh, d_nodes, d_indices);
    if (bvh->kind != bvh_kind::lbvh) return fail(ctx, GBRT_ERR_INVALID_ARG, "export_bvh2: not a built tree");
    uint32_t n = bvh->num_prims;
    if (n == 0) return GBRT_OK;
    cudaStream_t s = ctx->stream;
    if (n == 1)
    {
        export_single_leaf<<<1, 1, 0, s>>>(bvh->tris, bvh->sorted_ids, d_nodes, d_indices);
        GBRT_LAUNCH_CHECK(ctx, "export_single_leaf");
        return GBRT_OK;
    }
    export_collapse<<<blocks_for(bvh->num_inner), kBlock, 0, s>>>(bvh->nodes, int(bvh->num_inner), bvh->sorted_ids,
                                                                  d_nodes);
    GBRT_LAUNCH_CHECK(ctx, "export_collapse");
    iota<<<blocks_for(n), kBlock, 0, s>>>(d_indices, n);
    GBRT_LAUNCH_CHECK(ctx, "iota");
    return GBRT_OK;
}

gbrt_status morton_codes_input_order(gbrt_context* ctx, gbrt_bvh const* bvh, uint32_t* d_codes)
{
    if (bvh->kind != bvh_kind::lbvh && bvh->kind != bvh_kind::ploc)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "morton_codes: not a built tree");
    if (bvh->num_prims == 0) return GBRT_OK;
    scatter_codes<<<blocks_for(bvh->num_prims), kBlock, 0, ctx->stream>>>(bvh->sorted_codes, bvh->sorted_ids,
                                                                           bvh->num_prims, d_codes);
    GBRT_LAUNCH_CHECK(ctx, "scatter_codes");
    return GBRT_OK;
}

gbrt_status build_lbvh_in_scratch(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n, void* scratch,
                                  size_t scratch_bytes, gbrt_bvh_node* d_nodes, uint32_t* d_indices)
{
    if (n == 0) return GBRT_OK;
    const lbvh_scratch_layout l = lbvh_scratch_layout_for(n);
    if (l.total > scratch_bytes || radix_sort_scratch_bytes(n) > l.total - l.sort)
        return fail(ctx, GBRT_ERR_TOO_LARGE, "LBVH build: scratch region too small for this many triangles");
    char* base = static_cast<char*>(scratch);
    float4* centroids = reinterpret_cast<float4*>(base + l.centroids);
    uint32_t* keys = reinterpret_cast<uint32_t*>(base + l.keys);
    uint32_t* vals = reinterpret_cast<uint32_t*>(base + l.vals);
    uint32_t* keys_alt = reinterpret_cast<uint32_t*>(base + l.keys_alt);
    uint32_t* vals_alt = reinterpret_cast<uint32_t*>(base + l.vals_alt);
    int* leaf_parent = reinterpret_cast<int*>(base + l.leaf_parent);
    uint32_t* arrivals = reinterpret_cast<uint32_t*>(base + l.arrivals);
    bvh2_node* nodes = reinterpret_cast<bvh2_node*>(base + l.nodes);
    tri48* tris = reinterpret_cast<tri48*>(base + l.tris);
    int* words = reinterpret_cast<int*>(base + l.words);
    uint32_t* root_height = reinterpret_cast<uint32_t*>(words + 6);
    cudaStream_t s = ctx->stream;

    init_build_words<<<1, 32, 0, s>>>(words);
    GBRT_LAUNCH_CHECK(ctx, "init_build_words");
    uint32_t grid = std::min<uint32_t>(blocks_for(n), uint32_t(ctx->num_sms) * 8);
    centroid_bounds<<<grid, kBlock, 0, s>>>(d_tris, n, centroids, words);
    GBRT_LAUNCH_CHECK(ctx, "centroid_bounds");
    morton_codes<<<blocks_for(n), kBlock, 0, s>>>(centroids, n, words, keys, vals);
    GBRT_LAUNCH_CHECK(ctx, "morton_codes");
    gbrt_status st = radix_sort_pairs(ctx, keys, vals, keys_alt, vals_alt, n, 30, base + l.sort);
    if (st != GBRT_OK) return st;

    if (n == 1)
    {
        emit_single<<<1, 1, 0, s>>>(d_tris, tris);
        GBRT_LAUNCH_CHECK(ctx, "emit_single");
        export_single_leaf<<<1, 1, 0, s>>>(tris, vals, d_nodes, d_indices);
        GBRT_LAUNCH_CHECK(ctx, "export_single_leaf");
        return GBRT_OK;
    }
    // every call starts from cleared nodes, arrival counters and parent links: the
    // region keeps whatever the previous build left in it
    GBRT_CUDA(ctx, cudaMemsetAsync(nodes, 0, size_t(n - 1) * sizeof(bvh2_node), s));
    GBRT_CUDA(ctx, cudaMemsetAsync(arrivals, 0, size_t(n) * 4, s));
    GBRT_CUDA(ctx, cudaMemsetAsync(leaf_parent, 0xFF, size_t(n) * 4, s));
    build_hierarchy<<<blocks_for(n - 1), kBlock, 0, s>>>(keys, int(n), nodes, leaf_parent, nullptr);
    GBRT_LAUNCH_CHECK(ctx, "build_hierarchy");
    refit_and_emit<<<blocks_for(n), kBlock, 0, s>>>(d_tris, vals, int(n), leaf_parent, nodes, arrivals, tris,
                                                    root_height, ctx->d_status);
    GBRT_LAUNCH_CHECK(ctx, "refit_and_emit");
    export_collapse<<<blocks_for(n - 1), kBlock, 0, s>>>(nodes, int(n - 1), vals, d_nodes);
    GBRT_LAUNCH_CHECK(ctx, "export_collapse");
    iota<<<blocks_for(n), kBlock, 0, s>>>(d_indices, n);
    GBRT_LAUNCH_CHECK(ctx, "iota");
    return GBRT_OK;
}

// Host conversion of a visionaray index BVH (bvh_node + indices) into the node-pair
// layout: inner nodes renumbered in depth-first order, each leaf's primitives copied
// contiguously in leaf order with the last one flagged.
gbrt_status upload_bvh2(gbrt_context* ctx, gbrt_bvh_node const* nodes, uint32_t num_nodes,
                        uint32_t const* indices, uint32_t num_indices, gbrt_triangle const* tris,
                        uint32_t num_tris, gbrt_bvh* bvh)
{
    bvh->kind = bvh_kind::uploaded;
    bvh->num_prims = num_tris;
    if (num_nodes == 0 || num_tris == 0)
    {
        bvh->num_inner = 0;
        bvh->root = ~0;
        bvh->num_prims = 0;
        return GBRT_OK;
    }
    std::vector<int32_t> inner_id(num_nodes, -1);
    std::vector<uint32_t> order;   // reference inner nodes in DFS order
    std::vector<tri48> out_tris;
    std::vector<int32_t> leaf_ref(num_nodes, 0);
    out_tris.reserve(num_indices);

    auto emit_leaf = [&](uint32_t r) -> gbrt_status {
        gbrt_bvh_node const& nd = nodes[r];
        if (nd.num_prims == 0) return GBRT_OK;
        if (uint64_t(nd.first_child_or_prim) + nd.num_prims > num_indices)
            return fail(ctx, GBRT_ERR_INVALID_ARG, "upload_bvh2: leaf range outside the index list");
        leaf_ref[r] = ~int32_t(out_tris.size());
        for (uint32_t k = 0; k < nd.num_prims; ++k)
        {
            uint32_t pi = indices[nd.first_child_or_prim + k];
            if (pi >= num_tris) return fail(ctx, GBRT_ERR_INVALID_ARG, "upload_bvh2: index outside triangles");
            gbrt_triangle const& t = tris[pi];
            tri48 o;
            uint32_t flags = k + 1 == nd.num_prims ? kLastInLeaf : 0u;
            o.t0 = make_float4(t.v1[0], t.v1[1], t.v1[2], 0.0f);
            o.t1 = make_float4(t.e1[0], t.e1[1], t.e1[2], 0.0f);
            o.t2 = make_float4(t.e2[0], t.e2[1], t.e2[2], 0.0f);
            memcpy(&o.t0.w, &t.prim_id, 4);
            memcpy(&o.t1.w, &t.geom_id, 4);
            memcpy(&o.t2.w, &flags, 4);
            out_tris.push_back(o);
        }
        return GBRT_OK;
    };

    // depth-first numbering of inner nodes, leaves emitted in visiting order
    std::vector<std::pair<uint32_t, uint32_t>> st{ { 0u, 1u } };
    uint32_t height = 0;
    while (!st.empty())
    {
        auto [r, depth] = st.back();
        st.pop_back();
        if (r >= num_nodes) return fail(ctx, GBRT_ERR_INVALID_ARG, "upload_bvh2: child outside the node list");
        gbrt_bvh_node const& nd = nodes[r];
        if (nd.num_prims != 0)
        {
            gbrt_status e = emit_leaf(r);
            if (e != GBRT_OK) return e;
            continue;
        }
        if (inner_id[r] >= 0) return fail(ctx, GBRT_ERR_INVALID_ARG, "upload_bvh2: node reached twice");
        inner_id[r] = int32_t(order.size());
        order.push_back(r);
        height = std::max(height, depth);
        st.push_back({ nd.first_child_or_prim + 1, depth + 1 });
        st.push_back({ nd.first_child_or_prim + 0, depth + 1 });
    }

    std::vector<bvh2_node> out_nodes(order.size());
    for (size_t k = 0; k < order.size(); ++k)
    {
        gbrt_bvh_node const& nd = nodes[order[k]];
        int32_t ch[2];
        gbrt_bvh_node const* cn[2];
        for (int s = 0; s < 2; ++s)
        {
            uint32_t c = nd.first_child_or_prim + uint32_t(s);
            cn[s] = &nodes[c];
            ch[s] = cn[s]->num_prims != 0 ? leaf_ref[c] : inner_id[c];
        }
        bvh2_node& o = out_nodes[k];
        o.xy0 = make_float4(cn[0]->bbox_min[0], cn[0]->bbox_max[0], cn[0]->bbox_min[1], cn[0]->bbox_max[1]);
        o.xy1 = make_float4(cn[1]->bbox_min[0], cn[1]->bbox_max[0], cn[1]->bbox_min[1], cn[1]->bbox_max[1]);
        o.z01 = make_float4(cn[0]->bbox_min[2], cn[0]->bbox_max[2], cn[1]->bbox_min[2], cn[1]->bbox_max[2]);
        o.link = make_int4(ch[0], ch[1], 0, -1);
    }

    bvh->num_inner = uint32_t(out_nodes.size());
    bvh->root = nodes[0].num_prims != 0 ? leaf_ref[0] : 0;
    for (int a = 0; a < 3; ++a)
    {
        bvh->lo[a] = nodes[0].bbox_min[a];
        bvh->hi[a] = nodes[0].bbox_max[a];
    }
    bvh->height = height;
    bvh->num_prims = uint32_t(out_tris.size());
    if (height + 1 > uint32_t(kStackSize))
        return fail(ctx, GBRT_ERR_STACK_OVERFLOW, "uploaded BVH deeper than the traversal stack");
    if (!out_nodes.empty())
    {
        GBRT_CUDA(ctx, cudaMalloc(&bvh->nodes, out_nodes.size() * sizeof(bvh2_node)));
        GBRT_CUDA(ctx, cudaMemcpy(bvh->nodes, out_nodes.data(), out_nodes.size() * sizeof(bvh2_node),
                                  cudaMemcpyHostToDevice));
    }
    GBRT_CUDA(ctx, cudaMalloc(&bvh->tris, out_tris.size() * sizeof(tri48)));
    GBRT_CUDA(ctx, cudaMemcpy(bvh->tris, out_tris.data(), out_tris.size() * sizeof(tri48), cudaMemcpyHostToDevice));
    return GBRT_OK;
}

} // namespace gbrt
