// High-quality BVH build by parallel locally-ordered clustering (PLOC: D. Meister and
// J. Bittner, "Parallel Locally-Ordered Clustering for Bounding Volume Hierarchy
// Construction", IEEE TVCG 24(3), 2018).  Not a visionaray builder: the reference's GPU
// builder is the LBVH (lbvh.cu), whose Morton splits cost the heightfield rays about
// 1.8x the node visits of its binned-SAH tree; this build reaches SAH-like trees on the
// GPU in a few milliseconds and feeds the same node-pair traversal.
//
// Clusters start as the triangles in Morton order (the LBVH's first stages).  Each
// iteration, every cluster finds the neighbour within kRadius positions whose union box
// has the smallest surface area (ties to the lower index); mutual nearest neighbours
// merge into a new node pair at the lower position, and a prefix sum compacts the
// surviving clusters in order and numbers the new nodes.  Iterations repeat until one
// cluster -- the root -- is left.  Node pairs carry both children's boxes, parent links
// and subtree heights, so refits and every traversal kernel apply unchanged; the leaf
// triangles are the Morton-ordered tri48 records of the LBVH.

#include "lbvh_device.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace gbrt {
namespace {

constexpr int kBlock = 256;
constexpr int kRadius = 16;   // neighbours searched on each side
constexpr int kScanItems = 4; // items per thread of the scan
constexpr int kScanTile = kBlock * kScanItems;

inline uint32_t blocks_for(uint64_t n) { return uint32_t((n + kBlock - 1) / kBlock); }
inline size_t align_up(size_t v) { return (v + 255) & ~size_t(255); }

// Leaf clusters: the box of the j-th triangle in Morton order (id ~j, height 0), and
// that triangle's tri48 record.
__global__ void __launch_bounds__(kBlock) ploc_leaves(gbrt_triangle const* __restrict__ tris_in,
                                                      const uint32_t* __restrict__ sorted_ids, uint32_t n,
                                                      float4* __restrict__ lo, float4* __restrict__ hi,
                                                      tri48* __restrict__ tris_out, uint32_t* __restrict__ status)
{
    uint32_t j = blockIdx.x * kBlock + threadIdx.x;
    if (j >= n) return;
    uint32_t id = __ldg(&sorted_ids[j]);
    if (id >= n)
    {
        atomicOr(status, kStatusBadIndex);
        id = 0;
    }
    tri_in t = load_tri(tris_in, id);
    tri48 o;
    o.t0 = make_float4(t.v1.x, t.v1.y, t.v1.z, __uint_as_float(t.prim_id));
    o.t1 = make_float4(t.e1.x, t.e1.y, t.e1.z, __uint_as_float(t.geom_id));
    o.t2 = make_float4(t.e2.x, t.e2.y, t.e2.z, __uint_as_float(kLastInLeaf));
    tris_out[j] = o;
    box3 b = tri_box(t);
    lo[j] = make_float4(b.lo.x, b.lo.y, b.lo.z, __int_as_float(~int(j)));
    hi[j] = make_float4(b.hi.x, b.hi.y, b.hi.z, __int_as_float(0));
}

__device__ __forceinline__ float union_area(float4 alo, float4 ahi, float4 blo, float4 bhi)
{
    float dx = fmaxf(ahi.x, bhi.x) - fminf(alo.x, blo.x);
    float dy = fmaxf(ahi.y, bhi.y) - fminf(alo.y, blo.y);
    float dz = fmaxf(ahi.z, bhi.z) - fminf(alo.z, blo.z);
    return dx * dy + dy * dz + dz * dx;
}

// Nearest neighbour of every cluster within kRadius positions (smallest union area, ties
// to the lower index); the block's clusters and their halo are staged in shared memory.
__global__ void __launch_bounds__(kBlock) ploc_nearest(const float4* __restrict__ lo, const float4* __restrict__ hi,
                                                       uint32_t m, int* __restrict__ nn)
{
    __shared__ float4 slo[kBlock + 2 * kRadius];
    __shared__ float4 shi[kBlock + 2 * kRadius];
    const int64_t b0 = int64_t(blockIdx.x) * kBlock;
    for (int k = threadIdx.x; k < kBlock + 2 * kRadius; k += kBlock)
    {
        int64_t g = b0 - kRadius + k;
        if (g >= 0 && g < int64_t(m))
        {
            slo[k] = lo[g];
            shi[k] = hi[g];
        }
    }
    __syncthreads();
    const int64_t i = b0 + threadIdx.x;
    if (i >= int64_t(m)) return;
    const int li = threadIdx.x + kRadius;
    const float4 alo = slo[li], ahi = shi[li];
    float best = FLT_MAX;
    int best_j = -1;
    const int64_t first = i - kRadius > 0 ? i - kRadius : 0;
    const int64_t last = i + kRadius < int64_t(m) - 1 ? i + kRadius : int64_t(m) - 1;
    for (int64_t j = first; j <= last; ++j)
    {
        if (j == i) continue;
        int lj = int(j - b0) + kRadius;
        float a = union_area(alo, ahi, slo[lj], shi[lj]);
        if (a < best)   // ascending j: ties keep the lower index
        {
            best = a;
            best_j = int(j);
        }
    }
    nn[i] = best_j;
}

// Merge and keep flags: a cluster merges (and owns the new node) when its nearest
// neighbour is mutual and lies after it; it disappears when the mutual neighbour lies
// before it.  Packed as (merge << 32) | keep for one prefix sum of both.
__global__ void __launch_bounds__(kBlock) ploc_flags(const int* __restrict__ nn, uint32_t m,
                                                     unsigned long long* __restrict__ flags)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= m) return;
    int j = nn[i];
    bool mutual = j >= 0 && uint32_t(j) < m && nn[j] == int(i);
    bool merge = mutual && int(i) < j;
    bool removed = mutual && int(i) > j;
    flags[i] = (static_cast<unsigned long long>(merge) << 32) | static_cast<unsigned long long>(!removed);
}

// Exclusive scan of 64-bit values, tile by tile (kScanTile per block), with the tile
// totals written to sums.
__global__ void __launch_bounds__(kBlock) scan_tiles(const unsigned long long* __restrict__ in, uint64_t m,
                                                     unsigned long long* __restrict__ out,
                                                     unsigned long long* __restrict__ sums)
{
    __shared__ unsigned long long warp_tot[kBlock / 32];
    const uint64_t base = uint64_t(blockIdx.x) * kScanTile + uint64_t(threadIdx.x) * kScanItems;
    unsigned long long v[kScanItems];
    unsigned long long run = 0;
    for (int k = 0; k < kScanItems; ++k)
    {
        v[k] = base + k < m ? in[base + k] : 0ull;
        unsigned long long x = v[k];
        v[k] = run;   // exclusive within the thread
        run += x;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long incl = run;
    for (int o = 1; o < 32; o <<= 1)
    {
        unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    unsigned long long warp_base = 0;
    for (int w = 0; w < warp; ++w) warp_base += warp_tot[w];
    const unsigned long long thread_base = warp_base + incl - run;
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < m) out[base + k] = thread_base + v[k];
    if (threadIdx.x == kBlock - 1) sums[blockIdx.x] = warp_base + incl;
}

__global__ void __launch_bounds__(kBlock) scan_add(unsigned long long* __restrict__ data, uint64_t m,
                                                   const unsigned long long* __restrict__ offsets)
{
    const uint64_t base = uint64_t(blockIdx.x) * kScanTile;
    const unsigned long long add = offsets[blockIdx.x];
    for (int k = threadIdx.x; k < kScanTile; k += kBlock)
        if (base + k < m) data[base + k] += add;
}

// Exclusive scan of data[0..m) into out; the total goes to *total.  Scratch holds the
// per-level tile totals (scan_scratch_words(m) 64-bit words).
size_t scan_scratch_words(uint64_t m)
{
    size_t words = 0;
    while (m > 1)
    {
        m = (m + kScanTile - 1) / kScanTile;
        words += 2 * m + 64;
    }
    return words + 64;
}

gbrt_status scan_u64(gbrt_context* ctx, const unsigned long long* in, unsigned long long* out, uint64_t m,
                     unsigned long long* scratch, unsigned long long* total, cudaStream_t s)
{
    if (m == 0) return GBRT_OK;
    const uint64_t tiles = (m + kScanTile - 1) / kScanTile;
    unsigned long long* sums = scratch;
    unsigned long long* sums_scan = scratch + tiles + 32;
    scan_tiles<<<uint32_t(tiles), kBlock, 0, s>>>(in, m, out, sums);
    GBRT_LAUNCH_CHECK(ctx, "scan_tiles");
    if (tiles == 1)
    {
        GBRT_CUDA(ctx, cudaMemcpyAsync(total, sums, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s));
        return GBRT_OK;
    }
    gbrt_status st = scan_u64(ctx, sums, sums_scan, tiles, sums_scan + tiles + 32, total, s);
    if (st != GBRT_OK) return st;
    scan_add<<<uint32_t(tiles), kBlock, 0, s>>>(out, m, sums_scan);
    GBRT_LAUNCH_CHECK(ctx, "scan_add");
    return GBRT_OK;
}

// One clustering step: merging clusters create node pairs [node_base, ...) in order,
// survivors are compacted in order into (out_lo, out_hi).
__global__ void __launch_bounds__(kBlock) ploc_merge(const float4* __restrict__ lo, const float4* __restrict__ hi,
                                                     const int* __restrict__ nn, uint32_t m,
                                                     const unsigned long long* __restrict__ flags,
                                                     const unsigned long long* __restrict__ pre, uint32_t node_base,
                                                     uint32_t num_inner, bvh2_node* __restrict__ nodes,
                                                     float4* __restrict__ out_lo, float4* __restrict__ out_hi,
                                                     uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= m) return;
    const unsigned long long f = flags[i];
    if (!(f & 1ull)) return;
    const unsigned long long p = pre[i];
    const uint32_t dst = uint32_t(p & 0xFFFFFFFFull);
    float4 alo = lo[i], ahi = hi[i];
    if (f >> 32)
    {
        const int j = nn[i];
        const uint32_t node = node_base + uint32_t(p >> 32);
        if (node >= num_inner || j < 0 || uint32_t(j) >= m)
        {
            atomicOr(status, kStatusBadIndex);
            return;
        }
        const float4 blo = lo[j], bhi = hi[j];
        const int ca = __float_as_int(alo.w), cb = __float_as_int(blo.w);
        if (ca >= int(node) || cb >= int(node))   // children were made in earlier steps
        {
            atomicOr(status, kStatusBadIndex);
            return;
        }
        const int height = max(__float_as_int(ahi.w), __float_as_int(bhi.w)) + 1;
        bvh2_node nd;
        nd.xy0 = make_float4(alo.x, ahi.x, alo.y, ahi.y);
        nd.xy1 = make_float4(blo.x, bhi.x, blo.y, bhi.y);
        nd.z01 = make_float4(alo.z, ahi.z, blo.z, bhi.z);
        nd.link = make_int4(ca, cb, height, -1);
        nodes[node] = nd;
        if (ca >= 0) nodes[ca].link.w = int(node << 1) | 0;
        if (cb >= 0) nodes[cb].link.w = int(node << 1) | 1;
        // merged as the LBVH merges (NaN and outward infinities of a leaf box skipped)
        alo = make_float4(ref_min(cas_lo(alo.x), cas_lo(blo.x)), ref_min(cas_lo(alo.y), cas_lo(blo.y)),
                          ref_min(cas_lo(alo.z), cas_lo(blo.z)), __int_as_float(int(node)));
        ahi = make_float4(ref_max(cas_hi(ahi.x), cas_hi(bhi.x)), ref_max(cas_hi(ahi.y), cas_hi(bhi.y)),
                          ref_max(cas_hi(ahi.z), cas_hi(bhi.z)), __int_as_float(height));
    }
    out_lo[dst] = alo;
    out_hi[dst] = ahi;
}

} // namespace

gbrt_status build_ploc(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n, gbrt_bvh* bvh)
{
    bvh->kind = bvh_kind::ploc;
    bvh->num_prims = n;
    bvh->num_inner = n > 0 ? n - 1 : 0;
    bvh->root = n > 1 ? int32_t(n - 2) : ~0;
    bvh->height = 0;
    if (n == 0) return GBRT_OK;
    cudaStream_t s = ctx->stream;
    GBRT_CUDA(ctx, cudaMalloc(&bvh->tris, size_t(n) * sizeof(tri48)));
    GBRT_CUDA(ctx, cudaMalloc(&bvh->sorted_codes, size_t(n) * 4));
    GBRT_CUDA(ctx, cudaMalloc(&bvh->sorted_ids, size_t(n) * 4));
    if (bvh->num_inner > 0) GBRT_CUDA(ctx, cudaMalloc(&bvh->nodes, size_t(bvh->num_inner) * sizeof(bvh2_node)));
    gbrt_status st = morton_order(ctx, d_tris, n, bvh->sorted_codes, bvh->sorted_ids);
    if (st != GBRT_OK) return st;

    // scratch (after the sort): clusters twice, neighbours, flags, prefix, scan levels
    size_t off_lo0 = 0, off_hi0 = align_up(size_t(n) * 16), off_lo1 = off_hi0 + align_up(size_t(n) * 16);
    size_t off_hi1 = off_lo1 + align_up(size_t(n) * 16), off_nn = off_hi1 + align_up(size_t(n) * 16);
    size_t off_flags = off_nn + align_up(size_t(n) * 4), off_pre = off_flags + align_up(size_t(n) * 8);
    size_t off_scan = off_pre + align_up(size_t(n) * 8), off_total = off_scan + align_up(scan_scratch_words(n) * 8);
    st = ensure_scratch(ctx, off_total + 256);
    if (st != GBRT_OK) return st;
    char* base = static_cast<char*>(ctx->scratch);
    float4* lo[2] = { reinterpret_cast<float4*>(base + off_lo0), reinterpret_cast<float4*>(base + off_lo1) };
    float4* hi[2] = { reinterpret_cast<float4*>(base + off_hi0), reinterpret_cast<float4*>(base + off_hi1) };
    int* nn = reinterpret_cast<int*>(base + off_nn);
    auto* flags = reinterpret_cast<unsigned long long*>(base + off_flags);
    auto* pre = reinterpret_cast<unsigned long long*>(base + off_pre);
    auto* scan_scratch = reinterpret_cast<unsigned long long*>(base + off_scan);
    auto* total = reinterpret_cast<unsigned long long*>(base + off_total);

    ploc_leaves<<<blocks_for(n), kBlock, 0, s>>>(d_tris, bvh->sorted_ids, n, lo[0], hi[0], bvh->tris, ctx->d_status);
    GBRT_LAUNCH_CHECK(ctx, "ploc_leaves");
    uint32_t m = n, node_base = 0;
    int cur = 0;
    for (uint32_t iter = 0; m > 1; ++iter)
    {
        if (iter >= n) return fail(ctx, GBRT_ERR_CUDA, "PLOC build: no progress");
        ploc_nearest<<<blocks_for(m), kBlock, 0, s>>>(lo[cur], hi[cur], m, nn);
        GBRT_LAUNCH_CHECK(ctx, "ploc_nearest");
        ploc_flags<<<blocks_for(m), kBlock, 0, s>>>(nn, m, flags);
        GBRT_LAUNCH_CHECK(ctx, "ploc_flags");
        st = scan_u64(ctx, flags, pre, m, scan_scratch, total, s);
        if (st != GBRT_OK) return st;
        ploc_merge<<<blocks_for(m), kBlock, 0, s>>>(lo[cur], hi[cur], nn, m, flags, pre, node_base, bvh->num_inner,
                                                    bvh->nodes, lo[cur ^ 1], hi[cur ^ 1], ctx->d_status);
        GBRT_LAUNCH_CHECK(ctx, "ploc_merge");
        unsigned long long t = 0;
        GBRT_CUDA(ctx, cudaMemcpyAsync(&t, total, sizeof(t), cudaMemcpyDeviceToHost, s));
        GBRT_CUDA(ctx, cudaStreamSynchronize(s));
        const uint32_t merges = uint32_t(t >> 32), keeps = uint32_t(t & 0xFFFFFFFFull);
        if (merges == 0 || keeps != m - merges)
            return fail(ctx, GBRT_ERR_CUDA, "PLOC build: inconsistent merge step");
        node_base += merges;
        m = keeps;
        cur ^= 1;
    }
    if (n > 1)
    {
        if (node_base != n - 1) return fail(ctx, GBRT_ERR_CUDA, "PLOC build: wrong node count");
        float4 root_lo, root_hi;
        GBRT_CUDA(ctx, cudaMemcpyAsync(&root_lo, lo[cur], sizeof(root_lo), cudaMemcpyDeviceToHost, s));
        GBRT_CUDA(ctx, cudaMemcpyAsync(&root_hi, hi[cur], sizeof(root_hi), cudaMemcpyDeviceToHost, s));
        GBRT_CUDA(ctx, cudaStreamSynchronize(s));
        int root = 0, height = 0;
        memcpy(&root, &root_lo.w, 4);
        memcpy(&height, &root_hi.w, 4);
        if (root != int(n - 2)) return fail(ctx, GBRT_ERR_CUDA, "PLOC build: unexpected root");
        bvh->root = root;
        bvh->height = uint32_t(height);
        bvh->lo[0] = root_lo.x;
        bvh->lo[1] = root_lo.y;
        bvh->lo[2] = root_lo.z;
        bvh->hi[0] = root_hi.x;
        bvh->hi[1] = root_hi.y;
        bvh->hi[2] = root_hi.z;
    }
    else
    {
        float4 l, h;
        GBRT_CUDA(ctx, cudaMemcpyAsync(&l, lo[0], sizeof(l), cudaMemcpyDeviceToHost, s));
        GBRT_CUDA(ctx, cudaMemcpyAsync(&h, hi[0], sizeof(h), cudaMemcpyDeviceToHost, s));
        GBRT_CUDA(ctx, cudaStreamSynchronize(s));
        bvh->lo[0] = l.x;
        bvh->lo[1] = l.y;
        bvh->lo[2] = l.z;
        bvh->hi[0] = h.x;
        bvh->hi[1] = h.y;
        bvh->hi[2] = h.z;
    }
    if (bvh->height + 1 > uint32_t(kStackSize))
        return fail(ctx, GBRT_ERR_STACK_OVERFLOW, "PLOC tree height exceeds the traversal stack");
    return GBRT_OK;
}

// The tree in visionaray's index_bvh layout (bvh.h:70-141): nodes numbered breadth
// first with the two children of a node adjacent, one primitive per leaf (first_prim
// = the original index, indices = 0, 1, 2, ...).  Built on the host from the node pairs.
gbrt_status export_generic(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_bvh_node* d_nodes, uint32_t* d_indices)
{
    const uint32_t n = bvh->num_prims;
    if (n == 0) return GBRT_OK;
    std::vector<bvh2_node> pairs(bvh->num_inner);
    std::vector<uint32_t> ids(n);
    cudaStream_t s = ctx->stream;
    if (bvh->num_inner)
        GBRT_CUDA(ctx, cudaMemcpyAsync(pairs.data(), bvh->nodes, pairs.size() * sizeof(bvh2_node),
                                       cudaMemcpyDeviceToHost, s));
    GBRT_CUDA(ctx, cudaMemcpyAsync(ids.data(), bvh->sorted_ids, size_t(n) * 4, cudaMemcpyDeviceToHost, s));
    GBRT_CUDA(ctx, cudaStreamSynchronize(s));
    std::vector<gbrt_bvh_node> out(2 * size_t(n) - 1);
    auto put = [](gbrt_bvh_node& d, float lx, float hx, float ly, float hy, float lz, float hz, uint32_t first,
                  uint16_t count) {
        d.bbox_min[0] = lx;
        d.bbox_max[0] = hx;
        d.bbox_min[1] = ly;
        d.bbox_max[1] = hy;
        d.bbox_min[2] = lz;
        d.bbox_max[2] = hz;
        d.first_child_or_prim = first;
        d.num_prims = count;
        d.ordered_traversal_axis = 0;
        d.ordered_traversal_sign = 0;
    };
    if (n == 1)
    {
        put(out[0], bvh->lo[0], bvh->hi[0], bvh->lo[1], bvh->hi[1], bvh->lo[2], bvh->hi[2], ids[0], 1);
    }
    else
    {
        put(out[0], bvh->lo[0], bvh->hi[0], bvh->lo[1], bvh->hi[1], bvh->lo[2], bvh->hi[2], 1u, 0);
        // (pair node, output slot of its first child)
        std::vector<std::pair<int, uint32_t>> queue{ { bvh->root, 1u } };
        uint32_t next = 3;
        for (size_t q = 0; q < queue.size(); ++q)
        {
            bvh2_node const& nd = pairs[size_t(queue[q].first)];
            const uint32_t slot = queue[q].second;
            const int child[2] = { nd.link.x, nd.link.y };
            const float4 xy[2] = { nd.xy0, nd.xy1 };
            const float zl[2] = { nd.z01.x, nd.z01.z }, zh[2] = { nd.z01.y, nd.z01.w };
            for (int c = 0; c < 2; ++c)
            {
                gbrt_bvh_node& d = out[slot + c];
                if (child[c] < 0)
                {
                    put(d, xy[c].x, xy[c].y, xy[c].z, xy[c].w, zl[c], zh[c], ids[size_t(~child[c])], 1);
                }
                else
                {
                    put(d, xy[c].x, xy[c].y, xy[c].z, xy[c].w, zl[c], zh[c], next, 0);
                    queue.push_back({ child[c], next });
                    next += 2;
                }
            }
        }
    }
    std::vector<uint32_t> idx(n);
    for (uint32_t k = 0; k < n; ++k) idx[k] = k;
    GBRT_CUDA(ctx, cudaMemcpyAsync(d_nodes, out.data(), out.size() * sizeof(gbrt_bvh_node), cudaMemcpyHostToDevice, s));
    GBRT_CUDA(ctx, cudaMemcpyAsync(d_indices, idx.data(), size_t(n) * 4, cudaMemcpyHostToDevice, s));
    GBRT_CUDA(ctx, cudaStreamSynchronize(s));
    return GBRT_OK;
}

} // namespace gbrt
