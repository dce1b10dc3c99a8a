// Device BVH traversal shared by the ray-query kernels (traverse.cu) and the path
// tracer (pathtrace.cu).
//
// Replaces the device branch of visionaray's intersect<Traversal>(ray, bvh, isect)
// (detail/bvh/intersect.inl:166-356), which visits BVH2 nodes one 32-byte box at a
// time with a 5-entry stack and a restart trail.  Here each step fetches one 64-byte
// record (two 256-bit read-only loads) holding both children's boxes, tests both,
// descends into the nearer hit child and pushes the farther one on a per-thread stack
// (Aila & Laine 2009 "while-while" form).  Leaves are contiguous runs of 48-byte
// triangles tested with the reference's exact ray/triangle arithmetic
// (device_math.cuh); a hit is accepted as update_if.h:68-107 does: tmin <= t <= tmax
// and t strictly below the best t so far.  Any-hit returns at the first accepted hit
// (detail/exit_traversal.h:49-56).
#pragma once

#include "api_internal.h"
#include "device_math.cuh"

namespace gbrt {

constexpr int kEmptyLink = INT32_MIN;   // stack sentinel: neither an inner node nor a leaf

__device__ __forceinline__ float4 ldg4(const void* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

struct trace_result
{
    int tri;   // leaf-order triangle index, -1 for a miss
    float t, u, v;
};

// Per-thread traversal stacks: `capacity` entries, set(i, v) / get(i).
template <int N>
struct local_stack
{
    static constexpr int capacity = N;
    int e[N];
    __device__ __forceinline__ void set(int i, int v) { e[i] = v; }
    __device__ __forceinline__ int get(int i) const { return e[i]; }
};

// The first Shared entries in shared memory, one column per thread (entry i of a thread
// at col[i * Stride], Stride = threads per block), so the 32 lanes of a warp touch 32
// different banks whatever their stack depths; deeper entries in local memory.
template <int Shared, int Total, int Stride>
struct shared_stack
{
    static_assert(Total > Shared, "the local part holds at least one entry");
    static constexpr int capacity = Total;
    int* col;
    int spill[Total - Shared];
    __device__ __forceinline__ void set(int i, int v)
    {
        if (i < Shared)
            col[i * Stride] = v;
        else
            spill[i - Shared] = v;
    }
    __device__ __forceinline__ int get(int i) const { return i < Shared ? col[i * Stride] : spill[i - Shared]; }
};

// The next stack entry to visit, kEmptyLink when the stack is empty.
template <class StackT>
__device__ __forceinline__ int pop_entry(StackT& stack, int& sp)
{
    return sp > 0 ? stack.get(--sp) : kEmptyLink;
}

// One node pair as two 256-bit read-only loads (ld.global.nc.v8.f32, sm_100 and later;
// records are 64-byte aligned): half the load instructions of four 128-bit loads.
// Measured on the heightfield workload (kernel alone, same rays and hits): closest hit
// 3.754 -> 3.669 ms, AO any hit 16.63 -> 16.19 ms per launch.
__device__ __forceinline__ void load_pair(const bvh2_node* np, float4& a, float4& b, float4& z, int4& link)
{
    float r[16];
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]), "=f"(r[7])
                 : "l"(np));
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(r[8]), "=f"(r[9]), "=f"(r[10]), "=f"(r[11]), "=f"(r[12]), "=f"(r[13]), "=f"(r[14]), "=f"(r[15])
                 : "l"(reinterpret_cast<const char*>(np) + 32));
    a = make_float4(r[0], r[1], r[2], r[3]);
    b = make_float4(r[4], r[5], r[6], r[7]);
    z = make_float4(r[8], r[9], r[10], r[11]);
    link = make_int4(__float_as_int(r[12]), __float_as_int(r[13]), __float_as_int(r[14]), __float_as_int(r[15]));
}

// A tree taller than the stack's capacity sets kStatusStackOverflow and skips the
// subtrees that did not fit.  t_best: a hit must be strictly closer than this (a
// closer hit found elsewhere, e.g. in another instance); the result's t is t_best
// when nothing closer was found.  NearFirst: of two hit children the nearer is visited
// first (ties to child 1, intersect.inl:283); without it child 0 goes first and the
// entry distances are not compared.  A closest-hit query needs the order.  An any-hit
// query's answer does not depend on it (which occluder it reports does): the ray
// queries' AO rays, short and issue-bound, run unordered (14.52 -> 14.00 ms per
// launch), while path-tracing shadow rays, long and towards a light, meet their
// occluders sooner in order (instanced box frame 781 vs 878 ms).
template <bool AnyHit, class StackT, bool NearFirst = true>
__device__ __forceinline__ trace_result traverse_bvh_with(StackT& stack, const bvh2_node* __restrict__ nodes,
                                                          const tri48* __restrict__ tris, int32_t root,
                                                          int32_t num_inner, int32_t num_tris, f3 o, f3 d,
                                                          float tmin, float tmax, uint32_t* __restrict__ status,
                                                          float t_best = FLT_MAX)
{
    const float ix = safe_rcp(d.x), iy = safe_rcp(d.y), iz = safe_rcp(d.z);
    // the loop carries the best triangle and its t only; u and v are recomputed from
    // that triangle at the end (the same test on the same inputs: the same values),
    // which keeps two registers free in the node loop
    int best_tri = -1;
    float best_t = t_best;

    int sp = 0;
    int node = root;

    while (node != kEmptyLink)
    {
        while (node >= 0)
        {
            if (node >= num_inner)
            {
                atomicOr(status, kStatusBadIndex);
                node = kEmptyLink;
                break;
            }
            float4 a, b, z;
            int4 link;
            load_pair(nodes + node, a, b, z, link);

            // slab test as (box - origin) * inv_dir, like detail/bvh/intersect.inl:257-276
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
            // any hit: best_t only bounds the triangle test (the first hit ends the query),
            // so the children are not culled by it (AO rays 14.00 -> 13.85 ms, same hits)
            bool h0 = tf0 >= tn0 && (AnyHit || tn0 < best_t);
            bool h1 = tf1 >= tn1 && (AnyHit || tn1 < best_t);

            if (h0 && h1)
            {
                bool first0 = !NearFirst || tn0 < tn1;
                int near_child = first0 ? link.x : link.y;
                int far_child = first0 ? link.y : link.x;
                if (sp < StackT::capacity)
                    stack.set(sp++, far_child);
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
                node = pop_entry(stack, sp);
            }
        }
        if (node == kEmptyLink) break;

        // leaf: contiguous triangles from ~node, the last one flagged
        for (int t = ~node;; ++t)
        {
            if (t >= num_tris)
            {
                atomicOr(status, kStatusBadIndex);
                break;
            }
            const tri48* tp = tris + t;
            float4 t0 = ldg4(&tp->t0);
            float4 t1 = ldg4(&tp->t1);
            float4 t2 = ldg4(&tp->t2);
            tri_hit h = intersect_triangle(o, d, { t0.x, t0.y, t0.z }, { t1.x, t1.y, t1.z }, { t2.x, t2.y, t2.z });
            if (h.hit && h.t < best_t && h.t >= tmin && h.t <= tmax)
            {
                if (AnyHit) return trace_result{ t, h.t, h.u, h.v };
                best_tri = t;
                best_t = h.t;
            }
            if (__float_as_uint(t2.w) & kLastInLeaf) break;
        }
        node = pop_entry(stack, sp);
    }
    trace_result best{ best_tri, best_t, 0.0f, 0.0f };
    if (!AnyHit && best_tri >= 0)
    {
        const tri48* tp = tris + best_tri;
        float4 t0 = ldg4(&tp->t0);
        float4 t1 = ldg4(&tp->t1);
        float4 t2 = ldg4(&tp->t2);
        tri_hit h = intersect_triangle(o, d, { t0.x, t0.y, t0.z }, { t1.x, t1.y, t1.z }, { t2.x, t2.y, t2.z });
        best.u = h.u;
        best.v = h.v;
    }
    return best;
}

// Stack: entries of a local-memory stack.
template <bool AnyHit, int Stack = kStackSize>
__device__ __forceinline__ trace_result traverse_bvh(const bvh2_node* __restrict__ nodes,
                                                     const tri48* __restrict__ tris, int32_t root,
                                                     int32_t num_inner, int32_t num_tris, f3 o, f3 d,
                                                     float tmin, float tmax, uint32_t* __restrict__ status)
{
    local_stack<Stack> stack;
    return traverse_bvh_with<AnyHit>(stack, nodes, tris, root, num_inner, num_tris, o, d, tmin, tmax, status);
}

// The child boxes and links of a wide node: eight loads of the plain 4-wide node ...
__device__ __forceinline__ void decode_node(const bvh4_node* __restrict__ np, float lx[4], float hx[4], float ly[4],
                                        float hy[4], float lz[4], float hz[4], int ch[4], int ct[4])
{
    float4 lox = ldg4(&np->lox), hix = ldg4(&np->hix);
    float4 loy = ldg4(&np->loy), hiy = ldg4(&np->hiy);
    float4 loz = ldg4(&np->loz), hiz = ldg4(&np->hiz);
    int4 ch4 = __ldg(&np->child);
    int4 ct4 = __ldg(&np->count);
    lx[0] = lox.x, lx[1] = lox.y, lx[2] = lox.z, lx[3] = lox.w;
    hx[0] = hix.x, hx[1] = hix.y, hx[2] = hix.z, hx[3] = hix.w;
    ly[0] = loy.x, ly[1] = loy.y, ly[2] = loy.z, ly[3] = loy.w;
    hy[0] = hiy.x, hy[1] = hiy.y, hy[2] = hiy.z, hy[3] = hiy.w;
    lz[0] = loz.x, lz[1] = loz.y, lz[2] = loz.z, lz[3] = loz.w;
    hz[0] = hiz.x, hz[1] = hiz.y, hz[2] = hiz.z, hz[3] = hiz.w;
    ch[0] = ch4.x, ch[1] = ch4.y, ch[2] = ch4.z, ch[3] = ch4.w;
    ct[0] = ct4.x, ct[1] = ct4.y, ct[2] = ct4.z, ct[3] = ct4.w;
}

// ... or eight 256-bit loads of the 8-wide node (one per plane, then the links) ...
__device__ __forceinline__ void ld8(const void* p, float r[8])
{
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]), "=f"(r[7])
        : "l"(p));
}

__device__ __forceinline__ void decode_node(const bvh8_node* __restrict__ np, float lx[8], float hx[8], float ly[8],
                                        float hy[8], float lz[8], float hz[8], int ch[8], int ct[8])
{
    ld8(np->lox, lx);
    ld8(np->hix, hx);
    ld8(np->loy, ly);
    ld8(np->hiy, hy);
    ld8(np->loz, lz);
    ld8(np->hiz, hz);
    float c[8], n[8];
    ld8(np->child, c);
    ld8(np->count, n);
#pragma unroll
    for (int k = 0; k < 8; ++k)
    {
        ch[k] = __float_as_int(c[k]);
        ct[k] = __float_as_int(n[k]);
    }
}

// ... or four loads of the quantised node, decoded as origin + q * 2^e rounded down for
// the low and up for the high planes (q * 2^e is exact), so no box shrinks.
__device__ __forceinline__ void decode_node(const bvh4q_node* __restrict__ np, float lx[4], float hx[4], float ly[4],
                                        float hy[4], float lz[4], float hz[4], int ch[4], int ct[4])
{
    const uint4* w = reinterpret_cast<const uint4*>(np);
    const uint4 w0 = __ldg(w), w1 = __ldg(w + 1), w2 = __ldg(w + 2), w3 = __ldg(w + 3);
    const float ox = __uint_as_float(w3.x), oy = __uint_as_float(w3.y), oz = __uint_as_float(w3.z);
    const int ex = int(int8_t(w3.w & 0xFFu)), ey = int(int8_t((w3.w >> 8) & 0xFFu)),
              ez = int(int8_t((w3.w >> 16) & 0xFFu));
    const float sx = __int_as_float((ex + 127) << 23), sy = __int_as_float((ey + 127) << 23),
                sz = __int_as_float((ez + 127) << 23);
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        const int sh = 8 * k;
        lx[k] = __fmaf_rd(float((w0.x >> sh) & 0xFFu), sx, ox);
        ly[k] = __fmaf_rd(float((w0.y >> sh) & 0xFFu), sy, oy);
        lz[k] = __fmaf_rd(float((w0.z >> sh) & 0xFFu), sz, oz);
        hx[k] = __fmaf_ru(float((w0.w >> sh) & 0xFFu), sx, ox);
        hy[k] = __fmaf_ru(float((w1.x >> sh) & 0xFFu), sy, oy);
        hz[k] = __fmaf_ru(float((w1.y >> sh) & 0xFFu), sz, oz);
    }
    // children: {int32 id; int16 count} packed at bytes 24 + 6k
    ch[0] = int(w1.z);
    ct[0] = int(int16_t(w1.w & 0xFFFFu));
    ch[1] = int(__byte_perm(w1.w, w2.x, 0x5432));
    ct[1] = int(int16_t(w2.x >> 16));
    ch[2] = int(w2.y);
    ct[2] = int(int16_t(w2.z & 0xFFFFu));
    ch[3] = int(__byte_perm(w2.z, w2.w, 0x5432));
    ct[3] = int(int16_t(w2.w >> 16));
}

// The same query over W-wide nodes (bvh_layout.cuh: 4-wide plain or quantised,
// 8-wide), from node `root`: one node fetch tests W boxes; hit leaves are tested at
// once (so best.t shrinks before the inner children are ordered), the hit inner
// children are visited nearest first and the others pushed with their entry distance,
// so a popped entry already beyond the best hit is dropped without a fetch.
template <bool AnyHit, int W, typename NodeW>
__device__ __forceinline__ trace_result traverse_bvhw(const NodeW* __restrict__ nodesw, int32_t num_nodesw,
                                                      const tri48* __restrict__ tris, int32_t num_tris, f3 o, f3 d,
                                                      float tmin, float tmax, uint32_t* __restrict__ status,
                                                      int32_t root = 0)
{
    constexpr int kStackW = W == 4 ? kStack4 : kStack8;
    const float ix = safe_rcp(d.x), iy = safe_rcp(d.y), iz = safe_rcp(d.z);
    trace_result best{ -1, FLT_MAX, 0.0f, 0.0f };
    int stack_node[kStackW];
    float stack_t[kStackW];
    int sp = 0;
    int node = root;

    while (true)
    {
        if (node < 0 || node >= num_nodesw)
        {
            atomicOr(status, kStatusBadIndex);
            break;
        }
        float lx[W], hx[W], ly[W], hy[W], lz[W], hz[W];
        int ch[W], ct[W];
        decode_node(nodesw + node, lx, hx, ly, hy, lz, hz, ch, ct);
        float tn[W];
        bool hit[W];
#pragma unroll
        for (int k = 0; k < W; ++k)
        {
            float x0 = (lx[k] - o.x) * ix, x1 = (hx[k] - o.x) * ix;
            float y0 = (ly[k] - o.y) * iy, y1 = (hy[k] - o.y) * iy;
            float z0 = (lz[k] - o.z) * iz, z1 = (hz[k] - o.z) * iz;
            tn[k] = fmaxf(tmin, fmaxf(fminf(x0, x1), fmaxf(fminf(y0, y1), fminf(z0, z1))));
            float tf = fminf(tmax, fminf(fmaxf(x0, x1), fminf(fmaxf(y0, y1), fmaxf(z0, z1))));
            hit[k] = ct[k] >= 0 && tf >= tn[k] && tn[k] < best.t;
        }
        // leaves first
#pragma unroll
        for (int k = 0; k < W; ++k)
        {
            if (!hit[k] || ct[k] <= 0) continue;
            int end = ch[k] + ct[k];
            if (ch[k] < 0 || end > num_tris)
            {
                atomicOr(status, kStatusBadIndex);
                continue;
            }
            for (int t = ch[k]; t < end; ++t)
            {
                const tri48* tp = tris + t;
                float4 t0 = ldg4(&tp->t0);
                float4 t1 = ldg4(&tp->t1);
                float4 t2 = ldg4(&tp->t2);
                tri_hit h = intersect_triangle(o, d, { t0.x, t0.y, t0.z }, { t1.x, t1.y, t1.z },
                                               { t2.x, t2.y, t2.z });
                if (h.hit && h.t < best.t && h.t >= tmin && h.t <= tmax)
                {
                    best = { t, h.t, h.u, h.v };
                    if (AnyHit) return best;
                }
            }
        }
        // inner children nearest first: a W-element insertion order by entry distance
        int order[W];
        float dist[W];
        int m = 0;
#pragma unroll
        for (int k = 0; k < W; ++k)
        {
            if (!hit[k] || ct[k] != 0 || !(tn[k] < best.t)) continue;
            int pos = m;
            while (pos > 0 && dist[pos - 1] > tn[k])
            {
                dist[pos] = dist[pos - 1];
                order[pos] = order[pos - 1];
                --pos;
            }
            dist[pos] = tn[k];
            order[pos] = ch[k];
            ++m;
        }
        if (m > 0)
        {
            for (int j = m - 1; j >= 1; --j)
            {
                if (sp < kStackW)
                {
                    stack_node[sp] = order[j];
                    stack_t[sp] = dist[j];
                    ++sp;
                }
                else
                {
                    atomicOr(status, kStatusStackOverflow);
                }
            }
            node = order[0];
            continue;
        }
        // pop the next entry still in front of the best hit
        node = -1;
        while (sp > 0)
        {
            --sp;
            if (stack_t[sp] < best.t)
            {
                node = stack_node[sp];
                break;
            }
        }
        if (node < 0) break;
    }
    return best;
}

// traverse_bvhw over 4-wide nodes from the root (node 0).
template <bool AnyHit, typename Node4>
__device__ __forceinline__ trace_result traverse_bvh4(const Node4* __restrict__ nodes4, int32_t num_nodes4,
                                                      const tri48* __restrict__ tris, int32_t num_tris, f3 o, f3 d,
                                                      float tmin, float tmax, uint32_t* __restrict__ status)
{
    return traverse_bvhw<AnyHit, 4>(nodes4, num_nodes4, tris, num_tris, o, d, tmin, tmax, status);
}

// Segment lookup of the batched kernels: the s with offs[s] <= i < offs[s + 1]
// (offs: count + 1 non-decreasing entries, offs[count] > i).
__device__ __forceinline__ uint32_t upper_segment(const uint32_t* __restrict__ offs, uint32_t count, uint32_t i)
{
    uint32_t lo = 0, hi = count;
    while (lo < hi)
    {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&offs[mid + 1]) <= i)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Everything a query needs from a BVH handle, passed to kernels by value.
struct bvh_view
{
    const bvh2_node* nodes;
    const bvh4_node* nodes4;
    const bvh4q_node* nodes4q;
    const bvh8_node* nodes8;
    const tri48* tris;
    int32_t root, num_inner, num_nodes4, num_tris, num_nodes8;
};

inline bvh_view view_of(gbrt_bvh const* b)
{
    return { b->nodes, b->nodes4, b->nodes4q, b->nodes8, b->tris, b->root, int32_t(b->num_inner),
             int32_t(b->num_nodes4), int32_t(b->num_prims), int32_t(b->num_nodes8) };
}

// Wide: the 4-wide nodes (present for trees with inner nodes built by the LBVH builder).
template <bool AnyHit, bool Wide>
__device__ __forceinline__ trace_result traverse_view(bvh_view const& v, f3 o, f3 d, float tmin, float tmax,
                                                      uint32_t* __restrict__ status)
{
    if (Wide) return traverse_bvh4<AnyHit>(v.nodes4, v.num_nodes4, v.tris, v.num_tris, o, d, tmin, tmax, status);
    return traverse_bvh<AnyHit>(v.nodes, v.tris, v.root, v.num_inner, v.num_tris, o, d, tmin, tmax, status);
}

// A query through the node pairs with the stack's first Shared entries in shared
// memory (a column per thread of a Block-thread block), or through the 4-wide nodes.
template <bool AnyHit, bool Wide, int Block, int Shared, bool NearFirst = true>
__device__ __forceinline__ trace_result traverse_view_shared(bvh_view const& v, f3 o, f3 d, float tmin, float tmax,
                                                             uint32_t* __restrict__ status)
{
    if constexpr (Wide)
    {
        return traverse_bvh4<AnyHit>(v.nodes4, v.num_nodes4, v.tris, v.num_tris, o, d, tmin, tmax, status);
    }
    else
    {
        __shared__ int stack_mem[Shared * Block];
        shared_stack<Shared, kStackSize, Block> stack;
        stack.col = stack_mem + threadIdx.x;
        return traverse_bvh_with<AnyHit, decltype(stack), NearFirst>(stack, v.nodes, v.tris, v.root, v.num_inner,
                                                                     v.num_tris, o, d, tmin, tmax, status);
    }
}

} // namespace gbrt
