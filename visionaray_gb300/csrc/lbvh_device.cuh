// Device helpers of the LBVH builders (lbvh.cu: one scene; batch.cu: many scenes in
// one pass): triangle loads and bounds in the reference's arithmetic, Karras splits,
// and the child-box slots of the node pairs used by the bottom-up refit.
#pragma once

#include "api_internal.h"
#include "device_math.cuh"

namespace gbrt {

struct tri_in
{
    f3 v1, e1, e2;
    uint32_t prim_id, geom_id;
};

__device__ __forceinline__ tri_in load_tri(gbrt_triangle const* __restrict__ tris, uint64_t i)
{
    const uint32_t* w = reinterpret_cast<const uint32_t*>(tris + i);
    uint32_t g = __ldg(w + 0), p = __ldg(w + 1);
    tri_in t;
    t.geom_id = g;
    t.prim_id = p;
    t.v1 = { __uint_as_float(__ldg(w + 2)), __uint_as_float(__ldg(w + 3)), __uint_as_float(__ldg(w + 4)) };
    t.e1 = { __uint_as_float(__ldg(w + 5)), __uint_as_float(__ldg(w + 6)), __uint_as_float(__ldg(w + 7)) };
    t.e2 = { __uint_as_float(__ldg(w + 8)), __uint_as_float(__ldg(w + 9)), __uint_as_float(__ldg(w + 10)) };
    return t;
}

struct box3
{
    f3 lo, hi;
};

// get_bounds(triangle) (math/detail/triangle.inl:43-52): insert v1, v1+e1, v1+e2 into
// an invalid box with the reference's min/max forms.
__device__ __forceinline__ box3 tri_box(tri_in const& t)
{
    f3 p1 = { __fadd_rn(t.v1.x, t.e1.x), __fadd_rn(t.v1.y, t.e1.y), __fadd_rn(t.v1.z, t.e1.z) };
    f3 p2 = { __fadd_rn(t.v1.x, t.e2.x), __fadd_rn(t.v1.y, t.e2.y), __fadd_rn(t.v1.z, t.e2.z) };
    box3 b;
    b.lo = { ref_min(FLT_MAX, t.v1.x), ref_min(FLT_MAX, t.v1.y), ref_min(FLT_MAX, t.v1.z) };
    b.hi = { ref_max(-FLT_MAX, t.v1.x), ref_max(-FLT_MAX, t.v1.y), ref_max(-FLT_MAX, t.v1.z) };
    b.lo = { ref_min(b.lo.x, p1.x), ref_min(b.lo.y, p1.y), ref_min(b.lo.z, p1.z) };
    b.hi = { ref_max(b.hi.x, p1.x), ref_max(b.hi.y, p1.y), ref_max(b.hi.z, p1.z) };
    b.lo = { ref_min(b.lo.x, p2.x), ref_min(b.lo.y, p2.y), ref_min(b.lo.z, p2.z) };
    b.hi = { ref_max(b.hi.x, p2.x), ref_max(b.hi.y, p2.y), ref_max(b.hi.z, p2.z) };
    return b;
}

__device__ __forceinline__ f3 box_center(box3 const& b)
{
    return { __fmul_rn(__fadd_rn(b.hi.x, b.lo.x), 0.5f), __fmul_rn(__fadd_rn(b.hi.y, b.lo.y), 0.5f),
             __fmul_rn(__fadd_rn(b.hi.z, b.lo.z), 0.5f) };
}

__device__ __forceinline__ float warp_min(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = ref_min(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = ref_max(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

// Karras delta: common-prefix length of sorted keys i and j, with the index as a
// tie-break for equal keys, -1 outside [0, n).
__device__ __forceinline__ int kdelta(const uint32_t* __restrict__ codes, int n, int i, uint32_t ci, int j)
{
    if (j < 0 || j >= n) return -1;
    uint32_t x = ci ^ __ldg(&codes[j]);
    return x == 0 ? 32 + __clz(uint32_t(i) ^ uint32_t(j)) : __clz(x);
}

// Karras node i of the n sorted keys (lbvh.h:120-185): its key range [first, last] and
// split position (left child covers [first, split], right [split + 1, last]).
__device__ __forceinline__ void karras_node(const uint32_t* __restrict__ codes, int n, int i, int& first, int& last,
                                            int& split)
{
    uint32_t ci = __ldg(&codes[i]);
    int d = kdelta(codes, n, i, ci, i + 1) >= kdelta(codes, n, i, ci, i - 1) ? 1 : -1;
    int dmin = kdelta(codes, n, i, ci, i - d);
    int lmax = 2;
    while (kdelta(codes, n, i, ci, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (kdelta(codes, n, i, ci, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = kdelta(codes, n, i, ci, j);
    int s = 0;
    int t = l;
    do
    {
        t = (t + 1) >> 1;
        if (kdelta(codes, n, i, ci, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    split = i + s * d + min(d, 0);
    first = min(i, j);
    last = max(i, j);
}

__device__ __forceinline__ void store_child_box(bvh2_node* node, int side, box3 const& b)
{
    float4 xy = make_float4(b.lo.x, b.hi.x, b.lo.y, b.hi.y);
    if (side == 0)
    {
        node->xy0 = xy;
        node->z01.x = b.lo.z;
        node->z01.y = b.hi.z;
    }
    else
    {
        node->xy1 = xy;
        node->z01.z = b.lo.z;
        node->z01.w = b.hi.z;
    }
}

// Loads through L2 (bypassing L1): the sibling's box was written by another SM.
__device__ __forceinline__ box3 load_union_cg(bvh2_node* node)
{
    float4 a = __ldcg(&node->xy0);
    float4 b = __ldcg(&node->xy1);
    float4 z = __ldcg(&node->z01);
    box3 r;
    r.lo = { ref_min(cas_lo(a.x), cas_lo(b.x)), ref_min(cas_lo(a.z), cas_lo(b.z)), ref_min(cas_lo(z.x), cas_lo(z.z)) };
    r.hi = { ref_max(cas_hi(a.y), cas_hi(b.y)), ref_max(cas_hi(a.w), cas_hi(b.w)), ref_max(cas_hi(z.y), cas_hi(z.w)) };
    return r;
}

// An inner node's box as the reference's assign_node_bounds leaves it (lbvh.h:332-372):
// the atomic fold of every leaf box below it, NaN and outward infinities skipped.
__device__ __forceinline__ box3 box_union_cas(box3 const& a, box3 const& b)
{
    box3 r;
    r.lo = { ref_min(cas_lo(a.lo.x), cas_lo(b.lo.x)), ref_min(cas_lo(a.lo.y), cas_lo(b.lo.y)),
             ref_min(cas_lo(a.lo.z), cas_lo(b.lo.z)) };
    r.hi = { ref_max(cas_hi(a.hi.x), cas_hi(b.hi.x)), ref_max(cas_hi(a.hi.y), cas_hi(b.hi.y)),
             ref_max(cas_hi(a.hi.z), cas_hi(b.hi.z)) };
    return r;
}

} // namespace gbrt
