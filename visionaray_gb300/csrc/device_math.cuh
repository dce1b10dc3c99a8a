// Device arithmetic of the hot path with explicit IEEE-754 rounding.
//
// nvcc contracts a*b + c into one fused multiply-add by default; visionaray's CPU
// path (the parity reference) rounds every product and sum separately.  Every
// expression here that feeds a result compared with that path uses the _rn
// intrinsics so that each operation is rounded exactly once, in the reference's
// order.  Division by a triangle's determinant is the correctly rounded 1/x
// (__frcp_rn), which equals the reference's `1.0f / div`.
#pragma once

#include <cfloat>
#include <cstdint>

namespace gbrt {

// min(x, y) = x < y ? x : y and max(x, y) = x < y ? y : x (visionaray
// math/detail/math.h:118-128).  Used where the reference's NaN behaviour matters
// (Morton quantisation, bounds).  Traversal box tests use fminf/fmaxf.
__device__ __forceinline__ float ref_min(float x, float y) { return x < y ? x : y; }
__device__ __forceinline__ float ref_max(float x, float y) { return x < y ? y : x; }

// The reference's float atomicMin / atomicMax (detail/bvh/lbvh.h:63-91) is a
// compare-and-swap loop from +FLT_MAX / -FLT_MAX that stores a value only when it lies
// below (above) the current one: NaN, +Inf into a minimum and -Inf into a maximum are
// never stored.  ref_min / ref_max over cas_lo / cas_hi of the arguments give those
// bounds in any order of arrival (signed zeros aside).
__device__ __forceinline__ float cas_lo(float x) { return x < FLT_MAX ? x : FLT_MAX; }
__device__ __forceinline__ float cas_hi(float x) { return x > -FLT_MAX ? x : -FLT_MAX; }

struct f3
{
    float x, y, z;
};

__device__ __forceinline__ f3 sub_rn(f3 a, f3 b)
{
    return { __fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z) };
}

// cross(u, v) of math/detail/vector3.inl:292-300, each product rounded.
__device__ __forceinline__ f3 cross_rn(f3 u, f3 v)
{
    return { __fsub_rn(__fmul_rn(u.y, v.z), __fmul_rn(u.z, v.y)),
             __fsub_rn(__fmul_rn(u.z, v.x), __fmul_rn(u.x, v.z)),
             __fsub_rn(__fmul_rn(u.x, v.y), __fmul_rn(u.y, v.x)) };
}

// dot(u, v) = (u.x*v.x + u.y*v.y) + u.z*v.z (math/detail/vector3.inl:304-307).
__device__ __forceinline__ float dot_rn(f3 u, f3 v)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(u.x, v.x), __fmul_rn(u.y, v.y)), __fmul_rn(u.z, v.z));
}

struct tri_hit
{
    bool hit;
    float t, u, v;
};

// Ray / triangle test of visionaray math/intersect.h:176-229: two-sided, rejects only
// a zero determinant, barycentric bounds b1 in [0,1], b2 >= 0, b1 + b2 <= 1.
__device__ __forceinline__ tri_hit intersect_triangle(f3 ori, f3 dir, f3 v1, f3 e1, f3 e2)
{
    tri_hit r{ false, -1.0f, 0.0f, 0.0f };
    f3 s1 = cross_rn(dir, e2);
    float div = dot_rn(s1, e1);
    if (!(div != 0.0f)) return r;
    float inv_div = __frcp_rn(div);
    f3 d = sub_rn(ori, v1);
    float b1 = __fmul_rn(dot_rn(d, s1), inv_div);
    if (!(b1 >= 0.0f && b1 <= 1.0f)) return r;
    f3 s2 = cross_rn(d, e1);
    float b2 = __fmul_rn(dot_rn(dir, s2), inv_div);
    if (!(b2 >= 0.0f && __fadd_rn(b1, b2) <= 1.0f)) return r;
    r.hit = true;
    r.t = __fmul_rn(dot_rn(e2, s2), inv_div);
    r.u = b1;
    r.v = b2;
    return r;
}

// Reciprocal direction as the reference forms it (detail/bvh/intersect.inl:62-67):
// 1/d, or FLT_MAX for a zero component.
__device__ __forceinline__ float safe_rcp(float d) { return d != 0.0f ? __frcp_rn(d) : FLT_MAX; }

// 30-bit Morton code: bit i of x, y, z goes to bit 3i, 3i+1, 3i+2 (the layout of
// visionaray morton.h:33-46).  Spreads 10 bits with the multiply-and-mask sequence
// popularised by Karras (NVIDIA developer blog, 2012).
__device__ __forceinline__ uint32_t spread10(uint32_t v)
{
    v &= 0x3FFu;
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z)
{
    return spread10(x) | (spread10(y) << 1) | (spread10(z) << 2);
}

// Float <-> totally ordered int (for atomicMin/atomicMax on float bounds without a
// CAS loop).  Valid for every non-NaN float.
__device__ __forceinline__ int float_to_ordered(float f)
{
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float ordered_to_float(int i)
{
    return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF);
}

} // namespace gbrt
