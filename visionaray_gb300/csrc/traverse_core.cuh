// Device BVH traversal shared by the ray-query kernels (traverse.cu) and the path
// tracer (pathtrace.cu).
//
// Replaces the device branch of visionaray's intersect<Traversal>(ray, bvh, isect)
// (detail/bvh/intersect.inl:166-356), which visits BVH2 nodes one 32-byte box at a
// time with a 5-entry stack and a restart trail.  Here each step fetches one 64-byte
// record (four 128-bit read-only loads) holding both children's boxes, tests both,
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

template <bool AnyHit>
__device__ __forceinline__ trace_result traverse_bvh(const bvh2_node* __restrict__ nodes,
                                                     const tri48* __restrict__ tris, int32_t root,
                                                     int32_t num_inner, int32_t num_tris, f3 o, f3 d,
                                                     float tmin, float tmax, uint32_t* __restrict__ status)
{
    const float ix = safe_rcp(d.x), iy = safe_rcp(d.y), iz = safe_rcp(d.z);
    trace_result best{ -1, FLT_MAX, 0.0f, 0.0f };

    int stack[kStackSize];
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
            const bvh2_node* np = nodes + node;
            float4 a = ldg4(&np->xy0);
            float4 b = ldg4(&np->xy1);
            float4 z = ldg4(&np->z01);
            int4 link = __ldg(&np->link);

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
            bool h0 = tf0 >= tn0 && tn0 < best.t;
            bool h1 = tf1 >= tn1 && tn1 < best.t;

            if (h0 && h1)
            {
                bool first0 = tn0 < tn1;   // ties go to child 1, as intersect.inl:283
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
            if (h.hit && h.t < best.t && h.t >= tmin && h.t <= tmax)
            {
                best = { t, h.t, h.u, h.v };
                if (AnyHit) return best;
            }
            if (__float_as_uint(t2.w) & kLastInLeaf) break;
        }
        node = sp > 0 ? stack[--sp] : kEmptyLink;
    }
    return best;
}

} // namespace gbrt
