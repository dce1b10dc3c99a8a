// Two-level traversal (a top-level tree over instances of bottom-level trees), shared
// by the ray queries (instances.cu) and the path tracer over instances (pathtrace.cu).
//
// visionaray's index_bvh<index_bvh_inst_t<P>> (bvh.h:678-782) keeps, per instance, the
// inverse of the transform's 3x3 part and the negated translation, and intersect.inl:
// 362-394 transforms the ray into the instance's space (transform_ray, bvh.h:748-755)
// before traversing its tree; t stays the world ray's parameter.  Here the top level is
// node pairs whose leaves are ~instance, and a hit bounds the rest of the traversal
// (the best t so far is every later tree's t_best).
#pragma once

#include "traverse_core.cuh"

namespace gbrt {

struct tlas_view
{
    const bvh2_node* nodes;
    const float4* records;   // 3 float4 per instance: rows of the inverse 3x3 | translation to undo
    const bvh_view* views;   // the instance's bottom-level tree
    int32_t root, num_inner, num_instances;
};

struct tlas_result
{
    int inst, tri;   // -1 for a miss; tri indexes the instance's tree's triangles
    float t, u, v;
};

// transform_ray (bvh.h:748-755): the world ray carried into instance `inst`'s space
// with the instance's inverse 3x3 rows and negated translation.
__device__ __forceinline__ void instance_ray(tlas_view const& tv, int inst, f3 o, f3 d, f3& oo, f3& dd)
{
    const float4 ra = tv.records[3 * inst + 0], rb = tv.records[3 * inst + 1], rc = tv.records[3 * inst + 2];
    const float px = __fadd_rn(o.x, ra.w), py = __fadd_rn(o.y, rb.w), pz = __fadd_rn(o.z, rc.w);
    oo = { __fadd_rn(__fadd_rn(__fmul_rn(ra.x, px), __fmul_rn(ra.y, py)), __fmul_rn(ra.z, pz)),
           __fadd_rn(__fadd_rn(__fmul_rn(rb.x, px), __fmul_rn(rb.y, py)), __fmul_rn(rb.z, pz)),
           __fadd_rn(__fadd_rn(__fmul_rn(rc.x, px), __fmul_rn(rc.y, py)), __fmul_rn(rc.z, pz)) };
    dd = { __fadd_rn(__fadd_rn(__fmul_rn(ra.x, d.x), __fmul_rn(ra.y, d.y)), __fmul_rn(ra.z, d.z)),
           __fadd_rn(__fadd_rn(__fmul_rn(rb.x, d.x), __fmul_rn(rb.y, d.y)), __fmul_rn(rb.z, d.z)),
           __fadd_rn(__fadd_rn(__fmul_rn(rc.x, d.x), __fmul_rn(rc.y, d.y)), __fmul_rn(rc.z, d.z)) };
}

// bstack: the bottom-level traversals' stack (a local_stack, or a shared_stack whose
// top entries sit in shared memory); the top level keeps its own 32 entries.
template <bool AnyHit, class BlasStack>
__device__ __forceinline__ tlas_result traverse_tlas_with(BlasStack& bstack, tlas_view const& tv, f3 o, f3 d,
                                                          float tmin, float tmax, uint32_t* __restrict__ status)
{
    const float ix = safe_rcp(d.x), iy = safe_rcp(d.y), iz = safe_rcp(d.z);
    // the loop carries the best instance, triangle and t; u and v are recomputed at the
    // end from that instance's carried ray and triangle (the same operations on the
    // same inputs, so the same values)
    tlas_result best{ -1, -1, FLT_MAX, 0.0f, 0.0f };
    int stack[32];
    int sp = 0;
    int node = tv.root;
    while (node != kEmptyLink)
    {
        while (node >= 0)
        {
            if (node >= tv.num_inner)
            {
                atomicOr(status, kStatusBadIndex);
                node = kEmptyLink;
                break;
            }
            float4 a, b, z;
            int4 link;
            load_pair(tv.nodes + node, a, b, z, link);
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
                bool first0 = tn0 < tn1;   // near first, any hit too (traverse_bvh_with)
                if (sp < 32)
                    stack[sp++] = first0 ? link.y : link.x;
                else
                    atomicOr(status, kStatusStackOverflow);
                node = first0 ? link.x : link.y;
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
        const int inst = ~node;
        if (inst >= tv.num_instances)
        {
            atomicOr(status, kStatusBadIndex);
            break;
        }
        f3 oo, dd;
        instance_ray(tv, inst, o, d, oo, dd);
        const bvh_view bv = tv.views[inst];
        if (bv.num_tris > 0)
        {
            trace_result h = traverse_bvh_with<AnyHit>(bstack, bv.nodes, bv.tris, bv.root, bv.num_inner, bv.num_tris,
                                                       oo, dd, tmin, tmax, status, best.t);
            if (h.tri >= 0)
            {
                if (AnyHit) return tlas_result{ inst, h.tri, h.t, h.u, h.v };
                best.inst = inst;
                best.tri = h.tri;
                best.t = h.t;
            }
        }
        node = sp > 0 ? stack[--sp] : kEmptyLink;
    }
    if (!AnyHit && best.inst >= 0)
    {
        f3 oo, dd;
        instance_ray(tv, best.inst, o, d, oo, dd);
        const tri48* tp = tv.views[best.inst].tris + best.tri;
        const float4 t0 = ldg4(&tp->t0), t1 = ldg4(&tp->t1), t2 = ldg4(&tp->t2);
        const tri_hit h = intersect_triangle(oo, dd, { t0.x, t0.y, t0.z }, { t1.x, t1.y, t1.z }, { t2.x, t2.y, t2.z });
        best.u = h.u;
        best.v = h.v;
    }
    return best;
}

template <bool AnyHit>
__device__ __forceinline__ tlas_result traverse_tlas(tlas_view const& tv, f3 o, f3 d, float tmin, float tmax,
                                                     uint32_t* __restrict__ status)
{
    local_stack<kStackSize> bstack;
    return traverse_tlas_with<AnyHit>(bstack, tv, o, d, tmin, tmax, status);
}

// traverse_tlas with the bottom-level stack's first Shared entries in shared memory (a
// column per thread of a Block-thread block).
template <bool AnyHit, int Block, int Shared>
__device__ __forceinline__ tlas_result traverse_tlas_shared(tlas_view const& tv, f3 o, f3 d, float tmin, float tmax,
                                                            uint32_t* __restrict__ status)
{
    __shared__ int stack_mem[Shared * Block];
    shared_stack<Shared, kStackSize, Block> bstack;
    bstack.col = stack_mem + threadIdx.x;
    return traverse_tlas_with<AnyHit>(bstack, tv, o, d, tmin, tmax, status);
}

} // namespace gbrt
