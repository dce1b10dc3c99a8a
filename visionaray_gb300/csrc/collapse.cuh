// Collapse of a node-pair BVH into W-wide nodes (W = 4 or 8), one tree level per
// launch: visionaray's bvh_collapser (detail/bvh/collapse.h:19-169) turns a BVH2 into
// BVH4/8 on the CPU; here every queued item (pair node, wide node) of a level is one
// thread, so all subtrees of a level -- and the trees of many scenes at once -- collapse
// in parallel.
//
// An item opens the pair node's two children and keeps opening the inner child of
// largest surface area until W children are reached; a child with at most leaf_max
// primitives becomes a leaf over its contiguous (Morton-ordered) triangle range, every
// other inner child gets a new wide node (an atomic counter) and goes to the next
// level's queue.  Each launch walks its queue with a grid-stride loop over the count the
// previous level left on the device, so a fixed grid serves every level and the
// collapse needs no host synchronisation (it can be captured in a CUDA graph).
#pragma once

#include "api_internal.h"

namespace gbrt {

// ranges[i]: the leaf range (first, last) of pair node i, in the triangle array's
// order; num_inner2: the number of pair nodes.
template <int W>
__global__ void __launch_bounds__(256) collapse_wide(const bvh2_node* __restrict__ nodes2,
                                                     const int2* __restrict__ ranges, const int2* __restrict__ q_in,
                                                     const uint32_t* __restrict__ count_in, int2* __restrict__ q_out,
                                                     uint32_t* __restrict__ count_out,
                                                     typename wide_node<W>::type* __restrict__ nodesw,
                                                     uint32_t* __restrict__ node_counter, uint32_t cap, int leaf_max,
                                                     int num_inner2, uint32_t* __restrict__ status)
{
    using NodeW = typename wide_node<W>::type;
    const uint32_t items = *count_in;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < items; i += gridDim.x * blockDim.x)
    {
        int2 item = q_in[i];
        int ref[W], first[W], cnt[W];
        float bx[W][6];   // lo.x hi.x lo.y hi.y lo.z hi.z
        int num = 0;
        auto open = [&](int node) {
            bvh2_node nd = nodes2[node];
            for (int side = 0; side < 2; ++side)
            {
                int link = side ? nd.link.y : nd.link.x;
                float4 xy = side ? nd.xy1 : nd.xy0;
                float zl = side ? nd.z01.z : nd.z01.x, zh = side ? nd.z01.w : nd.z01.y;
                ref[num] = link;
                bx[num][0] = xy.x;
                bx[num][1] = xy.y;
                bx[num][2] = xy.z;
                bx[num][3] = xy.w;
                bx[num][4] = zl;
                bx[num][5] = zh;
                if (link < 0)
                {
                    first[num] = ~link;
                    cnt[num] = 1;
                }
                else
                {
                    int2 r = link < num_inner2 ? ranges[link] : make_int2(0, -1);
                    first[num] = r.x;
                    cnt[num] = r.y - r.x + 1;
                }
                ++num;
            }
        };
        if (item.x < 0 || item.x >= num_inner2 || uint32_t(item.y) >= cap)
        {
            atomicOr(status, kStatusBadIndex);
            continue;
        }
        open(item.x);
        while (num < W)
        {
            int best = -1;
            float best_area = -1.0f;
            for (int k = 0; k < num; ++k)
            {
                if (ref[k] < 0 || cnt[k] <= leaf_max) continue;
                float dx = bx[k][1] - bx[k][0], dy = bx[k][3] - bx[k][2], dz = bx[k][5] - bx[k][4];
                float area = dx * dy + dy * dz + dz * dx;
                if (area > best_area)
                {
                    best_area = area;
                    best = k;
                }
            }
            if (best < 0) break;
            int node = ref[best];
            --num;
            ref[best] = ref[num];
            first[best] = first[num];
            cnt[best] = cnt[num];
            for (int c = 0; c < 6; ++c) bx[best][c] = bx[num][c];
            open(node);
        }
        // the node in registers: plane p of child k at word p * W + k (lo.x, hi.x,
        // lo.y, hi.y, lo.z, hi.z), then W child links and W counts
        NodeW out;
        float* f = reinterpret_cast<float*>(&out);
        int* ci = reinterpret_cast<int*>(&out);
        for (int k = 0; k < W; ++k)
        {
            int ch = -1, ct = -1;
            if (k < num)
            {
                for (int p = 0; p < 6; ++p) f[p * W + k] = bx[k][p];
                if (ref[k] < 0 || cnt[k] <= leaf_max)
                {
                    ch = first[k];
                    ct = cnt[k];
                }
                else
                {
                    uint32_t idx = atomicAdd(node_counter, 1u);
                    if (idx >= cap)
                    {
                        atomicOr(status, kStatusBadIndex);
                    }
                    else
                    {
                        ch = int(idx);
                        ct = 0;
                        uint32_t slot = atomicAdd(count_out, 1u);
                        if (slot < cap)
                            q_out[slot] = make_int2(ref[k], int(idx));
                        else
                            atomicOr(status, kStatusBadIndex);
                    }
                }
            }
            else
            {
                for (int p = 0; p < 6; ++p) f[p * W + k] = (p & 1) ? -FLT_MAX : FLT_MAX;
            }
            ci[6 * W + k] = ch;
            ci[7 * W + k] = ct;
        }
        nodesw[item.y] = out;
    }
}

} // namespace gbrt
