// The batched path tracer's persistent kernel, shared by batch_pt.cu (node pairs) and
// batch_pt_wide.cu (4- and 8-wide nodes of the arena's collapse).
//
// Warps of a grid sized to the GPU take tiles of `tile` pixels of any scene off one
// atomic counter, look their scene up by binary search over the pixel offsets, and run
// each pixel's samples and bounces in-thread: traversal of the scene's tree in the
// shared arena and the same shade_vertex as the wavefront renderer (pt_shade.cuh), so
// scene s's image equals gbrt_pathtrace_frame's bit for bit (through the node pairs;
// the wide nodes visit triangles in another order, so an equal-t tie may resolve to
// the other triangle).  Pixels are taken in row order, in 8x4 screen blocks, or -- with
// a sorted order -- in the order perm[] gives (pixels grouped by scene, then by the
// Morton cell of their primary hit).  Scenes with lights sample them as the megakernel
// renderer does: the light sample's shadow ray is an any-hit query right after the
// vertex is shaded.  Units including this header are compiled with --fmad=false.
#pragma once

#include "pt_shade.cuh"

#include <type_traits>

namespace gbrt {

// Per-scene frame constants (112 bytes).
struct __align__(16) batch_frame
{
    camera_basis cam;
    float4 bg;          // background with alpha 1 (missed camera rays)
    float3 ambient;
    float epsilon;
    uint32_t width, height, spp, num_bounces;
    uint32_t frame_id, flags;
    int32_t root;
    uint32_t blocks;    // 1: the frame can be walked in 8x4 pixel blocks
};
static_assert(sizeof(batch_frame) == 112, "frame record layout");

struct batch_args
{
    const batch_frame* __restrict__ frames;
    const uint32_t* pixel_offsets;
    uint32_t num_scenes, total_pixels, tile, order;
    const bvh2_node* nodes;
    const tri48* tris;
    int32_t total_inner, total_tris;
    const void* nodesw;              // the arena's W-wide nodes (scene s's root at node s)
    int32_t num_nodesw;
    const uint32_t* perm;            // null, or the global pixel taken at each work index
    const gbrt_material* materials;
    uint32_t num_materials;
    const float4* lights;            // 4 float4 per light
    const uint32_t* light_offsets;   // scene s: lights [light_offsets[s], light_offsets[s + 1])
    const float2* trig;
    uint32_t* work;
    float4* images;
    uint32_t* status;
};

using batch_kernel = void (*)(batch_args);

// Traversal stack entries kept in shared memory (a per-thread column, bank-conflict
// free); deeper entries in local memory.
constexpr int kBatchSharedStack = 8;
// Resident warps per SM the register allocation must allow (launch bounds): the full 64
// (32 registers, with spills) -- measured on the 512-scene batch, the frame kernel takes
// 87.7 / 79.8 / 74.9 / 71.8 / 67.4 ms at 24 / 32 / 40 / 48 / 64 warps: latency, not
// spill traffic, bounds it.
constexpr int kBatchWarpsPerSM = 64;
// The wide kernels hold W child boxes per visited node: 32 warps per SM (64 registers);
// at 64 warps their node arrays spill kilobytes per thread.
constexpr int kBatchWideWarpsPerSM = 32;

// Extended = false: a material table of matte and emissive slots only (the other
// materials' branches compiled out, as for the adjoint).  Lit = false: no scene has
// lights (the next-event path compiled out).  Width: 2 traverses the node pairs with
// a Stack-entry stack; 4 or 8 the arena's wide nodes (their own stack).
template <int Block, int Stack, bool Extended, bool Lit, int Width>
__global__ void __launch_bounds__(Block, (Width == 2 ? kBatchWarpsPerSM : kBatchWideWarpsPerSM) * 32 / Block)
    batch_pt(batch_args a)
{
    const uint32_t full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    __shared__ int stack_mem[Width == 2 ? kBatchSharedStack * Block : 1];
    // the wide kernels keep a two-entry pair stack for one-triangle scenes (a leaf root)
    using pair_stack = std::conditional_t<Width == 2,
                                          shared_stack<kBatchSharedStack < Stack ? kBatchSharedStack : Stack - 1, Stack,
                                                       Block>,
                                          local_stack<2>>;
    pair_stack stack;
    if constexpr (Width == 2) stack.col = stack_mem + threadIdx.x;
    using NodeW = typename wide_node<Width == 2 ? 4 : Width>::type;
    const NodeW* nodesw = static_cast<const NodeW*>(a.nodesw);
    shade_params sp;
    sp.materials = a.materials;
    sp.num_materials = a.num_materials;
    sp.lights = nullptr;
    sp.num_lights = 0;
    sp.tris = a.tris;
    sp.num_tris = a.total_tris;
    sp.albedo = nullptr;
    sp.emission = nullptr;
    sp.trig = a.trig;
    sp.bounce = 0;
    for (;;)
    {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(a.work, a.tile);
        base = __shfl_sync(full, base, 0);
        if (base >= a.total_pixels) break;
        for (uint32_t k = uint32_t(lane); k < a.tile; k += 32)
        {
            const uint32_t g0 = base + k;
            if (g0 >= a.total_pixels) break;
            const uint32_t g = a.perm ? __ldg(&a.perm[g0]) : g0;
            const uint32_t s = upper_segment(a.pixel_offsets, a.num_scenes, g);
            const batch_frame& f = a.frames[s];   // fields read where they are used
            const uint32_t first = __ldg(&a.pixel_offsets[s]);
            const uint32_t local = g - first;
            uint32_t pixel = local;
            if (!a.perm && a.order == GBRT_BATCH_ORDER_BLOCKS && f.blocks)
            {
                uint32_t blk = local >> 5, w = local & 31u, bw = f.width >> 3;
                pixel = ((blk / bw) * 4u + (w >> 3)) * f.width + (blk % bw) * 8u + (w & 7u);
            }
            if constexpr (Lit)
            {
                const uint32_t l0 = __ldg(&a.light_offsets[s]);
                sp.lights = a.lights + 4 * uint64_t(l0);
                sp.num_lights = __ldg(&a.light_offsets[s + 1]) - l0;
            }
            sp.epsilon = f.epsilon;
            sp.ambient = f.ambient;
            sp.frame = f.frame_id;
            sp.flags = f.flags;
            const v3 eye = { f.cam.eye.x, f.cam.eye.y, f.cam.eye.z };
            auto query = [&](auto any_hit, v3 o, v3 d, float tmin, float tmax) -> trace_result {
                constexpr bool kAny = decltype(any_hit)::value;
                if constexpr (Width != 2)
                {
                    if (f.root >= 0)
                        return traverse_bvhw<kAny, Width>(nodesw, a.num_nodesw, a.tris, a.total_tris, { o.x, o.y, o.z },
                                                          { d.x, d.y, d.z }, tmin, tmax, a.status, int32_t(s));
                }
                return traverse_bvh_with<kAny>(stack, a.nodes, a.tris, f.root, a.total_inner, a.total_tris,
                                               { o.x, o.y, o.z }, { d.x, d.y, d.z }, tmin, tmax, a.status);
            };
            float4 sum = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            for (uint32_t smp = 0; smp < f.spp; ++smp)
            {
                sp.sample = smp;
                v3 o = eye;
                v3 d = primary_dir(f.cam, f.width, f.height, f.frame_id, pixel, smp);
                path_state st{ { 1.0f, 1.0f, 1.0f }, { 0.0f, 0.0f, 0.0f }, 2u, kLastSpecular };
                for (uint32_t bounce = 0; bounce < f.num_bounces; ++bounce)
                {
                    trace_result h = query(std::false_type{}, o, d, 0.0f, FLT_MAX);
                    vertex_out out;
                    shade_vertex<Extended>(sp, pixel, bounce, o, d, 0.0f, FLT_MAX, h.tri, h.t, st, out, a.status);
                    if constexpr (Lit)
                    {
                        if (out.shadow)
                        {
                            trace_result sh = query(std::true_type{}, out.sh_o, out.sh_d, sp.epsilon, out.sh_tmax);
                            if (sh.tri < 0)
                                st.rad = { st.rad.x + out.contrib.x, st.rad.y + out.contrib.y,
                                           st.rad.z + out.contrib.z };
                        }
                    }
                    if (!out.cont) break;
                    o = out.next_o;
                    d = out.next_d;
                }
                // rr.color += result.color (sched_common.h:452-470)
                float4 c = (st.flags & kFirstHit) ? make_float4(st.rad.x, st.rad.y, st.rad.z, 1.0f) : f.bg;
                sum = make_float4(sum.x + c.x, sum.y + c.y, sum.z + c.z, sum.w + c.w);
            }
            // rr.color /= spp, then the blend with sfactor 1 and dfactor 0 (the
            // wavefront renderer's pt_blend with those factors)
            const float spp = float(f.spp);
            float4 av = make_float4(sum.x / spp, sum.y / spp, sum.z / spp, sum.w / spp);
            const float sf = 1.0f, df = 0.0f, dz = 0.0f;
            a.images[uint64_t(first) + pixel] = make_float4(av.x * sf + dz * df, av.y * sf + dz * df,
                                                            av.z * sf + dz * df, av.w * sf + dz * df);
        }
    }
}

// The wide kernels (batch_pt_wide.cu): the launch's block and width, null for any
// other width.
batch_kernel pick_wide_kernel(gbrt_batch_launch const& l, bool extended, bool lit);

} // namespace gbrt
