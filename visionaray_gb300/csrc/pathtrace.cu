// Wavefront path tracer: cuda_sched<basic_ray<float>>::frame(pathtracing::kernel{params},
// jittered-blend sampler) of visionaray (detail/cuda_sched.inl:32-69, 226-246,
// detail/pathtracing.inl:42-233) re-designed for the GPU.
//
// visionaray runs the whole path (all bounces, its traversal, shading and shadow
// ray) in one thread per pixel; threads of a warp diverge as soon as paths end at
// different bounces or traverse different subtrees.  Here a frame is a sequence of
// passes, one per sample index; each pass keeps one path per pixel and advances all
// live paths one bounce at a time through three kernels:
//   extend : closest-hit traversal of the live rays (queue in, hits out)
//   shade  : surface sampling, emission with MIS, next-event estimation (light
//            sample + shadow ray), throughput update, Russian roulette; live paths
//            and shadow rays are appended to compacted queues with one atomic per
//            warp (ballot + popc)
//   shadow : any-hit traversal of the shadow queue, unoccluded contributions added
// so every traversal launch runs over a dense queue of live rays.  The arithmetic is
// the reference's, operation for operation (this file is compiled with
// --fmad=false; divisions and square roots are IEEE), and the random numbers are
// the gbrt_rng.h stream, so a path can be replayed on the CPU bit for bit; the one
// deliberate difference is the hemisphere sample's cos/sin, evaluated in double and
// rounded once (the host's cosf/sinf may differ from that in the last bit).

#include "instances.cuh"
#include "pt_shade.cuh"

#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

struct gbrt_pt_scene
{
    gbrt_bvh const* bvh = nullptr;
    int device = 0;
    gbrt_material* materials = nullptr;
    uint32_t num_materials = 0;
    float4* lights = nullptr;   // 4 float4 per light: v1, e1, e2, intensity (cl * kl)
    uint32_t num_lights = 0;
    bool extended = false;      // some material is a mirror, glass or plastic
    gbrt::env_view* env = nullptr;   // device copy; null: the params' constant ambient light
    // a scene over a two-level tree (gbrt_pt_scene_create_instanced): the tree and each
    // instance's first material slot (device); bvh is null then
    gbrt_tlas const* tlas = nullptr;
    uint32_t* inst_geom = nullptr;
};

namespace gbrt {
namespace {

constexpr int kBlock = 128;
// Traversal kernels (extend, shadow): the stack's first 16 entries in shared memory and
// launch bounds for 12 resident blocks (48 warps, 40 registers, no spills).  Measured
// on the box frame (1920x1080x64, PLOC tree): 623 ms per frame; 8 shared entries 642;
// 16 blocks (32 registers, spilling) 666 with 16 entries, 671 with 8.
constexpr int kPtSharedStack = 16;
constexpr int kPtMinBlocks = 12;
// The adjoint's replay kernel: resident blocks its registers must allow -- 16 blocks
// (64 warps, 32 registers; the vertex records live in local memory anyway): backward
// 15.4 -> 13.0 ms per inverse-rendering step (8 blocks 13.4, 12 blocks 14.3).  Its
// traversal keeps the whole stack in local memory: a shared-memory top of 8 / 16
// entries took the 512x512x16 replay from 46.2 to 55.1 / 65.6 ms (the shared carve-out
// takes the L1 that the local vertex records use).
constexpr int kAdjointMinBlocks = 16;
// The shading kernel: 8 resident blocks (32 warps, at most 64 registers), the occupancy
// it has without the out-of-line material samplers' call overhead.
constexpr int kShadeMinBlocks = 8;

struct frame_buffers
{
    gbrt_ray* rays[2];
    uint32_t* path[2];
    uint4* hits;
    gbrt_ray* shadow_rays;
    uint32_t* shadow_path;
    float4* shadow_contrib;
    float4* throughput;
    float4* radiance;
    uint2* rng_flags;   // draw counter, flags
    float4* sum;
    uint32_t* counts;   // queue 0, queue 1, shadow queue
    // queue order by origin cell (GBRT_TRACE_SORT_RAYS): keys / values and their
    // double buffers, the sort's scratch
    uint32_t* keys;
    uint32_t* vals;
    uint32_t* keys_alt;
    uint32_t* vals_alt;
    void* sort_scratch;
};

// Appends the lanes with `take` to a queue: one atomic per warp.  Every lane of the
// warp must call it.
__device__ __forceinline__ uint32_t warp_append(bool take, uint32_t* counter)
{
    const uint32_t full = 0xFFFFFFFFu;
    uint32_t mask = __ballot_sync(full, take);
    if (mask == 0) return 0;
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, uint32_t(__popc(mask)));
    base = __shfl_sync(full, base, leader);
    return base + uint32_t(__popc(mask & ((1u << lane) - 1u)));
}

__device__ __forceinline__ void store_ray(gbrt_ray* dst, v3 o, v3 d, float tmin, float tmax)
{
    float4* p = reinterpret_cast<float4*>(dst);
    p[0] = make_float4(o.x, o.y, o.z, d.x);
    p[1] = make_float4(d.y, d.z, tmin, tmax);
}

// Jittered primary rays (detail/sched_common.h:209-233: jitter x drawn before y) through
// the pinhole camera (detail/pinhole_camera.inl:103-120).
__global__ void __launch_bounds__(kBlock) pt_raygen(frame_buffers fb, uint32_t width, uint32_t height,
                                                    uint32_t frame, uint32_t sample, camera_basis cam)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    uint32_t n = width * height;
    if (i == 0)
    {
        fb.counts[0] = n;
        fb.counts[1] = 0;
        fb.counts[2] = 0;
    }
    if (i >= n) return;
    v3 d = primary_dir(cam, width, height, frame, i, sample);
    store_ray(&fb.rays[0][i], { cam.eye.x, cam.eye.y, cam.eye.z }, d, 0.0f, FLT_MAX);
    fb.path[0][i] = i;
    fb.throughput[i] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    fb.radiance[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    fb.rng_flags[i] = make_uint2(2u, kLastSpecular);
}

template <bool Wide>
__global__ void __launch_bounds__(kBlock, kPtMinBlocks) pt_extend(frame_buffers fb, int q, bvh_view v,
                                                                  uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i == 0)
    {
        fb.counts[q ^ 1] = 0;   // the shade kernel that follows appends to these
        fb.counts[2] = 0;
    }
    uint32_t n = fb.counts[q];
    if (i >= n) return;
    const float4* rp = reinterpret_cast<const float4*>(&fb.rays[q][i]);
    float4 r0 = rp[0], r1 = rp[1];
    trace_result h = traverse_view_shared<false, Wide, kBlock, kPtSharedStack>(v, { r0.x, r0.y, r0.z },
                                                                              { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    fb.hits[i] = make_uint4(uint32_t(h.tri), __float_as_uint(h.t), 0u, 0u);
}


// Ray order of a queue (GBRT_TRACE_SORT_RAYS): the 24-bit Morton key of each queued
// ray's origin cell in the scene box; entries past the queue's length (read from the
// device) get the largest key, so a stable sort leaves them behind the queue.
__global__ void __launch_bounds__(kBlock) pt_queue_keys(const gbrt_ray* __restrict__ rays,
                                                        const uint32_t* __restrict__ count, uint32_t n, float3 lo,
                                                        float3 scale, uint32_t* __restrict__ keys,
                                                        uint32_t* __restrict__ vals)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    uint32_t key = 0xFFFFFFu;
    if (i < *count)
    {
        float4 r0 = ldg4(&rays[i]);
        float q[3] = { (r0.x - lo.x) * scale.x, (r0.y - lo.y) * scale.y, (r0.z - lo.z) * scale.z };
        uint32_t c[3];
        for (int a = 0; a < 3; ++a) c[a] = uint32_t(fminf(fmaxf(q[a], 0.0f), 255.0f));
        key = morton3(c[0], c[1], c[2]);
    }
    keys[i] = key;
    vals[i] = i;
}

// pt_extend over the queue in the order perm (thread i traces queue entry perm[i]).
template <bool Wide>
__global__ void __launch_bounds__(kBlock, kPtMinBlocks) pt_extend_sorted(frame_buffers fb, int q,
                                                                         const uint32_t* __restrict__ perm,
                                                                         bvh_view v, uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i == 0)
    {
        fb.counts[q ^ 1] = 0;
        fb.counts[2] = 0;
    }
    uint32_t n = fb.counts[q];
    if (i >= n) return;
    uint32_t j = __ldg(&perm[i]);
    if (j >= n)
    {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    const float4* rp = reinterpret_cast<const float4*>(&fb.rays[q][j]);
    float4 r0 = rp[0], r1 = rp[1];
    trace_result h = traverse_view_shared<false, Wide, kBlock, kPtSharedStack>(v, { r0.x, r0.y, r0.z },
                                                                              { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    fb.hits[j] = make_uint4(uint32_t(h.tri), __float_as_uint(h.t), 0u, 0u);
}

// One bounce for every live path of the queue.
// A scene over a two-level tree: per instance its tree, its instance-to-world rows and
// its first material slot; views null for a single tree.
struct inst_shade
{
    const bvh_view* views;
    const float4* forward;
    const uint32_t* geom_base;
    int32_t num_instances;
};

__global__ void __launch_bounds__(kBlock, kShadeMinBlocks) pt_shade(frame_buffers fb, int q, shade_params sp,
                                                   inst_shade is, uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    uint32_t n = fb.counts[q];
    bool live = i < n;

    vertex_out out;
    out.cont = false;
    out.shadow = false;
    uint32_t p = 0;
    float tmin = 0.0f, tmax = 0.0f;
    if (live)
    {
        p = fb.path[q][i];
        const float4* rp = reinterpret_cast<const float4*>(&fb.rays[q][i]);
        float4 r0 = rp[0], r1 = rp[1];
        tmin = r1.z;
        tmax = r1.w;
        uint4 hh = fb.hits[i];
        if (is.views && int(hh.x) >= 0)
        {
            // the hit instance's triangle, carried to world space by shade_vertex
            const int inst = int(hh.z);
            if (inst >= 0 && inst < is.num_instances)
            {
                const bvh_view bv = is.views[inst];
                sp.tris = bv.tris;
                sp.num_tris = bv.num_tris;
                sp.xform = is.forward + 3 * inst;
                sp.geom_base = is.geom_base[inst];
            }
            else
            {
                atomicOr(status, kStatusBadIndex);
                hh.x = 0xFFFFFFFFu;
            }
        }
        uint2 rf = fb.rng_flags[p];
        path_state st{ xyz(fb.throughput[p]), xyz(fb.radiance[p]), rf.x, rf.y };
        shade_vertex(sp, p, sp.bounce, { r0.x, r0.y, r0.z }, { r0.w, r1.x, r1.y }, r1.z, r1.w, int(hh.x),
                     __uint_as_float(hh.y), st, out, status);
        fb.throughput[p] = make_float4(st.thr.x, st.thr.y, st.thr.z, 0.0f);
        fb.radiance[p] = make_float4(st.rad.x, st.rad.y, st.rad.z, 0.0f);
        fb.rng_flags[p] = make_uint2(st.k, st.flags);
    }

    uint32_t slot = warp_append(out.cont, &fb.counts[q ^ 1]);
    if (out.cont)
    {
        store_ray(&fb.rays[q ^ 1][slot], out.next_o, out.next_d, tmin, tmax);
        fb.path[q ^ 1][slot] = p;
    }
    uint32_t sslot = warp_append(out.shadow, &fb.counts[2]);
    if (out.shadow)
    {
        store_ray(&fb.shadow_rays[sslot], out.sh_o, out.sh_d, sp.epsilon, out.sh_tmax);
        fb.shadow_path[sslot] = p;
        fb.shadow_contrib[sslot] = make_float4(out.contrib.x, out.contrib.y, out.contrib.z, 0.0f);
    }
}

template <bool Wide>
__global__ void __launch_bounds__(kBlock, kPtMinBlocks) pt_shadow(frame_buffers fb, bvh_view v,
                                                                  uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    uint32_t n = fb.counts[2];
    if (i >= n) return;
    const float4* rp = reinterpret_cast<const float4*>(&fb.shadow_rays[i]);
    float4 r0 = rp[0], r1 = rp[1];
    trace_result h = traverse_view_shared<true, Wide, kBlock, kPtSharedStack>(v, { r0.x, r0.y, r0.z },
                                                                             { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    if (h.tri < 0)
    {
        uint32_t p = fb.shadow_path[i];
        float4 c = fb.shadow_contrib[i];
        float4 r = fb.radiance[p];
        fb.radiance[p] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.0f);
    }
}

// pt_shadow over the shadow queue in the order perm.
template <bool Wide>
__global__ void __launch_bounds__(kBlock, kPtMinBlocks) pt_shadow_sorted(frame_buffers fb,
                                                                         const uint32_t* __restrict__ perm,
                                                                         bvh_view v, uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    uint32_t n = fb.counts[2];
    if (i >= n) return;
    uint32_t j = __ldg(&perm[i]);
    if (j >= n)
    {
        atomicOr(status, kStatusBadIndex);
        return;
    }
    const float4* rp = reinterpret_cast<const float4*>(&fb.shadow_rays[j]);
    float4 r0 = rp[0], r1 = rp[1];
    trace_result h = traverse_view_shared<true, Wide, kBlock, kPtSharedStack>(v, { r0.x, r0.y, r0.z },
                                                                             { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    if (h.tri < 0)
    {
        uint32_t p = fb.shadow_path[j];
        float4 c = fb.shadow_contrib[j];
        float4 r = fb.radiance[p];
        fb.radiance[p] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.0f);
    }
}

// Bottom-level stack entries of the two-level queries held in shared memory (0: the
// whole stack in local memory).  Measured on the instanced box (1920x1080x64, 256 blob
// instances): 984.5 ms per frame with the local stack, 1057.0 / 1061.1 ms with 8 / 16
// entries in shared memory at 12 blocks per SM; at 8 blocks with the SAH top level
// 780.4 ms local, 795.2 / 807.2 ms with 8 / 16 shared entries.
constexpr int kPtTlasSharedStack = 0;
// Resident blocks the two-level extend and shadow kernels' registers must allow: 8
// (64 registers, no spills; the top-level loop around the bottom-level one holds more
// state than one tree's traversal).  Measured on the instanced box: 980.6 ms per frame
// at 12 blocks (40 registers, spilling), 896.4 at 10, 874.1 at 8.
constexpr int kPtTlasMinBlocks = 8;

template <bool AnyHit>
__device__ __forceinline__ tlas_result trace_tlas(tlas_view const& tv, f3 o, f3 d, float tmin, float tmax,
                                                  uint32_t* __restrict__ status)
{
    if constexpr (kPtTlasSharedStack > 0)
        return traverse_tlas_shared<AnyHit, kBlock, kPtTlasSharedStack>(tv, o, d, tmin, tmax, status);
    else
        return traverse_tlas<AnyHit>(tv, o, d, tmin, tmax, status);
}

// pt_extend and pt_shadow over a two-level tree: hits carry the instance in z.
__global__ void __launch_bounds__(kBlock, kPtTlasMinBlocks) pt_extend_tlas(frame_buffers fb, int q, tlas_view tv,
                                                                       uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i == 0)
    {
        fb.counts[q ^ 1] = 0;   // the shade kernel that follows appends to these
        fb.counts[2] = 0;
    }
    uint32_t n = fb.counts[q];
    if (i >= n) return;
    const float4* rp = reinterpret_cast<const float4*>(&fb.rays[q][i]);
    float4 r0 = rp[0], r1 = rp[1];
    tlas_result h = trace_tlas<false>(tv, { r0.x, r0.y, r0.z }, { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    fb.hits[i] = make_uint4(uint32_t(h.tri), __float_as_uint(h.t), uint32_t(h.inst), 0u);
}

__global__ void __launch_bounds__(kBlock, kPtTlasMinBlocks) pt_shadow_tlas(frame_buffers fb, tlas_view tv,
                                                                       uint32_t* __restrict__ status)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    uint32_t n = fb.counts[2];
    if (i >= n) return;
    const float4* rp = reinterpret_cast<const float4*>(&fb.shadow_rays[i]);
    float4 r0 = rp[0], r1 = rp[1];
    tlas_result h = trace_tlas<true>(tv, { r0.x, r0.y, r0.z }, { r0.w, r1.x, r1.y }, r1.z, r1.w, status);
    if (h.tri < 0)
    {
        uint32_t p = fb.shadow_path[i];
        float4 c = fb.shadow_contrib[i];
        float4 r = fb.radiance[p];
        fb.radiance[p] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.0f);
    }
}

// rr.color += result.color over the samples (sched_common.h:452-470): the path's
// radiance with alpha 1 if the camera ray hit, else the background.
__global__ void __launch_bounds__(kBlock) pt_accumulate(frame_buffers fb, uint32_t n, uint32_t sample, float4 bg)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    float4 c = (fb.rng_flags[i].y & kFirstHit) ? make_float4(fb.radiance[i].x, fb.radiance[i].y, fb.radiance[i].z, 1.0f)
                                               : bg;
    if (sample == 0)
    {
        float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        fb.sum[i] = make_float4(z.x + c.x, z.y + c.y, z.z + c.z, z.w + c.w);
    }
    else
    {
        float4 s = fb.sum[i];
        fb.sum[i] = make_float4(s.x + c.x, s.y + c.y, s.z + c.z, s.w + c.w);
    }
}

// rr.color /= spp; accum = src * sfactor + dst * dfactor; color = accum
// (sched_common.h:472-511, pixel_access.h:1040-1043).
__global__ void __launch_bounds__(kBlock) pt_blend(frame_buffers fb, uint32_t n, float spp, float sfactor,
                                                   float dfactor, float4* __restrict__ accum,
                                                   float4* __restrict__ color)
{
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    float4 s = fb.sum[i];
    float4 a = make_float4(s.x / spp, s.y / spp, s.z / spp, s.w / spp);
    // dfactor == 0 overwrites: the previous contents (possibly never written) are not read
    float4 d = dfactor != 0.0f ? accum[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 o = make_float4(a.x * sfactor + d.x * dfactor, a.y * sfactor + d.y * dfactor, a.z * sfactor + d.z * dfactor,
                           a.w * sfactor + d.w * dfactor);
    accum[i] = o;
    if (color) color[i] = o;
}

// GBRT_PT_MEGAKERNEL: one thread per pixel runs the pixel's samples and bounces, the
// shadow ray of each bounce traced in-thread, in the wavefront's order of additions
// (shade adds emission / ambient, then the unoccluded next-event contribution), so the
// image is the wavefront's bit for bit.  Both queries of a thread share one stack whose
// first entries are in shared memory.  Measured slower than the wavefront on both
// path-tracing workloads (box scene 1920x1080x64: 1,374 vs 721 ms per frame; inverse-
// rendering forward: 23.8 vs 10.1 ms): a pixel's samples run one after the other in
// one thread (the sum must stay in sample order), and its lanes diverge across bounces,
// light samples and path lengths that the wavefront's compacted queues keep dense.
constexpr int kMegaMinBlocks = 16;

template <bool Wide>
__global__ void __launch_bounds__(kBlock, kMegaMinBlocks) pt_megakernel(bvh_view v, shade_params sp,
                                                                        camera_basis cam, uint32_t width,
                                                                        uint32_t height, uint32_t spp,
                                                                        uint32_t num_bounces, float4 bg,
                                                                        float sfactor, float dfactor,
                                                                        float4* __restrict__ accum,
                                                                        float4* __restrict__ color,
                                                                        uint32_t* __restrict__ status)
{
    __shared__ int stack_mem[kPtSharedStack * kBlock];
    shared_stack<kPtSharedStack, kStackSize, kBlock> stack;
    stack.col = stack_mem + threadIdx.x;
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= width * height) return;
    auto query = [&](auto any_hit, v3 o, v3 d, float tmin, float tmax) {
        if constexpr (Wide)
            return traverse_bvh4<decltype(any_hit)::value>(v.nodes4, v.num_nodes4, v.tris, v.num_tris,
                                                           { o.x, o.y, o.z }, { d.x, d.y, d.z }, tmin, tmax, status);
        else
            return traverse_bvh_with<decltype(any_hit)::value>(stack, v.nodes, v.tris, v.root, v.num_inner,
                                                               v.num_tris, { o.x, o.y, o.z }, { d.x, d.y, d.z },
                                                               tmin, tmax, status);
    };
    const v3 eye = { cam.eye.x, cam.eye.y, cam.eye.z };
    float4 sum = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (uint32_t smp = 0; smp < spp; ++smp)
    {
        sp.sample = smp;
        v3 o = eye;
        v3 d = primary_dir(cam, width, height, sp.frame, i, smp);
        path_state st{ { 1.0f, 1.0f, 1.0f }, { 0.0f, 0.0f, 0.0f }, 2u, kLastSpecular };
        for (uint32_t b = 0; v.num_tris > 0 && b < num_bounces; ++b)
        {
            trace_result h = query(std::false_type{}, o, d, 0.0f, FLT_MAX);
            vertex_out out;
            shade_vertex(sp, i, b, o, d, 0.0f, FLT_MAX, h.tri, h.t, st, out, status);
            if (out.shadow)
            {
                trace_result sh = query(std::true_type{}, out.sh_o, out.sh_d, sp.epsilon, out.sh_tmax);
                if (sh.tri < 0) st.rad = { st.rad.x + out.contrib.x, st.rad.y + out.contrib.y, st.rad.z + out.contrib.z };
            }
            if (!out.cont) break;
            o = out.next_o;
            d = out.next_d;
        }
        float4 c = (st.flags & kFirstHit) ? make_float4(st.rad.x, st.rad.y, st.rad.z, 1.0f) : bg;
        sum = make_float4(sum.x + c.x, sum.y + c.y, sum.z + c.z, sum.w + c.w);
    }
    // pt_blend's arithmetic
    const float n = float(spp);
    float4 a = make_float4(sum.x / n, sum.y / n, sum.z / n, sum.w / n);
    float4 dst = dfactor != 0.0f ? accum[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 out = make_float4(a.x * sfactor + dst.x * dfactor, a.y * sfactor + dst.y * dfactor,
                             a.z * sfactor + dst.z * dfactor, a.w * sfactor + dst.w * dfactor);
    accum[i] = out;
    if (color) color[i] = out;
}

constexpr int kMaxReplay = 16;   // path vertices the adjoint keeps (num_bounces limit)

// Adds `val` to base[3 * key ..] for every active lane; lanes with the same key are
// summed with shuffles first, so each distinct key costs one set of atomics per warp.
// Every lane of the warp must call it.
__device__ __forceinline__ void warp_add3(float* __restrict__ base, uint32_t key, v3 val, bool active)
{
    const uint32_t full = 0xFFFFFFFFu;
    uint32_t mask = __ballot_sync(full, active);
    if (!active) return;
    uint32_t peers = __match_any_sync(mask, key);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    v3 sum = { 0.0f, 0.0f, 0.0f };
    for (uint32_t m = peers; m; m &= m - 1)
    {
        int src = __ffs(m) - 1;
        sum.x += __shfl_sync(peers, val.x, src);
        sum.y += __shfl_sync(peers, val.y, src);
        sum.z += __shfl_sync(peers, val.z, src);
    }
    if (lane == leader)
    {
        atomicAdd(base + 3 * key + 0, sum.x);
        atomicAdd(base + 3 * key + 1, sum.y);
        atomicAdd(base + 3 * key + 2, sum.z);
    }
}

// Adjoint of thr' = u / p, p = max(u), the Russian-roulette normaliser with the
// decision held fixed: d/du of tbar . u / p.
__device__ __forceinline__ v3 roulette_adjoint(v3 tbar, v3 u, float p)
{
    v3 ub = tbar / p;
    float pb = -(tbar.x * u.x + tbar.y * u.y + tbar.z * u.z) / (p * p);
    if (u.x >= u.y && u.x >= u.z) ub.x += pb;
    else if (u.y >= u.z) ub.y += pb;
    else ub.z += pb;
    return ub;
}

// Adjoint w.r.t. the throughput of a next-event contribution N = w * thr * f with
// w = x^2 / (x^2 + y^2), y = b0 * max(thr) (the MIS weight's BSDF pdf scaled by the
// throughput, pathtracing.inl:180-182): adds dN/dthr . adj to tb.
__device__ __forceinline__ v3 nee_throughput_adjoint(vertex_rec const& r, v3 adj, v3 f, v3 tb)
{
    tb = tb + adj * f * r.w;
    float wbar = adj.x * r.thr.x * f.x + adj.y * r.thr.y * f.y + adj.z * r.thr.z * f.z;
    float yv = r.b0 * max_elem(r.thr);
    float den = r.x * r.x + yv * yv;
    float dwdy = -2.0f * r.x * r.x * yv / (den * den);
    float g = wbar * dwdy * r.b0;
    if (r.thr.x >= r.thr.y && r.thr.x >= r.thr.z) tb.x += g;
    else if (r.thr.y >= r.thr.z) tb.y += g;
    else tb.z += g;
    return tb;
}

// Path-replay backpropagation (Vicini, Speierer & Jakob 2021): one thread per
// (pixel, sample) re-traces its path from its random-number counter -- the same
// shade_vertex, so the replay is bit-identical to the forward frame -- keeping only
// this path's vertices, then sweeps them backwards to turn the pixel's adjoint
// dL/dI / spp into gradients w.r.t. the albedo of every matte vertex and the emission
// of every emissive vertex and sampled light.  Memory stays O(pixels): nothing of the
// forward frame is stored.  Geometry, visibility and the Russian-roulette decision are
// not differentiated (the roulette's 1 / p weight is).  Inst: the scene is a two-level
// tree (tv, is; v unused): each hit binds its instance's triangles, rows and material
// slots before it is shaded, as the wavefront shade kernel does.
template <bool Wide, bool Extended, bool Env, bool Inst>
__global__ void __launch_bounds__(kBlock, kAdjointMinBlocks) pt_adjoint(bvh_view v, tlas_view tv, inst_shade is,
                                                     shade_params sp, camera_basis cam, uint32_t width,
                                                     uint32_t height, uint32_t spp, uint32_t num_bounces,
                                                     const float4* __restrict__ img_adj, float* __restrict__ grad_albedo,
                                                     float* __restrict__ grad_emission, uint32_t* __restrict__ status)
{
    // one query of the replay: the scene's tree, or the two-level tree with the hit
    // instance bound into sp (closest-hit queries only; a shadow query binds nothing)
    auto query = [&](auto any_hit, v3 o, v3 d, float tmin, float tmax) -> trace_result {
        constexpr bool kAny = decltype(any_hit)::value;
        if constexpr (Inst)
        {
            tlas_result h = traverse_tlas<kAny>(tv, { o.x, o.y, o.z }, { d.x, d.y, d.z }, tmin, tmax, status);
            if (!kAny && h.tri >= 0)
            {
                const bvh_view bv = is.views[h.inst];
                sp.tris = bv.tris;
                sp.num_tris = bv.num_tris;
                sp.xform = is.forward + 3 * h.inst;
                sp.geom_base = is.geom_base[h.inst];
            }
            return trace_result{ h.tri, h.t, h.u, h.v };
        }
        else
        {
            return traverse_view<kAny, Wide>(v, { o.x, o.y, o.z }, { d.x, d.y, d.z }, tmin, tmax, status);
        }
    };
    const uint32_t full = 0xFFFFFFFFu;
    const uint32_t npix = width * height;
    const uint64_t gid = uint64_t(blockIdx.x) * kBlock + threadIdx.x;
    const bool active = gid < uint64_t(npix) * spp;
    const uint32_t pixel = active ? uint32_t(gid % npix) : 0u;
    const uint32_t sample = active ? uint32_t(gid / npix) : 0u;
    vertex_rec recs[kMaxReplay];
    int nrec = 0;
    v3 adj = { 0.0f, 0.0f, 0.0f };
    if (active)
    {
        sp.sample = sample;
        v3 d = primary_dir(cam, width, height, sp.frame, pixel, sample);
        v3 o = { cam.eye.x, cam.eye.y, cam.eye.z };
        path_state st{ { 1.0f, 1.0f, 1.0f }, { 0.0f, 0.0f, 0.0f }, 2u, kLastSpecular };
        for (uint32_t bounce = 0; bounce < num_bounces && bounce < uint32_t(kMaxReplay); ++bounce)
        {
            trace_result h = query(std::false_type{}, o, d, 0.0f, FLT_MAX);
            vertex_out out;
            shade_vertex<Extended, Env>(sp, pixel, bounce, o, d, 0.0f, FLT_MAX, h.tri, h.t, st, out, status);
            if (out.shadow)
            {
                trace_result sh = query(std::true_type{}, out.sh_o, out.sh_d, sp.epsilon, out.sh_tmax);
                if (sh.tri >= 0) out.rec.nee = 0;   // occluded: no contribution to differentiate
            }
            recs[nrec++] = out.rec;
            if (!out.cont) break;
            o = out.next_o;
            d = out.next_d;
        }
        if (st.flags & kFirstHit)
        {
            float4 a4 = img_adj[pixel];
            float inv = 1.0f / float(spp);
            adj = { a4.x * inv, a4.y * inv, a4.z * inv };
        }
    }
    // reverse sweep, warp-uniform so the gradient adds can be reduced per warp
    int kmax = __reduce_max_sync(full, nrec);
    v3 tbar = { 0.0f, 0.0f, 0.0f };   // adjoint of the throughput leaving vertex k
    for (int k = kmax - 1; k >= 0; --k)
    {
        bool here = active && k < nrec;
        v3 abar = { 0.0f, 0.0f, 0.0f }, ebar = { 0.0f, 0.0f, 0.0f }, lbar = { 0.0f, 0.0f, 0.0f };
        uint32_t geom = 0, lgeom = 0;
        bool add_a = false, add_e = false, add_l = false;
        if (here)
        {
            vertex_rec const& r = recs[k];
            geom = r.geom;
            if (r.kind == kVertexMiss)
            {
                // the ambient or environment light the ray left into
                tbar = adj * (Env ? r.f.spec : v3{ sp.ambient.x, sp.ambient.y, sp.ambient.z });
            }
            else if (r.kind == kVertexEnd)
            {
                tbar = { 0.0f, 0.0f, 0.0f };
            }
            else if (r.kind == kVertexSpecular || r.kind == kVertexPlastic)
            {
                // thr' = thr * spec (then / rr): a fixed factor, nothing to differentiate
                v3 ub = r.rr > 0.0f ? roulette_adjoint(tbar, r.thr * r.f.spec, r.rr) : tbar;
                v3 tb = ub * r.f.spec;
                if (r.kind == kVertexPlastic && r.nee)
                {
                    // N = w * thr * gnee * lint
                    tb = nee_throughput_adjoint(r, adj, r.gnee * r.lint, tb);
                    if (r.lgeom != 0xFFFFFFFFu && r.lgeom < sp.num_materials)
                    {
                        lgeom = r.lgeom;
                        lbar = adj * r.thr * r.gnee * (r.w * r.kl);
                        add_l = true;
                    }
                }
                tbar = tb;
            }
            else if (r.kind == kVertexEmission)
            {
                gbrt_material m = sp.materials[geom];
                v3 e = sp.emission ? param3(sp.emission, geom) : v3{ m.color[0], m.color[1], m.color[2] };
                ebar = adj * r.thr * (r.f.emit.mis * r.f.emit.scale);
                add_e = sp.emission != nullptr;
                tbar = adj * e * (r.f.emit.mis * r.f.emit.scale);
            }
            else
            {
                gbrt_material m = sp.materials[geom];
                v3 a = sp.albedo ? param3(sp.albedo, geom) : v3{ m.color[0], m.color[1], m.color[2] };
                // throughput update thr' = thr * a * sigma (then / rr)
                v3 ub = r.rr > 0.0f ? roulette_adjoint(tbar, r.thr * a * r.f.sigma, r.rr) : tbar;
                abar = ub * r.thr * r.f.sigma;
                v3 tb = ub * a * r.f.sigma;
                if (r.nee)
                {
                    // N = w * thr * a * gnee * lint
                    v3 f = r.gnee * r.lint;
                    abar = abar + adj * r.thr * f * r.w;
                    tb = nee_throughput_adjoint(r, adj, a * f, tb);
                    if (r.lgeom != 0xFFFFFFFFu && r.lgeom < sp.num_materials)
                    {
                        lgeom = r.lgeom;
                        lbar = adj * r.thr * a * r.gnee * (r.w * r.kl);
                        add_l = true;
                    }
                }
                tbar = tb;
                add_a = sp.albedo != nullptr;
            }
        }
        warp_add3(grad_albedo, geom, abar, add_a);
        warp_add3(grad_emission, geom, ebar, add_e);
        warp_add3(grad_emission, lgeom, lbar, add_l);
    }
}

inline size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

gbrt_status frame_buffers_for(gbrt_context* ctx, uint32_t n, frame_buffers& fb)
{
    size_t sizes[] = { size_t(n) * 32, size_t(n) * 32, size_t(n) * 4, size_t(n) * 4, size_t(n) * 16,
                       size_t(n) * 32, size_t(n) * 4,  size_t(n) * 16, size_t(n) * 16, size_t(n) * 16,
                       size_t(n) * 8,  size_t(n) * 16, 64, size_t(n) * 4, size_t(n) * 4, size_t(n) * 4,
                       size_t(n) * 4, radix_sort_scratch_bytes(n) };
    constexpr int kParts = int(sizeof(sizes) / sizeof(sizes[0]));
    size_t total = 0;
    for (size_t s : sizes) total += align256(s);
    if (ctx->pt_scratch_bytes < total)
    {
        if (ctx->pt_scratch)
        {
            GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            GBRT_CUDA(ctx, cudaFree(ctx->pt_scratch));
            ctx->pt_scratch = nullptr;
            ctx->pt_scratch_bytes = 0;
        }
        GBRT_CUDA(ctx, cudaMalloc(&ctx->pt_scratch, total));
        ctx->pt_scratch_bytes = total;
    }
    char* base = static_cast<char*>(ctx->pt_scratch);
    void* ptr[kParts];
    size_t off = 0;
    for (int k = 0; k < kParts; ++k)
    {
        ptr[k] = base + off;
        off += align256(sizes[k]);
    }
    fb.rays[0] = static_cast<gbrt_ray*>(ptr[0]);
    fb.rays[1] = static_cast<gbrt_ray*>(ptr[1]);
    fb.path[0] = static_cast<uint32_t*>(ptr[2]);
    fb.path[1] = static_cast<uint32_t*>(ptr[3]);
    fb.hits = static_cast<uint4*>(ptr[4]);
    fb.shadow_rays = static_cast<gbrt_ray*>(ptr[5]);
    fb.shadow_path = static_cast<uint32_t*>(ptr[6]);
    fb.shadow_contrib = static_cast<float4*>(ptr[7]);
    fb.throughput = static_cast<float4*>(ptr[8]);
    fb.radiance = static_cast<float4*>(ptr[9]);
    fb.rng_flags = static_cast<uint2*>(ptr[10]);
    fb.sum = static_cast<float4*>(ptr[11]);
    fb.counts = static_cast<uint32_t*>(ptr[12]);
    fb.keys = static_cast<uint32_t*>(ptr[13]);
    fb.vals = static_cast<uint32_t*>(ptr[14]);
    fb.keys_alt = static_cast<uint32_t*>(ptr[15]);
    fb.vals_alt = static_cast<uint32_t*>(ptr[16]);
    fb.sort_scratch = ptr[17];
    return GBRT_OK;
}


} // namespace
} // namespace gbrt

using namespace gbrt;

namespace gbrt {
namespace {

// Fills the sample-angle table: entry k holds cos and sin of theta = two_pi * u with
// u = k / 2^24, exactly as the shading code forms u (gbrt_rng_u01) and theta, each
// evaluated in double and rounded once to float.
__global__ void __launch_bounds__(kBlock) fill_trig(float2* __restrict__ table)
{
    const float two_pi = 6.28318530717958623199592693709e+00f;
    uint32_t k = blockIdx.x * kBlock + threadIdx.x;
    if (k >= (1u << 24)) return;
    float u = float(k) * (1.0f / 16777216.0f);
    float theta = two_pi * u;
    table[k] = make_float2(float(cos(double(theta))), float(sin(double(theta))));
}

} // namespace

gbrt_status ensure_trig_table(gbrt_context* ctx)
{
    if (ctx->d_trig) return GBRT_OK;
    device_guard g(ctx->device);
    GBRT_CUDA(ctx, cudaMalloc(&ctx->d_trig, (size_t(1) << 24) * sizeof(float2)));
    fill_trig<<<(1u << 24) / kBlock, kBlock, 0, ctx->stream>>>(ctx->d_trig);
    GBRT_LAUNCH_CHECK(ctx, "fill_trig");
    return GBRT_OK;
}

namespace {

// The device record of an area light: 4 float4 = v1 (w: the triangle's geom_id bits),
// e1 (w: 0), e2, intensity cl * kl (w: kl), as area_light::intensity
// (area_light.inl:22-25).
void area_record(gbrt_triangle const& t, const float cl[3], float kl, float4* r)
{
    uint32_t lg = t.geom_id;
    r[0] = make_float4(t.v1[0], t.v1[1], t.v1[2], 0.0f);
    memcpy(&r[0].w, &lg, 4);
    r[1] = make_float4(t.e1[0], t.e1[1], t.e1[2], 0.0f);
    r[2] = make_float4(t.e2[0], t.e2[1], t.e2[2], 0.0f);
    r[3] = make_float4(cl[0] * kl, cl[1] * kl, cl[2] * kl, kl);
}

// The device record of a point or spot light: position (w: no geom_id), e1.w = 1
// marks a delta light, and the sample's intensity: intensity(pos) * pi evaluated, as
// point_light::sample and spot_light::sample do, at pos = the light's own position
// (point_light.inl:16-56, spot_light.inl:14-62), in the reference's float arithmetic.
void delta_record(gbrt_light const& l, float4* r)
{
    const float pi = 3.14159265358979323846264338328e+00f;
    const float d[3] = { l.position[0] - l.position[0], l.position[1] - l.position[1], l.position[2] - l.position[2] };
    const float dist = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const float att = float(1.0 / (l.attenuation[0] + l.attenuation[1] * dist + l.attenuation[2] * dist * dist));
    float spot = 1.0f;
    if (l.kind == GBRT_LIGHT_SPOT)
    {
        // light_dir = position - pos = 0: normalize(-light_dir) = 0 * (1 / sqrt(0))
        const float nd[3] = { -d[0], -d[1], -d[2] };
        const float inv = 1.0f / std::sqrt(nd[0] * nd[0] + nd[1] * nd[1] + nd[2] * nd[2]);
        const float c = l.spot_direction[0] * (nd[0] * inv) + l.spot_direction[1] * (nd[1] * inv) +
                        l.spot_direction[2] * (nd[2] * inv);
        spot = c > std::cos(l.spot_cutoff) ? std::pow(c, l.spot_exponent) : 0.0f;
    }
    float in[3];
    for (int c = 0; c < 3; ++c) in[c] = ((l.cl[c] * l.kl) * att * spot) * pi;
    const uint32_t none = 0xFFFFFFFFu;
    r[0] = make_float4(l.position[0], l.position[1], l.position[2], 0.0f);
    memcpy(&r[0].w, &none, 4);
    r[1] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    r[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    r[3] = make_float4(in[0], in[1], in[2], l.kl);
}

gbrt_status create_scene(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_material const* h_materials,
                         uint32_t num_materials, std::vector<float4> const& light_records, gbrt_pt_scene** out)
{
    device_guard g(ctx->device);
    gbrt_status tst = ensure_trig_table(ctx);   // once per context, here rather than in a frame
    if (tst != GBRT_OK) return tst;
    auto* sc = new (std::nothrow) gbrt_pt_scene;
    if (!sc) return fail(ctx, GBRT_ERR_OUT_OF_MEMORY, "pt_scene_create: host allocation");
    sc->bvh = bvh;
    sc->device = ctx->device;
    sc->num_materials = num_materials;
    sc->num_lights = uint32_t(light_records.size() / 4);
    for (uint32_t k = 0; k < num_materials; ++k)
    {
        const uint32_t kind = h_materials[k].kind;
        sc->extended |= kind == GBRT_MATERIAL_MIRROR || kind == GBRT_MATERIAL_GLASS || kind == GBRT_MATERIAL_PLASTIC;
    }
    auto cleanup = [&]() {
        cudaFree(sc->materials);
        cudaFree(sc->lights);
        delete sc;
    };
    if (num_materials)
    {
        cudaError_t e = cudaMalloc(&sc->materials, size_t(num_materials) * sizeof(gbrt_material));
        if (e == cudaSuccess)
            e = cudaMemcpy(sc->materials, h_materials, size_t(num_materials) * sizeof(gbrt_material),
                           cudaMemcpyHostToDevice);
        if (e != cudaSuccess)
        {
            cleanup();
            return check_cuda(ctx, e, "pt_scene_create: materials");
        }
    }
    if (!light_records.empty())
    {
        cudaError_t e = cudaMalloc(&sc->lights, light_records.size() * sizeof(float4));
        if (e == cudaSuccess)
            e = cudaMemcpy(sc->lights, light_records.data(), light_records.size() * sizeof(float4),
                           cudaMemcpyHostToDevice);
        if (e != cudaSuccess)
        {
            cleanup();
            return check_cuda(ctx, e, "pt_scene_create: lights");
        }
    }
    *out = sc;
    return GBRT_OK;
}

} // namespace
} // namespace gbrt

extern "C" gbrt_status gbrt_pt_scene_create(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_material const* h_materials,
                                            uint32_t num_materials, gbrt_area_light const* h_lights,
                                            uint32_t num_lights, gbrt_pt_scene** out)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!out || !bvh) return fail(ctx, GBRT_ERR_INVALID_ARG, "pt_scene_create: null bvh or output");
    *out = nullptr;
    if ((num_materials && !h_materials) || (num_lights && !h_lights))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "pt_scene_create: null material or light array");
    for (uint32_t k = 0; k < num_materials; ++k)
        if (h_materials[k].kind > GBRT_MATERIAL_PLASTIC)
            return fail(ctx, GBRT_ERR_INVALID_ARG, "pt_scene_create: unknown material kind");
    std::vector<float4> rec(size_t(num_lights) * 4);
    for (uint32_t k = 0; k < num_lights; ++k)
        area_record(h_lights[k].geometry, h_lights[k].cl, h_lights[k].kl, &rec[4 * k]);
    return create_scene(ctx, bvh, h_materials, num_materials, rec, out);
}

extern "C" gbrt_status gbrt_pt_scene_create_lights(gbrt_context* ctx, gbrt_bvh const* bvh,
                                                   gbrt_material const* h_materials, uint32_t num_materials,
                                                   gbrt_light const* h_lights, uint32_t num_lights,
                                                   gbrt_pt_scene** out)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!out || !bvh) return fail(ctx, GBRT_ERR_INVALID_ARG, "pt_scene_create_lights: null bvh or output");
    *out = nullptr;
    if ((num_materials && !h_materials) || (num_lights && !h_lights))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "pt_scene_create_lights: null material or light array");
    for (uint32_t k = 0; k < num_materials; ++k)
        if (h_materials[k].kind > GBRT_MATERIAL_PLASTIC)
            return fail(ctx, GBRT_ERR_INVALID_ARG, "pt_scene_create_lights: unknown material kind");
    std::vector<float4> rec;
    gbrt_status st = light_records(ctx, h_lights, num_lights, rec, "pt_scene_create_lights");
    if (st != GBRT_OK) return st;
    return create_scene(ctx, bvh, h_materials, num_materials, rec, out);
}

gbrt_status gbrt::light_records(gbrt_context* ctx, gbrt_light const* h_lights, uint32_t num_lights,
                                std::vector<float4>& out, const char* who)
{
    out.assign(size_t(num_lights) * 4, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (uint32_t k = 0; k < num_lights; ++k)
    {
        gbrt_light const& l = h_lights[k];
        if (l.kind == GBRT_LIGHT_AREA)
            area_record(l.geometry, l.cl, l.kl, &out[4 * k]);
        else if (l.kind == GBRT_LIGHT_POINT || l.kind == GBRT_LIGHT_SPOT)
            delta_record(l, &out[4 * k]);
        else
            return fail(ctx, GBRT_ERR_INVALID_ARG, std::string(who) + ": unknown light kind");
    }
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_pt_scene_create_instanced(gbrt_context* ctx, gbrt_tlas const* tlas,
                                                      gbrt_material const* h_materials, uint32_t num_materials,
                                                      gbrt_light const* h_lights, uint32_t num_lights,
                                                      uint32_t const* h_inst_geom, gbrt_pt_scene** out)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!out || !tlas) return fail(ctx, GBRT_ERR_INVALID_ARG, "pt_scene_create_instanced: null tree or output");
    *out = nullptr;
    if ((num_materials && !h_materials) || (num_lights && !h_lights) || (tlas->num_instances && !h_inst_geom))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "pt_scene_create_instanced: null array");
    for (uint32_t k = 0; k < num_materials; ++k)
        if (h_materials[k].kind > GBRT_MATERIAL_PLASTIC)
            return fail(ctx, GBRT_ERR_INVALID_ARG, "pt_scene_create_instanced: unknown material kind");
    if (tlas->device != ctx->device) return fail(ctx, GBRT_ERR_INVALID_ARG, "pt_scene_create_instanced: tree on another device");
    std::vector<float4> rec;
    gbrt_status st = light_records(ctx, h_lights, num_lights, rec, "pt_scene_create_instanced");
    if (st != GBRT_OK) return st;
    gbrt_pt_scene* sc = nullptr;
    st = create_scene(ctx, nullptr, h_materials, num_materials, rec, &sc);
    if (st != GBRT_OK) return st;
    sc->tlas = tlas;
    if (tlas->num_instances)
    {
        device_guard g(ctx->device);
        cudaError_t e = cudaMalloc(&sc->inst_geom, size_t(tlas->num_instances) * 4);
        if (e == cudaSuccess)
            e = cudaMemcpy(sc->inst_geom, h_inst_geom, size_t(tlas->num_instances) * 4, cudaMemcpyHostToDevice);
        if (e != cudaSuccess)
        {
            gbrt_pt_scene_destroy(sc);
            return check_cuda(ctx, e, "pt_scene_create_instanced");
        }
    }
    *out = sc;
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_pinhole_camera_basis(gbrt_camera const* camera, uint32_t width, uint32_t height, float* out)
{
    if (!camera || !out || width == 0 || height == 0) return GBRT_ERR_INVALID_ARG;
    camera_basis b = camera_for(*camera, width, height);
    const float3 v[4] = { b.eye, b.U, b.V, b.W };
    for (int k = 0; k < 4; ++k)
    {
        out[3 * k + 0] = v[k].x;
        out[3 * k + 1] = v[k].y;
        out[3 * k + 2] = v[k].z;
    }
    return GBRT_OK;
}

namespace gbrt {
namespace {

// Rows 0-2 of the inverse of the column-major 4x4 `a`, as the reference's float inverse
// forms it (math/detail/matrix4.inl:353-388): the 2x2 minors of rows 0-1 (s0..s5) and
// rows 2-3 (c0..c5), the determinant from them, each cofactor sum over it.  m(r, c) =
// a[4c + r]; out[4r + c] = inverse(r, c).  False for a zero or non-finite determinant.
bool inverse_rows(const float a[16], float out[12])
{
    auto m = [&](int r, int c) { return a[4 * c + r]; };
    auto det2 = [](float m00, float m01, float m10, float m11) { return m00 * m11 - m10 * m01; };
    const float s0 = det2(m(0, 0), m(0, 1), m(1, 0), m(1, 1));
    const float s1 = det2(m(0, 0), m(0, 2), m(1, 0), m(1, 2));
    const float s2 = det2(m(0, 0), m(0, 3), m(1, 0), m(1, 3));
    const float s3 = det2(m(0, 1), m(0, 2), m(1, 1), m(1, 2));
    const float s4 = det2(m(0, 1), m(0, 3), m(1, 1), m(1, 3));
    const float s5 = det2(m(0, 2), m(0, 3), m(1, 2), m(1, 3));
    const float c5 = det2(m(2, 2), m(2, 3), m(3, 2), m(3, 3));
    const float c4 = det2(m(2, 1), m(2, 3), m(3, 1), m(3, 3));
    const float c3 = det2(m(2, 1), m(2, 2), m(3, 1), m(3, 2));
    const float c2 = det2(m(2, 0), m(2, 3), m(3, 0), m(3, 3));
    const float c1 = det2(m(2, 0), m(2, 2), m(3, 0), m(3, 2));
    const float c0 = det2(m(2, 0), m(2, 1), m(3, 0), m(3, 1));
    const float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    if (!(det != 0.0f) || !std::isfinite(det)) return false;
    out[0] = (m(1, 1) * c5 - m(1, 2) * c4 + m(1, 3) * c3) / det;
    out[4] = (-m(1, 0) * c5 + m(1, 2) * c2 + m(1, 3) * c1) / det;
    out[8] = (m(1, 0) * c4 - m(1, 1) * c2 + m(1, 3) * c0) / det;
    out[1] = (-m(0, 1) * c5 + m(0, 2) * c4 - m(0, 3) * c3) / det;
    out[5] = (m(0, 0) * c5 - m(0, 2) * c2 + m(0, 3) * c1) / det;
    out[9] = (-m(0, 0) * c4 + m(0, 1) * c2 - m(0, 3) * c0) / det;
    out[2] = (m(3, 1) * s5 - m(3, 2) * s4 + m(3, 3) * s3) / det;
    out[6] = (-m(3, 0) * s5 + m(3, 2) * s2 - m(3, 3) * s1) / det;
    out[10] = (m(3, 0) * s4 - m(3, 1) * s2 + m(3, 3) * s0) / det;
    out[3] = (-m(2, 1) * s5 + m(2, 2) * s4 - m(2, 3) * s3) / det;
    out[7] = (m(2, 0) * s5 - m(2, 2) * s2 + m(2, 3) * s1) / det;
    out[11] = (-m(2, 0) * s4 + m(2, 1) * s2 - m(2, 3) * s0) / det;
    return true;
}

} // namespace
} // namespace gbrt

extern "C" gbrt_status gbrt_pt_scene_set_environment(gbrt_context* ctx, gbrt_pt_scene* scene,
                                                     gbrt_environment const* env)
{
    using namespace gbrt;
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!scene) return fail(ctx, GBRT_ERR_INVALID_ARG, "set_environment: null scene");
    device_guard g(scene->device);
    if (!env)
    {
        // the stream may still render with the old record: free it after the stream drains
        GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFree(scene->env);
        scene->env = nullptr;
        return GBRT_OK;
    }
    if (!env->d_texels || (reinterpret_cast<uintptr_t>(env->d_texels) & 15u))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "set_environment: texels must be a 16-byte aligned device pointer");
    if (env->width == 0 || env->height == 0 || env->width > (1u << 16) || env->height > (1u << 16))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "set_environment: width and height must be 1 .. 65536");
    if (env->filter > GBRT_FILTER_LINEAR || env->address > GBRT_ADDRESS_CLAMP)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "set_environment: unknown filter or address mode");
    env_view v;
    if (!inverse_rows(env->light_to_world, v.m))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "set_environment: light_to_world is singular");
    v.texels = reinterpret_cast<const float4*>(env->d_texels);
    v.width = env->width;
    v.height = env->height;
    v.filter = env->filter;
    v.address = env->address;
    for (int k = 0; k < 3; ++k) v.scale[k] = env->scale[k];
    // frames already enqueued read the previous record: replace it once they are done
    GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (!scene->env) GBRT_CUDA(ctx, cudaMalloc(&scene->env, sizeof(env_view)));
    GBRT_CUDA(ctx, cudaMemcpy(scene->env, &v, sizeof(env_view), cudaMemcpyHostToDevice));
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_pt_scene_destroy(gbrt_pt_scene* scene)
{
    if (!scene) return GBRT_ERR_INVALID_ARG;
    device_guard g(scene->device);
    cudaFree(scene->materials);
    cudaFree(scene->lights);
    cudaFree(scene->env);
    cudaFree(scene->inst_geom);
    delete scene;
    return GBRT_OK;
}

namespace gbrt {
namespace {

gbrt_status check_frame_args(gbrt_context* ctx, gbrt_pt_scene const* scene, gbrt_camera const* camera,
                             gbrt_pt_params const* params, const void* img, const char* who)
{
    if (!scene || !camera || !params || !img) return fail(ctx, GBRT_ERR_INVALID_ARG, std::string(who) + ": null argument");
    gbrt_pt_params const& p = *params;
    if (p.width == 0 || p.height == 0 || p.spp == 0)
        return fail(ctx, GBRT_ERR_INVALID_ARG, std::string(who) + ": empty frame");
    if (uint64_t(p.width) * p.height > (1ull << 28))
        return fail(ctx, GBRT_ERR_TOO_LARGE, std::string(who) + ": more than 2^28 pixels");
    return GBRT_OK;
}

shade_params shade_params_for(gbrt_context const* ctx, gbrt_pt_scene const* scene, gbrt_pt_params const& p,
                              const float* albedo, const float* emission)
{
    shade_params sp;
    sp.trig = ctx->d_trig;
    sp.materials = scene->materials;
    sp.num_materials = scene->num_materials;
    sp.lights = scene->lights;
    sp.num_lights = scene->num_lights;
    sp.tris = scene->bvh ? scene->bvh->tris : nullptr;   // instanced scenes: set per hit
    sp.num_tris = scene->bvh ? int32_t(scene->bvh->num_prims) : 0;
    sp.epsilon = p.epsilon;
    sp.ambient = make_float3(p.ambient[0], p.ambient[1], p.ambient[2]);
    sp.frame = p.frame_id;
    sp.sample = 0;
    sp.bounce = 0;
    sp.flags = p.flags;
    sp.albedo = albedo;
    sp.emission = emission;
    sp.env = scene->env;
    return sp;
}

// The frame's average blended into accum and written to color (cuda_sched's blend).
gbrt_status finish_frame(gbrt_context* ctx, frame_buffers const& fb, gbrt_pt_params const& p, uint32_t blocks,
                         float* d_accum, float* d_color)
{
    const uint32_t n = p.width * p.height;
    pt_blend<<<blocks, kBlock, 0, ctx->stream>>>(fb, n, float(p.spp), p.sfactor, p.dfactor,
                                                 reinterpret_cast<float4*>(d_accum), reinterpret_cast<float4*>(d_color));
    GBRT_LAUNCH_CHECK(ctx, "pt_blend");
    return GBRT_OK;
}

// The wavefront frame of a scene over a two-level tree: each queue traced through the
// top-level tree and the instances' trees (traverse_tlas), each hit shaded with its
// instance's triangle carried to world space and its instance's material slots.
gbrt_status render_frame_instanced(gbrt_context* ctx, gbrt_pt_scene const* scene, camera_basis const& cam,
                                   gbrt_pt_params const& p, shade_params sp, float4 bg, uint32_t blocks,
                                   float* d_accum, float* d_color)
{
    if (p.flags & (GBRT_PT_MEGAKERNEL | GBRT_PT_SORT_QUEUES))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "pathtrace: the megakernel and sorted queues take a single tree");
    const uint32_t n = p.width * p.height;
    cudaStream_t s = ctx->stream;
    gbrt_tlas const* t = scene->tlas;
    const tlas_view tv{ t->nodes, t->records, t->views, t->num_instances > 0 ? t->root : kEmptyLink,
                        int32_t(t->num_inner), int32_t(t->num_instances) };
    const inst_shade is{ t->views, t->forward, scene->inst_geom, int32_t(t->num_instances) };
    frame_buffers fb;
    gbrt_status st = frame_buffers_for(ctx, n, fb);
    if (st != GBRT_OK) return st;
    for (uint32_t smp = 0; smp < p.spp; ++smp)
    {
        sp.sample = smp;
        pt_raygen<<<blocks, kBlock, 0, s>>>(fb, p.width, p.height, p.frame_id, smp, cam);
        GBRT_LAUNCH_CHECK(ctx, "pt_raygen");
        int q = 0;
        for (uint32_t b = 0; b < p.num_bounces && t->num_instances > 0; ++b)
        {
            sp.bounce = b;
            pt_extend_tlas<<<blocks, kBlock, 0, s>>>(fb, q, tv, ctx->d_status);
            GBRT_LAUNCH_CHECK(ctx, "pt_extend_tlas");
            pt_shade<<<blocks, kBlock, 0, s>>>(fb, q, sp, is, ctx->d_status);
            GBRT_LAUNCH_CHECK(ctx, "pt_shade");
            if (scene->num_lights > 0)
            {
                pt_shadow_tlas<<<blocks, kBlock, 0, s>>>(fb, tv, ctx->d_status);
                GBRT_LAUNCH_CHECK(ctx, "pt_shadow_tlas");
            }
            q ^= 1;
        }
        pt_accumulate<<<blocks, kBlock, 0, s>>>(fb, n, smp, bg);
        GBRT_LAUNCH_CHECK(ctx, "pt_accumulate");
    }
    return finish_frame(ctx, fb, p, blocks, d_accum, d_color);
}

// One frame of the wavefront path tracer into accum (blended) and color.
gbrt_status render_frame(gbrt_context* ctx, gbrt_pt_scene const* scene, gbrt_camera const& camera,
                         gbrt_pt_params const& p, const float* albedo, const float* emission, float* d_accum,
                         float* d_color)
{
    if ((reinterpret_cast<uintptr_t>(d_accum) & 15u) || (reinterpret_cast<uintptr_t>(d_color) & 15u))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "pathtrace: images must be 16-byte aligned");
    const uint32_t n = p.width * p.height;
    camera_basis cam = camera_for(camera, p.width, p.height);
    gbrt_bvh const* bvh = scene->bvh;
    gbrt_status tst = ensure_trig_table(ctx);   // a no-op unless the scene came from another context
    if (tst != GBRT_OK) return tst;
    shade_params sp = shade_params_for(ctx, scene, p, albedo, emission);
    // background: ambient_light(bg.xyz, bg.w).intensity with alpha 1 (kernels.h:172-174,
    // pathtracing.inl:62)
    float4 bg = make_float4(p.background[0] * p.background[3], p.background[1] * p.background[3],
                            p.background[2] * p.background[3], 1.0f);
    const uint32_t blocks = (n + kBlock - 1) / kBlock;
    cudaStream_t s = ctx->stream;
    if (scene->tlas)
        return render_frame_instanced(ctx, scene, cam, p, sp, bg, blocks, d_accum, d_color);
    const bvh_view v = view_of(bvh);
    const bool wide = bvh->nodes4 != nullptr && (ctx->trace_flags & GBRT_TRACE_WIDE_NODES);
    if (p.flags & GBRT_PT_MEGAKERNEL)
    {
        auto launch = [&](auto kernel) {
            kernel<<<blocks, kBlock, 0, s>>>(v, sp, cam, p.width, p.height, p.spp, p.num_bounces, bg, p.sfactor,
                                             p.dfactor, reinterpret_cast<float4*>(d_accum),
                                             reinterpret_cast<float4*>(d_color), ctx->d_status);
        };
        wide ? launch(pt_megakernel<true>) : launch(pt_megakernel<false>);
        GBRT_LAUNCH_CHECK(ctx, "pt_megakernel");
        return GBRT_OK;
    }
    frame_buffers fb;
    gbrt_status st = frame_buffers_for(ctx, n, fb);
    if (st != GBRT_OK) return st;
    // GBRT_PT_SORT_QUEUES: each bounce's ray and shadow queues ordered by origin cell of
    // the scene box before they are traced (as the ray queries order their rays).
    // Measured slower on the box scene (1920x1080x64: 847 vs 703 ms per frame; a sort of
    // the full queue per bounce and per shadow pass, for little coherence among diffuse
    // bounces), so it is an option.
    const bool sort = (p.flags & GBRT_PT_SORT_QUEUES) && bvh->num_prims > 0;
    const float3 lo = make_float3(bvh->lo[0], bvh->lo[1], bvh->lo[2]);
    float ext[3] = { bvh->hi[0] - bvh->lo[0], bvh->hi[1] - bvh->lo[1], bvh->hi[2] - bvh->lo[2] };
    const float3 scale = make_float3(ext[0] > 0.0f ? 256.0f / ext[0] : 0.0f, ext[1] > 0.0f ? 256.0f / ext[1] : 0.0f,
                                     ext[2] > 0.0f ? 256.0f / ext[2] : 0.0f);
    for (uint32_t smp = 0; smp < p.spp; ++smp)
    {
        sp.sample = smp;
        pt_raygen<<<blocks, kBlock, 0, s>>>(fb, p.width, p.height, p.frame_id, smp, cam);
        GBRT_LAUNCH_CHECK(ctx, "pt_raygen");
        int q = 0;
        if (bvh->num_prims > 0)
        {
            for (uint32_t b = 0; b < p.num_bounces; ++b)
            {
                sp.bounce = b;
                // camera rays are coherent in pixel order; later queues are ordered by origin
                if (sort && b > 0)
                {
                    pt_queue_keys<<<blocks, kBlock, 0, s>>>(fb.rays[q], fb.counts + q, n, lo, scale, fb.keys, fb.vals);
                    GBRT_LAUNCH_CHECK(ctx, "pt_queue_keys");
                    st = radix_sort_pairs(ctx, fb.keys, fb.vals, fb.keys_alt, fb.vals_alt, n, 24, fb.sort_scratch, s);
                    if (st != GBRT_OK) return st;
                    if (wide)
                        pt_extend_sorted<true><<<blocks, kBlock, 0, s>>>(fb, q, fb.vals, v, ctx->d_status);
                    else
                        pt_extend_sorted<false><<<blocks, kBlock, 0, s>>>(fb, q, fb.vals, v, ctx->d_status);
                }
                else if (wide)
                {
                    pt_extend<true><<<blocks, kBlock, 0, s>>>(fb, q, v, ctx->d_status);
                }
                else
                {
                    pt_extend<false><<<blocks, kBlock, 0, s>>>(fb, q, v, ctx->d_status);
                }
                GBRT_LAUNCH_CHECK(ctx, "pt_extend");
                pt_shade<<<blocks, kBlock, 0, s>>>(fb, q, sp, inst_shade{ nullptr, nullptr, nullptr, 0 },
                                                   ctx->d_status);
                GBRT_LAUNCH_CHECK(ctx, "pt_shade");
                if (scene->num_lights > 0)
                {
                    if (sort)
                    {
                        pt_queue_keys<<<blocks, kBlock, 0, s>>>(fb.shadow_rays, fb.counts + 2, n, lo, scale, fb.keys,
                                                                fb.vals);
                        GBRT_LAUNCH_CHECK(ctx, "pt_queue_keys");
                        st = radix_sort_pairs(ctx, fb.keys, fb.vals, fb.keys_alt, fb.vals_alt, n, 24, fb.sort_scratch,
                                              s);
                        if (st != GBRT_OK) return st;
                        if (wide)
                            pt_shadow_sorted<true><<<blocks, kBlock, 0, s>>>(fb, fb.vals, v, ctx->d_status);
                        else
                            pt_shadow_sorted<false><<<blocks, kBlock, 0, s>>>(fb, fb.vals, v, ctx->d_status);
                    }
                    else if (wide)
                    {
                        pt_shadow<true><<<blocks, kBlock, 0, s>>>(fb, v, ctx->d_status);
                    }
                    else
                    {
                        pt_shadow<false><<<blocks, kBlock, 0, s>>>(fb, v, ctx->d_status);
                    }
                    GBRT_LAUNCH_CHECK(ctx, "pt_shadow");
                }
                q ^= 1;
            }
        }
        pt_accumulate<<<blocks, kBlock, 0, s>>>(fb, n, smp, bg);
        GBRT_LAUNCH_CHECK(ctx, "pt_accumulate");
    }
    return finish_frame(ctx, fb, p, blocks, d_accum, d_color);
}

} // namespace
} // namespace gbrt

extern "C" gbrt_status gbrt_pathtrace_frame(gbrt_context* ctx, gbrt_pt_scene const* scene, gbrt_camera const* camera,
                                            gbrt_pt_params const* params, float* d_accum, float* d_color)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    gbrt_status st = check_frame_args(ctx, scene, camera, params, d_accum, "pathtrace_frame");
    if (st != GBRT_OK) return st;
    device_guard g(ctx->device);
    return render_frame(ctx, scene, *camera, *params, nullptr, nullptr, d_accum, d_color);
}

extern "C" gbrt_status gbrt_pathtrace_forward(gbrt_context* ctx, gbrt_pt_scene const* scene, gbrt_camera const* camera,
                                              gbrt_pt_params const* params, const float* d_albedo,
                                              const float* d_emission, float* d_image)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    gbrt_status st = check_frame_args(ctx, scene, camera, params, d_image, "pathtrace_forward");
    if (st != GBRT_OK) return st;
    if (!d_albedo || !d_emission) return fail(ctx, GBRT_ERR_INVALID_ARG, "pathtrace_forward: null parameters");
    gbrt_pt_params p = *params;
    p.sfactor = 1.0f;   // the image is this frame alone
    p.dfactor = 0.0f;
    device_guard g(ctx->device);
    return render_frame(ctx, scene, *camera, p, d_albedo, d_emission, d_image, nullptr);
}

extern "C" gbrt_status gbrt_pathtrace_backward(gbrt_context* ctx, gbrt_pt_scene const* scene, gbrt_camera const* camera,
                                               gbrt_pt_params const* params, const float* d_albedo,
                                               const float* d_emission, const float* d_image_adjoint,
                                               float* d_grad_albedo, float* d_grad_emission)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    gbrt_status st = check_frame_args(ctx, scene, camera, params, d_image_adjoint, "pathtrace_backward");
    if (st != GBRT_OK) return st;
    if (!d_albedo || !d_emission || !d_grad_albedo || !d_grad_emission)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "pathtrace_backward: null parameter or gradient array");
    if (reinterpret_cast<uintptr_t>(d_image_adjoint) & 15u)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "pathtrace_backward: adjoint image must be 16-byte aligned");
    gbrt_pt_params const& p = *params;
    if (p.num_bounces > uint32_t(kMaxReplay))
        return fail(ctx, GBRT_ERR_TOO_LARGE, "pathtrace_backward: at most 16 bounces");
    gbrt_tlas const* t = scene->tlas;
    gbrt_bvh const* bvh = scene->bvh;
    if ((t ? t->num_instances == 0 : bvh->num_prims == 0) || scene->num_materials == 0)
        return GBRT_OK;   // nothing to differentiate
    device_guard g(ctx->device);
    camera_basis cam = camera_for(*camera, p.width, p.height);
    gbrt_status tst = ensure_trig_table(ctx);
    if (tst != GBRT_OK) return tst;
    shade_params sp = shade_params_for(ctx, scene, p, d_albedo, d_emission);
    const uint64_t paths = uint64_t(p.width) * p.height * p.spp;
    if (paths > (1ull << 31)) return fail(ctx, GBRT_ERR_TOO_LARGE, "pathtrace_backward: more than 2^31 paths");
    const uint32_t blocks = uint32_t((paths + kBlock - 1) / kBlock);
    bvh_view v{};
    tlas_view tv{};
    inst_shade is{ nullptr, nullptr, nullptr, 0 };
    bool wide = false;
    if (t)
    {
        tv = tlas_view{ t->nodes, t->records, t->views, t->root, int32_t(t->num_inner), int32_t(t->num_instances) };
        is = inst_shade{ t->views, t->forward, scene->inst_geom, int32_t(t->num_instances) };
    }
    else
    {
        v = view_of(bvh);
        wide = bvh->nodes4 != nullptr && (ctx->trace_flags & GBRT_TRACE_WIDE_NODES);
    }
    // matte / emissive scenes get the replay without the other materials' branches
    // (an environment light takes the full replay)
    auto kernel = t ? (scene->env        ? pt_adjoint<false, true, true, true>
                       : scene->extended ? pt_adjoint<false, true, false, true>
                                         : pt_adjoint<false, false, false, true>)
                  : scene->env ? (wide ? pt_adjoint<true, true, true, false> : pt_adjoint<false, true, true, false>)
                  : wide ? (scene->extended ? pt_adjoint<true, true, false, false> : pt_adjoint<true, false, false, false>)
                         : (scene->extended ? pt_adjoint<false, true, false, false>
                                            : pt_adjoint<false, false, false, false>);
    kernel<<<blocks, kBlock, 0, ctx->stream>>>(v, tv, is, sp, cam, p.width, p.height, p.spp, p.num_bounces,
                                               reinterpret_cast<const float4*>(d_image_adjoint), d_grad_albedo,
                                               d_grad_emission, ctx->d_status);
    GBRT_LAUNCH_CHECK(ctx, "pt_adjoint");
    return GBRT_OK;
}
