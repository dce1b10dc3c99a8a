// Batched path tracing: one frame of every scene of a gbrt_batch in ONE persistent
// launch, the batched build and that frame captured in one CUDA graph, and the
// autotuner over the launch shape.
//
// visionaray renders a scene with cuda_sched::frame (detail/cuda_sched.inl:226-246):
// one launch per frame and scene, one thread per pixel running pathtracing::kernel
// (detail/pathtracing.inl:42-233).  Hundreds of small scenes then cost hundreds of
// builds, launches and synchronisations, and a 64x64 frame fills a fraction of the
// GPU.  Here warps of a grid sized to the GPU (SMs x resident blocks) take tiles of
// `tile` pixels of any scene off one atomic counter, look their scene up by binary
// search over the pixel offsets, and run each pixel's samples and bounces in-thread:
// traversal of the scene's tree in the shared arena (traverse_bvh from the scene's
// root) and the same shade_vertex as the wavefront renderer (pt_shade.cuh), so scene
// s's image equals gbrt_pathtrace_frame's bit for bit.  Scenes with lights
// (gbrt_batch_set_lights) sample them as the megakernel renderer does: the light
// sample's shadow ray is an any-hit query through the scene's tree right after the
// vertex is shaded.  This unit is compiled with --fmad=false like pathtrace.cu.

#include "pt_shade.cuh"

#include <new>
#include <string>
#include <vector>

namespace gbrt {
namespace {

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
    const batch_frame* frames;
    const uint32_t* pixel_offsets;
    uint32_t num_scenes, total_pixels, tile, order;
    const bvh2_node* nodes;
    const tri48* tris;
    int32_t total_inner, total_tris;
    const gbrt_material* materials;
    uint32_t num_materials;
    const float4* lights;            // 4 float4 per light
    const uint32_t* light_offsets;   // scene s: lights [light_offsets[s], light_offsets[s + 1])
    const float2* trig;
    uint32_t* work;
    float4* images;
    uint32_t* status;
};

// Traversal stack entries kept in shared memory (a per-thread column, bank-conflict
// free); deeper entries in local memory.
constexpr int kBatchSharedStack = 8;
// Resident warps per SM the register allocation must allow (launch bounds): the full 64
// (32 registers, with spills) -- measured on the 512-scene batch, the frame kernel takes
// 87.7 / 79.8 / 74.9 / 71.8 / 67.4 ms at 24 / 32 / 40 / 48 / 64 warps: latency, not
// spill traffic, bounds it.
constexpr int kBatchWarpsPerSM = 64;

// Extended = false: a material table of matte and emissive slots only (the other
// materials' branches compiled out, as for the adjoint).  Lit = false: no scene has
// lights (the next-event path compiled out).
template <int Block, int Stack, bool Extended, bool Lit>
__global__ void __launch_bounds__(Block, kBatchWarpsPerSM * 32 / Block) batch_pt(batch_args a)
{
    const uint32_t full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    __shared__ int stack_mem[kBatchSharedStack * Block];
    shared_stack<kBatchSharedStack < Stack ? kBatchSharedStack : Stack - 1, Stack, Block> stack;
    stack.col = stack_mem + threadIdx.x;
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
            const uint32_t g = base + k;
            if (g >= a.total_pixels) break;
            const uint32_t s = upper_segment(a.pixel_offsets, a.num_scenes, g);
            const batch_frame f = a.frames[s];
            const uint32_t first = __ldg(&a.pixel_offsets[s]);
            const uint32_t local = g - first;
            uint32_t pixel = local;
            if (a.order == GBRT_BATCH_ORDER_BLOCKS && f.blocks)
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
            float4 sum = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            for (uint32_t smp = 0; smp < f.spp; ++smp)
            {
                sp.sample = smp;
                v3 o = eye;
                v3 d = primary_dir(f.cam, f.width, f.height, f.frame_id, pixel, smp);
                path_state st{ { 1.0f, 1.0f, 1.0f }, { 0.0f, 0.0f, 0.0f }, 2u, kLastSpecular };
                for (uint32_t bounce = 0; bounce < f.num_bounces; ++bounce)
                {
                    trace_result h = traverse_bvh_with<false>(stack, a.nodes, a.tris, f.root, a.total_inner,
                                                              a.total_tris, { o.x, o.y, o.z }, { d.x, d.y, d.z }, 0.0f,
                                                              FLT_MAX, a.status);
                    vertex_out out;
                    shade_vertex<Extended>(sp, pixel, bounce, o, d, 0.0f, FLT_MAX, h.tri, h.t, st, out, a.status);
                    if constexpr (Lit)
                    {
                        if (out.shadow)
                        {
                            trace_result sh = traverse_bvh_with<true>(
                                stack, a.nodes, a.tris, f.root, a.total_inner, a.total_tris,
                                { out.sh_o.x, out.sh_o.y, out.sh_o.z }, { out.sh_d.x, out.sh_d.y, out.sh_d.z },
                                sp.epsilon, out.sh_tmax, a.status);
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

using batch_kernel = void (*)(batch_args);

template <int Block, bool Extended, bool Lit>
batch_kernel pick_stack(uint32_t stack)
{
    switch (stack)
    {
    case 16: return batch_pt<Block, 16, Extended, Lit>;
    case 24: return batch_pt<Block, 24, Extended, Lit>;
    case 32: return batch_pt<Block, 32, Extended, Lit>;
    case 64: return batch_pt<Block, 64, Extended, Lit>;
    default: return nullptr;
    }
}

template <bool Extended, bool Lit>
batch_kernel pick_block(gbrt_batch_launch const& l)
{
    switch (l.block)
    {
    case 128: return pick_stack<128, Extended, Lit>(l.stack);
    case 256: return pick_stack<256, Extended, Lit>(l.stack);
    case 512: return pick_stack<512, Extended, Lit>(l.stack);
    default: return nullptr;
    }
}

batch_kernel pick_kernel(gbrt_batch_launch const& l, bool extended, bool lit)
{
    if (lit) return extended ? pick_block<true, true>(l) : pick_block<false, true>(l);
    return extended ? pick_block<true, false>(l) : pick_block<false, false>(l);
}

bool launch_valid(gbrt_batch_launch const& l)
{
    return pick_kernel(l, false, false) != nullptr && (l.tile == 32 || l.tile == 64) &&
           (l.order == GBRT_BATCH_ORDER_ROWS || l.order == GBRT_BATCH_ORDER_BLOCKS);
}

} // namespace

gbrt_status batch_pathtrace(gbrt_context* ctx, gbrt_batch const* b, float* d_images, cudaStream_t stream)
{
    if (b->frames_set != b->num_scenes) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: frames not set");
    if (!d_images || (reinterpret_cast<uintptr_t>(d_images) & 15u))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: images null or not 16-byte aligned");
    batch_kernel kernel = pick_kernel(b->launch, b->extended_materials, b->num_lights > 0);
    if (!kernel) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: bad launch shape");
    int per_sm = 0;
    GBRT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, int(b->launch.block), 0));
    if (per_sm < 1) per_sm = 1;
    // enough warps for every tile, at most one full wave of resident blocks
    const uint64_t warps_needed = (uint64_t(b->total_pixels) + b->launch.tile - 1) / b->launch.tile;
    const uint64_t blocks_needed = (warps_needed * 32 + b->launch.block - 1) / b->launch.block;
    uint64_t blocks = uint64_t(ctx->num_sms) * uint64_t(per_sm);
    if (blocks_needed < blocks) blocks = blocks_needed;
    if (blocks == 0) return GBRT_OK;
    batch_args a;
    a.frames = static_cast<const batch_frame*>(b->d_frames);
    a.pixel_offsets = b->d_pixel_offsets;
    a.num_scenes = b->num_scenes;
    a.total_pixels = b->total_pixels;
    a.tile = b->launch.tile;
    a.order = b->launch.order;
    a.nodes = b->nodes;
    a.tris = b->tris;
    a.total_inner = int32_t(b->total_inner);
    a.total_tris = int32_t(b->total);
    a.materials = b->d_materials;
    a.num_materials = b->num_materials;
    a.lights = b->d_lights;
    a.light_offsets = b->d_light_offsets;
    if (!ctx->d_trig) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: frames not set on this context");
    a.trig = ctx->d_trig;
    a.work = b->d_work;
    a.images = reinterpret_cast<float4*>(d_images);
    a.status = ctx->d_status;
    GBRT_CUDA(ctx, cudaMemsetAsync(b->d_work, 0, 4, stream));
    kernel<<<uint32_t(blocks), b->launch.block, 0, stream>>>(a);
    GBRT_LAUNCH_CHECK(ctx, "batch_pt");
    return GBRT_OK;
}

} // namespace gbrt

using namespace gbrt;

extern "C" gbrt_status gbrt_batch_set_frames(gbrt_context* ctx, gbrt_batch* batch, gbrt_camera const* h_cameras,
                                             gbrt_pt_params const* h_params, gbrt_material const* h_materials,
                                             uint32_t num_materials)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!batch || !h_cameras || !h_params || (num_materials && !h_materials))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_set_frames: null argument");
    for (uint32_t k = 0; k < num_materials; ++k)
        if (h_materials[k].kind > GBRT_MATERIAL_PLASTIC)
            return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_set_frames: unknown material kind");
    // the sample-angle table, allocated here so that a captured frame allocates nothing
    gbrt_status tst = ensure_trig_table(ctx);
    if (tst != GBRT_OK) return tst;
    const uint32_t ns = batch->num_scenes;
    std::vector<batch_frame> frames(ns);
    std::vector<uint32_t> offs(ns + 1);
    uint64_t total = 0;
    for (uint32_t s = 0; s < ns; ++s)
    {
        gbrt_pt_params const& p = h_params[s];
        if (p.width == 0 || p.height == 0 || p.spp == 0)
            return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_set_frames: empty frame");
        offs[s] = uint32_t(total);
        total += uint64_t(p.width) * p.height;
        if (total > (1ull << 31)) return fail(ctx, GBRT_ERR_TOO_LARGE, "batch_set_frames: more than 2^31 pixels");
        batch_frame& f = frames[s];
        f.cam = camera_for(h_cameras[s], p.width, p.height);
        f.bg = make_float4(p.background[0] * p.background[3], p.background[1] * p.background[3],
                           p.background[2] * p.background[3], 1.0f);
        f.ambient = make_float3(p.ambient[0], p.ambient[1], p.ambient[2]);
        f.epsilon = p.epsilon;
        f.width = p.width;
        f.height = p.height;
        f.spp = p.spp;
        f.num_bounces = p.num_bounces;
        f.frame_id = p.frame_id;
        f.flags = p.flags;
        f.root = batch->roots[s];
        f.blocks = (p.width % 8 == 0 && p.height % 4 == 0) ? 1u : 0u;
    }
    offs[ns] = uint32_t(total);
    device_guard g(ctx->device);
    // the previous frame may still read these buffers
    GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (!batch->d_frames) GBRT_CUDA(ctx, cudaMalloc(&batch->d_frames, size_t(ns) * sizeof(batch_frame)));
    if (!batch->d_pixel_offsets) GBRT_CUDA(ctx, cudaMalloc(&batch->d_pixel_offsets, size_t(ns + 1) * 4));
    if (num_materials > batch->num_materials || !batch->d_materials)
    {
        cudaFree(batch->d_materials);
        batch->d_materials = nullptr;
        batch->num_materials = 0;
        GBRT_CUDA(ctx, cudaMalloc(&batch->d_materials, size_t(num_materials ? num_materials : 1) * sizeof(gbrt_material)));
    }
    GBRT_CUDA(ctx, cudaMemcpy(batch->d_frames, frames.data(), size_t(ns) * sizeof(batch_frame), cudaMemcpyHostToDevice));
    GBRT_CUDA(ctx, cudaMemcpy(batch->d_pixel_offsets, offs.data(), size_t(ns + 1) * 4, cudaMemcpyHostToDevice));
    if (num_materials)
        GBRT_CUDA(ctx, cudaMemcpy(batch->d_materials, h_materials, size_t(num_materials) * sizeof(gbrt_material),
                                  cudaMemcpyHostToDevice));
    batch->num_materials = num_materials;
    batch->extended_materials = false;
    for (uint32_t k = 0; k < num_materials; ++k)
    {
        const uint32_t kind = h_materials[k].kind;
        batch->extended_materials |=
            kind == GBRT_MATERIAL_MIRROR || kind == GBRT_MATERIAL_GLASS || kind == GBRT_MATERIAL_PLASTIC;
    }
    batch->total_pixels = uint32_t(total);
    batch->frames_set = ns;
    batch->graph_dirty = true;
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_batch_set_lights(gbrt_context* ctx, gbrt_batch* batch, gbrt_light const* h_lights,
                                             uint32_t num_lights, uint32_t const* h_light_offsets)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!batch || (num_lights && (!h_lights || !h_light_offsets)))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_set_lights: null argument");
    const uint32_t ns = batch->num_scenes;
    if (num_lights)
    {
        if (h_light_offsets[0] != 0 || h_light_offsets[ns] != num_lights)
            return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_set_lights: offsets must run from 0 to num_lights");
        for (uint32_t s = 0; s < ns; ++s)
            if (h_light_offsets[s + 1] < h_light_offsets[s])
                return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_set_lights: offsets decrease");
    }
    std::vector<float4> rec;
    gbrt_status st = light_records(ctx, h_lights, num_lights, rec, "batch_set_lights");
    if (st != GBRT_OK) return st;
    device_guard g(ctx->device);
    // the previous frame may still read these buffers
    GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(batch->d_lights);
    cudaFree(batch->d_light_offsets);
    batch->d_lights = nullptr;
    batch->d_light_offsets = nullptr;
    batch->num_lights = 0;
    batch->graph_dirty = true;
    if (num_lights == 0) return GBRT_OK;
    GBRT_CUDA(ctx, cudaMalloc(&batch->d_lights, rec.size() * sizeof(float4)));
    GBRT_CUDA(ctx, cudaMalloc(&batch->d_light_offsets, size_t(ns + 1) * 4));
    GBRT_CUDA(ctx, cudaMemcpy(batch->d_lights, rec.data(), rec.size() * sizeof(float4), cudaMemcpyHostToDevice));
    GBRT_CUDA(ctx, cudaMemcpy(batch->d_light_offsets, h_light_offsets, size_t(ns + 1) * 4, cudaMemcpyHostToDevice));
    batch->num_lights = num_lights;
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_batch_set_launch(gbrt_batch* batch, gbrt_batch_launch const* launch)
{
    if (!batch || !launch || !launch_valid(*launch)) return GBRT_ERR_INVALID_ARG;
    batch->launch = *launch;
    batch->graph_dirty = true;
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_batch_get_launch(gbrt_batch const* batch, gbrt_batch_launch* out)
{
    if (!batch || !out) return GBRT_ERR_INVALID_ARG;
    *out = batch->launch;
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_batch_height(gbrt_context* ctx, gbrt_batch const* batch, uint32_t* out)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!batch || !out) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_height: null argument");
    device_guard g(ctx->device);
    GBRT_CUDA(ctx, cudaMemcpyAsync(out, batch->d_height, 4, cudaMemcpyDeviceToHost, ctx->stream));
    GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_batch_pathtrace(gbrt_context* ctx, gbrt_batch const* batch, float* d_images)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!batch) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: null batch");
    device_guard g(ctx->device);
    return batch_pathtrace(ctx, batch, d_images, ctx->stream);
}

extern "C" gbrt_status gbrt_batch_run_graph(gbrt_context* ctx, gbrt_batch* batch, gbrt_triangle const* d_tris,
                                            float* d_images)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!batch || (batch->total && !d_tris)) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_run_graph: null argument");
    if (batch->frames_set != batch->num_scenes) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_run_graph: frames not set");
    device_guard g(ctx->device);
    if (!batch->graph || batch->graph_dirty || batch->graph_tris != d_tris || batch->graph_images != d_images)
    {
        if (batch->graph)
        {
            GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            cudaGraphExecDestroy(batch->graph);
            batch->graph = nullptr;
        }
        if (!batch->capture_stream)
            GBRT_CUDA(ctx, cudaStreamCreateWithFlags(&batch->capture_stream, cudaStreamNonBlocking));
        const uint64_t before = ctx->launches;
        GBRT_CUDA(ctx, cudaStreamBeginCapture(batch->capture_stream, cudaStreamCaptureModeThreadLocal));
        gbrt_status st = batch_build(ctx, batch, d_tris, batch->capture_stream);
        if (st == GBRT_OK) st = batch_pathtrace(ctx, batch, d_images, batch->capture_stream);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(batch->capture_stream, &graph);
        const uint64_t captured = ctx->launches - before;
        ctx->launches = before;   // nothing ran yet
        if (st != GBRT_OK)
        {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (e != cudaSuccess) return check_cuda(ctx, e, "batch_run_graph: capture");
        cudaGraphExec_t exec = nullptr;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return check_cuda(ctx, e, "batch_run_graph: instantiate");
        batch->graph = exec;
        batch->graph_launches = captured;
        batch->graph_tris = d_tris;
        batch->graph_images = d_images;
        batch->graph_dirty = false;
    }
    GBRT_CUDA(ctx, cudaGraphLaunch(batch->graph, ctx->stream));
    ctx->launches += batch->graph_launches;
    return GBRT_OK;
}

extern "C" gbrt_status gbrt_batch_autotune(gbrt_context* ctx, gbrt_batch* batch, float* d_images, uint32_t reps,
                                           gbrt_batch_launch* best, float* best_ms)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!batch || reps == 0) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_autotune: bad argument");
    if (batch->frames_set != batch->num_scenes) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_autotune: frames not set");
    device_guard g(ctx->device);
    uint32_t status = 0, height = 0;
    GBRT_CUDA(ctx, cudaMemcpyAsync(&status, ctx->d_status, 4, cudaMemcpyDeviceToHost, ctx->stream));
    GBRT_CUDA(ctx, cudaMemcpyAsync(&height, batch->d_height, 4, cudaMemcpyDeviceToHost, ctx->stream));
    GBRT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (status != 0) return fail(ctx, GBRT_ERR_CUDA, "batch_autotune: an earlier call left a status; synchronize first");
    if (batch->total == 0) height = 0;
    cudaEvent_t ev[2];
    GBRT_CUDA(ctx, cudaEventCreate(&ev[0]));
    if (cudaEventCreate(&ev[1]) != cudaSuccess)
    {
        cudaEventDestroy(ev[0]);
        return fail(ctx, GBRT_ERR_CUDA, "batch_autotune: event");
    }
    const gbrt_batch_launch saved = batch->launch;
    gbrt_batch_launch winner = saved;
    float winner_ms = -1.0f;
    gbrt_status result = GBRT_OK;
    const uint32_t blocks[] = { 128, 256, 512 }, tiles[] = { 32, 64 }, stacks[] = { 16, 24, 32, 64 },
                   orders[] = { GBRT_BATCH_ORDER_ROWS, GBRT_BATCH_ORDER_BLOCKS };
    for (uint32_t stk : stacks)
    {
        if (stk < height) continue;   // the tallest tree would overflow this stack
        for (uint32_t blk : blocks)
            for (uint32_t tl : tiles)
                for (uint32_t ord : orders)
                {
                    if (result != GBRT_OK) break;
                    batch->launch = { blk, tl, stk, ord };
                    gbrt_status st = batch_pathtrace(ctx, batch, d_images, ctx->stream);   // warm-up
                    for (uint32_t r = 0; st == GBRT_OK && r < reps; ++r)
                    {
                        if (r == 0 && cudaEventRecord(ev[0], ctx->stream) != cudaSuccess) st = GBRT_ERR_CUDA;
                        if (st == GBRT_OK) st = batch_pathtrace(ctx, batch, d_images, ctx->stream);
                    }
                    float ms = 0.0f;
                    if (st == GBRT_OK && (cudaEventRecord(ev[1], ctx->stream) != cudaSuccess ||
                                          cudaEventSynchronize(ev[1]) != cudaSuccess ||
                                          cudaEventElapsedTime(&ms, ev[0], ev[1]) != cudaSuccess))
                        st = GBRT_ERR_CUDA;
                    uint32_t cs = 0;
                    if (st == GBRT_OK &&
                        (cudaMemcpy(&cs, ctx->d_status, 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
                         (cs != 0 && cudaMemset(ctx->d_status, 0, 4) != cudaSuccess)))
                        st = GBRT_ERR_CUDA;
                    if (st != GBRT_OK)
                    {
                        result = st;
                        break;
                    }
                    if (cs != 0) continue;   // this shape raised a status: not a candidate
                    ms /= float(reps);
                    if (winner_ms < 0.0f || ms < winner_ms)
                    {
                        winner_ms = ms;
                        winner = batch->launch;
                    }
                }
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    batch->launch = winner_ms >= 0.0f ? winner : saved;
    batch->graph_dirty = true;
    if (result != GBRT_OK) return result == GBRT_ERR_CUDA ? fail(ctx, result, "batch_autotune: CUDA error") : result;
    if (winner_ms < 0.0f) return fail(ctx, GBRT_ERR_STACK_OVERFLOW, "batch_autotune: no launch shape ran cleanly");
    if (best) *best = winner;
    if (best_ms) *best_ms = winner_ms;
    return GBRT_OK;
}
