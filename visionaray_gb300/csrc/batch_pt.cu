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

#include "batch_pt.cuh"

#include <algorithm>
#include <new>
#include <string>
#include <vector>

namespace gbrt {
namespace {

template <int Block, bool Extended, bool Lit>
batch_kernel pick_stack(uint32_t stack)
{
    switch (stack)
    {
    case 16: return batch_pt<Block, 16, Extended, Lit, 2>;
    case 24: return batch_pt<Block, 24, Extended, Lit, 2>;
    case 32: return batch_pt<Block, 32, Extended, Lit, 2>;
    case 64: return batch_pt<Block, 64, Extended, Lit, 2>;
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
    if (l.width != 2) return pick_wide_kernel(l, extended, lit);
    if (lit) return extended ? pick_block<true, true>(l) : pick_block<false, true>(l);
    return extended ? pick_block<true, false>(l) : pick_block<false, false>(l);
}

bool launch_valid(gbrt_batch_launch const& l)
{
    gbrt_batch_launch pairs = l;
    pairs.width = 2;
    return pick_kernel(pairs, false, false) != nullptr && pick_kernel(l, false, false) != nullptr &&
           (l.tile == 32 || l.tile == 64) && (l.order == GBRT_BATCH_ORDER_ROWS || l.order == GBRT_BATCH_ORDER_BLOCKS) &&
           l.sort <= 1;
}

// The sorted pixel order's keys: pixel g's first primary ray (sample 0, as the frame
// draws it) traced to its closest hit; key = scene << (3 b) | the Morton code of the
// hit point's cell (b bits per axis) in the box of the scene's root, all ones for a
// miss; value = g.
__global__ void __launch_bounds__(256) batch_pixel_keys(batch_args a, uint32_t b, uint32_t* __restrict__ keys,
                                                        uint32_t* __restrict__ values)
{
    const uint32_t g = blockIdx.x * 256 + threadIdx.x;
    if (g >= a.total_pixels) return;
    const uint32_t s = upper_segment(a.pixel_offsets, a.num_scenes, g);
    const batch_frame f = a.frames[s];
    const uint32_t pixel = g - __ldg(&a.pixel_offsets[s]);
    const uint32_t cells = 1u << b;
    uint32_t code = (1u << (3 * b)) - 1u;
    if (f.root >= 0)
    {
        const v3 d = primary_dir(f.cam, f.width, f.height, f.frame_id, pixel, 0);
        trace_result h = traverse_bvh<false>(a.nodes, a.tris, f.root, a.total_inner, a.total_tris,
                                             { f.cam.eye.x, f.cam.eye.y, f.cam.eye.z }, { d.x, d.y, d.z }, 0.0f,
                                             FLT_MAX, a.status);
        if (h.tri >= 0)
        {
            const bvh2_node r = a.nodes[f.root];
            const float lo[3] = { fminf(r.xy0.x, r.xy1.x), fminf(r.xy0.z, r.xy1.z), fminf(r.z01.x, r.z01.z) };
            const float hi[3] = { fmaxf(r.xy0.y, r.xy1.y), fmaxf(r.xy0.w, r.xy1.w), fmaxf(r.z01.y, r.z01.w) };
            const float p[3] = { f.cam.eye.x + d.x * h.t, f.cam.eye.y + d.y * h.t, f.cam.eye.z + d.z * h.t };
            uint32_t c[3];
            for (int k = 0; k < 3; ++k)
            {
                const float ext = hi[k] - lo[k];
                const float q = ext > 0.0f ? (p[k] - lo[k]) / ext * float(cells) : 0.0f;
                c[k] = uint32_t(fminf(fmaxf(q, 0.0f), float(cells - 1)));   // NaN lands in cell 0
            }
            code = morton3(c[0], c[1], c[2]);
        }
    }
    keys[g] = (s << (3 * b)) | code;
    values[g] = g;
}

gbrt_status ensure_batch_sort(gbrt_context* ctx, gbrt_batch* b)
{
    if (b->sort_buf && b->sort_capacity >= b->total_pixels) return GBRT_OK;
    cudaFree(b->sort_buf);
    cudaFree(b->sort_scratch);
    b->sort_buf = nullptr;
    b->sort_scratch = nullptr;
    b->sort_capacity = 0;
    const uint32_t n = b->total_pixels > 0 ? b->total_pixels : 1;
    GBRT_CUDA(ctx, cudaMalloc(&b->sort_buf, 4 * size_t(n) * sizeof(uint32_t)));
    GBRT_CUDA(ctx, cudaMalloc(&b->sort_scratch, radix_sort_scratch_bytes(n)));
    b->sort_capacity = n;
    return GBRT_OK;
}

// What the current launch shape needs allocated before a frame (never during a capture).
gbrt_status ensure_batch_extras(gbrt_context* ctx, gbrt_batch* b)
{
    if (b->launch.width != 2)
    {
        gbrt_status st = ensure_batch_wide(ctx, b);
        if (st != GBRT_OK) return st;
    }
    if (b->launch.sort) return ensure_batch_sort(ctx, b);
    return GBRT_OK;
}

} // namespace

gbrt_status batch_frame_stage(gbrt_context* ctx, gbrt_batch* b, float* d_images, cudaStream_t stream,
                              bool force_collapse)
{
    if (b->frames_set != b->num_scenes) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: frames not set");
    if (!d_images || (reinterpret_cast<uintptr_t>(d_images) & 15u))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: images null or not 16-byte aligned");
    batch_kernel kernel = pick_kernel(b->launch, b->extended_materials, b->num_lights > 0);
    if (!kernel) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: bad launch shape");
    if (b->launch.width != 2 && !b->wide_nodes && b->total_inner > 0)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: wide nodes not allocated");
    if (b->launch.sort && (!b->sort_buf || b->sort_capacity < b->total_pixels))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: sort buffers not allocated");
    int per_sm = 0;
    GBRT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, int(b->launch.block), 0));
    if (per_sm < 1) per_sm = 1;
    // enough warps for every tile, at most one full wave of resident blocks
    const uint64_t warps_needed = (uint64_t(b->total_pixels) + b->launch.tile - 1) / b->launch.tile;
    const uint64_t blocks_needed = (warps_needed * 32 + b->launch.block - 1) / b->launch.block;
    uint64_t blocks = uint64_t(ctx->num_sms) * uint64_t(per_sm);
    if (blocks_needed < blocks) blocks = blocks_needed;
    if (blocks == 0) return GBRT_OK;
    if (b->launch.width != 2 &&
        (force_collapse || b->collapsed_width != b->launch.width || b->collapsed_gen != b->build_gen))
    {
        gbrt_status st = batch_collapse(ctx, b, b->launch.width, stream);
        if (st != GBRT_OK) return st;
    }
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
    a.nodesw = b->wide_nodes;
    a.num_nodesw = int32_t(b->wide_cap);
    a.perm = nullptr;
    a.materials = b->d_materials;
    a.num_materials = b->num_materials;
    a.lights = b->d_lights;
    a.light_offsets = b->d_light_offsets;
    if (!ctx->d_trig) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: frames not set on this context");
    a.trig = ctx->d_trig;
    a.work = b->d_work;
    a.images = reinterpret_cast<float4*>(d_images);
    a.status = ctx->d_status;
    if (b->launch.sort)
    {
        // scene bits + 3 cell bits per axis within 32-bit keys (7 per axis up to 2^11 scenes)
        uint32_t scene_bits = 0;
        while ((1u << scene_bits) < b->num_scenes) ++scene_bits;
        const uint32_t cell_bits = std::min<uint32_t>(7u, (32u - scene_bits) / 3u);
        const uint32_t n = b->total_pixels;
        uint32_t* keys = b->sort_buf;
        uint32_t* values = keys + b->sort_capacity;
        uint32_t* keys_alt = values + b->sort_capacity;
        uint32_t* values_alt = keys_alt + b->sort_capacity;
        batch_pixel_keys<<<(n + 255) / 256, 256, 0, stream>>>(a, cell_bits, keys, values);
        GBRT_LAUNCH_CHECK(ctx, "batch_pixel_keys");
        gbrt_status st = radix_sort_pairs(ctx, keys, values, keys_alt, values_alt, n, int(scene_bits + 3 * cell_bits),
                                          b->sort_scratch, stream);
        if (st != GBRT_OK) return st;
        a.perm = values;   // radix_sort_pairs leaves the result in (keys, values)
    }
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

extern "C" gbrt_status gbrt_batch_pathtrace(gbrt_context* ctx, gbrt_batch* batch, float* d_images)
{
    if (!ctx) return GBRT_ERR_INVALID_ARG;
    if (!batch) return fail(ctx, GBRT_ERR_INVALID_ARG, "batch_pathtrace: null batch");
    device_guard g(ctx->device);
    gbrt_status st = ensure_batch_extras(ctx, batch);
    if (st != GBRT_OK) return st;
    return batch_frame_stage(ctx, batch, d_images, ctx->stream, false);
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
        gbrt_status est = ensure_batch_extras(ctx, batch);   // nothing allocates inside the capture
        if (est != GBRT_OK) return est;
        const uint64_t before = ctx->launches;
        GBRT_CUDA(ctx, cudaStreamBeginCapture(batch->capture_stream, cudaStreamCaptureModeThreadLocal));
        gbrt_status st = batch_build(ctx, batch, d_tris, batch->capture_stream);
        if (st == GBRT_OK) st = batch_frame_stage(ctx, batch, d_images, batch->capture_stream, true);
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
    // one candidate: a warm-up run, then `reps` timed runs of the frame stage (with the
    // collapse and the pixel order it needs, as every graph replay does them)
    auto try_launch = [&](gbrt_batch_launch const& l) {
        if (result != GBRT_OK) return;
        batch->launch = l;
        gbrt_status st = ensure_batch_extras(ctx, batch);
        if (st == GBRT_OK) st = batch_frame_stage(ctx, batch, d_images, ctx->stream, true);   // warm-up
        for (uint32_t r = 0; st == GBRT_OK && r < reps; ++r)
        {
            if (r == 0 && cudaEventRecord(ev[0], ctx->stream) != cudaSuccess) st = GBRT_ERR_CUDA;
            if (st == GBRT_OK) st = batch_frame_stage(ctx, batch, d_images, ctx->stream, true);
        }
        float ms = 0.0f;
        if (st == GBRT_OK && (cudaEventRecord(ev[1], ctx->stream) != cudaSuccess ||
                              cudaEventSynchronize(ev[1]) != cudaSuccess ||
                              cudaEventElapsedTime(&ms, ev[0], ev[1]) != cudaSuccess))
            st = GBRT_ERR_CUDA;
        uint32_t cs = 0;
        if (st == GBRT_OK && (cudaMemcpy(&cs, ctx->d_status, 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
                              (cs != 0 && cudaMemset(ctx->d_status, 0, 4) != cudaSuccess)))
            st = GBRT_ERR_CUDA;
        if (st != GBRT_OK)
        {
            result = st;
            return;
        }
        if (cs != 0) return;   // this shape raised a status: not a candidate
        ms /= float(reps);
        if (winner_ms < 0.0f || ms < winner_ms)
        {
            winner_ms = ms;
            winner = l;
        }
    };
    // phase 1: the launch shape on the node pairs, rays unsorted
    const uint32_t blocks[] = { 128, 256, 512 }, tiles[] = { 32, 64 }, stacks[] = { 16, 24, 32, 64 },
                   orders[] = { GBRT_BATCH_ORDER_ROWS, GBRT_BATCH_ORDER_BLOCKS };
    for (uint32_t stk : stacks)
    {
        if (stk < height) continue;   // the tallest tree would overflow this stack
        for (uint32_t blk : blocks)
            for (uint32_t tl : tiles)
                for (uint32_t ord : orders)
                    try_launch({ blk, tl, stk, ord, 2, 0 });
    }
    // phase 2: BVH width and ray sorting at the winner's block, tile and order
    if (winner_ms >= 0.0f)
    {
        const gbrt_batch_launch base = winner;
        for (uint32_t width : { 2u, 4u, 8u })
            for (uint32_t sort : { 0u, 1u })
            {
                if (width == 2 && sort == 0) continue;   // timed in phase 1
                gbrt_batch_launch l = base;
                l.width = width;
                l.sort = sort;
                try_launch(l);
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
