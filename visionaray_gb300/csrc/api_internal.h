// Internal state behind the opaque handles of gbrt.h.
#pragma once

#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/visionaray_gb300/gbrt.h"
#include "bvh_layout.cuh"

// Device status bits, OR-ed by kernels into gbrt_context::d_status and reported by
// gbrt_context_synchronize.
enum : uint32_t
{
    kStatusStackOverflow = 1u << 0,
    kStatusBadIndex      = 1u << 2,   // a node/triangle index outside its array was skipped
};

struct gbrt_context
{
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    uint64_t launches = 0;

    uint32_t* d_status = nullptr;     // one word of status bits

    // Reusable scratch for builds (grown on demand, freed with the context).
    void* scratch = nullptr;
    size_t scratch_bytes = 0;

    // Host-buffer trace path: two staging slots, each on its own stream.
    static constexpr int kSlots = 2;
    cudaStream_t slot_stream[kSlots] = { nullptr, nullptr };
    cudaEvent_t slot_done[kSlots] = { nullptr, nullptr };
    void* slot_rays[kSlots] = { nullptr, nullptr };
    void* slot_hits[kSlots] = { nullptr, nullptr };
    size_t slot_capacity = 0;   // rays per slot

    // Path-tracer wavefront state (grown on demand, freed with the context).
    void* pt_scratch = nullptr;
    size_t pt_scratch_bytes = 0;
    // The path tracer's sample angles: cos and sin (rounded once from double) of
    // 2 pi u for each of the 2^24 values u = k / 2^24 a random draw takes (float2 per
    // k, 128 MB), filled once by ensure_trig_table (pathtrace.cu).
    float2* d_trig = nullptr;

    // Ray queries: GBRT_TRACE_* flags and the ray-order scratch of the context stream
    // and of each host-path slot.
    uint32_t trace_flags = 0;
    uint32_t trace_refill = 8;   // persistent traversal: idle lanes that trigger a refill
    uint32_t host_chunk = 1u << 23;   // host-buffer queries: rays per chunk (256 MB of rays)
    void* trace_scratch = nullptr;
    size_t trace_scratch_bytes = 0;
    void* slot_trace_scratch[kSlots] = { nullptr, nullptr };
    size_t slot_trace_scratch_bytes = 0;

    // Kernel timing (gbrt_context_set_kernel_timing): a CUDA event pair around the
    // traversal kernel of each ray query, in a ring of kTimingRing pairs
    // (timing_events[2k] start, [2k + 1] stop); timing_count queries recorded so far.
    static constexpr uint32_t kTimingRing = 256;
    bool kernel_timing = false;
    cudaEvent_t timing_events[2 * kTimingRing] = {};
    uint32_t timing_count = 0;
};

namespace gbrt {
// Records the start event of the next ring slot on `stream` when kernel timing is on,
// and its stop event when it goes out of scope: wraps one traversal kernel launch.
struct kernel_timer
{
    cudaStream_t stream;
    cudaEvent_t stop = nullptr;
    kernel_timer(gbrt_context* ctx, cudaStream_t s) : stream(s)
    {
        if (!ctx->kernel_timing) return;
        const uint32_t k = ctx->timing_count % gbrt_context::kTimingRing;
        cudaEventRecord(ctx->timing_events[2 * k], s);
        stop = ctx->timing_events[2 * k + 1];
        ++ctx->timing_count;
    }
    ~kernel_timer()
    {
        if (stop) cudaEventRecord(stop, stream);
    }
};
} // namespace gbrt

enum class bvh_kind
{
    lbvh,
    uploaded,
    ploc,   // ploc.cu: same node pairs and Morton-ordered leaves as the LBVH
};

struct gbrt_bvh
{
    bvh_kind kind = bvh_kind::lbvh;
    int device = 0;
    uint32_t num_prims = 0;
    uint32_t num_inner = 0;      // inner nodes (records in `nodes`)
    int32_t root = 0;            // >= 0 inner node, < 0 leaf (~first triangle)
    uint32_t height = 0;         // levels of inner nodes on the longest root-leaf path
    gbrt::bvh2_node* nodes = nullptr;
    gbrt::tri48* tris = nullptr; // leaf order
    // LBVH only: sorted Morton codes and, per sorted position, the input index.
    uint32_t* sorted_codes = nullptr;
    uint32_t* sorted_ids = nullptr;
    // Scene bounds (the root box; invalid for an empty tree), used to order rays by
    // origin and to bound instances.
    float lo[3] = { FLT_MAX, FLT_MAX, FLT_MAX };
    float hi[3] = { -FLT_MAX, -FLT_MAX, -FLT_MAX };
    // 4-wide tree collapsed from the node pairs (LBVH only; null: traverse the pairs).
    gbrt::bvh4_node* nodes4 = nullptr;
    uint32_t num_nodes4 = 0;
    uint32_t leaf_max4 = 0;
    gbrt::bvh4q_node* nodes4q = nullptr;   // the same nodes quantised (GBRT_TRACE_COMPRESSED_NODES)
    gbrt::bvh8_node* nodes8 = nullptr;     // 8-wide collapse (GBRT_TRACE_WIDE8_NODES)
    uint32_t num_nodes8 = 0;
};

namespace gbrt {
// Frees a tree's wide collapse (4-wide, quantised and 8-wide nodes).
inline void free_wide_nodes(gbrt_bvh* b)
{
    cudaFree(b->nodes4);
    b->nodes4 = nullptr;
    b->num_nodes4 = 0;
    cudaFree(b->nodes4q);
    b->nodes4q = nullptr;
    cudaFree(b->nodes8);
    b->nodes8 = nullptr;
    b->num_nodes8 = 0;
}
} // namespace gbrt


// Many scenes built and traced as one arena (batch.cu, batch_pt.cu).  Scene s owns
// the sorted primitives [offsets[s], offsets[s + 1]) and the inner node pairs
// [inner_offsets[s], inner_offsets[s + 1]); its root is roots[s] (an inner index, ~leaf
// for a one-triangle scene, INT32_MIN for an empty one).
namespace gbrt {
struct bvh_view;
}

struct gbrt_tlas
{
    int device = 0;
    uint32_t num_instances = 0;
    uint32_t num_inner = 0;
    int32_t root = INT32_MIN;
    gbrt::bvh2_node* nodes = nullptr;   // top-level node pairs, leaves ~instance
    float4* records = nullptr;          // 3 float4 per instance: rows of A^-1 | trans_inv
    float4* forward = nullptr;          // 3 float4 per instance: rows of A | translation
    gbrt::bvh_view* views = nullptr;    // the instance's bottom-level tree
    std::vector<gbrt_bvh const*> blas;  // the same trees, host side
};

struct gbrt_batch
{
    int device = 0;
    uint32_t num_scenes = 0;
    uint32_t total = 0;         // primitives of all scenes
    uint32_t total_inner = 0;   // inner node pairs of all scenes
    std::vector<uint32_t> offsets, inner_offsets;
    std::vector<int32_t> roots;
    uint32_t* d_offsets = nullptr;
    uint32_t* d_inner_offsets = nullptr;
    int32_t* d_roots = nullptr;
    gbrt::bvh2_node* nodes = nullptr;
    gbrt::tri48* tris = nullptr;
    uint32_t* sorted_codes = nullptr;
    uint32_t* sorted_ids = nullptr;
    uint32_t* d_height = nullptr;   // the tallest scene tree (atomicMax)
    void* scratch = nullptr;        // build temporaries, sized at creation
    size_t scratch_bytes = 0;
    // frame setup (gbrt_batch_set_frames)
    void* d_frames = nullptr;       // per-scene camera basis, frame size, root (batch_pt.cu)
    uint32_t* d_pixel_offsets = nullptr;
    uint32_t total_pixels = 0;
    uint32_t frames_set = 0;        // scenes whose frames are on the device (0 or num_scenes)
    gbrt_material* d_materials = nullptr;
    uint32_t num_materials = 0;
    bool extended_materials = false;   // some material is a mirror, glass or plastic
    uint32_t* d_work = nullptr;     // persistent-kernel work counter
    // per arena inner node: its leaf range (first, last) in triangle-array indices, for
    // the wide collapse (written by every build)
    int2* ranges = nullptr;
    // W-wide collapse of the arena (launch.width 4 or 8; allocated on first use): room
    // for wide_cap 8-wide nodes (scene s's root at node s), two level queues, the
    // per-level counts and the node counter; the build generation it was made from
    void* wide_nodes = nullptr;
    int2* wide_queue[2] = { nullptr, nullptr };
    uint32_t* wide_counts = nullptr;
    uint32_t wide_cap = 0;
    uint32_t collapsed_width = 0;
    uint64_t build_gen = 0, collapsed_gen = 0;
    // sorted pixel order (launch.sort; allocated on first use): keys, values and their
    // alternates (4 x sort_capacity words) and the radix sort's scratch
    uint32_t* sort_buf = nullptr;
    void* sort_scratch = nullptr;
    uint32_t sort_capacity = 0;
    // lights (gbrt_batch_set_lights): 4 float4 per light, scene s's lights at
    // [light_offsets[s], light_offsets[s + 1])
    float4* d_lights = nullptr;
    uint32_t* d_light_offsets = nullptr;
    uint32_t num_lights = 0;
    gbrt_batch_launch launch = { 128, 32, 64, GBRT_BATCH_ORDER_ROWS, 2, 0 };
    // the captured build + frame
    cudaStream_t capture_stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_launches = 0;    // kernels per replay
    bool graph_dirty = true;
    const void* graph_tris = nullptr;
    void* graph_images = nullptr;
};

namespace gbrt {

// Makes `dev` current for the guard's lifetime.
struct device_guard
{
    int prev = -1;
    explicit device_guard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~device_guard()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

// Sets ctx->last_error and returns `st`.
gbrt_status fail(gbrt_context* ctx, gbrt_status st, std::string const& what);
// Maps a CUDA error to a status, recording `where`.
gbrt_status check_cuda(gbrt_context* ctx, cudaError_t err, const char* where);
// Grows the context scratch to at least `bytes`.
gbrt_status ensure_scratch(gbrt_context* ctx, size_t bytes);

// pathtrace.cu: the device records (4 float4 each) of area, point and spot lights, as
// path-tracing scenes hold them; fails on an unknown light kind.
gbrt_status light_records(gbrt_context* ctx, gbrt_light const* h_lights, uint32_t num_lights,
                          std::vector<float4>& out, const char* who);

// lbvh.cu
gbrt_status build_lbvh(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n, gbrt_bvh* bvh);
gbrt_status refit_lbvh(gbrt_context* ctx, gbrt_bvh* bvh, gbrt_triangle const* d_tris);
gbrt_status morton_order(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n, uint32_t* codes_out,
                         uint32_t* ids_out);
// ploc.cu
gbrt_status build_ploc(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n, gbrt_bvh* bvh);
gbrt_status export_generic(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_bvh_node* d_nodes, uint32_t* d_indices);
gbrt_status export_bvh2(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_bvh_node* d_nodes,
                        uint32_t* d_indices);
gbrt_status morton_codes_input_order(gbrt_context* ctx, gbrt_bvh const* bvh, uint32_t* d_codes);
gbrt_status upload_bvh2(gbrt_context* ctx, gbrt_bvh_node const* nodes, uint32_t num_nodes,
                        uint32_t const* indices, uint32_t num_indices, gbrt_triangle const* tris,
                        uint32_t num_tris, gbrt_bvh* bvh);

// Partition of one caller-supplied region holding every buffer of an LBVH build of
// up to n primitives (offsets in bytes, each 256-byte aligned).  The sort's share
// mirrors radix_sort_scratch_bytes (4096-key tiles, 256 digits, 4096-entry scan
// chunks); build_lbvh_in_scratch re-checks it at run time.
struct lbvh_scratch_layout
{
    size_t centroids, keys, vals, keys_alt, vals_alt, leaf_parent, arrivals, nodes, tris, words, sort, total;
};

constexpr size_t scratch_align(size_t v) { return (v + 255) & ~size_t(255); }

constexpr lbvh_scratch_layout lbvh_scratch_layout_for(uint32_t n)
{
    lbvh_scratch_layout l{};
    size_t o = 0;
    l.centroids = o;   o = scratch_align(o + size_t(n) * 16);
    l.keys = o;        o = scratch_align(o + size_t(n) * 4);
    l.vals = o;        o = scratch_align(o + size_t(n) * 4);
    l.keys_alt = o;    o = scratch_align(o + size_t(n) * 4);
    l.vals_alt = o;    o = scratch_align(o + size_t(n) * 4);
    l.leaf_parent = o; o = scratch_align(o + size_t(n) * 4);
    l.arrivals = o;    o = scratch_align(o + size_t(n) * 4);
    l.nodes = o;       o = scratch_align(o + size_t(n) * 64);
    l.tris = o;        o = scratch_align(o + size_t(n) * 48);
    l.words = o;       o = scratch_align(o + 8 * 4);
    l.sort = o;
    size_t tiles = (size_t(n) + 4095) / 4096;
    size_t len = 256 * tiles;
    size_t chunks = (len + 4095) / 4096;
    o = scratch_align(o + (len + chunks + 64) * 4);
    l.total = o;
    return l;
}

// LBVH build whose every temporary and the node-pair tree live in `scratch`
// (laid out by lbvh_scratch_layout_for(n)); writes the reference's cuda_index_bvh
// layout (2n-1 nodes, n indices) to d_nodes / d_indices.  Allocates nothing, does
// not synchronise; stream-ordered on ctx->stream.
gbrt_status build_lbvh_in_scratch(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n, void* scratch,
                                  size_t scratch_bytes, gbrt_bvh_node* d_nodes, uint32_t* d_indices);

// radix_sort.cu: stable LSD sort of (key, value) pairs by the low `key_bits` bits.
// Result lands in (keys, values); keys_alt/values_alt are same-sized scratch.  With
// sorted_values non-null nothing is copied back: *sorted_values is values or
// values_alt, whichever the last pass wrote.
size_t radix_sort_scratch_bytes(uint32_t n);
gbrt_status radix_sort_pairs(gbrt_context* ctx, uint32_t* keys, uint32_t* values,
                             uint32_t* keys_alt, uint32_t* values_alt, uint32_t n, int key_bits,
                             void* scratch, cudaStream_t stream, uint32_t** sorted_values = nullptr);
inline gbrt_status radix_sort_pairs(gbrt_context* ctx, uint32_t* keys, uint32_t* values,
                                    uint32_t* keys_alt, uint32_t* values_alt, uint32_t n, int key_bits,
                                    void* scratch)
{
    return radix_sort_pairs(ctx, keys, values, keys_alt, values_alt, n, key_bits, scratch, ctx->stream);
}

// traverse.cu: `scratch` (trace_scratch_bytes(n) bytes, may be null when rays are not
// reordered) holds the ray order.
size_t trace_scratch_bytes(uint32_t n);
gbrt_status trace(gbrt_context* ctx, gbrt_bvh const* bvh, gbrt_ray const* d_rays, uint32_t n,
                  gbrt_hit* d_hits, bool any_hit, cudaStream_t stream, void* scratch = nullptr,
                  size_t scratch_bytes = 0);

// batch.cu: the batched build, enqueued on `stream` (allocates nothing, does not
// synchronise, so it can be captured).
gbrt_status batch_build(gbrt_context* ctx, gbrt_batch* b, gbrt_triangle const* d_tris, cudaStream_t stream);
// Levels of the arena's wide collapse (every tree is at most kStackSize - 1 deep).
constexpr uint32_t kBatchCollapseLevels = kStackSize;
// Allocates the wide collapse's nodes and queues (once; not during a capture).
gbrt_status ensure_batch_wide(gbrt_context* ctx, gbrt_batch* b);
// Collapses every scene's tree of the last build into width-wide nodes on `stream`
// (allocates nothing, does not synchronise).
gbrt_status batch_collapse(gbrt_context* ctx, gbrt_batch* b, uint32_t width, cudaStream_t s);
// batch_pt.cu: the batched frame on `stream`, with what the launch shape needs before
// it (the wide collapse, the pixel order); force_collapse re-collapses even when the
// last build's collapse at this width is current.
gbrt_status batch_frame_stage(gbrt_context* ctx, gbrt_batch* b, float* d_images, cudaStream_t stream,
                              bool force_collapse);

} // namespace gbrt

// Launch bookkeeping: counts the kernel and checks the launch.
#define GBRT_LAUNCH_CHECK(ctx, name)                                                       \
    do                                                                                     \
    {                                                                                      \
        (ctx)->launches++;                                                                 \
        cudaError_t e_ = cudaGetLastError();                                               \
        if (e_ != cudaSuccess) return gbrt::check_cuda((ctx), e_, name);                   \
    } while (0)

#define GBRT_CUDA(ctx, call)                                                               \
    do                                                                                     \
    {                                                                                      \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) return gbrt::check_cuda((ctx), e_, #call);                  \
    } while (0)

namespace gbrt {
// Allocates and fills gbrt_context::d_trig if it is not there yet (pathtrace.cu).
gbrt_status ensure_trig_table(gbrt_context* ctx);
} // namespace gbrt
