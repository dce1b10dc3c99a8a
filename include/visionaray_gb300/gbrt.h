/*
 * gbrt.h -- C ABI of the GB300-native ray-tracing hot path (visionaray_gb300).
 *
 * This is the drop-in boundary for visionaray's GPU ray-tracing path.  Every entry
 * point below names the visionaray interface it replaces (file:line inside the
 * visionaray source tree).  All types are plain C; no CUDA or C++ type crosses the
 * boundary except an opaque `void*` CUDA stream.
 *
 * Conventions
 *   - Device pointers unless the name ends in `_host`.  Caller owns input and output
 *     buffers; the library owns BVH arenas behind opaque handles.
 *   - Every call returns a gbrt_status.  Nothing aborts, throws or prints.
 *     gbrt_last_error() gives a one-line description of the last failure on a context.
 *   - Calls are asynchronous on the context's stream unless documented otherwise,
 *     like visionaray's cuda_sched::frame (detail/cuda_sched.inl:226-246).
 *   - A context is used by one host thread at a time (no internal locking).
 */
#ifndef VISIONARAY_GB300_GBRT_H
#define VISIONARAY_GB300_GBRT_H 1

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBRT_ABI_VERSION 3

typedef enum gbrt_status
{
    GBRT_OK                 = 0,
    GBRT_ERR_INVALID_ARG    = 1,  /* null pointer, bad size, bad enum                  */
    GBRT_ERR_OUT_OF_MEMORY  = 2,  /* device allocation failed                           */
    GBRT_ERR_CUDA           = 3,  /* a CUDA runtime call or kernel launch failed        */
    GBRT_ERR_WATCHDOG       = 4,  /* reserved, never returned: no kernel of this library
                                   * waits on a flag, a peer or a barrier             */
    GBRT_ERR_STACK_OVERFLOW = 5,  /* traversal stack exceeded (tree deeper than limit)  */
    GBRT_ERR_TOO_LARGE      = 6   /* input larger than a documented maximum             */
} gbrt_status;

/* visionaray basic_triangle<3, float, unsigned> (math/triangle.h:18-36 with the
 * primitive<unsigned> base of math/primitive.h:15-21): 44 bytes, no padding.      */
typedef struct gbrt_triangle
{
    uint32_t geom_id;
    uint32_t prim_id;
    float    v1[3];
    float    e1[3];
    float    e2[3];
} gbrt_triangle;

/* visionaray basic_ray<float> (math/ray.h:16-45): 32 bytes.                        */
typedef struct gbrt_ray
{
    float ori[3];
    float dir[3];
    float tmin;
    float tmax;
} gbrt_ray;

/* The traced result of one ray: the fields of visionaray's
 * hit_record<ray, primitive<unsigned>> (math/intersect.h:151-169) that the hot path
 * consumes.  prim_id is the hit triangle's own prim_id field, or GBRT_NO_HIT.
 * A miss stores t = FLT_MAX and u = v = 0, as the reference record does.           */
typedef struct gbrt_hit
{
    uint32_t prim_id;
    float    t;
    float    u;
    float    v;
} gbrt_hit;

#define GBRT_NO_HIT 0xFFFFFFFFu

/* visionaray bvh_node (bvh.h:70-141): 32 bytes.  Inner: num_prims == 0 and
 * first_child indexes the first of two adjacent children.  Leaf: first_prim indexes
 * the bvh's index list, num_prims > 0.                                            */
typedef struct gbrt_bvh_node
{
    float    bbox_min[3];
    float    bbox_max[3];
    uint32_t first_child_or_prim;
    uint16_t num_prims;
    uint8_t  ordered_traversal_axis;
    uint8_t  ordered_traversal_sign;
} gbrt_bvh_node;

typedef struct gbrt_context gbrt_context;
typedef struct gbrt_bvh     gbrt_bvh;
typedef struct gbrt_tlas    gbrt_tlas;

/* ------------------------------------------------------------------------------ */
/* Context                                                                         */

/* Binds a context to CUDA device `device` and stream `stream` (a cudaStream_t, or
 * NULL for the legacy default stream).  No visionaray counterpart: visionaray's
 * builders and schedulers take the stream per call (detail/cuda_sched.h:39,
 * detail/bvh/lbvh.h:669-679); the context carries it once instead.               */
gbrt_status gbrt_context_create(int device, void* stream, gbrt_context** out);
gbrt_status gbrt_context_destroy(gbrt_context* ctx);
gbrt_status gbrt_context_set_stream(gbrt_context* ctx, void* stream);
/* Blocks until all work queued on the context's stream is done and reports any
 * deferred device-side error (a traversal stack overflow, an out-of-range index).  */
gbrt_status gbrt_context_synchronize(gbrt_context* ctx);
const char* gbrt_last_error(gbrt_context const* ctx);
int         gbrt_abi_version(void);

/* Ray-query options of a context (GBRT_TRACE_* bits, default 0).  No visionaray
 * counterpart: visionaray traces each ray in the calling thread, in the caller's
 * order.  GBRT_TRACE_SORT_RAYS orders a call's rays (from 65,536 rays up) by the Morton
 * cell of their origin before tracing, so that a warp's rays share their upper tree
 * path; hits are still returned per input ray and are identical bit for bit.        */
#define GBRT_TRACE_SORT_RAYS 1u
/* With this flag set when gbrt_bvh_build_lbvh runs, the tree is also collapsed into
 * 4-wide nodes (leaves of up to 4 triangles), and queries on a context with the flag
 * traverse those instead of the binary node pairs.  Off by default: on the 8.4M-
 * triangle heightfield the 128-byte 4-wide nodes trace slower than the 64-byte pairs. */
#define GBRT_TRACE_WIDE_NODES 2u
/* Persistent traversal: a grid that just fills the GPU, whose warps refill idle lanes
 * with new rays from an atomic counter instead of idling until their slowest ray ends
 * (node pairs only; hits identical bit for bit).                                     */
#define GBRT_TRACE_PERSISTENT 4u
/* With this flag set when gbrt_bvh_build_lbvh runs, the 4-wide nodes are also stored
 * quantised to 64 bytes in the layout of visionaray's bvh_compressed_node<4> (bvh.h:
 * 319-426; 8-bit offsets in power-of-two units, rounded outward), and ray queries on a
 * context with the flag traverse those.  Implies the 4-wide collapse.  Path tracing
 * keeps the node pairs (or the 4-wide nodes).                                         */
#define GBRT_TRACE_COMPRESSED_NODES 8u
/* With this flag set when gbrt_bvh_build_lbvh runs, the tree is also collapsed into
 * 8-wide nodes (256 bytes, eight children's boxes per fetch; bvh_collapser's BVH8,
 * detail/bvh/collapse.h:19-169), and ray queries on a context with the flag traverse
 * those (it takes precedence over the 4-wide flags).                                */
#define GBRT_TRACE_WIDE8_NODES 16u
gbrt_status gbrt_context_set_trace_flags(gbrt_context* ctx, uint32_t flags);

/* Persistent traversal: a warp refills once at least min_idle_lanes (1..32, default 8)
 * of its lanes are idle.                                                           */
gbrt_status gbrt_context_set_trace_refill(gbrt_context* ctx, uint32_t min_idle_lanes);

/* Host-buffer queries (gbrt_trace_*_host) move rays and hits in chunks of this many
 * rays (2^16 .. 2^26, default 2^23), alternating between two device slots so one
 * chunk's copies overlap another's traversal.                                      */
gbrt_status gbrt_context_set_host_chunk(gbrt_context* ctx, uint32_t rays);

/* ------------------------------------------------------------------------------ */
/* BVH construction                                                                */

/* GPU LBVH build (Karras 2012) over `n` triangles in device memory.
 * Replaces lbvh_builder::build(cuda_index_bvh<P>{}, P* prims, size_t n)
 * (detail/bvh/lbvh.h:681-844): 30-bit Morton codes of centroids quantised exactly as
 * lbvh.h:253-267, a stable sort by code, Karras hierarchy (lbvh.h:120-185, 281-330)
 * and a bottom-up refit.  One primitive per leaf, as the reference.  The tree keeps
 * its own copy of the triangles, so `d_tris` may be freed after the call.
 * n == 0 yields an empty tree whose traces report misses.                         */
gbrt_status gbrt_bvh_build_lbvh(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n,
                                gbrt_bvh** out);

/* Same, with the triangles in host memory (copied in on the context's stream).    */
gbrt_status gbrt_bvh_build_lbvh_host(gbrt_context* ctx, gbrt_triangle const* h_tris, uint32_t n,
                                     gbrt_bvh** out);

/* Uploads a BVH2 built elsewhere (e.g. visionaray's binned_sah_builder,
 * detail/bvh/sah.h:176-807) from host memory: `nodes` in visionaray bvh_node layout,
 * `indices` the index list (primitive(i) = tris[indices[i]], bvh.h:550-553).
 * Replaces the host->device copy constructor of cuda_index_bvh (bvh.h:963-1009).
 * Synchronous.                                                                     */
gbrt_status gbrt_bvh_upload_bvh2_host(gbrt_context* ctx,
                                      gbrt_bvh_node const* nodes, uint32_t num_nodes,
                                      uint32_t const* indices, uint32_t num_indices,
                                      gbrt_triangle const* tris, uint32_t num_tris,
                                      gbrt_bvh** out);

gbrt_status gbrt_bvh_destroy(gbrt_bvh* bvh);

/* Sizes of the reference-layout export below: 2n-1 nodes and n indices for an
 * LBVH of n > 0 triangles.                                                         */
gbrt_status gbrt_bvh_counts(gbrt_bvh const* bvh, uint32_t* num_prims, uint32_t* num_bvh2_nodes,
                            uint32_t* depth_bound);

/* High-quality build (no visionaray counterpart; the reference's GPU builder is the
 * LBVH): parallel locally-ordered clustering (Meister & Bittner 2018) from the Morton
 * order -- mutual nearest neighbours within 16 positions by union surface area merge,
 * level by level -- giving trees close to the binned SAH builder's (sah.h:176-807) at
 * GPU build speed.  Same handle, traversal and refit as an LBVH; export_bvh2 writes
 * the generic index_bvh layout (breadth first, children adjacent).  Synchronous.    */
gbrt_status gbrt_bvh_build_ploc(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n, gbrt_bvh** out);

/* Writes the tree in visionaray's cuda_index_bvh node layout, exactly as the
 * reference's lbvh::collapse kernel emits it (detail/bvh/lbvh.h:374-451): root at 0,
 * the children of Karras inner node i at 1+2i and 2+2i, leaves with one primitive
 * and first_prim = the primitive's original index; indices = 0,1,2,... (lbvh.h:453).
 * d_nodes holds num_bvh2_nodes entries, d_indices num_prims entries (device).
 * Only for trees built by gbrt_bvh_build_lbvh.                                    */
gbrt_status gbrt_bvh_export_bvh2(gbrt_context* ctx, gbrt_bvh const* bvh,
                                 gbrt_bvh_node* d_nodes, uint32_t* d_indices);

/* lbvh_builder::build (detail/bvh/lbvh.h:681-844) into an existing tree: the full
 * GPU LBVH build of n triangles (device, the same count the tree was built with, any
 * positions) written into the tree's own arrays, so a scene whose geometry changes
 * every frame is rebuilt without device allocations (a 4-wide collapse, if the
 * context asks for one, is still allocated anew).  The result equals
 * gbrt_bvh_build_lbvh's for the same triangles.  Path-tracing scenes made from the
 * tree see the new tree.  Synchronises the context stream (the tree height).        */
gbrt_status gbrt_bvh_rebuild_lbvh(gbrt_context* ctx, gbrt_bvh* bvh, gbrt_triangle const* d_tris, uint32_t n);

/* bvh_refitter::refit(tree, prims, n) (detail/bvh/refit.h:25-117) on the GPU: new
 * positions of the same n triangles (device, the build's input order); the tree keeps
 * its topology and leaf order, the leaf triangles and every node box are recomputed
 * (bottom-up, one pass).  For trees built by gbrt_bvh_build_lbvh; a 4-wide collapse is
 * dropped.  Synchronises the context stream.                                        */
gbrt_status gbrt_bvh_refit(gbrt_context* ctx, gbrt_bvh* bvh, gbrt_triangle const* d_tris, uint32_t n);

/* LBVH build that allocates no device memory, for callers that cannot allocate:
 * hosts that own the whole device-memory budget and give a library only its output
 * buffers, and per-frame rebuild loops where cudaMalloc/cudaFree would synchronise
 * the device.  No counterpart in visionaray (its builder always allocates,
 * detail/bvh/lbvh.h:693-834).  Same tree as gbrt_bvh_build_lbvh + gbrt_bvh_export_bvh2:
 * d_nodes receives 2n-1 nodes, d_indices n indices (device buffers of the caller).
 * All temporaries live in one fixed device array of this library (about 10 MB, held
 * by every GPU that loads it until exit), so n is limited to 65,536 triangles
 * (GBRT_ERR_TOO_LARGE beyond).  Calls share that array: consecutive calls on a stream
 * are independent, calls that overlap on the GPU race.  The first call on a device
 * looks up the array's address; make it before any stream capture.  Asynchronous on
 * the context stream.                                                              */
gbrt_status gbrt_bvh_build_lbvh_noalloc(gbrt_context* ctx, gbrt_triangle const* d_tris, uint32_t n,
                                        gbrt_bvh_node* d_nodes, uint32_t* d_indices);

/* Writes the 30-bit Morton code of every primitive, in input order, exactly as
 * lbvh::assign_morton_codes computes it (detail/bvh/lbvh.h:242-269).  Only for trees
 * built by gbrt_bvh_build_lbvh.  d_codes holds num_prims entries.                  */
gbrt_status gbrt_bvh_morton_codes(gbrt_context* ctx, gbrt_bvh const* bvh, uint32_t* d_codes);

/* ------------------------------------------------------------------------------ */
/* Traversal                                                                       */

/* closest_hit(ray, refs, refs + 1) over one BVH for `n` rays
 * (detail/traverse_linear.inl:192-225 -> detail/bvh/intersect.inl:41-357 with the
 * ray/triangle test of math/intersect.h:176-229).  A hit is accepted iff the
 * triangle test hits with tmin <= t <= tmax and t strictly below the best t so far
 * (update_if.h:68-107).                                                            */
gbrt_status gbrt_trace_closest_hit(gbrt_context* ctx, gbrt_bvh const* bvh,
                                   gbrt_ray const* d_rays, uint32_t n, gbrt_hit* d_hits);

/* any_hit(ray, refs, refs + 1) (detail/traverse_linear.inl:156-189): stops at the
 * first accepted hit (detail/exit_traversal.h:49-56).  Which triangle is reported
 * depends on traversal order; whether a hit exists does not.  These queries visit the
 * two hit children of a node in index order rather than nearest first (fewer
 * instructions per node), so the reported triangle can differ from the reference's. */
gbrt_status gbrt_trace_any_hit(gbrt_context* ctx, gbrt_bvh const* bvh,
                               gbrt_ray const* d_rays, uint32_t n, gbrt_hit* d_hits);

/* The same two calls with rays and hits in host memory (pinned memory gives
 * full copy speed).  Rays are copied in, traced and copied out in chunks that
 * overlap copies with traversal.  Synchronous: on return, h_hits is complete.      */
gbrt_status gbrt_trace_closest_hit_host(gbrt_context* ctx, gbrt_bvh const* bvh,
                                        gbrt_ray const* h_rays, uint32_t n, gbrt_hit* h_hits);
gbrt_status gbrt_trace_any_hit_host(gbrt_context* ctx, gbrt_bvh const* bvh,
                                    gbrt_ray const* h_rays, uint32_t n, gbrt_hit* h_hits);

/* ------------------------------------------------------------------------------ */
/* Path tracing                                                                    */

/* One material per geom_id (materials[geom_id], get_surface.h:158), a member of
 * visionaray's generic_material:
 *   matte    (Lambertian, detail/material/matte.inl): cd = color, kd = scale
 *   emissive (detail/material/emissive.inl): ce = color, ls = scale
 *   mirror   (detail/material/mirror.inl, specular_reflection brdf.h:293-352):
 *            cr = color, kr = scale, conductor Fresnel with ior and absorption
 *   glass    (detail/material/glass.inl, specular_transmission brdf.h:360-469):
 *            ct = color, kt = scale, cr = color2, kr = scale2, ior
 *   plastic  (detail/material/plastic.inl, lambertian + blinn brdf.h:26-84, 118-191):
 *            cd = color, kd = scale, cs = color2, ks = scale2,
 *            specular_exp = exponent
 * (the path-tracing configurations use matte and emissive).  Scene creation and
 * gbrt_batch_set_frames reject any other kind with GBRT_ERR_INVALID_ARG.            */
#define GBRT_MATERIAL_MATTE    0u
#define GBRT_MATERIAL_EMISSIVE 1u
#define GBRT_MATERIAL_MIRROR   2u
#define GBRT_MATERIAL_GLASS    3u
#define GBRT_MATERIAL_PLASTIC  4u
typedef struct gbrt_material
{
    uint32_t kind;
    float    color[3];
    float    scale;
    float    ior[3];
    float    absorption[3];
    float    color2[3];
    float    scale2;
    float    exponent;
} gbrt_material;

/* area_light<float, basic_triangle<3, float>> (area_light.h, detail/area_light.inl:
 * 27-53): the emitting triangle and its intensity cl * kl.                         */
typedef struct gbrt_area_light
{
    gbrt_triangle geometry;
    float         cl[3];
    float         kl;
} gbrt_area_light;

/* One member of visionaray's generic_light<area_light, point_light, spot_light>
 * (generic_light.h) for next-event estimation:
 *   area  (detail/area_light.inl:27-53): geometry, cl, kl -- as gbrt_area_light
 *   point (detail/point_light.inl:16-56): position, cl, kl and the constant, linear
 *         and quadratic attenuation.  Its sample is a delta light of pdf 1 whose
 *         intensity is cl * kl * pi / constant attenuation: point_light::sample
 *         evaluates the attenuation at the light's own position (distance 0), so
 *         there is no distance falloff; it draws three random numbers (an unused
 *         normal)
 *   spot  (detail/spot_light.inl): as point plus spot_direction, spot_cutoff
 *         (radians) and spot_exponent.  spot_light::sample evaluates the cone at the
 *         light's own position too: normalize(0) is NaN, the cone test fails and the
 *         sample's intensity is 0 -- a spot light takes its share of the light picks
 *         and adds nothing, as in the reference
 * A light's draw count (1 pick + 2 for an area light, 1 + 3 for a point or spot
 * light) follows the reference's, so random streams stay matched.                  */
#define GBRT_LIGHT_AREA  0u
#define GBRT_LIGHT_POINT 1u
#define GBRT_LIGHT_SPOT  2u
typedef struct gbrt_light
{
    uint32_t      kind;
    float         cl[3];
    float         kl;
    gbrt_triangle geometry;
    float         position[3];
    float         attenuation[3];   /* constant, linear, quadratic */
    float         spot_direction[3];
    float         spot_cutoff;
    float         spot_exponent;
} gbrt_light;

/* pinhole_camera after look_at(eye, center, up) and perspective(fovy, w / h, ...)
 * (pinhole_camera.h, detail/pinhole_camera.inl:87-120).                            */
typedef struct gbrt_camera
{
    float eye[3];
    float center[3];
    float up[3];
    float fovy_degrees;
} gbrt_camera;

/* pinhole_camera::begin_frame (detail/pinhole_camera.inl:87-97) for a width x height
 * image: out = {eye, U, V, W} (12 floats); the primary ray through pixel coordinates
 * (x, y) has direction normalize(U * (2 (x + 0.5) / width - 1) + V * (2 (y + 0.5) /
 * height - 1) + W) (pinhole_camera.inl:103-120).  Host-only, no context.            */
gbrt_status gbrt_pinhole_camera_basis(gbrt_camera const* camera, uint32_t width, uint32_t height, float* out);

/* One frame of the jittered-blend pixel sampler (pixel_sampler_types.h,
 * detail/sched_common.h:427-526) around pathtracing::kernel (pathtracing.inl:42-233):
 * per pixel, spp jittered samples are averaged, then accum = sfactor * average +
 * dfactor * accum, and color = accum (dfactor == 0 overwrites accum without reading
 * it).  Random numbers come from gbrt_rng.h with (frame_id, pixel = y * width + x,
 * sample).                                                                        */
typedef struct gbrt_pt_params
{
    uint32_t width;
    uint32_t height;
    uint32_t spp;
    uint32_t num_bounces;    /* kernel_params::num_bounces (kernels.h:66)                */
    float    epsilon;        /* kernel_params::epsilon: ray-offset distance              */
    uint32_t frame_id;
    float    sfactor;
    float    dfactor;
    float    background[4];  /* make_kernel_params' bg_color: rgb * w for missed pixels  */
    float    ambient[3];     /* ambient light seen by rays that leave the scene          */
    uint32_t flags;          /* GBRT_PT_* bits                                           */
} gbrt_pt_params;

/* visionaray offsets a shadow ray's origin by epsilon towards the light sample AND ends
 * it at tmax = distance - epsilon (pathtracing.inl:171-176), so the sampled light
 * point lies exactly at tmax and the light's own triangle occludes it whenever
 * rounding lands its hit at or below tmax (about 80% of samples in FP32, 90% in
 * FP64).  Without this flag the kernel reproduces that behaviour bit for bit; with it
 * shadow rays end at distance - 2 * epsilon, as the reference evidently intends.     */
#define GBRT_PT_SHADOW_RANGE_FIX 1u
/* Disables Russian roulette (pathtracing.inl:201-213): paths run to num_bounces.  The
 * differentiable renderer uses it so that finite differences at common random numbers
 * are smooth in the albedos (a roulette decision would jump).                     */
#define GBRT_PT_NO_RUSSIAN_ROULETTE 2u
/* Scheduling only: one thread per pixel runs all its samples and bounces (one launch
 * per frame, shadow rays traced in-thread) instead of the wavefront passes.  Same
 * arithmetic and random numbers: the images are identical bit for bit.  About 2x
 * slower than the wavefront on the box and inverse-rendering workloads (GB300).     */
#define GBRT_PT_MEGAKERNEL 4u
/* Scheduling only: each bounce's ray and shadow queues are ordered by the Morton cell
 * of their origins before they are traced (images identical bit for bit).  Slower on
 * the box scene (GB300): the per-bounce sort costs more than the coherence it buys.  */
#define GBRT_PT_SORT_QUEUES 8u

typedef struct gbrt_pt_scene gbrt_pt_scene;

/* Binds a BVH, its materials (indexed by geom_id) and area lights (host arrays,
 * copied) into a renderable scene; the BVH must outlive the scene.  Plays the role of
 * make_kernel_params(prims, materials, lights, ...) (kernels.h:136-188).          */
gbrt_status gbrt_pt_scene_create(gbrt_context* ctx, gbrt_bvh const* bvh,
                                 gbrt_material const* h_materials, uint32_t num_materials,
                                 gbrt_area_light const* h_lights, uint32_t num_lights,
                                 gbrt_pt_scene** out);
/* As gbrt_pt_scene_create with a generic_light<area_light, point_light, spot_light>
 * list (make_kernel_params over generic lights, kernels.h:136-188; the light is
 * picked uniformly, sampling.h:195-213).                                          */
gbrt_status gbrt_pt_scene_create_lights(gbrt_context* ctx, gbrt_bvh const* bvh,
                                        gbrt_material const* h_materials, uint32_t num_materials,
                                        gbrt_light const* h_lights, uint32_t num_lights,
                                        gbrt_pt_scene** out);

/* make_kernel_params over an index_bvh<index_bvh_inst_t<P>> (bvh.h:678-782: the
 * primitives of a two-level tree) for pathtracing::kernel: a scene whose rays are
 * traced through the instances of a gbrt_tlas (intersect.inl:362-394), each hit shaded
 * with its instance's triangle in world space (the instance's transform applied to the
 * triangle's edges) and material slot h_inst_geom[instance] + the triangle's geom_id
 * (h_inst_geom: one host entry per instance).  Lights as for
 * gbrt_pt_scene_create_lights, in world space.  gbrt_pathtrace_frame and
 * gbrt_pathtrace_forward render it (wavefront scheduling only: not with
 * GBRT_PT_MEGAKERNEL or GBRT_PT_SORT_QUEUES) and gbrt_pathtrace_backward replays its
 * paths (gradients per material slot).  The tlas and its trees must outlive the scene. */
gbrt_status gbrt_pt_scene_create_instanced(gbrt_context* ctx, gbrt_tlas const* tlas,
                                           gbrt_material const* h_materials, uint32_t num_materials,
                                           gbrt_light const* h_lights, uint32_t num_lights,
                                           uint32_t const* h_inst_geom, gbrt_pt_scene** out);
gbrt_status gbrt_pt_scene_destroy(gbrt_pt_scene* scene);

/* An environment light in place of the constant ambient light: the kernel's amb_light
 * as environment_light<float, texture_ref<vec4, 2>> (environment_light.h:22-58,
 * detail/environment_light.inl:18-34).  A ray that leaves the scene adds
 * tex2D(texture, (u, v)).xyz * scale * throughput, where d = world_to_light * (dir, 0),
 * u = atan2(d.x, d.z) / 2 pi (+1 below 0) and v = acos(d.y) / pi; world_to_light is
 * the inverse of light_to_world computed as the reference's float cofactor inverse
 * (math/detail/matrix4.inl:353-388).  The texture is d_texels: width * height RGBA32F
 * texels in device memory, texel (x, y) at offset y * width + x, 16-byte aligned, read
 * through the CPU texture's filters (texture/detail/filter/nearest.h, linear.h) and
 * address modes (texture/detail/texture_common.h:91-126).  The scene keeps the pointer:
 * the texels stay valid and unchanged while the scene renders with them.           */
#define GBRT_FILTER_NEAREST 0u
#define GBRT_FILTER_LINEAR  1u
#define GBRT_ADDRESS_WRAP   0u
#define GBRT_ADDRESS_MIRROR 1u
#define GBRT_ADDRESS_CLAMP  2u
typedef struct gbrt_environment
{
    const float* d_texels;
    uint32_t     width;
    uint32_t     height;
    uint32_t     filter;              /* GBRT_FILTER_*                                */
    uint32_t     address;             /* GBRT_ADDRESS_*, both texture axes            */
    float        scale[3];
    float        light_to_world[16];  /* 4x4, column-major (visionaray's mat4)        */
} gbrt_environment;

/* Sets (env != NULL) or removes (NULL: the params' ambient light again) the scene's
 * environment light (environment_light::texture / scale / set_light_to_world_transform).
 * Bad sizes, modes, a null or misaligned texel pointer, or a singular transform are
 * GBRT_ERR_INVALID_ARG.  The batched renderer keeps the constant ambient light.    */
gbrt_status gbrt_pt_scene_set_environment(gbrt_context* ctx, gbrt_pt_scene* scene, gbrt_environment const* env);

/* Renders one frame: cuda_sched<basic_ray<float>>::frame(pathtracing::kernel{params},
 * make_sched_params(jittered_blend, cam, rt)) (detail/cuda_sched.inl:226-246) as a
 * wavefront path tracer.  d_accum and d_color are RGBA32F device images of
 * width * height pixels (row y at offset y * width); d_color may be NULL.
 * Asynchronous on the context stream.                                             */
gbrt_status gbrt_pathtrace_frame(gbrt_context* ctx, gbrt_pt_scene const* scene,
                                 gbrt_camera const* camera, gbrt_pt_params const* params,
                                 float* d_accum, float* d_color);

/* Differentiable rendering (no visionaray counterpart: the reference has no adjoint).
 * Parameters are per material slot (geom_id), 3 floats each, in device memory: the
 * albedo of matte slots (replacing their color; scale stays kd) and the emission of
 * emissive slots (replacing ce; scale stays ls); an area light whose triangle's
 * geom_id is an emissive slot shines emission[geom_id] * kl.
 * forward: one frame of the path tracer with those parameters; d_image (RGBA32F)
 * receives the per-pixel sample average (sfactor/dfactor are ignored).           */
gbrt_status gbrt_pathtrace_forward(gbrt_context* ctx, gbrt_pt_scene const* scene,
                                   gbrt_camera const* camera, gbrt_pt_params const* params,
                                   const float* d_albedo, const float* d_emission, float* d_image);

/* backward: path-replay backpropagation of an image adjoint d_image_adjoint = dL/dI
 * (RGBA32F, alpha ignored) into d_grad_albedo and d_grad_emission (3 floats per slot,
 * ADDED to; zero them first).  Each (pixel, sample) path is re-traced from its random
 * numbers -- the same shading code as the forward frame, so the same path -- and its
 * vertices swept backwards; nothing of the forward frame is stored (memory O(pixels)).
 * Gradients are accumulated with warp-reduced FP32 atomics.  Geometry, visibility and
 * roulette decisions are not differentiated.  num_bounces <= 16.  A scene over
 * instances (gbrt_pt_scene_create_instanced) replays through the same two-level tree;
 * a slot's gradient sums the vertices of every instance that uses the slot.      */
gbrt_status gbrt_pathtrace_backward(gbrt_context* ctx, gbrt_pt_scene const* scene,
                                    gbrt_camera const* camera, gbrt_pt_params const* params,
                                    const float* d_albedo, const float* d_emission,
                                    const float* d_image_adjoint, float* d_grad_albedo,
                                    float* d_grad_emission);

/* ------------------------------------------------------------------------------ */
/* Two-level instancing: index_bvh_inst_t (bvh.h:678-782) and the top-level BVH over
 * instances, traversed as intersect(ray, instance) does (detail/bvh/intersect.inl:
 * 362-394): the ray is carried into the instance's space and its tree traversed.      */

/* An instance: a bottom-level tree and visionaray's mat4x3 transform, 4 columns of 3
 * floats (col0, col1, col2, col3).  As in index_bvh_inst_t(ref, transform), the
 * linear map is top_left(transform) (matrix4x3.inl:206-219: row i of the map is
 * column i of the matrix) and the translation is col3: world = top_left * p + col3.
 * The inverse is computed as the reference does (matrix3.inl:285-305, float) and a
 * ray is mapped as transform_ray (bvh.h:742-750): ori' = A (ori - col3), dir' = A dir. */
typedef struct gbrt_instance
{
    gbrt_bvh const* blas;
    float transform[12];
} gbrt_instance;

/* hit_record_bvh_inst (detail/bvh/hit_record.h:57-75): prim_id of the instance's
 * triangle, inst_id = the instance's index (GBRT_NO_HIT on a miss), t, u, v in the
 * instance space's parameterisation (t is the world ray's parameter), geom_id.      */
typedef struct gbrt_hit_inst
{
    uint32_t prim_id;
    uint32_t inst_id;
    float    t;
    float    u;
    float    v;
    uint32_t geom_id;
    uint32_t reserved[2];
} gbrt_hit_inst;


/* Builds the top-level tree over h_instances (host array; the bottom-level trees must
 * outlive the tlas): instance bounds as get_bounds(instance) computes them
 * (detail/bvh/get_bounds.inl:30-56: the 8 corners of the tree's root box mapped to
 * world space), a median-split hierarchy of node pairs over them (one instance per
 * leaf).  Synchronous.                                                              */
gbrt_status gbrt_tlas_build(gbrt_context* ctx, gbrt_instance const* h_instances, uint32_t num_instances,
                            gbrt_tlas** out);
gbrt_status gbrt_tlas_destroy(gbrt_tlas* tlas);

/* closest_hit / any_hit over the instances (device rays and hits, 16-byte aligned):
 * per ray, the closest (any) hit of any instance within [tmin, tmax].               */
gbrt_status gbrt_tlas_trace_closest_hit(gbrt_context* ctx, gbrt_tlas const* tlas, gbrt_ray const* d_rays,
                                        uint32_t n, gbrt_hit_inst* d_hits);
gbrt_status gbrt_tlas_trace_any_hit(gbrt_context* ctx, gbrt_tlas const* tlas, gbrt_ray const* d_rays,
                                    uint32_t n, gbrt_hit_inst* d_hits);

/* ------------------------------------------------------------------------------ */
/* Batches of scenes (no visionaray counterpart: the reference builds and renders one
 * scene per call, lbvh.h:681-844 and cuda_sched.inl:226-246).                      */

typedef struct gbrt_batch gbrt_batch;

/* Creates a batch of num_scenes scenes over one concatenated triangle array: scene s
 * owns triangles [h_offsets[s], h_offsets[s + 1]) (h_offsets: num_scenes + 1 host
 * entries, non-decreasing, h_offsets[0] = 0).  Allocates the whole BVH arena and the
 * build temporaries once, so the build and frame calls below only enqueue kernels.   */
gbrt_status gbrt_batch_create(gbrt_context* ctx, uint32_t const* h_offsets, uint32_t num_scenes,
                              gbrt_batch** out);
gbrt_status gbrt_batch_destroy(gbrt_batch* batch);

/* Builds every scene's LBVH in one pass (per-scene Morton normalisation, one sort by
 * (scene, code), Karras hierarchies and refit over all segments): each scene's tree is
 * the one gbrt_bvh_build_lbvh builds for that scene alone.  Enqueue only
 * (asynchronous, no allocation, no synchronisation).                              */
gbrt_status gbrt_batch_build(gbrt_context* ctx, gbrt_batch* batch, gbrt_triangle const* d_tris);

/* Reference-layout export of scene s (as gbrt_bvh_export_bvh2 for that scene).     */
gbrt_status gbrt_batch_export_bvh2(gbrt_context* ctx, gbrt_batch const* batch, uint32_t scene,
                                   gbrt_bvh_node* d_nodes, uint32_t* d_indices);

/* closest_hit of rays of all scenes in one launch: scene s traces rays
 * [h_ray_offsets[s], h_ray_offsets[s + 1]) (num_scenes + 1 host entries).          */
gbrt_status gbrt_batch_trace_closest_hit(gbrt_context* ctx, gbrt_batch const* batch,
                                         gbrt_ray const* d_rays, uint32_t const* h_ray_offsets,
                                         gbrt_hit* d_hits);

/* Per-scene frame setup for gbrt_batch_pathtrace: h_cameras / h_params (num_scenes
 * entries; params' sfactor / dfactor ignored, each scene's image is overwritten) and
 * materials (indexed by geom_id, shared by all scenes).  Copies to the device.       */
gbrt_status gbrt_batch_set_frames(gbrt_context* ctx, gbrt_batch* batch, gbrt_camera const* h_cameras,
                                  gbrt_pt_params const* h_params, gbrt_material const* h_materials,
                                  uint32_t num_materials);

/* Launch shape of gbrt_batch_pathtrace (the autotuner's search space).            */
#define GBRT_BATCH_ORDER_ROWS 0u    /* a warp's pixels are consecutive in a row       */
#define GBRT_BATCH_ORDER_BLOCKS 1u  /* a warp's 32 pixels are an 8x4 screen block
                                       (scenes with width % 8 == 0, height % 4 == 0;
                                       rows otherwise)                                */
typedef struct gbrt_batch_launch
{
    uint32_t block;  /* threads per block: 128, 256 or 512                         */
    uint32_t tile;   /* pixels a warp takes from the work queue per grab: 32 or 64  */
    uint32_t stack;  /* traversal stack entries: 16, 24, 32 or 64 (a tree taller
                        than this sets GBRT_ERR_STACK_OVERFLOW); width 2 only       */
    uint32_t order;  /* GBRT_BATCH_ORDER_*                                          */
    uint32_t width;  /* BVH width: 2 (node pairs), 4 or 8 (each frame first collapses
                        the last build's trees, bvh_collapser's BVH4/8; hits equal
                        the pairs' except equal-t ties)                             */
    uint32_t sort;   /* 1: rays sorted -- each frame first traces every pixel's first
                        primary ray and takes pixels in the order of (scene, Morton
                        cell of that hit) instead of `order`; 0: off               */
} gbrt_batch_launch;

/* Sets / reads the launch shape (default {128, 32, 64, ROWS, 2, 0}).                */
gbrt_status gbrt_batch_set_launch(gbrt_batch* batch, gbrt_batch_launch const* launch);
gbrt_status gbrt_batch_get_launch(gbrt_batch const* batch, gbrt_batch_launch* out);

/* Tallest tree of the last gbrt_batch_build (edges from a root to its deepest leaf);
 * synchronises the context stream.                                                 */
gbrt_status gbrt_batch_height(gbrt_context* ctx, gbrt_batch const* batch, uint32_t* out);

/* One frame of every scene in a single persistent launch: warps take tiles of pixels of
 * any scene from one atomic work queue and run the path tracer (the same shading as
 * gbrt_pathtrace_frame, so scene s's image equals the one gbrt_pathtrace_frame
 * renders with its camera, params and lights).  d_images: RGBA32F, 16-byte aligned,
 * scene s at pixel offset sum_{t<s} width_t * height_t.  Enqueue only.              */
gbrt_status gbrt_batch_pathtrace(gbrt_context* ctx, gbrt_batch* batch, float* d_images);

/* The lights of each scene of a batch (make_kernel_params' light list per scene,
 * pathtracing.inl:42-233 next-event estimation): h_lights (host, area / point / spot
 * records as for gbrt_pt_scene_create_lights), scene s sampling
 * h_lights[h_light_offsets[s] .. h_light_offsets[s + 1]) (num_scenes + 1 host
 * entries from 0 to num_lights; null when num_lights is 0).  Replaces earlier lights;
 * scenes without lights keep the params' ambient light only.  Synchronises the
 * context stream.                                                                   */
gbrt_status gbrt_batch_set_lights(gbrt_context* ctx, gbrt_batch* batch, gbrt_light const* h_lights,
                                  uint32_t num_lights, uint32_t const* h_light_offsets);

/* gbrt_batch_build + gbrt_batch_pathtrace captured once into a CUDA graph and
 * replayed on the context stream on every call (re-captured when d_tris, d_images,
 * the frames, the lights or the launch shape change); with width 4 or 8 the graph
 * holds the collapse, with sorting the pixel order, so every replay redoes both.    */
gbrt_status gbrt_batch_run_graph(gbrt_context* ctx, gbrt_batch* batch, gbrt_triangle const* d_tris,
                                 float* d_images);

/* Autotuner: times gbrt_batch_pathtrace (after gbrt_batch_build and
 * gbrt_batch_set_frames) over the search space, `reps` runs each after one warm-up
 * run, and keeps the fastest (also written to *best, with its time per frame in
 * *best_ms; either may be NULL): first every block x tile x stack x order on the node
 * pairs without sorting (stacks that hold the tallest tree), then, at the winner's
 * block, tile and order, BVH width {2, 4, 8} x ray sorting {off, on} with each frame's
 * collapse and sort timed in.  Shapes whose run raised a status are skipped.
 * d_images is overwritten.                                                          */
gbrt_status gbrt_batch_autotune(gbrt_context* ctx, gbrt_batch* batch, float* d_images, uint32_t reps,
                                gbrt_batch_launch* best, float* best_ms);

/* Number of kernels the library launched on this context since creation (the
 * count covers every kernel of every call).                                        */
uint64_t gbrt_kernel_launch_count(gbrt_context const* ctx);

/* Instrumentation (no visionaray counterpart: the reference times nothing itself).
 * While enabled, every ray query (gbrt_trace_*) records a CUDA event pair around its
 * traversal kernel -- after the ray order is computed -- on the stream it runs on, in
 * a ring of the 256 most recent queries.  gbrt_context_kernel_times waits for the
 * recorded events, writes the durations (ms) of the most recent min(recorded, max,
 * 256) queries, oldest first, to out_ms, their number to *count, and clears the
 * record.  Enabling also clears it.                                                */
gbrt_status gbrt_context_set_kernel_timing(gbrt_context* ctx, int enable);
gbrt_status gbrt_context_kernel_times(gbrt_context* ctx, float* out_ms, uint32_t max, uint32_t* count);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* VISIONARAY_GB300_GBRT_H */
