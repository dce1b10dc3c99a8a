// visionaray_gb300.hpp -- header-only C++ shim over the C ABI (gbrt.h) that keeps the
// shape of visionaray's API for the GPU ray-tracing path, so a visionaray caller
// changes a namespace and a few types, not its control flow:
//
//   visionaray                                          visionaray_gb300
//   lbvh_builder builder;                               visionaray_gb300::lbvh_builder builder(ctx);
//   auto bvh = builder.build(cuda_index_bvh<P>{},       auto bvh = builder.build(visionaray_gb300::cuda_index_bvh{},
//                            d_prims, n);                                        d_prims, n);
//   (lbvh.h:681-844)
//   closest_hit(ray, refs, refs + 1)  (per ray,         visionaray_gb300::closest_hit(ctx, bvh, d_rays, n, d_hits)
//   traverse_linear.inl:192-225)                        (batched: a device functor cannot cross a C ABI)
//   any_hit(ray, refs, refs + 1)  (:156-189)            visionaray_gb300::any_hit(ctx, bvh, d_rays, n, d_hits)
//   auto kp = make_kernel_params(prims, materials,      auto kp = visionaray_gb300::make_kernel_params(ctx, bvh,
//       lights, bounces, eps, bg, ambient)                  materials, lights, bounces, eps, bg, ambient)
//   (kernels.h:136-188)
//   pathtracing::kernel<decltype(kp)> k; k.params = kp; visionaray_gb300::pathtracing::kernel<...> k; k.params = &kp;
//   cuda_sched<R>(8, 8).frame(k, make_sched_params(     visionaray_gb300::cuda_sched(ctx).frame(k,
//       jittered_blend, cam, rt))                           sched_params{camera, width, height, spp, ...})
//   (detail/cuda_sched.inl:226-246)                     (the built-in path tracer only: a user lambda is device
//                                                        code that cannot cross a C ABI)
//
// Errors: the reference prints through CUDA_SAFE_CALL (cuda/safe_call.h:18-23) and
// carries on; the shim throws visionaray_gb300::error carrying the gbrt_status.
#pragma once

#include <array>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gbrt.h"

namespace visionaray_gb300 {

struct error : std::runtime_error
{
    gbrt_status status;
    error(gbrt_status st, std::string const& what) : std::runtime_error(what), status(st) {}
};

inline void check(gbrt_status st, gbrt_context const* ctx, const char* where)
{
    if (st != GBRT_OK)
        throw error(st, std::string(where) + ": " + (ctx ? gbrt_last_error(ctx) : "invalid argument"));
}

// One device + one CUDA stream (the stream argument of cuda_sched::frame and the
// copy stream of lbvh_builder, detail/cuda_sched.h:39, detail/bvh/lbvh.h:669-679).
class context
{
public:
    explicit context(int device = 0, void* stream = nullptr)
    {
        check(gbrt_context_create(device, stream, &h_), nullptr, "gbrt_context_create");
    }
    ~context()
    {
        if (h_) gbrt_context_destroy(h_);
    }
    context(context const&) = delete;
    context& operator=(context const&) = delete;

    gbrt_context* get() const { return h_; }
    void synchronize() { check(gbrt_context_synchronize(h_), h_, "gbrt_context_synchronize"); }
    void set_stream(void* stream) { check(gbrt_context_set_stream(h_, stream), h_, "gbrt_context_set_stream"); }
    unsigned long long kernel_launches() const { return gbrt_kernel_launch_count(h_); }

private:
    gbrt_context* h_ = nullptr;
};

// Owning device BVH over basic_triangle<3, float, unsigned> (bvh.h:1093).  Move-only:
// the reference's deep copy between host and device trees is the upload below.
class cuda_index_bvh
{
public:
    cuda_index_bvh() = default;
    cuda_index_bvh(context& ctx, gbrt_bvh* h) : ctx_(&ctx), h_(h) {}
    ~cuda_index_bvh() { reset(); }
    cuda_index_bvh(cuda_index_bvh&& o) noexcept : ctx_(o.ctx_), h_(std::exchange(o.h_, nullptr)) {}
    cuda_index_bvh& operator=(cuda_index_bvh&& o) noexcept
    {
        if (this != &o)
        {
            reset();
            ctx_ = o.ctx_;
            h_ = std::exchange(o.h_, nullptr);
        }
        return *this;
    }
    cuda_index_bvh(cuda_index_bvh const&) = delete;
    cuda_index_bvh& operator=(cuda_index_bvh const&) = delete;

    // Host index_bvh (nodes + index list + primitives) copied to the device
    // (bvh.h:963-1009).
    static cuda_index_bvh upload(context& ctx, std::vector<gbrt_bvh_node> const& nodes,
                                 std::vector<uint32_t> const& indices, gbrt_triangle const* prims, size_t n)
    {
        gbrt_bvh* h = nullptr;
        check(gbrt_bvh_upload_bvh2_host(ctx.get(), nodes.data(), uint32_t(nodes.size()), indices.data(),
                                        uint32_t(indices.size()), prims, uint32_t(n), &h),
              ctx.get(), "gbrt_bvh_upload_bvh2_host");
        return cuda_index_bvh(ctx, h);
    }

    gbrt_bvh* get() const { return h_; }
    size_t num_primitives() const
    {
        uint32_t n = 0;
        gbrt_bvh_counts(h_, &n, nullptr, nullptr);
        return n;
    }
    size_t num_nodes() const
    {
        uint32_t nn = 0;
        gbrt_bvh_counts(h_, nullptr, &nn, nullptr);
        return nn;
    }

    // The tree in the reference's cuda_index_bvh node layout (device buffers sized
    // num_nodes() and num_primitives()).
    void export_nodes(gbrt_bvh_node* d_nodes, uint32_t* d_indices) const
    {
        check(gbrt_bvh_export_bvh2(ctx_->get(), h_, d_nodes, d_indices), ctx_->get(), "gbrt_bvh_export_bvh2");
    }

private:
    void reset()
    {
        if (h_) gbrt_bvh_destroy(h_);
        h_ = nullptr;
    }
    context* ctx_ = nullptr;
    gbrt_bvh* h_ = nullptr;
};

// lbvh_builder (detail/bvh/lbvh.h:473-851), GPU build.  P must have the layout of
// basic_triangle<3, float, unsigned> (44 bytes).
struct lbvh_builder
{
    explicit lbvh_builder(context& ctx) : ctx_(&ctx) {}

    template <typename P>
    cuda_index_bvh build(cuda_index_bvh /* tag, as the reference's Tree{} */, P const* d_primitives, size_t num_prims)
    {
        static_assert(sizeof(P) == sizeof(gbrt_triangle), "P must be laid out as basic_triangle<3, float, unsigned>");
        if (num_prims > 0xFFFFFFFFu) throw error(GBRT_ERR_TOO_LARGE, "lbvh_builder::build: too many primitives");
        gbrt_bvh* h = nullptr;
        check(gbrt_bvh_build_lbvh(ctx_->get(), reinterpret_cast<gbrt_triangle const*>(d_primitives),
                                  uint32_t(num_prims), &h),
              ctx_->get(), "gbrt_bvh_build_lbvh");
        return cuda_index_bvh(*ctx_, h);
    }

private:
    context* ctx_;
};

// Parallel locally-ordered clustering build (no visionaray counterpart; a tree of
// lower SAH cost than the LBVH over the same Morton order).  P as for lbvh_builder.
struct ploc_builder
{
    explicit ploc_builder(context& ctx) : ctx_(&ctx) {}

    template <typename P>
    cuda_index_bvh build(cuda_index_bvh /* tag */, P const* d_primitives, size_t num_prims)
    {
        static_assert(sizeof(P) == sizeof(gbrt_triangle), "P must be laid out as basic_triangle<3, float, unsigned>");
        if (num_prims > 0xFFFFFFFFu) throw error(GBRT_ERR_TOO_LARGE, "ploc_builder::build: too many primitives");
        gbrt_bvh* h = nullptr;
        check(gbrt_bvh_build_ploc(ctx_->get(), reinterpret_cast<gbrt_triangle const*>(d_primitives),
                                  uint32_t(num_prims), &h),
              ctx_->get(), "gbrt_bvh_build_ploc");
        return cuda_index_bvh(*ctx_, h);
    }

private:
    context* ctx_;
};

// bvh_refitter (detail/bvh/refit.h:25-117), GPU refit of an LBVH-built tree to new
// positions of its primitives (device, the build's order).
struct bvh_refitter
{
    explicit bvh_refitter(context& ctx) : ctx_(&ctx) {}

    template <typename P>
    void refit(cuda_index_bvh& tree, P const* d_primitives, size_t num_prims)
    {
        static_assert(sizeof(P) == sizeof(gbrt_triangle), "P must be laid out as basic_triangle<3, float, unsigned>");
        if (num_prims > 0xFFFFFFFFu) throw error(GBRT_ERR_TOO_LARGE, "bvh_refitter::refit: too many primitives");
        check(gbrt_bvh_refit(ctx_->get(), tree.get(), reinterpret_cast<gbrt_triangle const*>(d_primitives),
                             uint32_t(num_prims)),
              ctx_->get(), "gbrt_bvh_refit");
    }

private:
    context* ctx_;
};

// Batched closest_hit / any_hit over one BVH (device buffers, asynchronous on the
// context stream).
inline void closest_hit(context& ctx, cuda_index_bvh const& bvh, gbrt_ray const* d_rays, size_t n, gbrt_hit* d_hits)
{
    check(gbrt_trace_closest_hit(ctx.get(), bvh.get(), d_rays, uint32_t(n), d_hits), ctx.get(),
          "gbrt_trace_closest_hit");
}

inline void any_hit(context& ctx, cuda_index_bvh const& bvh, gbrt_ray const* d_rays, size_t n, gbrt_hit* d_hits)
{
    check(gbrt_trace_any_hit(ctx.get(), bvh.get(), d_rays, uint32_t(n), d_hits), ctx.get(), "gbrt_trace_any_hit");
}

// environment_light<float, texture_ref<vec4, 2>> (environment_light.h:22-58): a
// device RGBA32F lat-long texture (width * height texels, row-major; it must outlive
// the kernel_params it is set on), the texture's filter and address modes, the scale
// and light_to_world (column-major).  kernel_params::set_environment puts it in place
// of the ambient light.
struct environment_light
{
    const float* d_texels = nullptr;
    unsigned width = 0, height = 0;
    unsigned filter = GBRT_FILTER_LINEAR, address = GBRT_ADDRESS_CLAMP;
    std::array<float, 3> scale{ { 1.0f, 1.0f, 1.0f } };
    std::array<float, 16> light_to_world{ { 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f,
                                            0.0f, 0.0f, 0.0f, 1.0f } };

    void set_light_to_world_transform(std::array<float, 16> const& m) { light_to_world = m; }
};

// make_kernel_params(prims, materials, lights, num_bounces, epsilon, bg_color,
// ambient_color) (kernels.h:136-188) for the built-in path tracer: the scene (a BVH
// that must outlive it, materials indexed by geom_id, lights; host arrays, copied)
// and the per-frame constants.  Move-only.
class kernel_params
{
public:
    kernel_params(context& ctx, cuda_index_bvh const& bvh, std::vector<gbrt_material> const& materials,
                  std::vector<gbrt_light> const& lights, unsigned num_bounces, float epsilon,
                  std::array<float, 4> background, std::array<float, 3> ambient)
        : ctx_(&ctx), num_bounces(num_bounces), epsilon(epsilon), background(background), ambient(ambient)
    {
        check(gbrt_pt_scene_create_lights(ctx.get(), bvh.get(), materials.data(), uint32_t(materials.size()),
                                          lights.data(), uint32_t(lights.size()), &scene_),
              ctx.get(), "gbrt_pt_scene_create_lights");
    }
    ~kernel_params()
    {
        if (scene_) gbrt_pt_scene_destroy(scene_);
    }
    kernel_params(kernel_params&& o) noexcept
        : ctx_(o.ctx_), scene_(std::exchange(o.scene_, nullptr)), num_bounces(o.num_bounces), epsilon(o.epsilon),
          background(o.background), ambient(o.ambient)
    {
    }
    kernel_params(kernel_params const&) = delete;
    kernel_params& operator=(kernel_params const&) = delete;
    kernel_params& operator=(kernel_params&&) = delete;

    gbrt_pt_scene* scene() const { return scene_; }
    context& ctx() const { return *ctx_; }

    // amb_light = env (kernels.h:423-424 with an environment_light)
    void set_environment(environment_light const& env)
    {
        gbrt_environment e{};
        e.d_texels = env.d_texels;
        e.width = env.width;
        e.height = env.height;
        e.filter = env.filter;
        e.address = env.address;
        for (int c = 0; c < 3; ++c) e.scale[c] = env.scale[size_t(c)];
        for (int k = 0; k < 16; ++k) e.light_to_world[k] = env.light_to_world[size_t(k)];
        check(gbrt_pt_scene_set_environment(ctx_->get(), scene_, &e), ctx_->get(), "gbrt_pt_scene_set_environment");
    }

private:
    context* ctx_;
    gbrt_pt_scene* scene_ = nullptr;

public:
    unsigned num_bounces;
    float epsilon;
    std::array<float, 4> background;
    std::array<float, 3> ambient;
};

inline kernel_params make_kernel_params(context& ctx, cuda_index_bvh const& bvh,
                                        std::vector<gbrt_material> const& materials,
                                        std::vector<gbrt_light> const& lights, unsigned num_bounces, float epsilon,
                                        std::array<float, 4> background, std::array<float, 3> ambient)
{
    return kernel_params(ctx, bvh, materials, lights, num_bounces, epsilon, background, ambient);
}

// The same with area_light<float, basic_triangle> records.
inline kernel_params make_kernel_params(context& ctx, cuda_index_bvh const& bvh,
                                        std::vector<gbrt_material> const& materials,
                                        std::vector<gbrt_area_light> const& area_lights, unsigned num_bounces,
                                        float epsilon, std::array<float, 4> background, std::array<float, 3> ambient)
{
    std::vector<gbrt_light> lights(area_lights.size());
    for (size_t i = 0; i < area_lights.size(); ++i)
    {
        lights[i] = gbrt_light{};
        lights[i].kind = GBRT_LIGHT_AREA;
        lights[i].geometry = area_lights[i].geometry;
        for (int c = 0; c < 3; ++c) lights[i].cl[c] = area_lights[i].cl[c];
        lights[i].kl = area_lights[i].kl;
    }
    return kernel_params(ctx, bvh, materials, lights, num_bounces, epsilon, background, ambient);
}

namespace pathtracing {

// pathtracing::kernel<Params> (detail/pathtracing.inl:33-233): holds the parameters it
// renders with (by pointer here: kernel_params owns device memory).
template <typename Params>
struct kernel
{
    Params const* params = nullptr;
};

} // namespace pathtracing

// What make_sched_params(pixel_sampler::jittered_blend_type, camera, render_target)
// carries for one frame (detail/sched_common.h:427-526): the pinhole camera, the image
// size, samples per pixel, the blend accum = sfactor * frame + dfactor * accum, the
// frame number that seeds the random stream, and the render target (RGBA32F device
// images; d_color may be null).
struct sched_params
{
    gbrt_camera camera;
    uint32_t width = 0, height = 0, spp = 1, frame_id = 0;
    float sfactor = 1.0f, dfactor = 0.0f;
    float* d_accum = nullptr;
    float* d_color = nullptr;
    uint32_t flags = 0;   // GBRT_PT_* bits
};

// cuda_sched<R>::frame (detail/cuda_sched.inl:226-246) for the built-in path tracer:
// asynchronous on the context stream.
class cuda_sched
{
public:
    explicit cuda_sched(context& ctx) : ctx_(&ctx) {}

    void frame(pathtracing::kernel<kernel_params> const& k, sched_params const& sp)
    {
        if (!k.params) throw error(GBRT_ERR_INVALID_ARG, "cuda_sched::frame: kernel without params");
        kernel_params const& kp = *k.params;
        gbrt_pt_params p{};
        p.width = sp.width;
        p.height = sp.height;
        p.spp = sp.spp;
        p.num_bounces = kp.num_bounces;
        p.epsilon = kp.epsilon;
        p.frame_id = sp.frame_id;
        p.sfactor = sp.sfactor;
        p.dfactor = sp.dfactor;
        for (int c = 0; c < 4; ++c) p.background[c] = kp.background[size_t(c)];
        for (int c = 0; c < 3; ++c) p.ambient[c] = kp.ambient[size_t(c)];
        p.flags = sp.flags;
        check(gbrt_pathtrace_frame(ctx_->get(), kp.scene(), &sp.camera, &p, sp.d_accum, sp.d_color), ctx_->get(),
              "gbrt_pathtrace_frame");
    }

private:
    context* ctx_;
};

} // namespace visionaray_gb300
