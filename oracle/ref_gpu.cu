// Device-code driver around visionaray's own GPU traversal and path-tracing kernel.
// TEST AND BENCHMARK INFRASTRUCTURE ONLY: compiled from the unmodified visionaray
// headers (where they are present) into oracle/_ref/vsnray_ref_gpu.cubin for sm_103a,
// which oracle/ref_gpu.py loads with the CUDA driver API on the GPU host (device code
// does not depend on the host architecture).  It times the reference's GPU path beside
// the product's kernels on the same trees, rays and random numbers.  Nothing in the
// product loads it.
//
// Calls used, as a visionaray user's kernel makes them:
//   closest_hit / any_hit over an index_bvh_ref_t (detail/traverse_linear.inl:156-225,
//     whose device branch is the short-stack traversal of detail/bvh/intersect.inl:166-356)
//   pathtracing::kernel::operator() (detail/pathtracing.inl:42-233) with
//     generic_material<matte, emissive> per geom_id and triangle area lights (and an
//     extended instantiation: generic_material<matte, emissive, mirror, glass, plastic>
//     and generic_light<area_light, point_light, spot_light>), one thread
//     per pixel as cuda_sched's render kernel runs it (detail/cuda_sched.inl:32-69),
//     samples averaged and blended as sample_pixel_impl does (sched_common.h:427-526)
// Host-side helpers of visionaray (make_kernel_params, area_light's constructor,
// pinhole_camera's setup) cannot run on the GPU host, so the kernel-parameter struct,
// the light and material objects are filled in device code, and the camera basis comes
// in as a parameter (the pinhole_camera::primary_ray arithmetic, pinhole_camera.inl:
// 103-120, with the default image region).

#include <cfloat>
#include <cstdint>
#include <cstring>
#include <utility>

#include <visionaray/area_light.h>
#include <visionaray/bvh.h>
#include <visionaray/generic_light.h>
#include <visionaray/generic_material.h>
#include <visionaray/kernels.h>
#include <visionaray/material.h>
#include <visionaray/math/math.h>
#include <visionaray/point_light.h>
#include <visionaray/spot_light.h>
#include <visionaray/traverse.h>

#include "../include/visionaray_gb300/gbrt.h"
#include "../include/visionaray_gb300/gbrt_rng.h"

using namespace visionaray;

using triangle_t = basic_triangle<3, float, unsigned>;
using tree_ref_t = index_bvh_ref_t<triangle_t>;
using mat_t = generic_material<matte<float>, emissive<float>>;
using light_t = area_light<float, triangle_t>;
// the extended instantiation: every material kind and generic lights
using mat_ext_t = generic_material<matte<float>, emissive<float>, mirror<float>, glass<float>, plastic<float>>;
using light_ext_t = generic_light<area_light<float, triangle_t>, point_light<float>, spot_light<float>>;
template <typename Mat, typename Light>
using kparams_of = decltype(make_kernel_params(std::declval<tree_ref_t const*>(), std::declval<tree_ref_t const*>(),
                                               std::declval<Mat const*>(), std::declval<Light const*>(),
                                               std::declval<Light const*>(), 0u, 0.0f, vec4(), vec4()));

static_assert(sizeof(triangle_t) == sizeof(gbrt_triangle), "triangle layout");
static_assert(sizeof(bvh_node) == sizeof(gbrt_bvh_node), "node layout");
static_assert(sizeof(basic_ray<float>) == sizeof(gbrt_ray), "ray layout");

// The six pointers of an index_bvh_ref_t: primitives, nodes and indices, each as
// [first, last).
struct ref_ptrs
{
    const void* p[6];
};
static_assert(sizeof(tree_ref_t) == sizeof(ref_ptrs), "index_bvh_ref_t is six pointers");

__device__ inline tree_ref_t make_ref(ref_ptrs const& r)
{
    tree_ref_t b;
    memcpy(static_cast<void*>(&b), &r, sizeof(b));
    return b;
}

__device__ inline void store_hit(gbrt_hit* out, bool hit, unsigned prim, float t, float u, float v)
{
    out->prim_id = hit ? prim : GBRT_NO_HIT;
    out->t = t;
    out->u = u;
    out->v = v;
}

extern "C" __global__ void vsnray_ref_closest_hit(ref_ptrs tree, const gbrt_ray* rays, unsigned n, gbrt_hit* hits)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    tree_ref_t ref = make_ref(tree);
    basic_ray<float> r;
    memcpy(static_cast<void*>(&r), &rays[i], sizeof(r));
    auto hr = closest_hit(r, &ref, &ref + 1);
    store_hit(&hits[i], hr.hit, hr.prim_id, hr.t, hr.u, hr.v);
}

extern "C" __global__ void vsnray_ref_any_hit(ref_ptrs tree, const gbrt_ray* rays, unsigned n, gbrt_hit* hits)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    tree_ref_t ref = make_ref(tree);
    basic_ray<float> r;
    memcpy(static_cast<void*>(&r), &rays[i], sizeof(r));
    auto hr = any_hit(r, &ref, &ref + 1);
    store_hit(&hits[i], hr.hit, hr.prim_id, hr.t, hr.u, hr.v);
}

// Materials per geom_id and area lights as visionaray objects (one thread per item):
// refs[0] = the tree, mats[nm], lights[nl].
extern "C" __global__ void vsnray_ref_pt_setup(ref_ptrs tree, tree_ref_t* refs, const gbrt_material* in_m, unsigned nm,
                                               mat_t* mats, const gbrt_area_light* in_l, unsigned nl, light_t* lights)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) refs[0] = make_ref(tree);
    if (i < nm)
    {
        vec3 c(in_m[i].color[0], in_m[i].color[1], in_m[i].color[2]);
        if (in_m[i].kind == GBRT_MATERIAL_EMISSIVE)
        {
            emissive<float> e;
            e.ce() = from_rgb(c);
            e.ls() = in_m[i].scale;
            static_cast<mat_t::base_type&>(mats[i]) = e;   // variant's device assignment
        }
        else
        {
            matte<float> m;
            m.ca() = from_rgb(vec3(0.0f));
            m.ka() = 0.0f;
            m.cd() = from_rgb(c);
            m.kd() = in_m[i].scale;
            static_cast<mat_t::base_type&>(mats[i]) = m;
        }
    }
    if (i < nl)
    {
        light_t l;
        memcpy(static_cast<void*>(&l.geometry()), &in_l[i].geometry, sizeof(triangle_t));
        l.set_cl(vec3(in_l[i].cl[0], in_l[i].cl[1], in_l[i].cl[2]));
        l.set_kl(in_l[i].kl);
        lights[i] = l;
    }
}

// The extended instantiation's materials (all five kinds) and lights (area, point,
// spot), with the field mapping of gbrt.h.
extern "C" __global__ void vsnray_ref_pt_setup_ext(ref_ptrs tree, tree_ref_t* refs, const gbrt_material* in_m,
                                                   unsigned nm, mat_ext_t* mats, const gbrt_light* in_l, unsigned nl,
                                                   light_ext_t* lights)
{
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) refs[0] = make_ref(tree);
    if (i < nm)
    {
        gbrt_material const& g = in_m[i];
        vec3 c(g.color[0], g.color[1], g.color[2]), c2(g.color2[0], g.color2[1], g.color2[2]);
        vec3 ior(g.ior[0], g.ior[1], g.ior[2]), ab(g.absorption[0], g.absorption[1], g.absorption[2]);
        auto& dst = static_cast<mat_ext_t::base_type&>(mats[i]);
        if (g.kind == GBRT_MATERIAL_EMISSIVE)
        {
            emissive<float> e;
            e.ce() = from_rgb(c);
            e.ls() = g.scale;
            dst = e;
        }
        else if (g.kind == GBRT_MATERIAL_MIRROR)
        {
            mirror<float> m;
            m.cr() = from_rgb(c);
            m.kr() = g.scale;
            m.ior() = from_rgb(ior);
            m.absorption() = from_rgb(ab);
            dst = m;
        }
        else if (g.kind == GBRT_MATERIAL_GLASS)
        {
            glass<float> m;
            m.ct() = from_rgb(c);
            m.kt() = g.scale;
            m.cr() = from_rgb(c2);
            m.kr() = g.scale2;
            m.ior() = from_rgb(ior);
            dst = m;
        }
        else if (g.kind == GBRT_MATERIAL_PLASTIC)
        {
            plastic<float> m;
            m.ca() = from_rgb(vec3(0.0f));
            m.ka() = 0.0f;
            m.cd() = from_rgb(c);
            m.kd() = g.scale;
            m.cs() = from_rgb(c2);
            m.ks() = g.scale2;
            m.specular_exp() = g.exponent;
            dst = m;
        }
        else
        {
            matte<float> m;
            m.ca() = from_rgb(vec3(0.0f));
            m.ka() = 0.0f;
            m.cd() = from_rgb(c);
            m.kd() = g.scale;
            dst = m;
        }
    }
    if (i < nl)
    {
        gbrt_light const& g = in_l[i];
        vec3 cl(g.cl[0], g.cl[1], g.cl[2]), pos(g.position[0], g.position[1], g.position[2]);
        auto& dst = static_cast<light_ext_t::base_type&>(lights[i]);
        if (g.kind == GBRT_LIGHT_POINT)
        {
            point_light<float> l;
            l.set_cl(cl);
            l.set_kl(g.kl);
            l.set_position(pos);
            l.set_constant_attenuation(g.attenuation[0]);
            l.set_linear_attenuation(g.attenuation[1]);
            l.set_quadratic_attenuation(g.attenuation[2]);
            dst = l;
        }
        else if (g.kind == GBRT_LIGHT_SPOT)
        {
            spot_light<float> l;
            l.set_cl(cl);
            l.set_kl(g.kl);
            l.set_position(pos);
            l.set_spot_direction(vec3(g.spot_direction[0], g.spot_direction[1], g.spot_direction[2]));
            l.set_spot_cutoff(g.spot_cutoff);
            l.set_spot_exponent(g.spot_exponent);
            l.set_constant_attenuation(g.attenuation[0]);
            l.set_linear_attenuation(g.attenuation[1]);
            l.set_quadratic_attenuation(g.attenuation[2]);
            dst = l;
        }
        else
        {
            area_light<float, triangle_t> l;
            memcpy(static_cast<void*>(&l.geometry()), &g.geometry, sizeof(triangle_t));
            l.set_cl(cl);
            l.set_kl(g.kl);
            dst = l;
        }
    }
}

struct camera_basis
{
    float eye[3], U[3], V[3], W[3];
};

// One frame: thread (x, y) runs the pixel's spp samples through pathtracing::kernel with
// the gbrt_rng.h stream (jitter x drawn before y), averages them and blends
// accum = avg * sfactor + accum * dfactor.
template <typename Mat, typename Light>
__device__ void pathtrace_pixel(const tree_ref_t* refs, const Mat* mats, const Light* lights, unsigned nl,
                                camera_basis const& cam, gbrt_pt_params const& p, float* accum)
{
    using kparams_t = kparams_of<Mat, Light>;
    unsigned x = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.width || y >= p.height) return;
    kparams_t kp;
    kp.prims.begin = refs;
    kp.prims.end = refs + 1;
    kp.geometric_normals = nullptr;
    kp.shading_normals = nullptr;
    kp.tex_coords = nullptr;
    kp.materials = mats;
    kp.colors = nullptr;
    kp.textures = nullptr;
    kp.lights.begin = lights;
    kp.lights.end = lights + nl;
    kp.num_bounces = p.num_bounces;
    kp.epsilon = p.epsilon;
    kp.background.set_cl(vec3(p.background[0], p.background[1], p.background[2]));
    kp.background.set_kl(p.background[3]);
    kp.amb_light.set_cl(vec3(p.ambient[0], p.ambient[1], p.ambient[2]));
    kp.amb_light.set_kl(1.0f);
    pathtracing::kernel<kparams_t> kernel;
    kernel.params = kp;

    const vec3 eye(cam.eye[0], cam.eye[1], cam.eye[2]);
    const vec3 U(cam.U[0], cam.U[1], cam.U[2]), V(cam.V[0], cam.V[1], cam.V[2]), W(cam.W[0], cam.W[1], cam.W[2]);
    const unsigned pix = y * p.width + x;
    vec4 sum(0.0f);
    for (unsigned s = 0; s < p.spp; ++s)
    {
        gbrt_sample_generator gen{ p.frame_id, pix, s, 0u };
        float jx = gen.next() - 0.5f;
        float jy = gen.next() - 0.5f;
        float sx = ((float(x) + jx) + 0.5f) / float(p.width);
        float sy = ((float(y) + jy) + 0.5f) / float(p.height);
        basic_ray<float> r;
        r.ori = eye;
        r.dir = normalize(U * (2.0f * sx - 1.0f) + V * (2.0f * sy - 1.0f) + W);
        r.tmin = 0.0f;
        r.tmax = FLT_MAX;
        auto res = kernel(r, gen);
        sum += res.color;
    }
    sum /= float(p.spp);
    float* a = accum + 4 * size_t(pix);
    vec4 dst = p.dfactor != 0.0f ? vec4(a[0], a[1], a[2], a[3]) : vec4(0.0f);
    vec4 out = sum * p.sfactor + dst * p.dfactor;
    a[0] = out.x;
    a[1] = out.y;
    a[2] = out.z;
    a[3] = out.w;
}

extern "C" __global__ void vsnray_ref_pathtrace(const tree_ref_t* refs, const mat_t* mats, const light_t* lights,
                                                unsigned nl, camera_basis cam, gbrt_pt_params p, float* accum)
{
    pathtrace_pixel(refs, mats, lights, nl, cam, p, accum);
}

extern "C" __global__ void vsnray_ref_pathtrace_ext(const tree_ref_t* refs, const mat_ext_t* mats,
                                                    const light_ext_t* lights, unsigned nl, camera_basis cam,
                                                    gbrt_pt_params p, float* accum)
{
    pathtrace_pixel(refs, mats, lights, nl, cam, p, accum);
}

// sizeof of the visionaray objects the host allocates arrays of: tree ref, material,
// light, and the GPU LBVH build's construction node, prim ref and box.
extern "C" __global__ void vsnray_ref_sizes(unsigned* out)
{
    out[0] = unsigned(sizeof(tree_ref_t));
    out[1] = unsigned(sizeof(mat_t));
    out[2] = unsigned(sizeof(light_t));
    out[3] = unsigned(sizeof(mat_ext_t));
    out[4] = unsigned(sizeof(light_ext_t));
    out[5] = unsigned(sizeof(detail::lbvh::node));
    out[6] = unsigned(sizeof(detail::lbvh::prim_ref));
    out[7] = unsigned(sizeof(aabb));
}

// visionaray's GPU LBVH build kernels (detail/bvh/lbvh.h:215-466), kept in this cubin
// so that oracle/ref_gpu.py can launch them in lbvh_builder::build's order
// (lbvh.h:681-844) and time the reference's GPU build beside the product's.  Taking
// their addresses instantiates them (the bounds kernel for the triangle type); they
// keep the reference's names, which the loader finds by enumerating the module.
void* vsnray_ref_lbvh_kernels[] = {
    reinterpret_cast<void*>(&detail::lbvh::compute_bounds_and_centroids<triangle_t>),
    reinterpret_cast<void*>(&detail::lbvh::assign_morton_codes),
    reinterpret_cast<void*>(&detail::lbvh::init_nodes),
    reinterpret_cast<void*>(&detail::lbvh::build_hierarchy),
    reinterpret_cast<void*>(&detail::lbvh::assign_node_bounds),
    reinterpret_cast<void*>(&detail::lbvh::collapse),
    reinterpret_cast<void*>(&detail::lbvh::sequence),
};
