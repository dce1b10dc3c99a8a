// Thin extern "C" driver around visionaray's own CPU code, compiled from the
// unmodified visionaray headers (see oracle/Makefile).  TEST INFRASTRUCTURE ONLY:
// it pins the oracle restatement (oracle.cpp) to the reference and generates the
// golden vectors in tests/golden.  Nothing in the product links it.
//
// Calls used: binned_sah_builder / lbvh_builder ::build (detail/bvh/sah.h:197-205,
// detail/bvh/lbvh.h:534-542), closest_hit / any_hit (detail/traverse_linear.inl:156-225)
// with a counting basic_intersector (intersector.h:24-87), detail::lbvh::determine_range
// (detail/bvh/lbvh.h:120-185) and sah_cost (detail/bvh/statistics.h:34-68).

#include <atomic>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include <visionaray/area_light.h>
#include <visionaray/environment_light.h>
#include <visionaray/texture/texture.h>
#include <visionaray/bvh.h>
#include <visionaray/generic_light.h>
#include <visionaray/generic_material.h>
#include <visionaray/kernels.h>
#include <visionaray/material.h>
#include <visionaray/math/math.h>
#include <visionaray/pinhole_camera.h>
#include <visionaray/point_light.h>
#include <visionaray/spot_light.h>
#include <visionaray/traverse.h>
#include <visionaray/detail/bvh/refit.h>
#include <visionaray/detail/bvh/statistics.h>

#include "../include/visionaray_gb300/gbrt_rng.h"
#include "oracle.h"

using namespace visionaray;

using triangle_t = basic_triangle<3, float, unsigned>;
static_assert(sizeof(triangle_t) == sizeof(gbrt_triangle), "triangle layout");
static_assert(sizeof(bvh_node) == sizeof(gbrt_bvh_node), "node layout");
static_assert(sizeof(basic_ray<float>) == sizeof(gbrt_ray), "ray layout");

namespace {

struct counting_intersector : basic_intersector<counting_intersector>
{
    using basic_intersector<counting_intersector>::operator();

    uint64_t boxes = 0;
    uint64_t tris = 0;

    template <typename R, typename T, typename V>
    hit_record<R, basic_aabb<T>> operator()(R const& ray, basic_aabb<T> const& box, V&& inv_dir)
    {
        ++boxes;
        return intersect(ray, box, inv_dir);
    }

    template <typename R>
    hit_record<R, primitive<unsigned>> operator()(R const& ray, triangle_t const& tri)
    {
        ++tris;
        return intersect(ray, tri);
    }
};

struct ref_tree
{
    std::vector<triangle_t> prims;
    index_bvh<triangle_t> tree;
};

std::vector<triangle_t> to_prims(const gbrt_triangle* tris, uint32_t n)
{
    std::vector<triangle_t> v(n);
    if (n) std::memcpy(v.data(), tris, size_t(n) * sizeof(triangle_t));
    return v;
}

} // namespace

extern "C" {

void* ref_build_sah(const gbrt_triangle* tris, uint32_t n, int max_leaf)
{
    auto* t = new ref_tree;
    t->prims = to_prims(tris, n);
    binned_sah_builder builder;
    t->tree = builder.build(index_bvh<triangle_t>{}, t->prims.data(), t->prims.size(), max_leaf);
    return t;
}

void* ref_build_lbvh_cpu(const gbrt_triangle* tris, uint32_t n, int max_leaf)
{
    auto* t = new ref_tree;
    t->prims = to_prims(tris, n);
    lbvh_builder builder;
    t->tree = builder.build(index_bvh<triangle_t>{}, t->prims.data(), t->prims.size(), max_leaf);
    return t;
}

uint32_t ref_num_nodes(void* h) { return uint32_t(static_cast<ref_tree*>(h)->tree.num_nodes()); }
uint32_t ref_num_indices(void* h) { return uint32_t(static_cast<ref_tree*>(h)->tree.num_indices()); }

void ref_copy(void* h, gbrt_bvh_node* nodes, uint32_t* indices)
{
    auto* t = static_cast<ref_tree*>(h);
    auto r = t->tree.ref();
    std::memcpy(nodes, r.nodes(), r.num_nodes() * sizeof(bvh_node));
    std::memcpy(indices, r.indices(), r.num_indices() * sizeof(unsigned));
}

void ref_free(void* h) { delete static_cast<ref_tree*>(h); }

// bvh_refitter::refit (detail/bvh/refit.h:25-117) of the tree to new positions of its
// n triangles (input order).
void ref_refit(void* h, const gbrt_triangle* tris, uint32_t n)
{
    auto* t = static_cast<ref_tree*>(h);
    t->prims = to_prims(tris, n);
    bvh_refitter refitter;
    refitter.refit(t->tree, t->prims.data(), t->prims.size());
}

float ref_sah_cost(void* h) { return sah_cost(static_cast<ref_tree*>(h)->tree); }

// Sorted (id, code) pairs of the CPU lbvh_builder::init (lbvh.h:544-599).
void ref_lbvh_sorted_refs(const gbrt_triangle* tris, uint32_t n, int32_t* ids, uint32_t* codes)
{
    auto prims = to_prims(tris, n);
    lbvh_builder builder;
    builder.init(prims.data(), prims.data() + n);
    for (uint32_t i = 0; i < n; ++i)
    {
        ids[i] = builder.prim_refs[i].id;
        codes[i] = builder.prim_refs[i].morton_code;
    }
}

// Karras children through the reference's own determine_range (lbvh.h:120-185) and
// the child rule of build_hierarchy (lbvh.h:300-328).
void ref_karras_children(const uint32_t* codes, uint32_t n, int32_t* left, int32_t* right)
{
    std::vector<detail::lbvh::prim_ref> refs(n);
    for (uint32_t i = 0; i < n; ++i)
    {
        refs[i].id = int(i);
        refs[i].morton_code = codes[i];
    }
    int num_inner = int(n) - 1;
    for (int i = 0; i < num_inner; ++i)
    {
        int split = -1;
        vec2i range = detail::lbvh::determine_range(refs.data(), int(n), i, split);
        left[i] = split == range.x ? num_inner + split : split;
        right[i] = split + 1 == range.y ? num_inner + split + 1 : split + 1;
    }
}

int ref_trace(void* h, const gbrt_ray* rays, uint64_t nrays, int any_hit_flag, int nthreads,
              gbrt_hit* hits, uint64_t* counters)
{
    auto* t = static_cast<ref_tree*>(h);
    auto bref = t->tree.ref();
    if (nthreads <= 0) nthreads = int(std::max(1u, std::thread::hardware_concurrency()));
    std::atomic<uint64_t> next{ 0 }, nbox{ 0 }, ntri{ 0 };
    const uint64_t chunk = 4096;
    auto worker = [&]() {
        counting_intersector isect;
        for (;;)
        {
            uint64_t b = next.fetch_add(chunk);
            if (b >= nrays) break;
            uint64_t e = std::min(nrays, b + chunk);
            for (uint64_t i = b; i < e; ++i)
            {
                basic_ray<float> r;
                std::memcpy(&r, &rays[i], sizeof(r));
                auto hr = any_hit_flag ? any_hit(r, &bref, &bref + 1, isect)
                                       : closest_hit(r, &bref, &bref + 1, isect);
                hits[i].prim_id = hr.hit ? hr.prim_id : GBRT_NO_HIT;
                hits[i].t = hr.t;
                hits[i].u = hr.u;
                hits[i].v = hr.v;
            }
        }
        nbox += isect.boxes;
        ntri += isect.tris;
    };
    if (t->tree.num_nodes() == 0)
    {
        for (uint64_t i = 0; i < nrays; ++i) hits[i] = { GBRT_NO_HIT, FLT_MAX, 0.0f, 0.0f };
    }
    else if (nthreads == 1)
    {
        worker();
    }
    else
    {
        std::vector<std::thread> pool;
        for (int i = 0; i < nthreads; ++i) pool.emplace_back(worker);
        for (auto& th : pool) th.join();
    }
    if (counters)
    {
        counters[0] = nbox.load();
        counters[1] = ntri.load();
    }
    return 0;
}

// Two-level instancing with visionaray's own types: a binned-SAH index_bvh per mesh,
// index_bvh_inst_t instances (bvh.h:678-782, via index_bvh::inst(transform),
// bvh.h:933-936) with set_inst_id(k), a binned-SAH top-level index_bvh over the
// instances, and closest_hit / any_hit through it (intersect.inl:362-394).
// mesh_tris[m] holds mesh_sizes[m] triangles; instance k uses mesh inst_mesh[k] and
// the mat4x3 columns transforms[12k .. 12k+11].
void ref_trace_instances(uint32_t num_meshes, const gbrt_triangle* const* mesh_tris, const uint32_t* mesh_sizes,
                         uint32_t num_instances, const uint32_t* inst_mesh, const float* transforms,
                         const gbrt_ray* rays, uint64_t nrays, int any_hit_flag, gbrt_hit_inst* hits)
{
    using blas_t = index_bvh<triangle_t>;
    using inst_t = blas_t::bvh_inst;
    std::vector<std::vector<triangle_t>> prims(num_meshes);
    std::vector<blas_t> blas(num_meshes);
    binned_sah_builder builder;
    for (uint32_t m = 0; m < num_meshes; ++m)
    {
        prims[m] = to_prims(mesh_tris[m], mesh_sizes[m]);
        blas[m] = builder.build(blas_t{}, prims[m].data(), prims[m].size());
    }
    std::vector<inst_t> insts;
    for (uint32_t k = 0; k < num_instances; ++k)
    {
        const float* t = transforms + 12 * size_t(k);
        mat4x3 xf(vec3(t[0], t[1], t[2]), vec3(t[3], t[4], t[5]), vec3(t[6], t[7], t[8]), vec3(t[9], t[10], t[11]));
        insts.push_back(blas[inst_mesh[k]].inst(xf));
        insts.back().set_inst_id(int(k));
    }
    index_bvh<inst_t> tlas = builder.build(index_bvh<inst_t>{}, insts.data(), insts.size());
    auto tref = tlas.ref();
    for (uint64_t i = 0; i < nrays; ++i)
    {
        basic_ray<float> r;
        std::memcpy(&r, &rays[i], sizeof(r));
        auto hr = any_hit_flag ? any_hit(r, &tref, &tref + 1) : closest_hit(r, &tref, &tref + 1);
        gbrt_hit_inst& h = hits[i];
        h.prim_id = hr.hit ? hr.prim_id : GBRT_NO_HIT;
        h.inst_id = hr.hit ? unsigned(hr.inst_id) : GBRT_NO_HIT;
        h.t = hr.t;
        h.u = hr.u;
        h.v = hr.v;
        h.geom_id = hr.hit ? hr.geom_id : 0u;
        h.reserved[0] = h.reserved[1] = 0u;
    }
}

// visionaray's pathtracing::kernel (detail/pathtracing.inl:42-233) over a binned-SAH
} // extern "C"

namespace {

// index_bvh, generic_material<matte, emissive, mirror, glass, plastic> per geom_id and the lights `al`,
// driven per (pixel, sample) by the gbrt_rng.h stream: the jittered primary ray
// (sched_common.h:209-233, jitter x drawn before y) through visionaray's own
// pinhole_camera, samples averaged and blended into accum as sample_pixel_impl does
// (sched_common.h:427-526).  accum is RGBA32F, read and written.
// kernel_params KP with its ambient light type replaced by Amb (kernels.h:20-66).
template <typename KP, typename Amb>
struct with_ambient;
template <typename NB, typename CB, typename P, typename N, typename TC, typename M, typename C, typename Tx,
          typename L, typename BG, typename A, typename Amb>
struct with_ambient<kernel_params<NB, CB, P, N, TC, M, C, Tx, L, BG, A>, Amb>
{
    using type = kernel_params<NB, CB, P, N, TC, M, C, Tx, L, BG, Amb>;
};

template <typename Light>
void render_reference(const gbrt_triangle* tris, uint32_t n, const gbrt_material* mats, uint32_t nmat,
                      std::vector<Light> const& al, const gbrt_camera* cam, const gbrt_pt_params* p, float* accum,
                      int nthreads, const gbrt_environment* env)
{
    using mat_t = generic_material<matte<float>, emissive<float>, mirror<float>, glass<float>, plastic<float>>;
    auto prims = to_prims(tris, n);
    binned_sah_builder builder;
    auto tree = builder.build(index_bvh<triangle_t>{}, prims.data(), prims.size());
    std::vector<decltype(tree.ref())> refs{ tree.ref() };

    std::vector<mat_t> materials(nmat);
    for (uint32_t i = 0; i < nmat; ++i)
    {
        vec3 c(mats[i].color[0], mats[i].color[1], mats[i].color[2]);
        if (mats[i].kind == GBRT_MATERIAL_EMISSIVE)
        {
            emissive<float> e;
            e.ce() = from_rgb(c);
            e.ls() = mats[i].scale;
            materials[i] = e;
        }
        else if (mats[i].kind == GBRT_MATERIAL_MIRROR)
        {
            mirror<float> m;
            m.cr() = from_rgb(c);
            m.kr() = mats[i].scale;
            m.ior() = from_rgb(vec3(mats[i].ior[0], mats[i].ior[1], mats[i].ior[2]));
            m.absorption() = from_rgb(vec3(mats[i].absorption[0], mats[i].absorption[1], mats[i].absorption[2]));
            materials[i] = m;
        }
        else if (mats[i].kind == GBRT_MATERIAL_GLASS)
        {
            glass<float> g;
            g.ct() = from_rgb(c);
            g.kt() = mats[i].scale;
            g.cr() = from_rgb(vec3(mats[i].color2[0], mats[i].color2[1], mats[i].color2[2]));
            g.kr() = mats[i].scale2;
            g.ior() = from_rgb(vec3(mats[i].ior[0], mats[i].ior[1], mats[i].ior[2]));
            materials[i] = g;
        }
        else if (mats[i].kind == GBRT_MATERIAL_PLASTIC)
        {
            plastic<float> pl;
            pl.ca() = from_rgb(vec3(0.0f));
            pl.ka() = 0.0f;
            pl.cd() = from_rgb(c);
            pl.kd() = mats[i].scale;
            pl.cs() = from_rgb(vec3(mats[i].color2[0], mats[i].color2[1], mats[i].color2[2]));
            pl.ks() = mats[i].scale2;
            pl.specular_exp() = mats[i].exponent;
            materials[i] = pl;
        }
        else
        {
            matte<float> m;
            m.ca() = from_rgb(vec3(0.0f));
            m.ka() = 0.0f;
            m.cd() = from_rgb(c);
            m.kd() = mats[i].scale;
            materials[i] = m;
        }
    }
    auto kp = make_kernel_params(refs.data(), refs.data() + 1, materials.data(), al.data(), al.data() + al.size(),
                                 p->num_bounces, p->epsilon,
                                 vec4(p->background[0], p->background[1], p->background[2], p->background[3]),
                                 vec4(p->ambient[0], p->ambient[1], p->ambient[2], 1.0f));

    pinhole_camera c;
    float fovy = cam->fovy_degrees * constants::degrees_to_radians<float>();
    c.perspective(fovy, float(p->width) / float(p->height), 0.001f, 1000.0f);
    c.look_at(vec3(cam->eye[0], cam->eye[1], cam->eye[2]), vec3(cam->center[0], cam->center[1], cam->center[2]),
              vec3(cam->up[0], cam->up[1], cam->up[2]));
    c.begin_frame();

    uint64_t npix = uint64_t(p->width) * p->height;
    if (nthreads <= 0) nthreads = int(std::max(1u, std::thread::hardware_concurrency()));
    auto run = [&](auto const& params) {
    pathtracing::kernel<std::decay_t<decltype(params)>> kernel;
    kernel.params = params;
    std::atomic<uint64_t> next{ 0 };
    auto worker = [&]() {
        for (;;)
        {
            uint64_t b = next.fetch_add(64);
            if (b >= npix) break;
            for (uint64_t pix = b; pix < std::min(npix, b + 64); ++pix)
            {
                int x = int(pix % p->width), y = int(pix / p->width);
                vec4 sum(0.0f);
                for (uint32_t s = 0; s < p->spp; ++s)
                {
                    gbrt_sample_generator gen{ p->frame_id, uint32_t(pix), s, 0u };
                    float jx = gen.next() - 0.5f;
                    float jy = gen.next() - 0.5f;
                    auto r = c.primary_ray(basic_ray<float>{}, float(x) + jx, float(y) + jy, float(p->width),
                                           float(p->height));
                    auto res = kernel(r, gen);
                    sum += res.color;
                }
                sum /= float(p->spp);
                float* a = accum + 4 * pix;
                vec4 dst(a[0], a[1], a[2], a[3]);
                vec4 out = sum * p->sfactor + dst * p->dfactor;
                a[0] = out.x;
                a[1] = out.y;
                a[2] = out.z;
                a[3] = out.w;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < nthreads; ++i) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
    };
    if (!env)
    {
        run(kp);
        return;
    }
    // environment_light<float, texture_ref<vec4, 2>> as the viewer sets it up
    // (src/viewer/viewer.cpp:1480-1492): a host texture, its modes, scale and transform
    texture<vec4, 2> tex(env->width, env->height);
    tex.reset(reinterpret_cast<vec4 const*>(env->d_texels));
    tex.set_address_mode(env->address == GBRT_ADDRESS_WRAP ? Wrap : (env->address == GBRT_ADDRESS_MIRROR ? Mirror : Clamp));
    tex.set_filter_mode(env->filter == GBRT_FILTER_NEAREST ? Nearest : Linear);
    environment_light<float, texture_ref<vec4, 2>> el;
    el.texture() = texture_ref<vec4, 2>(tex);
    el.scale() = from_rgb(vec3(env->scale[0], env->scale[1], env->scale[2]));
    const float* a = env->light_to_world;
    el.set_light_to_world_transform(mat4(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11],
                                         a[12], a[13], a[14], a[15]));
    typename with_ambient<decltype(kp), decltype(el)>::type kp2{
        { kp.prims.begin, kp.prims.end }, kp.geometric_normals, kp.shading_normals, kp.tex_coords, kp.materials,
        kp.colors, kp.textures, { kp.lights.begin, kp.lights.end }, kp.num_bounces, kp.epsilon, kp.background, el };
    run(kp2);
}


area_light<float, triangle_t> area_of(gbrt_light const& l)
{
    triangle_t g;
    std::memcpy(&g, &l.geometry, sizeof(g));
    area_light<float, triangle_t> a(g);
    a.set_cl(vec3(l.cl[0], l.cl[1], l.cl[2]));
    a.set_kl(l.kl);
    return a;
}

} // namespace

// Lights all area lights: area_light<float, basic_triangle> as the path-tracing
// configurations use; otherwise generic_light<area_light, point_light, spot_light>.
extern "C" void ref_pathtrace(const gbrt_triangle* tris, uint32_t n, const gbrt_material* mats, uint32_t nmat,
                              const gbrt_light* lights, uint32_t nl, const gbrt_camera* cam,
                              const gbrt_pt_params* p, float* accum, int nthreads, const gbrt_environment* env)
{
    bool all_area = true;
    for (uint32_t i = 0; i < nl; ++i) all_area = all_area && lights[i].kind == GBRT_LIGHT_AREA;
    if (all_area)
    {
        std::vector<area_light<float, triangle_t>> al;
        for (uint32_t i = 0; i < nl; ++i) al.push_back(area_of(lights[i]));
        render_reference(tris, n, mats, nmat, al, cam, p, accum, nthreads, env);
        return;
    }
    using light_t = generic_light<area_light<float, triangle_t>, point_light<float>, spot_light<float>>;
    std::vector<light_t> al;
    for (uint32_t i = 0; i < nl; ++i)
    {
        gbrt_light const& l = lights[i];
        vec3 cl(l.cl[0], l.cl[1], l.cl[2]), pos(l.position[0], l.position[1], l.position[2]);
        if (l.kind == GBRT_LIGHT_POINT)
        {
            point_light<float> pl;
            pl.set_cl(cl);
            pl.set_kl(l.kl);
            pl.set_position(pos);
            pl.set_constant_attenuation(l.attenuation[0]);
            pl.set_linear_attenuation(l.attenuation[1]);
            pl.set_quadratic_attenuation(l.attenuation[2]);
            al.push_back(pl);
        }
        else if (l.kind == GBRT_LIGHT_SPOT)
        {
            spot_light<float> sl;
            sl.set_cl(cl);
            sl.set_kl(l.kl);
            sl.set_position(pos);
            sl.set_spot_direction(vec3(l.spot_direction[0], l.spot_direction[1], l.spot_direction[2]));
            sl.set_spot_cutoff(l.spot_cutoff);
            sl.set_spot_exponent(l.spot_exponent);
            sl.set_constant_attenuation(l.attenuation[0]);
            sl.set_linear_attenuation(l.attenuation[1]);
            sl.set_quadratic_attenuation(l.attenuation[2]);
            al.push_back(sl);
        }
        else
        {
            al.push_back(area_of(l));
        }
    }
    render_reference(tris, n, mats, nmat, al, cam, p, accum, nthreads, env);
}

