// CPU restatement of visionaray's path tracer -- TEST INFRASTRUCTURE ONLY (see
// oracle.h).  One template, instantiated in float (to pin against the reference's own
// FP32 kernel at matched random numbers) and in double (the FP64 host oracle the CUDA
// path is checked against).  Build with -ffp-contract=off.
//
// Restates detail/pathtracing.inl:42-233 with, for the materials and lights the
// configurations use: matte + lambertian (detail/material/matte.inl:40-70,
// brdf.h:26-84), emissive (detail/material/emissive.inl:20-44), area_light on a
// triangle (detail/area_light.inl:27-53), mirror (detail/material/mirror.inl,
// specular_reflection at brdf.h:293-352, conductor Fresnel at fresnel.h:18-35), glass
// (detail/material/glass.inl, specular_transmission at brdf.h:360-469, dielectric
// Fresnel at fresnel.h:37-56), plastic (detail/material/plastic.inl, lambertian and
// blinn at brdf.h:26-84, 118-191), sample_random_light (sampling.h:195-213),
// cosine_sample_hemisphere (sampling.h:117-127), power_heuristic (sampling.h:73-79),
// sample_surface on a triangle (math/detail/triangle.inl:69-83), get_surface /
// get_normal / get_area (get_surface.h:129-160, get_normal.h:108-113,
// get_area.h:92-105), the pinhole camera (detail/pinhole_camera.inl:87-120) and the
// jittered-blend sampler (detail/sched_common.h:209-233, 427-526).

#include "oracle.h"

#include "../include/visionaray_gb300/gbrt_rng.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

template <typename T>
struct vec
{
    T x, y, z;
};

template <typename T> inline vec<T> operator+(vec<T> a, vec<T> b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
template <typename T> inline vec<T> operator-(vec<T> a, vec<T> b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
template <typename T> inline vec<T> operator-(vec<T> a) { return { -a.x, -a.y, -a.z }; }
template <typename T> inline vec<T> operator*(vec<T> a, vec<T> b) { return { a.x * b.x, a.y * b.y, a.z * b.z }; }
template <typename T> inline vec<T> operator*(vec<T> a, T s) { return { a.x * s, a.y * s, a.z * s }; }
template <typename T> inline vec<T> operator*(T s, vec<T> a) { return { s * a.x, s * a.y, s * a.z }; }
template <typename T> inline vec<T> operator/(vec<T> a, T s) { return { a.x / s, a.y / s, a.z / s }; }
template <typename T> inline T dot(vec<T> u, vec<T> v) { return u.x * v.x + u.y * v.y + u.z * v.z; }
template <typename T> inline vec<T> cross(vec<T> u, vec<T> v)
{
    return { u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x };
}
template <typename T> inline T length(vec<T> v) { return std::sqrt(dot(v, v)); }
// normalize(v) = v * rsqrt(dot(v, v)), rsqrt(x) = 1 / sqrt(x) on the host
// (math/detail/vector3.inl:332-335, math/detail/math.h:596-599)
template <typename T> inline vec<T> normalize(vec<T> v) { return v * (T(1.0) / std::sqrt(dot(v, v))); }
template <typename T> inline vec<T> faceforward(vec<T> n, vec<T> i, vec<T> nref)
{
    return dot(nref, i) < T(0.0) ? -n : n;   // math/detail/vector.inl:677-685
}
template <typename T> inline T max_element(vec<T> v)
{
    T m = v.x < v.y ? v.y : v.x;
    return m < v.z ? v.z : m;
}
template <typename T> inline T power_heuristic(T p1, T p2) { return (p1 * p1) / (p1 * p1 + p2 * p2); }

template <typename T> inline vec<T> load(const float* p) { return { T(p[0]), T(p[1]), T(p[2]) }; }

template <typename T>
struct tri_t
{
    vec<T> v1, e1, e2;
    uint32_t prim_id, geom_id;
};

template <typename T> inline tri_t<T> load_tri(gbrt_triangle const& t)
{
    return { load<T>(t.v1), load<T>(t.e1), load<T>(t.e2), t.prim_id, t.geom_id };
}

template <typename T>
struct hit_t
{
    bool hit = false;
    T t = T(FLT_MAX);
    uint32_t index = 0;   // primitive list index (position in the index list)
};

// math/intersect.h:176-229 in T
template <typename T>
inline bool intersect(vec<T> ori, vec<T> dir, tri_t<T> const& tri, T& t_out)
{
    vec<T> s1 = cross(dir, tri.e2);
    T div = dot(s1, tri.e1);
    if (!(div != T(0.0))) return false;
    T inv_div = T(1.0) / div;
    vec<T> d = ori - tri.v1;
    T b1 = dot(d, s1) * inv_div;
    if (!(b1 >= T(0.0) && b1 <= T(1.0))) return false;
    vec<T> s2 = cross(d, tri.e1);
    T b2 = dot(dir, s2) * inv_div;
    if (!(b2 >= T(0.0) && b1 + b2 <= T(1.0))) return false;
    t_out = dot(tri.e2, s2) * inv_div;
    return true;
}

template <typename T> inline T tmin_(T a, T b) { return a < b ? a : b; }
template <typename T> inline T tmax_(T a, T b) { return a < b ? b : a; }

struct scene_arrays
{
    const gbrt_triangle* tris;
    const gbrt_bvh_node* nodes;
    uint32_t num_nodes;
    const uint32_t* indices;
};

// detail/bvh/intersect.inl:51-165 (scalar ray, ordered by split axis and sign) in T.
template <typename T>
hit_t<T> traverse(scene_arrays const& s, vec<T> ori, vec<T> dir, T tmin, T tmax, bool any_hit, uint64_t& nbox,
                  uint64_t& ntri)
{
    hit_t<T> best;
    if (s.num_nodes == 0) return best;
    vec<T> inv = { dir.x != T(0) ? T(1) / dir.x : T(FLT_MAX), dir.y != T(0) ? T(1) / dir.y : T(FLT_MAX),
                   dir.z != T(0) ? T(1) / dir.z : T(FLT_MAX) };
    uint32_t st[64];
    int sp = 0;
    st[sp++] = 0;
    while (sp > 0)
    {
        gbrt_bvh_node const* nd = &s.nodes[st[--sp]];
        bool leaf = false;
        while (true)
        {
            vec<T> lo = load<T>(nd->bbox_min), hi = load<T>(nd->bbox_max);
            vec<T> t1 = (lo - ori) * inv, t2 = (hi - ori) * inv;
            T tn = tmax_(tmin_(t1.x, t2.x), tmax_(tmin_(t1.y, t2.y), tmin_(t1.z, t2.z)));
            T tf = tmin_(tmax_(t1.x, t2.x), tmin_(tmax_(t1.y, t2.y), tmax_(t1.z, t2.z)));
            ++nbox;
            if (!(tf >= tn && tn < best.t && tf >= tmin && tn <= tmax)) break;
            if (nd->num_prims != 0)
            {
                leaf = true;
                break;
            }
            T dc = nd->ordered_traversal_axis == 0 ? dir.x : (nd->ordered_traversal_axis == 1 ? dir.y : dir.z);
            float dcf = float(dc);
            uint32_t bits;
            std::memcpy(&bits, &dcf, 4);
            int32_t sign_rd = int32_t(bits) >> 31;
            uint32_t near_addr = (int32_t(nd->ordered_traversal_sign) ^ sign_rd) != 0 ? 1u : 0u;
            if (sp < 64) st[sp++] = nd->first_child_or_prim + (near_addr ? 0u : 1u);
            nd = &s.nodes[nd->first_child_or_prim + near_addr];
        }
        if (!leaf) continue;
        for (uint32_t i = nd->first_child_or_prim; i != nd->first_child_or_prim + nd->num_prims; ++i)
        {
            T t;
            ++ntri;
            if (!intersect(ori, dir, load_tri<T>(s.tris[s.indices[i]]), t)) continue;
            if (!(t < best.t && t >= tmin && t <= tmax)) continue;
            best.hit = true;
            best.t = t;
            best.index = i;
            if (any_hit) return best;
        }
    }
    return best;
}

struct pt_counters
{
    uint64_t closest = 0, shadow = 0, boxes = 0, tris = 0;
};

// Differentiable-renderer inputs (null: the materials' own colors) and the per-vertex
// record the adjoint sweeps backwards.
struct pt_params_ext
{
    const float* albedo = nullptr;
    const float* emission = nullptr;
    // cosine_sample_hemisphere(gen.next(), gen.next()) (sampling.h:117-127): the order
    // of the two draws is unspecified C++; visionaray's CPU build (g++) draws the second
    // argument first, its device build (nvcc) the first argument first
    bool draws_in_order = false;
    // environment_light in place of the ambient light (null: ambient); env_m = rows 0-2
    // of world_to_light
    const gbrt_environment* env = nullptr;
    float env_m[12] = {};
};

// Rows 0-2 of the inverse of the column-major 4x4 `a` by the reference's float cofactor
// expansion (math/detail/matrix4.inl:353-388; m(r, c) = a[4c + r], out[4r + c]).
void inverse_rows(const float a[16], float out[12])
{
    auto m = [&](int r, int c) { return a[4 * c + r]; };
    auto det2 = [](float m00, float m01, float m10, float m11) { return m00 * m11 - m10 * m01; };
    float s0 = det2(m(0, 0), m(0, 1), m(1, 0), m(1, 1)), s1 = det2(m(0, 0), m(0, 2), m(1, 0), m(1, 2));
    float s2 = det2(m(0, 0), m(0, 3), m(1, 0), m(1, 3)), s3 = det2(m(0, 1), m(0, 2), m(1, 1), m(1, 2));
    float s4 = det2(m(0, 1), m(0, 3), m(1, 1), m(1, 3)), s5 = det2(m(0, 2), m(0, 3), m(1, 2), m(1, 3));
    float c5 = det2(m(2, 2), m(2, 3), m(3, 2), m(3, 3)), c4 = det2(m(2, 1), m(2, 3), m(3, 1), m(3, 3));
    float c3 = det2(m(2, 1), m(2, 2), m(3, 1), m(3, 2)), c2 = det2(m(2, 0), m(2, 3), m(3, 0), m(3, 3));
    float c1 = det2(m(2, 0), m(2, 2), m(3, 0), m(3, 2)), c0 = det2(m(2, 0), m(2, 1), m(3, 0), m(3, 1));
    float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    out[0] = (+m(1, 1) * c5 - m(1, 2) * c4 + m(1, 3) * c3) / det;
    out[4] = (-m(1, 0) * c5 + m(1, 2) * c2 + m(1, 3) * c1) / det;
    out[8] = (+m(1, 0) * c4 - m(1, 1) * c2 + m(1, 3) * c0) / det;
    out[1] = (-m(0, 1) * c5 + m(0, 2) * c4 - m(0, 3) * c3) / det;
    out[5] = (+m(0, 0) * c5 - m(0, 2) * c2 + m(0, 3) * c1) / det;
    out[9] = (-m(0, 0) * c4 + m(0, 1) * c2 - m(0, 3) * c0) / det;
    out[2] = (+m(3, 1) * s5 - m(3, 2) * s4 + m(3, 3) * s3) / det;
    out[6] = (-m(3, 0) * s5 + m(3, 2) * s2 - m(3, 3) * s1) / det;
    out[10] = (+m(3, 0) * s4 - m(3, 1) * s2 + m(3, 3) * s0) / det;
    out[3] = (-m(2, 1) * s5 + m(2, 2) * s4 - m(2, 3) * s3) / det;
    out[7] = (+m(2, 0) * s5 - m(2, 2) * s2 + m(2, 3) * s1) / det;
    out[11] = (-m(2, 0) * s4 + m(2, 1) * s2 - m(2, 3) * s0) / det;
}

// remap_texture_coordinate (texture/detail/texture_common.h:91-126) for one axis of n
// texels; clamp(x, a, b) = max(a, min(x, b)) (math/detail/math.h:530-533).
template <typename T>
T tex_remap(T c, uint32_t n, uint32_t address)
{
    const T fn = T(int(n));
    if (address == GBRT_ADDRESS_WRAP) return c - std::floor(c);
    if (address == GBRT_ADDRESS_MIRROR)
    {
        T f = std::floor(c);
        return (int(f) & 1) == 1 ? T(int(n) - 1) / fn - (c - f) : c - f;
    }
    T lo = c < T(1.0) - T(1.0) / fn ? c : T(1.0) - T(1.0) / fn;
    return T(0.0) < lo ? lo : T(0.0);
}

// convert_to_int of coord * size; an index outside the texture (the reference reads out
// of bounds there) is clamped to the edge.
template <typename T>
int tex_index(T c, uint32_t n)
{
    T x = c * T(int(n));
    int i = x != x ? 0 : (x >= T(2147483647.0) ? int(n) - 1 : (x <= T(-2147483648.0) ? 0 : int(x)));
    return std::min(std::max(i, 0), int(n) - 1);
}

// environment_light::intensity (detail/environment_light.inl:18-34) with tex2D's CPU
// nearest / linear filter (texture/detail/filter/nearest.h:44-66, linear.h:56-96;
// lerp_r(a, b, x) = (1 - x) a + x b, math/detail/math.h:550-555), in T.
template <typename T>
vec<T> env_intensity(pt_params_ext const& ext, vec<T> dir)
{
    gbrt_environment const& e = *ext.env;
    const float* m = ext.env_m;
    const T two_pi = T(6.28318530717958647692528676656e+00);
    const T inv_pi = T(3.18309886183790691216444201928e-01);
    T dx = T(m[0]) * dir.x + T(m[1]) * dir.y + T(m[2]) * dir.z + T(m[3]) * T(0.0);
    T dy = T(m[4]) * dir.x + T(m[5]) * dir.y + T(m[6]) * dir.z + T(m[7]) * T(0.0);
    T dz = T(m[8]) * dir.x + T(m[9]) * dir.y + T(m[10]) * dir.z + T(m[11]) * T(0.0);
    T x = std::atan2(dx, dz);
    x = x < T(0.0) ? x + two_pi : x;
    T y = std::acos(dy);
    T u = x / two_pi, v = y * inv_pi;
    auto texel = [&](int ix, int iy) {
        const float* t = e.d_texels + 4 * (size_t(iy) * e.width + size_t(ix));
        return vec<T>{ T(t[0]), T(t[1]), T(t[2]) };
    };
    vec<T> c;
    if (e.filter == GBRT_FILTER_NEAREST)
    {
        c = texel(tex_index(tex_remap(u, e.width, e.address), e.width),
                  tex_index(tex_remap(v, e.height, e.address), e.height));
    }
    else
    {
        const T fw = T(int(e.width)), fh = T(int(e.height));
        T c1x = tex_remap(u - T(0.5) / fw, e.width, e.address), c1y = tex_remap(v - T(0.5) / fh, e.height, e.address);
        T c2x = tex_remap(u + T(0.5) / fw, e.width, e.address), c2y = tex_remap(v + T(0.5) / fh, e.height, e.address);
        int lx = tex_index(c1x, e.width), ly = tex_index(c1y, e.height);
        int hx = tex_index(c2x, e.width), hy = tex_index(c2y, e.height);
        T ux = c1x * fw - T(lx), uy = c1y * fh - T(ly);
        auto lerp = [](vec<T> a, vec<T> b, T t) { return (T(1.0) - t) * a + t * b; };
        c = lerp(lerp(texel(lx, ly), texel(hx, ly), ux), lerp(texel(lx, hy), texel(hx, hy), ux), uy);
    }
    return { c.x * T(e.scale[0]), c.y * T(e.scale[1]), c.z * T(e.scale[2]) };
}

enum : uint32_t
{
    kMiss = 0,
    kEmission = 1,
    kMatte = 2,
    kEnd = 3,
    kSpecular = 4,
    kPlastic = 5,
};

template <typename T>
struct vrec
{
    uint32_t kind = kMiss, geom = 0, lgeom = 0xFFFFFFFFu, nee = 0;
    vec<T> thr{ 0, 0, 0 };
    T sigma = 0, mis = 0, escale = 0, kfac = 0, w = 0, x = 0, b0 = 0, kl = 0, rr = 0;
    vec<T> lint{ 0, 0, 0 };
    vec<T> spec{ 0, 0, 0 };   // a specular or plastic vertex's throughput factor src * cos / pdf
    vec<T> gnee{ 0, 0, 0 };   // plastic next-event contribution = w * thr * gnee * lint
};

// pathtracing::kernel::operator() (detail/pathtracing.inl:42-233) for one camera ray.
template <typename T>
inline T trig_cos(T x, bool via_double) { return via_double ? T(std::cos(double(x))) : std::cos(x); }
template <typename T>
inline T trig_sin(T x, bool via_double) { return via_double ? T(std::sin(double(x))) : std::sin(x); }

template <typename T>
inline T trig_pow(T x, T y, bool via_double) { return via_double ? T(std::pow(double(x), double(y))) : std::pow(x, y); }

// blinn::f (brdf.h:128-141) in T
template <typename T>
vec<T> blinn_f(gbrt_material const& m, vec<T> n, vec<T> wo, vec<T> wi, bool trig_double)
{
    const T pi = T(3.14159265358979323846264338328e+00);
    vec<T> h = normalize(wo + wi);
    T hdotn = std::max(T(0.0), dot(h, n));
    T sat = std::max(T(0.0), std::min(dot(wi, h), T(1.0)));
    T fr = trig_pow(T(1.0) - sat, T(5.0), trig_double);
    T nfactor = (T(m.exponent) + T(2.0)) / (T(8.0) * pi);
    T lobe = trig_pow(hdotn, T(m.exponent), trig_double);
    T out[3];
    for (int c = 0; c < 3; ++c)
    {
        T spec = T(m.color2[c]) * T(m.scale2);
        T schlick = spec + (T(1.0) - spec) * fr;
        out[c] = (schlick * nfactor) * lobe;
    }
    return { out[0], out[1], out[2] };
}

// blinn::pdf (brdf.h:182-190) in T
template <typename T>
T blinn_pdf(gbrt_material const& m, vec<T> n, vec<T> wo, vec<T> wi, bool trig_double)
{
    const T pi = T(3.14159265358979323846264338328e+00);
    vec<T> h = normalize(wi + wo);
    T costheta = dot(n, h);
    T vdoth = dot(wo, h);
    return ((T(m.exponent) + T(1.0)) * trig_pow(costheta, T(m.exponent), trig_double)) /
           (T(2.0) * pi * T(4.0) * vdoth);
}

template <typename T>
vec<T> radiance(scene_arrays const& s, gbrt_material const* mats, uint32_t nmat, gbrt_light const* lights,
                uint32_t nl, gbrt_pt_params const& p, vec<T> ori, vec<T> dir, T tmin, T tmax,
                gbrt_sample_generator& gen, bool& first_hit, pt_counters& cnt, bool trig_double,
                pt_params_ext const& ext = {}, vrec<T>* recs = nullptr, int* nrec = nullptr)
{
    if (nrec) *nrec = 0;
    const T inv_pi = T(3.18309886183790691216444201928e-01);
    const T pi = T(3.14159265358979323846264338328e+00);
    const T two_pi = T(6.28318530717958623199592693709e+00);
    const T eps = T(p.epsilon);
    vec<T> intensity = { 0, 0, 0 };
    vec<T> throughput = { 1, 1, 1 };
    bool active = true;
    bool last_specular = true;
    const vec<T> ambient = { T(p.ambient[0]), T(p.ambient[1]), T(p.ambient[2]) };
    first_hit = false;

    for (uint32_t bounce = 0; bounce < p.num_bounces; ++bounce)
    {
        hit_t<T> hr = traverse(s, ori, dir, tmin, tmax, false, cnt.boxes, cnt.tris);
        ++cnt.closest;
        vrec<T> rec;
        rec.thr = throughput;
        if (active && !hr.hit)
        {
            rec.spec = ext.env ? env_intensity<T>(ext, dir) : ambient;
            intensity = intensity + rec.spec * throughput;
        }
        active = active && hr.hit;
        if (!active)
        {
            if (recs && *nrec < 16) recs[(*nrec)++] = rec;
            break;
        }
        if (bounce == 0) first_hit = true;

        tri_t<T> tri = load_tri<T>(s.tris[s.indices[hr.index]]);
        vec<T> view_dir = -dir;
        vec<T> isect = ori + dir * hr.t;
        vec<T> gn = normalize(cross(tri.e1, tri.e2));
        vec<T> sn = gn;
        uint32_t geom = tri.geom_id < nmat ? tri.geom_id : 0u;
        gbrt_material m = tri.geom_id < nmat ? mats[tri.geom_id] : gbrt_material{ GBRT_MATERIAL_MATTE, { 0, 0, 0 }, 0 };
        vec<T> mcol = { T(m.color[0]), T(m.color[1]), T(m.color[2]) };
        bool emission = m.kind == GBRT_MATERIAL_EMISSIVE;
        const bool mirror = m.kind == GBRT_MATERIAL_MIRROR, glass = m.kind == GBRT_MATERIAL_GLASS;
        const bool plastic = m.kind == GBRT_MATERIAL_PLASTIC;
        const bool specular = mirror || glass;
        bool glossy = false;
        if (!emission && !specular && !plastic && ext.albedo) mcol = load<T>(ext.albedo + 3 * geom);
        if (emission && ext.emission) mcol = load<T>(ext.emission + 3 * geom);
        rec.geom = geom;

        // surf.sample(view_dir, refl_dir, brdf_pdf, inter, gen)
        vec<T> refl = { 0, 0, 0 };
        T brdf_pdf;
        vec<T> src;
        if (mirror)
        {
            // specular_reflection::sample_f (brdf.h:317-340) with the conductor Fresnel
            // term (fresnel.h:18-35), on the unflipped shading normal
            vec<T> wo = view_dir;
            refl = T(2.0) * dot(sn, wo) * sn - wo;
            brdf_pdf = T(1.0);
            T cosi = std::abs(dot(sn, wo));
            T f[3];
            for (int c = 0; c < 3; ++c)
            {
                T eta = T(m.ior[c]), k = T(m.absorption[c]);
                T rs2 = ((eta * eta + k * k) - T(2.0) * eta * cosi + cosi * cosi) /
                        ((eta * eta + k * k) + T(2.0) * eta * cosi + cosi * cosi);
                T rp2 = ((eta * eta + k * k) * cosi * cosi - T(2.0) * eta * cosi + T(1.0)) /
                        ((eta * eta + k * k) * cosi * cosi + T(2.0) * eta * cosi + T(1.0));
                f[c] = ((rs2 + rp2) / T(2.0)) * (T(m.color[c]) * T(m.scale));
            }
            T dn = std::abs(dot(sn, refl));
            src = { f[0] / dn, f[1] / dn, f[2] / dn };
        }
        else if (glass)
        {
            // specular_transmission::sample_f (brdf.h:385-456), dielectric Fresnel term
            // (fresnel.h:37-56) evaluated with (ior1, ior2) as the reference passes them
            vec<T> wo = view_dir;
            T cosi = dot(sn, wo);
            cosi = cosi < T(1.0) ? cosi : T(1.0);
            cosi = T(-1.0) < cosi ? cosi : T(-1.0);
            bool entering = cosi > T(0.0);
            vec<T> N = entering ? sn : -sn;
            const T ior1[3] = { T(1.0), T(1.0), T(1.0) };
            const T ior2[3] = { T(m.ior[0]), T(m.ior[1]), T(m.ior[2]) };
            T etai0 = entering ? ior1[0] : ior2[0], etat0 = entering ? ior2[0] : ior1[0];
            if (!entering) cosi = std::abs(cosi);
            T eta = etai0 / etat0;
            T sini = std::sqrt(std::max(T(0.0), T(1.0) - cosi * cosi));
            T sint = eta * sini;
            T cost = std::sqrt(std::max(T(0.0), T(1.0) - sint * sint));
            T R[3];
            for (int c = 0; c < 3; ++c)
            {
                T rs = (ior1[c] * cosi - ior2[c] * cost) / (ior1[c] * cosi + ior2[c] * cost);
                T rp = (ior2[c] * cosi - ior1[c] * cost) / (ior2[c] * cosi + ior1[c] * cost);
                R[c] = (rs * rs + rp * rp) / T(2.0);
            }
            if (sint >= T(1.0)) R[0] = R[1] = R[2] = T(1.0);
            // refract(wo, N, eta) (vector.inl:695-707) and reflect(wo, N)
            T rc = dot(N, wo);
            T rsin = std::max(T(0.0), T(1.0) - rc * rc);
            T rsint = eta * eta * rsin;
            vec<T> refracted = rsint >= T(1.0) ? vec<T>{ 0, 0, 0 } : eta * -wo + (eta * rc - std::sqrt(T(1.0) - rsint)) * N;
            vec<T> reflected = T(2.0) * dot(N, wo) * N - wo;
            T u = T(gen.next());
            T val[3];
            if (u < R[0])
            {
                refl = reflected;
                brdf_pdf = R[0];
                for (int c = 0; c < 3; ++c) val[c] = R[c] * (T(m.color2[c]) * T(m.scale2));
            }
            else
            {
                refl = normalize(refracted);
                brdf_pdf = T(1.0) - R[0];
                for (int c = 0; c < 3; ++c) val[c] = (T(1.0) - R[c]) * (T(m.color[c]) * T(m.scale));
            }
            T dn = dot(N, refl);
            src = { val[0] / dn, val[1] / dn, val[2] / dn };
        }
        else if (plastic)
        {
            // plastic::sample (detail/material/plastic.inl:42-95): the lobe drawn by the
            // mean reflectances, whose own pdf is returned (no selection probability)
            T prob_diff = ((T(m.color[0]) + T(m.color[1])) + T(m.color[2])) / T(3.0) * T(m.scale);
            T prob_spec = ((T(m.color2[0]) + T(m.color2[1])) + T(m.color2[2])) / T(3.0) * T(m.scale2);
            bool all_zero = prob_diff == T(0.0) && prob_spec == T(0.0);
            prob_diff = all_zero ? T(0.5) : prob_diff;
            prob_spec = all_zero ? T(0.5) : prob_spec;
            prob_diff = prob_diff / (prob_diff + prob_spec);
            T u = T(gen.next());
            vec<T> n = faceforward(sn, view_dir, gn);
            vec<T> w = n;
            vec<T> v = std::abs(w.x) > std::abs(w.y) ? normalize(vec<T>{ -w.z, T(0), w.x })
                                                     : normalize(vec<T>{ T(0), w.z, -w.y });
            vec<T> uu = cross(v, w);
            if (u < prob_diff)
            {
                T u1, u2;
                if (ext.draws_in_order)
                {
                    u1 = T(gen.next());
                    u2 = T(gen.next());
                }
                else
                {
                    u2 = T(gen.next());
                    u1 = T(gen.next());
                }
                T r = std::sqrt(u1);
                T theta = two_pi * u2;
                vec<T> sp = { r * trig_cos(theta, trig_double), r * trig_sin(theta, trig_double),
                              std::sqrt(T(1.0) - u1) };
                refl = normalize(uu * sp.x + v * sp.y + w * sp.z);
                brdf_pdf = dot(n, refl) * inv_pi;
                src = (mcol * T(m.scale)) * inv_pi;
            }
            else
            {
                // blinn::sample_f (brdf.h:143-180)
                T u1 = T(gen.next());
                T u2 = T(gen.next());
                T costheta = trig_pow(u1, T(1.0) / (T(m.exponent) + T(1.0)), trig_double);
                T sintheta = std::sqrt(std::max(T(0.0), T(1.0) - costheta * costheta));
                T phi = u2 * two_pi;
                vec<T> h = normalize(sintheta * trig_cos(phi, trig_double) * uu +
                                     sintheta * trig_sin(phi, trig_double) * v + costheta * w);
                refl = T(2.0) * dot(h, view_dir) * h - view_dir;
                T vdoth = dot(view_dir, h);
                brdf_pdf = ((T(m.exponent) + T(1.0)) * trig_pow(costheta, T(m.exponent), trig_double)) /
                           (T(2.0) * pi * T(4.0) * vdoth);
                src = blinn_f(m, n, view_dir, refl, trig_double);
                glossy = true;
            }
        }
        else if (!emission)
        {
            vec<T> n = faceforward(sn, view_dir, gn);
            vec<T> w = n;
            vec<T> v = std::abs(w.x) > std::abs(w.y) ? normalize(vec<T>{ -w.z, T(0), w.x })
                                                     : normalize(vec<T>{ T(0), w.z, -w.y });
            vec<T> u = cross(v, w);
            // cosine_sample_hemisphere(gen.next(), gen.next()): the reference build
            // evaluates the second argument first
            T u1, u2;
            if (ext.draws_in_order)
            {
                u1 = T(gen.next());
                u2 = T(gen.next());
            }
            else
            {
                u2 = T(gen.next());
                u1 = T(gen.next());
            }
            T r = std::sqrt(u1);
            T theta = two_pi * u2;
            vec<T> sp = { r * trig_cos(theta, trig_double), r * trig_sin(theta, trig_double),
                          std::sqrt(T(1.0) - u1) };
            refl = normalize(u * sp.x + v * sp.y + w * sp.z);
            brdf_pdf = dot(n, refl) * inv_pi;
            src = (mcol * T(m.scale)) * inv_pi;
        }
        else
        {
            brdf_pdf = T(1.0);
            src = mcol * T(m.scale);
        }
        bool zero_pdf = brdf_pdf <= T(0.0);

        T light_pdf = T(0.0);
        if (nl > 0 && emission)
        {
            T A = T(0.5) * length(cross(tri.e1, tri.e2));
            T ld = length(isect - ori);
            vec<T> L = normalize(isect - ori);
            T ldotln = std::abs(dot(-L, gn));
            T solid_angle = (ldotln * A) / (ld * ld);
            light_pdf = T(1.0) / solid_angle;
        }
        T mis = (bounce > 0 && nl > 0 && !last_specular) ? power_heuristic(brdf_pdf, light_pdf / T(float(nl)))
                                                          : T(1.0);
        if (active && emission) intensity = intensity + (throughput * mis) * src;
        active = active && !emission && !zero_pdf;
        rec.kind = emission ? kEmission : (zero_pdf ? kEnd : (specular ? kSpecular : (plastic ? kPlastic : kMatte)));
        rec.mis = mis;
        rec.escale = T(m.scale);

        vec<T> n = faceforward(sn, view_dir, gn);
        if (nl > 0)
        {
            // sample_random_light (sampling.h:195-213) + the light's sample
            T ul = T(gen.next());
            int light_id = static_cast<int>(float(ul) * float(nl));
            if (light_id >= int(nl)) light_id = int(nl) - 1;
            gbrt_light const& lsrc = lights[light_id];
            vec<T> ldir, lint, L, ln;
            T dist, lpdf;
            uint32_t lgeom = 0xFFFFFFFFu;
            if (lsrc.kind == GBRT_LIGHT_AREA)
            {
                // area_light::sample + sample_surface (area_light.inl:27-53, triangle.inl:69-83)
                tri_t<T> lt = load_tri<T>(lsrc.geometry);
                T s1 = T(gen.next());
                T s2 = T(gen.next());
                vec<T> lv1 = lt.v1, lv2 = lt.v1 + lt.e1, lv3 = lt.v1 + lt.e2;
                T sq = std::sqrt(s1);
                vec<T> pos = lv1 * (T(1.0) - sq) + lv2 * sq * (T(1.0) - s2) + lv3 * sq * s2;
                ldir = pos - isect;
                dist = length(ldir);
                lint = { T(lsrc.cl[0]) * T(lsrc.kl), T(lsrc.cl[1]) * T(lsrc.kl), T(lsrc.cl[2]) * T(lsrc.kl) };
                lgeom = lsrc.geometry.geom_id;
                if (ext.emission && lgeom < nmat) lint = load<T>(ext.emission + 3 * lgeom) * T(lsrc.kl);
                vec<T> lnormal = normalize(cross(lt.e1, lt.e2));
                T larea = T(0.5) * length(cross(lt.e1, lt.e2));
                T ldotln0 = std::abs(dot(-normalize(ldir), lnormal));
                T solid_angle = (ldotln0 * larea) / (dist * dist);
                lpdf = T(1.0) / solid_angle;
                L = normalize(ldir);
                ln = faceforward(lnormal, -L, lnormal);
                if (!ext.emission) lgeom = 0xFFFFFFFFu;
            }
            else
            {
                // point_light::sample / spot_light::sample (point_light.inl:16-56,
                // spot_light.inl:14-62): intensity(pos) * pi at pos = the light's own
                // position, three draws for an unused normal, a delta light of pdf 1
                vec<T> pos = load<T>(lsrc.position);
                ldir = pos - isect;
                dist = length(ldir);
                vec<T> dd = pos - pos;
                T d = length(dd);
                T att = T(1.0 / (T(lsrc.attenuation[0]) + T(lsrc.attenuation[1]) * d + T(lsrc.attenuation[2]) * d * d));
                vec<T> in = vec<T>{ T(lsrc.cl[0]) * T(lsrc.kl), T(lsrc.cl[1]) * T(lsrc.kl), T(lsrc.cl[2]) * T(lsrc.kl) } * att;
                if (lsrc.kind == GBRT_LIGHT_SPOT)
                {
                    T c = dot(load<T>(lsrc.spot_direction), normalize(-dd));
                    T spot = c > T(std::cos(lsrc.spot_cutoff)) ? std::pow(c, T(lsrc.spot_exponent)) : T(0.0);
                    in = in * spot;
                }
                lint = in * pi;
                gen.next();
                gen.next();
                gen.next();
                lpdf = T(1.0);
                L = normalize(ldir);
                ln = faceforward(-L, -L, -L);
            }
            T ldotn = dot(L, n);
            T ldotln = std::abs(dot(-L, ln));
            // shadow ray (pathtracing.inl:171-176); GBRT_PT_SHADOW_RANGE_FIX ends it one
            // more epsilon before the light sample
            T shadow_tmax = (p.flags & GBRT_PT_SHADOW_RANGE_FIX) ? dist - eps - eps : dist - eps;
            hit_t<T> sh = traverse(s, isect + L * eps, L, eps, shadow_tmax, true, cnt.boxes, cnt.tris);
            ++cnt.shadow;
            // a specular surface's shade() is 0 (brdf.h:306-315, 374-383): no contribution
            if (!emission && !specular)
            {
                vec<T> n2 = faceforward(sn, view_dir, gn);
                // surf.pdf(view, L, inter): the lobe the sample chose (plastic.inl:97-110)
                T bpdf = glossy ? blinn_pdf(m, n2, view_dir, L, trig_double) : dot(n2, L) * inv_pi;
                T b0 = bpdf;
                T prob = max_element(throughput);
                bpdf = bpdf * prob;
                T ndotl = std::max(T(0.0), dot(n2, L));
                vec<T> cd = (mcol * T(m.scale)) * inv_pi;
                // plastic::shade (plastic.inl:20-39): (diffuse + Blinn) * pi * intensity * n.l
                vec<T> brdf = plastic ? cd + blinn_f(m, n2, view_dir, L, trig_double) : cd;
                vec<T> shade = ((brdf * pi) * lint) * ndotl;
                vec<T> src2 = (shade * inv_pi) / ldotn;
                T mis2 = power_heuristic(lpdf / T(float(nl)), bpdf);
                if (active && !sh.hit && ldotn > T(0.0) && ldotln > T(0.0))
                {
                    intensity = intensity + (((throughput * mis2) * src2) * (ldotn / lpdf)) * T(float(nl));
                    rec.nee = 1;
                    rec.lgeom = lgeom;
                    rec.kl = T(lsrc.kl);
                    rec.lint = lint;
                    rec.w = mis2;
                    rec.x = lpdf / T(float(nl));
                    rec.b0 = b0;
                    rec.kfac = T(m.scale) * inv_pi * pi * ndotl * inv_pi / ldotn * (ldotn / lpdf) * T(float(nl));
                    rec.gnee = brdf * (pi * ndotl * inv_pi / ldotn * (ldotn / lpdf) * T(float(nl)));
                }
            }
        }

        rec.spec = src * (dot(n, refl) / brdf_pdf);
        throughput = throughput * (src * (dot(n, refl) / brdf_pdf));
        if (zero_pdf) throughput = { 0, 0, 0 };
        rec.sigma = T(m.scale) * inv_pi * (dot(n, refl) / brdf_pdf);

        if (bounce >= 2 && !(p.flags & GBRT_PT_NO_RUSSIAN_ROULETTE))
        {
            T prob = max_element(throughput);
            bool terminate = T(gen.next()) > prob;
            active = active && !terminate;
            throughput = throughput / prob;
            rec.rr = prob;
            if (recs && *nrec < 16) recs[(*nrec)++] = rec;
            if (!active) break;
        }
        else if (recs && *nrec < 16)
        {
            recs[(*nrec)++] = rec;
        }
        if (!active) break;   // emission / zero pdf: nothing further reaches the image
        ori = isect + refl * eps;
        dir = refl;
        last_specular = specular;
    }
    return intensity;
}

template <typename T>
void render(scene_arrays const& s, gbrt_material const* mats, uint32_t nmat, gbrt_light const* lights,
            uint32_t nl, gbrt_camera const& cam, gbrt_pt_params const& p, int nthreads, double* out,
            pt_counters& total, bool trig_double, pt_params_ext const& ext = {}, const uint32_t* plist = nullptr,
            uint64_t nlist = 0)
{
    // plist: render only these pixels (row-major indices), out[4 k ...] for plist[k]
    // pinhole_camera::begin_frame (detail/pinhole_camera.inl:87-97) in T
    vec<T> eye = load<T>(cam.eye), center = load<T>(cam.center), up = load<T>(cam.up);
    vec<T> f = normalize(eye - center);
    vec<T> sv = normalize(cross(up, f));
    vec<T> uv = cross(f, sv);
    T fovy = T(cam.fovy_degrees) * T(1.74532925199432957692369076849e-02);
    T aspect = T(p.width) / T(p.height);
    T th = std::tan(fovy / T(2.0));
    vec<T> U = sv * th * aspect;
    vec<T> V = uv * th;
    vec<T> W = -f;

    uint64_t npix = plist ? nlist : uint64_t(p.width) * p.height;
    if (nthreads <= 0) nthreads = int(std::max(1u, std::thread::hardware_concurrency()));
    std::atomic<uint64_t> next{ 0 };
    std::vector<pt_counters> per(static_cast<size_t>(nthreads));
    auto worker = [&](int tid) {
        for (;;)
        {
            uint64_t b = next.fetch_add(plist ? 1 : 64);
            if (b >= npix) break;
            for (uint64_t k = b; k < std::min(npix, b + (plist ? 1 : 64)); ++k)
            {
                uint64_t pix = plist ? plist[k] : k;
                T x = T(pix % p.width), y = T(pix / p.width);
                vec<T> sum = { 0, 0, 0 };
                T alpha = 0;
                for (uint32_t smp = 0; smp < p.spp; ++smp)
                {
                    gbrt_sample_generator gen{ p.frame_id, uint32_t(pix), smp, 0u };
                    T jx = T(gen.next() - 0.5f);
                    T jy = T(gen.next() - 0.5f);
                    // pinhole_camera::primary_ray (detail/pinhole_camera.inl:103-120)
                    T sx = (x + jx + T(0.5)) / T(p.width);
                    T sy = (y + jy + T(0.5)) / T(p.height);
                    T u = T(2.0) * sx - T(1.0);
                    T v = T(2.0) * sy - T(1.0);
                    vec<T> d = normalize(U * u + V * v + W);
                    bool hit = false;
                    vec<T> c = radiance<T>(s, mats, nmat, lights, nl, p, eye, d, T(0.0), T(FLT_MAX), gen, hit,
                                           per[size_t(tid)], trig_double, ext);
                    if (hit)
                    {
                        sum = sum + c;
                        alpha = alpha + T(1.0);
                    }
                    else
                    {
                        vec<T> bg = { T(p.background[0]) * T(p.background[3]), T(p.background[1]) * T(p.background[3]),
                                      T(p.background[2]) * T(p.background[3]) };
                        sum = sum + bg;
                        alpha = alpha + T(1.0);
                    }
                }
                T inv = T(float(p.spp));
                out[4 * k + 0] = double(sum.x / inv);
                out[4 * k + 1] = double(sum.y / inv);
                out[4 * k + 2] = double(sum.z / inv);
                out[4 * k + 3] = double(alpha / inv);
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) pool.emplace_back(worker, t);
    for (auto& th : pool) th.join();
    for (auto const& c : per)
    {
        total.closest += c.closest;
        total.shadow += c.shadow;
        total.boxes += c.boxes;
        total.tris += c.tris;
    }
}

// Reverse sweep over one path's vertices (the adjoint of radiance<T>'s contributions
// w.r.t. albedo and emission, roulette and geometry decisions held fixed).
template <typename T>
void sweep(vrec<T> const* recs, int nrec, vec<T> adj, gbrt_material const* mats, pt_params_ext const& ext,
           double* ga, double* ge)
{
    vec<T> tbar = { 0, 0, 0 };
    for (int k = nrec - 1; k >= 0; --k)
    {
        vrec<T> const& r = recs[k];
        gbrt_material const& m = mats[r.geom];
        if (r.kind == kMiss)
        {
            tbar = adj * r.spec;   // the ambient or environment light the ray left into
        }
        else if (r.kind == kEnd)
        {
            tbar = { 0, 0, 0 };
        }
        else if (r.kind == kSpecular || r.kind == kPlastic)
        {
            // thr' = thr * spec (then / rr): a fixed factor, nothing to differentiate
            vec<T> ub = tbar;
            if (r.rr > T(0))
            {
                vec<T> uu = r.thr * r.spec;
                T pr = r.rr;
                ub = tbar / pr;
                T pb = -(tbar.x * uu.x + tbar.y * uu.y + tbar.z * uu.z) / (pr * pr);
                if (uu.x >= uu.y && uu.x >= uu.z) ub.x += pb;
                else if (uu.y >= uu.z) ub.y += pb;
                else ub.z += pb;
            }
            vec<T> tb = ub * r.spec;
            if (r.kind == kPlastic && r.nee)
            {
                // N = w * thr * gnee * lint, w = x^2 / (x^2 + y^2), y = b0 * max(thr)
                vec<T> f = r.gnee * r.lint;
                tb = tb + adj * f * r.w;
                T wbar = adj.x * r.thr.x * f.x + adj.y * r.thr.y * f.y + adj.z * r.thr.z * f.z;
                T yv = r.b0 * max_element(r.thr);
                T den = r.x * r.x + yv * yv;
                T g = wbar * (-T(2) * r.x * r.x * yv / (den * den)) * r.b0;
                if (r.thr.x >= r.thr.y && r.thr.x >= r.thr.z) tb.x += g;
                else if (r.thr.y >= r.thr.z) tb.y += g;
                else tb.z += g;
                if (r.lgeom != 0xFFFFFFFFu)
                {
                    vec<T> lb = adj * r.thr * r.gnee * (r.w * r.kl);
                    ge[3 * r.lgeom + 0] += double(lb.x);
                    ge[3 * r.lgeom + 1] += double(lb.y);
                    ge[3 * r.lgeom + 2] += double(lb.z);
                }
            }
            tbar = tb;
        }
        else if (r.kind == kEmission)
        {
            vec<T> e = ext.emission ? load<T>(ext.emission + 3 * r.geom)
                                    : vec<T>{ T(m.color[0]), T(m.color[1]), T(m.color[2]) };
            vec<T> eb = adj * r.thr * (r.mis * r.escale);
            if (ext.emission)
            {
                ge[3 * r.geom + 0] += double(eb.x);
                ge[3 * r.geom + 1] += double(eb.y);
                ge[3 * r.geom + 2] += double(eb.z);
            }
            tbar = adj * e * (r.mis * r.escale);
        }
        else
        {
            vec<T> a = ext.albedo ? load<T>(ext.albedo + 3 * r.geom)
                                  : vec<T>{ T(m.color[0]), T(m.color[1]), T(m.color[2]) };
            vec<T> ub = tbar;
            if (r.rr > T(0))
            {
                vec<T> uu = r.thr * a * r.sigma;
                T pr = r.rr;
                ub = tbar / pr;
                T pb = -(tbar.x * uu.x + tbar.y * uu.y + tbar.z * uu.z) / (pr * pr);
                if (uu.x >= uu.y && uu.x >= uu.z) ub.x += pb;
                else if (uu.y >= uu.z) ub.y += pb;
                else ub.z += pb;
            }
            vec<T> abar = ub * r.thr * r.sigma;
            vec<T> tb = ub * a * r.sigma;
            if (r.nee)
            {
                vec<T> f = r.lint * r.kfac;
                abar = abar + adj * r.thr * f * r.w;
                tb = tb + adj * a * f * r.w;
                T wbar = adj.x * r.thr.x * a.x * f.x + adj.y * r.thr.y * a.y * f.y + adj.z * r.thr.z * a.z * f.z;
                T yv = r.b0 * max_element(r.thr);
                T den = r.x * r.x + yv * yv;
                T g = wbar * (-T(2) * r.x * r.x * yv / (den * den)) * r.b0;
                if (r.thr.x >= r.thr.y && r.thr.x >= r.thr.z) tb.x += g;
                else if (r.thr.y >= r.thr.z) tb.y += g;
                else tb.z += g;
                if (r.lgeom != 0xFFFFFFFFu)
                {
                    vec<T> lb = adj * r.thr * a * (r.w * r.kfac * r.kl);
                    ge[3 * r.lgeom + 0] += double(lb.x);
                    ge[3 * r.lgeom + 1] += double(lb.y);
                    ge[3 * r.lgeom + 2] += double(lb.z);
                }
            }
            if (ext.albedo)
            {
                ga[3 * r.geom + 0] += double(abar.x);
                ga[3 * r.geom + 1] += double(abar.y);
                ga[3 * r.geom + 2] += double(abar.z);
            }
            tbar = tb;
        }
    }
}

template <typename T>
void adjoint(scene_arrays const& s, gbrt_material const* mats, uint32_t nmat, gbrt_light const* lights,
             uint32_t nl, gbrt_camera const& cam, gbrt_pt_params const& p, pt_params_ext const& ext,
             const double* img_adj, int nthreads, double* grad_albedo, double* grad_emission, double* image)
{
    vec<T> eye = load<T>(cam.eye), center = load<T>(cam.center), up = load<T>(cam.up);
    vec<T> f = normalize(eye - center);
    vec<T> sv = normalize(cross(up, f));
    vec<T> uv = cross(f, sv);
    T fovy = T(cam.fovy_degrees) * T(1.74532925199432957692369076849e-02);
    T aspect = T(p.width) / T(p.height);
    T th = std::tan(fovy / T(2.0));
    vec<T> U = sv * th * aspect, V = uv * th, W = -f;
    uint64_t npix = uint64_t(p.width) * p.height;
    if (nthreads <= 0) nthreads = int(std::max(1u, std::thread::hardware_concurrency()));
    std::vector<std::vector<double>> ga(static_cast<size_t>(nthreads), std::vector<double>(3 * size_t(nmat), 0.0));
    std::vector<std::vector<double>> ge(static_cast<size_t>(nthreads), std::vector<double>(3 * size_t(nmat), 0.0));
    std::atomic<uint64_t> next{ 0 };
    auto worker = [&](int tid) {
        pt_counters cnt;
        vrec<T> recs[16];
        for (;;)
        {
            uint64_t b = next.fetch_add(64);
            if (b >= npix) break;
            for (uint64_t pix = b; pix < std::min(npix, b + 64); ++pix)
            {
                T x = T(pix % p.width), y = T(pix / p.width);
                vec<T> sum = { 0, 0, 0 };
                for (uint32_t smp = 0; smp < p.spp; ++smp)
                {
                    gbrt_sample_generator gen{ p.frame_id, uint32_t(pix), smp, 0u };
                    T jx = T(gen.next() - 0.5f);
                    T jy = T(gen.next() - 0.5f);
                    T sx = (x + jx + T(0.5)) / T(p.width);
                    T sy = (y + jy + T(0.5)) / T(p.height);
                    vec<T> d = normalize(U * (T(2.0) * sx - T(1.0)) + V * (T(2.0) * sy - T(1.0)) + W);
                    bool hit = false;
                    int nrec = 0;
                    vec<T> c = radiance<T>(s, mats, nmat, lights, nl, p, eye, d, T(0.0), T(FLT_MAX), gen, hit, cnt,
                                           std::is_same<T, float>::value, ext, recs, &nrec);
                    if (!hit) continue;
                    sum = sum + c;
                    vec<T> adj = { T(img_adj[4 * pix + 0]) / T(float(p.spp)), T(img_adj[4 * pix + 1]) / T(float(p.spp)),
                                   T(img_adj[4 * pix + 2]) / T(float(p.spp)) };
                    sweep<T>(recs, nrec, adj, mats, ext, ga[size_t(tid)].data(), ge[size_t(tid)].data());
                }
                if (image)
                {
                    image[4 * pix + 0] = double(sum.x / T(float(p.spp)));
                    image[4 * pix + 1] = double(sum.y / T(float(p.spp)));
                    image[4 * pix + 2] = double(sum.z / T(float(p.spp)));
                    image[4 * pix + 3] = 1.0;
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) pool.emplace_back(worker, t);
    for (auto& t : pool) t.join();
    for (size_t i = 0; i < 3 * size_t(nmat); ++i)
    {
        double a = 0.0, e = 0.0;
        for (int t = 0; t < nthreads; ++t)
        {
            a += ga[size_t(t)][i];
            e += ge[size_t(t)][i];
        }
        grad_albedo[i] = a;
        grad_emission[i] = e;
    }
}

} // namespace

extern "C" void orc_pathtrace_adjoint(const gbrt_triangle* tris, const gbrt_bvh_node* nodes, uint32_t num_nodes,
                                      const uint32_t* indices, const gbrt_material* mats, uint32_t nmat,
                                      const gbrt_light* lights, uint32_t nl, const gbrt_camera* cam,
                                      const gbrt_pt_params* p, const float* albedo, const float* emission,
                                      const double* img_adj, int fp64, int nthreads, double* grad_albedo,
                                      double* grad_emission, double* image, const gbrt_environment* env)
{
    scene_arrays s{ tris, nodes, num_nodes, indices };
    pt_params_ext ext;
    ext.albedo = albedo;
    ext.emission = emission;
    ext.env = env;
    if (env) inverse_rows(env->light_to_world, ext.env_m);
    if (fp64)
        adjoint<double>(s, mats, nmat, lights, nl, *cam, *p, ext, img_adj, nthreads, grad_albedo, grad_emission, image);
    else
        adjoint<float>(s, mats, nmat, lights, nl, *cam, *p, ext, img_adj, nthreads, grad_albedo, grad_emission, image);
}

extern "C" void orc_pathtrace(const gbrt_triangle* tris, const gbrt_bvh_node* nodes, uint32_t num_nodes,
                              const uint32_t* indices, const gbrt_material* mats, uint32_t nmat,
                              const gbrt_light* lights, uint32_t nl, const gbrt_camera* cam,
                              const gbrt_pt_params* p, int mode, int nthreads, double* out_rgba, uint64_t* counters,
                              const gbrt_environment* env)
{
    scene_arrays s{ tris, nodes, num_nodes, indices };
    pt_counters c;
    pt_params_ext ext;
    ext.env = env;
    if (env) inverse_rows(env->light_to_world, ext.env_m);
    ext.draws_in_order = (mode & 4) != 0;   // the device build's draw order
    mode &= 3;
    if (mode == 1)
        render<double>(s, mats, nmat, lights, nl, *cam, *p, nthreads, out_rgba, c, false, ext);
    else
        render<float>(s, mats, nmat, lights, nl, *cam, *p, nthreads, out_rgba, c, mode == 2, ext);
    if (counters)
    {
        counters[0] = c.closest;
        counters[1] = c.shadow;
        counters[2] = c.boxes;
        counters[3] = c.tris;
    }
}

// orc_pathtrace on the listed pixels only (row-major indices into the width x height
// frame, each < width * height): out_rgba[4 k ...] is pixel plist[k]'s average.
extern "C" void orc_pathtrace_pixels(const gbrt_triangle* tris, const gbrt_bvh_node* nodes, uint32_t num_nodes,
                                     const uint32_t* indices, const gbrt_material* mats, uint32_t nmat,
                                     const gbrt_light* lights, uint32_t nl, const gbrt_camera* cam,
                                     const gbrt_pt_params* p, int mode, int nthreads, const uint32_t* plist,
                                     uint64_t nlist, double* out_rgba, uint64_t* counters,
                                     const gbrt_environment* env)
{
    scene_arrays s{ tris, nodes, num_nodes, indices };
    pt_counters c;
    pt_params_ext ext;
    ext.env = env;
    if (env) inverse_rows(env->light_to_world, ext.env_m);
    ext.draws_in_order = (mode & 4) != 0;
    mode &= 3;
    if (mode == 1)
        render<double>(s, mats, nmat, lights, nl, *cam, *p, nthreads, out_rgba, c, false, ext, plist, nlist);
    else
        render<float>(s, mats, nmat, lights, nl, *cam, *p, nthreads, out_rgba, c, mode == 2, ext, plist, nlist);
    if (counters)
    {
        counters[0] = c.closest;
        counters[1] = c.shadow;
        counters[2] = c.boxes;
        counters[3] = c.tris;
    }
}
