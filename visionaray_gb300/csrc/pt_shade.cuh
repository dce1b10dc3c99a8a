// Path-tracing shading shared by the wavefront renderer and its adjoint (pathtrace.cu)
// and the batched persistent renderer (batch_pt.cu): the vector helpers in the
// reference's float arithmetic, the pinhole camera, and one bounce of
// pathtracing::kernel (shade_vertex).  Every unit including this header is compiled
// with --fmad=false, so all of them evaluate these expressions identically.
#pragma once

#include "traverse_core.cuh"

#include "../../include/visionaray_gb300/gbrt_rng.h"

#include <cmath>

namespace gbrt {
namespace {

constexpr uint32_t kLastSpecular = 1u;
constexpr uint32_t kFirstHit = 2u;

struct v3
{
    float x, y, z;
};
__device__ __forceinline__ v3 operator+(v3 a, v3 b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
__device__ __forceinline__ v3 operator-(v3 a, v3 b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
__device__ __forceinline__ v3 operator-(v3 a) { return { -a.x, -a.y, -a.z }; }
__device__ __forceinline__ v3 operator*(v3 a, v3 b) { return { a.x * b.x, a.y * b.y, a.z * b.z }; }
__device__ __forceinline__ v3 operator*(v3 a, float s) { return { a.x * s, a.y * s, a.z * s }; }
__device__ __forceinline__ v3 operator/(v3 a, float s) { return { a.x / s, a.y / s, a.z / s }; }
__device__ __forceinline__ float dot3(v3 u, v3 v) { return u.x * v.x + u.y * v.y + u.z * v.z; }
__device__ __forceinline__ v3 cross3(v3 u, v3 v)
{
    return { u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x };
}
__device__ __forceinline__ float length3(v3 v) { return sqrtf(dot3(v, v)); }
// normalize(v) = v * (1 / sqrt(dot(v, v))) (math/detail/vector3.inl:332-335)
__device__ __forceinline__ v3 normalize3(v3 v) { return v * (1.0f / sqrtf(dot3(v, v))); }
__device__ __forceinline__ v3 faceforward3(v3 n, v3 i, v3 nref) { return dot3(nref, i) < 0.0f ? -n : n; }
__device__ __forceinline__ float max_elem(v3 v)
{
    float m = v.x < v.y ? v.y : v.x;
    return m < v.z ? v.z : m;
}
__device__ __forceinline__ float power_heuristic(float p1, float p2) { return (p1 * p1) / (p1 * p1 + p2 * p2); }
__device__ __forceinline__ v3 xyz(float4 a) { return { a.x, a.y, a.z }; }
// pow evaluated in double and rounded once to float.  pow with a
// non-negative integer exponent up to 1024 (the Blinn exponents of typical scenes and
// Schlick's fifth power) is binary exponentiation in double: at most 2 log2(y) roundings
// of 2^-53 each, so the float result is the double pow's except for values within about
// 2^-27 of a float rounding boundary, at a few multiplications instead of the double
// pow's log and exp (FP64 issue is slow on this GPU: the general pow made the Blinn
// lobe 40 % of a glossy frame).
__device__ __forceinline__ float pow_d(float x, float y)
{
    if (y >= 0.0f && y <= 1024.0f && y == truncf(y))
    {
        unsigned n = unsigned(y);
        double b = double(x), r = 1.0;
        while (n)
        {
            if (n & 1u) r *= b;
            n >>= 1;
            if (n) b *= b;
        }
        return float(r);
    }
    return float(pow(double(x), double(y)));
}

// blinn::f (brdf.h:128-141): Schlick's Fresnel term on cs * ks and the normalised
// Blinn-Phong lobe
__device__ __forceinline__ v3 blinn_f(gbrt_material const& m, v3 n, v3 wo, v3 wi)
{
    const float pi = 3.14159265358979323846264338328e+00f;
    v3 h = normalize3(wo + wi);
    float hdotn = fmaxf(0.0f, dot3(h, n));
    float sat = fmaxf(0.0f, fminf(dot3(wi, h), 1.0f));   // saturate (math/detail/math.h:537-540)
    float fr = pow_d(1.0f - sat, 5.0f);
    float nfactor = (m.exponent + 2.0f) / (8.0f * pi);
    float lobe = pow_d(hdotn, m.exponent);
    float out[3];
    for (int c = 0; c < 3; ++c)
    {
        float spec = m.color2[c] * m.scale2;
        float schlick = spec + (1.0f - spec) * fr;
        out[c] = (schlick * nfactor) * lobe;
    }
    return { out[0], out[1], out[2] };
}

// blinn::pdf (brdf.h:182-190)
__device__ __forceinline__ float blinn_pdf(gbrt_material const& m, v3 n, v3 wo, v3 wi)
{
    const float pi = 3.14159265358979323846264338328e+00f;
    v3 h = normalize3(wi + wo);
    float costheta = dot3(n, h);
    float vdoth = dot3(wo, h);
    return ((m.exponent + 1.0f) * pow_d(costheta, m.exponent)) / (2.0f * pi * 4.0f * vdoth);
}

struct camera_basis
{
    float3 eye, U, V, W;
};

// Primary ray direction of `pixel` for sample `sample`: jitter x drawn before y
// (detail/sched_common.h:209-233) through the pinhole camera
// (detail/pinhole_camera.inl:103-120).
__device__ __forceinline__ v3 primary_dir(camera_basis const& cam, uint32_t width, uint32_t height, uint32_t frame,
                                          uint32_t pixel, uint32_t sample)
{
    float x = float(pixel % width), y = float(pixel / width);
    float jx = gbrt_rng_u01(frame, pixel, sample, 0) - 0.5f;
    float jy = gbrt_rng_u01(frame, pixel, sample, 1) - 0.5f;
    float sx = ((x + jx) + 0.5f) / float(width);
    float sy = ((y + jy) + 0.5f) / float(height);
    float u = 2.0f * sx - 1.0f;
    float v = 2.0f * sy - 1.0f;
    v3 U = { cam.U.x, cam.U.y, cam.U.z }, V = { cam.V.x, cam.V.y, cam.V.z }, W = { cam.W.x, cam.W.y, cam.W.z };
    return normalize3(U * u + V * v + W);
}

// environment_light<float, texture_ref<vec4, 2>> (environment_light.h:22-58): the
// texture, the scale and rows 0-2 of world_to_light (4 columns each).
struct env_view
{
    const float4* texels = nullptr;   // null: the constant ambient light
    uint32_t width = 0, height = 0, filter = 0, address = 0;
    float scale[3] = { 0.0f, 0.0f, 0.0f };
    float m[12] = {};
};

struct shade_params
{
    const gbrt_material* materials;
    uint32_t num_materials;
    const float4* lights;   // 4 float4 per light: v1 | geom bits, e1, e2, intensity | kl
    uint32_t num_lights;
    const tri48* tris;
    int32_t num_tris;
    float epsilon;
    float3 ambient;
    uint32_t frame, sample, bounce, flags;
    // differentiable renderer: matte colors and emissive colors (3 floats per material
    // slot) replacing the materials' own; light intensity = emission[geom] * kl
    const float* albedo;
    const float* emission;
    // (cos, sin) of 2 pi u for the 2^24 values of a draw u (gbrt_context::d_trig)
    const float2* trig;
    const env_view* env = nullptr;   // device record; null: the constant ambient light
    // a hit inside an instance of a two-level tree: the instance's instance-to-world
    // rows (3 float4: A | translation) and its first material slot; null / 0 for a hit
    // in a single tree (tris then is the hit instance's tree's triangles)
    const float4* xform = nullptr;
    uint32_t geom_base = 0;
};

// The 3x3 rows of an instance-to-world map applied to a direction (an edge).
__device__ __forceinline__ v3 apply_rows(const float4* __restrict__ r, v3 e)
{
    const float4 a = r[0], b = r[1], c = r[2];
    return { a.x * e.x + a.y * e.y + a.z * e.z, b.x * e.x + b.y * e.y + b.z * e.z, c.x * e.x + c.y * e.y + c.z * e.z };
}

// remap_texture_coordinate (texture/detail/texture_common.h:91-126) for one axis of n
// texels; clamp(x, a, b) = max(a, min(x, b)) (math/detail/math.h:530-533).
__device__ __forceinline__ float tex_remap(float c, uint32_t n, uint32_t address)
{
    const float fn = float(int(n));
    if (address == GBRT_ADDRESS_WRAP) return c - floorf(c);
    if (address == GBRT_ADDRESS_MIRROR)
    {
        float f = floorf(c);
        return (int(f) & 1) == 1 ? float(int(n) - 1) / fn - (c - f) : c - f;
    }
    return ref_max(0.0f, ref_min(c, 1.0f - 1.0f / fn));
}

// A texel index: convert_to_int (truncation) as the filters take it, kept inside the
// row (an index the reference would read outside the texture, from a coordinate that
// rounds to 1.0 under Wrap or from NaN, reads the edge texel here).
__device__ __forceinline__ int tex_index(float c, uint32_t n)
{
    int i = int(c * float(int(n)));
    return min(max(i, 0), int(n) - 1);
}

__device__ __forceinline__ float4 tex_lerp(float4 a, float4 b, float x)
{
    // lerp_r(a, b, x) = (1 - x) * a + x * b (math/detail/math.h:550-555)
    const float w = 1.0f - x;
    return make_float4(w * a.x + x * b.x, w * a.y + x * b.y, w * a.z + x * b.z, w * a.w + x * b.w);
}

// environment_light::intensity (detail/environment_light.inl:18-34): the direction in
// light space, its lat-long coordinates and tex2D (filter/nearest.h:44-66, filter/
// linear.h:56-96) times the scale.  Inlined: a call would give every kernel that
// shades a call frame (measured slower on the adjoint's replay).
__device__ __forceinline__ v3 env_intensity(const env_view* __restrict__ ev, v3 dir)
{
    const env_view e = *ev;
    const float two_pi = 6.28318530717958647692528676656e+00f;
    const float inv_pi = 3.18309886183790691216444201928e-01f;
    const float dx = e.m[0] * dir.x + e.m[1] * dir.y + e.m[2] * dir.z + e.m[3] * 0.0f;
    const float dy = e.m[4] * dir.x + e.m[5] * dir.y + e.m[6] * dir.z + e.m[7] * 0.0f;
    const float dz = e.m[8] * dir.x + e.m[9] * dir.y + e.m[10] * dir.z + e.m[11] * 0.0f;
    float x = atan2f(dx, dz);
    x = x < 0.0f ? x + two_pi : x;
    const float y = acosf(dy);
    const float u = x / two_pi;
    const float v = y * inv_pi;
    float4 t;
    if (e.filter == GBRT_FILTER_NEAREST)
    {
        const int ix = tex_index(tex_remap(u, e.width, e.address), e.width);
        const int iy = tex_index(tex_remap(v, e.height, e.address), e.height);
        t = __ldg(&e.texels[size_t(iy) * e.width + ix]);
    }
    else
    {
        const float fw = float(int(e.width)), fh = float(int(e.height));
        const float c1x = tex_remap(u - 0.5f / fw, e.width, e.address);
        const float c1y = tex_remap(v - 0.5f / fh, e.height, e.address);
        const float c2x = tex_remap(u + 0.5f / fw, e.width, e.address);
        const float c2y = tex_remap(v + 0.5f / fh, e.height, e.address);
        const int lx = tex_index(c1x, e.width), ly = tex_index(c1y, e.height);
        const int hx = tex_index(c2x, e.width), hy = tex_index(c2y, e.height);
        const float4 s0 = __ldg(&e.texels[size_t(ly) * e.width + lx]);
        const float4 s1 = __ldg(&e.texels[size_t(ly) * e.width + hx]);
        const float4 s2 = __ldg(&e.texels[size_t(hy) * e.width + lx]);
        const float4 s3 = __ldg(&e.texels[size_t(hy) * e.width + hx]);
        const float ux = c1x * fw - float(lx);
        const float uy = c1y * fh - float(ly);
        t = tex_lerp(tex_lerp(s0, s1, ux), tex_lerp(s2, s3, ux), uy);
    }
    return v3{ t.x * e.scale[0], t.y * e.scale[1], t.z * e.scale[2] };
}

// cos and sin of the float angle 2 pi u (u a draw of gbrt_rng_u01, a multiple of
// 2^-24), each evaluated in double and rounded once to float -- looked up: the table
// holds exactly those values for every u, computed once, so the shading kernels
// issue no double-precision trigonometry (FP64 issue is slow on this GPU).
__device__ __forceinline__ float2 trig_of(const float2* __restrict__ table, float u)
{
    return __ldg(&table[uint32_t(u * 16777216.0f) & 0xFFFFFFu]);
}

struct path_state
{
    v3 thr, rad;
    uint32_t k, flags;
};

// What the adjoint needs of one path vertex (the throughput entering it and the
// albedo-independent factors of its contributions).
enum : uint32_t
{
    kVertexMiss = 0,
    kVertexEmission = 1,
    kVertexMatte = 2,
    kVertexEnd = 3,   // matte with a zero pdf: the path stops without contributing
    kVertexSpecular = 4,   // mirror / glass: next throughput = thr * spec (not differentiated)
    kVertexPlastic = 5,    // plastic: thr * spec as specular, NEE = w * thr * gnee * lint
};

struct vertex_rec
{
    uint32_t kind, geom, lgeom, nee;
    v3 thr;           // throughput entering the vertex
    float rr;         // Russian roulette normaliser (0: none)
    float w, x, b0;   // NEE: w = power_heuristic(x, b0 * max(thr))
    float kl;         // NEE: lint = emission[lgeom] * kl
    v3 lint;
    v3 gnee;          // NEE: contribution = w * thr * albedo * gnee * lint (matte),
                      //      w * thr * gnee * lint (plastic)
    union
    {
        v3 spec;      // specular, plastic: next throughput = thr * spec (then / rr); miss: the light seen
        float sigma;  // matte: next throughput = thr * albedo * sigma (then / rr)
        struct
        {
            float mis, scale;   // emission: contribution = thr * mis * emission * scale
        } emit;
    } f;
};

struct vertex_out
{
    bool cont, shadow;
    v3 next_o, next_d;
    v3 sh_o, sh_d;
    float sh_tmax;
    v3 contrib;
    vertex_rec rec;
};

__device__ __forceinline__ v3 param3(const float* a, uint32_t i) { return { a[3 * i], a[3 * i + 1], a[3 * i + 2] }; }

struct lobe_sample
{
    v3 refl, src;
    float pdf;
    uint32_t k;        // the random-number counter after the draws
    uint32_t glossy;   // the Blinn lobe was sampled (inter = GlossyReflection)
};

// plastic::sample (detail/material/plastic.inl:42-95) on the faceforwarded normal nn:
// one draw picks the lobe by the mean reflectances, and the pdf returned is the chosen
// lobe's alone.  Out of line, like plastic_nee below: the double-precision pow and
// exp2 / log2 would otherwise raise the register pressure of every kernel that shades.
__device__ __noinline__ lobe_sample sample_plastic(const gbrt_material* __restrict__ mp,
                                                   const float2* __restrict__ trig, v3 nn, v3 view,
                                                   uint32_t frame, uint32_t p, uint32_t sample, uint32_t k)
{
    const float inv_pi = 3.18309886183790691216444201928e-01f;
    const float pi = 3.14159265358979323846264338328e+00f;
    const gbrt_material m = *mp;
    lobe_sample out;
    float prob_diff = ((m.color[0] + m.color[1]) + m.color[2]) / 3.0f * m.scale;
    float prob_spec = ((m.color2[0] + m.color2[1]) + m.color2[2]) / 3.0f * m.scale2;
    const bool all_zero = prob_diff == 0.0f && prob_spec == 0.0f;
    prob_diff = all_zero ? 0.5f : prob_diff;
    prob_spec = all_zero ? 0.5f : prob_spec;
    prob_diff = prob_diff / (prob_diff + prob_spec);
    const float u = gbrt_rng_u01(frame, p, sample, k++);
    v3 w = nn;
    v3 v = fabsf(w.x) > fabsf(w.y) ? normalize3(v3{ -w.z, 0.0f, w.x }) : normalize3(v3{ 0.0f, w.z, -w.y });
    v3 uu = cross3(v, w);
    if (u < prob_diff)
    {
        // lambertian::sample_f as for matte (second argument drawn first)
        float u2 = gbrt_rng_u01(frame, p, sample, k++);
        float u1 = gbrt_rng_u01(frame, p, sample, k++);
        float r = sqrtf(u1);
        const float2 cs = trig_of(trig, u2);   // theta = two_pi * u2
        v3 s3 = { r * cs.x, r * cs.y, sqrtf(1.0f - u1) };
        out.refl = normalize3(uu * s3.x + v * s3.y + w * s3.z);
        out.pdf = dot3(nn, out.refl) * inv_pi;
        out.src = (v3{ m.color[0], m.color[1], m.color[2] } * m.scale) * inv_pi;
        out.glossy = 0u;
    }
    else
    {
        // blinn::sample_f (brdf.h:143-180): half vector around n, wi = reflect(wo, h)
        float u1 = gbrt_rng_u01(frame, p, sample, k++);
        float u2 = gbrt_rng_u01(frame, p, sample, k++);
        // pow(u1, 1 / (exp + 1)) as exp2(y log2 u1) in double: |y log2 u1| <= 24, so the
        // double result is within ~2^-48 relative of pow's and rounds to the same float
        // except within ~2^-25 of a rounding boundary; cheaper than the double pow
        float costheta = float(exp2(double(1.0f / (m.exponent + 1.0f)) * log2(double(u1))));
        float sintheta = sqrtf(fmaxf(0.0f, 1.0f - costheta * costheta));
        const float2 cs = trig_of(trig, u2);   // phi = u2 * two_pi
        v3 h = normalize3(uu * (sintheta * cs.x) + v * (sintheta * cs.y) + w * costheta);
        out.refl = h * (2.0f * dot3(h, view)) - view;
        float vdoth = dot3(view, h);
        out.pdf = ((m.exponent + 1.0f) * pow_d(costheta, m.exponent)) / (2.0f * pi * 4.0f * vdoth);
        out.src = blinn_f(m, nn, view, out.refl);
        out.glossy = 1u;
    }
    out.k = k;
    return out;
}

// mirror::sample and glass::sample on the unflipped shading normal sn (out of line,
// as sample_plastic).
__device__ __noinline__ lobe_sample sample_specular(const gbrt_material* __restrict__ mp, v3 sn, v3 view,
                                                    uint32_t frame, uint32_t p, uint32_t sample, uint32_t k)
{
    const gbrt_material m = *mp;
    lobe_sample out;
    out.glossy = 0u;
    if (m.kind == GBRT_MATERIAL_MIRROR)
    {
        // mirror::sample -> specular_reflection::sample_f(sr.normal, view) (brdf.h:317-340):
        // wi = reflect(wo, n), pdf 1, conductor Fresnel (fresnel.h:18-35) * cr * kr / |n.wi|
        const v3 wo = view;
        out.refl = sn * (2.0f * dot3(sn, wo)) - wo;
        out.pdf = 1.0f;
        const float cosi = fabsf(dot3(sn, wo));
        const float cr[3] = { m.color[0], m.color[1], m.color[2] };
        float f[3];
        for (int c = 0; c < 3; ++c)
        {
            const float eta = m.ior[c], kap = m.absorption[c];
            const float a = eta * eta + kap * kap;
            const float rs2 = ((a - 2.0f * eta * cosi) + cosi * cosi) / ((a + 2.0f * eta * cosi) + cosi * cosi);
            const float rp2 = ((a * cosi * cosi - 2.0f * eta * cosi) + 1.0f) / ((a * cosi * cosi + 2.0f * eta * cosi) + 1.0f);
            f[c] = ((rs2 + rp2) / 2.0f) * (cr[c] * m.scale);
        }
        const float dn = fabsf(dot3(sn, out.refl));
        out.src = { f[0] / dn, f[1] / dn, f[2] / dn };
    }
    else
    {
        // glass::sample -> specular_transmission::sample_f(sr.normal, view) (brdf.h:385-456)
        const v3 wo = view;
        float cosi = dot3(sn, wo);
        cosi = cosi < 1.0f ? cosi : 1.0f;          // clamp(x, -1, 1) = max(-1, min(x, 1))
        cosi = -1.0f < cosi ? cosi : -1.0f;
        const bool entering = cosi > 0.0f;
        const v3 N = entering ? sn : -sn;
        const float ior1[3] = { 1.0f, 1.0f, 1.0f }, ior2[3] = { m.ior[0], m.ior[1], m.ior[2] };
        const float etai0 = entering ? ior1[0] : ior2[0], etat0 = entering ? ior2[0] : ior1[0];
        if (!entering) cosi = fabsf(cosi);
        const float eta = etai0 / etat0;
        const float sini = sqrtf(fmaxf(0.0f, 1.0f - cosi * cosi));
        const float sint = eta * sini;
        const float cost = sqrtf(fmaxf(0.0f, 1.0f - sint * sint));
        // fresnel_reflectance(dielectric_tag, ior1, ior2, cosi, cost) (fresnel.h:37-56)
        float R[3];
        for (int c = 0; c < 3; ++c)
        {
            const float rs = (ior1[c] * cosi - ior2[c] * cost) / (ior1[c] * cosi + ior2[c] * cost);
            const float rp = (ior2[c] * cosi - ior1[c] * cost) / (ior2[c] * cosi + ior1[c] * cost);
            R[c] = (rs * rs + rp * rp) / 2.0f;
        }
        if (sint >= 1.0f) R[0] = R[1] = R[2] = 1.0f;   // total internal reflection
        // refract(wo, N, eta) (vector.inl:695-707; not normalised) and reflect(wo, N)
        const float rc = dot3(N, wo);
        const float rsin = fmaxf(0.0f, 1.0f - rc * rc);
        const float rsint = eta * eta * rsin;
        const v3 refracted = rsint >= 1.0f ? v3{ 0.0f, 0.0f, 0.0f } : (-wo) * eta + N * (eta * rc - sqrtf(1.0f - rsint));
        const v3 reflected = N * (2.0f * dot3(N, wo)) - wo;
        const float u = gbrt_rng_u01(frame, p, sample, k++);
        float val[3];
        if (u < R[0])
        {
            out.refl = reflected;
            out.pdf = R[0];
            const float cr[3] = { m.color2[0], m.color2[1], m.color2[2] };
            for (int c = 0; c < 3; ++c) val[c] = R[c] * (cr[c] * m.scale2);
        }
        else
        {
            out.refl = normalize3(refracted);
            out.pdf = 1.0f - R[0];
            const float ct[3] = { m.color[0], m.color[1], m.color[2] };
            for (int c = 0; c < 3; ++c) val[c] = (1.0f - R[c]) * (ct[c] * m.scale);
        }
        const float dn = dot3(N, out.refl);
        out.src = { val[0] / dn, val[1] / dn, val[2] / dn };
    }
    out.k = k;
    return out;
}

struct nee_terms
{
    v3 brdf;     // (diffuse + Blinn) reflectance toward L
    float pdf;   // surf.pdf(view, L, inter)
};

// A plastic surface's next-event terms toward L: plastic::pdf (plastic.inl:97-110,
// the sampled lobe's) and the reflectance inside plastic::shade (plastic.inl:20-39)
// added to the diffuse term cd.
__device__ __noinline__ nee_terms plastic_nee(const gbrt_material* __restrict__ mp, v3 nn, v3 view, v3 L, v3 cd,
                                              uint32_t glossy)
{
    const float inv_pi = 3.18309886183790691216444201928e-01f;
    const gbrt_material m = *mp;
    nee_terms out;
    out.pdf = glossy ? blinn_pdf(m, nn, view, L) : dot3(nn, L) * inv_pi;
    out.brdf = cd + blinn_f(m, nn, view, L);
    return out;
}

// One bounce of pathtracing::kernel::operator() (detail/pathtracing.inl:65-221) for one
// path whose ray (ori, dir) hit triangle `tri` at `t` (tri < 0: missed).  Updates the
// path state, adds emission / ambient to st.rad, and returns the next ray and the NEE
// shadow ray with its unoccluded contribution.  Shared by the wavefront shade kernel
// and the adjoint's replay, so both compute bit-identical paths.
// Extended = false compiles out the mirror, glass and plastic branches, for scenes
// whose materials are all matte or emissive (any other kind then shades as matte).
// Env = false compiles out the environment light (the adjoint's replay of scenes
// without one: the miss record then carries nothing and the sweep reads the ambient).
template <bool Extended = true, bool Env = true>
__device__ __forceinline__ void shade_vertex(shade_params const& sp, uint32_t p, uint32_t bounce, v3 ori, v3 dir,
                                             float tmin, float tmax, int tri, float t, path_state& st,
                                             vertex_out& out, uint32_t* __restrict__ status)
{
    const float inv_pi = 3.18309886183790691216444201928e-01f;
    const float pi = 3.14159265358979323846264338328e+00f;
    out.cont = false;
    out.shadow = false;
    vertex_rec& rec = out.rec;
    rec.kind = kVertexMiss;
    rec.thr = st.thr;
    rec.nee = 0;
    rec.rr = 0.0f;
    rec.geom = 0;
    rec.lgeom = 0xFFFFFFFFu;

    if (tri < 0 || tri >= sp.num_tris)
    {
        // the ray left the scene: ambient or environment light (pathtracing.inl:71-79)
        v3 amb = { sp.ambient.x, sp.ambient.y, sp.ambient.z };
        if (Env)
        {
            if (sp.env) amb = env_intensity(sp.env, dir);
            rec.f.spec = amb;
        }
        st.rad = st.rad + amb * st.thr;
        return;
    }
    if (bounce == 0) st.flags |= kFirstHit;
    float4 t1 = ldg4(&sp.tris[tri].t1);
    float4 t2 = ldg4(&sp.tris[tri].t2);
    v3 e1 = xyz(t1), e2 = xyz(t2);
    uint32_t geom = __float_as_uint(t1.w);
    if (sp.xform)
    {
        // the instance's triangle in world space (its normal and area), its material
        // slot after the instance's first
        e1 = apply_rows(sp.xform, e1);
        e2 = apply_rows(sp.xform, e2);
        geom += sp.geom_base;
    }
    v3 view = -dir;
    v3 isect = ori + dir * t;
    v3 gn = normalize3(cross3(e1, e2));
    v3 sn = gn;
    gbrt_material m;
    if (geom < sp.num_materials)
    {
        m = sp.materials[geom];
    }
    else
    {
        atomicOr(status, kStatusBadIndex);
        m = gbrt_material{ GBRT_MATERIAL_MATTE, { 0.0f, 0.0f, 0.0f }, 0.0f };
        geom = 0;
    }
    bool emission = m.kind == GBRT_MATERIAL_EMISSIVE;
    const bool specular = Extended && (m.kind == GBRT_MATERIAL_MIRROR || m.kind == GBRT_MATERIAL_GLASS);
    const bool plastic = Extended && m.kind == GBRT_MATERIAL_PLASTIC;
    bool glossy = false;   // plastic: the Blinn lobe was sampled (inter = GlossyReflection)
    v3 mcol = { m.color[0], m.color[1], m.color[2] };
    if (!emission && !specular && !plastic && sp.albedo) mcol = param3(sp.albedo, geom);
    if (emission && sp.emission) mcol = param3(sp.emission, geom);
    rec.geom = geom;

    v3 refl = { 0.0f, 0.0f, 0.0f };
    float brdf_pdf;
    v3 src;
    if (specular)
    {
        lobe_sample ls = sample_specular(sp.materials + geom, sn, view, sp.frame, p, sp.sample, st.k);
        refl = ls.refl;
        brdf_pdf = ls.pdf;
        src = ls.src;
        st.k = ls.k;
    }
    else if (plastic)
    {
        lobe_sample ls = sample_plastic(sp.materials + geom, sp.trig, faceforward3(sn, view, gn), view, sp.frame, p,
                                        sp.sample, st.k);
        refl = ls.refl;
        brdf_pdf = ls.pdf;
        src = ls.src;
        glossy = ls.glossy != 0u;
        st.k = ls.k;
    }
    else if (!emission)
    {
        // matte::sample -> lambertian::sample_f (matte.inl:40-56, brdf.h:50-76)
        v3 nn = faceforward3(sn, view, gn);
        v3 w = nn;
        v3 v = fabsf(w.x) > fabsf(w.y) ? normalize3(v3{ -w.z, 0.0f, w.x }) : normalize3(v3{ 0.0f, w.z, -w.y });
        v3 u = cross3(v, w);
        // cosine_sample_hemisphere(gen.next(), gen.next()), second argument drawn
        // first as in the reference build (sampling.h:117-127)
        float u2 = gbrt_rng_u01(sp.frame, p, sp.sample, st.k++);
        float u1 = gbrt_rng_u01(sp.frame, p, sp.sample, st.k++);
        float r = sqrtf(u1);
        // theta = two_pi * u2; its cos and sin evaluated in double, rounded once to float
        const float2 cs = trig_of(sp.trig, u2);
        v3 s3 = { r * cs.x, r * cs.y, sqrtf(1.0f - u1) };
        refl = normalize3(u * s3.x + v * s3.y + w * s3.z);
        brdf_pdf = dot3(nn, refl) * inv_pi;
        src = (mcol * m.scale) * inv_pi;
    }
    else
    {
        brdf_pdf = 1.0f;   // emissive::sample (emissive.inl:28-44)
        src = mcol * m.scale;
    }
    bool zero_pdf = brdf_pdf <= 0.0f;

    float light_pdf = 0.0f;
    if (sp.num_lights > 0 && emission)
    {
        float A = 0.5f * length3(cross3(e1, e2));
        float ld = length3(isect - ori);
        v3 L = normalize3(isect - ori);
        float ldotln = fabsf(dot3(-L, gn));
        float solid_angle = (ldotln * A) / (ld * ld);
        light_pdf = 1.0f / solid_angle;
    }
    float mis = (bounce > 0 && sp.num_lights > 0 && !(st.flags & kLastSpecular))
                    ? power_heuristic(brdf_pdf, light_pdf / float(sp.num_lights))
                    : 1.0f;
    if (emission)
    {
        st.rad = st.rad + (st.thr * mis) * src;
        rec.kind = kVertexEmission;
        rec.f.emit.mis = mis;
        rec.f.emit.scale = m.scale;
        return;
    }
    if (zero_pdf)
    {
        rec.kind = kVertexEnd;
        return;
    }
    rec.kind = specular ? kVertexSpecular : (plastic ? kVertexPlastic : kVertexMatte);
    v3 nn = faceforward3(sn, view, gn);
    if (sp.num_lights > 0)
    {
        // sample_random_light (sampling.h:195-213) and the light's sample: an area light
        // (area_light.inl:27-53, sample_surface triangle.inl:69-83) draws two numbers, a
        // point or spot light (point_light.inl:35-56) three for a normal it does not use
        float ul = gbrt_rng_u01(sp.frame, p, sp.sample, st.k++);
        int lid = int(ul * float(sp.num_lights));
        if (lid >= int(sp.num_lights)) lid = int(sp.num_lights) - 1;
        const float4* lp = sp.lights + 4 * lid;
        const float4 l0 = lp[0], l1 = lp[1], l3 = lp[3];
        const bool delta = l1.w != 0.0f;
        if (specular)
        {
            // a specular surface's shade() is 0: the light is sampled (its draws taken)
            // but the next-event contribution is zero
            st.k += delta ? 3u : 2u;
        }
        else
        {
            v3 lint = xyz(l3);
            uint32_t lgeom = __float_as_uint(l0.w);
            if (sp.emission && lgeom < sp.num_materials) lint = param3(sp.emission, lgeom) * l3.w;
            v3 ldir, L, ln;
            float dist, lpdf;
            if (delta)
            {
                st.k += 3;
                ldir = xyz(l0) - isect;
                dist = length3(ldir);
                lpdf = 1.0f;
                L = normalize3(ldir);
                ln = faceforward3(-L, -L, -L);   // select(delta_light, -L, normal), faceforwarded
            }
            else
            {
                v3 lv1 = xyz(l0), le1 = xyz(l1), le2 = xyz(lp[2]);
                float s1 = gbrt_rng_u01(sp.frame, p, sp.sample, st.k++);
                float s2 = gbrt_rng_u01(sp.frame, p, sp.sample, st.k++);
                v3 lv2 = lv1 + le1, lv3 = lv1 + le2;
                float sq = sqrtf(s1);
                v3 pos = lv1 * (1.0f - sq) + lv2 * sq * (1.0f - s2) + lv3 * sq * s2;
                ldir = pos - isect;
                dist = length3(ldir);
                v3 lnormal = normalize3(cross3(le1, le2));
                float larea = 0.5f * length3(cross3(le1, le2));
                float ldotln0 = fabsf(dot3(-normalize3(ldir), lnormal));
                float lsolid = (ldotln0 * larea) / (dist * dist);
                lpdf = 1.0f / lsolid;
                L = normalize3(ldir);
                ln = faceforward3(lnormal, -L, lnormal);
            }
            float ldotn = dot3(L, nn);
            float ldotln = fabsf(dot3(-L, ln));
            float bpdf0 = dot3(nn, L) * inv_pi;
            v3 cd = (mcol * m.scale) * inv_pi;
            v3 brdf = cd;
            if (plastic)
            {
                nee_terms nt = plastic_nee(sp.materials + geom, nn, view, L, cd, glossy ? 1u : 0u);
                bpdf0 = nt.pdf;
                brdf = nt.brdf;
            }
            float bpdf = bpdf0 * max_elem(st.thr);
            float ndotl = fmaxf(0.0f, dot3(nn, L));
            // (plastic::shade, plastic.inl:20-39: (diffuse + Blinn) * pi * intensity * n.l)
            v3 shade = ((brdf * pi) * lint) * ndotl;
            v3 src2 = (shade * inv_pi) / ldotn;
            float x = lpdf / float(sp.num_lights);
            float mis2 = power_heuristic(x, bpdf);
            if (ldotn > 0.0f && ldotln > 0.0f)
            {
                out.contrib = (((st.thr * mis2) * src2) * (ldotn / lpdf)) * float(sp.num_lights);
                out.shadow = true;
                out.sh_o = isect + L * sp.epsilon;
                out.sh_d = L;
                out.sh_tmax = (sp.flags & GBRT_PT_SHADOW_RANGE_FIX) ? dist - sp.epsilon - sp.epsilon : dist - sp.epsilon;
                rec.nee = 1;
                rec.lgeom = sp.emission ? lgeom : 0xFFFFFFFFu;
                rec.kl = l3.w;
                rec.lint = lint;
                rec.w = mis2;
                rec.x = x;
                rec.b0 = bpdf0;
                // contribution = w * thr * albedo * lint * kfac (matte), w * thr * gnee * lint (plastic)
                if (plastic)
                {
                    rec.gnee = brdf * (pi * ndotl * inv_pi / ldotn * (ldotn / lpdf) * float(sp.num_lights));
                }
                else
                {
                    const float kfac = m.scale * inv_pi * pi * ndotl * inv_pi / ldotn * (ldotn / lpdf) * float(sp.num_lights);
                    rec.gnee = { kfac, kfac, kfac };
                }
            }
        }
    }
    float cosp = dot3(nn, refl) / brdf_pdf;
    if (specular || plastic)
        rec.f.spec = src * cosp;
    else
        rec.f.sigma = m.scale * inv_pi * cosp;
    st.thr = st.thr * (src * cosp);
    bool terminate = false;
    if (bounce >= 2 && !(sp.flags & GBRT_PT_NO_RUSSIAN_ROULETTE))
    {
        // Russian roulette (pathtracing.inl:201-213)
        float prob = max_elem(st.thr);
        terminate = gbrt_rng_u01(sp.frame, p, sp.sample, st.k++) > prob;
        st.thr = st.thr / prob;
        rec.rr = prob;
    }
    if (!terminate)
    {
        out.cont = true;
        out.next_o = isect + refl * sp.epsilon;
        out.next_d = refl;
        // last_specular = inter is a specular reflection or transmission
        if (specular)
            st.flags |= kLastSpecular;
        else
            st.flags &= ~kLastSpecular;
    }
    (void)tmin;
    (void)tmax;
}

// pinhole_camera::begin_frame (detail/pinhole_camera.inl:87-97) in float, with
// perspective()'s fovy in radians and aspect = width / height.
camera_basis camera_for(gbrt_camera const& c, uint32_t width, uint32_t height)
{
    auto sub = [](const float* a, const float* b) { return float3{ a[0] - b[0], a[1] - b[1], a[2] - b[2] }; };
    auto dot = [](float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; };
    auto cross = [](float3 u, float3 v) {
        return float3{ u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x };
    };
    auto scale = [](float3 a, float s) { return float3{ a.x * s, a.y * s, a.z * s }; };
    auto normalize = [&](float3 v) { return scale(v, 1.0f / std::sqrt(dot(v, v))); };
    float3 f = normalize(sub(c.eye, c.center));
    float3 up = { c.up[0], c.up[1], c.up[2] };
    float3 s = normalize(cross(up, f));
    float3 u = cross(f, s);
    float fovy = c.fovy_degrees * 1.74532925199432957692369076849e-02f;
    float aspect = float(width) / float(height);
    float th = std::tan(fovy / 2.0f);
    camera_basis b;
    b.eye = { c.eye[0], c.eye[1], c.eye[2] };
    b.U = scale(scale(s, th), aspect);
    b.V = scale(u, th);
    b.W = { -f.x, -f.y, -f.z };
    return b;
}

} // namespace
} // namespace gbrt
