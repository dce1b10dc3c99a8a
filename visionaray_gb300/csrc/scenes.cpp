// Deterministic synthetic workloads (see scenes.h).  Compiled with -ffp-contract=off:
// every floating-point expression below is evaluated as written, one IEEE-754
// rounding per operation, on every host architecture.

#include "scenes.h"

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

// SplitMix64 finaliser (Steele, Lea & Flood 2014) used as a counter-based hash.
inline uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

inline uint64_t rng_bits(uint64_t seed, uint64_t stream, uint64_t index)
{
    return mix64(mix64(seed * 0x9E3779B97F4A7C15ull + stream) + index * 0xD1B54A32D192ED03ull);
}

inline float u01f(uint64_t seed, uint64_t stream, uint64_t index)
{
    return float(rng_bits(seed, stream, index) >> 40) * 0x1p-24f;
}

inline double u01d(uint64_t seed, uint64_t stream, uint64_t index)
{
    return double(rng_bits(seed, stream, index) >> 11) * 0x1p-53;
}

constexpr double kPi      = 3.14159265358979311600e+00;
constexpr double kHalfPi  = 1.57079632679489655800e+00;
constexpr double kTwoPi   = 6.28318530717958623200e+00;
constexpr double kTwoPiLo = 2.44929359829470635445e-16;

// sin on [-pi/2, pi/2] from its Taylor series to r^23 in Horner form
// (truncation error below 1e-20 there).
inline double sin_reduced(double r)
{
    double r2 = r * r;
    double acc = 1.0;
    for (int k = 11; k >= 1; --k)
    {
        acc = 1.0 - (r2 / double((2 * k) * (2 * k + 1))) * acc;
    }
    return r * acc;
}

// Portable sine: reduction by 2*pi in two parts, then folding into [-pi/2, pi/2].
inline double det_sin(double x)
{
    double k = std::nearbyint(x / kTwoPi);
    double r = (x - k * kTwoPi) - k * kTwoPiLo;
    if (r > kHalfPi)
    {
        r = kPi - r;
    }
    else if (r < -kHalfPi)
    {
        r = -kPi - r;
    }
    return sin_reduced(r);
}

inline double det_cos(double x)
{
    return det_sin(x + kHalfPi);
}

struct d3
{
    double x, y, z;
};

inline d3 cross(d3 a, d3 b)
{
    return { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x };
}

inline d3 normalize(d3 a)
{
    double l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return { a.x / l, a.y / l, a.z / l };
}

// Cosine-weighted direction about unit normal n from two uniforms; the tangent frame
// is the branchless orthonormal basis of Duff et al., "Building an Orthonormal Basis,
// Revisited" (JCGT 2017).
inline d3 cosine_direction(d3 n, double r1, double r2)
{
    double rad = std::sqrt(r1);
    double phi = kTwoPi * r2;
    double lx = rad * det_cos(phi);
    double ly = rad * det_sin(phi);
    double lz = std::sqrt(1.0 - r1 > 0.0 ? 1.0 - r1 : 0.0);

    double sign = n.z >= 0.0 ? 1.0 : -1.0;
    double a = -1.0 / (sign + n.z);
    double b = n.x * n.y * a;
    d3 t1 = { 1.0 + sign * n.x * n.x * a, sign * b, -sign * n.x };
    d3 t2 = { b, sign + n.y * n.y * a, -n.y };

    d3 d = { lx * t1.x + ly * t2.x + lz * n.x,
             lx * t1.y + ly * t2.y + lz * n.y,
             lx * t1.z + ly * t2.z + lz * n.z };
    return normalize(d);
}

inline void set_tri(gbrt_triangle& t, uint32_t id, uint32_t geom, const float p0[3],
                    const float p1[3], const float p2[3])
{
    t.geom_id = geom;
    t.prim_id = id;
    for (int a = 0; a < 3; ++a)
    {
        t.v1[a] = p0[a];
        t.e1[a] = p1[a] - p0[a];
        t.e2[a] = p2[a] - p0[a];
    }
}

} // namespace

extern "C" float gbrt_scene_u01(uint64_t seed, uint64_t stream, uint64_t index)
{
    return u01f(seed, stream, index);
}

extern "C" void gbrt_scene_soup(uint32_t n, uint64_t seed, float offset, gbrt_triangle* out)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < int64_t(n); ++i)
    {
        float c[3];
        for (int a = 0; a < 3; ++a)
        {
            c[a] = u01f(seed, uint64_t(a), uint64_t(i));
        }
        float p[3][3];
        for (int k = 0; k < 3; ++k)
        {
            for (int a = 0; a < 3; ++a)
            {
                float u = u01f(seed, uint64_t(3 + 3 * k + a), uint64_t(i));
                float o = (2.0f * u - 1.0f) * offset;
                p[k][a] = c[a] + o;
            }
        }
        set_tri(out[i], uint32_t(i), 0u, p[0], p[1], p[2]);
    }
}

extern "C" void gbrt_scene_heightfield(uint32_t grid, uint64_t seed, double base_amplitude,
                                       double base_frequency, int octaves, gbrt_triangle* out)
{
    if (octaves > 16)
    {
        octaves = 16;
    }
    double amp[16], freq[16], dx[16], dy[16], phase[16];
    for (int k = 0; k < octaves; ++k)
    {
        amp[k] = base_amplitude / double(1u << k);
        freq[k] = base_frequency * double(1u << k);
        double theta = kTwoPi * u01d(seed, 100 + uint64_t(k), 0);
        dx[k] = det_cos(theta);
        dy[k] = det_sin(theta);
        phase[k] = kTwoPi * u01d(seed, 200 + uint64_t(k), 0);
    }

    uint64_t nv = uint64_t(grid) + 1;
    std::vector<float> heights(nv * nv);
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < int64_t(nv); ++j)
    {
        double y = double(j) / double(grid);
        for (uint64_t i = 0; i < nv; ++i)
        {
            double x = double(i) / double(grid);
            double h = 0.0;
            for (int k = 0; k < octaves; ++k)
            {
                h = h + amp[k] * det_sin(kTwoPi * freq[k] * (dx[k] * x + dy[k] * y) + phase[k]);
            }
            heights[uint64_t(j) * nv + i] = float(h);
        }
    }

#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < int64_t(grid); ++j)
    {
        for (uint32_t i = 0; i < grid; ++i)
        {
            float x0 = float(double(i) / double(grid));
            float x1 = float(double(i + 1) / double(grid));
            float y0 = float(double(j) / double(grid));
            float y1 = float(double(j + 1) / double(grid));
            float const* h0 = &heights[uint64_t(j) * nv];
            float const* h1 = &heights[uint64_t(j + 1) * nv];
            float p00[3] = { x0, y0, h0[i] };
            float p10[3] = { x1, y0, h0[i + 1] };
            float p11[3] = { x1, y1, h1[i + 1] };
            float p01[3] = { x0, y1, h1[i] };
            uint64_t c = uint64_t(j) * grid + i;
            set_tri(out[2 * c + 0], uint32_t(2 * c + 0), 0u, p00, p10, p11);
            set_tri(out[2 * c + 1], uint32_t(2 * c + 1), 0u, p00, p11, p01);
        }
    }
}

extern "C" void gbrt_rays_pinhole(const float eye[3], const float center[3], const float up[3],
                                  float fovy_degrees, uint32_t w, uint32_t h, gbrt_ray* out)
{
    d3 e = { eye[0], eye[1], eye[2] };
    d3 c = { center[0], center[1], center[2] };
    d3 u = { up[0], up[1], up[2] };
    d3 f = normalize({ e.x - c.x, e.y - c.y, e.z - c.z });
    d3 s = normalize(cross(u, f));
    d3 v = cross(f, s);
    double half = fovy_degrees * (kPi / 180.0) * 0.5;
    double tan_half = det_sin(half) / det_cos(half);
    double aspect = double(w) / double(h);
    d3 U = { s.x * tan_half * aspect, s.y * tan_half * aspect, s.z * tan_half * aspect };
    d3 V = { v.x * tan_half, v.y * tan_half, v.z * tan_half };
    d3 W = { -f.x, -f.y, -f.z };

#pragma omp parallel for schedule(static)
    for (int64_t y = 0; y < int64_t(h); ++y)
    {
        for (uint32_t x = 0; x < w; ++x)
        {
            double sx = (double(x) + 0.5) / double(w);
            double sy = (double(y) + 0.5) / double(h);
            double uu = 2.0 * sx - 1.0;
            double vv = 2.0 * sy - 1.0;
            d3 d = normalize({ U.x * uu + V.x * vv + W.x,
                               U.y * uu + V.y * vv + W.y,
                               U.z * uu + V.z * vv + W.z });
            gbrt_ray& r = out[uint64_t(y) * w + x];
            r.ori[0] = eye[0];
            r.ori[1] = eye[1];
            r.ori[2] = eye[2];
            r.dir[0] = float(d.x);
            r.dir[1] = float(d.y);
            r.dir[2] = float(d.z);
            r.tmin = 0.0f;
            r.tmax = FLT_MAX;
        }
    }
}

extern "C" void gbrt_rays_surface(const gbrt_triangle* tris, uint32_t ntris, uint32_t n_origins,
                                  uint64_t seed, float offset, uint32_t ao_per_origin,
                                  float ao_tmax, gbrt_ray* closest_out, gbrt_ray* ao_out)
{
    if (ntris == 0)
    {
        return;
    }
#pragma omp parallel for schedule(static)
    for (int64_t o = 0; o < int64_t(n_origins); ++o)
    {
        uint64_t ti = uint64_t(u01d(seed, 300, uint64_t(o)) * double(ntris));
        if (ti >= ntris)
        {
            ti = ntris - 1;
        }
        gbrt_triangle const& t = tris[ti];
        double r1 = u01d(seed, 301, uint64_t(o));
        double r2 = u01d(seed, 302, uint64_t(o));
        double sr = std::sqrt(r1);
        double b1 = sr * (1.0 - r2);
        double b2 = sr * r2;
        d3 v1 = { t.v1[0], t.v1[1], t.v1[2] };
        d3 e1 = { t.e1[0], t.e1[1], t.e1[2] };
        d3 e2 = { t.e2[0], t.e2[1], t.e2[2] };
        d3 p = { v1.x + b1 * e1.x + b2 * e2.x, v1.y + b1 * e1.y + b2 * e2.y,
                 v1.z + b1 * e1.z + b2 * e2.z };
        d3 n = normalize(cross(e1, e2));
        if (n.z < 0.0)
        {
            n = { -n.x, -n.y, -n.z };
        }
        float ori[3] = { float(p.x + double(offset) * n.x), float(p.y + double(offset) * n.y),
                         float(p.z + double(offset) * n.z) };

        auto emit = [&](gbrt_ray& r, uint64_t stream, float tmax) {
            d3 d = cosine_direction(n, u01d(seed, stream, uint64_t(o)),
                                    u01d(seed, stream + 1, uint64_t(o)));
            r.ori[0] = ori[0];
            r.ori[1] = ori[1];
            r.ori[2] = ori[2];
            r.dir[0] = float(d.x);
            r.dir[1] = float(d.y);
            r.dir[2] = float(d.z);
            r.tmin = 0.0f;
            r.tmax = tmax;
        };

        if (closest_out)
        {
            emit(closest_out[o], 303, FLT_MAX);
        }
        if (ao_out)
        {
            for (uint32_t k = 0; k < ao_per_origin; ++k)
            {
                emit(ao_out[uint64_t(o) * ao_per_origin + k], 305 + 2 * uint64_t(k), ao_tmax);
            }
        }
    }
}

namespace {

// Regular icosahedron: 12 vertices (0, +-1, +-phi) cyclic, 20 faces.
const double kPhi = 1.61803398874989490253;
const double kIcoVerts[12][3] = {
    { -1, kPhi, 0 }, { 1, kPhi, 0 }, { -1, -kPhi, 0 }, { 1, -kPhi, 0 },
    { 0, -1, kPhi }, { 0, 1, kPhi }, { 0, -1, -kPhi }, { 0, 1, -kPhi },
    { kPhi, 0, -1 }, { kPhi, 0, 1 }, { -kPhi, 0, -1 }, { -kPhi, 0, 1 } };
const int kIcoFaces[20][3] = {
    { 0, 11, 5 }, { 0, 5, 1 }, { 0, 1, 7 }, { 0, 7, 10 }, { 0, 10, 11 },
    { 1, 5, 9 }, { 5, 11, 4 }, { 11, 10, 2 }, { 10, 7, 6 }, { 7, 1, 8 },
    { 3, 9, 4 }, { 3, 4, 2 }, { 3, 2, 6 }, { 3, 6, 8 }, { 3, 8, 9 },
    { 4, 9, 5 }, { 2, 4, 11 }, { 6, 2, 10 }, { 8, 6, 7 }, { 9, 8, 1 } };

void box_quad(gbrt_triangle* out, uint32_t first, const float a[3], const float b[3], const float c[3],
              const float d[3])
{
    // quad a-b-c-d as (a, b, c) and (a, c, d)
    set_tri(out[0], first, first, a, b, c);
    set_tri(out[1], first + 1, first + 1, a, c, d);
}

} // namespace

extern "C" uint64_t gbrt_scene_box_count(uint32_t n_blobs, uint32_t subdiv)
{
    return 14 + uint64_t(n_blobs) * 20 * subdiv * subdiv;
}

extern "C" void gbrt_scene_box(uint32_t n_blobs, uint32_t subdiv, uint64_t seed, float light_y,
                               gbrt_triangle* tris, float* albedo)
{
    // the box: 6 faces of [0,1]^3
    const float P[8][3] = { { 0, 0, 0 }, { 1, 0, 0 }, { 1, 1, 0 }, { 0, 1, 0 },
                            { 0, 0, 1 }, { 1, 0, 1 }, { 1, 1, 1 }, { 0, 1, 1 } };
    const int F[6][4] = { { 0, 1, 2, 3 }, { 5, 4, 7, 6 }, { 4, 0, 3, 7 },
                          { 1, 5, 6, 2 }, { 4, 5, 1, 0 }, { 3, 2, 6, 7 } };
    for (int f = 0; f < 6; ++f)
        box_quad(tris + 2 * f, uint32_t(2 * f), P[F[f][0]], P[F[f][1]], P[F[f][2]], P[F[f][3]]);
    // the light quad just below the ceiling
    const float L[4][3] = { { 0.375f, light_y, 0.375f }, { 0.625f, light_y, 0.375f },
                            { 0.625f, light_y, 0.625f }, { 0.375f, light_y, 0.625f } };
    box_quad(tris + 12, 12u, L[0], L[1], L[2], L[3]);

    const uint64_t per_blob = uint64_t(20) * subdiv * subdiv;
#pragma omp parallel for schedule(dynamic)
    for (int64_t b = 0; b < int64_t(n_blobs); ++b)
    {
        double radius = 0.03 + 0.05 * u01d(seed, 400, uint64_t(b));
        double margin = radius * 1.2;
        d3 c = { margin + (1.0 - 2.0 * margin) * u01d(seed, 401, uint64_t(b)),
                 margin + (1.0 - 2.0 * margin) * u01d(seed, 402, uint64_t(b)),
                 margin + (1.0 - 2.0 * margin) * u01d(seed, 403, uint64_t(b)) };
        double ph[3] = { kTwoPi * u01d(seed, 404, uint64_t(b)), kTwoPi * u01d(seed, 405, uint64_t(b)),
                         kTwoPi * u01d(seed, 406, uint64_t(b)) };
        auto vertex = [&](d3 a, d3 bb, d3 cc, uint32_t i, uint32_t j, float out[3]) {
            double s = double(i) / double(subdiv), t = double(j) / double(subdiv);
            d3 p = { a.x + (bb.x - a.x) * s + (cc.x - a.x) * t, a.y + (bb.y - a.y) * s + (cc.y - a.y) * t,
                     a.z + (bb.z - a.z) * s + (cc.z - a.z) * t };
            d3 d = normalize(p);
            double noise = det_sin(7.0 * d.x + ph[0]) * det_sin(9.0 * d.y + ph[1]) * det_sin(8.0 * d.z + ph[2]);
            double r = radius * (1.0 + 0.15 * noise);
            out[0] = float(c.x + r * d.x);
            out[1] = float(c.y + r * d.y);
            out[2] = float(c.z + r * d.z);
        };
        uint64_t k = 14 + uint64_t(b) * per_blob;
        for (int f = 0; f < 20; ++f)
        {
            d3 A = normalize({ kIcoVerts[kIcoFaces[f][0]][0], kIcoVerts[kIcoFaces[f][0]][1], kIcoVerts[kIcoFaces[f][0]][2] });
            d3 B = normalize({ kIcoVerts[kIcoFaces[f][1]][0], kIcoVerts[kIcoFaces[f][1]][1], kIcoVerts[kIcoFaces[f][1]][2] });
            d3 C = normalize({ kIcoVerts[kIcoFaces[f][2]][0], kIcoVerts[kIcoFaces[f][2]][1], kIcoVerts[kIcoFaces[f][2]][2] });
            for (uint32_t j = 0; j < subdiv; ++j)
            {
                for (uint32_t i = 0; i + j < subdiv; ++i)
                {
                    float p00[3], p10[3], p01[3];
                    vertex(A, B, C, i, j, p00);
                    vertex(A, B, C, i + 1, j, p10);
                    vertex(A, B, C, i, j + 1, p01);
                    set_tri(tris[k], uint32_t(k), uint32_t(k), p00, p10, p01);
                    ++k;
                    if (i + j + 1 < subdiv)
                    {
                        float p11[3];
                        vertex(A, B, C, i + 1, j + 1, p11);
                        set_tri(tris[k], uint32_t(k), uint32_t(k), p10, p11, p01);
                        ++k;
                    }
                }
            }
        }
    }
    if (albedo)
    {
        uint64_t n = gbrt_scene_box_count(n_blobs, subdiv);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < int64_t(n); ++i)
        {
            for (int a = 0; a < 3; ++a)
                albedo[3 * i + a] = (i == 12 || i == 13) ? 0.0f
                                                          : 0.2f + 0.6f * u01f(seed, 410 + uint64_t(a), uint64_t(i));
        }
    }
}
