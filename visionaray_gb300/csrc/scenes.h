/*
 * scenes.h -- deterministic synthetic workloads for the ray-tracing hot path.
 *
 * These generators have no counterpart in visionaray's library: they stand in for
 * the scenes the benchmarks are defined on (random triangle soups, a procedural
 * heightfield, pinhole primary rays, surface-sampled secondary rays).  Every value
 * comes from a counter-based hash of (seed, stream, index) and from IEEE-754 basic
 * operations only (+ - * / sqrt, no fused multiply-add, no libm transcendental), so
 * x86-64 and AArch64 hosts produce bit-identical triangles and rays.  The library is
 * compiled with -ffp-contract=off for that reason.
 */
#ifndef VISIONARAY_GB300_SCENES_H
#define VISIONARAY_GB300_SCENES_H 1

#include <stdint.h>

#include "../../include/visionaray_gb300/gbrt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Random triangle soup: triangle i has its centre uniform in [0,1]^3 and three vertex
 * offsets uniform in [-offset, offset]^3; v1 = c + o0, e1 = o1 - o0 style edges
 * computed from the float vertices.  prim_id = i, geom_id = 0.                     */
void gbrt_scene_soup(uint32_t n, uint64_t seed, float offset, gbrt_triangle* out);

/* Heightfield over [0,1]^2 (z up): grid x grid cells, two triangles per cell, heights
 * a sum of `octaves` sines along seeded random directions with seeded phases,
 * amplitude halving and frequency doubling per octave.  2*grid*grid triangles;
 * triangle 2c is (P00,P10,P11) and 2c+1 is (P00,P11,P01) of cell c = j*grid + i.
 * prim_id = triangle index, geom_id = 0.                                           */
void gbrt_scene_heightfield(uint32_t grid, uint64_t seed, double base_amplitude,
                            double base_frequency, int octaves, gbrt_triangle* out);

/* Pinhole primary rays, one per pixel centre, in the semantics of visionaray's
 * pinhole_camera (look_at + perspective, detail/pinhole_camera.inl:87-120):
 * ray index y*w + x, tmin = 0, tmax = FLT_MAX.                                     */
void gbrt_rays_pinhole(const float eye[3], const float center[3], const float up[3],
                       float fovy_degrees, uint32_t w, uint32_t h, gbrt_ray* out);

/* Secondary rays from surface points: origin o picks a triangle uniformly, a uniform
 * point on it, and offsets it by `offset` along the normal (the normal flipped to
 * +z).  closest_out[o] gets one cosine-weighted direction with tmax = FLT_MAX;
 * ao_out[o*ao_per_origin + k] gets ao_per_origin further cosine-weighted directions
 * with tmax = ao_tmax.  Either output may be NULL.                                  */
void gbrt_rays_surface(const gbrt_triangle* tris, uint32_t ntris, uint32_t n_origins,
                       uint64_t seed, float offset, uint32_t ao_per_origin, float ao_tmax,
                       gbrt_ray* closest_out, gbrt_ray* ao_out);

/* Closed unit box with a ceiling quad light and noisy icosphere blobs (the path-
 * tracing scene).  Layout: triangles 0..11 the box [0,1]^3, 12..13 the light quad
 * (0.375..0.625 in x and z, at y = light_y), then n_blobs blobs of 20*subdiv^2
 * triangles each: a geodesic sphere (each icosahedron face cut into subdiv^2
 * triangles) of radius uniform in [0.03, 0.08], radially displaced by up to 15% with
 * a smooth seeded noise, centred uniformly inside the box.  geom_id = prim_id =
 * triangle index.  Writes gbrt_scene_box_count() triangles to `tris`; `albedo` (3
 * floats per triangle, may be NULL) gets per-triangle albedo uniform in [0.2, 0.8]
 * (the light quad's entries are 0).                                                */
uint64_t gbrt_scene_box_count(uint32_t n_blobs, uint32_t subdiv);
void gbrt_scene_box(uint32_t n_blobs, uint32_t subdiv, uint64_t seed, float light_y,
                    gbrt_triangle* tris, float* albedo);

/* Wavefront OBJ ingestion (the reference viewer's load_obj, src/common/
 * obj_loader.cpp): vertices, faces as triangle fans with 1-based or negative
 * indices, degenerate triangles rejected, prim_id = running index, geom_id = the
 * material slot activated by the last known "usemtl" (names from the files of
 * "mtllib").  Writes up to `capacity` triangles to out (may be NULL) and returns the
 * triangle count, -1 when the file cannot be read.                               */
int64_t gbrt_obj_load(const char* path, gbrt_triangle* out, uint64_t capacity);
/* The material slots of that file as matte (Kd) or emissive (Ke != 0) materials, one
 * per activated usemtl (a single default slot when there is none); returns the slot
 * count, -1 when the file cannot be read.                                          */
int64_t gbrt_obj_materials(const char* path, gbrt_material* out, uint64_t capacity);

/* Stanford PLY ingestion (the reference viewer's load_ply, src/common/
 * ply_loader.cpp): the vertex element's x, y, z and the face element's
 * vertex_indices, triangles (v1, e1, e2) without a degeneracy test, prim_id = running
 * index, geom_id = 0; faces of more than three vertices as fans.  ascii and binary
 * (either byte order) bodies.  Writes up to `capacity` triangles to out (may be NULL)
 * and returns the triangle count, -1 when the file cannot be read or is malformed
 * (including a face index outside the vertex list).                               */
int64_t gbrt_ply_load(const char* path, gbrt_triangle* out, uint64_t capacity);

/* Uniform float in [0,1) of the counter-based generator used above (exposed so that
 * tests can reproduce any value).                                                  */
float gbrt_scene_u01(uint64_t seed, uint64_t stream, uint64_t index);

#ifdef __cplusplus
}
#endif

#endif
