/*
 * oracle.h -- CPU restatement of visionaray's ray-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA path in
 * visionaray_gb300: only tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it.  The product never calls it and has no CPU fallback.
 *
 * Every function restates, in its own code, the algorithm of the visionaray file:line
 * it cites, keeping the exact floating-point operation order (the library is built
 * with -ffp-contract=off, so no multiply-add is fused) so that its results match the
 * reference's CPU path bit for bit.  Parity pin: the restatement is checked against
 * the reference's own CPU code compiled from its headers (oracle/_ref, built by
 * oracle/Makefile where the visionaray sources are present) and against golden
 * vectors in tests/golden that were generated from that build.
 */
#ifndef VISIONARAY_GB300_ORACLE_H
#define VISIONARAY_GB300_ORACLE_H 1

#include <stdint.h>

#include "../include/visionaray_gb300/gbrt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_bvh orc_bvh;

/* binned_sah_builder{}.build(index_bvh<P>{}, tris, n, max_leaf) with object splits
 * only (detail/bvh/sah.h:176-807, detail/bvh/build_top_down.h:27-173).            */
orc_bvh* orc_build_sah(const gbrt_triangle* tris, uint32_t n, int max_leaf_size);

/* CPU lbvh_builder{}.build(index_bvh<P>{}, tris, n, max_leaf): top-down Morton split
 * (detail/bvh/lbvh.h:473-656).  max_leaf_size must be >= 2: with 1, equal adjacent
 * codes make the reference recurse forever (lbvh.h:505-508); NULL is returned.    */
orc_bvh* orc_build_lbvh_cpu(const gbrt_triangle* tris, uint32_t n, int max_leaf_size);

/* The GPU lbvh_builder's result restated on the CPU (detail/bvh/lbvh.h:215-451):
 * Morton codes, stable sort, Karras hierarchy, bottom-up bounds and the collapse into
 * the cuda_index_bvh node layout.                                                  */
orc_bvh* orc_build_karras(const gbrt_triangle* tris, uint32_t n);

uint32_t orc_bvh_num_nodes(const orc_bvh* b);
uint32_t orc_bvh_num_indices(const orc_bvh* b);
uint32_t orc_bvh_depth(const orc_bvh* b);
void     orc_bvh_copy(const orc_bvh* b, gbrt_bvh_node* nodes, uint32_t* indices);
void     orc_bvh_free(orc_bvh* b);

/* 30-bit Morton codes in input order (detail/bvh/lbvh.h:242-269 and :577-594).     */
void orc_morton_codes(const gbrt_triangle* tris, uint32_t n, uint32_t* codes);

/* Karras inner-node children for sorted codes (detail/bvh/lbvh.h:120-185, 281-330):
 * left[i], right[i] for inner i in [0, n-2]; a value >= n-1 denotes leaf (v-(n-1)). */
void orc_karras_children(const uint32_t* sorted_codes, uint32_t n, int32_t* left, int32_t* right);

/* sah_cost(bvh, ci, cl, cp) (detail/bvh/statistics.h:34-68).                        */
float orc_sah_cost(const gbrt_bvh_node* nodes, uint32_t num_nodes, float ci, float cl, float cp);

/* Single ray / triangle test (math/intersect.h:176-229); returns the hit flag.     */
/* Two-level instancing (index_bvh_inst_t, bvh.h:678-782; intersect.inl:362-394),
 * brute force over the instances in index order: per instance the ray is mapped with
 * the reference's float inverse of top_left(transform) (matrix3.inl:285-305,
 * matrix4x3.inl:206-219) and traced through that instance's tree as orc_trace does;
 * a hit replaces the best one when strictly closer (is_closer).  hits: gbrt_hit_inst
 * (geom_id 0).                                                                     */
typedef struct orc_instance
{
    const gbrt_bvh_node* nodes;
    uint32_t num_nodes;
    const uint32_t* indices;
    const gbrt_triangle* tris;
    float transform[12];
} orc_instance;
void orc_trace_instances(const orc_instance* instances, uint32_t num_instances, const gbrt_ray* rays,
                         uint64_t nrays, int any_hit, int nthreads, gbrt_hit_inst* hits);

/* bvh_refitter::refit (detail/bvh/refit.h:25-117): out = nodes with every box
 * recomputed from the triangles' (new) bounds, topology unchanged.                 */
void orc_refit(const gbrt_bvh_node* nodes, uint32_t num_nodes, const uint32_t* indices,
               const gbrt_triangle* tris, gbrt_bvh_node* out);

int orc_intersect_triangle(const gbrt_ray* ray, const gbrt_triangle* tri, gbrt_hit* out);

/* Scalar ray / box slab test (math/intersect.h:44-62, no tmin/tmax clamp); returns
 * the hit flag and writes tnear, tfar.                                             */
int orc_intersect_box(const gbrt_ray* ray, const float bmin[3], const float bmax[3], float* tnear,
                      float* tfar);

/* closest_hit / any_hit of rays over one index BVH given by its arrays, with the CPU
 * full-stack traversal (detail/bvh/intersect.inl:51-165).  counters (may be NULL)
 * receives {box tests, triangle tests} summed over all rays.  nthreads <= 0 uses the
 * machine's hardware concurrency.  Returns 0, or -1 if a ray's stack overflowed the
 * reference's 32 entries.                                                          */
int orc_trace(const gbrt_bvh_node* nodes, uint32_t num_nodes, const uint32_t* indices,
              const gbrt_triangle* tris, const gbrt_ray* rays, uint64_t nrays, int any_hit,
              int nthreads, gbrt_hit* hits, uint64_t* counters);

/* Brute force over all triangles (traverse_linear.inl:71-113 over a primitive list). */
void orc_trace_linear(const gbrt_triangle* tris, uint32_t ntris, const gbrt_ray* rays,
                      uint64_t nrays, int any_hit, int nthreads, gbrt_hit* hits);

/* Path tracing (oracle/pathtrace.cpp): one frame's per-pixel average color (RGBA, before
 * the blend) of visionaray's pathtracing::kernel over the index BVH given by its
 * arrays, at the gbrt_rng.h random stream.  mode 0: float, the host's cosf/sinf (the
 * reference build's arithmetic); 1: double (the FP64 oracle); 2: float with the
 * hemisphere sample's cos/sin evaluated in double and rounded once (the CUDA path's
 * arithmetic); mode | 4: the hemisphere sample's two draws in argument order (the
 * order visionaray's device build evaluates them in).  lights: area, point and spot
 * lights (gbrt_light).  counters (may be NULL) receives {closest rays, shadow rays,
 * box tests, triangle tests}.  env (may be NULL): an environment light in place of the
 * ambient light, its d_texels a HOST pointer here.                                   */
void orc_pathtrace(const gbrt_triangle* tris, const gbrt_bvh_node* nodes, uint32_t num_nodes,
                   const uint32_t* indices, const gbrt_material* mats, uint32_t nmat,
                   const gbrt_light* lights, uint32_t nl, const gbrt_camera* cam,
                   const gbrt_pt_params* p, int mode, int nthreads, double* out_rgba,
                   uint64_t* counters, const gbrt_environment* env);

/* Path-replay adjoint of the path tracer at the gbrt_rng.h stream: per-slot gradients
 * of sum(I * img_adj) w.r.t. the albedo / emission parameters (3 per material slot;
 * either may be NULL to use the materials' colors and skip that gradient), written to
 * grad_albedo / grad_emission (3 * nmat doubles each); image (may be NULL) receives
 * the rendered per-pixel average.  fp64 != 0: double arithmetic (the FP64 host
 * adjoint); else float with the CUDA path's cos/sin.                               */
void orc_pathtrace_adjoint(const gbrt_triangle* tris, const gbrt_bvh_node* nodes, uint32_t num_nodes,
                           const uint32_t* indices, const gbrt_material* mats, uint32_t nmat,
                           const gbrt_light* lights, uint32_t nl, const gbrt_camera* cam,
                           const gbrt_pt_params* p, const float* albedo, const float* emission,
                           const double* img_adj, int fp64, int nthreads, double* grad_albedo,
                           double* grad_emission, double* image, const gbrt_environment* env);

#ifdef __cplusplus
}
#endif

#endif
