/*
 * hairgb_bake.h -- C ABI of the hair-mesh baker (host code, C++ with OpenMP).
 *
 * Turns explicit strands (polylines) into the bundle cages the per-frame
 * pipeline generates strands from: GpuBundle / GpuLayer / style buffers as
 * hg_groom_upload takes them (16 layers of four corners and an 8 x 8 x 16
 * style residual volume per bundle).  Replaces the interface of
 * bake_hair_mesh / bake_hair_mesh_with_scalp (src/bake.rs:89-213); the
 * algorithm is this library's own (see csrc/bake.cpp): strands resampled to
 * 16 points, clusters split top-down by 2-means on whole strands until each
 * cage (a principal-axis root parallelogram, least-squares bilinear layers,
 * a regularised least-squares style volume) reproduces its members and its
 * uniform (u, v) fill stays on the strands; ambient occlusion from
 * Beer-Lambert transmittance through a voxel grid of strand density.
 * Deterministic: the same input gives the same bytes.
 */
#ifndef HAIRGB_BAKE_H
#define HAIRGB_BAKE_H

#include <stdint.h>
#include "hairgb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hg_bake_result hg_bake_result;

#define HG_BAKE_AMBIENT_OCCLUSION 1u

/* points: float3[n_points]; strand i is points[first[i] .. first[i]+count[i]).
 * Strands with fewer than two points are left out; every other strand lands
 * in exactly one bundle.  Returns NULL on invalid input (a strand outside the
 * point array). */
hg_bake_result* hg_bake(const float* points, uint32_t n_points, const uint32_t* first, const uint32_t* count,
                        uint32_t n_strands, uint32_t flags);
/* The same with the scalp mesh the strands grow from (bake_hair_mesh_with_scalp):
 * scalp_vertices float3[n_scalp_vertices], scalp_indices u32[n_scalp_indices]
 * (triangles).  Strands whose roots lie within 25 units of the scalp start
 * clustered per connected scalp region, their root quads lie across the scalp
 * normal, and the scalp occludes in the ambient occlusion.  NULL on an index
 * outside the vertex array. */
hg_bake_result* hg_bake_scalp(const float* points, uint32_t n_points, const uint32_t* first, const uint32_t* count,
                              uint32_t n_strands, const float* scalp_vertices, uint32_t n_scalp_vertices,
                              const uint32_t* scalp_indices, uint32_t n_scalp_indices, uint32_t flags);
uint32_t hg_bake_bundle_count(const hg_bake_result* r);
uint32_t hg_bake_layer_count(const hg_bake_result* r);
uint32_t hg_bake_style_count(const hg_bake_result* r);
/* bounds: min xyz then max xyz of the cage corners. */
void hg_bake_copy(const hg_bake_result* r, hg_gpu_bundle* bundles, hg_gpu_layer* layers, float* style,
                  float bounds[6]);
void hg_bake_free(hg_bake_result* r);

#ifdef __cplusplus
}
#endif
#endif
