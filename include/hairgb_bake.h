/*
 * hairgb_bake.h -- C ABI of the hair-mesh baker (host code, C++).
 *
 * Turns explicit strands (polylines) into the bundle cages the per-frame
 * pipeline generates strands from: GpuBundle / GpuLayer / style buffers as
 * GpuGroom::upload expects them.  Replaces bake_hair_mesh
 * (src/bake.rs:89-213) for grooms without a scalp mesh: roots are clustered
 * in a 3-D grid (src/bake.rs:340-397), sparse clusters are absorbed
 * (src/bake.rs:399-440), clusters are split until their cage is coherent
 * (src/bake.rs:977-1061), and corners get baked ambient occlusion
 * (src/bake.rs:1139-1179).
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
 * Returns NULL on invalid input (a strand outside the point array). */
hg_bake_result* hg_bake(const float* points, uint32_t n_points, const uint32_t* first, const uint32_t* count,
                        uint32_t n_strands, uint32_t flags);
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
