/*
 * hair_oracle.h -- CPU oracle for the hair pipeline.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of bevy_hair's per-frame compute passes, used by the
 * tests as the parity checker and by bench.py as the timed CPU baseline.  The
 * product (libhairgb.so and the bevy_hair_gb300 package) never links, loads or
 * calls it.
 *
 * Pinning: the reference cannot run here (it is a Rust/wgpu crate; no Rust
 * toolchain and no graphics stack).  The oracle's helper functions are pinned
 * against every known-answer test the reference holds for this path
 * (src/gbuffer.rs:65-104, src/lod.rs:76-134, tests/golden/reference_kat.json).
 * The raster, deep-opacity, shade, filter and composite pixel outputs have no
 * reference test; for them the oracle defines the result ("parity unpinned"
 * beyond the helper KATs).
 *
 * Float semantics the oracle defines (WGSL leaves them to the backend):
 *  - f32 IEEE round-to-nearest, no FMA contraction (-ffp-contract=off), no FTZ;
 *  - expressions evaluate left to right as written in the WGSL source;
 *  - M * v sums columns in order: ((c0*x + c1*y) + c2*z) + c3*w;
 *  - dot = ((ax*bx + ay*by) + az*bz); length = sqrt(dot); inverseSqrt(x) =
 *    1/sqrt(x) with two correctly rounded steps; normalize(v) = v*inverseSqrt;
 *  - mix(a, b, t) = a*(1-t) + b*t;  clamp(x, l, h) = min(max(x, l), h) with
 *    IEEE minNum/maxNum (fminf/fmaxf);
 *  - u32(f)/i32(f) truncate toward zero and saturate; NaN converts to 0;
 *  - i32 add/sub wrap (two's complement);
 *  - control_points_for_lod's pow(2, floor(log2(c - 1))) is evaluated exactly
 *    (c - 1 is an integer in [15, 126]): 2^(index of the highest set bit).
 */
#ifndef HAIR_ORACLE_H
#define HAIR_ORACLE_H

#include <stdint.h>
#include "../include/hairgb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_counts {
    uint64_t samples;        /* DDA samples (camera) or Bresenham visits (DOM) */
    uint64_t cons_min;       /* atomicMin on conservative */
    uint64_t center_min;     /* atomicMin on center */
    uint64_t beta_min;       /* atomicMin on beta */
    uint64_t dom_min;        /* mode 1 atomicMin */
    uint64_t dom_add;        /* mode 2 atomicAdd */
    uint64_t segments;       /* segments drawn (ncp - 1 per ref) */
} oracle_counts;

void oracle_set_threads(int n);
int oracle_get_threads(void);

/* helpers pinned by the reference KATs */
uint32_t oracle_pcg(uint32_t x);
uint64_t oracle_pack_gb(uint32_t depth, uint32_t tx, uint32_t ty, uint32_t u, uint32_t v, uint32_t w, uint32_t ao);
void oracle_unpack_gb(uint64_t word, uint32_t out[7]);
uint32_t oracle_pack_beta(uint32_t depth, float beta);
uint32_t oracle_quantize_depth(float dist, float near_, float far_);
float oracle_dequantize_depth(uint32_t depth, float near_, float far_);
uint32_t oracle_control_points_for_lod(float l);
float oracle_lod_selection(float extent, float screen_h, float lambda);
uint32_t oracle_strand_count_lod(float l, uint32_t strand_count, float delta, int culled);
float oracle_dom_optical_depth(const uint32_t* layers, uint32_t n_layers, float t);
float oracle_depth_correction(float beta);
void oracle_oct_encode(const float n[3], uint32_t out[2]);
void oracle_oct_decode(uint32_t tx, uint32_t ty, float out[3]);

/* passes */
void oracle_clear(uint64_t* center, uint64_t* cons, uint32_t* beta, uint64_t pixels);
void oracle_clear_dom(uint32_t* dom, uint64_t texels);
void oracle_lod(const hg_hair_params* p, const hg_gpu_bundle* bundles, const hg_gpu_layer* layers,
                hg_lod_record* lod_out);
void oracle_scan(const hg_hair_params* p, const hg_lod_record* lod, hg_strand_ref* refs,
                 uint32_t capacity, uint32_t indirect[4]);
/* Control points of one strand as the raster generates them (model space):
 * pos_ao[ncp*4], tan[ncp*4], uvw_ao[ncp*4].  Returns ncp. */
uint32_t oracle_strand_points(const hg_gpu_bundle* bundles, const hg_gpu_layer* layers, const float* style,
                              const hg_strand_ref* ref, float* pos_ao, float* tan, float* uvw_ao);
void oracle_raster(const hg_hair_params* p, const hg_gpu_bundle* bundles, const hg_gpu_layer* layers,
                   const float* style, const hg_strand_ref* refs, uint32_t n_refs,
                   uint64_t* center, uint64_t* cons, uint32_t* beta, uint32_t* dom,
                   const float* scene_depth, oracle_counts* counts);
/* The light probe of shade.wesl:330-427 (hg_env_desc with host texels). */
typedef struct oracle_env {
    const uint32_t* spec;
    uint32_t spec_size, spec_levels;
    const uint32_t* diff;
    uint32_t diff_size, diff_levels;
    float rot[4];
    float intensity;
} oracle_env;

/* mlp: NULL for shade model 0 (Karis fit); else the surrogate's parameters
 * for shade models 1 and 2 (mlp_arch 0, HG_MLP_PARAMS floats) or 3 (mlp_arch
 * 1, HG_MLP_COMPACT_PARAMS floats).  env: NULL without a light probe. */
void oracle_shade(const hg_hair_params* p, const uint64_t* center, const uint32_t* beta, const uint32_t* dom,
                  const hg_light* lights, uint32_t n_lights, uint32_t ortho, float exposure, const float* mlp,
                  uint32_t mlp_arch, const oracle_env* env, float* shaded, float* shaded_depth);
/* One trilinear cubemap sample (RGB9E5 mip chain) for the sampler tests. */
void oracle_sample_cube(const uint32_t* texels, uint32_t size, uint32_t levels, const float dir[3], float lod,
                        float out[3]);
/* The surrogate network on raw inputs (n x 10) -> raw outputs: the 4 x 64
 * network (n x 12 lobes), or the given architecture (0: 4 x 64, n x 12;
 * 1: the compact 2 x 32, n x 3 BSDF channels). */
void oracle_mlp_forward(const float* params, const float* raw, uint32_t n, float* net);
void oracle_mlp_forward_arch(const float* params, uint32_t arch, const float* raw, uint32_t n, float* net);
void oracle_filter(const hg_hair_params* p, const uint64_t* center, const uint64_t* cons,
                   const float* shaded, const float* shaded_depth, float* filtered, float* filtered_depth);
/* hair_shadow.wesl:52-75: light is a ShadowLight (28 floats). */
void oracle_hair_visibility(const float* light, const uint32_t* dom, uint32_t dom_w, uint32_t dom_h,
                            const float* points, uint32_t n, float* out);
/* FP64 hair lobes (marschner.c): in[10] = sin_i, sin_o, cos_phi, sin_phi,
 * sigma_a rgb, beta_m, beta_n, eta -> out[12] = R, TT, TRT, B (rgb each).
 * oracle_lobes_batch model 0: exact azimuthal integrals; 1: shade.wesl's Karis fits. */
void oracle_marschner_lobes(const double in[10], double tilt, double out[12]);
void oracle_karis_lobes(const double in[10], double tilt, double out[12]);
void oracle_lobes_batch(int model, const double* in, unsigned n, double tilt, double* out);
void oracle_composite(const hg_hair_params* p, const float* color_src, const float* depth_src,
                      float* color_dst, float* depth_dst);

#ifdef __cplusplus
}
#endif
#endif
