/*
 * hair_oracle.c -- CPU oracle for the hair pipeline.  TEST INFRASTRUCTURE ONLY.
 *
 * Restates the reference's per-frame compute passes in plain C so that the
 * tests can check the CUDA library against it and bench.py can time it as the
 * CPU baseline.  Nothing in the product links or loads this file.
 * Float semantics are defined in hair_oracle.h; build with
 * -O2 -ffp-contract=off (see oracle/Makefile).  Integer outputs are made with
 * commutative atomic min/add, so the multi-threaded result equals the serial one.
 *
 * Parity status: helper functions pinned by the reference KATs
 * (src/gbuffer.rs:65-104, src/lod.rs:76-134); pass outputs unpinned (no
 * reference test covers them) and defined here.
 */
#include "hair_oracle.h"

#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ config */

static int g_threads = 0;

void oracle_set_threads(int n) { g_threads = n; }

int oracle_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ vectors */

typedef struct { float x, y; } v2;
typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } v4;

static inline v2 V2(float x, float y) { v2 r = {x, y}; return r; }
static inline v3 V3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v4 V4(float x, float y, float z, float w) { v4 r = {x, y, z, w}; return r; }
static inline v3 xyz(v4 a) { return V3(a.x, a.y, a.z); }
static inline v3 ld3(const float* p) { return V3(p[0], p[1], p[2]); }
static inline v4 ld4(const float* p) { return V4(p[0], p[1], p[2], p[3]); }

static inline v2 add2(v2 a, v2 b) { return V2(a.x + b.x, a.y + b.y); }
static inline v2 sub2(v2 a, v2 b) { return V2(a.x - b.x, a.y - b.y); }
static inline v2 mul2s(v2 a, float s) { return V2(a.x * s, a.y * s); }
static inline float dot2(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
static inline float len2(v2 a) { return sqrtf(dot2(a, a)); }

static inline v3 add3(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 mul3s(v3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline v3 div3(v3 a, v3 b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline v3 div3s(v3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
static inline v3 spl3(float s) { return V3(s, s, s); }
static inline float dot3(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline float len3(v3 a) { return sqrtf(dot3(a, a)); }
static inline v3 max3s(v3 a, float s) { return V3(fmaxf(a.x, s), fmaxf(a.y, s), fmaxf(a.z, s)); }
static inline v3 min3s(v3 a, float s) { return V3(fminf(a.x, s), fminf(a.y, s), fminf(a.z, s)); }
static inline v3 cross3(v3 a, v3 b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

static inline float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
static inline float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
static inline v2 mix2(v2 a, v2 b, float t) { return V2(mixf(a.x, b.x, t), mixf(a.y, b.y, t)); }
static inline v3 mix3(v3 a, v3 b, float t) {
    return V3(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t));
}
static inline float inverse_sqrt(float x) { return 1.0f / sqrtf(x); }
static inline v3 normalize3(v3 v) { return mul3s(v, inverse_sqrt(dot3(v, v))); }

/* common.wgsl:144-150 */
static inline v3 safe_normalize(v3 v) {
    float l2 = dot3(v, v);
    if (l2 < 1e-10f) return V3(0.0f, 1.0f, 0.0f);
    return mul3s(v, inverse_sqrt(l2));
}

/* WGSL u32(f32) / i32(f32): truncate, saturate, NaN -> 0. */
static inline uint32_t f2u(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)f;
}
static inline int32_t f2i(float f) {
    if (f != f) return 0;
    if (f <= -2147483648.0f) return INT32_MIN;
    if (f >= 2147483648.0f) return INT32_MAX;
    return (int32_t)f;
}
static inline int32_t iadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t isub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t iabs(int32_t a) { return a < 0 ? (int32_t)(0u - (uint32_t)a) : a; }

/* Column-major M * v, columns summed in order. */
static inline v4 mat_mul(const float* m, v4 v) {
    v4 r;
    r.x = ((m[0] * v.x + m[4] * v.y) + m[8] * v.z) + m[12] * v.w;
    r.y = ((m[1] * v.x + m[5] * v.y) + m[9] * v.z) + m[13] * v.w;
    r.z = ((m[2] * v.x + m[6] * v.y) + m[10] * v.z) + m[14] * v.w;
    r.w = ((m[3] * v.x + m[7] * v.y) + m[11] * v.z) + m[15] * v.w;
    return r;
}

/* ------------------------------------------------------------------ atomics */

static inline void amin64(uint64_t* p, uint64_t v) {
    uint64_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (v < cur && !__atomic_compare_exchange_n(p, &cur, v, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
}
static inline void amin32(uint32_t* p, uint32_t v) {
    uint32_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (v < cur && !__atomic_compare_exchange_n(p, &cur, v, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
}

/* ------------------------------------------------------------------ common.wgsl */

#define LAYER_COUNT 16u
#define STYLE_U 8u
#define STYLE_V 8u
#define STYLE_W 16u
#define DOM_LAYERS 16u
#define DOM_EMPTY 0xffffffffu
#define PI_F 3.14159265f
#define EMPTY_U64 0xffffffffffffffffull

/* common.wgsl:56-60 */
uint32_t oracle_pcg(uint32_t input) {
    uint32_t state = input * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

/* common.wgsl:62-66 */
static inline v2 pcg_uv(uint32_t seed) {
    uint32_t a = oracle_pcg(seed);
    uint32_t b = oracle_pcg(a ^ 0x9e3779b9u);
    const float s = 1.0f / 4294967296.0f;
    return V2((float)a * s, (float)b * s);
}

/* common.wgsl:68-76 */
uint64_t oracle_pack_gb(uint32_t depth, uint32_t tx, uint32_t ty, uint32_t u, uint32_t v, uint32_t w, uint32_t ao) {
    uint64_t high = (uint64_t)((depth << 8u) | (tx & 0xffu));
    uint64_t low = (uint64_t)(((ty & 0xffu) << 24u) | ((u & 0x3fu) << 18u) | ((v & 0x3fu) << 12u) |
                              ((w & 0x3fu) << 6u) | (ao & 0x3fu));
    return (high << 32u) | low;
}

/* common.wgsl:94-104: depth, tx, ty, u, v, w, ao */
void oracle_unpack_gb(uint64_t word, uint32_t out[7]) {
    uint32_t low = (uint32_t)(word & 0xffffffffull);
    uint32_t high = (uint32_t)(word >> 32u);
    out[0] = high >> 8u;
    out[1] = high & 0xffu;
    out[2] = low >> 24u;
    out[3] = (low >> 18u) & 0x3fu;
    out[4] = (low >> 12u) & 0x3fu;
    out[5] = (low >> 6u) & 0x3fu;
    out[6] = low & 0x3fu;
}

static inline int is_empty(uint64_t word) { return ((uint32_t)(word >> 32u) >> 8u) == 0x00ffffffu; }

/* raster.wgsl:113-114 */
uint32_t oracle_pack_beta(uint32_t depth, float beta) {
    uint32_t q = f2u(clampf(beta, 0.0f, 1.0f) * 255.0f + 0.5f);
    return (depth << 8u) | q;
}

/* common.wgsl:110-113 */
uint32_t oracle_quantize_depth(float dist, float near_, float far_) {
    float q = clampf((dist - near_) / fmaxf(far_ - near_, 1e-3f), 0.0f, 1.0f);
    uint32_t r = f2u(q * 16777214.0f);
    return r < 0x00fffffeu ? r : 0x00fffffeu;
}

/* common.wgsl:115-117 */
float oracle_dequantize_depth(uint32_t depth, float near_, float far_) {
    return mixf(near_, far_, (float)depth / 16777214.0f);
}

/* common.wgsl:119-130 */
void oracle_oct_encode(const float nin[3], uint32_t out[2]) {
    v3 n = normalize3(V3(nin[0], nin[1], nin[2]));
    float denom = (fabsf(n.x) + fabsf(n.y)) + fabsf(n.z);
    float dm = fmaxf(denom, 1e-6f);
    v2 p = V2(n.x / dm, n.y / dm);
    if (n.z < 0.0f) {
        v2 old = p;
        p.x = (1.0f - fabsf(old.y)) * (old.x >= 0.0f ? 1.0f : -1.0f);
        p.y = (1.0f - fabsf(old.x)) * (old.y >= 0.0f ? 1.0f : -1.0f);
    }
    float ex = clampf(p.x * 0.5f + 0.5f, 0.0f, 1.0f);
    float ey = clampf(p.y * 0.5f + 0.5f, 0.0f, 1.0f);
    out[0] = f2u(ex * 255.0f + 0.5f);
    out[1] = f2u(ey * 255.0f + 0.5f);
}

/* common.wgsl:132-142 */
void oracle_oct_decode(uint32_t tx, uint32_t ty, float out[3]) {
    float ex = (float)tx / 255.0f, ey = (float)ty / 255.0f;
    float fx = ex * 2.0f - 1.0f, fy = ey * 2.0f - 1.0f;
    v3 n = V3(fx, fy, (1.0f - fabsf(fx)) - fabsf(fy));
    if (n.z < 0.0f) {
        float ox = n.x, oy = n.y;
        n.x = (1.0f - fabsf(oy)) * (ox >= 0.0f ? 1.0f : -1.0f);
        n.y = (1.0f - fabsf(ox)) * (oy >= 0.0f ? 1.0f : -1.0f);
    }
    n = normalize3(n);
    out[0] = n.x;
    out[1] = n.y;
    out[2] = n.z;
}

static inline v3 oct_decode_v(uint32_t tx, uint32_t ty) {
    float o[3];
    oracle_oct_decode(tx, ty, o);
    return V3(o[0], o[1], o[2]);
}

/* common.wgsl:152-166 */
static inline v3 calc_tangent(uint32_t idx, uint32_t count, v3 prev, v3 curr, v3 next) {
    v3 dir;
    float scale;
    if (idx == 0u) {
        dir = safe_normalize(sub3(next, curr));
        scale = len3(sub3(next, curr));
    } else if (idx + 1u >= count) {
        dir = safe_normalize(sub3(curr, prev));
        scale = len3(sub3(curr, prev));
    } else {
        dir = safe_normalize(sub3(next, prev));
        scale = len3(sub3(next, prev)) * 0.5f;
    }
    return mul3s(dir, fmaxf(scale, 1e-4f));
}

/* common.wgsl:168-176 */
static inline v3 hermite(v3 p0, v3 p1, v3 m0, v3 m1, float t) {
    float t2 = t * t;
    float t3 = t2 * t;
    float h00 = (2.0f * t3 - 3.0f * t2) + 1.0f;
    float h10 = (t3 - 2.0f * t2) + t;
    float h01 = -2.0f * t3 + 3.0f * t2;
    float h11 = t3 - t2;
    return add3(add3(add3(mul3s(p0, h00), mul3s(m0, h10)), mul3s(p1, h01)), mul3s(m1, h11));
}

/* common.wgsl:178-182 (vec4) */
static inline v4 bilinear4(v4 c00, v4 c10, v4 c01, v4 c11, v2 uv) {
    float u = uv.x, v = uv.y;
    float w00 = (1.0f - u) * (1.0f - v), w10 = u * (1.0f - v), w01 = (1.0f - u) * v, w11 = u * v;
    v4 r;
    r.x = ((c00.x * w00 + c10.x * w10) + c01.x * w01) + c11.x * w11;
    r.y = ((c00.y * w00 + c10.y * w10) + c01.y * w01) + c11.y * w11;
    r.z = ((c00.z * w00 + c10.z * w10) + c01.z * w01) + c11.z * w11;
    r.w = ((c00.w * w00 + c10.w * w10) + c01.w * w01) + c11.w * w11;
    return r;
}

/* common.wgsl:184-191 */
static inline uint32_t quant63(float c) {
    uint32_t q = f2u(clampf(c, 0.0f, 1.0f) * 63.0f + 0.5f);
    return q > 63u ? 63u : q;
}

/* common.wgsl:197-203 */
static inline v3 to_world(const hg_hair_params* p, v3 q) {
    return xyz(mat_mul(p->world_from_model, V4(q.x, q.y, q.z, 1.0f)));
}
static inline v3 dir_world(const hg_hair_params* p, v3 d) {
    return safe_normalize(xyz(mat_mul(p->world_from_model, V4(d.x, d.y, d.z, 0.0f))));
}

/* common.wgsl:205-219 */
typedef struct { v2 screen; float view_dist; float clip_depth; int in_front; } projected;

static inline projected project_world(const hg_hair_params* p, v3 world) {
    v4 clip = mat_mul(p->clip_from_world, V4(world.x, world.y, world.z, 1.0f));
    float w = fmaxf(clip.w, 1e-5f);
    float nx = clip.x / w, ny = clip.y / w, nz = clip.z / w;
    projected r;
    r.screen.x = (nx * 0.5f + 0.5f) * p->screen[0];
    r.screen.y = (1.0f - (ny * 0.5f + 0.5f)) * p->screen[1];
    r.view_dist = dot3(sub3(world, ld3(p->camera_pos)), ld3(p->camera_forward));
    r.clip_depth = nz;
    r.in_front = clip.w > 0.0f && r.view_dist > p->screen[2] * 0.5f;
    return r;
}

/* common.wgsl:221-229 */
static inline v3 reconstruct_world(const hg_hair_params* p, int32_t px, int32_t py, float view_dist) {
    float ux = ((float)px + 0.5f) / fmaxf(p->screen[0], 1.0f);
    float uy = ((float)py + 0.5f) / fmaxf(p->screen[1], 1.0f);
    float ndx = ux * 2.0f - 1.0f;
    float ndy = (1.0f - uy) * 2.0f - 1.0f;
    v4 far_h = mat_mul(p->world_from_clip, V4(ndx, ndy, 0.0f, 1.0f));
    float fw = fmaxf(far_h.w, 1e-5f);
    v3 far_p = V3(far_h.x / fw, far_h.y / fw, far_h.z / fw);
    v3 cam = ld3(p->camera_pos);
    v3 dir = sub3(far_p, cam);
    float denom = fmaxf(dot3(dir, ld3(p->camera_forward)), 1e-4f);
    return add3(cam, mul3s(dir, view_dist / denom));
}

/* common.wgsl:231-238 with the power-of-two snap evaluated exactly. */
uint32_t oracle_control_points_for_lod(float l) {
    float c_raw = fmaxf(floorf(sqrtf(clampf(l, 0.0f, 1.0f)) * 127.0f), (float)LAYER_COUNT);
    if (c_raw < 3.0f) return f2u(fmaxf(c_raw, 2.0f));
    uint32_t c1 = f2u(c_raw - 1.0f);
    uint32_t k = 31u - (uint32_t)__builtin_clz(c1);
    uint32_t snapped = (1u << k) + 1u;
    return snapped < 127u ? snapped : 127u;
}

/* lod.wgsl:47-55 (Eq. 2): L from the screen-space AABB diagonal; src/lod.rs:5-11. */
float oracle_lod_selection(float extent, float screen_h, float lambda) {
    return clampf(extent / fmaxf(screen_h, 1.0f) * lambda, 0.0f, 1.0f);
}

/* lod.wgsl:49-53 (Eq. 1); src/lod.rs:13-21. */
uint32_t oracle_strand_count_lod(float l, uint32_t strand_count, float delta, int culled) {
    if (culled) return 0u;
    float n = (float)strand_count;
    float raw = ceilf(l * (n + delta));
    return f2u(clampf(raw, 1.0f, n));
}

/* shade.wesl:246-260; src/lod.rs:46-57. */
float oracle_dom_optical_depth(const uint32_t* layers, uint32_t n_layers, float t) {
    float occ = 0.0f;
    for (uint32_t slice = 0; slice < n_layers; ++slice) {
        float count = (float)layers[slice];
        float i = (float)slice;
        if (i + 1.0f <= t) {
            occ += count;
        } else if (i < t) {
            occ += count * (t - i);
        }
    }
    return occ;
}

/* shade.wesl:296-298 (Eq. 8); src/lod.rs:33-39. */
float oracle_depth_correction(float beta) { return -logf(fmaxf(beta, 1e-4f)); }

/* ------------------------------------------------------------------ clear passes */

/* clear.wgsl:7-16 */
void oracle_clear(uint64_t* center, uint64_t* cons, uint32_t* beta, uint64_t pixels) {
    for (uint64_t i = 0; i < pixels; ++i) {
        center[i] = EMPTY_U64;
        cons[i] = EMPTY_U64;
        beta[i] = 0xffffffffu;
    }
}

/* clear_dom.wgsl:8-21: the first W*H words are front depths, the rest counters. */
void oracle_clear_dom(uint32_t* dom, uint64_t texels) {
    for (uint64_t i = 0; i < texels; ++i) dom[i] = DOM_EMPTY;
    memset(dom + texels, 0, (size_t)texels * DOM_LAYERS * sizeof(uint32_t));
}

/* ------------------------------------------------------------------ lod / scan */

/* lod.wgsl:6-59 */
void oracle_lod(const hg_hair_params* p, const hg_gpu_bundle* bundles, const hg_gpu_layer* layers,
                hg_lod_record* lod_out) {
    uint32_t count = p->pass_mode[1];
    for (uint32_t b = 0; b < count; ++b) {
        hg_gpu_bundle bundle = bundles[b];
        v2 mn = V2(1e20f, 1e20f), mx = V2(-1e20f, -1e20f);
        int any_front = 0, any_point = 0;
        for (uint32_t layer = 0; layer < LAYER_COUNT; ++layer) {
            for (uint32_t corner = 0; corner < 4u; ++corner) {
                const hg_gpu_layer* vert = &layers[bundle.layer_offset + layer * 4u + corner];
                v3 world = to_world(p, ld3(vert->pos_ao));
                v4 clip = mat_mul(p->clip_from_world, V4(world.x, world.y, world.z, 1.0f));
                float dist = dot3(sub3(world, ld3(p->camera_pos)), ld3(p->camera_forward));
                if (clip.w > 0.0f && dist > 0.0f) any_front = 1;
                projected pr = project_world(p, world);
                mn.x = fminf(mn.x, pr.screen.x);
                mn.y = fminf(mn.y, pr.screen.y);
                mx.x = fmaxf(mx.x, pr.screen.x);
                mx.y = fmaxf(mx.y, pr.screen.y);
                any_point = 1;
            }
        }
        int culled = !any_point || !any_front || mx.x < 0.0f || mx.y < 0.0f || mn.x > p->screen[0] ||
                     mn.y > p->screen[1];
        uint32_t n_lod = 0u, cps = LAYER_COUNT;
        if (!culled) {
            if (p->pass_mode[3] == 1u) {
                n_lod = bundle.strand_count;
                cps = oracle_control_points_for_lod(1.0f);
            } else if (p->flags[0] == 0u) {
                n_lod = bundle.strand_count;
                cps = 127u;
            } else {
                float diag = len2(sub2(mx, mn));
                float l = clampf(diag / fmaxf(p->screen[1], 1.0f) * p->appearance[2], 0.0f, 1.0f);
                float delta = (float)oracle_pcg(b ^ 0x9e3779b9u) * (1.0f / 4294967296.0f);
                float n = (float)bundle.strand_count;
                float raw = ceilf(l * (n + delta));
                n_lod = f2u(clampf(raw, 1.0f, n));
                cps = oracle_control_points_for_lod(l);
            }
        }
        lod_out[b].n_lod = n_lod;
        lod_out[b].control_points = cps;
        lod_out[b].strand_count = bundle.strand_count;
        lod_out[b].pad = 0u;
    }
}

/* scan.wgsl:6-24 */
void oracle_scan(const hg_hair_params* p, const hg_lod_record* lod, hg_strand_ref* refs, uint32_t capacity,
                 uint32_t indirect[4]) {
    uint32_t total = 0u;
    uint32_t count = p->pass_mode[1];
    for (uint32_t b = 0; b < count; ++b) {
        hg_lod_record rec = lod[b];
        for (uint32_t s = 0; s < rec.n_lod; ++s) {
            if (total >= capacity) break;
            refs[total].bundle = b;
            refs[total].strand = s;
            refs[total].n_lod = rec.n_lod;
            refs[total].control_points = rec.control_points;
            total += 1u;
        }
    }
    indirect[0] = total;
    indirect[1] = 1u;
    indirect[2] = 1u;
}

/* ------------------------------------------------------------------ strand generation */

/* raster.wgsl:34-60 */
static inline v3 sample_style(const float* style, uint32_t offset, v2 uv, float w) {
    float u = clampf(uv.x, 0.0f, 1.0f) * (float)(STYLE_U - 1u);
    float v = clampf(uv.y, 0.0f, 1.0f) * (float)(STYLE_V - 1u);
    float ww = clampf(w, 0.0f, 1.0f) * (float)(STYLE_W - 1u);
    uint32_t u0 = f2u(floorf(u)), v0 = f2u(floorf(v)), w0 = f2u(floorf(ww));
    uint32_t u1 = u0 + 1u < STYLE_U - 1u ? u0 + 1u : STYLE_U - 1u;
    uint32_t v1 = v0 + 1u < STYLE_V - 1u ? v0 + 1u : STYLE_V - 1u;
    uint32_t w1 = w0 + 1u < STYLE_W - 1u ? w0 + 1u : STYLE_W - 1u;
    float tu = u - (float)u0, tv = v - (float)v0, tw = ww - (float)w0;
#define STY(iu, iv, iw) ld3(style + 4u * (offset + ((iw) * STYLE_V + (iv)) * STYLE_U + (iu)))
    v3 c000 = STY(u0, v0, w0), c100 = STY(u1, v0, w0), c010 = STY(u0, v1, w0), c110 = STY(u1, v1, w0);
    v3 c001 = STY(u0, v0, w1), c101 = STY(u1, v0, w1), c011 = STY(u0, v1, w1), c111 = STY(u1, v1, w1);
#undef STY
    v3 c00 = mix3(c000, c100, tu);
    v3 c01 = mix3(c010, c110, tu);
    v3 c10 = mix3(c001, c101, tu);
    v3 c11 = mix3(c011, c111, tu);
    return mix3(mix3(c00, c01, tv), mix3(c10, c11, tv), tw);
}

typedef struct {
    uint32_t ncp;
    v4 pos[128];  /* xyz position, w ao */
    v3 tan[128];
    v4 uvw[128];  /* uv, w, ao */
} strand_cps;

/* raster.wgsl:231-317: layer sampling, layer tangents, control points and
 * their tangents.  The lane partition and shuffles of the WGSL only schedule
 * the work; every value equals the array-indexed form used here. */
static void generate_strand(const hg_gpu_bundle* bundles, const hg_gpu_layer* layers, const float* style,
                            const hg_strand_ref* ref, strand_cps* out) {
    hg_gpu_bundle bundle = bundles[ref->bundle];
    v2 uv = pcg_uv(ref->strand ^ (ref->bundle * 0x85ebca6bu));
    v4 lp[LAYER_COUNT];
    v3 lt[LAYER_COUNT];
    for (uint32_t l = 0; l < LAYER_COUNT; ++l) {
        const hg_gpu_layer* c = &layers[bundle.layer_offset + l * 4u];
        lp[l] = bilinear4(ld4(c[0].pos_ao), ld4(c[1].pos_ao), ld4(c[2].pos_ao), ld4(c[3].pos_ao), uv);
    }
    for (uint32_t l = 0; l < LAYER_COUNT; ++l) {
        v3 curr = xyz(lp[l]);
        v3 prev = l == 0u ? curr : xyz(lp[l - 1u]);
        v3 next = l + 1u >= LAYER_COUNT ? curr : xyz(lp[l + 1u]);
        lt[l] = calc_tangent(l, LAYER_COUNT, prev, curr, next);
    }
    uint32_t ncp = ref->control_points;
    ncp = ncp < 2u ? 2u : (ncp > 127u ? 127u : ncp);
    out->ncp = ncp;
    uint32_t den = ncp - 1u > 1u ? ncp - 1u : 1u;
    for (uint32_t idx = 0; idx < ncp; ++idx) {
        /* eval_cp, raster.wgsl:62-75 */
        float w = (float)idx / (float)den;
        float layers_f = w * (float)(LAYER_COUNT - 1u);
        uint32_t i0 = f2u(floorf(layers_f));
        if (i0 > LAYER_COUNT - 1u) i0 = LAYER_COUNT - 1u;
        uint32_t i1 = i0 + 1u < LAYER_COUNT - 1u ? i0 + 1u : LAYER_COUNT - 1u;
        float t = layers_f - (float)i0;
        v3 base = hermite(xyz(lp[i0]), xyz(lp[i1]), lt[i0], lt[i1], t);
        float ao = mixf(lp[i0].w, lp[i1].w, t);
        v3 residual = sample_style(style, bundle.style_offset, uv, w);
        v3 pos = add3(base, residual);
        out->pos[idx] = V4(pos.x, pos.y, pos.z, ao);
        out->uvw[idx] = V4(uv.x, uv.y, w, ao);
    }
    for (uint32_t idx = 0; idx < ncp; ++idx) {
        v3 curr = xyz(out->pos[idx]);
        v3 prev = idx > 0u ? xyz(out->pos[idx - 1u]) : curr;
        v3 next = idx + 1u < ncp ? xyz(out->pos[idx + 1u]) : curr;
        out->tan[idx] = safe_normalize(calc_tangent(idx, ncp, prev, curr, next));
    }
}

uint32_t oracle_strand_points(const hg_gpu_bundle* bundles, const hg_gpu_layer* layers, const float* style,
                              const hg_strand_ref* ref, float* pos_ao, float* tan, float* uvw_ao) {
    strand_cps s;
    generate_strand(bundles, layers, style, ref, &s);
    for (uint32_t i = 0; i < s.ncp; ++i) {
        memcpy(pos_ao + 4 * i, &s.pos[i], 16);
        tan[4 * i + 0] = s.tan[i].x;
        tan[4 * i + 1] = s.tan[i].y;
        tan[4 * i + 2] = s.tan[i].z;
        tan[4 * i + 3] = 0.0f;
        memcpy(uvw_ao + 4 * i, &s.uvw[i], 16);
    }
    return s.ncp;
}

/* ------------------------------------------------------------------ raster */

typedef struct {
    const hg_hair_params* p;
    uint64_t* center;
    uint64_t* cons;
    uint32_t* beta;
    uint32_t* dom;
    const float* scene;
    oracle_counts c;
} raster_ctx;

/* raster.wgsl:77-116 */
static void write_pixel(raster_ctx* rc, int32_t px, int32_t py, float t, v3 p0, v3 p1, v3 t0, v3 t1, v3 uvw0,
                        v3 uvw1, float ao0, float ao1, int center_hit, float beta) {
    const hg_hair_params* p = rc->p;
    int32_t width = f2i(p->screen[0]), height = f2i(p->screen[1]);
    if (px < 0 || py < 0 || px >= width || py >= height) return;
    v3 world = mix3(p0, p1, t);
    v3 tangent = safe_normalize(mix3(t0, t1, t));
    v3 uvw = mix3(uvw0, uvw1, t);
    float ao = mixf(ao0, ao1, t);
    float dist = dot3(sub3(world, ld3(p->camera_pos)), ld3(p->camera_forward));
    if (dist <= p->screen[2]) return;
    uint32_t pix = (uint32_t)py * (uint32_t)width + (uint32_t)px;
    if (rc->scene) {
        v4 clip = mat_mul(p->clip_from_world, V4(world.x, world.y, world.z, 1.0f));
        float clip_depth = clip.z / fmaxf(clip.w, 1e-5f);
        float scene = rc->scene[pix];
        if (p->pass_mode[2] == 1u) {
            if (clip_depth < scene) return;
        } else if (clip_depth > scene) {
            return;
        }
    }
    uint32_t depth = oracle_quantize_depth(dist, p->screen[2], p->screen[3]);
    float tn[3] = {tangent.x, tangent.y, tangent.z};
    uint32_t oct[2];
    oracle_oct_encode(tn, oct);
    uint32_t ao_q = f2u(clampf(ao, 0.0f, 1.0f) * 63.0f + 0.5f);
    if (p->flags[2] == 0u) ao_q = 63u;
    uint64_t payload = oracle_pack_gb(depth, oct[0], oct[1], quant63(uvw.x), quant63(uvw.y), quant63(uvw.z), ao_q);
    amin64(&rc->cons[pix], payload);
    rc->c.cons_min++;
    if (center_hit) {
        amin64(&rc->center[pix], payload);
        amin32(&rc->beta[pix], oracle_pack_beta(depth, beta));
        rc->c.center_min++;
        rc->c.beta_min++;
    }
}

/* raster.wgsl:192-223 */
static void draw_segment(raster_ctx* rc, v3 p0, v3 p1, v3 t0, v3 t1, v3 uvw0, v3 uvw1, float ao0, float ao1,
                         float beta) {
    const hg_hair_params* p = rc->p;
    projected a = project_world(p, p0);
    projected b = project_world(p, p1);
    if (!a.in_front && !b.in_front) return;
    v2 delta = sub2(b.screen, a.screen);
    int32_t steps = f2i(ceilf(fmaxf(fabsf(delta.x), fabsf(delta.y))));
    int32_t n = steps < 1 ? 1 : (steps > 96 ? 96 : steps);
    float diameter = fmaxf(p->appearance[3], 0.05f);
    v2 prev = a.screen;
    for (int32_t i = 0; i <= n; ++i) {
        float t = (float)i / (float)n;
        v2 screen = mix2(a.screen, b.screen, t);
        int32_t pxx = f2i(floorf(screen.x)), pyy = f2i(floorf(screen.y));
        v2 center = V2((float)pxx + 0.5f, (float)pyy + 0.5f);
        v2 seg = sub2(b.screen, a.screen);
        float denom = fmaxf(dot2(seg, seg), 1e-6f);
        float closest = clampf(dot2(sub2(center, a.screen), seg) / denom, 0.0f, 1.0f);
        float dist = len2(sub2(center, add2(a.screen, mul2s(seg, closest))));
        int center_hit = dist <= diameter * 0.5f;
        rc->c.samples++;
        write_pixel(rc, pxx, pyy, t, p0, p1, t0, t1, uvw0, uvw1, ao0, ao1, center_hit, beta);
        if (i > 0) {
            int32_t qx = f2i(floorf(prev.x)), qy = f2i(floorf(prev.y));
            if (qx != pxx && qy != pyy) {
                write_pixel(rc, qx, pyy, t, p0, p1, t0, t1, uvw0, uvw1, ao0, ao1, 0, beta);
                write_pixel(rc, pxx, qy, t, p0, p1, t0, t1, uvw0, uvw1, ao0, ao1, 0, beta);
            }
        }
        prev = screen;
    }
}

/* raster.wgsl:118-148 */
static void write_dom_pixel(raster_ctx* rc, int32_t px, int32_t py, v3 world) {
    const hg_hair_params* p = rc->p;
    int32_t width = f2i(p->screen[0]), height = f2i(p->screen[1]);
    if (px < 0 || py < 0 || px >= width || py >= height) return;
    float near_ = p->screen[2], far_ = p->screen[3];
    float dist = dot3(sub3(world, ld3(p->camera_pos)), ld3(p->camera_forward));
    if (dist <= near_ || dist >= far_) return;
    uint32_t dom_w = f2u(p->dom_info[0]);
    uint32_t pix = (uint32_t)py * dom_w + (uint32_t)px;
    uint32_t q = oracle_quantize_depth(dist, near_, far_);
    if (p->pass_mode[0] == 1u) {
        amin32(&rc->dom[pix], q);
        rc->c.dom_min++;
        return;
    }
    uint32_t front_q = __atomic_load_n(&rc->dom[pix], __ATOMIC_RELAXED);
    if (front_q == DOM_EMPTY) return;
    float z_front = oracle_dequantize_depth(front_q, near_, far_);
    float thickness = fmaxf(far_ - near_, 1e-3f) / (float)DOM_LAYERS;
    float t = fmaxf(dist - z_front, 0.0f) / thickness;
    uint32_t slice = f2u(t);
    if (slice > DOM_LAYERS - 1u) slice = DOM_LAYERS - 1u;
    uint32_t pixels = dom_w * f2u(p->dom_info[1]);
    __atomic_fetch_add(&rc->dom[pixels + pix * DOM_LAYERS + slice], 1u, __ATOMIC_RELAXED);
    rc->c.dom_add++;
}

/* raster.wgsl:150-190 */
static void draw_dom_segment(raster_ctx* rc, v3 p0, v3 p1, int include_start) {
    const hg_hair_params* p = rc->p;
    projected a = project_world(p, p0);
    projected b = project_world(p, p1);
    if (!a.in_front && !b.in_front) return;
    int32_t x0 = f2i(floorf(a.screen.x)), y0 = f2i(floorf(a.screen.y));
    int32_t x1 = f2i(floorf(b.screen.x)), y1 = f2i(floorf(b.screen.y));
    int32_t dx = iabs(isub(x1, x0)), dy = iabs(isub(y1, y0));
    int32_t sx = x0 < x1 ? 1 : -1, sy = y0 < y1 ? 1 : -1;
    int32_t err = isub(dx, dy);
    v2 seg = sub2(b.screen, a.screen);
    float seg_len2 = fmaxf(dot2(seg, seg), 1e-6f);
    int skip = !include_start && (x0 != x1 || y0 != y1);
    for (int step = 0; step < 1024; ++step) {
        if (!skip) {
            v2 center = V2((float)x0 + 0.5f, (float)y0 + 0.5f);
            float t = clampf(dot2(sub2(center, a.screen), seg) / seg_len2, 0.0f, 1.0f);
            rc->c.samples++;
            write_dom_pixel(rc, x0, y0, mix3(p0, p1, t));
        }
        skip = 0;
        if (x0 == x1 && y0 == y1) break;
        int32_t e2 = iadd(err, err);
        if (e2 > (int32_t)(0u - (uint32_t)dy)) {
            err = isub(err, dy);
            x0 = iadd(x0, sx);
        }
        if (e2 < dx) {
            err = iadd(err, dx);
            y0 = iadd(y0, sy);
        }
    }
}

/* raster.wgsl:225-337 over refs[0..n_refs). */
void oracle_raster(const hg_hair_params* p, const hg_gpu_bundle* bundles, const hg_gpu_layer* layers,
                   const float* style, const hg_strand_ref* refs, uint32_t n_refs, uint64_t* center, uint64_t* cons,
                   uint32_t* beta, uint32_t* dom, const float* scene_depth, oracle_counts* counts) {
    oracle_counts total;
    memset(&total, 0, sizeof(total));
    int nthreads = oracle_get_threads();
#pragma omp parallel num_threads(nthreads)
    {
        raster_ctx rc;
        rc.p = p;
        rc.center = center;
        rc.cons = cons;
        rc.beta = beta;
        rc.dom = dom;
        rc.scene = scene_depth;
        memset(&rc.c, 0, sizeof(rc.c));
        strand_cps* s = (strand_cps*)__builtin_alloca(sizeof(strand_cps));
#pragma omp for schedule(dynamic, 64)
        for (int64_t r = 0; r < (int64_t)n_refs; ++r) {
            const hg_strand_ref* ref = &refs[r];
            generate_strand(bundles, layers, style, ref, s);
            hg_gpu_bundle bundle = bundles[ref->bundle];
            uint32_t sc = bundle.strand_count > 1u ? bundle.strand_count : 1u;
            float bval = (float)ref->n_lod / (float)sc;
            for (uint32_t idx = 0; idx + 1u < s->ncp; ++idx) {
                v3 p0 = to_world(p, xyz(s->pos[idx]));
                v3 p1 = to_world(p, xyz(s->pos[idx + 1u]));
                rc.c.segments++;
                if (p->pass_mode[0] != 0u) {
                    draw_dom_segment(&rc, p0, p1, idx == 0u);
                } else {
                    v3 t0 = dir_world(p, s->tan[idx]);
                    v3 t1 = dir_world(p, s->tan[idx + 1u]);
                    draw_segment(&rc, p0, p1, t0, t1, xyz(s->uvw[idx]), xyz(s->uvw[idx + 1u]), s->uvw[idx].w,
                                 s->uvw[idx + 1u].w, bval);
                }
            }
        }
#pragma omp critical
        {
            total.samples += rc.c.samples;
            total.cons_min += rc.c.cons_min;
            total.center_min += rc.c.center_min;
            total.beta_min += rc.c.beta_min;
            total.dom_min += rc.c.dom_min;
            total.dom_add += rc.c.dom_add;
            total.segments += rc.c.segments;
        }
    }
    if (counts) *counts = total;
}

/* ------------------------------------------------------------------ shade */

#define IOR 1.55f
#define DENSITY_FRONT 0.7f
#define DENSITY_BACK 0.7f
#define SCATTER_STEPS 8u

typedef struct { v3 r, tt, trt; } lobes;
typedef struct { v3 alpha, beta; } shape_t;
typedef struct {
    lobes fwd;
    v3 a_f, alpha_f, beta_f2, a_back, delta_b, sigma_b2;
} dual_t;

static inline v3 vexp(v3 a) { return V3(expf(a.x), expf(a.y), expf(a.z)); }
static inline v3 vsqrt(v3 a) { return V3(sqrtf(a.x), sqrtf(a.y), sqrtf(a.z)); }

/* shade.wesl:51-54 */
static inline v3 gaussian3(v3 b, v3 x) {
    v3 bb = max3s(b, 1e-3f);
    float k = sqrtf(2.0f * PI_F);
    v3 num = vexp(div3(mul3(mul3s(x, -0.5f), x), mul3(bb, bb)));
    return div3(num, mul3s(bb, k));
}

/* shade.wesl:56-60 */
static inline float fresnel(float cos_t) {
    float r0 = (1.0f - IOR) / (1.0f + IOR);
    float f0 = r0 * r0;
    return f0 + (1.0f - f0) * powf(1.0f - clampf(cos_t, 0.0f, 1.0f), 5.0f);
}

/* shade.wesl:70-77 */
static inline v3 absorption_from_color(v3 color, float roughness) {
    float b = clampf(roughness, 0.0f, 1.0f);
    float b2 = b * b;
    float b3 = b2 * b;
    float d = ((((5.969f - 0.215f * b) + 2.532f * b2) - 10.73f * b3) + 5.574f * b2 * b2) + 0.245f * b3 * b2;
    v3 c = V3(clampf(color.x, 1e-4f, 1.0f), clampf(color.y, 1e-4f, 1.0f), clampf(color.z, 1e-4f, 1.0f));
    v3 l = V3(logf(c.x) / d, logf(c.y) / d, logf(c.z) / d);
    return mul3(l, l);
}

/* shade.wesl:94-116 */
static inline lobes azimuthal(float cos_theta_d, float cos_phi, v3 sigma_a) {
    float cos_half_phi = sqrtf(clampf(0.5f + 0.5f * cos_phi, 0.0f, 1.0f));
    float n_r = 0.25f * cos_half_phi * fresnel(cos_theta_d * cos_half_phi);
    float eta = 1.19f / cos_theta_d + 0.36f * cos_theta_d;
    float a = 1.0f / eta;
    float h = cos_half_phi * (1.0f + a * (0.6f - 0.8f * cos_phi));
    float f_tt = fresnel(cos_theta_d * sqrtf(clampf(1.0f - h * h, 0.0f, 1.0f)));
    float path = 2.0f * sqrtf(clampf(1.0f - h * h * a * a, 0.0f, 1.0f));
    v3 t_tt = vexp(div3s(mul3s(mul3s(sigma_a, -1.0f), path), cos_theta_d));
    float k_tt = expf(-3.65f * cos_phi - 3.98f) * (1.0f - f_tt) * (1.0f - f_tt);
    float f_trt = fresnel(cos_theta_d * 0.5f);
    v3 t_trt = vexp(div3s(mul3s(mul3s(sigma_a, -1.0f), 3.2f), cos_theta_d));
    float k_trt = expf(17.0f * cos_phi - 16.78f) * (1.0f - f_trt) * (1.0f - f_trt) * f_trt;
    lobes r;
    r.r = spl3(n_r);
    r.tt = mul3s(t_tt, k_tt);
    r.trt = mul3s(t_trt, k_trt);
    return r;
}

/* shade.wesl:124-128 */
static inline shape_t lobe_shape(float roughness, float tilt) {
    float b = clampf(roughness * roughness, 0.02f, 1.0f);
    shape_t s;
    s.alpha = V3(tilt, -0.5f * tilt, -1.5f * tilt);
    s.beta = V3(b, 0.5f * b, 2.0f * b);
    return s;
}

/* shade.wesl:148-150 */
static inline v3 lobe_mean(lobes l, v3 total, v3 q) {
    v3 num = add3(add3(mul3s(l.r, q.x), mul3s(l.tt, q.y)), mul3s(l.trt, q.z));
    return div3(num, max3s(total, 1e-5f));
}

/* shade.wesl:153-190 */
static dual_t dual_scatter(float cos_theta_d, v3 sigma_a, shape_t shape) {
    lobes fwd = {spl3(0.0f), spl3(0.0f), spl3(0.0f)}, back = fwd;
    for (uint32_t i = 0; i < SCATTER_STEPS; ++i) {
        float u = ((float)i + 0.5f) / (float)SCATTER_STEPS;
        lobes b = azimuthal(cos_theta_d, cosf(u * 0.5f * PI_F), sigma_a);
        lobes f = azimuthal(cos_theta_d, cosf((1.0f + u) * 0.5f * PI_F), sigma_a);
        back.r = add3(back.r, b.r);
        back.tt = add3(back.tt, b.tt);
        back.trt = add3(back.trt, b.trt);
        fwd.r = add3(fwd.r, f.r);
        fwd.tt = add3(fwd.tt, f.tt);
        fwd.trt = add3(fwd.trt, f.trt);
    }
    float w = PI_F / (float)SCATTER_STEPS;
    fwd.r = mul3s(fwd.r, w);
    fwd.tt = mul3s(fwd.tt, w);
    fwd.trt = mul3s(fwd.trt, w);
    back.r = mul3s(back.r, w);
    back.tt = mul3s(back.tt, w);
    back.trt = mul3s(back.trt, w);

    dual_t d;
    d.fwd = fwd;
    v3 a_f = min3s(add3(add3(fwd.r, fwd.tt), fwd.trt), 0.95f);
    v3 a_b = add3(add3(back.r, back.tt), back.trt);
    v3 beta2 = mul3(shape.beta, shape.beta);
    v3 alpha_f = lobe_mean(fwd, a_f, shape.alpha);
    v3 beta_f2 = lobe_mean(fwd, a_f, beta2);
    v3 alpha_b = lobe_mean(back, a_b, shape.alpha);
    v3 beta_b2 = lobe_mean(back, a_b, beta2);
    v3 af2 = mul3(a_f, a_f);
    v3 rest = V3(1.0f - af2.x, 1.0f - af2.y, 1.0f - af2.z);
    v3 ab2 = mul3(a_b, a_b);
    v3 ab3 = mul3(ab2, a_b);
    v3 rest3 = mul3(mul3(rest, rest), rest);
    v3 a_back = add3(div3(mul3(a_b, af2), rest), div3(mul3(ab3, af2), rest3));
    v3 rr = mul3(rest, rest);
    v3 t1 = V3(1.0f - 2.0f * ab2.x / rr.x, 1.0f - 2.0f * ab2.y / rr.y, 1.0f - 2.0f * ab2.z / rr.z);
    v3 num2 = add3(mul3s(rr, 2.0f), mul3(mul3s(af2, 4.0f), ab2));
    v3 delta_b = add3(mul3(alpha_b, t1), div3(mul3(alpha_b, num2), rest3));
    v3 beta_f = vsqrt(beta_f2);
    v3 beta_b = vsqrt(beta_b2);
    v3 lead = add3(spl3(1.0f), mul3s(af2, DENSITY_BACK));
    v3 s1 = vsqrt(add3(mul3s(beta_f2, 2.0f), beta_b2));
    v3 s2 = vsqrt(add3(mul3s(beta_f2, 2.0f), mul3s(beta_b2, 3.0f)));
    v3 numer = mul3(lead, add3(mul3(a_b, s1), mul3(ab3, s2)));
    v3 den = max3s(add3(a_b, mul3(ab3, add3(mul3s(beta_f, 2.0f), mul3s(beta_b, 3.0f)))), 1e-5f);
    v3 sigma_b = div3(numer, den);
    d.a_f = a_f;
    d.alpha_f = alpha_f;
    d.beta_f2 = beta_f2;
    d.a_back = a_back;
    d.delta_b = delta_b;
    d.sigma_b2 = mul3(sigma_b, sigma_b);
    return d;
}

/* shade.wesl:228-242: forward-scattered spread through `depth` of hair. */
static v3 spread_term(shape_t shape, const dual_t* ds, float theta_h, float depth, float direct) {
    v3 sigma_f2 = mul3s(ds->beta_f2, depth);
    v3 transmit = V3(powf(ds->a_f.x, depth), powf(ds->a_f.y, depth), powf(ds->a_f.z, depth));
    v3 beta2 = mul3(shape.beta, shape.beta);
    v3 x = spl3(theta_h);
    v3 g0 = gaussian3(vsqrt(add3(spl3(beta2.x), sigma_f2)), sub3(x, spl3(shape.alpha.x)));
    v3 g1 = gaussian3(vsqrt(add3(spl3(beta2.y), sigma_f2)), sub3(x, spl3(shape.alpha.y)));
    v3 g2 = gaussian3(vsqrt(add3(spl3(beta2.z), sigma_f2)), sub3(x, spl3(shape.alpha.z)));
    v3 spread = add3(add3(mul3(g0, ds->fwd.r), mul3(g1, ds->fwd.tt)), mul3(g2, ds->fwd.trt));
    v3 gb = gaussian3(vsqrt(add3(ds->sigma_b2, sigma_f2)), sub3(x, ds->delta_b));
    v3 back_spread = div3s(mul3(mul3s(ds->a_back, 2.0f), gb), PI_F);
    v3 inner = add3(div3s(spread, PI_F), mul3s(back_spread, PI_F * DENSITY_BACK));
    return mul3(mul3s(transmit, (1.0f - direct)), mul3s(inner, DENSITY_FRONT));
}

/* shade.wesl:193-244 */
static v3 hair_bsdf(v3 tangent, v3 view, v3 light, v3 sigma_a, shape_t shape, const dual_t* ds, float shadow,
                    float depth) {
    v3 t = safe_normalize(tangent);
    v3 v = safe_normalize(view);
    v3 l = safe_normalize(light);
    float sin_i = clampf(dot3(t, l), -1.0f, 1.0f);
    float sin_o = clampf(dot3(t, v), -1.0f, 1.0f);
    float theta_i = asinf(sin_i);
    float theta_o = asinf(sin_o);
    float theta_h = theta_i + theta_o;
    float cos_theta_d = fmaxf(cosf(0.5f * fabsf(theta_i - theta_o)), 1e-3f);
    v3 t_i = sub3(l, mul3s(t, sin_i));
    v3 t_o = sub3(v, mul3s(t, sin_o));
    float proj = sqrtf(fmaxf(dot3(t_i, t_i) * dot3(t_o, t_o), 1e-8f));
    float cos_phi = clampf(dot3(t_i, t_o) / proj, -1.0f, 1.0f);

    lobes n = azimuthal(cos_theta_d, cos_phi, sigma_a);
    v3 m = gaussian3(shape.beta, sub3(spl3(theta_h), shape.alpha));
    v3 single = add3(add3(mul3s(n.r, m.x), mul3s(n.tt, m.y)), mul3s(n.trt, m.z));
    v3 g = gaussian3(vsqrt(ds->sigma_b2), sub3(spl3(theta_h), ds->delta_b));
    v3 back = div3s(mul3(mul3s(ds->a_back, 2.0f), g), PI_F);
    float direct = expf(-depth);
    v3 color = mul3s(add3(single, mul3s(back, DENSITY_BACK)), direct);
    if (depth > 1e-3f) color = add3(color, spread_term(shape, ds, theta_h, depth, direct));
    return mul3s(color, shadow);
}

/* ------------------------------------------------- learned surrogate
 * The shade pass's network (hg_mlp.cuh) in FP32 with its FP16 rounding of
 * weights and activations: 10 -> 64 -> 64 -> 64 -> 64 -> 12, ReLU,
 * parameters W1[64][16] b1 W2[64][64] b2 W3 b3 W4 b4 W5[16][64] b5.  The
 * tensor cores sum the products in their own order, so single activations can
 * land one FP16 step apart; comparisons use a tolerance. */

/* Round to the nearest IEEE binary16 value (ties to even), returned as float. */
static float round_half(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    uint32_t sign = u & 0x80000000u, a = u & 0x7fffffffu;
    if (a >= 0x7f800000u) return f;
    float af;
    memcpy(&af, &a, 4);
    float r;
    if (af >= 65520.0f) {
        r = INFINITY;
    } else if (af < 6.103515625e-05f) {          /* below the smallest normal half: steps of 2^-24 */
        const float q = 5.9604644775390625e-08f;
        r = nearbyintf(af / q) * q;
    } else {
        uint32_t lsb = (a >> 13) & 1u;
        a = (a + 0x0fffu + lsb) & ~0x1fffu;
        memcpy(&r, &a, 4);
    }
    uint32_t ru;
    memcpy(&ru, &r, 4);
    ru |= sign;
    memcpy(&r, &ru, 4);
    return r;
}

static void mlp_layer(const float* w, const float* b, const float* in, int n_in, int n_out, int relu, float* out) {
    for (int j = 0; j < n_out; ++j) {
        float acc = b[j];
        for (int k = 0; k < n_in; ++k) acc += round_half(w[j * n_in + k]) * in[k];
        out[j] = relu ? round_half(fmaxf(acc, 0.0f)) : acc;
    }
}

/* arch 0: 10 -> 4 x 64 -> 12 lobes (hg_mlp.cuh); arch 1: the compact
 * 10 -> 2 x 32 -> 3 (hg_mlp_small.cuh), parameters W1[32][16] b1 W2[32][32]
 * b2 W3[16][32] b3, whose outputs are the per-light BSDF rgb
 * (R + TT + TRT + 0.7 B) as log1p(bsdf / 1e-3).  Same normalisation and
 * roundings; net holds 12 (arch 0) or 3 (arch 1) values per sample. */
void oracle_mlp_forward_arch(const float* params, uint32_t arch, const float* raw, uint32_t n, float* net) {
    const int hid = arch == 1u ? 32 : 64, hidden_layers = arch == 1u ? 2 : 4, n_out = arch == 1u ? 3 : 12;
    for (uint32_t s = 0; s < n; ++s) {
        const float* r = raw + 10 * (size_t)s;
        float x[16] = {0}, h0[64], h1[64], y[16];
        x[0] = r[0];
        x[1] = r[1];
        x[2] = r[2];
        x[3] = r[3];
        for (int c = 0; c < 3; ++c) x[4 + c] = (logf(fmaxf(r[4 + c], 1e-6f)) - (-0.91629073f)) * 0.33380820f;
        x[7] = (r[7] - 0.165f) * 7.4074074f;
        x[8] = (r[8] - 0.5f) * 3.3333333f;
        x[9] = (r[9] - 1.55f) * 10.0f;
        for (int k = 0; k < 16; ++k) x[k] = round_half(x[k]);
        const float* p = params;
        mlp_layer(p, p + 16 * hid, x, 16, hid, 1, h0);
        p += 16 * hid + hid;
        float *in = h0, *out = h1;
        for (int l = 1; l < hidden_layers; ++l) {
            mlp_layer(p, p + hid * hid, in, hid, hid, 1, out);
            p += hid * hid + hid;
            float* t = in;
            in = out;
            out = t;
        }
        mlp_layer(p, p + 16 * hid, in, hid, 16, 0, y);
        for (int c = 0; c < n_out; ++c) net[(size_t)n_out * s + c] = y[c];
    }
}

void oracle_mlp_forward(const float* params, const float* raw, uint32_t n, float* net) {
    oracle_mlp_forward_arch(params, 0u, raw, n, net);
}

static inline float mlp_decode(float y) { return 1e-3f * expm1f(fmaxf(y, 0.0f)); }

/* Shade model 1: the network's R, TT, TRT and back-scattering per light; the
 * shadowed forward spread keeps dual_scatter's statistics.  beta_n is the
 * fibre roughness clamped to [0.2, 0.8]. */
static v3 surrogate_bsdf(const float* mlp, uint32_t arch, v3 tangent, v3 view, v3 light, v3 sigma_a, shape_t shape,
                         const dual_t* ds, float depth, float roughness) {
    v3 t = safe_normalize(tangent);
    v3 v = safe_normalize(view);
    v3 l = safe_normalize(light);
    float sin_i = clampf(dot3(t, l), -1.0f, 1.0f);
    float sin_o = clampf(dot3(t, v), -1.0f, 1.0f);
    float theta_h = asinf(sin_i) + asinf(sin_o);
    v3 t_i = sub3(l, mul3s(t, sin_i));
    v3 t_o = sub3(v, mul3s(t, sin_o));
    float proj = sqrtf(fmaxf(dot3(t_i, t_i) * dot3(t_o, t_o), 1e-8f));
    float cos_phi = clampf(dot3(t_i, t_o) / proj, -1.0f, 1.0f);
    float raw[10] = {sin_i, sin_o, cos_phi, sqrtf(fmaxf(1.0f - cos_phi * cos_phi, 0.0f)), sigma_a.x, sigma_a.y,
                     sigma_a.z, shape.beta.x, clampf(roughness, 0.2f, 0.8f), IOR};
    float y[12];
    oracle_mlp_forward_arch(mlp, arch, raw, 1, y);
    v3 bsdf;
    if (arch == 1u) {
        bsdf = V3(mlp_decode(y[0]), mlp_decode(y[1]), mlp_decode(y[2]));
    } else {
        v3 single = V3(mlp_decode(y[0]) + mlp_decode(y[3]) + mlp_decode(y[6]),
                       mlp_decode(y[1]) + mlp_decode(y[4]) + mlp_decode(y[7]),
                       mlp_decode(y[2]) + mlp_decode(y[5]) + mlp_decode(y[8]));
        v3 back = V3(mlp_decode(y[9]), mlp_decode(y[10]), mlp_decode(y[11]));
        bsdf = add3(single, mul3s(back, DENSITY_BACK));
    }
    float direct = expf(-depth);
    v3 color = mul3s(bsdf, direct);
    if (depth > 1e-3f) color = add3(color, spread_term(shape, ds, theta_h, depth, direct));
    return color;
}

static v3 light_lobe(const float* mlp, uint32_t arch, v3 tangent, v3 view, v3 incident, v3 sigma_a, shape_t shape,
                     const dual_t* ds, float depth, float roughness) {
    if (mlp) return surrogate_bsdf(mlp, arch, tangent, view, incident, sigma_a, shape, ds, depth, roughness);
    return hair_bsdf(tangent, view, incident, sigma_a, shape, ds, 1.0f, depth);
}

/* ------------------------------------------------- light probe
 * probe_radiance (shade.wesl:330-427, ENVIRONMENT_MAP): RGB9E5 cubemaps,
 * major-axis face selection, bilinear within a face with clamp-to-edge,
 * linear between mips.  Bevy's GPU sampler also filters across face edges
 * (seamless cubemaps), so parity with the reference here is unpinned; the
 * oracle defines the sampler the kernel follows. */
static v3 rgb9e5(uint32_t w) {
    int e = (int)(w >> 27) - 24;
    return V3(ldexpf((float)(w & 0x1ffu), e), ldexpf((float)((w >> 9) & 0x1ffu), e),
              ldexpf((float)((w >> 18) & 0x1ffu), e));
}

static int cube_face_uv(v3 d, float* s, float* t) {
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z), ma, sc, tc;
    int face;
    if (ax >= ay && ax >= az) {
        face = d.x >= 0.0f ? 0 : 1;
        ma = ax;
        sc = d.x >= 0.0f ? -d.z : d.z;
        tc = -d.y;
    } else if (ay >= az) {
        face = d.y >= 0.0f ? 2 : 3;
        ma = ay;
        sc = d.x;
        tc = d.y >= 0.0f ? d.z : -d.z;
    } else {
        face = d.z >= 0.0f ? 4 : 5;
        ma = az;
        sc = d.z >= 0.0f ? d.x : -d.x;
        tc = -d.y;
    }
    float inv = 1.0f / fmaxf(ma, 1e-20f);
    *s = 0.5f * (sc * inv + 1.0f);
    *t = 0.5f * (tc * inv + 1.0f);
    return face;
}

static v3 cube_bilinear(const uint32_t* level, uint32_t n, int face, float s, float t) {
    float u = s * (float)n - 0.5f, v = t * (float)n - 0.5f;
    float fu = floorf(u), fv = floorf(v), wu = u - fu, wv = v - fv;
    int last = (int)n - 1;
    int x0 = (int)fu, y0 = (int)fv;
    int x1 = x0 + 1, y1 = y0 + 1;
    x0 = x0 < 0 ? 0 : (x0 > last ? last : x0);
    x1 = x1 < 0 ? 0 : (x1 > last ? last : x1);
    y0 = y0 < 0 ? 0 : (y0 > last ? last : y0);
    y1 = y1 < 0 ? 0 : (y1 > last ? last : y1);
    const uint32_t* f = level + (size_t)face * n * n;
    v3 c00 = rgb9e5(f[y0 * n + x0]), c10 = rgb9e5(f[y0 * n + x1]);
    v3 c01 = rgb9e5(f[y1 * n + x0]), c11 = rgb9e5(f[y1 * n + x1]);
    v3 a = add3(mul3s(c00, 1.0f - wu), mul3s(c10, wu));
    v3 b = add3(mul3s(c01, 1.0f - wu), mul3s(c11, wu));
    return add3(mul3s(a, 1.0f - wv), mul3s(b, wv));
}

static v3 sample_cube(const uint32_t* texels, uint32_t size, uint32_t levels, v3 dir, float lod) {
    float s, t;
    int face = cube_face_uv(dir, &s, &t);
    lod = clampf(lod, 0.0f, (float)(levels - 1));
    uint32_t l0 = (uint32_t)lod, l1 = l0 + 1u < levels ? l0 + 1u : levels - 1u;
    float w = lod - (float)l0;
    size_t off = 0;
    for (uint32_t l = 0; l < l0; ++l) {
        size_t n = size >> l ? size >> l : 1;
        off += 6 * n * n;
    }
    uint32_t n0 = size >> l0 ? size >> l0 : 1;
    v3 a = cube_bilinear(texels + off, n0, face, s, t);
    if (l1 == l0 || w <= 0.0f) return a;
    off += 6 * (size_t)n0 * n0;
    v3 b = cube_bilinear(texels + off, size >> l1 ? size >> l1 : 1, face, s, t);
    return add3(mul3s(a, 1.0f - w), mul3s(b, w));
}

void oracle_sample_cube(const uint32_t* texels, uint32_t size, uint32_t levels, const float dir[3], float lod,
                        float out[3]) {
    v3 c = sample_cube(texels, size, levels, V3(dir[0], dir[1], dir[2]), lod);
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
}

/* quat_rotate + the left-handed flip (shade.wesl:329-339) */
static v3 cubemap_dir(const float q[4], v3 dir) {
    v3 qv = V3(q[0], q[1], q[2]);
    v3 t = mul3s(cross3(qv, dir), 2.0f);
    v3 r = add3(add3(dir, mul3s(t, q[3])), cross3(qv, t));
    r.z = -r.z;
    return r;
}

/* scatter_tint (shade.wesl:81-85), luminance (:62-64) */
static v3 scatter_tint(v3 albedo, float shadow) {
    float lum = albedo.x * 0.2126f + albedo.y * 0.7152f + albedo.z * 0.0722f;
    v3 hue = mul3s(albedo, 1.0f / fmaxf(lum, 1e-4f));
    float e = 0.5f - 0.5f * clampf(shadow, 0.0f, 1.0f);
    return V3(powf(hue.x, e), powf(hue.y, e), powf(hue.z, e));
}

static v3 probe_radiance(const oracle_env* env, v3 tangent, v3 fiber_n, v3 view, v3 albedo, float roughness,
                         float tilt) {
    float theta_o = asinf(clampf(dot3(tangent, view), -1.0f, 1.0f));
    float theta_i = tilt - theta_o;
    v3 spec_dir = cubemap_dir(env->rot, add3(mul3s(tangent, sinf(theta_i)), mul3s(fiber_n, cosf(theta_i))));
    v3 diff_dir = cubemap_dir(env->rot, fiber_n);
    v3 spec = sample_cube(env->spec, env->spec_size, env->spec_levels, spec_dir,
                          roughness * (float)(env->spec_levels - 1));
    v3 diff = sample_cube(env->diff, env->diff_size, env->diff_levels, diff_dir, 0.0f);
    float cos_o = fmaxf(cosf(theta_o), 1e-3f);
    float f_r = fresnel(cos_o), f_trt = fresnel(cos_o * 0.5f);
    v3 sigma_a = absorption_from_color(albedo, roughness);
    float k = 0.76f * (1.0f - f_trt) * (1.0f - f_trt) * f_trt;
    v3 trt = V3(k * expf(-sigma_a.x * 3.2f / cos_o), k * expf(-sigma_a.y * 3.2f / cos_o),
                k * expf(-sigma_a.z * 3.2f / cos_o));
    v3 scatter = mul3(albedo, scatter_tint(albedo, 0.5f));
    v3 r = add3(mul3(spec, add3(spl3(f_r), trt)), mul3(diff, scatter));
    return mul3s(r, env->intensity);
}

/* shade.wesl:262-277 */
static float dom_texel_visibility(const hg_hair_params* p, const uint32_t* dom, int32_t x, int32_t y, float dist,
                                  float near_, float far_, uint32_t dom_w, uint32_t dom_h) {
    if (x < 0 || y < 0 || x >= (int32_t)dom_w || y >= (int32_t)dom_h) return 1.0f;
    uint32_t pix = (uint32_t)y * dom_w + (uint32_t)x;
    uint32_t front_q = dom[pix];
    if (front_q == DOM_EMPTY) return 1.0f;
    float z_front = oracle_dequantize_depth(front_q, near_, far_);
    float thickness = fmaxf(far_ - near_, 1e-3f) / (float)DOM_LAYERS;
    float rel = fmaxf((dist - z_front) - thickness * 0.05f, 0.0f);
    uint32_t pixels = dom_w * dom_h;
    float occ = oracle_dom_optical_depth(dom + pixels + (size_t)pix * DOM_LAYERS, DOM_LAYERS, rel / thickness);
    return expf(-occ * p->filter_params[3]);
}

/* shade.wesl:279-310 */
static float dom_visibility(const hg_hair_params* p, const uint32_t* dom, v3 world, float beta) {
    if (p->flags[3] == 0u) return 1.0f;
    v4 clip = mat_mul(p->light_clip_from_world, V4(world.x, world.y, world.z, 1.0f));
    if (clip.w <= 0.0f) return 1.0f;
    float nx = clip.x / clip.w, ny = clip.y / clip.w;
    float ux = nx * 0.5f + 0.5f, uy = 1.0f - (ny * 0.5f + 0.5f);
    if (ux < 0.0f || uy < 0.0f || ux > 1.0f || uy > 1.0f) return 1.0f;
    uint32_t dom_w = f2u(p->dom_info[0]), dom_h = f2u(p->dom_info[1]);
    float near_ = p->dom_info[2], far_ = p->dom_info[3];
    float dist = dot3(sub3(world, ld3(p->light_eye)), ld3(p->light_forward)) -
                 (-logf(fmaxf(beta, 1e-4f)) * p->filter_params[2]);
    float fx = ux * (float)dom_w - 0.5f, fy = uy * (float)dom_h - 0.5f;
    float flx = floorf(fx), fly = floorf(fy);
    int32_t x0 = f2i(flx), y0 = f2i(fly);
    float tx = fx - flx, ty = fy - fly;
    float v00 = dom_texel_visibility(p, dom, x0, y0, dist, near_, far_, dom_w, dom_h);
    float v10 = dom_texel_visibility(p, dom, x0 + 1, y0, dist, near_, far_, dom_w, dom_h);
    float v01 = dom_texel_visibility(p, dom, x0, y0 + 1, dist, near_, far_, dom_w, dom_h);
    float v11 = dom_texel_visibility(p, dom, x0 + 1, y0 + 1, dist, near_, far_, dom_w, dom_h);
    return mixf(mixf(v00, v10, tx), mixf(v01, v11, tx), ty);
}

/* Inverse-square falloff with a smooth range window (Karis 2013, "Real Shading
 * in Unreal Engine 4"; Lagarde & de Rousiers 2014, "Moving Frostbite to PBR").
 * Stands in for bevy_pbr's getDistanceAttenuation, which is not vendored. */
static inline float distance_attenuation(float dist2, float inv_range2) {
    float factor = dist2 * inv_range2;
    float smooth = clampf(1.0f - factor * factor, 0.0f, 1.0f);
    return (smooth * smooth) / fmaxf(dist2, 1e-4f);
}
static inline float range_falloff(float dist2, float inv_range2) {
    float factor = dist2 * inv_range2;
    float smooth = clampf(1.0f - factor * factor, 0.0f, 1.0f);
    return smooth * smooth;
}

/* shade.wesl:312-327 with the spot axis given directly. */
static inline float spot_mask(const hg_light* L, v3 world) {
    v3 spot_dir = ld3(L->direction);
    v3 light_to_frag = sub3(ld3(L->position), world);
    float cd = dot3(mul3s(spot_dir, -1.0f), safe_normalize(light_to_frag));
    float att = clampf(cd * L->spot[0] + L->spot[1], 0.0f, 1.0f);
    return att * att;
}

/* shade.wesl:429-521: point, spot, directional then rect lights. */
static v3 direct_light(const hg_hair_params* p, const uint32_t* dom, const hg_light* lights, uint32_t n_lights,
                       v3 world, v3 tangent, v3 view, v3 albedo, float roughness, float tilt, float beta,
                       const float* mlp, uint32_t mlp_arch) {
    shape_t shape = lobe_shape(roughness, tilt);
    float tv = dot3(tangent, view);
    float cos_theta_o = sqrtf(fmaxf(1.0f - tv * tv, 1e-6f));
    v3 sigma_a = absorption_from_color(albedo, roughness);
    dual_t ds = dual_scatter(cos_theta_o, sigma_a, shape);
    v3 color = spl3(0.0f);
    for (uint32_t kind = 0; kind < 4u; ++kind) {
        int dom_left = 1;
        for (uint32_t i = 0; i < n_lights; ++i) {
            const hg_light* L = &lights[i];
            if (L->kind != kind) continue;
            if (kind == HG_LIGHT_POINT || kind == HG_LIGHT_SPOT) {
                v3 light_to_frag = sub3(ld3(L->position), world);
                float dist2 = dot3(light_to_frag, light_to_frag);
                v3 incident = safe_normalize(light_to_frag);
                float inv_r2 = 1.0f / fmaxf(L->range * L->range, 1e-8f);
                float att = distance_attenuation(dist2, inv_r2);
                v3 lobe = light_lobe(mlp, mlp_arch, tangent, view, incident, sigma_a, shape, &ds, 0.0f, roughness);
                v3 c = mul3s(mul3(lobe, ld3(L->color)), att);
                if (kind == HG_LIGHT_SPOT) c = mul3s(c, spot_mask(L, world));
                color = add3(color, c);
            } else if (kind == HG_LIGHT_DIRECTIONAL) {
                v3 incident = ld3(L->direction);
                int casts = (L->flags & HG_LIGHT_CASTS_SHADOWS) != 0u;
                float depth = 0.0f;
                if (dom_left && casts) {
                    depth = -logf(fmaxf(dom_visibility(p, dom, world, beta), 1e-6f));
                    dom_left = 0;
                }
                v3 lobe = light_lobe(mlp, mlp_arch, tangent, view, incident, sigma_a, shape, &ds, depth, roughness);
                color = add3(color, mul3(lobe, ld3(L->color)));
            } else {
                v3 to_center = sub3(ld3(L->position), world);
                float dist2 = fmaxf(dot3(to_center, to_center), 1e-4f);
                v3 incident = mul3s(to_center, inverse_sqrt(dist2));
                v3 normal = safe_normalize(cross3(ld3(L->up), ld3(L->right)));
                float facing = fmaxf(dot3(normal, incident), 0.0f);
                float solid = L->spot[0] * L->spot[1] * facing / dist2;
                float range2 = fmaxf(L->range * L->range, 1e-4f);
                float falloff = range_falloff(dist2, 1.0f / range2);
                v3 lobe = light_lobe(mlp, mlp_arch, tangent, view, incident, sigma_a, shape, &ds, 0.0f, roughness);
                color = add3(color, mul3s(mul3s(mul3(lobe, ld3(L->color)), solid), falloff));
            }
        }
    }
    return color;
}

/* shade.wesl:523-593 without the environment probe (probe_radiance is zero
 * in the specialization without ENVIRONMENT_MAP, shade.wesl:384-394). */
void oracle_shade(const hg_hair_params* p, const uint64_t* center, const uint32_t* beta_buf, const uint32_t* dom,
                  const hg_light* lights, uint32_t n_lights, uint32_t ortho, float exposure, const float* mlp,
                  uint32_t mlp_arch, const oracle_env* env, float* shaded, float* shaded_depth) {
    uint32_t width = f2u(p->screen[0]), height = f2u(p->screen[1]);
    int nthreads = oracle_get_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
    for (int64_t pix_i = 0; pix_i < (int64_t)width * height; ++pix_i) {
        uint32_t pix = (uint32_t)pix_i;
        uint32_t x = pix % width, y = pix / width;
        uint64_t word = center[pix];
        if (is_empty(word)) {
            shaded[4 * pix + 0] = shaded[4 * pix + 1] = shaded[4 * pix + 2] = shaded[4 * pix + 3] = 0.0f;
            shaded_depth[pix] = 0.0f;
            continue;
        }
        uint32_t u[7];
        oracle_unpack_gb(word, u);
        float view_dist = oracle_dequantize_depth(u[0], p->screen[2], p->screen[3]);
        v3 world = reconstruct_world(p, (int32_t)x, (int32_t)y, view_dist);
        v3 tangent = oct_decode_v(u[1], u[2]);
        v3 uvw = V3((float)u[3] / 63.0f, (float)u[4] / 63.0f, (float)u[5] / 63.0f);
        float ao = (float)u[6] / 63.0f;
        if (p->flags[2] == 0u) ao = 1.0f;
        float beta = (float)(beta_buf[pix] & 0xffu) / 255.0f;
        float roughness = fmaxf(p->appearance[0] * (0.65f + 0.7f * uvw.z), 0.04f);
        float tilt = p->appearance[1];
        v3 albedo = mul3s(ld3(p->albedo), 0.65f + 0.35f * uvw.z);
        v3 view;
        if (ortho) {
            view = safe_normalize(V3(p->clip_from_world[2], p->clip_from_world[6], p->clip_from_world[10]));
        } else {
            view = safe_normalize(sub3(ld3(p->camera_pos), world));
        }
        v3 color = direct_light(p, dom, lights, n_lights, world, tangent, view, albedo, roughness, tilt, beta, mlp, mlp_arch);
        if (env) {
            v3 fiber_n = safe_normalize(sub3(view, mul3s(tangent, dot3(view, tangent))));
            color = add3(color, mul3s(probe_radiance(env, tangent, fiber_n, view, albedo, roughness, tilt), ao));
        }
        color = mul3s(color, exposure);
        shaded[4 * pix + 0] = color.x;
        shaded[4 * pix + 1] = color.y;
        shaded[4 * pix + 2] = color.z;
        shaded[4 * pix + 3] = 1.0f;
        shaded_depth[pix] = view_dist;
    }
}

/* ------------------------------------------------------------------ filter */

/* filter.wgsl:9-18 */
static inline v2 screen_tangent(const hg_hair_params* p, v3 world, v3 tangent) {
    projected a = project_world(p, world);
    projected b = project_world(p, add3(world, tangent));
    v2 d = sub2(b.screen, a.screen);
    float len = len2(d);
    if (len < 1e-3f) return V2(1.0f, 0.0f);
    return V2(d.x / len, d.y / len);
}

/* filter.wgsl:20-135 */
void oracle_filter(const hg_hair_params* p, const uint64_t* center, const uint64_t* cons, const float* shaded,
                   const float* shaded_depth, float* filtered, float* filtered_depth) {
    (void)shaded_depth;
    int32_t width = f2i(p->screen[0]), height = f2i(p->screen[1]);
    int nthreads = oracle_get_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
    for (int64_t pix_i = 0; pix_i < (int64_t)width * height; ++pix_i) {
        int32_t px = (int32_t)(pix_i % width), py = (int32_t)(pix_i / width);
        uint32_t pix = (uint32_t)pix_i;
        uint64_t center_word = center[pix], cons_word = cons[pix];
        int center_hit = !is_empty(center_word), cons_hit = !is_empty(cons_word);
        if (!center_hit && !cons_hit) {
            filtered[4 * pix + 0] = filtered[4 * pix + 1] = filtered[4 * pix + 2] = filtered[4 * pix + 3] = 0.0f;
            filtered_depth[pix] = 0.0f;
            continue;
        }
        uint32_t u[7];
        oracle_unpack_gb(center_hit ? center_word : cons_word, u);
        v3 tangent = oct_decode_v(u[1], u[2]);
        uint32_t depth_q = u[0];
        float view_dist = oracle_dequantize_depth(depth_q, p->screen[2], p->screen[3]);
        v3 world = reconstruct_world(p, px, py, view_dist);
        v2 ts = screen_tangent(p, world, tangent);
        v4 cc = ld4(shaded + 4 * (size_t)pix);
        const int32_t radius = 5;
        float s_par = fmaxf(p->filter_params[0], 0.05f);
        float s_perp = fmaxf(p->filter_params[1], 0.02f);
        float sigma_par = (float)radius * s_par;
        float sigma_perp = (float)radius * s_perp;
        const float sigma_c = 0.9f, depth_reject = 1.45e-3f, closer_eps = 5e-4f, strip = 0.5f;
        v3 accum = spl3(0.0f);
        float weight = 0.0f, h_center = 0.0f, h_cons = 0.0f;
        int promote = !center_hit;
        for (int32_t dy = -radius; dy <= radius; ++dy) {
            for (int32_t dx = -radius; dx <= radius; ++dx) {
                int32_t qx = px + dx, qy = py + dy;
                if (qx < 0 || qy < 0 || qx >= width || qy >= height) continue;
                uint32_t qpix = (uint32_t)qy * (uint32_t)width + (uint32_t)qx;
                v2 d = V2((float)dx, (float)dy);
                float d_par = dot2(d, ts);
                float d_perp = len2(sub2(d, mul2s(ts, d_par)));
                uint64_t qc = center[qpix], qn = cons[qpix];
                if (d_perp <= strip) {
                    if (!is_empty(qc)) {
                        h_center += 1.0f;
                    } else if (!is_empty(qn)) {
                        h_cons += 1.0f;
                    }
                }
                if (is_empty(qc)) continue;
                uint32_t qu[7];
                oracle_unpack_gb(qc, qu);
                float q_norm = (float)qu[0] / 16777214.0f;
                float p_norm = (float)depth_q / 16777214.0f;
                if (fabsf(q_norm - p_norm) > depth_reject) continue;
                float spatial = expf((-d_par * d_par) / (sigma_par * sigma_par) -
                                     (d_perp * d_perp) / (sigma_perp * sigma_perp));
                float color_w = 1.0f;
                v3 qcol = ld3(shaded + 4 * (size_t)qpix);
                if (!promote && cc.w > 0.0f) {
                    float chroma = len3(sub3(xyz(cc), qcol));
                    color_w = expf((-chroma * chroma) / (sigma_c * sigma_c));
                }
                float w = spatial * color_w;
                accum = add3(accum, mul3s(qcol, w));
                weight += w;
            }
        }
        v3 color = xyz(cc);
        if (weight > 1e-5f) color = div3s(accum, weight);
        float alpha = 1.0f;
        float coverage = h_center / fmaxf(h_center + h_cons, 1.0f);
        float cons_depth = 1.0f;
        if (cons_hit) {
            uint32_t cu[7];
            oracle_unpack_gb(cons_word, cu);
            cons_depth = (float)cu[0] / 16777214.0f;
        }
        float center_depth = (float)depth_q / 16777214.0f;
        int closer = cons_hit && center_hit && (center_depth - cons_depth) >= closer_eps;
        alpha = closer ? 1.0f : clampf(coverage, 0.0f, 1.0f);
        if (promote && weight <= 1e-5f) {
            alpha = 0.0f;
            color = spl3(0.0f);
        }
        filtered[4 * pix + 0] = color.x;
        filtered[4 * pix + 1] = color.y;
        filtered[4 * pix + 2] = color.z;
        filtered[4 * pix + 3] = alpha;
        filtered_depth[pix] = view_dist;
    }
}

/* ------------------------------------------------------------------ composite */

/* composite.wgsl:162-181 with BlendState::ALPHA_BLENDING and the
 * GreaterEqual (reverse-Z) / LessEqual depth test, depth writes on
 * (src/render/pipeline.rs:299-339). */
void oracle_composite(const hg_hair_params* p, const float* color_src, const float* depth_src, float* color_dst,
                      float* depth_dst) {
    int32_t width = f2i(p->screen[0]), height = f2i(p->screen[1]);
    int reverse = p->pass_mode[2] == 1u;
    for (int32_t py = 0; py < height; ++py) {
        for (int32_t px = 0; px < width; ++px) {
            uint32_t pix = (uint32_t)py * (uint32_t)width + (uint32_t)px;
            v4 c = ld4(color_src + 4 * (size_t)pix);
            if (c.w < 0.001f) continue;
            float view_dist = depth_src[pix];
            v3 world = reconstruct_world(p, px, py, view_dist);
            v4 clip = mat_mul(p->clip_from_world, V4(world.x, world.y, world.z, 1.0f));
            float depth = clampf(clip.z / fmaxf(clip.w, 1e-5f), 0.0f, 1.0f);
            float dst_depth = depth_dst[pix];
            int pass = reverse ? depth >= dst_depth : depth <= dst_depth;
            if (!pass) continue;
            depth_dst[pix] = depth;
            float* d = color_dst + 4 * (size_t)pix;
            float ia = 1.0f - c.w;
            d[0] = c.x * c.w + d[0] * ia;
            d[1] = c.y * c.w + d[1] * ia;
            d[2] = c.z * c.w + d[2] * ia;
            d[3] = c.w * 1.0f + d[3] * ia;
        }
    }
}

/* ------------------------------------------------------------------ receivers */

/* hair_shadow.wesl:30-50; light = ShadowLight (16 + 4 + 4 + 4 floats). */
static float receiver_texel(const float* light, const uint32_t* dom, uint32_t dom_w, uint32_t dom_h, int32_t x,
                            int32_t y, float dist) {
    if (x < 0 || y < 0 || x >= (int32_t)dom_w || y >= (int32_t)dom_h) return 1.0f;
    uint32_t pix = (uint32_t)y * dom_w + (uint32_t)x;
    uint32_t front_q = dom[pix];
    if (front_q == DOM_EMPTY) return 1.0f;
    float near_ = light[24], far_ = light[25];
    float z_front = mixf(near_, far_, (float)front_q / 16777214.0f);
    float thickness = fmaxf(far_ - near_, 1e-3f) / (float)DOM_LAYERS;
    float t = fmaxf(dist - z_front, 0.0f) / thickness;
    const uint32_t* base = dom + (size_t)dom_w * dom_h + (size_t)pix * DOM_LAYERS;
    float hits = 0.0f;
    for (uint32_t slice = 0; slice < DOM_LAYERS; ++slice)
        hits += (float)base[slice] * clampf(t - (float)slice, 0.0f, 1.0f);
    return expf(-hits * light[26]);
}

/* hair_shadow.wesl:52-75 for n points (float4, xyz used). */
void oracle_hair_visibility(const float* light, const uint32_t* dom, uint32_t dom_w, uint32_t dom_h,
                            const float* points, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        v3 world = ld3(points + 4 * (size_t)i);
        out[i] = 1.0f;
        if (light[27] == 0.0f) continue;
        v4 clip = mat_mul(light, V4(world.x, world.y, world.z, 1.0f));
        if (clip.w <= 0.0f) continue;
        float nx = clip.x / clip.w, ny = clip.y / clip.w;
        float ux = nx * 0.5f + 0.5f, uy = 1.0f - (ny * 0.5f + 0.5f);
        if (ux < 0.0f || uy < 0.0f || ux > 1.0f || uy > 1.0f) continue;
        float dist = dot3(sub3(world, ld3(light + 16)), ld3(light + 20));
        float fx = ux * (float)dom_w - 0.5f, fy = uy * (float)dom_h - 0.5f;
        float flx = floorf(fx), fly = floorf(fy);
        int32_t x0 = f2i(flx), y0 = f2i(fly);
        float tx = fx - flx, ty = fy - fly;
        float v00 = receiver_texel(light, dom, dom_w, dom_h, x0, y0, dist);
        float v10 = receiver_texel(light, dom, dom_w, dom_h, x0 + 1, y0, dist);
        float v01 = receiver_texel(light, dom, dom_w, dom_h, x0, y0 + 1, dist);
        float v11 = receiver_texel(light, dom, dom_w, dom_h, x0 + 1, y0 + 1, dist);
        out[i] = mixf(mixf(v00, v10, tx), mixf(v01, v11, tx), ty);
    }
}
