// Device-side math with the float semantics the visibility buffer needs to be
// reproducible bit for bit: IEEE f32 round-to-nearest operations evaluated in
// the order the shaders write them (common.wgsl), correctly rounded sqrt and
// division, truncating saturating float->int conversions, wrapping i32
// arithmetic.  Translation units that include this file for bit-exact work are
// compiled with -fmad=false -prec-div=true -prec-sqrt=true -ftz=false, so no
// a*b+c is contracted into an FMA.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/hairgb.h"

namespace hg {

constexpr uint32_t kLayerCount = HG_LAYER_COUNT;
constexpr uint32_t kStyleU = 8, kStyleV = 8, kStyleW = 16;
constexpr uint32_t kDomLayers = HG_DOM_LAYERS;
constexpr uint32_t kDomEmpty = 0xffffffffu;
constexpr unsigned long long kEmptyU64 = 0xffffffffffffffffull;
constexpr float kPi = 3.14159265f;

// Device error word bits (read back by hg_synchronize).
constexpr uint32_t kErrBadRef = 1u << 0;
constexpr uint32_t kErrBadBundle = 1u << 1;

struct f3 {
    float x, y, z;
};

__device__ __forceinline__ f3 mk3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 xyz(float4 a) { return {a.x, a.y, a.z}; }
__device__ __forceinline__ f3 add3(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 mul3s(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float len3(f3 a) { return __fsqrt_rn(dot3(a, a)); }
__device__ __forceinline__ float dot2(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ float len2(float2 a) { return __fsqrt_rn(dot2(a, a)); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ f3 mix3(f3 a, f3 b, float t) {
    return {mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)};
}
__device__ __forceinline__ float2 mix2(float2 a, float2 b, float t) {
    return make_float2(mixf(a.x, b.x, t), mixf(a.y, b.y, t));
}
// inverseSqrt as two correctly rounded steps.
__device__ __forceinline__ float inv_sqrt(float x) { return __fdiv_rn(1.0f, __fsqrt_rn(x)); }
__device__ __forceinline__ f3 normalize3(f3 v) { return mul3s(v, inv_sqrt(dot3(v, v))); }
__device__ __forceinline__ f3 safe_normalize(f3 v) {
    float l2 = dot3(v, v);
    if (l2 < 1e-10f) return {0.0f, 1.0f, 0.0f};
    return mul3s(v, inv_sqrt(l2));
}

// Truncating conversions; the hardware conversion saturates and maps NaN to 0.
__device__ __forceinline__ uint32_t f2u(float f) { return __float2uint_rz(f); }
__device__ __forceinline__ int32_t f2i(float f) { return __float2int_rz(f); }
__device__ __forceinline__ int32_t iadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t isub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
__device__ __forceinline__ int32_t iabs(int32_t a) { return a < 0 ? (int32_t)(0u - (uint32_t)a) : a; }

// Column-major M * (x, y, z, w), columns summed in order.
__device__ __forceinline__ float4 mat_mul(const float* m, float x, float y, float z, float w) {
    float4 r;
    r.x = ((m[0] * x + m[4] * y) + m[8] * z) + m[12] * w;
    r.y = ((m[1] * x + m[5] * y) + m[9] * z) + m[13] * w;
    r.z = ((m[2] * x + m[6] * y) + m[10] * z) + m[14] * w;
    r.w = ((m[3] * x + m[7] * y) + m[11] * z) + m[15] * w;
    return r;
}

__device__ __forceinline__ uint32_t pcg(uint32_t input) {
    uint32_t state = input * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

__device__ __forceinline__ float2 pcg_uv(uint32_t seed) {
    uint32_t a = pcg(seed);
    uint32_t b = pcg(a ^ 0x9e3779b9u);
    const float s = 1.0f / 4294967296.0f;
    return make_float2(__uint2float_rn(a) * s, __uint2float_rn(b) * s);
}

__device__ __forceinline__ unsigned long long pack_gb(uint32_t depth, uint32_t tx, uint32_t ty, uint32_t u,
                                                      uint32_t v, uint32_t w, uint32_t ao) {
    uint32_t high = (depth << 8u) | (tx & 0xffu);
    uint32_t low = ((ty & 0xffu) << 24u) | ((u & 0x3fu) << 18u) | ((v & 0x3fu) << 12u) | ((w & 0x3fu) << 6u) |
                   (ao & 0x3fu);
    return ((unsigned long long)high << 32u) | (unsigned long long)low;
}

__device__ __forceinline__ bool is_empty(unsigned long long w) { return ((uint32_t)(w >> 32u) >> 8u) == 0x00ffffffu; }

__device__ __forceinline__ uint32_t quantize_depth(float dist, float near_, float far_) {
    float q = clampf(__fdiv_rn(dist - near_, fmaxf(far_ - near_, 1e-3f)), 0.0f, 1.0f);
    uint32_t r = f2u(q * 16777214.0f);
    return r < 0x00fffffeu ? r : 0x00fffffeu;
}

// Explicitly rounded operations: the view distance is an output (shaded_depth,
// filtered_depth), so it stays exact even in translation units built with FMA
// contraction.
__device__ __forceinline__ float dequantize_depth(uint32_t depth, float near_, float far_) {
    float t = __fdiv_rn(__uint2float_rn(depth), 16777214.0f);
    return __fadd_rn(__fmul_rn(near_, __fsub_rn(1.0f, t)), __fmul_rn(far_, t));
}

__device__ __forceinline__ uint32_t quant63(float c) {
    uint32_t q = f2u(clampf(c, 0.0f, 1.0f) * 63.0f + 0.5f);
    return q > 63u ? 63u : q;
}

// oct_encode (common.wgsl:119-130); returns tx | ty << 8.
__device__ __forceinline__ uint32_t oct_encode(f3 nin) {
    f3 n = normalize3(nin);
    float denom = (fabsf(n.x) + fabsf(n.y)) + fabsf(n.z);
    float dm = fmaxf(denom, 1e-6f);
    float px = __fdiv_rn(n.x, dm), py = __fdiv_rn(n.y, dm);
    if (n.z < 0.0f) {
        float ox = px, oy = py;
        px = (1.0f - fabsf(oy)) * (ox >= 0.0f ? 1.0f : -1.0f);
        py = (1.0f - fabsf(ox)) * (oy >= 0.0f ? 1.0f : -1.0f);
    }
    float ex = clampf(px * 0.5f + 0.5f, 0.0f, 1.0f);
    float ey = clampf(py * 0.5f + 0.5f, 0.0f, 1.0f);
    return f2u(ex * 255.0f + 0.5f) | (f2u(ey * 255.0f + 0.5f) << 8u);
}

// oct_decode (common.wgsl:132-142)
__device__ __forceinline__ f3 oct_decode(uint32_t tx, uint32_t ty) {
    float ex = __fdiv_rn(__uint2float_rn(tx), 255.0f), ey = __fdiv_rn(__uint2float_rn(ty), 255.0f);
    float fx = ex * 2.0f - 1.0f, fy = ey * 2.0f - 1.0f;
    f3 n = {fx, fy, (1.0f - fabsf(fx)) - fabsf(fy)};
    if (n.z < 0.0f) {
        float ox = n.x, oy = n.y;
        n.x = (1.0f - fabsf(oy)) * (ox >= 0.0f ? 1.0f : -1.0f);
        n.y = (1.0f - fabsf(ox)) * (oy >= 0.0f ? 1.0f : -1.0f);
    }
    return normalize3(n);
}

// calc_tangent (common.wgsl:152-166)
__device__ __forceinline__ f3 calc_tangent(uint32_t idx, uint32_t count, f3 prev, f3 curr, f3 next) {
    f3 d;
    float scale;
    if (idx == 0u) {
        d = sub3(next, curr);
        scale = len3(d);
    } else if (idx + 1u >= count) {
        d = sub3(curr, prev);
        scale = len3(d);
    } else {
        d = sub3(next, prev);
        scale = len3(d) * 0.5f;
    }
    return mul3s(safe_normalize(d), fmaxf(scale, 1e-4f));
}

struct Projected {
    float2 screen;
    float view_dist;
    float clip_depth;
    bool in_front;
};

// project_world (common.wgsl:212-219)
__device__ __forceinline__ Projected project_world(const hg_hair_params& p, f3 w) {
    float4 clip = mat_mul(p.clip_from_world, w.x, w.y, w.z, 1.0f);
    float cw = fmaxf(clip.w, 1e-5f);
    float nx = __fdiv_rn(clip.x, cw), ny = __fdiv_rn(clip.y, cw), nz = __fdiv_rn(clip.z, cw);
    Projected r;
    r.screen.x = (nx * 0.5f + 0.5f) * p.screen[0];
    r.screen.y = (1.0f - (ny * 0.5f + 0.5f)) * p.screen[1];
    r.view_dist = dot3(sub3(w, mk3(p.camera_pos[0], p.camera_pos[1], p.camera_pos[2])),
                       mk3(p.camera_forward[0], p.camera_forward[1], p.camera_forward[2]));
    r.clip_depth = nz;
    r.in_front = clip.w > 0.0f && r.view_dist > p.screen[2] * 0.5f;
    return r;
}

// reconstruct_world (common.wgsl:221-229)
__device__ __forceinline__ f3 reconstruct_world(const hg_hair_params& p, int32_t px, int32_t py, float view_dist) {
    float ux = __fdiv_rn(__int2float_rn(px) + 0.5f, fmaxf(p.screen[0], 1.0f));
    float uy = __fdiv_rn(__int2float_rn(py) + 0.5f, fmaxf(p.screen[1], 1.0f));
    float ndx = ux * 2.0f - 1.0f;
    float ndy = (1.0f - uy) * 2.0f - 1.0f;
    float4 fh = mat_mul(p.world_from_clip, ndx, ndy, 0.0f, 1.0f);
    float fw = fmaxf(fh.w, 1e-5f);
    f3 far_p = {__fdiv_rn(fh.x, fw), __fdiv_rn(fh.y, fw), __fdiv_rn(fh.z, fw)};
    f3 cam = {p.camera_pos[0], p.camera_pos[1], p.camera_pos[2]};
    f3 dir = sub3(far_p, cam);
    float denom = fmaxf(dot3(dir, mk3(p.camera_forward[0], p.camera_forward[1], p.camera_forward[2])), 1e-4f);
    return add3(cam, mul3s(dir, __fdiv_rn(view_dist, denom)));
}

}  // namespace hg
