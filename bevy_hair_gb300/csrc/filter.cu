// Reconnection filter (filter.wgsl:20-135) and the headless composite
// (composite.wgsl:162-181 + ALPHA_BLENDING + depth test, pipeline.rs:299-339).
// The filter's coverage decisions (strip test, depth rejection, "closer")
// come from float comparisons, so this file is compiled with -fmad=false like
// the raster to keep them reproducible.
#include <cuda_runtime.h>

#include "hg_device.cuh"
#include "hg_internal.h"

namespace hg {
namespace {

constexpr int kFilterRadius = 5;
constexpr int kTileX = 32, kTileY = 8;

struct FilterArgs {
    hg_hair_params p;
    const unsigned long long* center;
    const unsigned long long* cons;
    const float4* shaded;
    float4* filtered;
    float* filtered_depth;
};

// screen_tangent (filter.wgsl:9-18)
__device__ __forceinline__ float2 screen_tangent(const hg_hair_params& p, f3 world, f3 tangent) {
    Projected a = project_world(p, world);
    Projected b = project_world(p, add3(world, tangent));
    float2 d = sub2(b.screen, a.screen);
    float l = len2(d);
    if (l < 1e-3f) return make_float2(1.0f, 0.0f);
    return make_float2(__fdiv_rn(d.x, l), __fdiv_rn(d.y, l));
}

// The largest x with sqrt_rn(x) <= r (sqrt_rn is monotone), found from r*r by
// stepping one ulp at a time (a few steps at most; bounded by 8 each way).
__device__ __forceinline__ float sqrt_bound(float r) {
    float x = r * r;
    for (int k = 0; k < 8 && __fsqrt_rn(x) > r; ++k) x = nextafterf(x, 0.0f);
    for (int k = 0; k < 8; ++k) {
        const float up = nextafterf(x, __int_as_float(0x7f800000));
        if (!(__fsqrt_rn(up) <= r)) break;
        x = up;
    }
    return x;
}

// One TX x TY tile per CTA (tile (bx, by) of view a: fields p, center, cons,
// shaded, filtered, filtered_depth).  The (TX+10) x (TY+10) neighbourhood is
// staged in shared memory once: per texel the centre word's normalised depth
// f32(depth)/16777214 (the exact value filter.wgsl:94 computes per tap; -1
// marks an empty centre with a conservative hit, -2 both empty) and the shaded
// colour.  Pixels without hair are written at once; the tile's hair pixels
// are then listed and handed to the first threads, one each, so the 121-tap
// loop runs in full warps instead of the lanes of the hair pixels of every
// row.  Coverage decisions use exact arithmetic; the colour weights only
// scale colour, so they use the fast exponential.
template <int TX, int TY, class V>
__device__ __forceinline__ void filter_tile(const V& a, int32_t bx, int32_t by) {
    constexpr int kHaloX = TX + 2 * kFilterRadius, kHaloY = TY + 2 * kFilterRadius;
    constexpr int kWarps = TX * TY / 32;
    static_assert(TX * TY % 32 == 0, "whole warps per tile");
    __shared__ float s_norm[kHaloY][kHaloX];
    __shared__ float4 s_col[kHaloY][kHaloX];
    __shared__ uint16_t s_list[TX * TY];
    __shared__ int s_warp_hair[kWarps];
    const hg_hair_params& p = a.p;
    const int32_t width = f2i(p.screen[0]), height = f2i(p.screen[1]);
    const int32_t x0 = bx * TX - kFilterRadius, y0 = by * TY - kFilterRadius;
    const int tid = threadIdx.y * TX + threadIdx.x;
    {
        const int32_t ox = bx * TX + threadIdx.x, oy = by * TY + threadIdx.y;
        const bool own_inside = ox < width && oy < height;
        const uint32_t own = (uint32_t)oy * (uint32_t)width + (uint32_t)ox;
        const bool own_hair = own_inside && (!is_empty(__ldg(&a.center[own])) || !is_empty(__ldg(&a.cons[own])));
        // pixels without hair (and every pixel of a tile without hair, which
        // needs no halo) are written now
        if (own_inside && !own_hair) {
            a.filtered[own] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            a.filtered_depth[own] = 0.0f;
        }
        const uint32_t ballot = __ballot_sync(0xffffffffu, own_hair);
        if ((tid & 31) == 0) s_warp_hair[tid >> 5] = __popc(ballot);
        __syncthreads();
        int base = 0, total = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const int c = s_warp_hair[w];
            base += w < (tid >> 5) ? c : 0;
            total += c;
        }
        if (total == 0) return;
        if (own_hair) s_list[base + __popc(ballot & ((1u << (tid & 31)) - 1u))] = (uint16_t)tid;
        // the halo: per texel the normalised centre depth (or -1 / -2) and
        // the shaded colour, as the tap loop reads them
        for (int i = tid; i < kHaloX * kHaloY; i += TX * TY) {
            const int hx = i % kHaloX, hy = i / kHaloX;
            const int32_t gx = x0 + hx, gy = y0 + hy;
            float nrm = -2.0f;
            float4 col = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (gx >= 0 && gy >= 0 && gx < width && gy < height) {
                const size_t q = (size_t)gy * width + gx;
                const unsigned long long c = __ldg(&a.center[q]);
                if (!is_empty(c)) {
                    nrm = __fdiv_rn(__uint2float_rn((uint32_t)(c >> 40)), 16777214.0f);
                    col = __ldg(&a.shaded[q]);
                } else if (!is_empty(__ldg(&a.cons[q]))) {
                    nrm = -1.0f;
                }
            }
            s_norm[hy][hx] = nrm;
            s_col[hy][hx] = col;
        }
        __syncthreads();
        if (tid >= total) return;  // no hair pixel left for this thread
    }
    // this thread's hair pixel
    const int src = s_list[tid];
    const int sx = src % TX, sy = src / TX;
    const int32_t px = bx * TX + sx, py = by * TY + sy;
    const uint32_t pix = (uint32_t)py * (uint32_t)width + (uint32_t)px;
    const unsigned long long center_word = __ldg(&a.center[pix]);
    const unsigned long long cons_word = __ldg(&a.cons[pix]);
    const bool center_hit = !is_empty(center_word), cons_hit = !is_empty(cons_word);
    const int lx = sx + kFilterRadius, ly = sy + kFilterRadius;
    const unsigned long long w = center_hit ? center_word : cons_word;
    const uint32_t high = (uint32_t)(w >> 32), low = (uint32_t)w;
    const f3 tangent = oct_decode(high & 0xffu, low >> 24u);
    const uint32_t depth_q = high >> 8u;
    const float view_dist = dequantize_depth(depth_q, p.screen[2], p.screen[3]);
    const f3 world = reconstruct_world(p, px, py, view_dist);
    const float2 ts = screen_tangent(p, world, tangent);
    const float4 cc = __ldg(&a.shaded[pix]);

    const float s_par = fmaxf(p.filter_params[0], 0.05f);
    const float s_perp = fmaxf(p.filter_params[1], 0.02f);
    const float sigma_par = (float)kFilterRadius * s_par;
    const float sigma_perp = (float)kFilterRadius * s_perp;
    // exp(-x) = 2^(-x log2 e): the weights' scales folded into one factor each
    const float k_par = 1.4426950408889634f / (sigma_par * sigma_par);
    const float k_perp = 1.4426950408889634f / (sigma_perp * sigma_perp);
    const float k_col = 1.4426950408889634f / (0.9f * 0.9f);
    const float depth_reject = 1.45e-3f, closer_eps = 5e-4f;
    const float strip2 = sqrt_bound(0.5f);  // the strip half-width of filter.wgsl:63
    const float p_norm = __fdiv_rn(__uint2float_rn(depth_q), 16777214.0f);
    const bool promote = !center_hit;
    const bool use_color = !promote && cc.w > 0.0f;

    float ax = 0.0f, ay = 0.0f, az = 0.0f, weight = 0.0f, h_center = 0.0f, h_cons = 0.0f;
#pragma unroll 1
    for (int dy = -kFilterRadius; dy <= kFilterRadius; ++dy) {
        const int32_t qy = py + dy;
        if (qy < 0 || qy >= height) continue;
#pragma unroll
        for (int dx = -kFilterRadius; dx <= kFilterRadius; ++dx) {
            const int32_t qx = px + dx;
            if (qx < 0 || qx >= width) continue;
            const float fdx = (float)dx, fdy = (float)dy;
            const float d_par = fdx * ts.x + fdy * ts.y;
            const float ex = fdx - ts.x * d_par, ey = fdy - ts.y * d_par;
            // d_perp = sqrt_rn(e2); d_perp <= 0.5 exactly when e2 <= strip2
            const float e2 = ex * ex + ey * ey;
            const float nrm = s_norm[ly + dy][lx + dx];
            if (e2 <= strip2) {
                if (nrm >= 0.0f) {
                    h_center += 1.0f;
                } else if (nrm == -1.0f) {
                    h_cons += 1.0f;
                }
            }
            if (nrm < 0.0f) continue;
            if (fabsf(nrm - p_norm) > depth_reject) continue;
            const float4 qcol = s_col[ly + dy][lx + dx];
            // The colour weights are compared within a tolerance, so they use
            // fused multiply-adds (this file is otherwise built without
            // contraction for the exact strip and coverage tests above).
            float e = __fmaf_rn(d_par * d_par, k_par, e2 * k_perp);
            if (use_color) {
                const float cx = cc.x - qcol.x, cy = cc.y - qcol.y, cz = cc.z - qcol.z;
                e = __fmaf_rn(__fmaf_rn(cz, cz, __fmaf_rn(cy, cy, cx * cx)), k_col, e);
            }
            const float wgt = exp2f(-e);
            ax = __fmaf_rn(qcol.x, wgt, ax);
            ay = __fmaf_rn(qcol.y, wgt, ay);
            az = __fmaf_rn(qcol.z, wgt, az);
            weight += wgt;
        }
    }
    float cx = cc.x, cy = cc.y, cz = cc.z;
    if (weight > 1e-5f) {
        const float inv = 1.0f / weight;
        cx = ax * inv;
        cy = ay * inv;
        cz = az * inv;
    }
    const float coverage = __fdiv_rn(h_center, fmaxf(h_center + h_cons, 1.0f));
    const float cons_depth = cons_hit ? __fdiv_rn(__uint2float_rn((uint32_t)(cons_word >> 40)), 16777214.0f) : 1.0f;
    const float center_depth = p_norm;
    const bool closer = cons_hit && center_hit && (center_depth - cons_depth) >= closer_eps;
    float alpha = closer ? 1.0f : clampf(coverage, 0.0f, 1.0f);
    if (promote && weight <= 1e-5f) {
        alpha = 0.0f;
        cx = cy = cz = 0.0f;
    }
    a.filtered[pix] = make_float4(cx, cy, cz, alpha);
    a.filtered_depth[pix] = view_dist;
}

__global__ void __launch_bounds__(kTileX* kTileY) filter_kernel(const FilterArgs a) {
    filter_tile<kTileX, kTileY>(a, blockIdx.x, blockIdx.y);
}

// Tile t of the camera views' concatenated tile space -> (view, bx, by).
__device__ __forceinline__ uint32_t tile_view(const uint32_t* __restrict__ prefix, uint32_t n, uint32_t t) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (prefix[mid] <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <int TX, int TY>
__global__ void __launch_bounds__(TX* TY) batch_filter_kernel(const BatchView* __restrict__ views,
                                                             const uint32_t* __restrict__ prefix, uint32_t n_cam) {
    const uint32_t v = tile_view(prefix, n_cam, blockIdx.x);
    const BatchView& a = views[v];
    const uint32_t t = blockIdx.x - prefix[v];
    const uint32_t tiles_x = (a.width + TX - 1) / TX;
    filter_tile<TX, TY>(a, (int32_t)(t % tiles_x), (int32_t)(t / tiles_x));
}

struct CompositeArgs {
    hg_hair_params p;
    const float4* color_src;
    const float* depth_src;
    float4* color;
    float* depth;
};

// composite.wgsl:162-181; blend src*a + dst*(1-a) (alpha: a + dst_a*(1-a)),
// depth test GreaterEqual when reverse-Z else LessEqual, depth write on.
template <class V>
__device__ __forceinline__ void composite_pixel(const V& a, const float4* __restrict__ color_src,
                                                const float* __restrict__ depth_src, int32_t px, int32_t py) {
    const hg_hair_params& p = a.p;
    const int32_t width = f2i(p.screen[0]), height = f2i(p.screen[1]);
    if (px >= width || py >= height) return;
    const uint32_t pix = (uint32_t)py * (uint32_t)width + (uint32_t)px;
    const float4 c = __ldg(&color_src[pix]);
    if (c.w < 0.001f) return;
    const float view_dist = __ldg(&depth_src[pix]);
    const f3 world = reconstruct_world(p, px, py, view_dist);
    const float4 clip = mat_mul(p.clip_from_world, world.x, world.y, world.z, 1.0f);
    const float depth = clampf(__fdiv_rn(clip.z, fmaxf(clip.w, 1e-5f)), 0.0f, 1.0f);
    const float dst_depth = a.depth[pix];
    const bool pass = p.pass_mode[2] == 1u ? depth >= dst_depth : depth <= dst_depth;
    if (!pass) return;
    a.depth[pix] = depth;
    float4 d = a.color[pix];
    const float ia = 1.0f - c.w;
    d.x = c.x * c.w + d.x * ia;
    d.y = c.y * c.w + d.y * ia;
    d.z = c.z * c.w + d.z * ia;
    d.w = c.w * 1.0f + d.w * ia;
    a.color[pix] = d;
}

__global__ void composite_kernel(const CompositeArgs a) {
    composite_pixel(a, a.color_src, a.depth_src, blockIdx.x * blockDim.x + threadIdx.x,
                    blockIdx.y * blockDim.y + threadIdx.y);
}

__global__ void batch_composite_kernel(const BatchView* __restrict__ views, const uint32_t* __restrict__ prefix,
                                       uint32_t n_cam, uint32_t source_filtered) {
    const uint32_t v = tile_view(prefix, n_cam, blockIdx.x);
    const BatchView& a = views[v];
    const uint32_t t = blockIdx.x - prefix[v];
    const uint32_t tiles_x = (a.width + blockDim.x - 1) / blockDim.x;
    composite_pixel(a, source_filtered ? a.filtered : a.shaded, source_filtered ? a.filtered_depth : a.shaded_depth,
                    (int32_t)((t % tiles_x) * blockDim.x + threadIdx.x),
                    (int32_t)((t / tiles_x) * blockDim.y + threadIdx.y));
}

__global__ void clear_color_kernel(float4* __restrict__ color, float* __restrict__ depth, size_t pixels,
                                   float depth_clear) {
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < pixels; i += stride) {
        color[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        depth[i] = depth_clear;
    }
}

}  // namespace

cudaError_t launch_filter(hg_ctx* ctx, const hg_hair_params& p) {
    FilterArgs a;
    a.p = p;
    a.center = ctx->center;
    a.cons = ctx->cons;
    a.shaded = ctx->shaded;
    a.filtered = ctx->filtered;
    a.filtered_depth = ctx->filtered_depth;
    dim3 block(kTileX, kTileY);
    dim3 grid((ctx->width + kTileX - 1) / kTileX, (ctx->height + kTileY - 1) / kTileY);
    filter_kernel<<<grid, block, 0, ctx->stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_composite(hg_ctx* ctx, const hg_hair_params& p, uint32_t source_filtered) {
    CompositeArgs a;
    a.p = p;
    a.color_src = source_filtered ? ctx->filtered : ctx->shaded;
    a.depth_src = source_filtered ? ctx->filtered_depth : ctx->shaded_depth;
    a.color = ctx->color;
    a.depth = ctx->depth;
    dim3 block(32, 8);
    dim3 grid((ctx->width + 31) / 32, (ctx->height + 7) / 8);
    composite_kernel<<<grid, block, 0, ctx->stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_batch_filter_composite(hg_ctx* ctx, const BatchDev& b) {
    cudaError_t e;
    if (b.filter && b.total_ftiles) {
        if (b.filter_tile == 1) batch_filter_kernel<16, 16><<<b.total_ftiles, dim3(16, 16), 0, ctx->stream>>>(
            b.views, b.ftile_prefix, b.n_cam);
        else batch_filter_kernel<kTileX, kTileY><<<b.total_ftiles, dim3(kTileX, kTileY), 0, ctx->stream>>>(
            b.views, b.ftile_prefix, b.n_cam);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (!b.composite || !b.total_px) return cudaSuccess;
    const int threads = 256;
    const int blocks = (int)std::min<uint64_t>((b.total_px + threads - 1) / threads, (uint64_t)ctx->sm_count * 8);
    clear_color_kernel<<<blocks, threads, 0, ctx->stream>>>(b.color, b.depth, b.total_px, b.depth_clear);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    batch_composite_kernel<<<b.total_tiles, dim3(b.tile_w, b.tile_h), 0, ctx->stream>>>(b.views, b.tile_prefix,
                                                                                       b.n_cam, b.filter);
    return cudaGetLastError();
}

cudaError_t launch_clear_color(hg_ctx* ctx, float depth_clear) {
    size_t pixels = (size_t)ctx->width * ctx->height;
    int threads = 256;
    int blocks = (int)std::min<size_t>((pixels + threads - 1) / threads, (size_t)ctx->sm_count * 8);
    if (blocks < 1) blocks = 1;
    clear_color_kernel<<<blocks, threads, 0, ctx->stream>>>(ctx->color, ctx->depth, pixels, depth_clear);
    return cudaGetLastError();
}

}  // namespace hg
