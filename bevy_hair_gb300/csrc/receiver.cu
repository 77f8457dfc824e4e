// Deep-opacity lookups for other surfaces (hair_shadow.wesl:30-75) and the
// published light view (src/render/pass.rs:574-579).
#include <cuda_runtime.h>

#include "hg_device.cuh"
#include "hg_internal.h"

namespace hg {
namespace {

// texel_visibility (hair_shadow.wesl:30-50)
__device__ __forceinline__ float texel_visibility(const uint32_t* __restrict__ dom, uint32_t dom_w, uint32_t dom_h,
                                                  int32_t x, int32_t y, float dist, const hg_shadow_light& L) {
    if (x < 0 || y < 0 || x >= (int32_t)dom_w || y >= (int32_t)dom_h) return 1.0f;
    const uint32_t pix = (uint32_t)y * dom_w + (uint32_t)x;
    const uint32_t front_q = __ldg(&dom[pix]);
    if (front_q == kDomEmpty) return 1.0f;
    const float near_ = L.depth[0], far_ = L.depth[1];
    const float z_front = dequantize_depth(front_q, near_, far_);
    const float thickness = fmaxf(far_ - near_, 1e-3f) / (float)kDomLayers;
    const float t = fmaxf(dist - z_front, 0.0f) / thickness;
    const uint32_t* c = dom + (size_t)dom_w * dom_h + (size_t)pix * kDomLayers;
    float hits = 0.0f;
#pragma unroll
    for (int s = 0; s < (int)kDomLayers; ++s) hits += (float)__ldg(c + s) * clampf(t - (float)s, 0.0f, 1.0f);
    return expf(-hits * L.depth[2]);
}

__global__ void visibility_kernel(const hg_shadow_light L, const uint32_t* __restrict__ dom, uint32_t dom_w,
                                  uint32_t dom_h, const float4* __restrict__ points, uint32_t n,
                                  float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 w4 = __ldg(&points[i]);
    float vis = 1.0f;
    // hair_visibility (hair_shadow.wesl:52-75)
    if (L.depth[3] != 0.0f) {
        const float4 clip = mat_mul(L.light_clip_from_world, w4.x, w4.y, w4.z, 1.0f);
        if (clip.w > 0.0f) {
            const float nx = clip.x / clip.w, ny = clip.y / clip.w;
            const float ux = nx * 0.5f + 0.5f, uy = 1.0f - (ny * 0.5f + 0.5f);
            if (!(ux < 0.0f || uy < 0.0f || ux > 1.0f || uy > 1.0f)) {
                const float dist = dot3(sub3(xyz(w4), mk3(L.light_eye[0], L.light_eye[1], L.light_eye[2])),
                                        mk3(L.light_forward[0], L.light_forward[1], L.light_forward[2]));
                const float fx = ux * (float)dom_w - 0.5f, fy = uy * (float)dom_h - 0.5f;
                const float flx = floorf(fx), fly = floorf(fy);
                const int32_t x0 = f2i(flx), y0 = f2i(fly);
                const float tx = fx - flx, ty = fy - fly;
                const float v00 = texel_visibility(dom, dom_w, dom_h, x0, y0, dist, L);
                const float v10 = texel_visibility(dom, dom_w, dom_h, x0 + 1, y0, dist, L);
                const float v01 = texel_visibility(dom, dom_w, dom_h, x0, y0 + 1, dist, L);
                const float v11 = texel_visibility(dom, dom_w, dom_h, x0 + 1, y0 + 1, dist, L);
                vis = mixf(mixf(v00, v10, tx), mixf(v01, v11, tx), ty);
            }
        }
    }
    out[i] = vis;
}

}  // namespace

cudaError_t launch_visibility(hg_ctx* ctx, const hg_shadow_light& L, const float* points, uint32_t n, float* out) {
    if (n == 0) return cudaSuccess;
    const int threads = 256;
    visibility_kernel<<<(n + threads - 1) / threads, threads, 0, ctx->stream>>>(
        L, ctx->dom, ctx->dom_w, ctx->dom_h, reinterpret_cast<const float4*>(points), n, out);
    return cudaGetLastError();
}

}  // namespace hg
