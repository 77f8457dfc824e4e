// The compact shading surrogate: 10 inputs -> 2 x 32 ReLU -> 3 outputs, the
// same inputs and normalisation as the 4 x 64 network (hg_mlp.cuh), FP16
// weights and activations with FP32 accumulation on mma.sync m16n8k16.  It
// predicts what the shade pass adds per light at zero deep-opacity depth,
// the BSDF R + TT + TRT + 0.7 B per colour channel, as log1p(bsdf / 1e-3):
// one value per channel instead of twelve lobes, which is what lets the
// shading kernel decode a single row per lane.
//
// Parameter layout (float, HG_MLP_COMPACT_PARAMS): W1[32][16] b1[32]
// W2[32][32] b2[32] W3[16][32] b3[16]; W[out][in].  Inputs beyond 10 and
// outputs beyond 3 are padding (zero weights, ignored).
#pragma once

#include "hg_mlp.cuh"

namespace hg {
namespace mlps {

constexpr int kIn = mlp::kIn;    // 16 (10 used)
constexpr int kHid = 32;
constexpr int kOut = mlp::kOut;  // 16 (3 used)
constexpr int kUsedOut = 3;
constexpr float kBack = 0.7f;  // the shade pass's back-scattering density
constexpr int kW1 = 0, kB1 = kW1 + kHid * kIn;
constexpr int kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid;
constexpr int kW3 = kB2 + kHid, kB3 = kW3 + kOut * kHid;
constexpr int kParams = kB3 + kOut;  // 2128
static_assert(kParams == 2128, "parameter layout");

// Shared-memory weights for the mma.sync forward: rows padded by 8 halves
// (conflict-free ldmatrix), 16-byte aligned rows.
constexpr int kPadIn = kIn + 8, kPadHid = kHid + 8;
struct Weights {
    __half w1[kHid][kPadIn];
    __half w2[kHid][kPadHid];
    __half w3[kOut][kPadHid];
    float b1[kHid], b2[kHid], b3[kOut];
};

__device__ __forceinline__ void load(Weights& s, const __half* __restrict__ w16, const float* __restrict__ params,
                                     int tid, int nthreads) {
    mlp::copy_rows<kPadIn>(s.w1, w16 + kW1, kHid, kIn, tid, nthreads);
    mlp::copy_rows<kPadHid>(s.w2, w16 + kW2, kHid, kHid, tid, nthreads);
    mlp::copy_rows<kPadHid>(s.w3, w16 + kW3, kOut, kHid, tid, nthreads);
    for (int i = tid; i < kHid; i += nthreads) {
        s.b1[i] = params[kB1 + i];
        s.b2[i] = params[kB2 + i];
        if (i < kOut) s.b3[i] = params[kB3 + i];
    }
}

// C fragments of a 32-wide layer -> ReLU -> FP16 A fragments of the next.
__device__ __forceinline__ void relu_to_a(const float acc[2][4][4], uint32_t a[2][2][4]) {
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int kt = 0; kt < 2; ++kt) {
            const float* lo = acc[mt][2 * kt];
            const float* hi = acc[mt][2 * kt + 1];
            a[mt][kt][0] = mlp::pack_relu(lo[0], lo[1]);
            a[mt][kt][1] = mlp::pack_relu(lo[2], lo[3]);
            a[mt][kt][2] = mlp::pack_relu(hi[0], hi[1]);
            a[mt][kt][3] = mlp::pack_relu(hi[2], hi[3]);
        }
}

// Forward pass of the 32 samples held by the warp's lanes (x: this lane's
// normalised inputs; y: 12 columns of its outputs in the transformed space,
// the first kUsedOut meaningful, the rest padding).  Every lane of the warp
// calls it.
__device__ __forceinline__ void forward(const Weights& w, mlp::WarpIo& io, const float x[mlp::kUsedIn],
                                        float y[mlp::kUsedOut]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t a0[2][1][4];
    mlp::input_frags(io, x, a0, lane, g, t);
    float acc[2][4][4];
    uint32_t a[2][2][4];
    mlp::layer_ldsm<4, 1, kPadIn>(acc, a0, w.w1, w.b1, lane);
    relu_to_a(acc, a);
    mlp::layer_ldsm<4, 2, kPadHid>(acc, a, w.w2, w.b2, lane);
    relu_to_a(acc, a);
    float out[2][2][4];
    mlp::layer_ldsm<2, 2, kPadHid>(out, a, w.w3, w.b3, lane);
    mlp::output_rows(io, out, y, lane, g, t);
}

// ---------------------------------------------------------------- training
// Training target of channel c from the twelve transformed FP64 lobes of
// hg_mlp_samples (log1p(lobe / 1e-3)): log1p(bsdf / 1e-3) with bsdf =
// R + TT + TRT + kBack * B.
__device__ __forceinline__ float bsdf_target(const float* t12, int c) {
    const float s = expm1f(t12[c]) + expm1f(t12[3 + c]) + expm1f(t12[6 + c]) + kBack * expm1f(t12[9 + c]);
    return log1pf(s);
}

}  // namespace mlps
}  // namespace hg
