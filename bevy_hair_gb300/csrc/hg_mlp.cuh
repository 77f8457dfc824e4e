// The shading surrogate's network: 10 inputs -> 4 x 64 ReLU -> 12 outputs,
// FP16 weights and activations, FP32 accumulation on the tensor cores
// (mma.sync m16n8k16).  A warp evaluates 32 samples at once: the output
// fragments of one layer are the input fragments of the next, so hidden
// activations stay in registers.
//
// FP16 rather than BF16: the inputs include sin(theta) and the longitudinal
// lobes are Gaussians as narrow as 0.03 rad, so an 8-bit significand (2^-8
// steps in sin theta) already moves a lobe flank by tens of percent; FP16's
// 11 bits keep that below the fitting error at the same tensor-core rate.
//
// Parameter layout (float, HG_MLP_PARAMS): W1[64][16] b1[64] W2[64][64] b2[64]
// W3[64][64] b3[64] W4[64][64] b4[64] W5[16][64] b5[16]; W[out][in].  Inputs
// beyond 10 and outputs beyond 12 are padding (zero weights, ignored).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace hg {
namespace mlp {

constexpr int kIn = 16;    // padded input width (10 used)
constexpr int kHid = 64;
constexpr int kOut = 16;   // padded output width (12 used)
constexpr int kUsedIn = 10, kUsedOut = 12;
constexpr int kParams = kHid * kIn + kHid + 3 * (kHid * kHid + kHid) + kOut * kHid + kOut;  // 14608
// Offsets into the float parameter vector.
constexpr int kW1 = 0, kB1 = kW1 + kHid * kIn;
constexpr int kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid;
constexpr int kW3 = kB2 + kHid, kB3 = kW3 + kHid * kHid;
constexpr int kW4 = kB3 + kHid, kB4 = kW4 + kHid * kHid;
constexpr int kW5 = kB4 + kHid, kB5 = kW5 + kOut * kHid;
static_assert(kB5 + kOut == kParams, "parameter layout");
// Transposed copies used by the backward pass: W2^T, W3^T, W4^T [64][64], W5^T [64][16].
constexpr int kT2 = 0, kT3 = kT2 + kHid * kHid, kT4 = kT3 + kHid * kHid, kT5 = kT4 + kHid * kHid;
constexpr int kTransposed = kT5 + kHid * kOut;  // 13312

// Target transform: the network predicts log1p(lobe / kScale).
constexpr float kScale = 1e-3f;

// Input normalisation ranges (the training distribution).
constexpr float kSigmaLogMid = -0.91629073f;   // log(0.4): log sigma_a in [log 0.02, log 8]
constexpr float kSigmaLogInv = 0.33380820f;    // 1 / log(20)
constexpr float kBetaMMid = 0.165f, kBetaMInv = 7.4074074f;   // beta_m in [0.03, 0.3]
constexpr float kBetaNMid = 0.5f, kBetaNInv = 3.3333333f;     // beta_n in [0.2, 0.8]
constexpr float kEtaMid = 1.55f, kEtaInv = 10.0f;

// Shared-memory weight rows are padded by 8 halves so that the eight rows a
// B fragment reads fall in different banks.
constexpr int kPadIn = kIn + 8, kPadHid = kHid + 8;
struct FwdWeights {
    __half w1[kHid][kPadIn];
    __half w2[kHid][kPadHid];
    __half w3[kHid][kPadHid];
    __half w4[kHid][kPadHid];
    __half w5[kOut][kPadHid];
    float b1[kHid], b2[kHid], b3[kHid], b4[kHid], b5[kOut];
};
struct BwdWeights {
    __half w2t[kHid][kPadHid];
    __half w3t[kHid][kPadHid];
    __half w4t[kHid][kPadHid];
    __half w5t[kHid][kPadIn];
};

// Copy a rows x cols block of halves (cols a multiple of 8) into padded
// shared rows with 16-byte moves.
template <int PAD>
__device__ __forceinline__ void copy_rows(__half (*dst)[PAD], const __half* __restrict__ src, int rows, int cols,
                                          int tid, int nthreads) {
    const int per_row = cols / 8;
    for (int i = tid; i < rows * per_row; i += nthreads) {
        const int r = i / per_row, c = (i - r * per_row) * 8;
        *reinterpret_cast<uint4*>(&dst[r][c]) = __ldg(reinterpret_cast<const uint4*>(src + r * cols + c));
    }
}

// Load the forward weights (FP16, parameter layout) and FP32 biases; every
// thread of the block takes part.
__device__ __forceinline__ void load_fwd(FwdWeights& s, const __half* __restrict__ w16,
                                         const float* __restrict__ params, int tid, int nthreads) {
    copy_rows<kPadIn>(s.w1, w16 + kW1, kHid, kIn, tid, nthreads);
    copy_rows<kPadHid>(s.w2, w16 + kW2, kHid, kHid, tid, nthreads);
    copy_rows<kPadHid>(s.w3, w16 + kW3, kHid, kHid, tid, nthreads);
    copy_rows<kPadHid>(s.w4, w16 + kW4, kHid, kHid, tid, nthreads);
    copy_rows<kPadHid>(s.w5, w16 + kW5, kOut, kHid, tid, nthreads);
    for (int i = tid; i < kHid; i += nthreads) {
        s.b1[i] = params[kB1 + i];
        s.b2[i] = params[kB2 + i];
        s.b3[i] = params[kB3 + i];
        s.b4[i] = params[kB4 + i];
        if (i < kOut) s.b5[i] = params[kB5 + i];
    }
}

__device__ __forceinline__ void load_bwd(BwdWeights& s, const __half* __restrict__ wt16, int tid, int nthreads) {
    copy_rows<kPadHid>(s.w2t, wt16 + kT2, kHid, kHid, tid, nthreads);
    copy_rows<kPadHid>(s.w3t, wt16 + kT3, kHid, kHid, tid, nthreads);
    copy_rows<kPadHid>(s.w4t, wt16 + kT4, kHid, kHid, tid, nthreads);
    copy_rows<kPadIn>(s.w5t, wt16 + kT5, kHid, kOut, tid, nthreads);
}

__device__ __forceinline__ uint32_t pack_h2(float lo, float hi) {
    __half2 v = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ uint32_t ld32(const __half* p) { return *reinterpret_cast<const uint32_t*>(p); }

// D += A(16x16, row) * B(16x8, col), FP16 inputs, FP32 accumulate.
__device__ __forceinline__ void mma(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Network inputs of one evaluation from the shading quantities:
// sin_i, sin_o, cos_phi, sin_phi, sigma_a rgb, beta_m, beta_n, eta.
__device__ __forceinline__ void normalise(const float raw[kUsedIn], float x[kUsedIn]) {
    x[0] = raw[0];
    x[1] = raw[1];
    x[2] = raw[2];
    x[3] = raw[3];
    x[4] = (logf(fmaxf(raw[4], 1e-6f)) - kSigmaLogMid) * kSigmaLogInv;
    x[5] = (logf(fmaxf(raw[5], 1e-6f)) - kSigmaLogMid) * kSigmaLogInv;
    x[6] = (logf(fmaxf(raw[6], 1e-6f)) - kSigmaLogMid) * kSigmaLogInv;
    x[7] = (raw[7] - kBetaMMid) * kBetaMInv;
    x[8] = (raw[8] - kBetaNMid) * kBetaNInv;
    x[9] = (raw[9] - kEtaMid) * kEtaInv;
}

// Per-warp staging for the input/output transposes (row = lane).
struct WarpIo {
    __half x[32][kIn + 8];
    float y[32][kOut + 1];
};

// One layer: acc[mt][nt] = bias + A[mt] * W^T for N = 8*NT outputs, K = 16*KT
// inputs; bias may be null (zero).
template <int NT, int KT, int PAD>
__device__ __forceinline__ void layer(float acc[2][NT][4], const uint32_t a[2][KT][4], const __half (*w)[PAD],
                                      const float* bias, int g, int t) {
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const float bl = bias ? bias[nt * 8 + 2 * t] : 0.0f, bh = bias ? bias[nt * 8 + 2 * t + 1] : 0.0f;
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            acc[mt][nt][0] = bl;
            acc[mt][nt][1] = bh;
            acc[mt][nt][2] = bl;
            acc[mt][nt][3] = bh;
        }
    }
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const __half* row = w[nt * 8 + g] + kt * 16 + 2 * t;
            const uint32_t b0 = ld32(row), b1 = ld32(row + 8);
            mma(acc[0][nt], a[0][kt], b0, b1);
            mma(acc[1][nt], a[1][kt], b0, b1);
        }
    }
}

// C fragments of a 64-wide layer -> A fragments of the next (C n-tiles 2kt
// and 2kt+1 form k-tile kt).  RELU applies max(x, 0) first.
template <bool RELU>
__device__ __forceinline__ void c_to_a(const float acc[2][8][4], uint32_t a[2][4][4]) {
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const float* lo = acc[mt][2 * kt];
            const float* hi = acc[mt][2 * kt + 1];
            if (RELU) {
                a[mt][kt][0] = pack_h2(fmaxf(lo[0], 0.0f), fmaxf(lo[1], 0.0f));
                a[mt][kt][1] = pack_h2(fmaxf(lo[2], 0.0f), fmaxf(lo[3], 0.0f));
                a[mt][kt][2] = pack_h2(fmaxf(hi[0], 0.0f), fmaxf(hi[1], 0.0f));
                a[mt][kt][3] = pack_h2(fmaxf(hi[2], 0.0f), fmaxf(hi[3], 0.0f));
            } else {
                a[mt][kt][0] = pack_h2(lo[0], lo[1]);
                a[mt][kt][1] = pack_h2(lo[2], lo[3]);
                a[mt][kt][2] = pack_h2(hi[0], hi[1]);
                a[mt][kt][3] = pack_h2(hi[2], hi[3]);
            }
        }
}

// Bit (mt*8 + nt)*4 + e of the mask is set when the FP16 activation at C
// position (mt, nt, e) is positive, i.e. where the ReLU passes gradients.
__device__ __forceinline__ uint64_t relu_mask(const uint32_t a[2][4][4]) {
    uint64_t m = 0;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const uint32_t word = a[mt][nt >> 1][(nt & 1) * 2 + (e >> 1)];
                const uint32_t bits = (e & 1) ? (word >> 16) : (word & 0xffffu);
                if (bits & 0x7fffu) m |= 1ull << ((mt * 8 + nt) * 4 + e);
            }
    return m;
}

// Stage this lane's 16 inputs as FP16 and build the first layer's A fragments.
__device__ __forceinline__ void input_frags(WarpIo& io, const float x[kUsedIn], uint32_t a0[2][1][4], int lane,
                                            int g, int t) {
#pragma unroll
    for (int k = 0; k < kIn; k += 2)
        *reinterpret_cast<uint32_t*>(&io.x[lane][k]) =
            pack_h2(k < kUsedIn ? x[k] : 0.0f, k + 1 < kUsedIn ? x[k + 1] : 0.0f);
    __syncwarp();
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const int r = mt * 16 + g;
        a0[mt][0][0] = ld32(&io.x[r][2 * t]);
        a0[mt][0][1] = ld32(&io.x[r + 8][2 * t]);
        a0[mt][0][2] = ld32(&io.x[r][2 * t + 8]);
        a0[mt][0][3] = ld32(&io.x[r + 8][2 * t + 8]);
    }
    __syncwarp();
}

// Output C fragments -> this lane's row of 12 network outputs.
__device__ __forceinline__ void output_rows(WarpIo& io, const float out[2][2][4], float y[kUsedOut], int lane, int g,
                                            int t) {
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
            const int r = mt * 16 + g, c = nt * 8 + 2 * t;
            io.y[r][c] = out[mt][nt][0];
            io.y[r][c + 1] = out[mt][nt][1];
            io.y[r + 8][c] = out[mt][nt][2];
            io.y[r + 8][c + 1] = out[mt][nt][3];
        }
    __syncwarp();
#pragma unroll
    for (int c = 0; c < kUsedOut; ++c) y[c] = io.y[lane][c];
    __syncwarp();
}

// Forward pass of the 32 samples held by the warp's lanes: x[] are this
// lane's normalised inputs, y[] receives this lane's 12 network outputs
// (transformed space).  Every lane of the warp must call it.
__device__ __forceinline__ void forward(const FwdWeights& w, WarpIo& io, const float x[kUsedIn],
                                        float y[kUsedOut]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t a0[2][1][4];
    input_frags(io, x, a0, lane, g, t);
    float acc[2][8][4];
    uint32_t a[2][4][4];
    layer<8, 1, kPadIn>(acc, a0, w.w1, w.b1, g, t);
    c_to_a<true>(acc, a);
    layer<8, 4, kPadHid>(acc, a, w.w2, w.b2, g, t);
    c_to_a<true>(acc, a);
    layer<8, 4, kPadHid>(acc, a, w.w3, w.b3, g, t);
    c_to_a<true>(acc, a);
    layer<8, 4, kPadHid>(acc, a, w.w4, w.b4, g, t);
    c_to_a<true>(acc, a);
    float out[2][2][4];
    layer<2, 4, kPadHid>(out, a, w.w5, w.b5, g, t);
    output_rows(io, out, y, lane, g, t);
}

// ---------------------------------------------------------------- inference path
// The same network with the weight fragments read by ldmatrix (four B
// fragments per instruction) and ReLU fused into the FP16 conversion; the
// values are identical to forward().

__device__ __forceinline__ void ldsm_x4(uint32_t r[4], const void* p) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// max(x, 0) of two floats rounded to an FP16 pair (lo in the low half).
__device__ __forceinline__ uint32_t pack_relu(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.f16x2.f32 %0, %1, %2;\n" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

template <int NT, int KT, int PAD>
__device__ __forceinline__ void layer_ldsm(float acc[2][NT][4], const uint32_t a[2][KT][4], const __half (*w)[PAD],
                                           const float* bias, int lane) {
    const int t = lane & 3, mat = lane >> 3, r = lane & 7;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const float bl = bias[nt * 8 + 2 * t], bh = bias[nt * 8 + 2 * t + 1];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            acc[mt][nt][0] = bl;
            acc[mt][nt][1] = bh;
            acc[mt][nt][2] = bl;
            acc[mt][nt][3] = bh;
        }
    }
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
#pragma unroll
        for (int nt = 0; nt < NT; nt += 2) {
            uint32_t b[4];
            ldsm_x4(b, &w[(nt + (mat >> 1)) * 8 + r][kt * 16 + (mat & 1) * 8]);
            mma(acc[0][nt], a[0][kt], b[0], b[1]);
            mma(acc[1][nt], a[1][kt], b[0], b[1]);
            mma(acc[0][nt + 1], a[0][kt], b[2], b[3]);
            mma(acc[1][nt + 1], a[1][kt], b[2], b[3]);
        }
    }
}

__device__ __forceinline__ void relu_to_a(const float acc[2][8][4], uint32_t a[2][4][4]) {
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const float* lo = acc[mt][2 * kt];
            const float* hi = acc[mt][2 * kt + 1];
            a[mt][kt][0] = pack_relu(lo[0], lo[1]);
            a[mt][kt][1] = pack_relu(lo[2], lo[3]);
            a[mt][kt][2] = pack_relu(hi[0], hi[1]);
            a[mt][kt][3] = pack_relu(hi[2], hi[3]);
        }
}

__device__ __forceinline__ void forward_fast(const FwdWeights& w, WarpIo& io, const float x[kUsedIn],
                                             float y[kUsedOut]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t a0[2][1][4];
    input_frags(io, x, a0, lane, g, t);
    float acc[2][8][4];
    uint32_t a[2][4][4];
    layer_ldsm<8, 1, kPadIn>(acc, a0, w.w1, w.b1, lane);
    relu_to_a(acc, a);
    layer_ldsm<8, 4, kPadHid>(acc, a, w.w2, w.b2, lane);
    relu_to_a(acc, a);
    layer_ldsm<8, 4, kPadHid>(acc, a, w.w3, w.b3, lane);
    relu_to_a(acc, a);
    layer_ldsm<8, 4, kPadHid>(acc, a, w.w4, w.b4, lane);
    relu_to_a(acc, a);
    float out[2][2][4];
    layer_ldsm<2, 4, kPadHid>(out, a, w.w5, w.b5, lane);
    output_rows(io, out, y, lane, g, t);
}

// Network output (transformed) -> lobe value.
__device__ __forceinline__ float decode(float y) { return kScale * expm1f(fmaxf(y, 0.0f)); }
// The same with exp(y) - 1: at most ~1e-7 absolute before the 1e-3 scale,
// far below the network's own error.
__device__ __forceinline__ float decode_fast(float y) { return kScale * (__expf(fmaxf(y, 0.0f)) - 1.0f); }

}  // namespace mlp
}  // namespace hg
