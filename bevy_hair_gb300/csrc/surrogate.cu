// Learned shading surrogate: FP64 training samples of the hair lobes, the
// FP16 tensor-core networks' inference and training kernels (4 x 64: forward
// + backward per warp, split-K weight gradients, Adam; compact 2 x 32:
// forward, backward and weight gradients per warp on mma.sync, block-summed
// gradients, Adam), and their C entry
// points.  The reference has no counterpart; the shading it replaces is the
// Karis fit of shade.wesl:94-190.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstddef>

#include <cmath>
#include <cstring>
#include <mutex>
#include <new>

#include "hg_internal.h"
#include "hg_mlp.cuh"
#include "hg_mlp_small.cuh"
#include "hg_mlp_tc.cuh"

namespace hg {
namespace {

using namespace mlp;

constexpr int kGl = 64;
__constant__ double c_gl_x[kGl];
__constant__ double c_gl_w[kGl];
constexpr double kPiD = 3.14159265358979323846;

// ------------------------------------------------------------ FP64 lobes
//
// Single scattering S_p = M_p(theta_i + theta_o - alpha_p; beta_p) N_p(phi)
// (Marschner et al. 2003; d'Eon et al. 2011; Chiang et al. 2016) with
//   N_p(phi) = 1/2 Int A_p(h) D(phi - Phi_p(h); beta_n) dh,
// integrated over gamma_i = asin h with 64-point Gauss-Legendre (smooth in
// gamma_i; ~3e-11 relative against a 20001-point Simpson rule),
//   Phi_p = 2 p gamma_t - 2 gamma_i + p pi,  A_0 = F,  A_1 = (1-F)^2 T,  A_2 = (1-F)^2 F T^2,
// and the local back-scattering of the dual-scattering model (Zinke et al.
// 2008, Eqs. 13-17) from the same lobes' exact forward/backward azimuthal
// masses (wrapped-Gaussian CDF).  Longitudinal shapes follow shade.wesl:124-128.

__device__ double fresnel_d(double c, double eta) {
    c = fmin(fmax(c, 0.0), 1.0);
    const double st2 = (1.0 - c * c) / (eta * eta);
    if (st2 >= 1.0) return 1.0;
    const double ct = sqrt(1.0 - st2);
    const double rs = (c - eta * ct) / (c + eta * ct);
    const double rp = (eta * c - ct) / (eta * c + ct);
    return 0.5 * (rs * rs + rp * rp);
}

__device__ double gauss_d(double b, double x) {
    const double bb = fmax(b, 1e-3);
    return exp(-0.5 * x * x / (bb * bb)) / (2.5066282746310002 * bb);
}

struct NodeTerms {
    double f, gi, gt, tr[3];
};

// One quadrature node at gamma_i = u (h = sin u).
__device__ __forceinline__ NodeTerms node_terms(double u, double cos_td, double eta_p, double cos_tt, double eta,
                                                const double sa[3]) {
    NodeTerms n;
    n.gi = u;
    n.gt = asin(sin(u) / eta_p);
    n.f = fresnel_d(cos_td * cos(u), eta);
    const double path = 2.0 * cos(n.gt) / cos_tt;
#pragma unroll
    for (int c = 0; c < 3; ++c) n.tr[c] = exp(-sa[c] * path);
    return n;
}

__device__ __forceinline__ double attenuation(const NodeTerms& n, int p, int c) {
    const double omf2 = (1.0 - n.f) * (1.0 - n.f);
    return p == 0 ? n.f : (p == 1 ? omf2 * n.tr[c] : omf2 * n.f * n.tr[c] * n.tr[c]);
}

__device__ void lobes_fp64(const float* in, double tilt, double out[12]) {
    const double sin_i = fmin(fmax((double)in[0], -1.0), 1.0), sin_o = fmin(fmax((double)in[1], -1.0), 1.0);
    const double phi = atan2((double)in[3], (double)in[2]);
    const double sa[3] = {in[4], in[5], in[6]};
    const double beta_m = in[7], beta_n = in[8], eta = in[9];
    const double th_i = asin(sin_i), th_o = asin(sin_o), th_h = th_i + th_o;
    const double alpha[3] = {tilt, -0.5 * tilt, -1.5 * tilt};
    const double beta[3] = {beta_m, 0.5 * beta_m, 2.0 * beta_m};
    const double two_pi = 2.0 * kPiD;

    // single scattering at theta_d = (theta_o - theta_i) / 2
    {
        const double td = 0.5 * (th_o - th_i);
        const double cos_td = fmax(cos(td), 1e-3), sin_td = sin(td);
        const double eta_p = sqrt(eta * eta - sin_td * sin_td) / cos_td;
        const double sin_tt = sin_td / eta, cos_tt = sqrt(1.0 - sin_tt * sin_tt);
        const double inv2s2 = 0.5 / (beta_n * beta_n), norm = 1.0 / (2.5066282746310002 * beta_n);
        double n[3][3] = {};
        for (int i = 0; i < kGl; ++i) {
            const NodeTerms nt = node_terms(c_gl_x[i], cos_td, eta_p, cos_tt, eta, sa);
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                const double d = remainder(phi - (2.0 * p * nt.gt - 2.0 * nt.gi + p * kPiD), two_pi);
                const double dm = d - two_pi, dp = d + two_pi;
                const double D = norm * (exp(-d * d * inv2s2) + exp(-dp * dp * inv2s2) + exp(-dm * dm * inv2s2));
                const double wd = c_gl_w[i] * D;
#pragma unroll
                for (int c = 0; c < 3; ++c) n[p][c] += wd * attenuation(nt, p, c);
            }
        }
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            const double m = gauss_d(beta[p], th_h - alpha[p]);
#pragma unroll
            for (int c = 0; c < 3; ++c) out[3 * p + c] = m * 0.5 * n[p][c];
        }
    }

    // dual scattering at the specular cone, theta_d = theta_o (shade.wesl:444)
    const double cos_to = fmax(sqrt(fmax(1.0 - sin_o * sin_o, 1e-6)), 1e-3);
    const double sin_to = sqrt(fmax(0.0, 1.0 - cos_to * cos_to));
    const double eta_p = sqrt(eta * eta - sin_to * sin_to) / cos_to;
    const double sin_tt = sin_to / eta, cos_tt = sqrt(1.0 - sin_tt * sin_tt);
    const double r = 1.0 / (beta_n * 1.4142135623730951);
    double fwd[3][3] = {}, back[3][3] = {};
    for (int i = 0; i < kGl; ++i) {
        const NodeTerms nt = node_terms(c_gl_x[i], cos_to, eta_p, cos_tt, eta, sa);
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            // Wrapped-Gaussian masses of [-pi/2, pi/2] (back) and [pi/2, 3pi/2]
            // (forward) about the wrapped exit azimuth: shifts -2..2 of the
            // points pi/2 + j pi, j = -5..5.
            const double c0 = remainder(2.0 * p * nt.gt - 2.0 * nt.gi + p * kPiD, two_pi);
            double e[11];
#pragma unroll
            for (int j = 0; j < 11; ++j) e[j] = erf((0.5 * kPiD + (j - 5) * kPiD - c0) * r);
            const double mb = 0.5 * (((e[9] - e[8]) + (e[7] - e[6])) + ((e[5] - e[4]) + (e[3] - e[2])) + (e[1] - e[0]));
            const double mf =
                0.5 * (((e[10] - e[9]) + (e[8] - e[7])) + ((e[6] - e[5]) + (e[4] - e[3])) + (e[2] - e[1]));
            const double w = c_gl_w[i];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double wa = w * attenuation(nt, p, c);
                back[p][c] += wa * mb;
                fwd[p][c] += wa * mf;
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double f[3], b[3];
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            f[p] = 0.5 * fwd[p][c];
            b[p] = 0.5 * back[p][c];
        }
        const double a_f = fmin(f[0] + f[1] + f[2], 0.95);
        const double a_b = b[0] + b[1] + b[2];
        const double b2[3] = {beta[0] * beta[0], beta[1] * beta[1], beta[2] * beta[2]};
        const double tf = fmax(a_f, 1e-5), tb = fmax(a_b, 1e-5);
        const double beta_f2 = (f[0] * b2[0] + f[1] * b2[1] + f[2] * b2[2]) / tf;
        const double alpha_b = (b[0] * alpha[0] + b[1] * alpha[1] + b[2] * alpha[2]) / tb;
        const double beta_b2 = (b[0] * b2[0] + b[1] * b2[1] + b[2] * b2[2]) / tb;
        const double af2 = a_f * a_f, rest = 1.0 - af2, ab2 = a_b * a_b, ab3 = ab2 * a_b;
        const double a_back = a_b * af2 / rest + ab3 * af2 / (rest * rest * rest);
        const double delta_b = alpha_b * (1.0 - 2.0 * ab2 / (rest * rest)) +
                               alpha_b * (2.0 * rest * rest + 4.0 * af2 * ab2) / (rest * rest * rest);
        const double beta_f = sqrt(beta_f2), beta_b = sqrt(beta_b2);
        const double sigma_b = (1.0 + 0.7 * af2) *
                               (a_b * sqrt(2.0 * beta_f2 + beta_b2) + ab3 * sqrt(2.0 * beta_f2 + 3.0 * beta_b2)) /
                               fmax(a_b + ab3 * (2.0 * beta_f + 3.0 * beta_b), 1e-5);
        out[9 + c] = 2.0 * a_back * gauss_d(sigma_b, th_h - delta_b) / kPiD;
    }
}

// SplitMix64 (Steele, Lea and Flood 2014) as a counter-based generator.
__device__ __forceinline__ uint64_t splitmix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ float unit_float(uint64_t seed, uint64_t index, uint32_t dim) {
    const uint64_t h = splitmix(seed ^ splitmix(index * 16u + dim));
    return (float)(uint32_t)(h >> 40) * 0x1p-24f;
}

struct SampleArgs {
    uint64_t seed, first;
    uint32_t n;
    double tilt;
    float* inputs;   // [n][10]
    float* targets;  // [n][12] log1p(lobe / kScale), nullable
    double* lobes;   // [n][12], nullable
};

// Training distribution: sin theta_i, sin theta_o uniform in [-1, 1); phi
// uniform in [0, pi); sigma_a log-uniform in [0.02, 8]; beta_m uniform in
// [0.03, 0.3]; beta_n uniform in [0.2, 0.8]; eta = 1.55.
__global__ void __launch_bounds__(128) samples_kernel(const SampleArgs a) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n) return;
    const uint64_t idx = a.first + k;
    float x[10];
    x[0] = 2.0f * unit_float(a.seed, idx, 0) - 1.0f;
    x[1] = 2.0f * unit_float(a.seed, idx, 1) - 1.0f;
    const double phi = kPiD * (double)unit_float(a.seed, idx, 2);
    x[2] = (float)cos(phi);
    x[3] = (float)sin(phi);
    const double l0 = log(0.02), span = log(400.0);
#pragma unroll
    for (int c = 0; c < 3; ++c) x[4 + c] = (float)exp(l0 + span * (double)unit_float(a.seed, idx, 3 + c));
    x[7] = 0.03f + 0.27f * unit_float(a.seed, idx, 6);
    x[8] = 0.2f + 0.6f * unit_float(a.seed, idx, 7);
    x[9] = 1.55f;
#pragma unroll
    for (int i = 0; i < 10; ++i) a.inputs[(size_t)k * 10 + i] = x[i];
    double out[12];
    lobes_fp64(x, a.tilt, out);
#pragma unroll
    for (int i = 0; i < 12; ++i) {
        if (a.lobes) a.lobes[(size_t)k * 12 + i] = out[i];
        if (a.targets) a.targets[(size_t)k * 12 + i] = (float)log1p(out[i] / (double)kScale);
    }
}

// ------------------------------------------------------------ inference

constexpr int kWarps = 8;

__device__ __forceinline__ void load_raw(const float* __restrict__ inputs, uint32_t i, bool valid, float raw[10]) {
    const float dflt[10] = {0.0f, 0.0f, 1.0f, 0.0f, 0.4f, 0.4f, 0.4f, kBetaMMid, kBetaNMid, kEtaMid};
#pragma unroll
    for (int c = 0; c < 10; ++c) raw[c] = valid ? __ldg(&inputs[(size_t)i * 10 + c]) : dflt[c];
}

struct InferArgs {
    const float* inputs;
    uint32_t n;
    const __half* w16;
    const float* params;
    float* lobes;  // [n][12] decoded, nullable
    float* net;    // [n][12] network outputs, nullable
};

__global__ void __launch_bounds__(kWarps * 32) infer_kernel(const InferArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    FwdWeights& w = *reinterpret_cast<FwdWeights*>(smem);
    WarpIo* io = reinterpret_cast<WarpIo*>(smem + sizeof(FwdWeights));
    load_fwd(w, a.w16, a.params, threadIdx.x, blockDim.x);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t base = (blockIdx.x * kWarps + warp) * 32u; base < a.n; base += gridDim.x * kWarps * 32u) {
        const uint32_t i = base + lane;
        const bool valid = i < a.n;
        float raw[10], x[10], y[12];
        load_raw(a.inputs, i, valid, raw);
        normalise(raw, x);
        forward_fast(w, io[warp], x, y);
        if (valid) {
#pragma unroll
            for (int c = 0; c < 12; ++c) {
                if (a.lobes) a.lobes[(size_t)i * 12 + c] = decode(y[c]);
                if (a.net) a.net[(size_t)i * 12 + c] = y[c];
            }
        }
    }
}

// The compact network (hg_mlp_small.cuh) on mma.sync, 32 samples per warp;
// three outputs per sample (the BSDF rgb).
__global__ void __launch_bounds__(kWarps * 32) infer_small_kernel(const InferArgs a) {
    __shared__ __align__(16) mlps::Weights w;
    __shared__ __align__(16) WarpIo io[kWarps];
    mlps::load(w, a.w16, a.params, threadIdx.x, blockDim.x);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t base = (blockIdx.x * kWarps + warp) * 32u; base < a.n; base += gridDim.x * kWarps * 32u) {
        const uint32_t i = base + lane;
        const bool valid = i < a.n;
        float raw[10], x[10], y[mlp::kUsedOut];  // forward() fills 12 columns; the first kUsedOut are outputs
        load_raw(a.inputs, i, valid, raw);
        normalise(raw, x);
        mlps::forward(w, io[warp], x, y);
        if (valid) {
#pragma unroll
            for (int c = 0; c < mlps::kUsedOut; ++c) {
                if (a.lobes) a.lobes[(size_t)i * mlps::kUsedOut + c] = decode(y[c]);
                if (a.net) a.net[(size_t)i * mlps::kUsedOut + c] = y[c];
            }
        }
    }
}

// Training of the compact network on the tensor cores (mma.sync m16n8k16,
// FP16 operands, FP32 accumulation).  A warp takes 32 samples at a time:
//  forward   the inference network itself (mlps::forward's layers), keeping
//            the FP16 activations and the ReLU masks;
//  backward  dY = 2 (y - target) for the three BSDF channels, then
//            dZ2 = (dY W3) . [Z2 > 0] and dZ1 = (dZ2 W2) . [Z1 > 0], each a
//            product with a transposed weight matrix held in shared memory;
//  gradients dW = dZ^T A over the warp's samples, with the activations and
//            deltas transposed to [unit][sample] in shared memory so the
//            sample dimension is the MMAs' K; bias gradients are the row sums
//            of the transposed deltas.
// The deltas enter the MMAs rounded to FP16 (the usual mixed-precision
// backward); the block sums its warps' gradients in shared memory and adds
// them to `grad` once.  The loss is the sum over samples and the three
// channels of (y - target)^2; the targets are formed from the twelve lobes
// of hg_mlp_samples (mlps::bsdf_target).
struct SmallTrainArgs {
    const float* inputs;   // [n][10] raw
    const float* targets;  // [n][12] transformed lobes
    uint32_t n;
    const __half* w16;
    const float* params;
    float* grad;  // += d(sum of squared errors) / d(params)
    float* loss;  // += sum of squared errors
};

constexpr int kSmallTrainWarps = 4;
constexpr int kSampPad = 40;  // halves per transposed row: 32 samples + 8 (conflict-free ldmatrix)

// Per-warp transposes: [unit][sample].
struct SmallStage {
    __half x[mlps::kIn][kSampPad];
    __half a1[mlps::kHid][kSampPad];
    __half a2[mlps::kHid][kSampPad];
    __half dy[mlps::kOut][kSampPad];
    __half dz2[mlps::kHid][kSampPad];
    __half dz1[mlps::kHid][kSampPad];
};

// Every array that ldmatrix reads starts on a 16-byte boundary (its rows are
// multiples of 16 bytes), which the static_asserts below check.
struct SmallTrainSmem {
    alignas(16) mlps::Weights w;                        // forward weights (padded rows) and biases
    alignas(16) __half w3t[mlps::kHid][mlps::kPadIn];  // W3^T: [hidden][output]
    alignas(16) __half w2t[mlps::kHid][mlps::kPadHid]; // W2^T: [hidden 1][hidden 2]
    float zero[mlps::kHid];
    float grad[mlps::kParams];
    float loss;
    alignas(16) mlp::WarpIo io[kSmallTrainWarps];
    alignas(16) SmallStage st[kSmallTrainWarps];
};
static_assert(offsetof(SmallTrainSmem, w) % 16 == 0 && offsetof(SmallTrainSmem, w3t) % 16 == 0 &&
                  offsetof(SmallTrainSmem, w2t) % 16 == 0 && offsetof(SmallTrainSmem, st) % 16 == 0 &&
                  offsetof(SmallTrainSmem, io) % 16 == 0,
              "ldmatrix operands on 16-byte boundaries");
static_assert(offsetof(mlps::Weights, w2) % 16 == 0 && offsetof(mlps::Weights, w3) % 16 == 0, "weight rows");
static_assert(sizeof(SmallStage) % 16 == 0 && offsetof(SmallStage, a1) % 16 == 0 && offsetof(SmallStage, a2) % 16 == 0 &&
                  offsetof(SmallStage, dy) % 16 == 0 && offsetof(SmallStage, dz2) % 16 == 0 &&
                  offsetof(SmallStage, dz1) % 16 == 0 && (kSampPad * 2) % 16 == 0,
              "transposed rows on 16-byte boundaries");
static_assert((mlps::kPadIn * 2) % 16 == 0 && (mlps::kPadHid * 2) % 16 == 0, "padded weight rows");
constexpr size_t kSmallTrainSmem = sizeof(SmallTrainSmem);

// A packed FP16 pair of A fragment a[mt][kt][r] (rows = samples) into the
// transpose dst[unit][sample].
template <int KT>
__device__ __forceinline__ void stage_frags(__half (*dst)[kSampPad], const uint32_t a[2][KT][4], int g, int t) {
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int kt = 0; kt < KT; ++kt)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int unit = kt * 16 + 2 * t + ((r >> 1) ? 8 : 0);
                const int sample = mt * 16 + g + ((r & 1) ? 8 : 0);
                const __half2 v = *reinterpret_cast<const __half2*>(&a[mt][kt][r]);
                dst[unit][sample] = __low2half(v);
                dst[unit + 1][sample] = __high2half(v);
            }
}

// C fragments of a 32-wide layer times a 32-bit mask (bit (mt*4 + nt)*4 + e)
// -> FP16 A fragments.
__device__ __forceinline__ void masked_to_a(const float acc[2][4][4], uint32_t mask, uint32_t a[2][2][4]) {
    auto m = [&](int mt, int nt, int e) { return (mask >> ((mt * 4 + nt) * 4 + e)) & 1u ? acc[mt][nt][e] : 0.0f; };
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int kt = 0; kt < 2; ++kt) {
            a[mt][kt][0] = mlp::pack_h2(m(mt, 2 * kt, 0), m(mt, 2 * kt, 1));
            a[mt][kt][1] = mlp::pack_h2(m(mt, 2 * kt, 2), m(mt, 2 * kt, 3));
            a[mt][kt][2] = mlp::pack_h2(m(mt, 2 * kt + 1, 0), m(mt, 2 * kt + 1, 1));
            a[mt][kt][3] = mlp::pack_h2(m(mt, 2 * kt + 1, 2), m(mt, 2 * kt + 1, 3));
        }
}

__device__ __forceinline__ uint32_t positive_mask(const float acc[2][4][4]) {
    uint32_t m = 0;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) m |= (acc[mt][nt][e] > 0.0f ? 1u : 0u) << ((mt * 4 + nt) * 4 + e);
    return m;
}

// dW[m][n] += sum over the 32 samples of A[m][s] B[n][s] for MT 16-row tiles
// of A (rows m0..) and NT 8-row tiles of B, both [unit][sample], added to the
// shared gradient at grad[(m) * ld + n].
template <int MT, int NT>
__device__ __forceinline__ void wgrad(const __half (*A)[kSampPad], const __half (*B)[kSampPad], float* grad, int ld,
                                      int lane) {
    const int g = lane >> 2, t = lane & 3, mat = lane >> 3, r = lane & 7;
    float acc[MT][NT][4];
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) acc[mt][nt][0] = acc[mt][nt][1] = acc[mt][nt][2] = acc[mt][nt][3] = 0.0f;
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
        uint32_t af[MT][4];
#pragma unroll
        for (int mt = 0; mt < MT; ++mt)
            mlp::ldsm_x4(af[mt], &A[mt * 16 + (lane & 7) + ((lane >> 3) & 1) * 8][kt * 16 + (lane >> 4) * 8]);
#pragma unroll
        for (int nt = 0; nt < NT; nt += 2) {
            uint32_t b[4];
            mlp::ldsm_x4(b, &B[(nt + (mat >> 1)) * 8 + r][kt * 16 + (mat & 1) * 8]);
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                mlp::mma(acc[mt][nt], af[mt], b[0], b[1]);
                mlp::mma(acc[mt][nt + 1], af[mt], b[2], b[3]);
            }
        }
    }
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int row = mt * 16 + g, col = nt * 8 + 2 * t;
            atomicAdd(&grad[row * ld + col], acc[mt][nt][0]);
            atomicAdd(&grad[row * ld + col + 1], acc[mt][nt][1]);
            atomicAdd(&grad[(row + 8) * ld + col], acc[mt][nt][2]);
            atomicAdd(&grad[(row + 8) * ld + col + 1], acc[mt][nt][3]);
        }
}

__global__ void __launch_bounds__(kSmallTrainWarps * 32) small_train_kernel(const SmallTrainArgs a) {
    extern __shared__ __align__(16) unsigned char smem_small[];
    SmallTrainSmem& S = *reinterpret_cast<SmallTrainSmem*>(smem_small);
    const int tid = threadIdx.x, nth = blockDim.x;
    mlps::load(S.w, a.w16, a.params, tid, nth);
    for (int i = tid; i < mlps::kHid * mlps::kOut; i += nth) {
        const int j = i / mlps::kOut, o = i % mlps::kOut;  // W3^T[j][o] = W3[o][j]
        S.w3t[j][o] = a.w16[mlps::kW3 + o * mlps::kHid + j];
    }
    for (int i = tid; i < mlps::kHid * mlps::kHid; i += nth) {
        const int j1 = i / mlps::kHid, j2 = i % mlps::kHid;  // W2^T[j1][j2] = W2[j2][j1]
        S.w2t[j1][j2] = a.w16[mlps::kW2 + j2 * mlps::kHid + j1];
    }
    for (int i = tid; i < mlps::kHid; i += nth) S.zero[i] = 0.0f;
    for (int i = tid; i < mlps::kParams; i += nth) S.grad[i] = 0.0f;
    if (tid == 0) S.loss = 0.0f;
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    mlp::WarpIo& io = S.io[warp];
    SmallStage& st = S.st[warp];
    float loss = 0.0f;
    bool any = false;
    for (uint32_t base = (blockIdx.x * kSmallTrainWarps + warp) * 32u; base < a.n;
         base += gridDim.x * kSmallTrainWarps * 32u) {
        any = true;
        const uint32_t k = base + lane;
        const bool valid = k < a.n;
        float raw[10], xn[10];
        load_raw(a.inputs, k, valid, raw);
        normalise(raw, xn);
        // forward (the inference roundings: FP16 inputs, weights and activations)
        uint32_t a0[2][1][4];
        mlp::input_frags(io, xn, a0, lane, g, t);
        float acc[2][4][4];
        uint32_t a1[2][2][4], a2[2][2][4];
        mlp::layer_ldsm<4, 1, mlps::kPadIn>(acc, a0, S.w.w1, S.w.b1, lane);
        const uint32_t mask1 = positive_mask(acc);
        mlps::relu_to_a(acc, a1);
        mlp::layer_ldsm<4, 2, mlps::kPadHid>(acc, a1, S.w.w2, S.w.b2, lane);
        const uint32_t mask2 = positive_mask(acc);
        mlps::relu_to_a(acc, a2);
        float out[2][2][4];
        mlp::layer_ldsm<2, 2, mlps::kPadHid>(out, a2, S.w.w3, S.w.b3, lane);
        float y[mlp::kUsedOut];  // output_rows fills 12 columns; the first mlps::kUsedOut are outputs
        mlp::output_rows(io, out, y, lane, g, t);
        // dY of this lane's sample, as the next product's A operand
        float dy[mlps::kUsedOut];
#pragma unroll
        for (int o = 0; o < mlps::kUsedOut; ++o) {
            float d = 0.0f;
            if (valid) {
                float t12[12];
#pragma unroll
                for (int c = 0; c < 12; ++c) t12[c] = __ldg(&a.targets[(size_t)k * 12 + c]);
                d = y[o] - mlps::bsdf_target(t12, o);
            }
            loss += d * d;
            dy[o] = 2.0f * d;
        }
        float dyx[mlp::kUsedIn];
#pragma unroll
        for (int c = 0; c < mlp::kUsedIn; ++c) dyx[c] = c < mlps::kUsedOut ? dy[c] : 0.0f;
        uint32_t ady[2][1][4];
        mlp::input_frags(io, dyx, ady, lane, g, t);
        // backward through the layers
        mlp::layer_ldsm<4, 1, mlps::kPadIn>(acc, ady, S.w3t, S.zero, lane);  // dY W3
        uint32_t dz2[2][2][4], dz1[2][2][4];
        masked_to_a(acc, mask2, dz2);
        mlp::layer_ldsm<4, 2, mlps::kPadHid>(acc, dz2, S.w2t, S.zero, lane);  // dZ2 W2
        masked_to_a(acc, mask1, dz1);
        // transposes [unit][sample]
        stage_frags<1>(st.x, a0, g, t);
        stage_frags<2>(st.a1, a1, g, t);
        stage_frags<2>(st.a2, a2, g, t);
        stage_frags<1>(st.dy, ady, g, t);
        stage_frags<2>(st.dz2, dz2, g, t);
        stage_frags<2>(st.dz1, dz1, g, t);
        __syncwarp();
        // weight gradients over the warp's samples, then bias gradients
        wgrad<1, 4>(st.dy, st.a2, S.grad + mlps::kW3, mlps::kHid, lane);
        wgrad<2, 4>(st.dz2, st.a1, S.grad + mlps::kW2, mlps::kHid, lane);
        wgrad<2, 2>(st.dz1, st.x, S.grad + mlps::kW1, mlps::kIn, lane);
        {
            float s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
#pragma unroll 8
            for (int q = 0; q < 32; ++q) {
                s1 += __half2float(st.dz1[lane][q]);
                s2 += __half2float(st.dz2[lane][q]);
                if (lane < mlps::kOut) s3 += __half2float(st.dy[lane][q]);
            }
            atomicAdd(&S.grad[mlps::kB1 + lane], s1);
            atomicAdd(&S.grad[mlps::kB2 + lane], s2);
            if (lane < mlps::kOut) atomicAdd(&S.grad[mlps::kB3 + lane], s3);
        }
        __syncwarp();
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
    if (lane == 0 && any) atomicAdd(&S.loss, loss);
    __syncthreads();
    for (int i = tid; i < mlps::kParams; i += nth) {
        const float gv = S.grad[i];
        if (gv != 0.0f) atomicAdd(&a.grad[i], gv);
    }
    if (tid == 0 && S.loss != 0.0f) atomicAdd(a.loss, S.loss);
}

// The same evaluation on tcgen05: four chains of two 128-row evaluations per CTA.
__global__ void __launch_bounds__(tc::kThreads, 1) infer_tc_kernel(const InferArgs a, uint32_t* err) {
    extern __shared__ __align__(128) uint8_t smem_tc[];
    tc::Chain c = tc::setup(smem_tc, a.w16, a.params);
    const uint32_t g = threadIdx.x >> 7;
    const uint32_t chunks = (a.n + tc::kM - 1) / tc::kM;
    const uint32_t pairs = (chunks + 1) / 2;
    bool failed = false;
    for (uint32_t pc = blockIdx.x * tc::kChains + g; pc < pairs; pc += gridDim.x * tc::kChains) {
        const bool two = 2 * pc + 1 < chunks;
        uint32_t idx[2];
        bool valid[2];
        for (uint32_t e = 0; e < 2; ++e) {
            idx[e] = (2 * pc + e) * tc::kM + c.row;
            valid[e] = idx[e] < a.n && (e == 0 || two);
            float raw[10], x[10];
            load_raw(a.inputs, idx[e], valid[e], raw);
            normalise(raw, x);
            tc::write_input_row(c, e, x);
        }
        float y[2][12];
        if (!tc::forward2(c, two, y[0], y[1])) {
            failed = true;
            break;
        }
        for (uint32_t e = 0; e < 2; ++e) {
            if (!valid[e]) continue;
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                if (a.lobes) a.lobes[(size_t)idx[e] * 12 + k] = decode(y[e][k]);
                if (a.net) a.net[(size_t)idx[e] * 12 + k] = y[e][k];
            }
        }
    }
    if (failed && c.row == 0) atomicOr(err, tc::kErrTimeout);
    tc::teardown(smem_tc, c, failed);
}

// ------------------------------------------------------------ training

// Per-warp transpose stage: [unit][32 samples + 8 pad].
struct Stage {
    __half v[kHid][40];
};

// Write packed fragments (KT k-tiles of 16 units, rows = the warp's 32
// samples) to dst[unit][col0 + sample] through the stage.
template <int KT>
__device__ __forceinline__ void store_t(Stage& st, const uint32_t a[2][KT][4], __half* __restrict__ dst, uint32_t ld,
                                        uint32_t col0, int lane, int g, int t) {
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int kt = 0; kt < KT; ++kt)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int unit = kt * 16 + 2 * t + ((r >> 1) ? 8 : 0);
                const int sample = mt * 16 + g + ((r & 1) ? 8 : 0);
                const __half2 v = *reinterpret_cast<const __half2*>(&a[mt][kt][r]);
                st.v[unit][sample] = __low2half(v);
                st.v[unit + 1][sample] = __high2half(v);
            }
    __syncwarp();
#pragma unroll
    for (int i = lane; i < KT * 16 * 4; i += 32) {
        const int u = i >> 2, c = (i & 3) * 8;
        *reinterpret_cast<uint4*>(dst + (size_t)u * ld + col0 + c) = *reinterpret_cast<const uint4*>(&st.v[u][c]);
    }
    __syncwarp();
}

__device__ __forceinline__ void apply_mask(float acc[2][8][4], uint64_t m) {
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (!((m >> ((mt * 8 + nt) * 4 + e)) & 1ull)) acc[mt][nt][e] = 0.0f;
}

struct TrainArgs {
    const float* inputs;   // [n][10]
    const float* targets;  // [n][12] transformed
    uint32_t n, ld;        // samples; row length of the transposed buffers (multiple of 32, >= n)
    const __half* w16;
    const __half* wt16;
    const float* params;
    __half* xt;    // [16][ld]   layer-1 inputs
    __half* ht;    // [4][64][ld] hidden activations h1..h4
    __half* dzt;   // [4][64][ld] pre-activation gradients of layers 1..4
    __half* dz5t;  // [16][ld]   output gradients
    float* loss;   // += sum of squared errors
};

// Forward and backward of 32 samples per warp.  The loss is the sum over
// samples and the 12 outputs of (y - target)^2, so dL/dy = 2 (y - target);
// the 1/(n*12) of the mean is applied by the optimiser.
__global__ void __launch_bounds__(kWarps * 32, 1) train_kernel(const TrainArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    FwdWeights& fw = *reinterpret_cast<FwdWeights*>(smem);
    BwdWeights& bw = *reinterpret_cast<BwdWeights*>(smem + sizeof(FwdWeights));
    WarpIo* io = reinterpret_cast<WarpIo*>(smem + sizeof(FwdWeights) + sizeof(BwdWeights));
    Stage* stage = reinterpret_cast<Stage*>(io + kWarps);
    load_fwd(fw, a.w16, a.params, threadIdx.x, blockDim.x);
    load_bwd(bw, a.wt16, threadIdx.x, blockDim.x);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint32_t base = (blockIdx.x * kWarps + warp) * 32u;
    if (base >= a.n) return;
    const uint32_t i = base + lane;
    const bool valid = i < a.n;
    WarpIo& w_io = io[warp];
    Stage& st = stage[warp];
    const size_t plane = (size_t)kHid * a.ld;

    float raw[10], x[10];
    load_raw(a.inputs, i, valid, raw);
    normalise(raw, x);
    uint32_t a0[2][1][4];
    input_frags(w_io, x, a0, lane, g, t);
    store_t<1>(st, a0, a.xt, a.ld, base, lane, g, t);

    float acc[2][8][4];
    uint32_t h[2][4][4];
    uint64_t m1, m2, m3, m4;
    layer<8, 1, kPadIn>(acc, a0, fw.w1, fw.b1, g, t);
    c_to_a<true>(acc, h);
    m1 = relu_mask(h);
    store_t<4>(st, h, a.ht, a.ld, base, lane, g, t);
    layer<8, 4, kPadHid>(acc, h, fw.w2, fw.b2, g, t);
    c_to_a<true>(acc, h);
    m2 = relu_mask(h);
    store_t<4>(st, h, a.ht + plane, a.ld, base, lane, g, t);
    layer<8, 4, kPadHid>(acc, h, fw.w3, fw.b3, g, t);
    c_to_a<true>(acc, h);
    m3 = relu_mask(h);
    store_t<4>(st, h, a.ht + 2 * plane, a.ld, base, lane, g, t);
    layer<8, 4, kPadHid>(acc, h, fw.w4, fw.b4, g, t);
    c_to_a<true>(acc, h);
    m4 = relu_mask(h);
    store_t<4>(st, h, a.ht + 3 * plane, a.ld, base, lane, g, t);
    float out[2][2][4];
    layer<2, 4, kPadHid>(out, h, fw.w5, fw.b5, g, t);

    // Targets into the C layout through the warp's output stage; column 16
    // flags a real sample.
#pragma unroll
    for (int c = 0; c < kUsedOut; ++c) w_io.y[lane][c] = valid ? __ldg(&a.targets[(size_t)i * 12 + c]) : 0.0f;
    w_io.y[lane][16] = valid ? 1.0f : 0.0f;
    __syncwarp();
    float lsum = 0.0f;
    uint32_t d5[2][1][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        float dy[2][4];
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int r = mt * 16 + g + ((e >> 1) ? 8 : 0), c = nt * 8 + 2 * t + (e & 1);
                float d = 0.0f;
                if (c < kUsedOut && w_io.y[r][16] != 0.0f) d = out[mt][nt][e] - w_io.y[r][c];
                lsum += d * d;
                dy[nt][e] = 2.0f * d;
            }
        d5[mt][0][0] = pack_h2(dy[0][0], dy[0][1]);
        d5[mt][0][1] = pack_h2(dy[0][2], dy[0][3]);
        d5[mt][0][2] = pack_h2(dy[1][0], dy[1][1]);
        d5[mt][0][3] = pack_h2(dy[1][2], dy[1][3]);
    }
    __syncwarp();
    store_t<1>(st, d5, a.dz5t, a.ld, base, lane, g, t);

    layer<8, 1, kPadIn>(acc, d5, bw.w5t, nullptr, g, t);
    apply_mask(acc, m4);
    c_to_a<false>(acc, h);
    store_t<4>(st, h, a.dzt + 3 * plane, a.ld, base, lane, g, t);
    layer<8, 4, kPadHid>(acc, h, bw.w4t, nullptr, g, t);
    apply_mask(acc, m3);
    c_to_a<false>(acc, h);
    store_t<4>(st, h, a.dzt + 2 * plane, a.ld, base, lane, g, t);
    layer<8, 4, kPadHid>(acc, h, bw.w3t, nullptr, g, t);
    apply_mask(acc, m2);
    c_to_a<false>(acc, h);
    store_t<4>(st, h, a.dzt + plane, a.ld, base, lane, g, t);
    layer<8, 4, kPadHid>(acc, h, bw.w2t, nullptr, g, t);
    apply_mask(acc, m1);
    c_to_a<false>(acc, h);
    store_t<4>(st, h, a.dzt, a.ld, base, lane, g, t);

#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0) atomicAdd(a.loss, lsum);
}

struct WgradArgs {
    const __half* xt;
    const __half* ht;
    const __half* dzt;
    const __half* dz5t;
    uint32_t ld, n_pad, chunk;
    float* grad;
};

__device__ __forceinline__ uint32_t ldg32(const __half* p) { return __ldg(reinterpret_cast<const unsigned int*>(p)); }

__device__ __forceinline__ float h2sum(uint32_t v) {
    const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&v));
    return f.x + f.y;
}

// dW[m0.., n0..] += A[m][k0:k1] * B[n][k0:k1]^T (A = dZ^T, B = H^T, both
// [unit][sample]); optional row sums of A for the bias gradient.
template <int NT>
__device__ __forceinline__ void wgrad_tile(const __half* __restrict__ A, const __half* __restrict__ B, uint32_t ld,
                                           int m0, int n0, uint32_t k0, uint32_t k1, float* gw, int n_cols, float* gb,
                                           int g, int t) {
    float acc[NT][4] = {};
    float s0 = 0.0f, s1 = 0.0f;
    const __half* r0 = A + (size_t)(m0 + g) * ld + 2 * t;
    const __half* r1 = A + (size_t)(m0 + g + 8) * ld + 2 * t;
#pragma unroll 2
    for (uint32_t k = k0; k < k1; k += 16) {
        const uint32_t af[4] = {ldg32(r0 + k), ldg32(r1 + k), ldg32(r0 + k + 8), ldg32(r1 + k + 8)};
        if (gb) {
            s0 += h2sum(af[0]) + h2sum(af[2]);
            s1 += h2sum(af[1]) + h2sum(af[3]);
        }
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const __half* br = B + (size_t)(n0 + nt * 8 + g) * ld + k + 2 * t;
            mma(acc[nt], af, ldg32(br), ldg32(br + 8));
        }
    }
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const int c = n0 + nt * 8 + 2 * t;
        atomicAdd(gw + (m0 + g) * n_cols + c, acc[nt][0]);
        atomicAdd(gw + (m0 + g) * n_cols + c + 1, acc[nt][1]);
        atomicAdd(gw + (m0 + g + 8) * n_cols + c, acc[nt][2]);
        atomicAdd(gw + (m0 + g + 8) * n_cols + c + 1, acc[nt][3]);
    }
    if (gb) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
        s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
        s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
        s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
        if (t == 0) {
            atomicAdd(gb + m0 + g, s0);
            atomicAdd(gb + m0 + g + 8, s1);
        }
    }
}

// grid (chunks, 5 layers), 4 warps.
__global__ void __launch_bounds__(128) wgrad_kernel(const WgradArgs a) {
    const int layer = blockIdx.y, warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint32_t k0 = blockIdx.x * a.chunk;
    const uint32_t k1 = min(k0 + a.chunk, a.n_pad);
    if (k0 >= k1) return;
    const size_t plane = (size_t)kHid * a.ld;
    switch (layer) {
        case 0:
            wgrad_tile<2>(a.dzt, a.xt, a.ld, 16 * warp, 0, k0, k1, a.grad + kW1, kIn, a.grad + kB1, g, t);
            break;
        case 1:
        case 2:
        case 3: {
            const int wofs = layer == 1 ? kW2 : (layer == 2 ? kW3 : kW4);
            const int bofs = layer == 1 ? kB2 : (layer == 2 ? kB3 : kB4);
            wgrad_tile<8>(a.dzt + layer * plane, a.ht + (layer - 1) * plane, a.ld, 16 * warp, 0, k0, k1,
                          a.grad + wofs, kHid, a.grad + bofs, g, t);
            break;
        }
        default:
            wgrad_tile<2>(a.dz5t, a.ht + 3 * plane, a.ld, 0, 16 * warp, k0, k1, a.grad + kW5, kHid,
                          warp == 0 ? a.grad + kB5 : nullptr, g, t);
            break;
    }
}

struct AdamArgs {
    float* params;
    float* m;
    float* v;
    float* grad;
    __half* w16;
    __half* wt16;
    float lr_t, beta1, beta2, eps_t, gscale;
    int update;
};

// Adam (Kingma and Ba 2015) with the bias corrections folded into lr_t and
// eps_t; then the FP16 forward and transposed copies.
__global__ void adam_kernel(const AdamArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    float p = a.params[i];
    if (a.update) {
        const float gr = a.grad[i] * a.gscale;
        const float m = a.beta1 * a.m[i] + (1.0f - a.beta1) * gr;
        const float v = a.beta2 * a.v[i] + (1.0f - a.beta2) * gr * gr;
        a.m[i] = m;
        a.v[i] = v;
        p -= a.lr_t * m / (sqrtf(v) + a.eps_t);
        a.params[i] = p;
        a.grad[i] = 0.0f;
    }
    const __half hp = __float2half_rn(p);
    a.w16[i] = hp;
    int tofs = -1, rows = 0, cols = kHid, rel = 0;
    if (i >= kW2 && i < kB2) tofs = kT2, rows = kHid, rel = i - kW2;
    else if (i >= kW3 && i < kB3) tofs = kT3, rows = kHid, rel = i - kW3;
    else if (i >= kW4 && i < kB4) tofs = kT4, rows = kHid, rel = i - kW4;
    else if (i >= kW5 && i < kB5) tofs = kT5, rows = kOut, rel = i - kW5;
    if (tofs >= 0) {
        const int r = rel / cols, c = rel - r * cols;
        a.wt16[tofs + c * rows + r] = hp;
    }
}

// Adam for the compact network (no transposed copies).
__global__ void adam_small_kernel(const AdamArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= mlps::kParams) return;
    float p = a.params[i];
    if (a.update) {
        const float gr = a.grad[i] * a.gscale;
        const float m = a.beta1 * a.m[i] + (1.0f - a.beta1) * gr;
        const float v = a.beta2 * a.v[i] + (1.0f - a.beta2) * gr * gr;
        a.m[i] = m;
        a.v[i] = v;
        p -= a.lr_t * m / (sqrtf(v) + a.eps_t);
        a.params[i] = p;
        a.grad[i] = 0.0f;
    }
    a.w16[i] = __float2half_rn(p);
}

// ------------------------------------------------------------ host side

constexpr size_t kFwdSmem = sizeof(FwdWeights) + kWarps * sizeof(WarpIo);
constexpr size_t kTrainSmem = sizeof(FwdWeights) + sizeof(BwdWeights) + kWarps * (sizeof(WarpIo) + sizeof(Stage));
static_assert(kTrainSmem <= 227 * 1024, "train kernel shared memory");

std::mutex g_init_mutex;
bool g_gl_ready[64] = {};
bool g_attr_ready[64] = {};
static_assert(tc::kSmemBytes <= 227 * 1024, "tcgen05 kernel shared memory");

// Gauss-Legendre nodes by Newton iteration on P_64, mapped to gamma_i in
// [-pi/2, pi/2] with the Jacobian cos(gamma_i) folded into the weights.
void gauss_legendre(double* x, double* w) {
    const int n = kGl;
    for (int i = 0; i < n; ++i) {
        double z = std::cos(kPiD * (i + 0.75) / (n + 0.5));
        double dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; ++k) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; ++k) {
            const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[i] = 0.5 * kPiD * z;
        w[i] = 0.5 * kPiD * 2.0 / ((1.0 - z * z) * dp * dp) * std::cos(x[i]);
    }
}

cudaError_t ensure_device_setup(int device) {
    std::lock_guard<std::mutex> lock(g_init_mutex);
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    cudaError_t e = cudaSuccess;
    if (!g_gl_ready[device]) {
        double x[kGl], w[kGl];
        gauss_legendre(x, w);
        e = cudaMemcpyToSymbol(c_gl_x, x, sizeof(x));
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gl_w, w, sizeof(w));
        if (e != cudaSuccess) return e;
        g_gl_ready[device] = true;
    }
    if (!g_attr_ready[device]) {
        e = cudaFuncSetAttribute(infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFwdSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tc::kSmemBytes);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(small_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kSmallTrainSmem);
        if (e != cudaSuccess) return e;
        g_attr_ready[device] = true;
    }
    return cudaSuccess;
}

hg_status fail(hg_ctx* ctx, hg_status s, const char* msg) {
    if (ctx) ctx->last_error = msg;
    return s;
}

hg_status cuda_fail(hg_ctx* ctx, cudaError_t e, const char* where) {
    if (ctx) ctx->last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? HG_OUT_OF_MEMORY : HG_CUDA_ERROR;
}

#define MLP_CUDA(ctx, expr)                                     \
    do {                                                        \
        cudaError_t e_ = (expr);                                \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #expr); \
    } while (0)

cudaError_t convert(hg_mlp* m, int update, float lr_t, float eps_t, float gscale) {
    AdamArgs a;
    a.params = m->params;
    a.m = m->adam_m;
    a.v = m->adam_v;
    a.grad = m->grad;
    a.w16 = reinterpret_cast<__half*>(m->w16);
    a.wt16 = reinterpret_cast<__half*>(m->wt16);
    a.lr_t = lr_t;
    a.beta1 = 0.9f;
    a.beta2 = 0.999f;
    a.eps_t = eps_t;
    a.gscale = gscale;
    a.update = update;
    if (m->arch == HG_MLP_ARCH_COMPACT)
        adam_small_kernel<<<(mlps::kParams + 255) / 256, 256, 0, m->ctx->stream>>>(a);
    else
        adam_kernel<<<(kParams + 255) / 256, 256, 0, m->ctx->stream>>>(a);
    return cudaGetLastError();
}

// Grow the transposed activation buffers to hold n samples.
cudaError_t ensure_scratch(hg_mlp* m, uint32_t n) {
    const uint32_t ld = (n + 31u) & ~31u;
    if (ld <= m->ld_capacity) return cudaSuccess;
    cudaStreamSynchronize(m->ctx->stream);
    if (m->scratch) cudaFree(m->scratch);
    m->scratch = nullptr;
    m->ld_capacity = 0;
    const size_t halves = (size_t)(kIn + 4 * kHid + 4 * kHid + kOut) * ld;
    cudaError_t e = cudaMalloc(&m->scratch, halves * sizeof(__half));
    if (e != cudaSuccess) return e;
    m->ld_capacity = ld;
    return cudaSuccess;
}

// Forward + backward + weight gradients of n samples into m->grad (sum of
// squared errors) and m->loss.
cudaError_t run_gradients(hg_mlp* m, const float* inputs, const float* targets, uint32_t n) {
    if (m->arch == HG_MLP_ARCH_COMPACT) {
        SmallTrainArgs s;
        s.inputs = inputs;
        s.targets = targets;
        s.n = n;
        s.w16 = reinterpret_cast<const __half*>(m->w16);
        s.params = m->params;
        s.grad = m->grad;
        s.loss = m->loss;
        // persistent warps: each takes several 32-sample tiles, each block adds its sums once
        const uint32_t tiles = (n + 31u) / 32u;
        const uint32_t want = (tiles + kSmallTrainWarps - 1) / kSmallTrainWarps;
        const uint32_t blocks = std::max(1u, std::min(want, (uint32_t)m->ctx->sm_count * 4u));
        small_train_kernel<<<blocks, kSmallTrainWarps * 32, kSmallTrainSmem, m->ctx->stream>>>(s);
        return cudaGetLastError();
    }
    const uint32_t ld = m->ld_capacity;
    __half* s = reinterpret_cast<__half*>(m->scratch);
    TrainArgs a;
    a.inputs = inputs;
    a.targets = targets;
    a.n = n;
    a.ld = ld;
    a.w16 = reinterpret_cast<const __half*>(m->w16);
    a.wt16 = reinterpret_cast<const __half*>(m->wt16);
    a.params = m->params;
    a.xt = s;
    a.ht = s + (size_t)kIn * ld;
    a.dzt = a.ht + (size_t)4 * kHid * ld;
    a.dz5t = a.dzt + (size_t)4 * kHid * ld;
    a.loss = m->loss;
    const uint32_t warps = (n + 31u) / 32u;
    train_kernel<<<(warps + kWarps - 1) / kWarps, kWarps * 32, kTrainSmem, m->ctx->stream>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    WgradArgs w;
    w.xt = a.xt;
    w.ht = a.ht;
    w.dzt = a.dzt;
    w.dz5t = a.dz5t;
    w.ld = ld;
    w.n_pad = warps * 32u;
    w.chunk = 2048u;
    w.grad = m->grad;
    dim3 grid((w.n_pad + w.chunk - 1) / w.chunk, 5);
    wgrad_kernel<<<grid, 128, 0, m->ctx->stream>>>(w);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_mlp_infer_tc(hg_mlp* m, const float* inputs, uint32_t n, float* lobes, float* net) {
    InferArgs a;
    a.inputs = inputs;
    a.n = n;
    a.w16 = reinterpret_cast<const __half*>(m->w16);
    a.params = m->params;
    a.lobes = lobes;
    a.net = net;
    const uint32_t pairs = ((n + tc::kM - 1) / tc::kM + 1) / 2;
    uint32_t blocks = (pairs + tc::kChains - 1) / tc::kChains;
    // one CTA per SM: it holds all 512 TMEM columns and most of the shared memory
    const uint32_t cap = (uint32_t)m->ctx->sm_count;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    infer_tc_kernel<<<blocks, tc::kThreads, tc::kSmemBytes, m->ctx->stream>>>(a, m->ctx->err);
    return cudaGetLastError();
}

cudaError_t launch_mlp_infer(hg_mlp* m, const float* inputs, uint32_t n, float* lobes, float* net) {
    InferArgs a;
    a.inputs = inputs;
    a.n = n;
    a.w16 = reinterpret_cast<const __half*>(m->w16);
    a.params = m->params;
    a.lobes = lobes;
    a.net = net;
    const uint32_t warps = (n + 31u) / 32u;
    uint32_t blocks = (warps + kWarps - 1) / kWarps;
    if (m->arch == HG_MLP_ARCH_COMPACT) {
        const uint32_t cap = (uint32_t)m->ctx->sm_count * 8u;
        if (blocks > cap) blocks = cap;
        infer_small_kernel<<<blocks, kWarps * 32, 0, m->ctx->stream>>>(a);
        return cudaGetLastError();
    }
    const uint32_t cap = (uint32_t)m->ctx->sm_count * 3u;
    if (blocks > cap) blocks = cap;
    infer_kernel<<<blocks, kWarps * 32, kFwdSmem, m->ctx->stream>>>(a);
    return cudaGetLastError();
}

}  // namespace hg

using hg::cuda_fail;
using hg::fail;

extern "C" {

hg_status hg_mlp_create(hg_ctx* ctx, hg_mlp** out) { return hg_mlp_create_arch(ctx, HG_MLP_ARCH_DEEP, out); }

hg_status hg_mlp_create_arch(hg_ctx* ctx, uint32_t arch, hg_mlp** out) {
    if (!ctx || !out) return HG_INVALID_ARG;
    *out = nullptr;
    if (arch != HG_MLP_ARCH_DEEP && arch != HG_MLP_ARCH_COMPACT)
        return fail(ctx, HG_INVALID_ARG, "unknown surrogate architecture");
    cudaSetDevice(ctx->device);
    MLP_CUDA(ctx, hg::ensure_device_setup(ctx->device));
    hg_mlp* m = new (std::nothrow) hg_mlp();
    if (!m) return fail(ctx, HG_OUT_OF_MEMORY, "allocating the surrogate");
    m->ctx = ctx;
    m->arch = arch;
    m->n_params = arch == HG_MLP_ARCH_COMPACT ? (uint32_t)hg::mlps::kParams : (uint32_t)hg::mlp::kParams;
    const size_t pf = sizeof(float) * m->n_params;
    cudaError_t e = cudaMalloc(&m->params, pf);
    if (e == cudaSuccess) e = cudaMalloc(&m->grad, pf);
    if (e == cudaSuccess) e = cudaMalloc(&m->adam_m, pf);
    if (e == cudaSuccess) e = cudaMalloc(&m->adam_v, pf);
    if (e == cudaSuccess) e = cudaMalloc(&m->w16, sizeof(__half) * m->n_params);
    if (e == cudaSuccess && arch == HG_MLP_ARCH_DEEP)
        e = cudaMalloc(&m->wt16, sizeof(__half) * hg::mlp::kTransposed);
    if (e == cudaSuccess) e = cudaMalloc(&m->loss, sizeof(float));
    for (void* p : {(void*)m->params, (void*)m->grad, (void*)m->adam_m, (void*)m->adam_v})
        if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, pf, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->loss, 0, sizeof(float), ctx->stream);
    if (e == cudaSuccess) e = hg::convert(m, 0, 0.0f, 0.0f, 0.0f);
    if (e != cudaSuccess) {
        hg_mlp_destroy(m);
        return cuda_fail(ctx, e, "creating the surrogate");
    }
    *out = m;
    return HG_OK;
}

void hg_mlp_destroy(hg_mlp* m) {
    if (!m) return;
    hg_ctx* ctx = m->ctx;
    if (ctx) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        if (ctx->surrogate == m) ctx->surrogate = nullptr;
    }
    for (void* p : {(void*)m->params, (void*)m->grad, (void*)m->adam_m, (void*)m->adam_v, (void*)m->w16,
                    (void*)m->wt16, (void*)m->loss, m->scratch})
        if (p) cudaFree(p);
    delete m;
}

uint32_t hg_mlp_param_count(const hg_mlp* m) { return m ? m->n_params : 0u; }

uint32_t hg_mlp_output_count(const hg_mlp* m) {
    if (!m) return 0u;
    return m->arch == HG_MLP_ARCH_COMPACT ? (uint32_t)hg::mlps::kUsedOut : (uint32_t)hg::mlp::kUsedOut;
}

hg_status hg_mlp_set_params(hg_mlp* m, const float* params, uint32_t count) {
    if (!m || !params) return HG_INVALID_ARG;
    hg_ctx* ctx = m->ctx;
    if (count != m->n_params) return fail(ctx, HG_INVALID_ARG, "parameter count must be hg_mlp_param_count");
    for (uint32_t i = 0; i < count; ++i)
        if (!std::isfinite(params[i])) return fail(ctx, HG_INVALID_ARG, "non-finite parameter");
    const size_t pf = sizeof(float) * count;
    MLP_CUDA(ctx, cudaMemcpyAsync(m->params, params, pf, cudaMemcpyHostToDevice, ctx->stream));
    MLP_CUDA(ctx, cudaMemsetAsync(m->adam_m, 0, pf, ctx->stream));
    MLP_CUDA(ctx, cudaMemsetAsync(m->adam_v, 0, pf, ctx->stream));
    MLP_CUDA(ctx, cudaMemsetAsync(m->grad, 0, pf, ctx->stream));
    MLP_CUDA(ctx, hg::convert(m, 0, 0.0f, 0.0f, 0.0f));
    MLP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    m->step = 0;
    return HG_OK;
}

hg_status hg_mlp_get_params(hg_mlp* m, float* params, uint32_t count) {
    if (!m || !params) return HG_INVALID_ARG;
    hg_ctx* ctx = m->ctx;
    if (count != m->n_params) return fail(ctx, HG_INVALID_ARG, "parameter count must be hg_mlp_param_count");
    MLP_CUDA(ctx, cudaMemcpyAsync(params, m->params, sizeof(float) * count, cudaMemcpyDeviceToHost, ctx->stream));
    MLP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HG_OK;
}

hg_status hg_mlp_samples(hg_ctx* ctx, uint64_t seed, uint64_t first, uint32_t count, float tilt, float* inputs,
                         float* targets, double* lobes) {
    if (!ctx) return HG_INVALID_ARG;
    if (count == 0) return HG_OK;
    if (!inputs) return fail(ctx, HG_INVALID_ARG, "null inputs buffer");
    if (!std::isfinite(tilt)) return fail(ctx, HG_INVALID_ARG, "non-finite tilt");
    cudaSetDevice(ctx->device);
    MLP_CUDA(ctx, cudaPeekAtLastError());  // an earlier error is reported, not cleared
    MLP_CUDA(ctx, hg::ensure_device_setup(ctx->device));
    hg::SampleArgs a;
    a.seed = seed;
    a.first = first;
    a.n = count;
    a.tilt = (double)tilt;
    a.inputs = inputs;
    a.targets = targets;
    a.lobes = lobes;
    hg::samples_kernel<<<(count + 127u) / 128u, 128, 0, ctx->stream>>>(a);
    MLP_CUDA(ctx, cudaGetLastError());
    return HG_OK;
}

hg_status hg_mlp_infer(hg_mlp* m, const float* inputs, uint32_t count, float* lobes, float* net) {
    if (!m) return HG_INVALID_ARG;
    if (count == 0) return HG_OK;
    if (!inputs || (!lobes && !net)) return fail(m->ctx, HG_INVALID_ARG, "null buffer");
    MLP_CUDA(m->ctx, cudaPeekAtLastError());
    MLP_CUDA(m->ctx, hg::launch_mlp_infer(m, inputs, count, lobes, net));
    return HG_OK;
}

hg_status hg_mlp_infer_tc(hg_mlp* m, const float* inputs, uint32_t count, float* lobes, float* net) {
    if (!m) return HG_INVALID_ARG;
    if (m->arch != HG_MLP_ARCH_DEEP) return fail(m->ctx, HG_INVALID_ARG, "tcgen05 inference runs the 4 x 64 network");
    if (count == 0) return HG_OK;
    if (!inputs || (!lobes && !net)) return fail(m->ctx, HG_INVALID_ARG, "null buffer");
    MLP_CUDA(m->ctx, cudaPeekAtLastError());
    MLP_CUDA(m->ctx, hg::launch_mlp_infer_tc(m, inputs, count, lobes, net));
    return HG_OK;
}

hg_status hg_mlp_gradients(hg_mlp* m, const float* inputs, const float* targets, uint32_t count, float* grad,
                           float* loss) {
    if (!m) return HG_INVALID_ARG;
    hg_ctx* ctx = m->ctx;
    if (count == 0 || !inputs || !targets || !grad) return fail(ctx, HG_INVALID_ARG, "empty batch or null buffer");
    MLP_CUDA(ctx, cudaPeekAtLastError());
    if (m->arch == HG_MLP_ARCH_DEEP) MLP_CUDA(ctx, hg::ensure_scratch(m, count));
    const size_t pf = sizeof(float) * m->n_params;
    MLP_CUDA(ctx, cudaMemsetAsync(m->grad, 0, pf, ctx->stream));
    MLP_CUDA(ctx, cudaMemsetAsync(m->loss, 0, sizeof(float), ctx->stream));
    MLP_CUDA(ctx, hg::run_gradients(m, inputs, targets, count));
    MLP_CUDA(ctx, cudaMemcpyAsync(grad, m->grad, pf, cudaMemcpyDeviceToHost, ctx->stream));
    float l = 0.0f;
    MLP_CUDA(ctx, cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    MLP_CUDA(ctx, cudaMemsetAsync(m->grad, 0, pf, ctx->stream));
    MLP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (loss) *loss = l;
    return HG_OK;
}

hg_status hg_mlp_train_step(hg_mlp* m, const float* inputs, const float* targets, uint32_t count, float lr,
                            float* loss_sum) {
    if (!m) return HG_INVALID_ARG;
    hg_ctx* ctx = m->ctx;
    if (count == 0 || !inputs || !targets) return fail(ctx, HG_INVALID_ARG, "empty batch or null buffer");
    if (!(lr >= 0.0f) || !std::isfinite(lr)) return fail(ctx, HG_INVALID_ARG, "learning rate must be finite, >= 0");
    MLP_CUDA(ctx, cudaPeekAtLastError());
    if (m->arch == HG_MLP_ARCH_DEEP) MLP_CUDA(ctx, hg::ensure_scratch(m, count));
    MLP_CUDA(ctx, hg::run_gradients(m, inputs, targets, count));
    m->step += 1;
    const double b1t = 1.0 - std::pow(0.9, (double)m->step), b2t = 1.0 - std::pow(0.999, (double)m->step);
    const float lr_t = (float)(lr * std::sqrt(b2t) / b1t);
    const float eps_t = (float)(1e-8 * std::sqrt(b2t));
    MLP_CUDA(ctx, hg::convert(m, 1, lr_t, eps_t, 1.0f / ((float)count * (float)hg_mlp_output_count(m))));
    if (loss_sum) {
        MLP_CUDA(ctx, cudaMemcpyAsync(loss_sum, m->loss, sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    MLP_CUDA(ctx, cudaMemsetAsync(m->loss, 0, sizeof(float), ctx->stream));
    return HG_OK;
}

hg_status hg_karis_lobes(hg_ctx* ctx, const float* inputs, uint32_t count, float tilt, float* lobes) {
    if (!ctx) return HG_INVALID_ARG;
    if (count == 0) return HG_OK;
    if (!inputs || !lobes) return fail(ctx, HG_INVALID_ARG, "null buffer");
    if (!std::isfinite(tilt)) return fail(ctx, HG_INVALID_ARG, "non-finite tilt");
    cudaSetDevice(ctx->device);
    MLP_CUDA(ctx, cudaPeekAtLastError());
    MLP_CUDA(ctx, hg::launch_karis_lobes(ctx, inputs, count, tilt, lobes));
    return HG_OK;
}

hg_status hg_mlp_bind(hg_ctx* ctx, hg_mlp* m) {
    if (!ctx) return HG_INVALID_ARG;
    if (m && m->ctx != ctx) return fail(ctx, HG_INVALID_ARG, "surrogate belongs to another context");
    ctx->surrogate = m;
    return HG_OK;
}

}  // extern "C"
