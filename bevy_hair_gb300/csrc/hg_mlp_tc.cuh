// The shading surrogate's network on the 5th-generation tensor cores
// (tcgen05): 128 rows per MMA (M = 128), accumulators in tensor memory,
// operands in shared memory.  Same network and numerics as hg_mlp.cuh
// (FP16 weights and activations, FP32 accumulation), with the biases folded
// into the products: every layer's input carries two constant-1 columns whose
// weights are the FP16 high and low parts of the bias, which keeps the bias
// to ~2^-22 relative.
//
// A "chain" is one warpgroup (4 warps, 128 threads; thread r owns row r) that
// runs two evaluations at once, each with its own input tile X (128 x 16),
// hidden tile H (128 x 80), 64 TMEM columns and mbarrier.  Per layer one
// thread issues an evaluation's MMAs and commits them to its mbarrier; all
// 128 threads wait (bounded), read their row of the accumulator with
// tcgen05.ld, apply ReLU + FP16 conversion and write it as the next layer's
// input row.  While the warps work on one evaluation's accumulator the
// tensor core runs the other's layer.  A CTA holds four chains (512
// threads), all of the SM's 512 TMEM columns and 227 KB of shared memory.
//
// Shared-memory operand layout (K-major, no swizzle): 8 x 16-byte core
// matrices; element (row, k) at (row/8)*SBO + (k/8)*LBO + (row%8)*16 + (k%8)*2
// with LBO = 128 (core matrices adjacent along K are contiguous) and
// SBO = (K/8)*128.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "hg_mlp.cuh"

namespace hg {
namespace mlp {
namespace tc {

constexpr uint32_t kM = 128;
constexpr uint32_t kKin = 16;   // 10 inputs, 2 bias columns, 4 zeros
constexpr uint32_t kKhid = 80;  // 64 activations, 2 bias columns, 14 zeros
constexpr uint32_t kLbo = 128;
constexpr uint32_t kSboIn = (kKin / 8) * 128, kSboHid = (kKhid / 8) * 128;
// Shared-memory byte offsets of one CTA (two chains).
constexpr uint32_t kOffW1 = 0;
constexpr uint32_t kOffW2 = kOffW1 + kHid * kKin * 2;
constexpr uint32_t kOffW3 = kOffW2 + kHid * kKhid * 2;
constexpr uint32_t kOffW4 = kOffW3 + kHid * kKhid * 2;
constexpr uint32_t kOffW5 = kOffW4 + kHid * kKhid * 2;
constexpr uint32_t kWeightBytes = kOffW5 + kOut * kKhid * 2;  // 35,328
constexpr uint32_t kXBytes = kM * kKin * 2, kHBytes = kM * kKhid * 2;
constexpr uint32_t kEvals = 2;    // evaluations in flight per chain
constexpr uint32_t kChains = 4;   // warpgroups per CTA
constexpr uint32_t kEvalBytes = kXBytes + kHBytes;
constexpr uint32_t kGroupBytes = kEvals * kEvalBytes;
constexpr uint32_t kOffBar = kWeightBytes + kChains * kGroupBytes;  // kChains * kEvals mbarriers, then the TMEM address
constexpr uint32_t kOffSlot = kOffBar + 8 * kChains * kEvals;
constexpr uint32_t kSmemBytes = kOffSlot + 16;
constexpr uint32_t kTmemCols = 512;  // per chain 128: per evaluation 64 (hidden accumulator; the output reuses 0..15)
constexpr uint32_t kThreads = 128 * kChains;
static_assert(kSmemBytes <= 232448, "shared memory per CTA");
static_assert(kWeightBytes % 128 == 0 && kGroupBytes % 128 == 0, "tile alignment");
// Instruction descriptors (kind::f16): D F32, A and B F16, both K-major, M = 128.
constexpr uint32_t kIdescHid = (1u << 4) | ((64u >> 3) << 17) | ((kM >> 4) << 24);
constexpr uint32_t kIdescOut = (1u << 4) | ((16u >> 3) << 17) | ((kM >> 4) << 24);
// Bounded waits: iterations of mbarrier.try_wait before a chain gives up.
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr uint32_t kErrTimeout = 2u;

__device__ __forceinline__ uint32_t canon(uint32_t row, uint32_t k, uint32_t sbo) {
    return (row >> 3) * sbo + (k >> 3) * kLbo + (row & 7u) * 16u + (k & 7u) * 2u;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start, LBO, SBO (all >> 4), version 1,
// base offset 0, no swizzle.
__device__ __forceinline__ uint64_t desc(uint32_t saddr, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(kLbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ void tmem_alloc(uint32_t slot_saddr, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(slot_saddr), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void commit(uint32_t mbar_saddr) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar_saddr)
                 : "memory");
}
__device__ __forceinline__ void mbar_init(uint32_t mbar_saddr, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar_saddr), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }

// Wait for phase `parity` of the mbarrier, at most kWaitLimit polls.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar_saddr, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar_saddr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Barrier over one warpgroup (named barrier `id`, 128 threads) that returns
// the OR of `pred` over its threads.
__device__ __forceinline__ bool group_sync_or(uint32_t id, bool pred) {
    uint32_t r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.or.pred p, %2, 128, q;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)pred), "r"(id)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t v[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t v[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

__device__ __forceinline__ void st_shared_v4(uint32_t saddr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(saddr), "r"(a), "r"(b), "r"(c), "r"(d)
                 : "memory");
}

__device__ __forceinline__ void store_half(uint8_t* smem, uint32_t off, __half v) {
    *reinterpret_cast<__half*>(smem + off) = v;
}

// The weight tiles of the CTA (every thread takes part): W[n][k] in the
// canonical layout, the two bias columns after the real inputs.
__device__ __forceinline__ void load_weights(uint8_t* smem, const __half* __restrict__ w16,
                                             const float* __restrict__ params, int tid, int nthreads) {
    auto bias_parts = [](float b, __half& hi, __half& lo) {
        hi = __float2half_rn(b);
        lo = __float2half_rn(b - __half2float(hi));
    };
    for (int i = tid; i < (int)(kHid * kKin); i += nthreads) {
        const uint32_t n = i / kKin, k = i % kKin;
        __half v = __float2half_rn(0.0f);
        if (k < (uint32_t)kUsedIn) {
            v = w16[kW1 + n * kIn + k];
        } else if (k == (uint32_t)kUsedIn || k == (uint32_t)kUsedIn + 1) {
            __half hi, lo;
            bias_parts(params[kB1 + n], hi, lo);
            v = k == (uint32_t)kUsedIn ? hi : lo;
        }
        store_half(smem, kOffW1 + canon(n, k, kSboIn), v);
    }
    const int woff[3] = {kW2, kW3, kW4}, boff[3] = {kB2, kB3, kB4};
    const uint32_t soff[3] = {kOffW2, kOffW3, kOffW4};
    for (int l = 0; l < 3; ++l)
        for (int i = tid; i < (int)(kHid * kKhid); i += nthreads) {
            const uint32_t n = i / kKhid, k = i % kKhid;
            __half v = __float2half_rn(0.0f);
            if (k < (uint32_t)kHid) {
                v = w16[woff[l] + n * kHid + k];
            } else if (k == (uint32_t)kHid || k == (uint32_t)kHid + 1) {
                __half hi, lo;
                bias_parts(params[boff[l] + n], hi, lo);
                v = k == (uint32_t)kHid ? hi : lo;
            }
            store_half(smem, soff[l] + canon(n, k, kSboHid), v);
        }
    for (int i = tid; i < (int)(kOut * kKhid); i += nthreads) {
        const uint32_t n = i / kKhid, k = i % kKhid;
        __half v = __float2half_rn(0.0f);
        if (k < (uint32_t)kHid) {
            v = w16[kW5 + n * kHid + k];
        } else if (k == (uint32_t)kHid || k == (uint32_t)kHid + 1) {
            __half hi, lo;
            bias_parts(params[kB5 + n], hi, lo);
            v = k == (uint32_t)kHid ? hi : lo;
        }
        store_half(smem, kOffW5 + canon(n, k, kSboHid), v);
    }
}

struct Chain {
    uint32_t w;              // shared address of the weights
    uint32_t x[kEvals];      // shared addresses of the input tiles
    uint32_t h[kEvals];      // and of the hidden tiles
    uint32_t mbar[kEvals];   // shared addresses of the mbarriers
    uint32_t tmem[kEvals];   // TMEM addresses of the accumulators (lane 0)
    uint32_t phase[kEvals];  // parity of each mbarrier's next phase
    uint32_t bar_id;         // named barrier of the warpgroup
    uint32_t row;            // this thread's row, 0..127
};

// Row r of an H tile: the constant columns 64..79 (1, 1, then zeros), written once.
__device__ __forceinline__ void init_hidden_row(uint32_t h, uint32_t row) {
    const uint32_t one2 = 0x3C003C00u;  // two FP16 ones
    st_shared_v4(h + canon(row, 64, kSboHid), one2, 0u, 0u, 0u);
    st_shared_v4(h + canon(row, 72, kSboHid), 0u, 0u, 0u, 0u);
}

// Row r of evaluation e's X from the normalised inputs (columns 10, 11 are the bias ones).
__device__ __forceinline__ void write_input_row(const Chain& c, uint32_t e, const float x[kUsedIn]) {
    st_shared_v4(c.x[e] + canon(c.row, 0, kSboIn), pack_h2(x[0], x[1]), pack_h2(x[2], x[3]), pack_h2(x[4], x[5]),
                 pack_h2(x[6], x[7]));
    st_shared_v4(c.x[e] + canon(c.row, 8, kSboIn), pack_h2(x[8], x[9]), 0x3C003C00u, 0u, 0u);
}

__device__ __forceinline__ void issue(uint32_t d, uint32_t a, uint32_t a_sbo, uint32_t b, uint32_t b_sbo,
                                      uint32_t ksteps, uint32_t idesc) {
    for (uint32_t ks = 0; ks < ksteps; ++ks)
        mma(d, desc(a + ks * 2u * kLbo, a_sbo), desc(b + ks * 2u * kLbo, b_sbo), idesc, ks);
}

// Epilogue of one hidden layer of evaluation e: accumulator -> ReLU -> FP16 -> H row.
__device__ __forceinline__ void hidden_epilogue(const Chain& c, uint32_t e) {
    const uint32_t lane_base = (c.row & ~31u) << 16;
    uint32_t v[64];
    tmem_ld32(c.tmem[e] + lane_base, v);
    tmem_ld32(c.tmem[e] + lane_base + 32u, v + 32);
    tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 8; ++j)
        st_shared_v4(c.h[e] + canon(c.row, 8u * j, kSboHid),
                     pack_relu(__uint_as_float(v[8 * j]), __uint_as_float(v[8 * j + 1])),
                     pack_relu(__uint_as_float(v[8 * j + 2]), __uint_as_float(v[8 * j + 3])),
                     pack_relu(__uint_as_float(v[8 * j + 4]), __uint_as_float(v[8 * j + 5])),
                     pack_relu(__uint_as_float(v[8 * j + 6]), __uint_as_float(v[8 * j + 7])));
}

// The evaluations whose inputs are in X[0] (and X[1] when `two`): y0 / y1
// receive this thread's 12 network outputs of each.  Every thread of the
// warpgroup calls it with the same `two`.  Returns false (for the whole
// warpgroup) when an MMA did not complete in time; the chain is then
// unusable.
__device__ __forceinline__ bool forward2(Chain& c, bool two, float y0[kUsedOut], float y1[kUsedOut]) {
    const uint32_t ne = two ? 2u : 1u;
    fence_proxy_async();
    if (group_sync_or(c.bar_id, false)) return false;
    if (c.row == 0) {
        fence_after();
        for (uint32_t e = 0; e < ne; ++e) {
            issue(c.tmem[e], c.x[e], kSboIn, c.w + kOffW1, kSboIn, kKin / 16, kIdescHid);
            commit(c.mbar[e]);
        }
    }
    const uint32_t next_w[4] = {kOffW2, kOffW3, kOffW4, kOffW5};
    for (int layer = 0; layer < 4; ++layer) {
        for (uint32_t e = 0; e < ne; ++e) {
            const bool ok = mbar_wait(c.mbar[e], c.phase[e]);
            if (ok) c.phase[e] ^= 1u;  // after a timeout the phase stays the outstanding one
            fence_after();
            hidden_epilogue(c, e);
            fence_proxy_async();
            fence_before();
            if (group_sync_or(c.bar_id, !ok)) return false;
            if (c.row == 0) {
                fence_after();
                if (layer < 3)
                    issue(c.tmem[e], c.h[e], kSboHid, c.w + next_w[layer], kSboHid, kKhid / 16, kIdescHid);
                else
                    issue(c.tmem[e], c.h[e], kSboHid, c.w + next_w[layer], kSboHid, kKhid / 16, kIdescOut);
                commit(c.mbar[e]);
            }
        }
    }
    const uint32_t lane_base = (c.row & ~31u) << 16;
    bool ok_all = true;
    for (uint32_t e = 0; e < ne; ++e) {
        const bool ok = mbar_wait(c.mbar[e], c.phase[e]);
        if (ok) c.phase[e] ^= 1u;
        ok_all = ok_all && ok;
        fence_after();
        uint32_t o[16];
        tmem_ld16(c.tmem[e] + lane_base, o);
        tmem_wait_ld();
        float* y = e == 0 ? y0 : y1;
#pragma unroll
        for (int i = 0; i < kUsedOut; ++i) y[i] = __uint_as_float(o[i]);
    }
    fence_before();
    return !group_sync_or(c.bar_id, !ok_all);
}

// CTA set-up: weights, the constant columns of every H tile, mbarriers, TMEM.
// Every thread calls it; returns this thread's chain.
__device__ __forceinline__ Chain setup(uint8_t* smem, const __half* w16, const float* params) {
    const uint32_t tid = threadIdx.x, g = tid >> 7;
    const uint32_t base = smem_addr(smem);
    Chain c;
    c.w = base;
    c.bar_id = 1u + g;
    c.row = tid & 127u;
    for (uint32_t e = 0; e < kEvals; ++e) {
        c.x[e] = base + kWeightBytes + g * kGroupBytes + e * kEvalBytes;
        c.h[e] = c.x[e] + kXBytes;
        c.mbar[e] = base + kOffBar + 8u * (g * kEvals + e);
        c.phase[e] = 0;
        init_hidden_row(c.h[e], c.row);
    }
    load_weights(smem, w16, params, (int)tid, (int)blockDim.x);
    if (tid == 0) {
        for (uint32_t k = 0; k < kChains * kEvals; ++k) mbar_init(base + kOffBar + 8u * k, 1);
        fence_mbar_init();
    }
    if (tid < 32) {
        tmem_alloc(base + kOffSlot, kTmemCols);
        tmem_relinquish();
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tbase = *reinterpret_cast<volatile uint32_t*>(smem + kOffSlot);
    for (uint32_t e = 0; e < kEvals; ++e) c.tmem[e] = tbase + g * 128u + e * 64u;
    return c;
}

// CTA tear-down after every chain has finished (or given up): bounded waits
// for a failed chain's outstanding commits, then the TMEM is freed.
__device__ __forceinline__ void teardown(uint8_t* smem, Chain& c, bool failed) {
    if (failed)
        for (uint32_t e = 0; e < kEvals; ++e) (void)mbar_wait(c.mbar[e], c.phase[e]);
    fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        fence_after();
        tmem_dealloc(*reinterpret_cast<volatile uint32_t*>(smem + kOffSlot), kTmemCols);
    }
}

}  // namespace tc
}  // namespace mlp
}  // namespace hg
