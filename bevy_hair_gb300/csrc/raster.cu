// Visibility passes: clear, clear_dom, lod, scan and raster (camera G-buffer
// and deep-opacity map).  Everything here feeds the integer visibility
// outputs, so this file is compiled with -fmad=false and follows the float
// semantics of hg_device.cuh.
//
// Reference passes: clear.wgsl, clear_dom.wgsl, lod.wgsl, scan.wgsl,
// raster.wgsl (src/render/shaders/).
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "hg_device.cuh"
#include "hg_internal.h"

namespace hg {
namespace {

// ------------------------------------------------------------------ clear

// clear.wgsl:7-16.  Four pixels per thread with 16-byte stores.
__global__ void clear_kernel(unsigned long long* __restrict__ center, unsigned long long* __restrict__ cons,
                             uint32_t* __restrict__ beta, size_t pixels) {
    size_t quads = pixels / 4;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    const ulonglong2 e2 = make_ulonglong2(kEmptyU64, kEmptyU64);
    const uint4 e4 = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < quads; q += stride) {
        reinterpret_cast<ulonglong2*>(center)[2 * q] = e2;
        reinterpret_cast<ulonglong2*>(center)[2 * q + 1] = e2;
        reinterpret_cast<ulonglong2*>(cons)[2 * q] = e2;
        reinterpret_cast<ulonglong2*>(cons)[2 * q + 1] = e2;
        reinterpret_cast<uint4*>(beta)[q] = e4;
    }
    size_t tail = quads * 4 + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tail < pixels) {
        center[tail] = kEmptyU64;
        cons[tail] = kEmptyU64;
        beta[tail] = 0xffffffffu;
    }
}

// clear_dom.wgsl:8-21: words below `texels` are front depths, the rest counters.
__global__ void clear_dom_kernel(uint32_t* __restrict__ dom, size_t texels, size_t words) {
    size_t quads = words / 4;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < quads; q += stride) {
        size_t w = q * 4;
        uint4 v;
        v.x = w + 0 < texels ? kDomEmpty : 0u;
        v.y = w + 1 < texels ? kDomEmpty : 0u;
        v.z = w + 2 < texels ? kDomEmpty : 0u;
        v.w = w + 3 < texels ? kDomEmpty : 0u;
        reinterpret_cast<uint4*>(dom)[q] = v;
    }
    size_t tail = quads * 4 + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tail < words) dom[tail] = tail < texels ? kDomEmpty : 0u;
}

// ------------------------------------------------------------------ lod

__device__ __forceinline__ f3 to_world(const hg_hair_params& p, f3 q) {
    float4 r = mat_mul(p.world_from_model, q.x, q.y, q.z, 1.0f);
    return {r.x, r.y, r.z};
}
__device__ __forceinline__ f3 dir_world(const hg_hair_params& p, f3 d) {
    float4 r = mat_mul(p.world_from_model, d.x, d.y, d.z, 0.0f);
    return safe_normalize({r.x, r.y, r.z});
}

// control_points_for_lod (common.wgsl:231-238); the power-of-two snap is
// evaluated exactly from the highest set bit of c - 1.
__device__ __forceinline__ uint32_t control_points_for_lod(float l) {
    float c_raw = fmaxf(floorf(__fsqrt_rn(clampf(l, 0.0f, 1.0f)) * 127.0f), (float)kLayerCount);
    if (c_raw < 3.0f) return f2u(fmaxf(c_raw, 2.0f));
    uint32_t c1 = f2u(c_raw - 1.0f);
    uint32_t snapped = (1u << (31 - __clz(c1))) + 1u;
    return snapped < 127u ? snapped : 127u;
}

constexpr uint32_t kDepthBuckets = 1024;

// lod.wgsl:6-59, one warp per bundle (two of the 64 cage corners per lane).
// Also writes the bundle's nearest view distance as one of kDepthBuckets
// buckets between near and far, for the front-to-back draw order.
__device__ __forceinline__ void lod_bundle(const hg_hair_params& p, const hg_gpu_bundle* __restrict__ bundles,
                                           const float4* __restrict__ layers, hg_lod_record* __restrict__ out,
                                           uint32_t* __restrict__ depth_key, uint32_t b, uint32_t lane) {
    hg_gpu_bundle bundle = bundles[b];
    float mnx = 1e20f, mny = 1e20f, mxx = -1e20f, mxy = -1e20f, mnd = 3.0e38f;
    bool front = false;
    for (uint32_t c = lane; c < 64u; c += 32u) {
        float4 pa = __ldg(&layers[2u * (bundle.layer_offset + c)]);
        f3 world = to_world(p, xyz(pa));
        float4 clip = mat_mul(p.clip_from_world, world.x, world.y, world.z, 1.0f);
        float dist = dot3(sub3(world, mk3(p.camera_pos[0], p.camera_pos[1], p.camera_pos[2])),
                          mk3(p.camera_forward[0], p.camera_forward[1], p.camera_forward[2]));
        if (clip.w > 0.0f && dist > 0.0f) front = true;
        mnd = fminf(mnd, dist);
        Projected pr = project_world(p, world);
        mnx = fminf(mnx, pr.screen.x);
        mny = fminf(mny, pr.screen.y);
        mxx = fmaxf(mxx, pr.screen.x);
        mxy = fmaxf(mxy, pr.screen.y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
        mnd = fminf(mnd, __shfl_xor_sync(0xffffffffu, mnd, o));
    }
    bool any_front = __any_sync(0xffffffffu, front);
    if (lane != 0) return;
    const float rel = (mnd - p.screen[2]) / fmaxf(p.screen[3] - p.screen[2], 1e-3f);
    depth_key[b] = min(f2u(clampf(rel, 0.0f, 1.0f) * (float)kDepthBuckets), kDepthBuckets - 1u);
    bool culled = !any_front || mxx < 0.0f || mxy < 0.0f || mnx > p.screen[0] || mny > p.screen[1];
    uint32_t n_lod = 0u, cps = kLayerCount;
    if (!culled) {
        if (p.pass_mode[3] == 1u) {
            n_lod = bundle.strand_count;
            cps = control_points_for_lod(1.0f);
        } else if (p.flags[0] == 0u) {
            n_lod = bundle.strand_count;
            cps = 127u;
        } else {
            float2 d = make_float2(mxx - mnx, mxy - mny);
            float diag = len2(d);
            float l = clampf(__fdiv_rn(diag, fmaxf(p.screen[1], 1.0f)) * p.appearance[2], 0.0f, 1.0f);
            float delta = __uint2float_rn(pcg(b ^ 0x9e3779b9u)) * (1.0f / 4294967296.0f);
            float n = __uint2float_rn(bundle.strand_count);
            float raw = ceilf(l * (n + delta));
            n_lod = f2u(clampf(raw, 1.0f, n));
            cps = control_points_for_lod(l);
        }
    }
    out[b] = hg_lod_record{n_lod, cps, bundle.strand_count, 0u};
}

__global__ void lod_kernel(const hg_hair_params p, const hg_gpu_bundle* __restrict__ bundles,
                           const float4* __restrict__ layers, hg_lod_record* __restrict__ out,
                           uint32_t* __restrict__ depth_key, uint32_t count) {
    uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t lane = threadIdx.x & 31u;
    if (b >= count) return;
    lod_bundle(p, bundles, layers, out, depth_key, b, lane);
}

// ------------------------------------------------------------------ scan

// scan.wgsl:6-24 in two parallel steps.  Step 1 (one CTA): exclusive scan of
// n_lod into offsets and the indirect arguments (total, 1, 1) with the total
// clamped to the refs capacity.
constexpr int kScanThreads = 1024;
constexpr uint32_t kScanItems = 16;  // bundles per thread per scan pass

// Block-wide exclusive scan of one value per thread; returns the thread's
// exclusive prefix and, through *total, the block's sum.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane];
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= (uint32_t)o) wi += y;
        }
        warp_sums[lane] = wi - w;
        if (lane == 31) warp_sums[32] = wi;
    }
    __syncthreads();
    const uint32_t r = warp_sums[warp] + incl - v;
    *total = warp_sums[32];
    __syncthreads();
    return r;
}

// One pass of a block-wide exclusive scan over elements [base, base + 1024 *
// kScanItems) of n: warp w takes the 32 * kScanItems elements from base +
// 32 * kScanItems * w, lane-interleaved so loads and stores coalesce; all its
// loads are issued before the first shuffle.  store(i, carry + exclusive
// prefix) for every i < n in the pass; returns the pass total.
template <class Load, class Store>
__device__ __forceinline__ uint32_t scan_pass(uint32_t base, uint32_t n, uint32_t carry, uint32_t* warp_sums,
                                              Load load, Store store) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t wbase = base + warp * 32u * kScanItems;
    uint32_t v[kScanItems];
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
        const uint32_t i = wbase + k * 32u + lane;
        v[k] = i < n ? load(i) : 0u;
    }
    uint32_t pre[kScanItems];
    uint32_t wrun = 0;
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
        uint32_t incl = v[k];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        pre[k] = wrun + incl - v[k];
        wrun += __shfl_sync(0xffffffffu, incl, 31);
    }
    uint32_t total = 0;
    const uint32_t woff = block_exclusive_scan(lane == 31u ? wrun : 0u, warp_sums, &total);
#pragma unroll
    for (uint32_t k = 0; k < kScanItems; ++k) {
        const uint32_t i = wbase + k * 32u + lane;
        if (i < n) store(i, carry + woff + pre[k]);
    }
    return total;
}

__device__ __forceinline__ void scan_offsets_block(const hg_lod_record* __restrict__ lod, uint32_t count,
                                                   uint32_t capacity, uint32_t* __restrict__ offsets,
                                                   uint32_t* __restrict__ indirect,
                                                   const uint32_t* __restrict__ depth_key,
                                                   uint32_t* __restrict__ sorted, uint32_t* __restrict__ sorted_off,
                                                   uint32_t* __restrict__ order_meta) {
    __shared__ uint32_t warp_sums[33];
    __shared__ uint32_t bucket[kDepthBuckets];
    uint32_t carry = 0;
    for (uint32_t base = 0; base < count; base += kScanThreads * kScanItems)
        carry += scan_pass(
            base, count, carry, warp_sums, [&](uint32_t i) { return lod[i].n_lod; },
            [&](uint32_t i, uint32_t at) { offsets[i] = at; });
    if (threadIdx.x == 0) {
        uint32_t total = carry < capacity ? carry : capacity;
        offsets[count] = carry;
        indirect[0] = total;
        indirect[1] = 1u;
        indirect[2] = 1u;
        indirect[3] = 0u;
    }
    if (!sorted) return;
    // Draw order: live bundles (n_lod > 0) counting-sorted by depth bucket,
    // then their n_lod scanned in that order.  The raster visits strands in
    // this order (near bundles first) so most later samples fail the depth
    // test before any payload work; results do not depend on the order.
    const uint32_t full = carry;
    for (uint32_t k = threadIdx.x; k < kDepthBuckets; k += kScanThreads) bucket[k] = 0u;
    __syncthreads();
    // keys of live bundles, loaded a pass at a time before the shared atomics
    for (uint32_t base = 0; base < count; base += kScanThreads * kScanItems) {
        uint32_t key[kScanItems];
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            const uint32_t b = base + k * kScanThreads + threadIdx.x;
            key[k] = b < count && lod[b].n_lod ? depth_key[b] : kDepthBuckets;
        }
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k)
            if (key[k] < kDepthBuckets) atomicAdd(&bucket[key[k]], 1u);
    }
    __syncthreads();
    uint32_t live = 0;
    const uint32_t start = block_exclusive_scan(threadIdx.x < kDepthBuckets ? bucket[threadIdx.x] : 0u, warp_sums,
                                                &live);
    if (threadIdx.x < kDepthBuckets) bucket[threadIdx.x] = start;
    __syncthreads();
    for (uint32_t base = 0; base < count; base += kScanThreads * kScanItems) {
        uint32_t key[kScanItems];
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k) {
            const uint32_t b = base + k * kScanThreads + threadIdx.x;
            key[k] = b < count && lod[b].n_lod ? depth_key[b] : kDepthBuckets;
        }
#pragma unroll
        for (uint32_t k = 0; k < kScanItems; ++k)
            if (key[k] < kDepthBuckets) sorted[atomicAdd(&bucket[key[k]], 1u)] = base + k * kScanThreads + threadIdx.x;
    }
    __syncthreads();
    uint32_t run = 0;
    for (uint32_t base = 0; base < live; base += kScanThreads * kScanItems)
        run += scan_pass(
            base, live, run, warp_sums, [&](uint32_t i) { return lod[sorted[i]].n_lod; },
            [&](uint32_t i, uint32_t at) { sorted_off[i] = at; });
    if (threadIdx.x == 0) {
        sorted_off[live] = run;
        order_meta[0] = live;
        order_meta[1] = full <= capacity ? 1u : 0u;  // every ref exists, so the order is a permutation
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_offsets_kernel(const hg_lod_record* __restrict__ lod,
                                                                    uint32_t count, uint32_t capacity,
                                                                    uint32_t* __restrict__ offsets,
                                                                    uint32_t* __restrict__ indirect,
                                                                    const uint32_t* __restrict__ depth_key,
                                                                    uint32_t* __restrict__ sorted,
                                                                    uint32_t* __restrict__ sorted_off,
                                                                    uint32_t* __restrict__ order_meta) {
    scan_offsets_block(lod, count, capacity, offsets, indirect, depth_key, sorted, sorted_off, order_meta);
}

// Step 2: one warp per bundle writes its StrandRefs (bundle-major order, as
// the serial loop does); entries at or past the capacity are dropped.
__global__ void scan_expand_kernel(const hg_lod_record* __restrict__ lod, const uint32_t* __restrict__ offsets,
                                   uint32_t count, uint32_t capacity, hg_strand_ref* __restrict__ refs) {
    uint32_t lane = threadIdx.x & 31u;
    uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < count; b += warps) {
        hg_lod_record rec = lod[b];
        uint32_t off = offsets[b];
        for (uint32_t s = lane; s < rec.n_lod; s += 32u) {
            uint32_t i = off + s;
            if (i >= capacity) break;
            reinterpret_cast<uint4*>(refs)[i] = make_uint4(b, s, rec.n_lod, rec.control_points);
        }
    }
}

// Step 2 with a draw order: one warp per live bundle in depth order writes
// its StrandRefs at their reference positions and the matching draw-order
// entries (indices into refs).
__global__ void scan_expand_sorted_kernel(const hg_lod_record* __restrict__ lod, const uint32_t* __restrict__ offsets,
                                          const uint32_t* __restrict__ sorted, const uint32_t* __restrict__ sorted_off,
                                          const uint32_t* __restrict__ order_meta, uint32_t capacity,
                                          hg_strand_ref* __restrict__ refs, uint32_t* __restrict__ draw_order) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t live = order_meta[0];
    const bool valid = order_meta[1] != 0u;
    for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < live; k += warps) {
        const uint32_t b = sorted[k];
        const hg_lod_record rec = lod[b];
        const uint32_t off = offsets[b], dpos = sorted_off[k];
        for (uint32_t s = lane; s < rec.n_lod; s += 32u) {
            const uint32_t i = off + s;
            if (i >= capacity) break;
            reinterpret_cast<uint4*>(refs)[i] = make_uint4(b, s, rec.n_lod, rec.control_points);
            if (valid) draw_order[dpos + s] = i;
        }
    }
}

// ------------------------------------------------------------------ raster

constexpr int kRasterWarps = 4;
constexpr int kRasterThreads = kRasterWarps * 32;
// Resident blocks per SM.  The camera pass keeps its sample loop in 80
// registers without a spill in it at 6 (24 warps); at 7 (72 registers) the
// spilled values sit in the loop and reach L2 on every round (L1 is small
// next to 7 x 28 KB of shared memory), which costs more than the extra warps
// give.  The deep-opacity passes fit 60 registers and take 7 (shared memory
// allows no eighth).
template <int MODE>
constexpr int raster_min_blocks() { return MODE == 0 ? 6 : 7; }
// The deep-opacity rasters launch this many rounds of resident blocks, each
// warp striding over a few refs: blocks that finish early are replaced by
// fresh ones, which evens out the end of the pass (one round, every warp
// walking 24-48 refs, left a long tail: DOM depth 0.156 -> 0.148 ms on
// config 2, 0.473 -> 0.426 ms on config 3).  The camera stages keep one
// round (two measured 0.356 -> 0.364 ms).
constexpr int kDomGridRounds = 8;

// Per-warp shared memory, 7 KB.  The layer samples are needed only while
// control points are generated, so they share storage with the run list.
struct alignas(16) StrandSmem {
    float4 cp[128];  // control point: model position, then world position + in_front flag
    float4 ct[128];  // camera: world tangent xyz + w (uvw.z)
    float4 cs[128];  // screen xy, ao; camera: RN(1/n) for the segment's DDA step count n
    float vd[128];   // camera: view distance of the control point (project_world)
    hg_strand_ref next_ref;  // the warp's next ref, copied ahead (cp.async)
    uint32_t next_idx;       // the draw-order entry after it
    uint32_t pad_[3];
    uint32_t finm[4];        // camera: bit l of word k set when control point 32 k + l is finite
    union {
        struct {
            float4 lp[16];  // layer sample: position, ao
            float4 lt[16];  // layer tangent
            float4 ls[16];  // style residual of each w layer at the strand's (u, v)
        } gen;
        struct {
            int32_t off[128];  // camera: first sample of each non-empty segment, in order
            int32_t seg[128];  // camera: that segment's index | its DDA step count n << 8
        } run;
    } u;
};

// Segments are cut into at most this many DDA steps.
constexpr int kMaxSteps = 96;

// t = i / n, correctly rounded, for integers 0 <= i <= n <= kMaxSteps, from
// rcp = RN(1/n): q0 = RN(i * rcp), the exact remainder i - q0 * n by FMA, and
// one correction step q0 + rem * rcp (Markstein's refinement).  An exhaustive
// check over all (i, n) in that range against the exact quotient rounded to
// nearest finds no difference, so this equals __fdiv_rn(i, n) there.
__device__ __forceinline__ float step_t(int32_t i, int32_t n, float rcp) {
    const float fi = __int2float_rn(i), fn = __int2float_rn(n);
    const float q0 = __fmul_rn(fi, rcp);
    const float rem = __fmaf_rn(-q0, fn, fi);
    return __fmaf_rn(rem, rcp, q0);
}

struct RasterArgs {
    hg_hair_params p;
    const hg_gpu_bundle* bundles;
    const float4* layers;
    const float4* style;
    const hg_strand_ref* refs;
    const uint32_t* indirect;
    const uint32_t* draw_order;  // permutation of refs to visit, or nullptr
    const uint32_t* order_meta;  // (live bundles, order valid)
    const uint32_t* full_order;  // DOM depth pass: permutation for a draw of every strand, or nullptr
    uint32_t full_total;         // the ref count of such a draw
    const float4* cache;         // strand cache (kCacheCps positions then tangents per strand), or nullptr
    const uint32_t* strand_base; // first strand of each bundle in the cache
    unsigned long long* center;
    unsigned long long* cons;
    uint32_t* beta;
    uint32_t* dom;
    const float* scene;
    uint32_t* err;
    uint32_t bundle_count;
    // Camera pass: the refs (in draw order) this launch covers, in 1/256ths
    // of the ref count, and the tile depths built from the refs before them
    // (nullptr: no tile test).
    uint32_t part_lo, part_hi;
    const uint32_t* tile_depth;
    uint32_t tiles_x;
};

// sample_style (raster.wgsl:34-60), the trilinear style residual, is
// mix3(B(w0), B(w1), tw) with B(l) = mix3(mix3(c(u0,v0,l), c(u1,v0,l), tu),
// mix3(c(u0,v1,l), c(u1,v1,l), tu), tv), the bilinear lookup at the strand's
// (u, v) in layer l.  (u, v) is the same for every control point of a strand,
// so lanes 16..31 (idle while lanes 0..15 sample the layer cage) compute B
// for one layer each, and style_at finishes each control point with the same
// operations in the same order.
__device__ __forceinline__ void style_layers(const float4* __restrict__ style, uint32_t offset, float2 uv,
                                             float4* ls, uint32_t lane) {
    static_assert(kStyleW == 16, "one style layer per lane of the upper half-warp");
    if (lane >= 16u) {
        const uint32_t layer = lane - 16u;
        float u = clampf(uv.x, 0.0f, 1.0f) * (float)(kStyleU - 1u);
        float v = clampf(uv.y, 0.0f, 1.0f) * (float)(kStyleV - 1u);
        uint32_t u0 = f2u(floorf(u)), v0 = f2u(floorf(v));
        uint32_t u1 = min(u0 + 1u, kStyleU - 1u), v1 = min(v0 + 1u, kStyleV - 1u);
        float tu = u - __uint2float_rn(u0), tv = v - __uint2float_rn(v0);
        auto at = [&](uint32_t iu, uint32_t iv) {
            return xyz(__ldg(&style[offset + (layer * kStyleV + iv) * kStyleU + iu]));
        };
        const f3 c0 = mix3(at(u0, v0), at(u1, v0), tu);
        const f3 c1 = mix3(at(u0, v1), at(u1, v1), tu);
        const f3 r = mix3(c0, c1, tv);
        ls[layer] = make_float4(r.x, r.y, r.z, 0.0f);
    }
}

__device__ __forceinline__ f3 style_at(const float4* ls, float w) {
    float ww = clampf(w, 0.0f, 1.0f) * (float)(kStyleW - 1u);
    uint32_t w0 = f2u(floorf(ww));
    uint32_t w1 = min(w0 + 1u, kStyleW - 1u);
    float tw = ww - __uint2float_rn(w0);
    return mix3(xyz(ls[w0]), xyz(ls[w1]), tw);
}

__device__ __forceinline__ f3 hermite(f3 p0, f3 p1, f3 m0, f3 m1, float t) {
    float t2 = t * t;
    float t3 = t2 * t;
    float h00 = (2.0f * t3 - 3.0f * t2) + 1.0f;
    float h10 = (t3 - 2.0f * t2) + t;
    float h01 = -2.0f * t3 + 3.0f * t2;
    float h11 = t3 - t2;
    return add3(add3(add3(mul3s(p0, h00), mul3s(m0, h10)), mul3s(p1, h01)), mul3s(m1, h11));
}

__device__ __forceinline__ float4 bilinear4(float4 c00, float4 c10, float4 c01, float4 c11, float2 uv) {
    float u = uv.x, v = uv.y;
    float w00 = (1.0f - u) * (1.0f - v), w10 = u * (1.0f - v), w01 = (1.0f - u) * v, w11 = u * v;
    float4 r;
    r.x = ((c00.x * w00 + c10.x * w10) + c01.x * w01) + c11.x * w11;
    r.y = ((c00.y * w00 + c10.y * w10) + c01.y * w01) + c11.y * w11;
    r.z = ((c00.z * w00 + c10.z * w10) + c01.z * w01) + c11.z * w11;
    r.w = ((c00.w * w00 + c10.w * w10) + c01.w * w01) + c11.w * w11;
    return r;
}

__device__ __forceinline__ float4 shfl_up4(float4 v, int d) {
    return make_float4(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d),
                       __shfl_up_sync(0xffffffffu, v.z, d), __shfl_up_sync(0xffffffffu, v.w, d));
}
__device__ __forceinline__ float4 shfl_down4(float4 v, int d) {
    return make_float4(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d),
                       __shfl_down_sync(0xffffffffu, v.z, d), __shfl_down_sync(0xffffffffu, v.w, d));
}

__device__ __forceinline__ f3 shfl_up3(f3 v) {
    return {__shfl_up_sync(0xffffffffu, v.x, 1), __shfl_up_sync(0xffffffffu, v.y, 1),
            __shfl_up_sync(0xffffffffu, v.z, 1)};
}
__device__ __forceinline__ f3 shfl_down3(f3 v) {
    return {__shfl_down_sync(0xffffffffu, v.x, 1), __shfl_down_sync(0xffffffffu, v.y, 1),
            __shfl_down_sync(0xffffffffu, v.z, 1)};
}
__device__ __forceinline__ f3 shfl_idx3(f3 v, int src) {
    return {__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src),
            __shfl_sync(0xffffffffu, v.z, src)};
}

// Control points cached per frame: control_points_for_lod(1.0), the count of
// every deep-opacity strand and of camera strands at full detail.
constexpr uint32_t kCacheCps = 65;

// Model-space control points of one strand (raster.wgsl:231-284): layer
// samples on lanes 0..15 (neighbours over shuffles) and their finite-difference
// tangents into lp/lt, then eval_cp for control point j on lane j % 32, slot
// j / 32.
__device__ __forceinline__ void model_cps(const float4* __restrict__ layers, const float4* __restrict__ style,
                                          float4* lp, float4* lt, float4* ls, const hg_gpu_bundle& bundle, float2 uv,
                                          uint32_t ncp, uint32_t lane, f3 mp[4], float wk[4], float aok[4]) {
    float4 loaded = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (lane < kLayerCount) {
        const float4* c = layers + 2u * (bundle.layer_offset + lane * 4u);
        loaded = bilinear4(__ldg(c), __ldg(c + 2), __ldg(c + 4), __ldg(c + 6), uv);
    }
    float4 prev_l = shfl_up4(loaded, 1);
    float4 next_l = shfl_down4(loaded, 1);
    if (lane < kLayerCount) {
        f3 curr = xyz(loaded);
        f3 prev = lane == 0u ? curr : xyz(prev_l);
        f3 next = lane + 1u >= kLayerCount ? curr : xyz(next_l);
        f3 t = calc_tangent(lane, kLayerCount, prev, curr, next);
        lp[lane] = loaded;
        lt[lane] = make_float4(t.x, t.y, t.z, 0.0f);
    }
    style_layers(style, bundle.style_offset, uv, ls, lane);
    __syncwarp();
    const float den = __uint2float_rn(max(ncp - 1u, 1u));
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t idx = lane + 32u * k;
        mp[k] = mk3(0.0f, 0.0f, 0.0f);
        wk[k] = aok[k] = 0.0f;
        if (idx < ncp) {
            float w = __fdiv_rn(__uint2float_rn(idx), den);
            float layers_f = w * (float)(kLayerCount - 1u);
            uint32_t i0 = min(f2u(floorf(layers_f)), kLayerCount - 1u);
            uint32_t i1 = min(i0 + 1u, kLayerCount - 1u);
            float t = layers_f - __uint2float_rn(i0);
            float4 la = lp[i0], lb = lp[i1];
            f3 base = hermite(xyz(la), xyz(lb), xyz(lt[i0]), xyz(lt[i1]), t);
            f3 res = style_at(ls, w);
            mp[k] = add3(base, res);
            wk[k] = w;
            aok[k] = mixf(la.w, lb.w, t);
        }
    }
}

// Neighbours j-1 and j+1 of the control point in slot k of this lane: the next
// lane down/up of the same slot, or lane 31 / lane 0 of the adjacent slot.
// Every lane of the warp must call this (shuffles).
template <int K>
__device__ __forceinline__ void cp_neighbours(const f3 mp[4], uint32_t lane, f3& prev, f3& next) {
    prev = shfl_up3(mp[K]);
    next = shfl_down3(mp[K]);
    if (K > 0) {
        f3 w31 = shfl_idx3(mp[K > 0 ? K - 1 : 0], 31);
        if (lane == 0) prev = w31;
    }
    if (K < 3) {
        f3 w0 = shfl_idx3(mp[K < 3 ? K + 1 : 3], 0);
        if (lane == 31) next = w0;
    }
}

// World tangent of control point idx (raster.wgsl:286-317, then dir_world).
__device__ __forceinline__ f3 cp_world_tangent(const hg_hair_params& p, uint32_t idx, uint32_t ncp, f3 prev, f3 curr,
                                               f3 next) {
    const f3 pp = idx > 0u ? prev : curr;
    const f3 nn = idx + 1u < ncp ? next : curr;
    return dir_world(p, safe_normalize(calc_tangent(idx, ncp, pp, curr, nn)));
}

__device__ __forceinline__ bool finite3(float a, float b, float c) {
    const float inf = __int_as_float(0x7f800000);
    return fabsf(a) < inf && fabsf(b) < inf && fabsf(c) < inf;
}

// Projection and shared-memory layout of one control point.  Returns, for
// the camera pass, whether every value the camera raster mixes (world
// position, tangent, w, screen position, ao) is finite.
template <int MODE>
__device__ __forceinline__ bool store_cp(const hg_hair_params& p, StrandSmem& sm, uint32_t idx, f3 wp, f3 wt, float w,
                                         float ao) {
    const Projected pr = project_world(p, wp);
    sm.cp[idx] = make_float4(wp.x, wp.y, wp.z, pr.in_front ? 1.0f : 0.0f);
    if (MODE == 0) {
        sm.ct[idx] = make_float4(wt.x, wt.y, wt.z, w);
        sm.cs[idx] = make_float4(pr.screen.x, pr.screen.y, ao, 0.0f);
        sm.vd[idx] = pr.view_dist;
        return finite3(wp.x, wp.y, wp.z) && finite3(wt.x, wt.y, wt.z) && finite3(w, ao, pr.screen.x) &&
               finite3(pr.screen.y, 0.0f, 0.0f);
    }
    sm.cs[idx] = make_float4(pr.screen.x, pr.screen.y, 0.0f, 0.0f);
    return false;
}

template <int K, int MODE>
__device__ __forceinline__ void generate_slot(const hg_hair_params& p, StrandSmem& sm, const f3 mp[4],
                                              const float wk[4], const float aok[4], uint32_t ncp, uint32_t lane) {
    const uint32_t idx = lane + 32u * K;
    f3 prev = mp[K], next = mp[K];
    if (MODE == 0) cp_neighbours<K>(mp, lane, prev, next);
    bool fin = false;
    if (idx < ncp) {
        const f3 wp = to_world(p, mp[K]);
        const f3 wt = MODE == 0 ? cp_world_tangent(p, idx, ncp, prev, mp[K], next) : mk3(0.0f, 0.0f, 0.0f);
        fin = store_cp<MODE>(p, sm, idx, wp, wt, wk[K], aok[K]);
    }
    if (MODE == 0) {
        const uint32_t m = __ballot_sync(0xffffffffu, fin);
        if (lane == 0) sm.finm[K] = m;
    }
}

// Strand generation (raster.wgsl:231-317) for one warp.  Leaves world-space
// control points (+ in_front), screen positions and, for the camera pass,
// world tangents, w and ao in shared memory.  Strands at kCacheCps control
// points come from the frame's strand cache when one is given; the DOM passes
// need positions only.  With a non-null `deferred`, a cached camera strand's
// tangents (and w) are not read: *deferred gets their address in the cache
// for load_tangents, and sm.ct holds zeros until then.
template <int MODE, class Args>
__device__ __forceinline__ uint32_t generate_strand(const Args& a, StrandSmem& sm, const hg_strand_ref& ref,
                                                    const hg_gpu_bundle& bundle, float2 uv, uint32_t lane,
                                                    const float4** deferred = nullptr) {
    const hg_hair_params& p = a.p;
    const uint32_t ncp = min(max(ref.control_points, 2u), 127u);
    if (a.cache && ncp == kCacheCps) {
        const float4* pos = a.cache + (size_t)(a.strand_base[ref.bundle] + ref.strand) * (2u * kCacheCps);
        const float4* tan = pos + kCacheCps;
        const bool defer = MODE == 0 && deferred != nullptr;
        if (defer) *deferred = tan;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint32_t idx = lane + 32u * k;
            bool fin = false;
            if (idx < kCacheCps) {
                const float4 wp = __ldg(pos + idx);
                const float4 wt = MODE == 0 && !defer ? __ldg(tan + idx) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                fin = store_cp<MODE>(p, sm, idx, xyz(wp), xyz(wt), wt.w, wp.w);
            }
            if (MODE == 0) {
                const uint32_t m = __ballot_sync(0xffffffffu, fin);
                if (lane == 0) sm.finm[k] = m;
            }
        }
        if (MODE == 0 && lane == 0) sm.finm[3] = 0u;
        __syncwarp();
        return ncp;
    }
    f3 mp[4];
    float wk[4], aok[4];
    model_cps(a.layers, a.style, sm.u.gen.lp, sm.u.gen.lt, sm.u.gen.ls, bundle, uv, ncp, lane, mp, wk, aok);
    generate_slot<0, MODE>(p, sm, mp, wk, aok, ncp, lane);
    generate_slot<1, MODE>(p, sm, mp, wk, aok, ncp, lane);
    generate_slot<2, MODE>(p, sm, mp, wk, aok, ncp, lane);
    generate_slot<3, MODE>(p, sm, mp, wk, aok, ncp, lane);
    __syncwarp();
    return ncp;
}

// The largest x with sqrt_rn(x) <= r, so that sqrt_rn(d) <= r  <=>  d <= x for
// every d >= 0 (sqrt_rn is monotone).  Found from r*r by stepping one ulp at a
// time; a handful of steps at most, bounded here by 8 each way.
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

// The tangents (xyz, w) of a cached camera strand whose load generate_strand
// deferred, into sm.ct, and the finiteness of each into finm (and with the
// positions' bits).  Every lane of the warp calls it.
__device__ __forceinline__ void load_tangents(StrandSmem& sm, const float4* tan, uint32_t lane, uint32_t (&finm)[4]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const uint32_t idx = lane + 32u * k;
        bool fin = false;
        if (idx < kCacheCps) {
            const float4 wt = __ldg(tan + idx);
            sm.ct[idx] = wt;
            fin = finite3(wt.x, wt.y, wt.z) && finite3(wt.w, 0.0f, 0.0f);
        }
        finm[k] &= __ballot_sync(0xffffffffu, fin);
    }
    __syncwarp();
}

// The centre-disk test's bound on |o|^2: length(o) <= diameter / 2
// (raster.wgsl:206-212), the diameter at least 0.05.
__device__ __forceinline__ float camera_r2_max(const hg_hair_params& p) {
    return sqrt_bound(fmaxf(p.appearance[3], 0.05f) * 0.5f);
}

// High 32 bits of a G-buffer word, read through L2 (little endian: the second u32).
__device__ __forceinline__ uint32_t hi_word(const unsigned long long* w) {
    return __ldcg(reinterpret_cast<const unsigned int*>(w) + 1);
}

// The same through L1 (ld.global.ca).  L1 is not coherent with other SMs'
// atomics, so the value may be one the word held earlier in the pass; words
// only decrease, so it is still an upper bound of the current word.
__device__ __forceinline__ uint32_t hi_word_l1(const unsigned long long* w) {
    uint32_t r;
    asm("ld.global.ca.u32 %0, [%1];" : "=r"(r) : "l"(reinterpret_cast<const unsigned int*>(w) + 1));
    return r;
}

__device__ __forceinline__ bool on_screen(int32_t x, int32_t y, int32_t w, int32_t h) {
    return x >= 0 && y >= 0 && x < w && y < h;
}

// Flattened sample lists.  The camera and DOM rasters cut each segment of a
// strand into samples and hand them to the 32 lanes 32 at a time; segments
// with samples ("runs") are listed in order with their first sample.

// Lists a strand's runs: segment lane + 32 k has cnt[k] samples, and each
// segment with samples is appended in segment order with its first sample
// (sm.u.run.off) and tag[k] (sm.u.run.seg).  The four
// rounds' exclusive offsets come from two warp prefix sums, two rounds
// sharing a 32-bit word 16 bits each (a round's total is at most
// 32 (kMaxSteps + 1) < 2^16).  Leaves the strand's sample total and run
// count.  Every lane of the warp calls it.
__device__ __forceinline__ void append_runs4(StrandSmem& sm, const int32_t (&cnt)[4], const int32_t (&tag)[4],
                                             uint32_t lane, int32_t& total, int32_t& runs) {
    static_assert(32 * (kMaxSteps + 1) < 65536, "a round's sample count must fit 16 bits");
    uint32_t w01 = (uint32_t)cnt[0] | (uint32_t)cnt[1] << 16u, w23 = (uint32_t)cnt[2] | (uint32_t)cnt[3] << 16u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y01 = __shfl_up_sync(0xffffffffu, w01, o), y23 = __shfl_up_sync(0xffffffffu, w23, o);
        if ((int32_t)lane >= o) {
            w01 += y01;
            w23 += y23;
        }
    }
    const uint32_t t01 = __shfl_sync(0xffffffffu, w01, 31), t23 = __shfl_sync(0xffffffffu, w23, 31);
    const uint32_t below = (1u << lane) - 1u;
    int32_t carry = 0;
    runs = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t sh = 16u * (uint32_t)(k & 1);
        const int32_t incl = (int32_t)(((k < 2 ? w01 : w23) >> sh) & 0xffffu);
        const uint32_t live = __ballot_sync(0xffffffffu, cnt[k] > 0);
        if (cnt[k] > 0) {
            const int32_t r = runs + __popc(live & below);
            sm.u.run.off[r] = carry + incl - cnt[k];
            sm.u.run.seg[r] = tag[k];
        }
        carry += (int32_t)(((k < 2 ? t01 : t23) >> sh) & 0xffffu);
        runs += __popc(live);
    }
    total = carry;
}

// The run holding sample base + lane, for the window of samples [base,
// base + 32); rw is the run holding sample `base` and advances to the one
// holding base + 32.  Lane k holds the start of run rw+1+k: at most 32 runs
// start in (base, base + 32], one per sample.  Bit q of `starts` marks a run
// starting at base + q, so sample s lies in run rw + (starts in (base, s]).
// Every lane of the warp calls it.
__device__ __forceinline__ int32_t run_of_lane(const StrandSmem& sm, int32_t runs, int32_t& rw, int32_t base,
                                               uint32_t lane) {
    const int32_t rk = rw + 1 + (int32_t)lane;
    const int32_t ok = rk < runs ? sm.u.run.off[rk] : 0x7fffffff;
    const int32_t rel = ok - base;
    const uint32_t starts = __reduce_or_sync(0xffffffffu, rel > 0 && rel < 32 ? 1u << rel : 0u);
    const int32_t r = rw + __popc(starts & (0xffffffffu >> (31u - lane)));
    rw += __popc(__ballot_sync(0xffffffffu, ok <= base + 32));
    return r;
}

// Stage boundaries of the camera pass over the refs in draw order, in 1/256ths.
// The first stage draws the nearest 7/16 without tile depths; the tile depths
// it leaves then hide most of the rest.  Measured on 100k wavy strands at
// 1920x1080 (camera raster ms): first stage 1/8 0.440, 1/4 0.380, 3/8 0.352,
// 7/16 0.352, 1/2 0.352, 5/8 0.376, 3/4 0.401; three stages (3/8, 11/16)
// 0.369.
constexpr uint32_t kCameraFirstStage = 112;
constexpr uint32_t kCameraStages[] = {0, kCameraFirstStage, 256};
constexpr int kCameraStageCount = sizeof(kCameraStages) / sizeof(kCameraStages[0]);

// True when no sample of segment (pa, pb) (world, in sm.cp) / (A, B) (screen)
// can change a G-buffer word: every pixel it can reach is off screen, or
// (given tile depths) lies in tiles whose words all hold a nearer depth than
// the segment's nearest possible sample.  Conservative by construction:
//  - pixels: a sample sits at floor(mix(A, B, t)), and mix stays within
//    3 ulp of [min, max]; with |coordinates| < 2^20 that is < 0.2 px, so the
//    box floor(min) - 1 .. floor(max) + 1 holds every sample and both
//    diagonal side pixels (each a coordinate of a neighbouring sample);
//  - depth: a sample's computed view distance differs from the exact linear
//    one by < 21 u (M + C) (M, C: largest endpoint and camera coordinate,
//    u = 2^-24), an endpoint's by < 12 u (M + C); the bound below subtracts
//    1e-5 (M + C), about 5x their sum, and quantize_depth is monotone;
//  - a word with depth D < the sample's depth d rejects the sample's
//    payload (depth in the high bits) and its beta word (d << 8 | beta) alike.
// Non-finite or very large coordinates are never rejected, nor are segments
// whose pixel box spans more than 2 x 2 tiles (four fixed loads keep the test
// branch-free; it measured faster than walking up to six tiles).
__device__ __forceinline__ bool hidden_segment(const hg_hair_params& p, const uint32_t* tile_depth, uint32_t tiles_x,
                                               int32_t width, int32_t height, float4 pa, float4 pb, float4 A, float4 B,
                                               f3 cam, f3 fwd) {
    const float lim = 1048576.0f;
    if (!(fabsf(A.x) < lim && fabsf(A.y) < lim && fabsf(B.x) < lim && fabsf(B.y) < lim)) return false;
    const int32_t x0 = max(f2i(floorf(fminf(A.x, B.x))) - 1, 0), x1 = min(f2i(floorf(fmaxf(A.x, B.x))) + 1, width - 1);
    const int32_t y0 = max(f2i(floorf(fminf(A.y, B.y))) - 1, 0), y1 = min(f2i(floorf(fmaxf(A.y, B.y))) + 1, height - 1);
    if (x0 > x1 || y0 > y1) return true;  // nothing on screen
    if (!tile_depth) return false;
    const int32_t tx0 = x0 >> kTileShift, tx1 = x1 >> kTileShift, ty0 = y0 >> kTileShift, ty1 = y1 >> kTileShift;
    if (tx1 - tx0 > 1 || ty1 - ty0 > 1) return false;
    const float d0 = dot3(sub3(xyz(pa), cam), fwd), d1 = dot3(sub3(xyz(pb), cam), fwd);
    const float m = fmaxf(fmaxf(fmaxf(fabsf(pa.x), fabsf(pa.y)), fmaxf(fabsf(pa.z), fabsf(pb.x))),
                          fmaxf(fabsf(pb.y), fabsf(pb.z)));
    const float c = fmaxf(fmaxf(fabsf(cam.x), fabsf(cam.y)), fabsf(cam.z));
    if (!(fabsf(d0) < 1e30f && fabsf(d1) < 1e30f && m < 1e30f)) return false;
    const uint32_t lower = quantize_depth(fminf(d0, d1) - 1e-5f * (m + c), p.screen[2], p.screen[3]);
    // at most 2 x 2 tiles, read as four loads (repeats when the box spans one)
    const uint32_t* row0 = tile_depth + (uint32_t)ty0 * tiles_x;
    const uint32_t* row1 = tile_depth + (uint32_t)ty1 * tiles_x;
    const uint32_t held = max(max(__ldg(row0 + tx0), __ldg(row0 + tx1)), max(__ldg(row1 + tx0), __ldg(row1 + tx1)));
    return lower > held;
}

// Centre-disk test of segment (A, B) (screen) for the pixel centre (cx, cy)
// (raster.wgsl:206-212): length(o) <= r is sqrt_rn(|o|^2) <= r, i.e.
// |o|^2 <= r2_max.
__device__ __forceinline__ bool in_centre_disk(float4 A, float4 B, float cx, float cy, float r2_max) {
    const float gx = B.x - A.x, gy = B.y - A.y;
    const float denom = fmaxf(gx * gx + gy * gy, 1e-6f);
    const float closest = clampf(__fdiv_rn((cx - A.x) * gx + (cy - A.y) * gy, denom), 0.0f, 1.0f);
    const float ox = cx - (A.x + gx * closest), oy = cy - (A.y + gy * closest);
    return ox * ox + oy * oy <= r2_max;
}

// A lower bound of quantize_depth(d) for every d >= dist, within a few units
// of it and without a division: (dist - near) times a rounded reciprocal of
// the range differs from the correctly rounded quotient by at most 3 ulp of a
// value <= 1, i.e. 3 units after the scale by 16777214, plus half a unit for
// each rounded product, so after truncation the two quantised depths differ
// by at most 5 (both are clamped the same way, which keeps the bound; a NaN
// gives 0, which rejects nothing).
constexpr uint32_t kApproxDepthSlack = 8;
__device__ __forceinline__ uint32_t approx_depth(float dist, float near_, float inv_range) {
    const float q = clampf((dist - near_) * inv_range, 0.0f, 1.0f);
    const uint32_t r = f2u(q * 16777214.0f);
    return r < 0x00fffffeu ? r : 0x00fffffeu;
}

// The largest quantised depth among the words of tile (tx, ty), pixels
// (tx, ty) << kTileShift onwards (one warp, every lane gets it).
__device__ __forceinline__ uint32_t tile_max_depth(const unsigned long long* center, const unsigned long long* cons,
                                                   const uint32_t* beta, uint32_t width, uint32_t height, uint32_t tx,
                                                   uint32_t ty, uint32_t lane) {
    constexpr uint32_t kSide = 1u << kTileShift, kPixels = kSide * kSide;
    uint32_t held = 0;
#pragma unroll
    for (uint32_t k = 0; k < (kPixels + 31u) / 32u; ++k) {
        const uint32_t q = 32u * k + lane;
        const uint32_t x = (tx << kTileShift) + (q & (kSide - 1u)), y = (ty << kTileShift) + (q >> kTileShift);
        if (q < kPixels && x < width && y < height) {
            const size_t i = (size_t)y * width + x;
            held = max(held, max(hi_word(&cons[i]) >> 8, hi_word(&center[i]) >> 8));
            held = max(held, __ldcg(&beta[i]) >> 8);
        }
    }
    return __reduce_max_sync(0xffffffffu, held);
}

// One warp per tile: the largest quantised depth among the tile's
// conservative, centre and beta words (empty words count as the far value
// 0xffffff, which rejects nothing; pixels beyond the screen edge are never
// written and count as 0).
__global__ void __launch_bounds__(256) tile_depth_kernel(const unsigned long long* __restrict__ center,
                                                         const unsigned long long* __restrict__ cons,
                                                         const uint32_t* __restrict__ beta, uint32_t width,
                                                         uint32_t height, uint32_t tiles_x, uint32_t tiles,
                                                         uint32_t* __restrict__ tile_depth) {
    const uint32_t tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (tile >= tiles) return;
    const uint32_t held = tile_max_depth(center, cons, beta, width, height, tile % tiles_x, tile / tiles_x, lane);
    if (lane == 0) tile_depth[tile] = held;
}

// Camera raster of one generated strand.  The DDA of every segment
// (raster.wgsl:192-223) is flattened into one list of samples so the 32 lanes
// share the work evenly.  Consecutive samples sit on consecutive lanes, so the
// previous step's pixel (for the diagonal side pixels) comes from the
// neighbouring lane, or from lane 31 of the previous round; it is the same
// floor(mix(a, b, (i-1)/n)) the DDA loop carries.  Each sample computes its
// payload once (raster.wgsl:83-108) and writes the centre pixel and, on a
// diagonal step, the two side pixels.
template <class Args>
__device__ __forceinline__ void raster_camera(const Args& a, StrandSmem& sm, uint32_t ncp, float2 uv,
                                              float beta, uint32_t lane, float r2_max,
                                              const uint32_t* tile_depth = nullptr, uint32_t tiles_x = 0,
                                              const float4* deferred_tan = nullptr) {
    const hg_hair_params& p = a.p;
    const int32_t nseg = (int32_t)ncp - 1;
    const int32_t width = f2i(p.screen[0]), height = f2i(p.screen[1]);
    const f3 cam = mk3(p.camera_pos[0], p.camera_pos[1], p.camera_pos[2]);
    const f3 fwd = mk3(p.camera_forward[0], p.camera_forward[1], p.camera_forward[2]);
    // Sample offsets: a segment with both ends behind the camera, or hidden
    // behind the tile depths, has no samples, every other one n + 1 >= 2; the
    // non-empty segments are listed in order with their first sample.
    int32_t cnts[4];
    float mag = 0.0f;  // largest |coordinate| of the strand's control points
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int32_t j = (int32_t)lane + 32 * k;
        int32_t& cnt = cnts[k];
        cnt = 0;
        if (j < nseg) {
            float4 pa = sm.cp[j], pb = sm.cp[j + 1];
            mag = fmaxf(mag, fmaxf(fmaxf(fmaxf(fabsf(pa.x), fabsf(pa.y)), fmaxf(fabsf(pa.z), fabsf(pb.x))),
                                   fmaxf(fabsf(pb.y), fabsf(pb.z))));
            int32_t n = 0;
            if (pa.w != 0.0f || pb.w != 0.0f) {
                float4 A = sm.cs[j], B = sm.cs[j + 1];
                float dx = B.x - A.x, dy = B.y - A.y;
                int32_t steps = f2i(ceilf(fmaxf(fabsf(dx), fabsf(dy))));
                n = min(max(steps, 1), kMaxSteps);
                cnt = n + 1;
                if (hidden_segment(p, tile_depth, tiles_x, width, height, pa, pb, A, B, cam, fwd)) cnt = 0;
            }
            sm.cs[j].w = n > 0 ? __frcp_rn(__int2float_rn(n)) : 0.0f;
        }
    }
    // A segment's first sample (t = 0) is the previous segment's last (t = 1):
    // mix(a, b, 1) and mix(b, c, 0) both give b exactly when a and c are
    // finite, so position, depth, tangent, w and ao, hence the payload, agree,
    // and a first sample never writes side pixels.  Only the centre-disk test
    // differs (it measures against each segment).  So when the previous
    // segment has samples and both outer control points are finite, the
    // segment starts at its second sample, and the previous segment's last
    // sample takes the centre disk of either segment (tag bit 15).
    uint32_t livem[4], finm[4], skipm[4];
    int32_t tags[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        livem[k] = __ballot_sync(0xffffffffu, cnts[k] > 0);
        finm[k] = sm.finm[k];
    }
    if (deferred_tan) {
        // tangents only for a strand with samples (most strands of the
        // second stage have none)
        if ((livem[0] | livem[1] | livem[2] | livem[3]) == 0u) return;
        load_tangents(sm, deferred_tan, lane, finm);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t prev_live = lane > 0 ? livem[k] >> (lane - 1u) & 1u : (k > 0 ? livem[k > 0 ? k - 1 : 0] >> 31 : 0u);
        const uint32_t fin_prev = lane > 0 ? finm[k] >> (lane - 1u) & 1u : (k > 0 ? finm[k > 0 ? k - 1 : 0] >> 31 : 0u);
        const uint32_t fin_next = lane < 31 ? finm[k] >> (lane + 1u) & 1u : (k < 3 ? finm[k < 3 ? k + 1 : 3] & 1u : 0u);
        skipm[k] = __ballot_sync(0xffffffffu, cnts[k] > 0 && (prev_live & fin_prev & fin_next) != 0u);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t skip = skipm[k] >> lane & 1u;
        const uint32_t dup_next = lane < 31 ? skipm[k] >> (lane + 1u) & 1u : (k < 3 ? skipm[k < 3 ? k + 1 : 3] & 1u : 0u);
        tags[k] = 0;
        if (cnts[k] > 0) {
            tags[k] = ((int32_t)lane + 32 * k) | (int32_t)(skip << 7) | (cnts[k] - 1) << 8 | (int32_t)(dup_next << 15);
            cnts[k] -= (int32_t)skip;
        }
    }
    int32_t total, runs;
    append_runs4(sm, cnts, tags, lane, total, runs);
    __syncwarp();

    // Depth pre-test.  A sample's computed view distance lies within
    // 42 u (M + C) (u = 2^-24; M, C: largest control-point and camera
    // coordinate) of mix(vd[j], vd[j+1], t) computed in floats: 21 u (M + C)
    // from the exact linear distance, 12 u (M + C) for each endpoint's, and
    // below 9 u (M + C) for the float mix; 1e-5 (M + C) is four times that.
    // approx_depth of the lowered value minus kApproxDepthSlack is then below
    // the sample's quantised depth, and a sample whose bound is above every
    // word it could write changes nothing: it is dropped before its exact
    // position and depth are computed.  Non-finite values never drop a sample.
    const float cmag = fmaxf(fmaxf(fabsf(cam.x), fabsf(cam.y)), fabsf(cam.z));
    const float slack = 1e-5f * (__uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(mag))) + cmag);
    const float inv_range = __frcp_rn(fmaxf(p.screen[3] - p.screen[2], 1e-3f));
    const uint32_t beta_q = f2u(clampf(beta, 0.0f, 1.0f) * 255.0f + 0.5f);
    const bool ao_on = p.flags[2] != 0u;
    const uint32_t quv = quant63(uv.x) | quant63(uv.y) << 6u;
    int32_t carry_px = 0, carry_py = 0;
    int32_t rw = 0;  // the run holding sample `base`
    for (int32_t base = 0; base < total; base += 32) {
        const int32_t s = min(base + (int32_t)lane, total - 1);
        const bool active = base + (int32_t)lane < total;
        const int32_t r = run_of_lane(sm, runs, rw, base, lane);
        const int32_t jn = sm.u.run.seg[r];
        const int32_t j = jn & 0x7f, n = (jn >> 8) & 0x7f, i = s - sm.u.run.off[r] + ((jn >> 7) & 1);
        const float4 A = sm.cs[j], B = sm.cs[j + 1];
        const float t = step_t(i, n, A.w);
        const float sx = mixf(A.x, B.x, t), sy = mixf(A.y, B.y, t);
        const int32_t px = f2i(floorf(sx)), py = f2i(floorf(sy));
        int32_t qx = __shfl_up_sync(0xffffffffu, px, 1), qy = __shfl_up_sync(0xffffffffu, py, 1);
        if (lane == 0) {
            qx = carry_px;
            qy = carry_py;
        }
        carry_px = __shfl_sync(0xffffffffu, px, 31);
        carry_py = __shfl_sync(0xffffffffu, py, 31);
        if (!active) continue;
        const bool side = i > 0 && qx != px && qy != py;
        const bool on0 = on_screen(px, py, width, height);
        const bool on1 = side && on_screen(qx, py, width, height);
        const bool on2 = side && on_screen(px, qy, width, height);
        if (!(on0 || on1 || on2)) continue;
        const uint32_t pix0 = (uint32_t)py * (uint32_t)width + (uint32_t)px;
        const uint32_t pix1 = (uint32_t)py * (uint32_t)width + (uint32_t)qx;
        const uint32_t pix2 = (uint32_t)qy * (uint32_t)width + (uint32_t)px;
        // High words (depth, tangent x) of the current payloads, read through L1
        // before the payload is known.  Buffers only decrease during the pass,
        // so a stale read is an upper bound, and a payload whose high word is
        // above it cannot lower the word: its atomicMin is skipped.  Equal high
        // words go to the atomic, which decides.
        const uint32_t cur_c0 = on0 ? hi_word_l1(&a.cons[pix0]) : 0u;
        const uint32_t cur_m0 = on0 ? hi_word_l1(&a.center[pix0]) : 0u;
        const uint32_t cur_c1 = on1 ? hi_word_l1(&a.cons[pix1]) : 0u;
        const uint32_t cur_c2 = on2 ? hi_word_l1(&a.cons[pix2]) : 0u;
        {
            const uint32_t held = max(max(cur_c0, cur_m0), max(cur_c1, cur_c2)) >> 8u;
            const uint32_t bound = approx_depth(mixf(sm.vd[j], sm.vd[j + 1], t) - slack, p.screen[2], inv_range);
            if (bound > held + kApproxDepthSlack) continue;
        }

        // write_pixel (raster.wgsl:83-115): depth first; the rest of the payload
        // only when some word can still take it.
        const float4 c0 = sm.cp[j], c1 = sm.cp[j + 1];
        const f3 world = mix3(xyz(c0), xyz(c1), t);
        const float dist = dot3(sub3(world, cam), fwd);
        if (dist <= p.screen[2]) continue;
        const uint32_t depth = quantize_depth(dist, p.screen[2], p.screen[3]);
        const uint32_t lower = depth << 8u;  // high word of the smallest payload with this depth
        bool w0 = on0 && lower <= cur_c0;
        bool wm = on0 && depth <= cur_m0 >> 8u;
        bool w1 = on1 && lower <= cur_c1;
        bool w2 = on2 && lower <= cur_c2;
        if (wm) {
            const float cx = __int2float_rn(px) + 0.5f, cy = __int2float_rn(py) + 0.5f;
            wm = in_centre_disk(A, B, cx, cy, r2_max);
            // the next segment's dropped first sample: its own segment's disk
            if (!wm && i == n && (jn >> 15) != 0) wm = in_centre_disk(B, sm.cs[j + 2], cx, cy, r2_max);
        }
        if (!(w0 || wm || w1 || w2)) continue;
        if (a.scene) {
            const float4 clip = mat_mul(p.clip_from_world, world.x, world.y, world.z, 1.0f);
            const float clip_depth = __fdiv_rn(clip.z, fmaxf(clip.w, 1e-5f));
            const bool rev = p.pass_mode[2] == 1u;
            auto hidden = [&](uint32_t pix) {
                const float scene = __ldg(&a.scene[pix]);
                return rev ? clip_depth < scene : clip_depth > scene;
            };
            if ((w0 || wm) && hidden(pix0)) w0 = wm = false;
            if (w1 && hidden(pix1)) w1 = false;
            if (w2 && hidden(pix2)) w2 = false;
            if (!(w0 || wm || w1 || w2)) continue;
        }
        const float4 t0 = sm.ct[j], t1 = sm.ct[j + 1];
        const f3 tangent = safe_normalize(mix3(xyz(t0), xyz(t1), t));
        const uint32_t oct = oct_encode(tangent);
        const uint32_t ao_q = ao_on ? f2u(clampf(mixf(A.z, B.z, t), 0.0f, 1.0f) * 63.0f + 0.5f) : 63u;
        // mix(uv, uv, t) is uv, so its quantised value is the strand's own
        const unsigned long long payload = pack_gb(depth, oct & 0xffu, oct >> 8u, quv & 0x3fu, quv >> 6u,
                                                   quant63(mixf(t0.w, t1.w, t)), ao_q);
        const uint32_t high = (uint32_t)(payload >> 32u);
        if (w0 && high <= cur_c0) atomicMin(&a.cons[pix0], payload);
        if (wm) {
            if (high <= cur_m0) atomicMin(&a.center[pix0], payload);
            atomicMin(&a.beta[pix0], (depth << 8u) | beta_q);
        }
        if (w1 && high <= cur_c1) atomicMin(&a.cons[pix1], payload);
        if (w2 && high <= cur_c2) atomicMin(&a.cons[pix2], payload);
    }
}

// write_dom_pixel (raster.wgsl:118-148) for the Bresenham pixel (px, py) of
// the segment p0-p1 (screen a -> a + seg).
template <int MODE, class Args>
__device__ __forceinline__ void dom_write(const Args& a, int32_t px, int32_t py, int32_t width, int32_t height,
                                          float2 A, float2 seg, float seg_len2, f3 p0, f3 p1, float thickness) {
    const hg_hair_params& p = a.p;
    if (px < 0 || py < 0 || px >= width || py >= height) return;
    const uint32_t dom_w = f2u(p.dom_info[0]);
    const uint32_t pix = (uint32_t)py * dom_w + (uint32_t)px;
    // Mode 2 needs the texel's front depth (final after mode 1, and no word of
    // the front plane is written during mode 2, so the read-only path may
    // cache it); mode 1's atomicMin is fire-and-forget, which beats reading
    // the word first in this sequential per-lane loop.
    const uint32_t cur = MODE == 2 ? __ldg(&a.dom[pix]) : 0u;
    if (MODE == 2 && cur == kDomEmpty) return;
    const float2 ctr = make_float2(__int2float_rn(px) + 0.5f, __int2float_rn(py) + 0.5f);
    const float t = clampf(__fdiv_rn(dot2(sub2(ctr, A), seg), seg_len2), 0.0f, 1.0f);
    const f3 world = mix3(p0, p1, t);
    const float near_ = p.screen[2], far_ = p.screen[3];
    const float dist = dot3(sub3(world, mk3(p.camera_pos[0], p.camera_pos[1], p.camera_pos[2])),
                            mk3(p.camera_forward[0], p.camera_forward[1], p.camera_forward[2]));
    if (dist <= near_ || dist >= far_) return;
    if (MODE == 1) {
        atomicMin(&a.dom[pix], quantize_depth(dist, near_, far_));
        return;
    }
    const float z_front = dequantize_depth(cur, near_, far_);
    const float tt = __fdiv_rn(fmaxf(dist - z_front, 0.0f), thickness);
    const uint32_t slice = min(f2u(tt), kDomLayers - 1u);
    const uint32_t pixels = dom_w * f2u(p.dom_info[1]);
    atomicAdd(&a.dom[pixels + pix * kDomLayers + slice], 1u);
}

// draw_dom_segment (raster.wgsl:150-190), one segment per lane: the
// all-octant Bresenham walk from floor(a) to floor(b), at most 1024 steps, the
// start pixel skipped for all but the first segment unless the segment stays
// in one pixel.  (A flattened variant that spreads the walks' pixels evenly
// over the lanes, each pixel found in closed form, measured slower on config
// 2: segments average 3.3 pixels, and recomputing each pixel's segment state
// costs more than the idle lanes of the per-lane walk.)
template <int MODE, class Args>
__device__ __forceinline__ void raster_dom(const Args& a, StrandSmem& sm, uint32_t ncp, uint32_t lane) {
    const hg_hair_params& p = a.p;
    const int32_t width = f2i(p.screen[0]), height = f2i(p.screen[1]);
    // slice thickness of the layers pass (write_dom_pixel), the same for every texel
    const float thickness = __fdiv_rn(fmaxf(p.screen[3] - p.screen[2], 1e-3f), (float)kDomLayers);
    for (uint32_t j = lane; j + 1u < ncp; j += 32u) {
        float4 c0 = sm.cp[j], c1 = sm.cp[j + 1u];
        if (c0.w == 0.0f && c1.w == 0.0f) continue;
        float4 A4 = sm.cs[j], B4 = sm.cs[j + 1u];
        float2 A = make_float2(A4.x, A4.y), B = make_float2(B4.x, B4.y);
        int32_t x0 = f2i(floorf(A.x)), y0 = f2i(floorf(A.y));
        int32_t x1 = f2i(floorf(B.x)), y1 = f2i(floorf(B.y));
        int32_t dx = iabs(isub(x1, x0)), dy = iabs(isub(y1, y0));
        int32_t sx = x0 < x1 ? 1 : -1, sy = y0 < y1 ? 1 : -1;
        int32_t err = isub(dx, dy);
        float2 seg = sub2(B, A);
        float seg_len2 = fmaxf(dot2(seg, seg), 1e-6f);
        bool skip = j != 0u && (x0 != x1 || y0 != y1);
        f3 p0 = xyz(c0), p1 = xyz(c1);
        const int32_t ndy = (int32_t)(0u - (uint32_t)dy);
        for (int step = 0; step < 1024; ++step) {
            if (!skip) dom_write<MODE>(a, x0, y0, width, height, A, seg, seg_len2, p0, p1, thickness);
            skip = false;
            if (x0 == x1 && y0 == y1) break;
            int32_t e2 = iadd(err, err);
            if (e2 > ndy) {
                err = isub(err, dy);
                x0 = iadd(x0, sx);
            }
            if (e2 < dx) {
                err = iadd(err, dx);
                y0 = iadd(y0, sy);
            }
        }
    }
}

// Strand cache: every strand of the groom at kCacheCps control points, world
// space, warp per strand.  Per strand kCacheCps float4 (position, ao) then
// kCacheCps float4 (world tangent, w); the raster passes read these instead
// of regenerating the strand (raster.wgsl:231-317 is the same computation).
struct GenArgs {
    hg_hair_params p;
    const hg_gpu_bundle* bundles;
    const float4* layers;
    const float4* style;
    const uint32_t* strand_bundle;  // bundle of each strand
    const uint32_t* strand_base;    // first strand of each bundle
    float4* cache;
    uint32_t strands;
};

// The last control point (index 64) of up to 32 strands, finished together
// one per lane: the model-space point and its neighbour 63, w and ao, from
// generate_one, and the strand (and batch view) it belongs to.
struct CacheTails {
    float4 a[32];  // model point 64 xyz, ao
    float4 b[32];  // model point 63 xyz, w
    uint32_t strand[32];
    uint32_t view[32];
};

// Strand g of a groom into its cache slot (one warp): control points 0..63
// on the 32 lanes in two rounds.  Point 64 alone would take a third round at
// one lane in 32, so its inputs go to tails slot `slot` instead, and
// finish_tails completes 32 strands' last points in one round.
template <class Args>
__device__ __forceinline__ void generate_one(const Args& a, uint32_t g, float4* lp, float4* lt, float4* ls,
                                             uint32_t lane, CacheTails& tails, uint32_t slot, uint32_t view) {
    static_assert(kCacheCps == 65, "two full rounds of 32 control points and one tail point");
    const uint32_t b = a.strand_bundle[g];
    const uint32_t s = g - a.strand_base[b];
    const hg_gpu_bundle bundle = a.bundles[b];
    const float2 uv = pcg_uv(s ^ (b * 0x85ebca6bu));
    f3 mp[4];
    float wk[4], aok[4];
    model_cps(a.layers, a.style, lp, lt, ls, bundle, uv, kCacheCps, lane, mp, wk, aok);
    float4* pos = a.cache + (size_t)g * (2u * kCacheCps);
    float4* tan = pos + kCacheCps;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        f3 prev, next;
        if (k == 0) cp_neighbours<0>(mp, lane, prev, next);
        if (k == 1) cp_neighbours<1>(mp, lane, prev, next);
        const uint32_t idx = lane + 32u * k;
        const f3 wp = to_world(a.p, mp[k]);
        const f3 wt = cp_world_tangent(a.p, idx, kCacheCps, prev, mp[k], next);
        pos[idx] = make_float4(wp.x, wp.y, wp.z, aok[k]);
        tan[idx] = make_float4(wt.x, wt.y, wt.z, wk[k]);
    }
    // point 64 is slot 2 of lane 0; its neighbour 63 is slot 1 of lane 31
    const f3 p63 = shfl_idx3(mp[1], 31);
    if (lane == 0) {
        tails.a[slot] = make_float4(mp[2].x, mp[2].y, mp[2].z, aok[2]);
        tails.b[slot] = make_float4(p63.x, p63.y, p63.z, wk[2]);
        tails.strand[slot] = g;
        tails.view[slot] = view;
    }
    __syncwarp();
}

// Control point 64 of the strand in tails slot `slot` (a: that strand's
// arguments), written as generate_one's third round would (cp_world_tangent
// of the last point uses its previous neighbour and itself).  The lanes of a
// warp finish up to 32 slots at once.
template <class Args>
__device__ __forceinline__ void finish_tail(const Args& a, const CacheTails& tails, uint32_t slot) {
    const float4 ta = tails.a[slot], tb = tails.b[slot];
    const f3 curr = mk3(ta.x, ta.y, ta.z), prev = mk3(tb.x, tb.y, tb.z);
    const uint32_t idx = kCacheCps - 1u;
    const f3 wp = to_world(a.p, curr);
    const f3 wt = cp_world_tangent(a.p, idx, kCacheCps, prev, curr, curr);
    float4* pos = a.cache + (size_t)tails.strand[slot] * (2u * kCacheCps);
    pos[idx] = make_float4(wp.x, wp.y, wp.z, ta.w);
    pos[kCacheCps + idx] = make_float4(wt.x, wt.y, wt.z, tb.w);
}

__global__ void __launch_bounds__(kRasterThreads) generate_kernel(const GenArgs a) {
    __shared__ float4 lp[kRasterWarps][16];
    __shared__ float4 lt[kRasterWarps][16];
    __shared__ float4 ls[kRasterWarps][16];
    __shared__ CacheTails tails[kRasterWarps];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t nwarps = gridDim.x * kRasterWarps;
    uint32_t n = 0;
    for (uint32_t g = blockIdx.x * kRasterWarps + warp; g < a.strands; g += nwarps) {
        generate_one(a, g, lp[warp], lt[warp], ls[warp], lane, tails[warp], n, 0u);
        if (++n == 32u || g + nwarps >= a.strands) {
            if (lane < n) finish_tail(a, tails[warp], lane);
            __syncwarp();
            n = 0;
        }
    }
}

// Asynchronous global -> shared copies (cp.async) of the ref loop's next
// entries; the issuing lane waits for them before it or its warp reads them.
__device__ __forceinline__ void copy_async16(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void copy_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void copy_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void copy_async_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// sm.next_idx = the ref index drawn at position k: order[k], or k itself.
__device__ __forceinline__ void fetch_order(StrandSmem& sm, const uint32_t* order, uint32_t k) {
    if (order) copy_async4(&sm.next_idx, order + k);
    else sm.next_idx = k;
}

// Prefetches the strand cache slot of `ref` into L2 with one bulk prefetch:
// both of its arrays (2 x 65 float4, contiguous) for the camera pass, the
// positions for the deep-opacity passes.  Slots are 2,080 bytes apart from a
// 256-byte aligned base: the address and the size are multiples of 16 bytes
// as the instruction requires.  A hint only: nothing waits on it.
template <int MODE, class Args>
__device__ __forceinline__ void prefetch_cache_slot(const Args& a, const hg_strand_ref& ref) {
    if (!a.cache || ref.control_points != kCacheCps || ref.bundle >= a.bundle_count) return;
    const float4* slot = a.cache + (size_t)(a.strand_base[ref.bundle] + ref.strand) * (2u * kCacheCps);
    // the deep-opacity passes read the positions only (1,040 bytes)
    const uint32_t bytes = (MODE == 0 ? 2u : 1u) * kCacheCps * 16u;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(slot), "r"(bytes) : "memory");
}

// raster.wgsl:225-337: one warp per strand ref, persistent over the refs.
template <int MODE>
__global__ void __launch_bounds__(kRasterThreads, raster_min_blocks<MODE>()) raster_kernel(const RasterArgs a) {
    __shared__ StrandSmem smem[kRasterWarps];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    StrandSmem& sm = smem[warp];
    const unsigned long long total = a.indirect[0];
    const uint32_t r0 = (uint32_t)((total * a.part_lo) >> 8), r1 = (uint32_t)((total * a.part_hi) >> 8);
    const uint32_t* order = a.draw_order && a.order_meta[1] ? a.draw_order : nullptr;
    // A draw of every strand (no bundle culled or thinned: then, and only
    // then, the ref count is the groom's strand count) lays its refs out as
    // full_order expects.
    if (MODE == 1 && a.full_order && total == (unsigned long long)a.full_total) order = a.full_order;
    const uint32_t nwarps = gridDim.x * kRasterWarps;
    const float r2_max = MODE == 0 ? camera_r2_max(a.p) : 0.0f;
    // Software-pipelined over the refs: the draw-order entry two steps ahead
    // and the ref one step ahead are loaded before they are needed, and the
    // next strand's cache slot is prefetched into L2 while this strand is
    // drawn.  Without that every strand starts with a chain of dependent
    // loads (draw order, ref, strand base, cache slot) the warp waits on.
    uint32_t r = r0 + blockIdx.x * kRasterWarps + warp;
    if (lane == 0) {
        if (r < r1) copy_async16(&sm.next_ref, &a.refs[order ? order[r] : r]);
        if (r + nwarps < r1) fetch_order(sm, order, r + nwarps);
        copy_async_commit();
    }
    for (; r < r1; r += nwarps) {
        if (lane == 0) copy_async_wait();
        __syncwarp();
        const hg_strand_ref ref = sm.next_ref;
        const uint32_t next_idx = sm.next_idx;
        __syncwarp();
        const bool more = r + nwarps < r1;
        if (lane == 0) {
            if (more) copy_async16(&sm.next_ref, &a.refs[next_idx]);
            if (r + 2u * nwarps < r1) fetch_order(sm, order, r + 2u * nwarps);
            copy_async_commit();
        }
        if (ref.bundle >= a.bundle_count) {
            if (lane == 0) atomicOr(a.err, kErrBadRef);
            continue;
        }
        const hg_gpu_bundle bundle = a.bundles[ref.bundle];
        const float2 uv = pcg_uv(ref.strand ^ (ref.bundle * 0x85ebca6bu));
        // the second camera stage reads a cached strand's tangents only when
        // some segment of it is not hidden
        const float4* deferred = nullptr;
        const uint32_t ncp =
            generate_strand<MODE>(a, sm, ref, bundle, uv, lane, MODE == 0 && a.tile_depth ? &deferred : nullptr);
        if (lane == 0 && more) {
            copy_async_wait();
            prefetch_cache_slot<MODE>(a, sm.next_ref);
        }
        if (MODE == 0) {
            float beta = __fdiv_rn(__uint2float_rn(ref.n_lod), __uint2float_rn(max(bundle.strand_count, 1u)));
            raster_camera(a, sm, ncp, uv, beta, lane, r2_max, a.tile_depth, a.tiles_x, deferred);
        } else {
            raster_dom<MODE>(a, sm, ncp, lane);
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ batched frame
// Every pass of a batch of (groom, camera view, deep-opacity view) items in
// one launch each.  Work is indexed across views through prefix tables; a
// view's arguments are read in place from the device view table.

// Refs of a camera view drawn in the first stage: the nearest
// kCameraFirstStage / 256, as the single-view pass splits them.
__device__ __forceinline__ uint32_t camera_stage_split(uint32_t total) {
    return (uint32_t)(((unsigned long long)total * kCameraFirstStage) >> 8);
}

// Largest v in [0, n) with prefix[v] <= x, for x < prefix[n].  Plain loads:
// the prefix is in global memory for some callers and shared for others.
__device__ __forceinline__ uint32_t find_view(const uint32_t* prefix, uint32_t n, uint32_t x) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (prefix[mid] <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

// grid (X, items): block (x, i) clears item i's deep opacity map.
__global__ void batch_clear_dom_kernel(const BatchView* __restrict__ views, const uint32_t* __restrict__ dom_prefix,
                                       uint32_t* __restrict__ dom) {
    const BatchView& v = views[blockIdx.y];
    const size_t texels = (size_t)v.dom_w * v.dom_h, words = texels * (1 + kDomLayers);
    uint32_t* map = dom + dom_prefix[blockIdx.y];
    for (size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x; w < words; w += (size_t)gridDim.x * blockDim.x)
        map[w] = w < texels ? kDomEmpty : 0u;
}

__global__ void batch_lod_kernel(const BatchView* __restrict__ views, const uint32_t* __restrict__ prefix,
                                 uint32_t n_views, uint32_t total) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (w >= total) return;
    const uint32_t v = find_view(prefix, n_views, w);
    const BatchView& a = views[v];
    lod_bundle(a.p, a.bundles, a.layers, a.lod, a.depth_key, w - prefix[v], lane);
}

// Camera views also get the front-to-back draw order of the single-view scan.
__global__ void __launch_bounds__(kScanThreads) batch_scan_offsets_kernel(const BatchView* __restrict__ views) {
    const BatchView& a = views[blockIdx.x];
    const bool cam = a.p.pass_mode[0] == 0u && a.sorted;
    scan_offsets_block(a.lod, a.count, a.capacity, a.offsets, a.indirect, cam ? a.depth_key : nullptr,
                       cam ? a.sorted : nullptr, a.sorted_off, a.order_meta);
}

__global__ void batch_scan_expand_kernel(const BatchView* __restrict__ views, const uint32_t* __restrict__ prefix,
                                         uint32_t n_views, uint32_t total) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (w >= total) return;
    const uint32_t v = find_view(prefix, n_views, w);
    const BatchView& a = views[v];
    const uint32_t k = w - prefix[v];
    // camera views: warp k expands the k-th live bundle in draw order and
    // writes its draw-order entries; other views: bundle k
    const bool cam = a.p.pass_mode[0] == 0u && a.sorted;
    if (cam && k >= a.order_meta[0]) return;
    const uint32_t b = cam ? a.sorted[k] : k;
    const bool order = cam && a.order_meta[1] != 0u;
    const hg_lod_record rec = a.lod[b];
    const uint32_t off = a.offsets[b], dpos = cam ? a.sorted_off[k] : 0u;
    for (uint32_t s = lane; s < rec.n_lod; s += 32u) {
        const uint32_t i = off + s;
        if (i >= a.capacity) break;
        reinterpret_cast<uint4*>(a.refs)[i] = make_uint4(b, s, rec.n_lod, rec.control_points);
        if (order) a.draw_order[dpos + s] = i;
    }
}

// 8x8 tile depths of every camera view (tile_depth_kernel per view): warp per
// tile of the concatenated tile space.
__global__ void __launch_bounds__(256) batch_tile_depth_kernel(const BatchView* __restrict__ views,
                                                               const uint32_t* __restrict__ prefix, uint32_t n_cam,
                                                               uint32_t total) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (w >= total) return;
    const uint32_t v = find_view(prefix, n_cam, w);
    const BatchView& a = views[v];
    const uint32_t tile = w - prefix[v];
    const uint32_t held =
        tile_max_depth(a.center, a.cons, a.beta, a.width, a.height, tile % a.tiles_x, tile / a.tiles_x, lane);
    if (lane == 0) a.tile_depth[tile] = held;
}

__global__ void __launch_bounds__(kRasterThreads) batch_generate_kernel(const BatchView* __restrict__ views,
                                                                        const uint32_t* __restrict__ prefix,
                                                                        uint32_t n_cam, uint32_t total) {
    __shared__ float4 lp[kRasterWarps][16];
    __shared__ float4 lt[kRasterWarps][16];
    __shared__ float4 ls[kRasterWarps][16];
    __shared__ CacheTails tails[kRasterWarps];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t nwarps = gridDim.x * kRasterWarps;
    uint32_t n = 0;
    for (uint32_t g = blockIdx.x * kRasterWarps + warp; g < total; g += nwarps) {
        const uint32_t v = find_view(prefix, n_cam, g);
        generate_one(views[v], g - prefix[v], lp[warp], lt[warp], ls[warp], lane, tails[warp], n, v);
        if (++n == 32u || g + nwarps >= total) {
            if (lane < n) finish_tail(views[tails[warp].view[lane]], tails[warp], lane);
            __syncwarp();
            n = 0;
        }
    }
}

// Persistent raster over the refs of views [first, first + n): warps take
// `chunk` consecutive refs of the concatenated ref space at a time from a
// global counter, so grooms of very different sizes share the SMs.  Camera
// views draw their refs front to back (the scan's draw order) in two stages,
// as the single-view pass does: PHASE 0 runs the nearest 7/16 of every
// camera view's refs and every DOM depth view; PHASE 2 the rest of the camera
// refs, skipping segments hidden behind the tile depths built between the
// two; PHASE 1 the DOM views' layer pass.
template <int PHASE>
__global__ void __launch_bounds__(kRasterThreads, 6) batch_raster_kernel(const BatchView* __restrict__ views,
                                                                         uint32_t first, uint32_t n,
                                                                         uint32_t* __restrict__ counter,
                                                                         uint32_t chunk) {
    __shared__ StrandSmem smem[kRasterWarps];
    __shared__ uint32_t prefix[kBatchMaxViews + 1];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    // prefix of the views' ref totals: warp 0, eight views per lane
    if (warp == 0) {
        uint32_t t[kBatchMaxViews / 32];
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < (int)(kBatchMaxViews / 32); ++k) {
            const uint32_t v = lane * (kBatchMaxViews / 32) + k;
            uint32_t c = 0;
            if (v < n) {
                const BatchView& a = views[first + v];
                const uint32_t total = min(a.indirect[0], a.capacity);
                if (PHASE == 1 || a.p.pass_mode[0] != 0u) c = PHASE == 2 ? 0u : total;
                else c = PHASE == 0 ? camera_stage_split(total) : total - camera_stage_split(total);
            }
            t[k] = c;
            sum += t[k];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        uint32_t run = incl - sum;
#pragma unroll
        for (int k = 0; k < (int)(kBatchMaxViews / 32); ++k) {
            prefix[lane * (kBatchMaxViews / 32) + k] = run;
            run += t[k];
        }
        if (lane == 31) prefix[kBatchMaxViews] = incl;
    }
    __syncthreads();
    const uint32_t total = prefix[kBatchMaxViews];
    StrandSmem& sm = smem[warp];
    uint32_t v = 0;
    for (;;) {
        uint32_t start = 0;
        if (lane == 0) start = atomicAdd(counter, chunk);
        start = __shfl_sync(0xffffffffu, start, 0);
        if (start >= total) break;
        const uint32_t end = min(start + chunk, total);
        for (uint32_t r = start; r < end; ++r) {
            if (r < prefix[v] || r >= prefix[v + 1]) v = find_view(prefix, n, r);
            const BatchView& a = views[first + v];
            const bool cam = PHASE != 1 && a.p.pass_mode[0] == 0u;
            uint32_t pos = r - prefix[v];
            if (cam) {
                if (PHASE == 2) pos += camera_stage_split(min(a.indirect[0], a.capacity));
                if (a.sorted && a.order_meta[1]) pos = a.draw_order[pos];
            }
            const hg_strand_ref ref = a.refs[pos];
            if (ref.bundle >= a.bundle_count) {
                if (lane == 0) atomicOr(a.err, kErrBadRef);
                continue;
            }
            const hg_gpu_bundle bundle = a.bundles[ref.bundle];
            const float2 uv = pcg_uv(ref.strand ^ (ref.bundle * 0x85ebca6bu));
            if (PHASE == 1) {
                const uint32_t ncp = generate_strand<2>(a, sm, ref, bundle, uv, lane);
                raster_dom<2>(a, sm, ncp, lane);
            } else if (cam) {
                const float4* deferred = nullptr;
                const uint32_t ncp = generate_strand<0>(a, sm, ref, bundle, uv, lane, PHASE == 2 ? &deferred : nullptr);
                float beta = __fdiv_rn(__uint2float_rn(ref.n_lod), __uint2float_rn(max(bundle.strand_count, 1u)));
                raster_camera(a, sm, ncp, uv, beta, lane, camera_r2_max(a.p), PHASE == 2 ? a.tile_depth : nullptr,
                              a.tiles_x, deferred);
            } else {
                const uint32_t ncp = generate_strand<1>(a, sm, ref, bundle, uv, lane);
                raster_dom<1>(a, sm, ncp, lane);
            }
            __syncwarp();
        }
    }
}

// ------------------------------------------------------------------ binned camera raster
// The camera pass with each 32x32 screen tile's G-buffer words resolved in
// shared memory.  Every write is a commutative min, so the words equal the
// direct pass's.
//  1. bin_kernel: a warp per ref (in draw order) generates the strand exactly
//     as the direct pass does, keeps the control points' screen positions (and
//     world points of strands outside the strand cache), and lists each segment
//     as (tile, entry) pairs under the tiles its pixel box touches -- at most
//     2x2 tiles; a segment spanning more goes to a list of long segments.
//  2. bin_scan_kernel, bin_sort_kernel: per-tile counts scanned, the pairs
//     counting-sorted into per-tile runs of entries (roughly in draw order).
//  3. tile_resolve_kernel: a block per (tile, chunk of <= kBinChunk entries)
//     holds the tile's centre, conservative and beta words in shared memory,
//     draws the samples of its segments that land in the tile against them
//     (read-before-write and atomicMin in shared memory), and ends with one
//     global atomicMin per word it lowered.  long_segment_kernel draws the long
//     segments with global atomics.
constexpr int kBinShift = 5;                  // 32x32 pixel tiles
constexpr int kBinSize = 1 << kBinShift;
constexpr int kBinPixels = kBinSize * kBinSize;
constexpr uint32_t kBinChunk = 2048;          // entries per resolve work item
constexpr int kResolveWarps = 8;
constexpr int kResolveThreads = kResolveWarps * 32;
constexpr uint32_t kBinSegBits = 7;           // entry = draw slot << 7 | segment
constexpr uint32_t kBinMaxSlots = 1u << (32 - kBinSegBits);
constexpr uint32_t kNoCache = 0xffffffffu;

struct BinDev {
    float4* scr;
    float4* cpw;
    uint4* rinfo;
    uint2* pairs;
    uint32_t* entries;
    uint32_t* tile_count;
    uint32_t* tile_off;
    uint32_t* cursor;
    uint32_t* longs;
    uint32_t* meta;  // [0] pairs, [1] long segments, [2] largest chunk count of a tile, [3] work counter
    size_t pair_cap;
    uint32_t tiles_x, tiles_y;
};

// Tiles (up to 2x2) whose pixels segment (A, B) can reach, by the same pixel
// box as hidden_segment: floor(min) - 1 .. floor(max) + 1, clamped to the
// screen.  Returns the tile count (0: nothing on screen) or -1 for a segment
// that needs the long path (more than 2x2 tiles, or coordinates beyond 2^20).
__device__ __forceinline__ int segment_tiles(float4 A, float4 B, int32_t width, int32_t height, uint32_t tiles_x,
                                             uint32_t tile[4]) {
    const float lim = 1048576.0f;
    if (!(fabsf(A.x) < lim && fabsf(A.y) < lim && fabsf(B.x) < lim && fabsf(B.y) < lim)) return -1;
    const int32_t x0 = max(f2i(floorf(fminf(A.x, B.x))) - 1, 0), x1 = min(f2i(floorf(fmaxf(A.x, B.x))) + 1, width - 1);
    const int32_t y0 = max(f2i(floorf(fminf(A.y, B.y))) - 1, 0), y1 = min(f2i(floorf(fmaxf(A.y, B.y))) + 1, height - 1);
    if (x0 > x1 || y0 > y1) return 0;
    const int32_t tx0 = x0 >> kBinShift, tx1 = x1 >> kBinShift, ty0 = y0 >> kBinShift, ty1 = y1 >> kBinShift;
    if (tx1 - tx0 > 1 || ty1 - ty0 > 1) return -1;
    int n = 0;
    for (int32_t ty = ty0; ty <= ty1; ++ty)
        for (int32_t tx = tx0; tx <= tx1; ++tx) tile[n++] = (uint32_t)ty * tiles_x + (uint32_t)tx;
    return n;
}

// Step 1.  One warp per ref slot r (draw order); entry r << 7 | j for segment j.
__global__ void __launch_bounds__(kRasterThreads, 6) bin_kernel(const RasterArgs a, const BinDev d) {
    __shared__ StrandSmem smem[kRasterWarps];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    StrandSmem& sm = smem[warp];
    const uint32_t total = a.indirect[0];
    const uint32_t* order = a.draw_order && a.order_meta[1] ? a.draw_order : nullptr;
    const hg_hair_params& p = a.p;
    const int32_t width = f2i(p.screen[0]), height = f2i(p.screen[1]);
    const uint32_t nwarps = gridDim.x * kRasterWarps;
    for (uint32_t r = blockIdx.x * kRasterWarps + warp; r < total; r += nwarps) {
        const uint32_t ri = order ? order[r] : r;
        const hg_strand_ref ref = a.refs[ri];
        if (ref.bundle >= a.bundle_count) {
            if (lane == 0) atomicOr(a.err, kErrBadRef);
            continue;
        }
        const hg_gpu_bundle bundle = a.bundles[ref.bundle];
        const float2 uv = pcg_uv(ref.strand ^ (ref.bundle * 0x85ebca6bu));
        const uint32_t ncp = generate_strand<0>(a, sm, ref, bundle, uv, lane);
        const bool cached = a.cache && ncp == kCacheCps;
        if (lane == 0) {
            const float beta = __fdiv_rn(__uint2float_rn(ref.n_lod), __uint2float_rn(max(bundle.strand_count, 1u)));
            const uint32_t beta_q = f2u(clampf(beta, 0.0f, 1.0f) * 255.0f + 0.5f);
            const uint32_t quv = quant63(uv.x) | quant63(uv.y) << 6u;
            d.rinfo[r] = make_uint4(cached ? a.strand_base[ref.bundle] + ref.strand : kNoCache, quv | beta_q << 12u,
                                    ncp, ri);
        }
        float4* scr = d.scr + (size_t)r * 128u;
        float4* cpw = d.cpw + (size_t)r * 256u;
        for (uint32_t idx = lane; idx < ncp; idx += 32u) {
            const float4 cs = sm.cs[idx], cp = sm.cp[idx];
            scr[idx] = make_float4(cs.x, cs.y, cs.z, cp.w);
            if (!cached) {
                cpw[idx] = make_float4(cp.x, cp.y, cp.z, 0.0f);
                cpw[128u + idx] = sm.ct[idx];
            }
        }
        const int32_t nseg = (int32_t)ncp - 1;
#pragma unroll 1
        for (int k = 0; k < 4; ++k) {
            const int32_t j = (int32_t)lane + 32 * k;
            uint32_t tile[4] = {kNoCache, kNoCache, kNoCache, kNoCache};
            int nt = 0;
            if (j < nseg) {
                const float4 pa = sm.cp[j], pb = sm.cp[j + 1];
                if (pa.w != 0.0f || pb.w != 0.0f) nt = segment_tiles(sm.cs[j], sm.cs[j + 1], width, height, d.tiles_x, tile);
            }
            const uint32_t entry = r << kBinSegBits | (uint32_t)j;
            // long segments
            const uint32_t lmask = __ballot_sync(0xffffffffu, nt < 0);
            if (lmask) {
                uint32_t lbase = 0;
                if (lane == 0) lbase = atomicAdd(&d.meta[1], __popc(lmask));
                lbase = __shfl_sync(0xffffffffu, lbase, 0);
                if (nt < 0) d.longs[lbase + __popc(lmask & ((1u << lane) - 1u))] = entry;
                if (nt < 0) nt = 0;
            }
            // (tile, entry) pairs: one reservation per warp round
            int32_t incl = nt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int32_t)lane >= o) incl += y;
            }
            const uint32_t round_total = (uint32_t)__shfl_sync(0xffffffffu, incl, 31);
            if (round_total == 0) continue;
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&d.meta[0], round_total);
            base = __shfl_sync(0xffffffffu, base, 0);
            const uint32_t mine = base + (uint32_t)(incl - nt);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (q < nt) d.pairs[mine + q] = make_uint2(tile[q], entry);
                // per-tile counts, one atomic per distinct tile of the round
                const uint32_t key = q < nt ? tile[q] : kNoCache;
                const uint32_t group = __match_any_sync(0xffffffffu, key);
                if (key != kNoCache && lane == (uint32_t)(__ffs(group) - 1))
                    atomicAdd(&d.tile_count[key], (uint32_t)__popc(group));
            }
        }
    }
}

// Step 2a (one block): tile offsets, the sort cursors and the largest chunk
// count; resets the resolve work counter.
__global__ void __launch_bounds__(kScanThreads) bin_scan_kernel(const BinDev d) {
    __shared__ uint32_t warp_sums[33];
    __shared__ uint32_t s_max;
    const uint32_t tiles = d.tiles_x * d.tiles_y;
    if (threadIdx.x == 0) s_max = 0;
    __syncthreads();
    uint32_t carry = 0, local_max = 0;
    for (uint32_t base = 0; base < tiles; base += kScanThreads * kScanItems)
        carry += scan_pass(
            base, tiles, carry, warp_sums,
            [&](uint32_t i) {
                const uint32_t c = d.tile_count[i];
                local_max = max(local_max, (c + kBinChunk - 1) / kBinChunk);
                return c;
            },
            [&](uint32_t i, uint32_t at) {
                d.tile_off[i] = at;
                d.cursor[i] = at;
            });
    atomicMax(&s_max, local_max);
    __syncthreads();
    if (threadIdx.x == 0) {
        d.tile_off[tiles] = carry;
        d.meta[2] = s_max;
        d.meta[3] = 0u;
    }
}

// Step 2b: pairs into per-tile runs (one atomic per distinct tile of a warp).
__global__ void bin_sort_kernel(const BinDev d) {
    const uint32_t n = (uint32_t)min((size_t)d.meta[0], d.pair_cap);
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint2 pr = i < n ? d.pairs[i] : make_uint2(kNoCache, 0u);
        const uint32_t group = __match_any_sync(0xffffffffu, pr.x);
        const uint32_t leader = (uint32_t)(__ffs(group) - 1);
        uint32_t at = 0;
        if (pr.x != kNoCache && lane == leader) at = atomicAdd(&d.cursor[pr.x], (uint32_t)__popc(group));
        at = __shfl_sync(0xffffffffu, at, (int)leader);
        if (pr.x != kNoCache) d.entries[at + __popc(group & ((1u << lane) - 1u))] = pr.y;
    }
}

// A warp's batch of up to 32 segments in the resolve pass.
struct alignas(16) SegStage {
    float4 A[32], B[32];    // screen x, y, ao; A.w = RN(1/n), B.w = depth pre-test slack
    float4 pa[32], pb[32];  // world position, view distance
    float4 ta[32], tb[32];  // world tangent, w
    uint32_t meta[32];      // quv | beta_q << 12
    int32_t off[32];        // runs: first sample, in order
    int32_t seg[32];        // runs: batch slot | DDA steps n << 8
};

__device__ __forceinline__ uint32_t shared_hi(const unsigned long long* w) {
    return reinterpret_cast<const uint32_t*>(w)[1];
}

// Step 3.  Persistent blocks take work items v = chunk * tiles + tile from a
// counter, so every tile's first chunk is drawn before any second one.
__global__ void __launch_bounds__(kResolveThreads, 3) tile_resolve_kernel(const RasterArgs a, const BinDev d) {
    __shared__ unsigned long long s_center[kBinPixels], s_cons[kBinPixels];
    __shared__ uint32_t s_beta[kBinPixels];
    __shared__ uint32_t s_dirty[3][kBinPixels / 32];  // cons, centre, beta words lowered here
    __shared__ SegStage stage[kResolveWarps];
    __shared__ uint32_t s_item;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const hg_hair_params& p = a.p;
    const int32_t width = f2i(p.screen[0]), height = f2i(p.screen[1]);
    const uint32_t tiles = d.tiles_x * d.tiles_y;
    const uint32_t v_end = tiles * d.meta[2];
    const f3 cam = mk3(p.camera_pos[0], p.camera_pos[1], p.camera_pos[2]);
    const f3 fwd = mk3(p.camera_forward[0], p.camera_forward[1], p.camera_forward[2]);
    const float cmag = fmaxf(fmaxf(fabsf(cam.x), fabsf(cam.y)), fabsf(cam.z));
    const float inv_range = __frcp_rn(fmaxf(p.screen[3] - p.screen[2], 1e-3f));
    const float r2_max = camera_r2_max(p);
    const bool ao_on = p.flags[2] != 0u;
    const bool rev = p.pass_mode[2] == 1u;
    SegStage& st = stage[warp];
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(&d.meta[3], 1u);
        __syncthreads();
        const uint32_t v = s_item;
        __syncthreads();  // s_item is rewritten at the next item
        if (v >= v_end) break;
        const uint32_t chunk = v / tiles, tile = v - chunk * tiles;
        const uint32_t e_lo = d.tile_off[tile], e_hi = d.tile_off[tile + 1];
        const uint32_t e0 = e_lo + chunk * kBinChunk;
        if (e0 >= e_hi) continue;
        const uint32_t e1 = min(e_hi, e0 + kBinChunk);
        const int32_t tx = (int32_t)(tile % d.tiles_x), ty = (int32_t)(tile / d.tiles_x);
        const int32_t ox = tx << kBinShift, oy = ty << kBinShift;
        // The tile's words: empty for a tile's first chunk, else what global
        // memory holds now (any upper bound of the final words is correct).
        for (int q = threadIdx.x; q < kBinPixels; q += kResolveThreads) {
            const int32_t x = ox + (q & (kBinSize - 1)), y = oy + (q >> kBinShift);
            unsigned long long c = kEmptyU64, m = kEmptyU64;
            uint32_t bw = 0xffffffffu;
            if (chunk > 0 && x < width && y < height) {
                const size_t gi = (size_t)y * (size_t)width + (size_t)x;
                c = __ldcg(&a.cons[gi]);
                m = __ldcg(&a.center[gi]);
                bw = __ldcg(&a.beta[gi]);
            }
            s_cons[q] = c;
            s_center[q] = m;
            s_beta[q] = bw;
        }
        for (int q = threadIdx.x; q < 3 * kBinPixels / 32; q += kResolveThreads) (&s_dirty[0][0])[q] = 0u;
        __syncthreads();

        for (uint32_t wb = e0 + warp * 32u; wb < e1; wb += kResolveWarps * 32u) {
            // stage this warp's segments (lane k: entry wb + k)
            const uint32_t e = wb + lane;
            int32_t cnt = 0;
            if (e < e1) {
                const uint32_t entry = d.entries[e];
                const uint32_t r = entry >> kBinSegBits, j = entry & ((1u << kBinSegBits) - 1u);
                const uint4 info = d.rinfo[r];
                const float4* pos;
                const float4* tan;
                if (info.x != kNoCache) {
                    pos = a.cache + (size_t)info.x * (2u * kCacheCps);
                    tan = pos + kCacheCps;
                } else {
                    pos = d.cpw + (size_t)r * 256u;
                    tan = pos + 128;
                }
                const float4* scr = d.scr + (size_t)r * 128u;
                float4 A = __ldg(scr + j), B = __ldg(scr + j + 1);
                float4 pa = __ldg(pos + j), pb = __ldg(pos + j + 1);
                const float4 ta = __ldg(tan + j), tb = __ldg(tan + j + 1);
                const float dx = B.x - A.x, dy = B.y - A.y;
                const int32_t n = min(max(f2i(ceilf(fmaxf(fabsf(dx), fabsf(dy)))), 1), kMaxSteps);
                cnt = n + 1;
                const float m = fmaxf(fmaxf(fmaxf(fabsf(pa.x), fabsf(pa.y)), fmaxf(fabsf(pa.z), fabsf(pb.x))),
                                      fmaxf(fabsf(pb.y), fabsf(pb.z)));
                pa.w = dot3(sub3(xyz(pa), cam), fwd);
                pb.w = dot3(sub3(xyz(pb), cam), fwd);
                A.w = __frcp_rn(__int2float_rn(n));
                B.w = 1e-5f * (m + cmag);
                st.A[lane] = A;
                st.B[lane] = B;
                st.pa[lane] = pa;
                st.pb[lane] = pb;
                st.ta[lane] = ta;
                st.tb[lane] = tb;
                st.meta[lane] = info.y;
            }
            // runs: segment k's samples follow segment k-1's
            int32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int32_t)lane >= o) incl += y;
            }
            const uint32_t live = __ballot_sync(0xffffffffu, cnt > 0);
            if (cnt > 0) {
                const int32_t rr = __popc(live & ((1u << lane) - 1u));
                st.off[rr] = incl - cnt;
                st.seg[rr] = (int32_t)lane | (cnt - 1) << 8;
            }
            const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
            const int32_t runs = __popc(live);
            __syncwarp();

            int32_t carry_px = 0, carry_py = 0, rw = 0;
            for (int32_t base = 0; base < total; base += 32) {
                const int32_t s = min(base + (int32_t)lane, total - 1);
                const bool active = base + (int32_t)lane < total;
                // run of this lane's sample (as run_of_lane, over the stage)
                const int32_t rk = rw + 1 + (int32_t)lane;
                const int32_t okk = rk < runs ? st.off[rk] : 0x7fffffff;
                const int32_t rel = okk - base;
                const uint32_t starts = __reduce_or_sync(0xffffffffu, rel > 0 && rel < 32 ? 1u << rel : 0u);
                const int32_t rn = rw + __popc(starts & (0xffffffffu >> (31u - lane)));
                rw += __popc(__ballot_sync(0xffffffffu, okk <= base + 32));
                const int32_t jn = st.seg[rn];
                const int32_t k = jn & 0xff, i = s - st.off[rn];
                const float4 A = st.A[k], B = st.B[k];
                const float t = step_t(i, jn >> 8, A.w);
                const float sx = mixf(A.x, B.x, t), sy = mixf(A.y, B.y, t);
                const int32_t px = f2i(floorf(sx)), py = f2i(floorf(sy));
                int32_t qx = __shfl_up_sync(0xffffffffu, px, 1), qy = __shfl_up_sync(0xffffffffu, py, 1);
                if (lane == 0) {
                    qx = carry_px;
                    qy = carry_py;
                }
                carry_px = __shfl_sync(0xffffffffu, px, 31);
                carry_py = __shfl_sync(0xffffffffu, py, 31);
                if (!active) continue;
                const bool side = i > 0 && qx != px && qy != py;
                auto in_tile = [&](int32_t x, int32_t y) {
                    return on_screen(x, y, width, height) && (x >> kBinShift) == tx && (y >> kBinShift) == ty;
                };
                const bool on0 = in_tile(px, py);
                const bool on1 = side && in_tile(qx, py);
                const bool on2 = side && in_tile(px, qy);
                if (!(on0 || on1 || on2)) continue;
                const int32_t l0 = ((py - oy) << kBinShift) + (px - ox);
                const int32_t l1 = ((py - oy) << kBinShift) + (qx - ox);
                const int32_t l2 = ((qy - oy) << kBinShift) + (px - ox);
                const uint32_t cur_c0 = on0 ? shared_hi(&s_cons[l0]) : 0u;
                const uint32_t cur_m0 = on0 ? shared_hi(&s_center[l0]) : 0u;
                const uint32_t cur_c1 = on1 ? shared_hi(&s_cons[l1]) : 0u;
                const uint32_t cur_c2 = on2 ? shared_hi(&s_cons[l2]) : 0u;
                const float4 pa = st.pa[k], pb = st.pb[k];
                {
                    const uint32_t held = max(max(cur_c0, cur_m0), max(cur_c1, cur_c2)) >> 8u;
                    const uint32_t bound = approx_depth(mixf(pa.w, pb.w, t) - B.w, p.screen[2], inv_range);
                    if (bound > held + kApproxDepthSlack) continue;
                }
                // write_pixel (raster.wgsl:83-115), as raster_camera
                const f3 world = mix3(xyz(pa), xyz(pb), t);
                const float dist = dot3(sub3(world, cam), fwd);
                if (dist <= p.screen[2]) continue;
                const uint32_t depth = quantize_depth(dist, p.screen[2], p.screen[3]);
                const uint32_t lower = depth << 8u;
                bool w0 = on0 && lower <= cur_c0;
                bool wm = on0 && depth <= cur_m0 >> 8u;
                bool w1 = on1 && lower <= cur_c1;
                bool w2 = on2 && lower <= cur_c2;
                if (wm) {
                    const float cx = __int2float_rn(px) + 0.5f, cy = __int2float_rn(py) + 0.5f;
                    const float gx = B.x - A.x, gy = B.y - A.y;
                    const float denom = fmaxf(gx * gx + gy * gy, 1e-6f);
                    const float closest = clampf(__fdiv_rn((cx - A.x) * gx + (cy - A.y) * gy, denom), 0.0f, 1.0f);
                    const float ox2 = cx - (A.x + gx * closest), oy2 = cy - (A.y + gy * closest);
                    wm = ox2 * ox2 + oy2 * oy2 <= r2_max;
                }
                if (!(w0 || wm || w1 || w2)) continue;
                if (a.scene) {
                    const float4 clip = mat_mul(p.clip_from_world, world.x, world.y, world.z, 1.0f);
                    const float clip_depth = __fdiv_rn(clip.z, fmaxf(clip.w, 1e-5f));
                    auto hidden = [&](int32_t x, int32_t y) {
                        const float scene = __ldg(&a.scene[(size_t)y * (size_t)width + (size_t)x]);
                        return rev ? clip_depth < scene : clip_depth > scene;
                    };
                    if ((w0 || wm) && hidden(px, py)) w0 = wm = false;
                    if (w1 && hidden(qx, py)) w1 = false;
                    if (w2 && hidden(px, qy)) w2 = false;
                    if (!(w0 || wm || w1 || w2)) continue;
                }
                const float4 t0 = st.ta[k], t1 = st.tb[k];
                const f3 tangent = safe_normalize(mix3(xyz(t0), xyz(t1), t));
                const uint32_t oct = oct_encode(tangent);
                const uint32_t ao_q = ao_on ? f2u(clampf(mixf(A.z, B.z, t), 0.0f, 1.0f) * 63.0f + 0.5f) : 63u;
                const uint32_t mt = st.meta[k];
                const unsigned long long payload = pack_gb(depth, oct & 0xffu, oct >> 8u, mt & 0x3fu, (mt >> 6u) & 0x3fu,
                                                           quant63(mixf(t0.w, t1.w, t)), ao_q);
                const uint32_t high = (uint32_t)(payload >> 32u);
                auto lower_word = [&](unsigned long long* w, uint32_t* mask, int32_t l) {
                    if (payload < atomicMin(w, payload)) atomicOr(&mask[l >> 5], 1u << (l & 31));
                };
                if (w0 && high <= cur_c0) lower_word(&s_cons[l0], s_dirty[0], l0);
                if (wm) {
                    if (high <= cur_m0) lower_word(&s_center[l0], s_dirty[1], l0);
                    const uint32_t bw = (depth << 8u) | (mt >> 12u);
                    if (bw < atomicMin(&s_beta[l0], bw)) atomicOr(&s_dirty[2][l0 >> 5], 1u << (l0 & 31));
                }
                if (w1 && high <= cur_c1) lower_word(&s_cons[l1], s_dirty[0], l1);
                if (w2 && high <= cur_c2) lower_word(&s_cons[l2], s_dirty[0], l2);
            }
            __syncwarp();
        }
        __syncthreads();
        // one global atomicMin per word this item lowered
        for (int q = threadIdx.x; q < kBinPixels; q += kResolveThreads) {
            const uint32_t bit = 1u << (q & 31);
            const uint32_t dc = s_dirty[0][q >> 5] & bit, dm = s_dirty[1][q >> 5] & bit, db = s_dirty[2][q >> 5] & bit;
            if (!(dc | dm | db)) continue;
            const int32_t x = ox + (q & (kBinSize - 1)), y = oy + (q >> kBinShift);
            const size_t gi = (size_t)y * (size_t)width + (size_t)x;
            if (dc) atomicMin(&a.cons[gi], s_cons[q]);
            if (dm) atomicMin(&a.center[gi], s_center[q]);
            if (db) atomicMin(&a.beta[gi], s_beta[q]);
        }
        __syncthreads();
    }
}

// The long segments: one warp each, drawn as a one-segment strand by
// raster_camera (global atomics).
__global__ void __launch_bounds__(kRasterThreads) long_segment_kernel(const RasterArgs a, const BinDev d) {
    __shared__ StrandSmem smem[kRasterWarps];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    StrandSmem& sm = smem[warp];
    const uint32_t n = d.meta[1];
    const hg_hair_params& p = a.p;
    const f3 cam = mk3(p.camera_pos[0], p.camera_pos[1], p.camera_pos[2]);
    const f3 fwd = mk3(p.camera_forward[0], p.camera_forward[1], p.camera_forward[2]);
    for (uint32_t q = blockIdx.x * kRasterWarps + warp; q < n; q += gridDim.x * kRasterWarps) {
        const uint32_t entry = d.longs[q];
        const uint32_t r = entry >> kBinSegBits, j = entry & ((1u << kBinSegBits) - 1u);
        const uint4 info = d.rinfo[r];
        const hg_strand_ref ref = a.refs[info.w];
        const hg_gpu_bundle bundle = a.bundles[ref.bundle];
        const float2 uv = pcg_uv(ref.strand ^ (ref.bundle * 0x85ebca6bu));
        const float beta = __fdiv_rn(__uint2float_rn(ref.n_lod), __uint2float_rn(max(bundle.strand_count, 1u)));
        if (lane < 2u) {
            const float4* pos;
            const float4* tan;
            if (info.x != kNoCache) {
                pos = a.cache + (size_t)info.x * (2u * kCacheCps);
                tan = pos + kCacheCps;
            } else {
                pos = d.cpw + (size_t)r * 256u;
                tan = pos + 128;
            }
            const float4 sc = d.scr[(size_t)r * 128u + j + lane];
            const float4 wp = pos[j + lane];
            sm.cp[lane] = make_float4(wp.x, wp.y, wp.z, sc.w);
            sm.ct[lane] = tan[j + lane];
            sm.cs[lane] = make_float4(sc.x, sc.y, sc.z, 0.0f);
            sm.vd[lane] = dot3(sub3(xyz(wp), cam), fwd);
        }
        if (lane < 4u) sm.finm[lane] = 0u;  // a lone segment: no shared endpoint
        __syncwarp();
        raster_camera(a, sm, 2u, uv, beta, lane, camera_r2_max(a.p));
        __syncwarp();
    }
}

void free_bins(hg_bin_buffers& b) {
    for (void* ptr : {(void*)b.scr, (void*)b.cpw, (void*)b.rinfo, (void*)b.pairs, (void*)b.entries,
                      (void*)b.tile_count, (void*)b.tile_off, (void*)b.cursor, (void*)b.longs, (void*)b.meta})
        if (ptr) cudaFree(ptr);
    b = hg_bin_buffers{};
}

// The binned pass's scratch for this groom and a screen of `tiles` tiles.
cudaError_t ensure_bins(hg_groom* g, uint32_t tiles) {
    hg_bin_buffers& b = g->bins;
    if (b.meta && b.ref_cap >= g->ref_capacity && b.tile_cap >= tiles) return cudaSuccess;
    free_bins(b);
    const size_t refs = g->ref_capacity;
    b.pair_cap = refs * 126u * 4u;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto*& ptr, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc((void**)&ptr, std::max<size_t>(bytes, 16));
    };
    alloc(b.scr, refs * 128u * sizeof(float4));
    alloc(b.cpw, refs * 256u * sizeof(float4));
    alloc(b.rinfo, refs * sizeof(uint4));
    alloc(b.pairs, b.pair_cap * sizeof(uint2));
    alloc(b.entries, b.pair_cap * sizeof(uint32_t));
    alloc(b.tile_count, (size_t)tiles * 4u);
    alloc(b.tile_off, ((size_t)tiles + 1u) * 4u);
    alloc(b.cursor, (size_t)tiles * 4u);
    alloc(b.longs, refs * 126u * 4u);
    alloc(b.meta, 4u * 4u);
    if (e != cudaSuccess) {
        free_bins(b);
        return e;
    }
    b.ref_cap = (uint32_t)refs;
    b.tile_cap = tiles;
    return cudaSuccess;
}

cudaError_t launch_camera_binned(hg_ctx* ctx, hg_groom* g, const RasterArgs& a) {
    const uint32_t tiles_x = (ctx->width + kBinSize - 1) >> kBinShift;
    const uint32_t tiles_y = (ctx->height + kBinSize - 1) >> kBinShift;
    cudaError_t e = ensure_bins(g, tiles_x * tiles_y);
    if (e != cudaSuccess) return e;
    hg_bin_buffers& b = g->bins;
    BinDev d;
    d.scr = b.scr;
    d.cpw = b.cpw;
    d.rinfo = b.rinfo;
    d.pairs = b.pairs;
    d.entries = b.entries;
    d.tile_count = b.tile_count;
    d.tile_off = b.tile_off;
    d.cursor = b.cursor;
    d.longs = b.longs;
    d.meta = b.meta;
    d.pair_cap = b.pair_cap;
    d.tiles_x = tiles_x;
    d.tiles_y = tiles_y;
    if ((e = cudaMemsetAsync(b.tile_count, 0, (size_t)tiles_x * tiles_y * 4u, ctx->stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(b.meta, 0, 16, ctx->stream)) != cudaSuccess) return e;
    const int bin_blocks = (int)std::max<size_t>((g->ref_capacity + kRasterWarps - 1) / kRasterWarps, 1);
    bin_kernel<<<bin_blocks, kRasterThreads, 0, ctx->stream>>>(a, d);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    bin_scan_kernel<<<1, kScanThreads, 0, ctx->stream>>>(d);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    bin_sort_kernel<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(d);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    tile_resolve_kernel<<<ctx->sm_count * 3, kResolveThreads, 0, ctx->stream>>>(a, d);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    long_segment_kernel<<<ctx->sm_count * 2, kRasterThreads, 0, ctx->stream>>>(a, d);
    return cudaGetLastError();
}

int blocks_for(hg_ctx* ctx, const void* fn, int threads, size_t work_items, int per_block_items) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0);
    if (per_sm < 1) per_sm = 1;
    size_t need = (work_items + per_block_items - 1) / per_block_items;
    size_t cap = (size_t)ctx->sm_count * per_sm;
    size_t b = need < cap ? need : cap;
    return b < 1 ? 1 : (int)b;
}

// Screen targets of every camera view (contiguous arenas) and every deep
// opacity map.
cudaError_t launch_clear_arena(hg_ctx* ctx, const BatchDev& b) {
    const int threads = 256;
    if (b.total_px) {
        const int blocks = (int)std::min<uint64_t>((b.total_px / 4 + threads - 1) / threads + 1,
                                                   (uint64_t)ctx->sm_count * 8);
        clear_kernel<<<blocks, threads, 0, ctx->stream>>>(b.center, b.cons, b.beta, b.total_px);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (b.total_dom_words) {
        dim3 grid(std::max(1, 4 * ctx->sm_count / (int)std::max(b.n_cam, 1u)), b.n_cam);
        batch_clear_dom_kernel<<<grid, threads, 0, ctx->stream>>>(b.views, b.dom_prefix, b.dom);
        return cudaGetLastError();
    }
    return cudaSuccess;
}

}  // namespace

void release_bins(hg_groom* g) { free_bins(g->bins); }

cudaError_t launch_clear(hg_ctx* ctx) {
    size_t pixels = (size_t)ctx->width * ctx->height;
    int threads = 256;
    int blocks = (int)std::min<size_t>((pixels / 4 + threads - 1) / threads + 1, (size_t)ctx->sm_count * 8);
    clear_kernel<<<blocks, threads, 0, ctx->stream>>>(ctx->center, ctx->cons, ctx->beta, pixels);
    return cudaGetLastError();
}

cudaError_t launch_clear_dom(hg_ctx* ctx) {
    size_t texels = (size_t)ctx->dom_w * ctx->dom_h;
    size_t words = texels * (1 + kDomLayers);
    int threads = 256;
    int blocks = (int)std::min<size_t>((words / 4 + threads - 1) / threads + 1, (size_t)ctx->sm_count * 8);
    clear_dom_kernel<<<blocks, threads, 0, ctx->stream>>>(ctx->dom, texels, words);
    return cudaGetLastError();
}

cudaError_t launch_lod(hg_ctx* ctx, hg_groom* g, const hg_hair_params& p, int slot) {
    uint32_t count = std::min(p.pass_mode[1], g->bundle_count);
    if (count == 0) return cudaSuccess;
    int threads = 256;
    int blocks = (int)((count * 32u + threads - 1) / threads);
    lod_kernel<<<blocks, threads, 0, ctx->stream>>>(p, g->bundles, g->layers, g->lod[slot], g->depth_key[slot],
                                                    count);
    return cudaGetLastError();
}

cudaError_t launch_scan(hg_ctx* ctx, hg_groom* g, const hg_hair_params& p, int slot) {
    uint32_t count = std::min(p.pass_mode[1], g->bundle_count);
    // The camera pass draws near bundles first (its later stage skips what the
    // tile depths hide).  Sorting the DOM refs by light depth and staging the DOM
    // depth pass the same way measured slower (0.195 vs 0.170 ms on config 2):
    // its lanes walk one segment each, so a skipped segment rarely frees a warp.
    const bool order = p.pass_mode[0] == 0u;
    scan_offsets_kernel<<<1, kScanThreads, 0, ctx->stream>>>(
        g->lod[slot], count, g->ref_capacity, g->offsets[slot], g->indirect[slot], g->depth_key[slot],
        order ? g->sorted[slot] : nullptr, g->sorted_off[slot], g->order_meta[slot]);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || count == 0) return e;
    int threads = 256;
    int blocks = (int)std::min<uint32_t>((count * 32u + threads - 1) / threads, (uint32_t)ctx->sm_count * 8u);
    if (order) {
        scan_expand_sorted_kernel<<<blocks, threads, 0, ctx->stream>>>(g->lod[slot], g->offsets[slot], g->sorted[slot],
                                                                       g->sorted_off[slot], g->order_meta[slot],
                                                                       g->ref_capacity, g->refs[slot],
                                                                       g->draw_order[slot]);
    } else {
        scan_expand_kernel<<<blocks, threads, 0, ctx->stream>>>(g->lod[slot], g->offsets[slot], count,
                                                                g->ref_capacity, g->refs[slot]);
    }
    return cudaGetLastError();
}

cudaError_t launch_generate(hg_ctx* ctx, hg_groom* g, const hg_hair_params& p) {
    if (g->strand_total == 0) return cudaSuccess;
    GenArgs a;
    a.p = p;
    a.bundles = g->bundles;
    a.layers = g->layers;
    a.style = g->style;
    a.strand_bundle = g->strand_bundle;
    a.strand_base = g->strand_base;
    a.cache = g->cache;
    a.strands = g->strand_total;
    int blocks = blocks_for(ctx, (const void*)generate_kernel, kRasterThreads, g->strand_total, kRasterWarps);
    generate_kernel<<<blocks, kRasterThreads, 0, ctx->stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_raster(hg_ctx* ctx, hg_groom* g, const hg_hair_params& p, int slot, const float* scene) {
    if (g->bundle_count == 0) return cudaSuccess;
    RasterArgs a;
    a.p = p;
    a.bundles = g->bundles;
    a.layers = g->layers;
    a.style = g->style;
    a.refs = g->refs[slot];
    a.indirect = g->indirect[slot];
    a.draw_order = p.pass_mode[0] == 0u ? g->draw_order[slot] : nullptr;
    a.order_meta = g->order_meta[slot];
    a.full_order = p.pass_mode[0] == 1u ? g->dom_order : nullptr;
    a.full_total = g->strand_total;
    const bool cached = g->cache && g->cache_valid &&
                        std::memcmp(g->cache_model, p.world_from_model, sizeof(g->cache_model)) == 0;
    a.cache = cached ? g->cache : nullptr;
    a.strand_base = g->strand_base;
    a.center = ctx->center;
    a.cons = ctx->cons;
    a.beta = ctx->beta;
    a.dom = ctx->dom;
    a.scene = scene;
    a.err = ctx->err;
    a.bundle_count = g->bundle_count;
    a.part_lo = 0;
    a.part_hi = 256;
    a.tile_depth = nullptr;
    a.tiles_x = 0;
    uint32_t mode = p.pass_mode[0];
    // Persistent: as many blocks as stay resident (the deep-opacity passes:
    // kDomGridRounds times that; at most one warp per ref slot), each warp
    // walking the refs with a stride of the grid's warps, which lets it fetch
    // its next ref and prefetch that strand's cache slot while it draws the
    // current one.  (Handing refs out by atomic ticket instead, one or a few
    // at a time, measured 1.3-2x slower.)
    int blocks = (int)std::max<size_t>((g->ref_capacity + kRasterWarps - 1) / kRasterWarps, 1);
    if (mode == 0 && ctx->camera_raster == HG_CAMERA_RASTER_BINNED && g->ref_capacity <= kBinMaxSlots) {
        return launch_camera_binned(ctx, g, a);
    } else if (mode == 0) {
        // Refs in draw order (near bundles first), in stages; before each
        // stage after the first, the tile depths are rebuilt from the words
        // the earlier stages left, and segments behind them are skipped.
        const uint32_t tiles_x = tiles_along(ctx->width);
        const uint32_t tiles = tiles_x * tiles_along(ctx->height);
        for (int k = 0; k + 1 < kCameraStageCount; ++k) {
            a.part_lo = kCameraStages[k];
            a.part_hi = kCameraStages[k + 1];
            if (k > 0 && tiles && ctx->tile_depth) {
                tile_depth_kernel<<<(tiles + 7) / 8, 256, 0, ctx->stream>>>(ctx->center, ctx->cons, ctx->beta,
                                                                           ctx->width, ctx->height, tiles_x, tiles,
                                                                           ctx->tile_depth);
                cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) return e;
                a.tile_depth = ctx->tile_depth;
                a.tiles_x = tiles_x;
            }
            const size_t part = (g->ref_capacity * (a.part_hi - a.part_lo) + 255) / 256 + 1;
            const int stage_blocks = (int)std::max<size_t>(
                std::min<size_t>((part + kRasterWarps - 1) / kRasterWarps, (size_t)ctx->sm_count * raster_min_blocks<0>()),
                1);
            raster_kernel<0><<<stage_blocks, kRasterThreads, 0, ctx->stream>>>(a);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
    } else if (mode == 1) {
        raster_kernel<1><<<std::min(blocks, ctx->sm_count * raster_min_blocks<1>() * kDomGridRounds), kRasterThreads, 0,
                           ctx->stream>>>(a);
    } else {
        raster_kernel<2><<<std::min(blocks, ctx->sm_count * raster_min_blocks<2>() * kDomGridRounds), kRasterThreads, 0,
                           ctx->stream>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_batch_setup(hg_ctx* ctx, const BatchDev& b) {
    cudaError_t e = launch_clear_arena(ctx, b);
    if (e != cudaSuccess) return e;
    const int threads = 256;
    if (b.total_bundles) {
        const uint32_t blocks = (b.total_bundles * 32u + threads - 1) / threads;
        batch_lod_kernel<<<blocks, threads, 0, ctx->stream>>>(b.views, b.bundle_prefix, b.n_views, b.total_bundles);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    batch_scan_offsets_kernel<<<b.n_views, kScanThreads, 0, ctx->stream>>>(b.views);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (b.total_bundles) {
        const uint32_t blocks = (b.total_bundles * 32u + threads - 1) / threads;
        batch_scan_expand_kernel<<<blocks, threads, 0, ctx->stream>>>(b.views, b.bundle_prefix, b.n_views,
                                                                      b.total_bundles);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (b.total_strands) {
        const uint32_t need = (b.total_strands + kRasterWarps - 1) / kRasterWarps;
        const uint32_t blocks = std::max(1u, std::min(need, b.gen_blocks));
        batch_generate_kernel<<<blocks, kRasterThreads, 0, ctx->stream>>>(b.views, b.strand_prefix, b.n_cam,
                                                                          b.total_strands);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Resident blocks per SM of the batched raster and generate kernels (queried
// once, outside any stream capture).
cudaError_t batch_occupancy(uint32_t* raster_per_sm, uint32_t* gen_per_sm) {
    int r = 0, g = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, batch_raster_kernel<0>, kRasterThreads, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g, batch_generate_kernel, kRasterThreads, 0);
    *raster_per_sm = (uint32_t)std::max(r, 1);
    *gen_per_sm = (uint32_t)std::max(g, 1);
    return e;
}

cudaError_t launch_batch_raster(hg_ctx* ctx, const BatchDev& b) {
    cudaError_t e = cudaMemsetAsync(b.counters, 0, 3 * sizeof(uint32_t), ctx->stream);
    if (e != cudaSuccess) return e;
    const uint32_t per_sm = std::max(1u, b.raster_blocks_per_sm);
    const int blocks = ctx->sm_count * (int)per_sm;
    const uint32_t chunk = b.raster_chunk ? b.raster_chunk : 1u;
    // stage 1: nearest 7/16 of the camera refs + DOM depth views
    batch_raster_kernel<0><<<blocks, kRasterThreads, 0, ctx->stream>>>(b.views, 0u, b.n_views, b.counters, chunk);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // tile depths of the camera views, then stage 2: the rest of the camera refs
    if (b.total_tdepth) {
        const uint32_t tblocks = (b.total_tdepth + 7u) / 8u;
        batch_tile_depth_kernel<<<tblocks, 256, 0, ctx->stream>>>(b.views, b.tdepth_prefix, b.n_cam, b.total_tdepth);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    batch_raster_kernel<2><<<blocks, kRasterThreads, 0, ctx->stream>>>(b.views, 0u, b.n_cam, b.counters + 2, chunk);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (b.n_views > b.n_cam) {
        batch_raster_kernel<1><<<blocks, kRasterThreads, 0, ctx->stream>>>(b.views, b.n_cam, b.n_views - b.n_cam,
                                                                           b.counters + 1, chunk);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace hg

// ------------------------------------------------------------------ allocation-free scan
//
// hg_scan_noalloc: the scan pass for hosts that cannot allocate device memory
// while they record a frame -- for example an engine whose device memory is
// owned entirely by its own allocator or arena (a render graph that hands out
// every buffer up front), or a real-time host with a fixed memory budget
// that forbids allocation inside the frame loop.  The caller passes the
// LodRecords (input) and the StrandRef and indirect buffers (outputs) as
// device pointers; the only working memory the scan needs beyond them, the
// per-bundle offsets, lives in the file-scope array below instead of a
// cudaMalloc.

namespace hg {
namespace {

// Largest bundle count the allocation-free scan accepts: 65,536 bundles,
// i.e. 256 KB of offsets held on every device that loads this library.
constexpr uint32_t kNoAllocMaxBundles = 65536;
static __device__ __align__(256) uint32_t g_noalloc_offsets[kNoAllocMaxBundles + 1];

// Device address of g_noalloc_offsets, looked up once per CUDA context.  The
// host-side name g_noalloc_offsets is not a device address, so kernels are
// only ever given the address from cudaGetSymbolAddress.  The cache is keyed
// on the current context's unique ID (cuCtxGetId, reached through the
// runtime's driver entry points, so the library needs no link to libcuda):
// after a reset of the device's primary context (cudaDeviceReset) the module
// is loaded again, the array may sit at another address, and the new
// context's ID differs, so the address is looked up again.
using CtxGetCurrentFn = int (*)(void** ctx);
using CtxGetIdFn = int (*)(void* ctx, unsigned long long* id);

struct NoAllocSlot {
    unsigned long long ctx_id = 0;  // 0: never looked up (context IDs start at 1)
    uint32_t* ptr = nullptr;
};
constexpr int kNoAllocMaxDevices = 64;
NoAllocSlot g_noalloc_slot[kNoAllocMaxDevices];
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
std::mutex g_noalloc_mutex;

cudaError_t current_context_id(unsigned long long* id) {
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* f0 = nullptr;
        void* f1 = nullptr;
        cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = q0;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0);
        if (e == cudaSuccess)
            e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1);
        if (e != cudaSuccess) return e;
        if (q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
            return cudaErrorNotSupported;
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f1);
    }
    void* ctx = nullptr;
    if (g_ctx_get_current(&ctx) != 0 || !ctx) return cudaErrorDeviceUninitialized;
    return g_ctx_get_id(ctx, id) == 0 ? cudaSuccess : cudaErrorDeviceUninitialized;
}

cudaError_t noalloc_scratch(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    // makes the device's primary context current (created if need be)
    if ((e = cudaSetDevice(dev)) != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    unsigned long long id = 0;
    if ((e = current_context_id(&id)) != cudaSuccess) return e;
    NoAllocSlot& slot = g_noalloc_slot[dev];
    if (slot.ctx_id != id || !slot.ptr) {
        uint32_t* ptr = nullptr;
        e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_offsets);
        if (e != cudaSuccess) return e;
        slot.ptr = ptr;
        slot.ctx_id = id;
    }
    *out = slot.ptr;
    return cudaSuccess;
}

}  // namespace
}  // namespace hg

// See include/hairgb.h.  The first call on a device (the device current on
// the calling thread) looks up the scratch array's device address, and so
// does the first call after that device's primary context was reset; make
// those calls before any stream capture on that device.  Every call shares
// the one array, so calls that overlap on the GPU (different streams, no
// ordering between them) race on it; the offsets are fully rewritten by each
// call, so nothing needs clearing between calls.  A CUDA error already
// pending on the calling thread is reported (HG_CUDA_ERROR) before anything
// is launched and left in place, so the launch checks below see only this
// call's launches.
extern "C" hg_status hg_scan_noalloc(const hg_lod_record* lod, uint32_t bundle_count, uint32_t capacity,
                                     hg_strand_ref* refs, uint32_t* indirect, void* stream) {
    if (!indirect || (bundle_count && (!lod || !refs)) || capacity == 0) return HG_INVALID_ARG;
    if (bundle_count > hg::kNoAllocMaxBundles) return HG_CAPACITY_EXCEEDED;
    if (cudaPeekAtLastError() != cudaSuccess) return HG_CUDA_ERROR;
    uint32_t* offsets = nullptr;
    if (hg::noalloc_scratch(&offsets) != cudaSuccess) return HG_CUDA_ERROR;
    cudaStream_t st = (cudaStream_t)stream;
    hg::scan_offsets_kernel<<<1, hg::kScanThreads, 0, st>>>(lod, bundle_count, capacity, offsets, indirect, nullptr,
                                                            nullptr, nullptr, nullptr);
    if (cudaGetLastError() != cudaSuccess) return HG_CUDA_ERROR;
    if (bundle_count == 0) return HG_OK;
    int sms = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return HG_CUDA_ERROR;
    const int threads = 256;
    const int blocks = (int)std::min<uint32_t>((bundle_count * 32u + threads - 1) / threads, (uint32_t)sms * 8u);
    hg::scan_expand_kernel<<<blocks, threads, 0, st>>>(lod, offsets, bundle_count, capacity, refs);
    return cudaGetLastError() == cudaSuccess ? HG_OK : HG_CUDA_ERROR;
}
