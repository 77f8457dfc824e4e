// Measurement probes for the benchmark's roofline (libhairprobe.so, not part
// of the pipeline's C ABI): the L2 atomic throughput the raster passes are
// bound by, measured on this GPU with the access patterns the passes use.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// Each thread issues `iters` reductions.  pattern 0: a random word per
// operation; pattern 1: a warp covers 32 consecutive words (the DDA's
// neighbouring pixels).  op 0: 64-bit min, 1: 32-bit min, 2: 32-bit add.
template <int OP>
__global__ void atomics_kernel(void* buf, uint32_t words, uint32_t iters, int pattern) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t k = 0; k < iters; ++k) {
        uint32_t idx;
        if (pattern == 0) {
            idx = mix32(tid * 0x9e3779b9u + k) % words;
        } else {
            idx = (mix32((tid >> 5) * 0x9e3779b9u + k) % (words / 32u)) * 32u + lane;
        }
        const uint32_t v = mix32(idx ^ k);
        if (OP == 0) {
            atomicMin(reinterpret_cast<unsigned long long*>(buf) + idx, ((unsigned long long)v << 32) | k);
        } else if (OP == 1) {
            atomicMin(reinterpret_cast<uint32_t*>(buf) + idx, v);
        } else {
            atomicAdd(reinterpret_cast<uint32_t*>(buf) + idx, 1u);
        }
    }
}

}  // namespace

// Reductions per second of `op` (0: u64 min, 1: u32 min, 2: u32 add) over a
// buffer of `words` words with `pattern` (0 random, 1 warp-coherent), timed
// with CUDA events after one warm-up launch.  Returns 0 on success.
extern "C" int hg_probe_atomics(int op, int pattern, uint32_t words, double* ops_per_s) {
    if (!ops_per_s || words < 1024 || op < 0 || op > 2) return 1;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 2;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* buf = nullptr;
    const size_t bytes = (size_t)words * (op == 0 ? 8 : 4);
    if (cudaMalloc(&buf, bytes) != cudaSuccess) return 3;
    cudaMemset(buf, 0xff, bytes);
    const int threads = 256, blocks = sms * 8;
    const uint32_t iters = 256;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    auto launch = [&]() {
        if (op == 0) atomics_kernel<0><<<blocks, threads>>>(buf, words, iters, pattern);
        else if (op == 1) atomics_kernel<1><<<blocks, threads>>>(buf, words, iters, pattern);
        else atomics_kernel<2><<<blocks, threads>>>(buf, words, iters, pattern);
    };
    launch();
    cudaEventRecord(a);
    for (int r = 0; r < 5; ++r) launch();
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    const cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(buf);
    if (e != cudaSuccess || ms <= 0.0f) return 4;
    *ops_per_s = 5.0 * (double)blocks * threads * iters / (ms * 1e-3);
    return 0;
}
