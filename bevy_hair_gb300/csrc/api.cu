// C ABI of the hair pipeline: context and buffer ownership, argument
// validation, and the pass sequence of hair_pass (src/render/pass.rs:259-657).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/hairgb.h"
#include "hg_internal.h"

namespace {

hg_status fail(hg_ctx* ctx, hg_status s, const char* msg) {
    if (ctx) ctx->last_error = msg;
    return s;
}

hg_status cuda_fail(hg_ctx* ctx, cudaError_t e, const char* where) {
    if (ctx) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
        ctx->last_error = buf;
    }
    return e == cudaErrorMemoryAllocation ? HG_OUT_OF_MEMORY : HG_CUDA_ERROR;
}

#define HG_CUDA(ctx, expr)                                      \
    do {                                                        \
        cudaError_t e_ = (expr);                                \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #expr); \
    } while (0)

// A CUDA error already pending on the calling thread (a failed launch of the
// caller's own, or a device fault) is reported before a pass launches
// anything, and left in place for the caller: the launch checks below then
// read only the status of this call's own launches.
hg_status check_pending(hg_ctx* ctx) {
    const cudaError_t e = cudaPeekAtLastError();
    return e == cudaSuccess ? HG_OK : cuda_fail(ctx, e, "a CUDA error was pending before this call");
}

#define HG_PENDING(ctx)                          \
    do {                                         \
        hg_status p_ = check_pending(ctx);       \
        if (p_ != HG_OK) return p_;              \
    } while (0)

template <typename T>
void free_dev(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

constexpr uint32_t kGbufferBits = 1u << HG_BUF_CENTER | 1u << HG_BUF_CONSERVATIVE | 1u << HG_BUF_BETA;
constexpr uint32_t kColorBits = 1u << HG_BUF_COLOR | 1u << HG_BUF_DEPTH;

// Order work about to write `bits` (enqueued next on the context's current
// stream) after every asynchronous readback of those buffers.
cudaError_t guard_writes(hg_ctx* ctx, uint32_t bits) {
    if (!(ctx->pending_reads & bits)) return cudaSuccess;
    cudaError_t e = cudaStreamWaitEvent(ctx->stream, ctx->ev_copy_done, 0);
    if (e == cudaSuccess) ctx->pending_reads &= ~bits;
    return e;
}

void free_targets(hg_ctx* ctx) {
    free_dev(ctx->center);
    free_dev(ctx->cons);
    free_dev(ctx->beta);
    free_dev(ctx->dom);
    free_dev(ctx->shaded);
    free_dev(ctx->shaded_depth);
    free_dev(ctx->filtered);
    free_dev(ctx->filtered_depth);
    free_dev(ctx->color);
    free_dev(ctx->depth);
    free_dev(ctx->hair_list);
    free_dev(ctx->hair_count);
    free_dev(ctx->tile_depth);
    ctx->width = ctx->height = ctx->dom_w = ctx->dom_h = 0;
}

struct BufInfo {
    void* ptr;
    size_t bytes;
};

BufInfo buffer_info(hg_ctx* ctx, hg_buffer_id id) {
    size_t px = (size_t)ctx->width * ctx->height;
    size_t texels = (size_t)ctx->dom_w * ctx->dom_h;
    switch (id) {
        case HG_BUF_CENTER: return {ctx->center, px * 8};
        case HG_BUF_CONSERVATIVE: return {ctx->cons, px * 8};
        case HG_BUF_BETA: return {ctx->beta, px * 4};
        case HG_BUF_DOM: return {ctx->dom, texels * (1 + HG_DOM_LAYERS) * 4};
        case HG_BUF_SHADED: return {ctx->shaded, px * 16};
        case HG_BUF_SHADED_DEPTH: return {ctx->shaded_depth, px * 4};
        case HG_BUF_FILTERED: return {ctx->filtered, px * 16};
        case HG_BUF_FILTERED_DEPTH: return {ctx->filtered_depth, px * 4};
        case HG_BUF_COLOR: return {ctx->color, px * 16};
        case HG_BUF_DEPTH: return {ctx->depth, px * 4};
    }
    return {nullptr, 0};
}

hg_status check_targets(hg_ctx* ctx, bool need_dom) {
    if (!ctx->center || ctx->width == 0 || ctx->height == 0)
        return fail(ctx, HG_NOT_READY, "screen targets not allocated (call hg_ensure_targets)");
    if (need_dom && (!ctx->dom || ctx->dom_w == 0 || ctx->dom_h == 0))
        return fail(ctx, HG_NOT_READY, "deep opacity map not allocated (dom size is 0)");
    return HG_OK;
}

// The params' screen must match the targets the pass writes.
hg_status check_screen(hg_ctx* ctx, const hg_hair_params* p) {
    uint32_t mode = p->pass_mode[0];
    if (mode > 2u) return fail(ctx, HG_INVALID_ARG, "pass_mode.x must be 0, 1 or 2");
    if (mode == 0u) {
        if (p->screen[0] != (float)ctx->width || p->screen[1] != (float)ctx->height)
            return fail(ctx, HG_INVALID_ARG, "params.screen.xy differs from the screen targets");
        return check_targets(ctx, false);
    }
    if (p->screen[0] != (float)ctx->dom_w || p->screen[1] != (float)ctx->dom_h ||
        p->dom_info[0] != (float)ctx->dom_w || p->dom_info[1] != (float)ctx->dom_h)
        return fail(ctx, HG_INVALID_ARG, "DOM params screen.xy / dom_info.xy differ from the map size");
    return check_targets(ctx, true);
}

}  // namespace

extern "C" {

uint32_t hg_abi_version(void) { return HG_ABI_VERSION; }

const char* hg_status_string(hg_status s) {
    switch (s) {
        case HG_OK: return "ok";
        case HG_INVALID_ARG: return "invalid argument";
        case HG_OUT_OF_MEMORY: return "out of device memory";
        case HG_CUDA_ERROR: return "CUDA error";
        case HG_CAPACITY_EXCEEDED: return "capacity exceeded";
        case HG_DEVICE_TIMEOUT: return "device timeout";
        case HG_NOT_READY: return "not ready";
        case HG_DEVICE_ERROR: return "device reported an error";
    }
    return "unknown status";
}

const char* hg_last_error(const hg_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

hg_status hg_create(int device, void* stream, hg_ctx** out) {
    if (!out) return HG_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return HG_INVALID_ARG;
    hg_ctx* ctx = new (std::nothrow) hg_ctx();
    if (!ctx) return HG_OUT_OF_MEMORY;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) {
        if (stream) {
            ctx->stream = (cudaStream_t)stream;
        } else {
            e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
            ctx->own_stream = e == cudaSuccess;
        }
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = hg::ensure_shade_setup(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
    for (cudaEvent_t* ev : {&ctx->ev_fork, &ctx->ev_gen, &ctx->ev_join, &ctx->ev_copy_src, &ctx->ev_copy_done})
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->err, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->err, 0, sizeof(uint32_t), ctx->stream);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->lights, sizeof(hg_light) * HG_MAX_LIGHTS);
    if (e == cudaSuccess) {
        ctx->dual_table = new (std::nothrow) hg_dual_table();
        if (!ctx->dual_table) e = cudaErrorMemoryAllocation;
    }
    if (e == cudaSuccess) e = cudaMalloc(&ctx->dual_table->table, sizeof(float4) * hg::kDualTableFloat4);
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->lights_host, sizeof(hg_light) * HG_MAX_LIGHTS * hg_ctx::kLightSlots);
    for (int i = 0; i < hg_ctx::kLightSlots && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&ctx->light_events[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        hg_destroy(ctx);
        return e == cudaErrorMemoryAllocation ? HG_OUT_OF_MEMORY : HG_CUDA_ERROR;
    }
    *out = ctx;
    return HG_OK;
}

hg_status hg_destroy(hg_ctx* ctx) {
    if (!ctx) return HG_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    free_targets(ctx);
    free_dev(ctx->env_spec);
    free_dev(ctx->env_diff);
    free_dev(ctx->err);
    free_dev(ctx->lights);
    if (ctx->dual_table) {
        free_dev(ctx->dual_table->table);
        delete ctx->dual_table;
        ctx->dual_table = nullptr;
    }
    if (ctx->lights_host) cudaFreeHost(ctx->lights_host);
    for (int i = 0; i < hg_ctx::kLightSlots; ++i)
        if (ctx->light_events[i]) cudaEventDestroy(ctx->light_events[i]);
    if (ctx->side) {
        cudaStreamSynchronize(ctx->side);
        cudaStreamDestroy(ctx->side);
    }
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    for (cudaEvent_t ev : {ctx->ev_fork, ctx->ev_gen, ctx->ev_join, ctx->ev_copy_src, ctx->ev_copy_done})
        if (ev) cudaEventDestroy(ev);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return HG_OK;
}

// Texels of a cubemap mip chain: six faces of max(size >> l, 1)^2 per level.
static size_t cube_texels(uint32_t size, uint32_t levels) {
    size_t n = 0;
    for (uint32_t l = 0; l < levels; ++l) {
        const size_t s = std::max<size_t>(size >> l, 1);
        n += 6 * s * s;
    }
    return n;
}

static bool cube_shape_ok(uint32_t size, uint32_t levels) {
    if (size < 1 || size > 4096 || levels < 1) return false;
    uint32_t max_levels = 1;
    while ((size >> max_levels) > 0) ++max_levels;
    return levels <= max_levels;
}

hg_status hg_env_set(hg_ctx* ctx, const hg_env_desc* env) {
    if (!ctx) return HG_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (!env) {
        HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        free_dev(ctx->env_spec);
        free_dev(ctx->env_diff);
        ctx->env_spec_size = ctx->env_spec_levels = ctx->env_diff_size = ctx->env_diff_levels = 0;
        ctx->env_generation += 1;
        return HG_OK;
    }
    if (!env->specular || !env->diffuse) return fail(ctx, HG_INVALID_ARG, "null cubemap texels");
    if (!cube_shape_ok(env->specular_size, env->specular_levels) ||
        !cube_shape_ok(env->diffuse_size, env->diffuse_levels))
        return fail(ctx, HG_INVALID_ARG, "cubemap size must be 1..4096 with 1..1+log2(size) levels");
    for (float v : {env->rotation[0], env->rotation[1], env->rotation[2], env->rotation[3], env->intensity})
        if (!std::isfinite(v)) return fail(ctx, HG_INVALID_ARG, "non-finite probe rotation or intensity");
    HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    free_dev(ctx->env_spec);
    free_dev(ctx->env_diff);
    ctx->env_spec_size = ctx->env_spec_levels = ctx->env_diff_size = ctx->env_diff_levels = 0;
    // the old cubemaps are gone: graphs that captured them must not replay
    ctx->env_generation += 1;
    const size_t ns = cube_texels(env->specular_size, env->specular_levels);
    const size_t nd = cube_texels(env->diffuse_size, env->diffuse_levels);
    HG_CUDA(ctx, cudaMalloc((void**)&ctx->env_spec, ns * 4));
    HG_CUDA(ctx, cudaMalloc((void**)&ctx->env_diff, nd * 4));
    HG_CUDA(ctx, cudaMemcpy(ctx->env_spec, env->specular, ns * 4, cudaMemcpyHostToDevice));
    HG_CUDA(ctx, cudaMemcpy(ctx->env_diff, env->diffuse, nd * 4, cudaMemcpyHostToDevice));
    ctx->env_spec_size = env->specular_size;
    ctx->env_spec_levels = env->specular_levels;
    ctx->env_diff_size = env->diffuse_size;
    ctx->env_diff_levels = env->diffuse_levels;
    std::memcpy(ctx->env_rot, env->rotation, sizeof(ctx->env_rot));
    ctx->env_intensity = env->intensity;
    return HG_OK;
}

hg_status hg_synchronize(hg_ctx* ctx, uint32_t* device_error) {
    if (!ctx) return HG_INVALID_ARG;
    uint32_t word = 0;
    HG_CUDA(ctx, cudaMemcpyAsync(&word, ctx->err, sizeof(word), cudaMemcpyDeviceToHost, ctx->stream));
    HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (device_error) *device_error = word;
    if (word != 0) {
        HG_CUDA(ctx, cudaMemsetAsync(ctx->err, 0, sizeof(uint32_t), ctx->stream));
        return fail(ctx, word & 2u ? HG_DEVICE_TIMEOUT : HG_DEVICE_ERROR,
                    word & 2u ? "a tensor-core wait timed out" : "a kernel reported an invalid strand reference");
    }
    return HG_OK;
}

hg_status hg_ensure_targets(hg_ctx* ctx, uint32_t width, uint32_t height, uint32_t dom_w, uint32_t dom_h) {
    if (!ctx) return HG_INVALID_ARG;
    if (width == 0 || height == 0 || width > 16384 || height > 16384)
        return fail(ctx, HG_INVALID_ARG, "screen size must be 1..16384 per side");
    if (dom_w > 16384 || dom_h > 16384 || (dom_w == 0) != (dom_h == 0))
        return fail(ctx, HG_INVALID_ARG, "DOM size must be 0x0 or 1..16384 per side");
    if (width == ctx->width && height == ctx->height && dom_w == ctx->dom_w && dom_h == ctx->dom_h && ctx->center)
        return HG_OK;
    cudaSetDevice(ctx->device);
    HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    HG_CUDA(ctx, cudaStreamSynchronize(ctx->copy_stream));
    ctx->pending_reads = 0;
    free_targets(ctx);
    size_t px = (size_t)width * height;
    size_t texels = (size_t)dom_w * dom_h;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto*& p, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMalloc((void**)&p, bytes);
    };
    alloc(ctx->center, px * 8);
    alloc(ctx->cons, px * 8);
    alloc(ctx->beta, px * 4);
    alloc(ctx->dom, texels * (1 + HG_DOM_LAYERS) * 4);
    alloc(ctx->shaded, px * 16);
    alloc(ctx->shaded_depth, px * 4);
    alloc(ctx->filtered, px * 16);
    alloc(ctx->filtered_depth, px * 4);
    alloc(ctx->color, px * 16);
    alloc(ctx->depth, px * 4);
    alloc(ctx->hair_list, px * 4);
    alloc(ctx->hair_count, 16);
    alloc(ctx->tile_depth, (size_t)hg::tiles_along(width) * hg::tiles_along(height) * 4);
    if (e != cudaSuccess) {
        free_targets(ctx);
        return cuda_fail(ctx, e, "allocating screen targets");
    }
    ctx->width = width;
    ctx->height = height;
    ctx->dom_w = dom_w;
    ctx->dom_h = dom_h;
    return HG_OK;
}

hg_status hg_buffer(hg_ctx* ctx, hg_buffer_id id, void** device_ptr, size_t* bytes) {
    if (!ctx) return HG_INVALID_ARG;
    if ((unsigned)id > (unsigned)HG_BUF_DEPTH) return fail(ctx, HG_INVALID_ARG, "unknown buffer id");
    BufInfo b = buffer_info(ctx, id);
    if (device_ptr) *device_ptr = b.ptr;
    if (bytes) *bytes = b.bytes;
    return HG_OK;
}

hg_status hg_copy_out(hg_ctx* ctx, hg_buffer_id id, void* host, size_t bytes) {
    if (!ctx || !host) return HG_INVALID_ARG;
    if ((unsigned)id > (unsigned)HG_BUF_DEPTH) return fail(ctx, HG_INVALID_ARG, "unknown buffer id");
    BufInfo b = buffer_info(ctx, id);
    if (!b.ptr || bytes != b.bytes) return fail(ctx, HG_INVALID_ARG, "size differs from the buffer size");
    HG_CUDA(ctx, cudaMemcpyAsync(host, b.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HG_OK;
}

hg_status hg_copy_out_async(hg_ctx* ctx, hg_buffer_id id, void* host, size_t bytes) {
    if (!ctx || !host) return HG_INVALID_ARG;
    if ((unsigned)id > (unsigned)HG_BUF_DEPTH) return fail(ctx, HG_INVALID_ARG, "unknown buffer id");
    BufInfo b = buffer_info(ctx, id);
    if (!b.ptr || bytes != b.bytes) return fail(ctx, HG_INVALID_ARG, "size differs from the buffer size");
    HG_CUDA(ctx, cudaEventRecord(ctx->ev_copy_src, ctx->stream));
    HG_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_copy_src, 0));
    HG_CUDA(ctx, cudaMemcpyAsync(host, b.ptr, bytes, cudaMemcpyDeviceToHost, ctx->copy_stream));
    HG_CUDA(ctx, cudaEventRecord(ctx->ev_copy_done, ctx->copy_stream));
    ctx->pending_reads |= 1u << (unsigned)id;
    return HG_OK;
}

hg_status hg_copy_wait(hg_ctx* ctx) {
    if (!ctx) return HG_INVALID_ARG;
    HG_CUDA(ctx, cudaStreamSynchronize(ctx->copy_stream));
    return HG_OK;
}

hg_status hg_copy_in(hg_ctx* ctx, hg_buffer_id id, const void* host, size_t bytes) {
    if (!ctx || !host) return HG_INVALID_ARG;
    if ((unsigned)id > (unsigned)HG_BUF_DEPTH) return fail(ctx, HG_INVALID_ARG, "unknown buffer id");
    BufInfo b = buffer_info(ctx, id);
    if (!b.ptr || bytes != b.bytes) return fail(ctx, HG_INVALID_ARG, "size differs from the buffer size");
    HG_CUDA(ctx, guard_writes(ctx, 1u << (unsigned)id));
    HG_CUDA(ctx, cudaMemcpyAsync(b.ptr, host, bytes, cudaMemcpyHostToDevice, ctx->stream));
    HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HG_OK;
}

hg_status hg_groom_upload(hg_ctx* ctx, const hg_gpu_bundle* bundles, uint32_t bundle_count, const hg_gpu_layer* layers,
                          uint32_t layer_count, const float* style, uint32_t style_count, hg_groom** out) {
    if (!ctx || !out) return HG_INVALID_ARG;
    *out = nullptr;
    if (bundle_count && (!bundles || !layers || !style))
        return fail(ctx, HG_INVALID_ARG, "null groom array");
    uint64_t strands = 0;
    for (uint32_t b = 0; b < bundle_count; ++b) {
        if ((uint64_t)bundles[b].layer_offset + 64u > layer_count)
            return fail(ctx, HG_INVALID_ARG, "bundle layer_offset + 64 exceeds the layer count");
        if ((uint64_t)bundles[b].style_offset + HG_STYLE_TEXELS > style_count)
            return fail(ctx, HG_INVALID_ARG, "bundle style_offset + 1024 exceeds the style count");
        strands += bundles[b].strand_count;
    }
    if (strands > 0x7fffffffull) return fail(ctx, HG_CAPACITY_EXCEEDED, "more than 2^31 strands in one groom");
    hg_groom* g = new (std::nothrow) hg_groom();
    if (!g) return fail(ctx, HG_OUT_OF_MEMORY, "host allocation");
    g->bundle_count = bundle_count;
    g->layer_count = layer_count;
    g->style_count = style_count;
    g->strand_total = (uint32_t)strands;
    g->ref_capacity = std::max<uint32_t>(g->strand_total, 1u);
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto*& p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc((void**)&p, std::max<size_t>(bytes, 16));
    };
    alloc(g->bundles, (size_t)bundle_count * sizeof(hg_gpu_bundle));
    alloc(g->layers, (size_t)layer_count * sizeof(hg_gpu_layer));
    alloc(g->style, (size_t)style_count * 16);
    for (int s = 0; s < 2; ++s) {
        alloc(g->lod[s], (size_t)std::max<uint32_t>(bundle_count, 1u) * sizeof(hg_lod_record));
        alloc(g->refs[s], (size_t)g->ref_capacity * sizeof(hg_strand_ref));
        alloc(g->indirect[s], 16);
        alloc(g->offsets[s], ((size_t)bundle_count + 1) * 4);
        alloc(g->depth_key[s], (size_t)std::max<uint32_t>(bundle_count, 1u) * 4);
        alloc(g->sorted[s], (size_t)std::max<uint32_t>(bundle_count, 1u) * 4);
        alloc(g->sorted_off[s], ((size_t)bundle_count + 1) * 4);
        alloc(g->draw_order[s], (size_t)g->ref_capacity * 4);
        alloc(g->order_meta[s], 8);
    }
    // Per-strand bundle index and per-bundle first strand, for the strand cache.
    std::vector<uint32_t> base(bundle_count + 1u, 0u), owner(g->strand_total);
    for (uint32_t b = 0; b < bundle_count; ++b) {
        base[b + 1] = base[b] + bundles[b].strand_count;
        for (uint32_t s2 = base[b]; s2 < base[b + 1]; ++s2) owner[s2] = b;
    }
    alloc(g->strand_base, base.size() * 4);
    alloc(g->strand_bundle, (size_t)g->strand_total * 4);
    // The DOM depth pass's order for a full draw (every strand; its refs then
    // sit at base[b] + s): bundles in the order of a multiplicative hash of
    // their index, so that strands drawn at the same time come from bundles
    // far apart and contend less for the same texels.
    std::vector<uint32_t> hashed(bundle_count), dom_order;
    for (uint32_t b = 0; b < bundle_count; ++b) hashed[b] = b;
    std::stable_sort(hashed.begin(), hashed.end(),
                     [](uint32_t x, uint32_t y) { return x * 0x9e3779b1u < y * 0x9e3779b1u; });
    dom_order.reserve(g->strand_total);
    for (uint32_t b : hashed)
        for (uint32_t r = base[b]; r < base[b + 1]; ++r) dom_order.push_back(r);
    alloc(g->dom_order, (size_t)g->strand_total * 4);
    if (e == cudaSuccess && g->strand_total)
        e = cudaMemcpyAsync(g->dom_order, dom_order.data(), dom_order.size() * 4, cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g->strand_base, base.data(), base.size() * 4, cudaMemcpyHostToDevice,
                                              ctx->stream);
    if (e == cudaSuccess && g->strand_total)
        e = cudaMemcpyAsync(g->strand_bundle, owner.data(), owner.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && bundle_count) {
        e = cudaMemcpyAsync(g->bundles, bundles, (size_t)bundle_count * sizeof(hg_gpu_bundle), cudaMemcpyHostToDevice,
                            ctx->stream);
        if (e == cudaSuccess && layer_count)
            e = cudaMemcpyAsync(g->layers, layers, (size_t)layer_count * sizeof(hg_gpu_layer), cudaMemcpyHostToDevice,
                                ctx->stream);
        if (e == cudaSuccess && style_count)
            e = cudaMemcpyAsync(g->style, style, (size_t)style_count * 16, cudaMemcpyHostToDevice, ctx->stream);
    }
    for (int s = 0; s < 2 && e == cudaSuccess; ++s) {
        e = cudaMemsetAsync(g->indirect[s], 0, 16, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(g->lod[s], 0, (size_t)std::max<uint32_t>(bundle_count, 1u) * 16, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(g->order_meta[s], 0, 8, ctx->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        hg_groom_destroy(ctx, g);
        return cuda_fail(ctx, e, "uploading groom");
    }
    *out = g;
    return HG_OK;
}

hg_status hg_groom_destroy(hg_ctx* ctx, hg_groom* g) {
    if (!ctx || !g) return HG_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    free_dev(g->bundles);
    free_dev(g->layers);
    free_dev(g->style);
    free_dev(g->strand_base);
    free_dev(g->strand_bundle);
    free_dev(g->dom_order);
    free_dev(g->cache);
    hg::release_bins(g);
    for (int s = 0; s < 2; ++s) {
        free_dev(g->lod[s]);
        free_dev(g->refs[s]);
        free_dev(g->indirect[s]);
        free_dev(g->offsets[s]);
        free_dev(g->depth_key[s]);
        free_dev(g->sorted[s]);
        free_dev(g->sorted_off[s]);
        free_dev(g->draw_order[s]);
        free_dev(g->order_meta[s]);
    }
    delete g;
    return HG_OK;
}

hg_status hg_groom_buffer(hg_ctx* ctx, hg_groom* g, hg_view_slot slot, hg_groom_buffer_id id, void** device_ptr,
                          size_t* bytes) {
    if (!ctx || !g || (slot != HG_SLOT_CAMERA && slot != HG_SLOT_DOM)) return HG_INVALID_ARG;
    void* p = nullptr;
    size_t n = 0;
    switch (id) {
        case HG_GBUF_LOD: p = g->lod[slot]; n = (size_t)std::max<uint32_t>(g->bundle_count, 1u) * 16; break;
        case HG_GBUF_REFS: p = g->refs[slot]; n = (size_t)g->ref_capacity * 16; break;
        case HG_GBUF_INDIRECT: p = g->indirect[slot]; n = 16; break;
        case HG_GBUF_STRAND_CACHE:
            p = g->cache;
            n = g->cache ? (size_t)g->strand_total * 2u * hg::kStrandCacheCps * sizeof(float4) : 0;
            break;
        default: return fail(ctx, HG_INVALID_ARG, "unknown groom buffer id");
    }
    if (device_ptr) *device_ptr = p;
    if (bytes) *bytes = n;
    return HG_OK;
}

hg_status hg_groom_copy_out(hg_ctx* ctx, hg_groom* g, hg_view_slot slot, hg_groom_buffer_id id, void* host,
                            size_t bytes) {
    if (!ctx || !g || !host) return HG_INVALID_ARG;
    void* p = nullptr;
    size_t n = 0;
    hg_status s = hg_groom_buffer(ctx, g, slot, id, &p, &n);
    if (s != HG_OK) return s;
    if (bytes != n) return fail(ctx, HG_INVALID_ARG, "size differs from the groom buffer size");
    HG_CUDA(ctx, cudaMemcpyAsync(host, p, n, cudaMemcpyDeviceToHost, ctx->stream));
    HG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HG_OK;
}

hg_status hg_clear(hg_ctx* ctx) {
    if (!ctx) return HG_INVALID_ARG;
    hg_status s = check_targets(ctx, false);
    if (s != HG_OK) return s;
    HG_PENDING(ctx);
    HG_CUDA(ctx, guard_writes(ctx, kGbufferBits));
    HG_CUDA(ctx, hg::launch_clear(ctx));
    return HG_OK;
}

hg_status hg_clear_dom(hg_ctx* ctx) {
    if (!ctx) return HG_INVALID_ARG;
    hg_status s = check_targets(ctx, true);
    if (s != HG_OK) return s;
    HG_PENDING(ctx);
    HG_CUDA(ctx, guard_writes(ctx, 1u << HG_BUF_DOM));
    HG_CUDA(ctx, hg::launch_clear_dom(ctx));
    return HG_OK;
}

hg_status hg_lod(hg_ctx* ctx, hg_groom* g, const hg_hair_params* p, hg_view_slot slot) {
    if (!ctx || !g || !p || (slot != HG_SLOT_CAMERA && slot != HG_SLOT_DOM)) return HG_INVALID_ARG;
    HG_PENDING(ctx);
    HG_CUDA(ctx, hg::launch_lod(ctx, g, *p, slot));
    return HG_OK;
}

hg_status hg_scan(hg_ctx* ctx, hg_groom* g, const hg_hair_params* p, hg_view_slot slot) {
    if (!ctx || !g || !p || (slot != HG_SLOT_CAMERA && slot != HG_SLOT_DOM)) return HG_INVALID_ARG;
    HG_PENDING(ctx);
    HG_CUDA(ctx, hg::launch_scan(ctx, g, *p, slot));
    return HG_OK;
}

hg_status hg_generate(hg_ctx* ctx, hg_groom* g, const hg_hair_params* p) {
    if (!ctx || !g || !p) return HG_INVALID_ARG;
    HG_PENDING(ctx);
    if (!g->cache && g->strand_total) {
        cudaSetDevice(ctx->device);
        size_t bytes = (size_t)g->strand_total * 2u * hg::kStrandCacheCps * sizeof(float4);
        HG_CUDA(ctx, cudaMalloc((void**)&g->cache, bytes));
    }
    g->cache_valid = false;
    HG_CUDA(ctx, hg::launch_generate(ctx, g, *p));
    std::memcpy(g->cache_model, p->world_from_model, sizeof(g->cache_model));
    g->cache_valid = true;
    return HG_OK;
}

hg_status hg_raster(hg_ctx* ctx, hg_groom* g, const hg_hair_params* p, hg_view_slot slot, const float* scene_depth) {
    if (!ctx || !g || !p || (slot != HG_SLOT_CAMERA && slot != HG_SLOT_DOM)) return HG_INVALID_ARG;
    hg_status s = check_screen(ctx, p);
    if (s != HG_OK) return s;
    HG_PENDING(ctx);
    HG_CUDA(ctx, guard_writes(ctx, p->pass_mode[0] == 0u ? kGbufferBits : 1u << HG_BUF_DOM));
    HG_CUDA(ctx, hg::launch_raster(ctx, g, *p, slot, p->pass_mode[0] == 0u ? scene_depth : nullptr));
    return HG_OK;
}

hg_status hg_set_camera_raster(hg_ctx* ctx, uint32_t mode) {
    if (!ctx) return HG_INVALID_ARG;
    if (mode != HG_CAMERA_RASTER_DIRECT && mode != HG_CAMERA_RASTER_BINNED)
        return fail(ctx, HG_INVALID_ARG, "camera raster mode must be HG_CAMERA_RASTER_DIRECT or _BINNED");
    ctx->camera_raster = mode;
    return HG_OK;
}

hg_status hg_shade(hg_ctx* ctx, const hg_hair_params* p, const hg_shade_desc* d) {
    if (!ctx || !p || !d) return HG_INVALID_ARG;
    if (d->light_count > HG_MAX_LIGHTS) return fail(ctx, HG_CAPACITY_EXCEEDED, "more than HG_MAX_LIGHTS lights");
    if (d->light_count && !d->lights) return fail(ctx, HG_INVALID_ARG, "null light array");
    if (d->shade_model > 3u) return fail(ctx, HG_INVALID_ARG, "unknown shade model");
    if (d->shade_model != 0u && !ctx->surrogate)
        return fail(ctx, HG_NOT_READY, "shade models 1 to 3 need a surrogate bound with hg_mlp_bind");
    if (d->shade_model != 0u &&
        ctx->surrogate->arch != (d->shade_model == 3u ? HG_MLP_ARCH_COMPACT : HG_MLP_ARCH_DEEP))
        return fail(ctx, HG_INVALID_ARG, "shade models 1 and 2 take the 4 x 64 surrogate, model 3 the compact one");
    hg_status s = check_screen(ctx, p);
    if (s != HG_OK) return s;
    if (p->pass_mode[0] != 0u) return fail(ctx, HG_INVALID_ARG, "shade takes the camera params (pass_mode.x == 0)");
    if (p->flags[3] && !ctx->dom) return fail(ctx, HG_NOT_READY, "deep opacity enabled without a map");
    if (p->flags[3] && (p->dom_info[0] != (float)ctx->dom_w || p->dom_info[1] != (float)ctx->dom_h))
        return fail(ctx, HG_INVALID_ARG, "camera params dom_info.xy differ from the map size");
    HG_PENDING(ctx);
    // Stable order by kind: point, spot, directional, rect (shade.wesl:452-518).
    uint32_t n = 0;
    for (uint32_t i = 0; i < d->light_count; ++i)
        if (d->lights[i].kind > HG_LIGHT_RECT) return fail(ctx, HG_INVALID_ARG, "unknown light kind");
    if (d->light_count) {
        const int slot = ctx->light_slot;
        ctx->light_slot = (slot + 1) % hg_ctx::kLightSlots;
        HG_CUDA(ctx, cudaEventSynchronize(ctx->light_events[slot]));
        hg_light* staging = ctx->lights_host + (size_t)slot * HG_MAX_LIGHTS;
        for (uint32_t kind = 0; kind < 4u; ++kind)
            for (uint32_t i = 0; i < d->light_count; ++i)
                if (d->lights[i].kind == kind) staging[n++] = d->lights[i];
        HG_CUDA(ctx, cudaMemcpyAsync(ctx->lights, staging, n * sizeof(hg_light), cudaMemcpyHostToDevice, ctx->stream));
        HG_CUDA(ctx, cudaEventRecord(ctx->light_events[slot], ctx->stream));
    }
    HG_CUDA(ctx, guard_writes(ctx, 1u << HG_BUF_SHADED | 1u << HG_BUF_SHADED_DEPTH));
    HG_CUDA(ctx, hg::launch_shade(ctx, *p, n, d->ortho, d->exposure, d->shade_model));
    return HG_OK;
}

hg_status hg_filter(hg_ctx* ctx, const hg_hair_params* p) {
    if (!ctx || !p) return HG_INVALID_ARG;
    hg_status s = check_screen(ctx, p);
    if (s != HG_OK) return s;
    HG_PENDING(ctx);
    HG_CUDA(ctx, guard_writes(ctx, 1u << HG_BUF_FILTERED | 1u << HG_BUF_FILTERED_DEPTH));
    HG_CUDA(ctx, hg::launch_filter(ctx, *p));
    return HG_OK;
}

hg_status hg_composite(hg_ctx* ctx, const hg_hair_params* p, uint32_t source_filtered) {
    if (!ctx || !p) return HG_INVALID_ARG;
    hg_status s = check_screen(ctx, p);
    if (s != HG_OK) return s;
    HG_PENDING(ctx);
    HG_CUDA(ctx, guard_writes(ctx, kColorBits));
    HG_CUDA(ctx, hg::launch_composite(ctx, *p, source_filtered));
    return HG_OK;
}

hg_status hg_clear_color(hg_ctx* ctx, float depth_clear) {
    if (!ctx) return HG_INVALID_ARG;
    hg_status s = check_targets(ctx, false);
    if (s != HG_OK) return s;
    HG_PENDING(ctx);
    HG_CUDA(ctx, guard_writes(ctx, kColorBits));
    HG_CUDA(ctx, hg::launch_clear_color(ctx, depth_clear));
    return HG_OK;
}

hg_status hg_shadow_light_from(const hg_hair_params* dom, hg_shadow_light* out) {
    if (!dom || !out) return HG_INVALID_ARG;
    if (dom->pass_mode[0] != 1u && dom->pass_mode[0] != 2u) return HG_INVALID_ARG;
    // src/render/pass.rs:574-579: the light clip matrix, eye (w 1), forward
    // (w 0), and (near, far, DOM_SIGMA, 1); DOM_SIGMA travels in filter_params.w.
    std::memcpy(out->light_clip_from_world, dom->light_clip_from_world, sizeof(out->light_clip_from_world));
    for (int i = 0; i < 3; ++i) {
        out->light_eye[i] = dom->light_eye[i];
        out->light_forward[i] = dom->light_forward[i];
    }
    out->light_eye[3] = 1.0f;
    out->light_forward[3] = 0.0f;
    out->depth[0] = dom->dom_info[2];
    out->depth[1] = dom->dom_info[3];
    out->depth[2] = dom->filter_params[3];
    out->depth[3] = 1.0f;
    return HG_OK;
}

hg_status hg_hair_visibility(hg_ctx* ctx, const hg_shadow_light* light, const float* points, uint32_t n,
                             float* visibility) {
    if (!ctx || !light || (n && (!points || !visibility))) return HG_INVALID_ARG;
    hg_status s = check_targets(ctx, true);
    if (s != HG_OK) return s;
    HG_PENDING(ctx);
    HG_CUDA(ctx, hg::launch_visibility(ctx, *light, points, n, visibility));
    return HG_OK;
}

// hair_pass per-groom body (src/render/pass.rs:375-643).
hg_status hg_groom_frame(hg_ctx* ctx, hg_groom* g, const hg_frame_desc* d) {
    if (!ctx || !g || !d || !d->camera) return HG_INVALID_ARG;
    const hg_hair_params& cam = *d->camera;
    if (cam.pass_mode[0] != 0u) return fail(ctx, HG_INVALID_ARG, "camera params need pass_mode.x == 0");
    const bool dom = cam.flags[3] != 0u;
    if (dom && (!d->dom || d->dom->pass_mode[0] != 1u))
        return fail(ctx, HG_INVALID_ARG, "deep opacity needs DOM params with pass_mode.x == 1");
    // The camera and deep-opacity halves of the frame are independent until
    // shading, so the DOM half (and the colour-target clear) runs on the
    // context's side stream, forked from and joined back into the main stream
    // with events: work before and after the frame stays ordered on the main
    // stream.
    const cudaStream_t main_stream = ctx->stream;
    struct Restore {
        hg_ctx* c;
        cudaStream_t st;
        ~Restore() { c->stream = st; }
    } restore{ctx, main_stream};
    auto on = [&](cudaStream_t st) { ctx->stream = st; };
    HG_CUDA(ctx, cudaEventRecord(ctx->ev_fork, main_stream));
    HG_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
    hg_status s;
    // main: camera setup, then (with the DOM on) the strand cache: every strand
    // is drawn at full detail at least once, so each is generated once and the
    // camera and DOM rasters read it.
    on(main_stream);
    if ((s = hg_clear(ctx)) != HG_OK) return s;
    if ((s = hg_lod(ctx, g, &cam, HG_SLOT_CAMERA)) != HG_OK) return s;
    if ((s = hg_scan(ctx, g, &cam, HG_SLOT_CAMERA)) != HG_OK) return s;
    if (dom) {
        if ((s = hg_generate(ctx, g, &cam)) != HG_OK) return s;
        HG_CUDA(ctx, cudaEventRecord(ctx->ev_gen, main_stream));
    }
    // side: DOM setup, the two DOM rasters after the cache, colour clear
    on(ctx->side);
    if (dom) {
        hg_hair_params layers_params = *d->dom;
        layers_params.pass_mode[0] = 2u;
        if ((s = hg_clear_dom(ctx)) != HG_OK) return s;
        if ((s = hg_lod(ctx, g, d->dom, HG_SLOT_DOM)) != HG_OK) return s;
        if ((s = hg_scan(ctx, g, d->dom, HG_SLOT_DOM)) != HG_OK) return s;
        HG_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_gen, 0));
        if ((s = hg_raster(ctx, g, d->dom, HG_SLOT_DOM, nullptr)) != HG_OK) return s;
        if ((s = hg_raster(ctx, g, &layers_params, HG_SLOT_DOM, nullptr)) != HG_OK) return s;
    }
    if (d->composite && d->clear_color &&
        (s = hg_clear_color(ctx, cam.pass_mode[2] == 1u ? 0.0f : 1.0f)) != HG_OK)
        return s;
    HG_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->side));
    // main: camera raster, join, shade, filter, composite
    on(main_stream);
    if ((s = hg_raster(ctx, g, &cam, HG_SLOT_CAMERA, d->scene_depth)) != HG_OK) return s;
    HG_CUDA(ctx, cudaStreamWaitEvent(main_stream, ctx->ev_join, 0));
    if ((s = hg_shade(ctx, &cam, &d->shade)) != HG_OK) return s;
    const bool filter = cam.flags[1] != 0u;
    if (filter && (s = hg_filter(ctx, &cam)) != HG_OK) return s;
    if (d->composite && (s = hg_composite(ctx, &cam, filter ? 1u : 0u)) != HG_OK) return s;
    return HG_OK;
}

}  // extern "C"
