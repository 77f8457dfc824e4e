// Batched frames: many (groom, camera view, deep-opacity view) items drawn
// with one launch per pass, captured into a CUDA graph; the per-groom path
// for comparison; and the launch-shape autotuner.  The reference records one
// hair_pass per groom (src/render/pass.rs:259-657); this has no counterpart
// there.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/hairgb.h"
#include "hg_internal.h"

struct hg_batch {
    hg_ctx* ctx = nullptr;
    uint32_t n = 0, n_dom = 0;
    std::vector<hg_groom*> grooms;
    std::vector<uint32_t> w, h, dw, dh;
    std::vector<uint64_t> px_off, dom_off;   // per item, in pixels / words
    std::vector<hg_hair_params> cam, dom;    // host copies of the uniforms
    std::vector<uint8_t> have;
    // arenas
    unsigned long long* center = nullptr;
    unsigned long long* cons = nullptr;
    uint32_t* beta = nullptr;
    uint32_t* dommap = nullptr;
    float4* shaded = nullptr;
    float* shaded_depth = nullptr;
    float4* filtered = nullptr;
    float* filtered_depth = nullptr;
    float4* color = nullptr;
    float* depth = nullptr;
    // Scratch of the per-groom (HG_BATCH_SEPARATE) frames, which run one after
    // another on the context's stream: sized for the largest item.
    uint32_t* tile_depth = nullptr;
    uint32_t* hair_list = nullptr;
    // 8x8 tile depths of every camera view (the batched two-stage raster)
    uint32_t* tdepth = nullptr;
    uint32_t* hair_count = nullptr;
    uint64_t total_px = 0, total_dom = 0;
    // tables: pinned host copies and their device twins
    hg::BatchView* h_views = nullptr;
    hg::BatchView* d_views = nullptr;
    uint32_t* h_tab = nullptr;
    uint32_t* d_tab = nullptr;
    size_t tab_words = 0;
    hg_light* h_lights = nullptr;
    hg_light* d_lights = nullptr;
    uint32_t* d_counters = nullptr;
    hg::BatchDev dev;
    uint32_t raster_per_sm_max = 1, gen_per_sm = 1;
    hg_batch_tuning tuning{4u, 0u, 32u, 8u, 0u, 0.0f};
    // graph
    // The frame is two graphs: the passes up to shading, then filter + colour
    // clear + composite, so a wait for the previous frame's asynchronous
    // readback of the colour/depth arenas can sit between them.
    cudaGraph_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    bool graph_valid = false;
    bool pending_reads = false;  // an hg_batch_copy_out_async not yet waited for by a frame
    // The pinned tables are rebuilt at frame time (set_params only marks them
    // dirty) and uploaded ahead of the frame's kernels; `uploaded` follows the
    // last upload, so the host may rewrite them while that frame still runs.
    bool tables_dirty = true;
    cudaEvent_t uploaded = nullptr;
    uint32_t g_lights = 0, g_ortho = 0;
    float g_exposure = 0.0f;
    uint64_t g_env = 0;  // ctx->env_generation the graphs were captured at
    cudaEvent_t done = nullptr;
};

namespace {

hg_status fail(hg_ctx* ctx, hg_status s, const char* msg) {
    if (ctx) ctx->last_error = msg;
    return s;
}

hg_status cuda_fail(hg_ctx* ctx, cudaError_t e, const char* where) {
    if (ctx) ctx->last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? HG_OUT_OF_MEMORY : HG_CUDA_ERROR;
}

#define BATCH_CUDA(ctx, expr)                                    \
    do {                                                         \
        cudaError_t e_ = (expr);                                 \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #expr); \
    } while (0)

template <typename T>
void free_dev(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

uint64_t round_up64(uint64_t v) { return (v + 63u) & ~uint64_t(63u); }

// Table layout in h_tab / d_tab (u32): bundle prefix (n_views + 1), strand
// prefix (n + 1), tile prefix (n + 1), filter-tile prefix (n + 1), DOM word
// prefix (n + 1).
struct TabOffsets {
    size_t bundle, strand, tile, ftile, dom, tdepth, total;
};

TabOffsets tab_offsets(uint32_t n, uint32_t n_views) {
    TabOffsets t;
    t.bundle = 0;
    t.strand = t.bundle + n_views + 1;
    t.tile = t.strand + n + 1;
    t.ftile = t.tile + n + 1;
    t.dom = t.ftile + n + 1;
    t.tdepth = t.dom + n + 1;
    t.total = t.tdepth + n + 1;
    return t;
}

// Tile-depth words of a w x h camera view.
uint32_t tdepth_tiles(uint32_t w, uint32_t h) { return hg::tiles_along(w) * hg::tiles_along(h); }

void free_batch(hg_batch* b) {
    if (b->ctx && b->ctx->copy_stream) cudaStreamSynchronize(b->ctx->copy_stream);
    for (int k = 0; k < 2; ++k) {
        if (b->exec[k]) cudaGraphExecDestroy(b->exec[k]);
        if (b->graph[k]) cudaGraphDestroy(b->graph[k]);
    }
    free_dev(b->center);
    free_dev(b->cons);
    free_dev(b->beta);
    free_dev(b->dommap);
    free_dev(b->shaded);
    free_dev(b->shaded_depth);
    free_dev(b->filtered);
    free_dev(b->filtered_depth);
    free_dev(b->color);
    free_dev(b->depth);
    free_dev(b->tile_depth);
    free_dev(b->tdepth);
    free_dev(b->hair_list);
    free_dev(b->hair_count);
    free_dev(b->d_views);
    free_dev(b->d_tab);
    free_dev(b->d_lights);
    free_dev(b->d_counters);
    if (b->h_views) cudaFreeHost(b->h_views);
    if (b->h_tab) cudaFreeHost(b->h_tab);
    if (b->h_lights) cudaFreeHost(b->h_lights);
    if (b->done) cudaEventDestroy(b->done);
    if (b->uploaded) cudaEventDestroy(b->uploaded);
    delete b;
}

// The view table and the prefix tables from the host uniforms and the tuning.
void build_tables(hg_batch* b) {
    const uint32_t n = b->n, n_views = n + b->n_dom;
    const TabOffsets to = tab_offsets(n, n_views);
    hg_ctx* ctx = b->ctx;
    uint32_t dv = n;
    for (uint32_t i = 0; i < n; ++i) {
        hg_groom* g = b->grooms[i];
        for (int slot = 0; slot < 2; ++slot) {
            if (slot == 1 && b->dw[i] == 0) continue;
            hg::BatchView& v = b->h_views[slot == 0 ? i : dv++];
            std::memset(&v, 0, sizeof(v));
            v.p = slot == 0 ? b->cam[i] : b->dom[i];
            v.bundles = g->bundles;
            v.layers = g->layers;
            v.style = g->style;
            v.lod = g->lod[slot];
            v.depth_key = g->depth_key[slot];
            v.offsets = g->offsets[slot];
            v.indirect = g->indirect[slot];
            v.refs = g->refs[slot];
            if (slot == 0) {
                v.sorted = g->sorted[0];
                v.sorted_off = g->sorted_off[0];
                v.draw_order = g->draw_order[0];
                v.order_meta = g->order_meta[0];
                v.tiles_x = hg::tiles_along(b->w[i]);
            }
            v.cache = g->cache;
            v.strand_base = g->strand_base;
            v.strand_bundle = g->strand_bundle;
            const uint64_t po = b->px_off[i];
            v.center = b->center + po;
            v.cons = b->cons + po;
            v.beta = b->beta + po;
            v.dom = b->dw[i] ? b->dommap + b->dom_off[i] : nullptr;
            v.shaded = b->shaded + po;
            v.shaded_depth = b->shaded_depth + po;
            v.filtered = b->filtered + po;
            v.filtered_depth = b->filtered_depth + po;
            v.color = b->color + po;
            v.depth = b->depth + po;
            v.scene = nullptr;
            v.err = ctx->err;
            v.bundle_count = g->bundle_count;
            v.count = std::min(v.p.pass_mode[1], g->bundle_count);
            v.capacity = g->ref_capacity;
            v.strands = g->strand_total;
            v.width = slot == 0 ? b->w[i] : b->dw[i];
            v.height = slot == 0 ? b->h[i] : b->dh[i];
            v.dom_w = b->dw[i];
            v.dom_h = b->dh[i];
        }
    }
    uint32_t* t = b->h_tab;
    t[to.bundle] = 0;
    for (uint32_t v = 0; v < n_views; ++v) t[to.bundle + v + 1] = t[to.bundle + v] + b->h_views[v].count;
    const uint32_t tw = b->tuning.tile_w, th = b->tuning.tile_h;
    const uint32_t fx = b->tuning.filter_tile == 1 ? 16u : 32u, fy = b->tuning.filter_tile == 1 ? 16u : 8u;
    t[to.strand] = t[to.tile] = t[to.ftile] = t[to.dom] = t[to.tdepth] = 0;
    for (uint32_t i = 0; i < n; ++i) {
        t[to.tdepth + i + 1] = t[to.tdepth + i] + tdepth_tiles(b->w[i], b->h[i]);
        b->h_views[i].tile_depth = b->tdepth + t[to.tdepth + i];
        t[to.strand + i + 1] = t[to.strand + i] + b->grooms[i]->strand_total;
        t[to.tile + i + 1] = t[to.tile + i] + ((b->w[i] + tw - 1) / tw) * ((b->h[i] + th - 1) / th);
        t[to.ftile + i + 1] = t[to.ftile + i] + ((b->w[i] + fx - 1) / fx) * ((b->h[i] + fy - 1) / fy);
        t[to.dom + i] = (uint32_t)b->dom_off[i];  // below 2^32 (checked at creation)
    }
    t[to.dom + n] = (uint32_t)b->total_dom;
    hg::BatchDev& d = b->dev;
    d.views = b->d_views;
    d.n_views = n_views;
    d.n_cam = n;
    d.bundle_prefix = b->d_tab + to.bundle;
    d.strand_prefix = b->d_tab + to.strand;
    d.tile_prefix = b->d_tab + to.tile;
    d.ftile_prefix = b->d_tab + to.ftile;
    d.dom_prefix = b->d_tab + to.dom;
    d.tdepth_prefix = b->d_tab + to.tdepth;
    d.total_tdepth = t[to.tdepth + n];
    d.total_bundles = t[to.bundle + n_views];
    d.total_strands = t[to.strand + n];
    d.total_tiles = t[to.tile + n];
    d.total_ftiles = t[to.ftile + n];
    d.total_px = b->total_px;
    d.total_dom_words = b->total_dom;
    d.center = b->center;
    d.cons = b->cons;
    d.beta = b->beta;
    d.dom = b->dommap;
    d.color = b->color;
    d.depth = b->depth;
    d.counters = b->d_counters;
    d.lights = b->d_lights;
    d.filter = b->cam[0].flags[1] != 0u;
    d.composite = 1;
    d.depth_clear = b->cam[0].pass_mode[2] == 1u ? 0.0f : 1.0f;
    d.gen_blocks = (uint32_t)ctx->sm_count * b->gen_per_sm;
    d.raster_chunk = b->tuning.raster_chunk;
    d.raster_blocks_per_sm = b->tuning.raster_blocks_per_sm ? b->tuning.raster_blocks_per_sm : b->raster_per_sm_max;
    d.tile_w = tw;
    d.tile_h = th;
    d.filter_tile = b->tuning.filter_tile;
}

// Uploads and the batched passes, on ctx->stream (captured or direct).
// The view table, prefix tables and light list, pinned host -> device, on the
// work stream ahead of the frame's kernels.
cudaError_t upload_tables(hg_batch* b) {
    hg_ctx* ctx = b->ctx;
    const uint32_t n_views = b->n + b->n_dom;
    cudaError_t e = cudaMemcpyAsync(b->d_views, b->h_views, sizeof(hg::BatchView) * n_views, cudaMemcpyHostToDevice,
                                    ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_tab, b->h_tab, sizeof(uint32_t) * b->tab_words, cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e == cudaSuccess && b->dev.n_lights)
        e = cudaMemcpyAsync(b->d_lights, b->h_lights, sizeof(hg_light) * b->dev.n_lights, cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->uploaded, ctx->stream);
    return e;
}

// Part 0 of a frame: setup, raster, shade.  Part 1: filter, colour clear,
// composite (the only writers of the colour/depth arenas).
cudaError_t enqueue_part(hg_batch* b, int part) {
    hg_ctx* ctx = b->ctx;
    if (part == 1) return hg::launch_batch_filter_composite(ctx, b->dev);
    cudaError_t e = hg::launch_batch_setup(ctx, b->dev);
    if (e == cudaSuccess) e = hg::launch_batch_raster(ctx, b->dev);
    if (e == cudaSuccess) e = hg::launch_batch_shade(ctx, b->dev);
    return e;
}

// Rebuilds the pinned tables after set_params; the caller has waited for the
// last upload.  The graphs hold the launch sizes, so a change of them (bundle
// totals, filter flag, depth convention) forces a new capture.
void refresh_tables(hg_batch* b) {
    if (!b->tables_dirty) return;
    const hg::BatchDev before = b->dev;
    build_tables(b);
    const hg::BatchDev& d = b->dev;
    if (d.total_bundles != before.total_bundles || d.filter != before.filter || d.depth_clear != before.depth_clear)
        b->graph_valid = false;
    b->tables_dirty = false;
}

// Orders part 1 after any pending asynchronous readback of the arenas.
cudaError_t guard_readback(hg_batch* b) {
    if (!b->pending_reads) return cudaSuccess;
    cudaError_t e = cudaStreamWaitEvent(b->ctx->stream, b->ctx->ev_copy_done, 0);
    if (e == cudaSuccess) b->pending_reads = false;
    return e;
}

cudaError_t enqueue_frame(hg_batch* b) {
    cudaError_t e = upload_tables(b);
    if (e == cudaSuccess) e = enqueue_part(b, 0);
    if (e == cudaSuccess) e = guard_readback(b);
    if (e == cudaSuccess) e = enqueue_part(b, 1);
    return e;
}

hg_status capture(hg_batch* b) {
    hg_ctx* ctx = b->ctx;
    b->graph_valid = false;
    for (int k = 0; k < 2; ++k) {
        if (b->exec[k]) cudaGraphExecDestroy(b->exec[k]);
        if (b->graph[k]) cudaGraphDestroy(b->graph[k]);
        b->exec[k] = nullptr;
        b->graph[k] = nullptr;
    }
    for (int k = 0; k < 2; ++k) {
        BATCH_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = enqueue_part(b, k);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
        if (e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(ctx, e, "capturing the batched frame");
        }
        if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "ending the capture");
        b->graph[k] = g;
        BATCH_CUDA(ctx, cudaGraphInstantiate(&b->exec[k], g, 0));
    }
    b->graph_valid = true;
    b->g_lights = b->dev.n_lights;
    b->g_ortho = b->dev.ortho;
    b->g_exposure = b->dev.exposure;
    b->g_env = ctx->env_generation;
    return HG_OK;
}

// Every batched frame (graph or direct launches) regenerates each item's
// strand cache with the item's camera transform; the per-groom passes trust
// the cache when its recorded transform matches theirs.  Before the batched
// kernels are enqueued the caches are marked stale (a failed enqueue may
// leave them half written), and once the frame is enqueued the transform is
// recorded.
void invalidate_caches(hg_batch* b) {
    for (uint32_t i = 0; i < b->n; ++i) b->grooms[i]->cache_valid = false;
}

void note_cache_writes(hg_batch* b) {
    for (uint32_t i = 0; i < b->n; ++i) {
        hg_groom* g = b->grooms[i];
        if (!g->cache) continue;
        std::memcpy(g->cache_model, b->cam[i].world_from_model, sizeof(g->cache_model));
        g->cache_valid = true;
    }
}

cudaError_t launch_graphs(hg_batch* b) {
    cudaError_t e = cudaGraphLaunch(b->exec[0], b->ctx->stream);
    if (e == cudaSuccess) e = guard_readback(b);
    if (e == cudaSuccess) e = cudaGraphLaunch(b->exec[1], b->ctx->stream);
    return e;
}

// Lights sorted by kind into the pinned staging copy (what hg_shade does).
hg_status stage_lights(hg_batch* b, const hg_shade_desc* d) {
    hg_ctx* ctx = b->ctx;
    if (d->light_count > HG_MAX_LIGHTS) return fail(ctx, HG_CAPACITY_EXCEEDED, "more than HG_MAX_LIGHTS lights");
    if (d->light_count && !d->lights) return fail(ctx, HG_INVALID_ARG, "null light array");
    if (d->shade_model != 0u) return fail(ctx, HG_INVALID_ARG, "batched frames shade with model 0");
    uint32_t n = 0;
    for (uint32_t i = 0; i < d->light_count; ++i)
        if (d->lights[i].kind > HG_LIGHT_RECT) return fail(ctx, HG_INVALID_ARG, "unknown light kind");
    for (uint32_t kind = 0; kind < 4u; ++kind)
        for (uint32_t i = 0; i < d->light_count; ++i)
            if (d->lights[i].kind == kind) b->h_lights[n++] = d->lights[i];
    b->dev.n_lights = n;
    b->dev.ortho = d->ortho;
    b->dev.exposure = d->exposure;
    return HG_OK;
}

bool ready(const hg_batch* b) {
    for (uint32_t i = 0; i < b->n; ++i)
        if (!b->have[i]) return false;
    return true;
}

hg_status run_separate(hg_batch* b, const hg_shade_desc* d) {
    hg_ctx* ctx = b->ctx;
    for (uint32_t i = 0; i < b->n; ++i) {
        // A context that shares the real one's stream, events and light
        // staging but whose targets are this item's slices of the arenas.
        hg_ctx view = *ctx;
        const uint64_t po = b->px_off[i];
        view.width = b->w[i];
        view.height = b->h[i];
        view.dom_w = b->dw[i];
        view.dom_h = b->dh[i];
        view.center = b->center + po;
        view.cons = b->cons + po;
        view.beta = b->beta + po;
        view.dom = b->dw[i] ? b->dommap + b->dom_off[i] : nullptr;
        view.shaded = b->shaded + po;
        view.shaded_depth = b->shaded_depth + po;
        view.filtered = b->filtered + po;
        view.filtered_depth = b->filtered_depth + po;
        view.color = b->color + po;
        view.depth = b->depth + po;
        view.tile_depth = b->tile_depth;
        view.hair_list = b->hair_list;
        view.hair_count = b->hair_count;
        view.pending_reads = 0;  // the batch's arenas are never read back asynchronously
        hg_frame_desc f;
        std::memset(&f, 0, sizeof(f));
        f.camera = &b->cam[i];
        f.dom = b->dw[i] ? &b->dom[i] : nullptr;
        f.scene_depth = nullptr;
        f.shade = *d;
        f.composite = 1;
        f.clear_color = 1;
        hg_status s = hg_groom_frame(&view, b->grooms[i], &f);
        ctx->light_slot = view.light_slot;
        if (s != HG_OK) {
            ctx->last_error = view.last_error;
            return s;
        }
    }
    return HG_OK;
}

hg_status check_tuning(hg_batch* b, const hg_batch_tuning* t) {
    hg_ctx* ctx = b->ctx;
    if (t->raster_chunk < 1 || t->raster_chunk > 64) return fail(ctx, HG_INVALID_ARG, "raster_chunk must be 1..64");
    if (t->raster_blocks_per_sm > b->raster_per_sm_max)
        return fail(ctx, HG_INVALID_ARG, "raster_blocks_per_sm above the resident limit");
    if (!((t->tile_w == 16 || t->tile_w == 32 || t->tile_w == 64) && t->tile_w * t->tile_h == 256))
        return fail(ctx, HG_INVALID_ARG, "tile must be 16x16, 32x8 or 64x4");
    if (t->filter_tile > 1) return fail(ctx, HG_INVALID_ARG, "filter_tile must be 0 or 1");
    return HG_OK;
}

float time_graph(hg_batch* b, int warm, int reps, cudaError_t* err) {
    hg_ctx* ctx = b->ctx;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    *err = cudaEventCreate(&e0);
    if (*err == cudaSuccess) *err = cudaEventCreate(&e1);
    for (int i = 0; i < warm && *err == cudaSuccess; ++i) *err = launch_graphs(b);
    if (*err == cudaSuccess) *err = cudaEventRecord(e0, ctx->stream);
    for (int i = 0; i < reps && *err == cudaSuccess; ++i) *err = launch_graphs(b);
    if (*err == cudaSuccess) *err = cudaEventRecord(e1, ctx->stream);
    if (*err == cudaSuccess) *err = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (*err == cudaSuccess) *err = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return ms / (float)std::max(reps, 1);
}

}  // namespace

extern "C" {

hg_status hg_batch_create(hg_ctx* ctx, const hg_batch_item* items, uint32_t count, hg_batch** out) {
    if (!ctx || !out) return HG_INVALID_ARG;
    *out = nullptr;
    if (!items || count == 0 || count > HG_BATCH_MAX_ITEMS)
        return fail(ctx, HG_INVALID_ARG, "a batch holds 1..HG_BATCH_MAX_ITEMS items");
    for (uint32_t i = 0; i < count; ++i) {
        const hg_batch_item& it = items[i];
        if (!it.groom) return fail(ctx, HG_INVALID_ARG, "null groom in batch");
        for (uint32_t j = 0; j < i; ++j)
            if (items[j].groom == it.groom) return fail(ctx, HG_INVALID_ARG, "a groom appears in two batch items");
        if (it.width == 0 || it.height == 0 || it.width > 16384 || it.height > 16384)
            return fail(ctx, HG_INVALID_ARG, "item screen size must be 1..16384 per side");
        if (it.dom_w > 16384 || it.dom_h > 16384 || (it.dom_w == 0) != (it.dom_h == 0))
            return fail(ctx, HG_INVALID_ARG, "item DOM size must be 0x0 or 1..16384 per side");
    }
    cudaSetDevice(ctx->device);
    hg_batch* b = new (std::nothrow) hg_batch();
    if (!b) return fail(ctx, HG_OUT_OF_MEMORY, "allocating the batch");
    b->ctx = ctx;
    b->n = count;
    uint64_t px = 0, words = 0;
    for (uint32_t i = 0; i < count; ++i) {
        b->grooms.push_back(items[i].groom);
        b->w.push_back(items[i].width);
        b->h.push_back(items[i].height);
        b->dw.push_back(items[i].dom_w);
        b->dh.push_back(items[i].dom_h);
        b->px_off.push_back(px);
        b->dom_off.push_back(words);
        // Slices start on 64-element boundaries: the single-view kernels that
        // the per-groom path runs on them use 16-byte vector stores.
        px += round_up64((uint64_t)items[i].width * items[i].height);
        words += round_up64((uint64_t)items[i].dom_w * items[i].dom_h * (1 + HG_DOM_LAYERS));
        if (items[i].dom_w) b->n_dom += 1;
    }
    if (words >= (1ull << 32)) {
        free_batch(b);
        return fail(ctx, HG_CAPACITY_EXCEEDED, "the batch's deep opacity maps exceed 2^32 words");
    }
    b->total_px = px;
    b->total_dom = words;
    b->cam.resize(count);
    b->dom.resize(count);
    b->have.assign(count, 0);
    const uint32_t n_views = count + b->n_dom;
    const TabOffsets to = tab_offsets(count, n_views);
    b->tab_words = to.total;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto*& p, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMalloc((void**)&p, bytes);
    };
    alloc(b->center, px * 8);
    alloc(b->cons, px * 8);
    alloc(b->beta, px * 4);
    alloc(b->dommap, words * 4);
    alloc(b->shaded, px * 16);
    alloc(b->shaded_depth, px * 4);
    alloc(b->filtered, px * 16);
    alloc(b->filtered_depth, px * 4);
    alloc(b->color, px * 16);
    alloc(b->depth, px * 4);
    size_t max_px = 0, max_tiles = 0;
    for (uint32_t i = 0; i < count; ++i) {
        max_px = std::max(max_px, (size_t)b->w[i] * b->h[i]);
        max_tiles = std::max(max_tiles, (size_t)tdepth_tiles(b->w[i], b->h[i]));
    }
    alloc(b->tile_depth, max_tiles * 4);
    uint64_t tdepth_words = 0;
    for (uint32_t i = 0; i < count; ++i) tdepth_words += tdepth_tiles(b->w[i], b->h[i]);
    alloc(b->tdepth, tdepth_words * 4);
    alloc(b->hair_list, max_px * 4);
    alloc(b->hair_count, 16);
    alloc(b->d_views, sizeof(hg::BatchView) * n_views);
    alloc(b->d_tab, sizeof(uint32_t) * to.total);
    alloc(b->d_lights, sizeof(hg_light) * HG_MAX_LIGHTS);
    alloc(b->d_counters, sizeof(uint32_t) * 3);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_views, sizeof(hg::BatchView) * n_views);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_tab, sizeof(uint32_t) * to.total);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_lights, sizeof(hg_light) * HG_MAX_LIGHTS);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->uploaded, cudaEventDisableTiming);
    // every groom's strand cache (the batched camera and DOM rasters read it)
    for (uint32_t i = 0; i < count && e == cudaSuccess; ++i) {
        hg_groom* g = items[i].groom;
        if (!g->cache && g->strand_total)
            e = cudaMalloc((void**)&g->cache, (size_t)g->strand_total * 2u * hg::kStrandCacheCps * sizeof(float4));
    }
    if (e == cudaSuccess) e = hg::batch_occupancy(&b->raster_per_sm_max, &b->gen_per_sm);
    if (e != cudaSuccess) {
        free_batch(b);
        return cuda_fail(ctx, e, "creating the batch");
    }
    *out = b;
    return HG_OK;
}

void hg_batch_destroy(hg_batch* b) {
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    free_batch(b);
}

hg_status hg_batch_set_params(hg_batch* b, uint32_t item, const hg_hair_params* camera, const hg_hair_params* dom) {
    if (!b || !camera) return HG_INVALID_ARG;
    hg_ctx* ctx = b->ctx;
    if (item >= b->n) return fail(ctx, HG_INVALID_ARG, "item index out of range");
    const hg_hair_params& c = *camera;
    if (c.pass_mode[0] != 0u) return fail(ctx, HG_INVALID_ARG, "camera params need pass_mode.x == 0");
    if (c.screen[0] != (float)b->w[item] || c.screen[1] != (float)b->h[item])
        return fail(ctx, HG_INVALID_ARG, "camera screen.xy differs from the item's size");
    const bool has_dom = b->dw[item] != 0;
    if ((c.flags[3] != 0u) != has_dom)
        return fail(ctx, HG_INVALID_ARG, "camera flags[3] must be 1 exactly when the item has a map");
    if (has_dom) {
        if (!dom || dom->pass_mode[0] != 1u) return fail(ctx, HG_INVALID_ARG, "DOM params need pass_mode.x == 1");
        if (dom->screen[0] != (float)b->dw[item] || dom->screen[1] != (float)b->dh[item] ||
            dom->dom_info[0] != (float)b->dw[item] || dom->dom_info[1] != (float)b->dh[item] ||
            c.dom_info[0] != (float)b->dw[item] || c.dom_info[1] != (float)b->dh[item])
            return fail(ctx, HG_INVALID_ARG, "DOM screen / dom_info differ from the item's map size");
    }
    for (uint32_t j = 0; j < b->n; ++j)
        if (j != item && b->have[j] &&
            (b->cam[j].flags[1] != c.flags[1] || b->cam[j].pass_mode[2] != c.pass_mode[2]))
            return fail(ctx, HG_INVALID_ARG, "items must agree on the filter flag and the depth convention");
    // host copies only: the pinned tables are rebuilt at the next frame
    b->cam[item] = c;
    if (has_dom) b->dom[item] = *dom;
    b->have[item] = 1;
    b->tables_dirty = true;
    return HG_OK;
}

hg_status hg_batch_frame(hg_batch* b, const hg_shade_desc* shade, hg_batch_mode mode) {
    if (!b || !shade) return HG_INVALID_ARG;
    hg_ctx* ctx = b->ctx;
    if (!ready(b)) return fail(ctx, HG_NOT_READY, "set every item's params before a frame");
    cudaSetDevice(ctx->device);
    BATCH_CUDA(ctx, cudaPeekAtLastError());  // an earlier error is reported, not cleared
    if (mode == HG_BATCH_SEPARATE) {
        if (shade->shade_model != 0u) return fail(ctx, HG_INVALID_ARG, "batched frames shade with model 0");
        BATCH_CUDA(ctx, guard_readback(b));
        hg_status s = run_separate(b, shade);
        if (s == HG_OK) BATCH_CUDA(ctx, cudaEventRecord(b->done, ctx->stream));
        return s;
    }
    if (mode != HG_BATCH_GRAPH && mode != HG_BATCH_LAUNCHES) return fail(ctx, HG_INVALID_ARG, "unknown batch mode");
    // The previous frame's upload has read the pinned tables; its kernels may
    // still run while this frame's tables are written.
    BATCH_CUDA(ctx, cudaEventSynchronize(b->uploaded));
    refresh_tables(b);
    hg_status s = stage_lights(b, shade);
    if (s != HG_OK) return s;
    invalidate_caches(b);
    if (mode == HG_BATCH_LAUNCHES) {
        BATCH_CUDA(ctx, enqueue_frame(b));
    } else {
        if (!b->graph_valid || b->g_lights != b->dev.n_lights || b->g_ortho != b->dev.ortho ||
            b->g_exposure != b->dev.exposure || b->g_env != ctx->env_generation) {
            if ((s = capture(b)) != HG_OK) return s;
        }
        BATCH_CUDA(ctx, upload_tables(b));
        BATCH_CUDA(ctx, launch_graphs(b));
    }
    note_cache_writes(b);
    BATCH_CUDA(ctx, cudaEventRecord(b->done, ctx->stream));
    return HG_OK;
}

hg_status hg_batch_launches(hg_batch* b, hg_batch_mode mode, uint32_t* launches) {
    if (!b || !launches) return HG_INVALID_ARG;
    if (!ready(b)) return fail(b->ctx, HG_NOT_READY, "set every item's params first");
    BATCH_CUDA(b->ctx, cudaEventSynchronize(b->uploaded));
    refresh_tables(b);
    if (mode == HG_BATCH_SEPARATE) {
        // hg_groom_frame: clear, lod, scan (2 kernels), [generate, clear_dom, lod, scan (2), raster x2],
        // clear colour, camera raster (2 stages + tile depths), shade, [filter], composite
        uint32_t total = 0;
        for (uint32_t i = 0; i < b->n; ++i)
            total += 1 + 1 + 2 + (b->dw[i] ? 7u : 0u) + 1 + 3 + 1 + (b->cam[i].flags[1] ? 1u : 0u) + 1;
        *launches = total;
        return HG_OK;
    }
    const hg::BatchDev& d = b->dev;
    uint32_t k = 1;                                 // clear
    k += d.total_dom_words ? 1 : 0;                 // clear_dom
    k += d.total_bundles ? 2 : 0;                   // lod, scan expand
    k += 1;                                         // scan offsets
    k += d.total_strands ? 1 : 0;                   // generate
    k += 2 + (d.total_tdepth ? 1 : 0);              // raster stages 1 and 2 (+ tile depths between them)
    k += d.n_views > d.n_cam ? 1 : 0;               // DOM layers
    k += d.total_tiles ? 1 : 0;                     // shade
    k += d.filter ? 1 : 0;                          // filter
    k += 2;                                         // clear colour, composite
    *launches = k;
    return HG_OK;
}

hg_status hg_batch_profile(hg_batch* b, const hg_shade_desc* shade, float* ms) {
    if (!b || !shade || !ms) return HG_INVALID_ARG;
    hg_ctx* ctx = b->ctx;
    if (!ready(b)) return fail(ctx, HG_NOT_READY, "set every item's params before a frame");
    cudaSetDevice(ctx->device);
    BATCH_CUDA(ctx, cudaPeekAtLastError());
    BATCH_CUDA(ctx, cudaEventSynchronize(b->done));
    refresh_tables(b);
    hg_status s = stage_lights(b, shade);
    if (s != HG_OK) return s;
    invalidate_caches(b);
    cudaEvent_t ev[5] = {};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 5 && e == cudaSuccess; ++i) e = cudaEventCreate(&ev[i]);
    const uint32_t n_views = b->n + b->n_dom;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_views, b->h_views, sizeof(hg::BatchView) * n_views, cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_tab, b->h_tab, sizeof(uint32_t) * b->tab_words, cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e == cudaSuccess && b->dev.n_lights)
        e = cudaMemcpyAsync(b->d_lights, b->h_lights, sizeof(hg_light) * b->dev.n_lights, cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev[0], ctx->stream);
    if (e == cudaSuccess) e = hg::launch_batch_setup(ctx, b->dev);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], ctx->stream);
    if (e == cudaSuccess) e = hg::launch_batch_raster(ctx, b->dev);
    if (e == cudaSuccess) e = cudaEventRecord(ev[2], ctx->stream);
    if (e == cudaSuccess) e = hg::launch_batch_shade(ctx, b->dev);
    if (e == cudaSuccess) e = cudaEventRecord(ev[3], ctx->stream);
    if (e == cudaSuccess) e = hg::launch_batch_filter_composite(ctx, b->dev);
    if (e == cudaSuccess) e = cudaEventRecord(ev[4], ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[4]);
    for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]);
    for (int i = 0; i < 5; ++i)
        if (ev[i]) cudaEventDestroy(ev[i]);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "profiling the batched frame");
    note_cache_writes(b);
    BATCH_CUDA(ctx, cudaEventRecord(b->done, ctx->stream));
    return HG_OK;
}

hg_status hg_batch_set_tuning(hg_batch* b, const hg_batch_tuning* t) {
    if (!b || !t) return HG_INVALID_ARG;
    hg_status s = check_tuning(b, t);
    if (s != HG_OK) return s;
    BATCH_CUDA(b->ctx, cudaEventSynchronize(b->done));
    b->tuning = *t;
    b->graph_valid = false;
    if (ready(b)) {
        build_tables(b);
        b->tables_dirty = false;
    }
    return HG_OK;
}

hg_status hg_batch_get_tuning(hg_batch* b, hg_batch_tuning* t) {
    if (!b || !t) return HG_INVALID_ARG;
    *t = b->tuning;
    if (!t->raster_blocks_per_sm) t->raster_blocks_per_sm = b->raster_per_sm_max;
    return HG_OK;
}

hg_status hg_batch_tune(hg_batch* b, const hg_shade_desc* shade, hg_batch_tuning* results, uint32_t capacity,
                        uint32_t* count) {
    if (!b || !shade || !count) return HG_INVALID_ARG;
    hg_ctx* ctx = b->ctx;
    if (!ready(b)) return fail(ctx, HG_NOT_READY, "set every item's params before tuning");
    cudaSetDevice(ctx->device);
    BATCH_CUDA(ctx, cudaPeekAtLastError());
    BATCH_CUDA(ctx, cudaEventSynchronize(b->done));
    hg_status s = stage_lights(b, shade);
    if (s != HG_OK) return s;
    invalidate_caches(b);
    *count = 0;
    const hg_batch_tuning start = b->tuning;
    hg_batch_tuning best = start;
    if (!best.raster_blocks_per_sm) best.raster_blocks_per_sm = b->raster_per_sm_max;
    float best_ms = 3.0e38f;
    auto trial = [&](hg_batch_tuning t) -> hg_status {
        b->tuning = t;
        build_tables(b);
        b->tables_dirty = false;
        hg_status st = capture(b);
        if (st != HG_OK) return st;
        cudaError_t e = upload_tables(b);  // time_graph ends with a stream sync before the next rebuild
        if (e != cudaSuccess) return cuda_fail(ctx, e, "uploading a tuning candidate's tables");
        const float ms = time_graph(b, 2, 5, &e);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "timing a tuning candidate");
        t.ms = ms;
        if (results && *count < capacity) results[*count] = t;
        *count += 1;
        if (ms < best_ms) {
            best_ms = ms;
            best = t;
        }
        return HG_OK;
    };
    // 1. raster work chunk x persistent grid
    const uint32_t chunks[] = {1u, 2u, 4u, 8u, 16u};
    std::vector<uint32_t> grids = {b->raster_per_sm_max};
    if (b->raster_per_sm_max > 2) grids.push_back(b->raster_per_sm_max / 2);
    for (uint32_t c : chunks)
        for (uint32_t gsm : grids) {
            hg_batch_tuning t = best;
            t.raster_chunk = c;
            t.raster_blocks_per_sm = gsm;
            if ((s = trial(t)) != HG_OK) return s;
        }
    // 2. pixel tile of shade / composite
    const uint32_t tiles[][2] = {{16u, 16u}, {64u, 4u}};
    const hg_batch_tuning after_raster = best;
    for (const auto& tl : tiles) {
        hg_batch_tuning t = after_raster;
        t.tile_w = tl[0];
        t.tile_h = tl[1];
        if ((s = trial(t)) != HG_OK) return s;
    }
    // 3. filter tile
    {
        hg_batch_tuning t = best;
        t.filter_tile = 1u - best.filter_tile;
        if ((s = trial(t)) != HG_OK) return s;
    }
    b->tuning = best;
    build_tables(b);
    b->tables_dirty = false;
    b->graph_valid = false;
    note_cache_writes(b);
    BATCH_CUDA(ctx, cudaEventRecord(b->done, ctx->stream));
    return HG_OK;
}

hg_status hg_batch_buffer(hg_batch* b, uint32_t item, hg_buffer_id which, void** ptr, size_t* bytes) {
    if (!b || !ptr || !bytes) return HG_INVALID_ARG;
    if (item >= b->n) return fail(b->ctx, HG_INVALID_ARG, "item index out of range");
    const uint64_t po = b->px_off[item], px = (uint64_t)b->w[item] * b->h[item];
    const uint64_t texels = (uint64_t)b->dw[item] * b->dh[item];
    switch (which) {
        case HG_BUF_CENTER: *ptr = b->center + po, *bytes = px * 8; break;
        case HG_BUF_CONSERVATIVE: *ptr = b->cons + po, *bytes = px * 8; break;
        case HG_BUF_BETA: *ptr = b->beta + po, *bytes = px * 4; break;
        case HG_BUF_DOM:
            *ptr = texels ? b->dommap + b->dom_off[item] : nullptr, *bytes = texels * (1 + HG_DOM_LAYERS) * 4;
            break;
        case HG_BUF_SHADED: *ptr = b->shaded + po, *bytes = px * 16; break;
        case HG_BUF_SHADED_DEPTH: *ptr = b->shaded_depth + po, *bytes = px * 4; break;
        case HG_BUF_FILTERED: *ptr = b->filtered + po, *bytes = px * 16; break;
        case HG_BUF_FILTERED_DEPTH: *ptr = b->filtered_depth + po, *bytes = px * 4; break;
        case HG_BUF_COLOR: *ptr = b->color + po, *bytes = px * 16; break;
        case HG_BUF_DEPTH: *ptr = b->depth + po, *bytes = px * 4; break;
        default: return fail(b->ctx, HG_INVALID_ARG, "unknown buffer id");
    }
    return HG_OK;
}

hg_status hg_batch_copy_out_async(hg_batch* b, uint32_t item, hg_buffer_id which, void* host, size_t bytes) {
    if (!b || !host) return HG_INVALID_ARG;
    void* p = nullptr;
    size_t n = 0;
    hg_status s = hg_batch_buffer(b, item, which, &p, &n);
    if (s != HG_OK) return s;
    if (bytes != n) return fail(b->ctx, HG_INVALID_ARG, "size differs from the item's buffer");
    if (!n) return HG_OK;
    hg_ctx* ctx = b->ctx;
    BATCH_CUDA(ctx, cudaEventRecord(ctx->ev_copy_src, ctx->stream));
    BATCH_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_copy_src, 0));
    BATCH_CUDA(ctx, cudaMemcpyAsync(host, p, n, cudaMemcpyDeviceToHost, ctx->copy_stream));
    BATCH_CUDA(ctx, cudaEventRecord(ctx->ev_copy_done, ctx->copy_stream));
    b->pending_reads = true;
    return HG_OK;
}

hg_status hg_batch_copy_out(hg_batch* b, uint32_t item, hg_buffer_id which, void* host, size_t bytes) {
    if (!b || !host) return HG_INVALID_ARG;
    void* p = nullptr;
    size_t n = 0;
    hg_status s = hg_batch_buffer(b, item, which, &p, &n);
    if (s != HG_OK) return s;
    if (bytes != n) return fail(b->ctx, HG_INVALID_ARG, "size differs from the item's buffer");
    if (!n) return HG_OK;
    BATCH_CUDA(b->ctx, cudaMemcpyAsync(host, p, n, cudaMemcpyDeviceToHost, b->ctx->stream));
    BATCH_CUDA(b->ctx, cudaStreamSynchronize(b->ctx->stream));
    return HG_OK;
}

}  // extern "C"
