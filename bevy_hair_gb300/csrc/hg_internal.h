// Internal state of a hairgb context and the kernel launchers each
// translation unit provides.  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/hairgb.h"

// Scratch of the binned camera raster (raster.cu), per groom, allocated on
// its first binned frame and grown with the ref capacity and the screen.
struct hg_bin_buffers {
    uint32_t ref_cap = 0;         // refs (draw slots) the buffers hold
    uint32_t tile_cap = 0;        // 32x32 screen tiles
    size_t pair_cap = 0;          // ref_cap * 126 segments * 4 tiles
    float4* scr = nullptr;        // ref_cap * 128: screen x, y, ao, in_front of each control point
    float4* cpw = nullptr;        // ref_cap * 256: world position, then world tangent + w (strands not cached)
    uint4* rinfo = nullptr;       // ref_cap: cache slot or ~0u, quv | beta_q << 12, control points, ref index
    uint2* pairs = nullptr;       // pair_cap: (tile, entry) in the order the bin pass emitted them
    uint32_t* entries = nullptr;  // pair_cap: entries (draw slot << 7 | segment) sorted by tile
    uint32_t* tile_count = nullptr;  // tile_cap
    uint32_t* tile_off = nullptr;    // tile_cap + 1
    uint32_t* cursor = nullptr;      // tile_cap
    uint32_t* longs = nullptr;       // ref_cap * 126: segments drawn with global atomics
    uint32_t* meta = nullptr;        // pairs, long segments, largest chunk count, work counter
};

struct hg_groom {
    hg_gpu_bundle* bundles = nullptr;
    float4* layers = nullptr;  // 2 float4 per GpuLayer
    float4* style = nullptr;
    uint32_t bundle_count = 0;   // as uploaded (may be 0)
    uint32_t layer_count = 0;
    uint32_t style_count = 0;
    uint32_t strand_total = 0;   // sum of strand_count
    uint32_t ref_capacity = 1;   // max(strand_total, 1), scan.wgsl:14 capacity
    hg_lod_record* lod[2] = {nullptr, nullptr};
    hg_strand_ref* refs[2] = {nullptr, nullptr};
    uint32_t* indirect[2] = {nullptr, nullptr};  // (total, 1, 1, 0)
    uint32_t* offsets[2] = {nullptr, nullptr};   // exclusive scan of n_lod, bundle_count + 1
    // Front-to-back draw order of the camera pass (scheduling only).
    uint32_t* depth_key[2] = {nullptr, nullptr};   // per bundle: nearest-depth bucket
    uint32_t* sorted[2] = {nullptr, nullptr};      // live bundles in depth order
    uint32_t* sorted_off[2] = {nullptr, nullptr};  // scan of n_lod in that order, bundle_count + 1
    uint32_t* draw_order[2] = {nullptr, nullptr};  // permutation of refs, ref_capacity
    uint32_t* order_meta[2] = {nullptr, nullptr};  // (live bundles, order valid)
    // Draw order of the DOM depth pass when every strand is drawn (the usual
    // case): the refs of bundles in a hashed order (scheduling only).  Its
    // atomicMin on the front plane contends when neighbouring strands draw
    // together; the layers pass, whose counter adds gain from locality, keeps
    // the bundle order.
    uint32_t* dom_order = nullptr;  // strand_total
    // Strand cache (hg_generate): world-space control points of every strand.
    uint32_t* strand_bundle = nullptr;  // bundle of each strand, strand_total
    uint32_t* strand_base = nullptr;    // first strand of each bundle, bundle_count + 1
    float4* cache = nullptr;            // strand_total * 2 * 65 float4, allocated on first use
    bool cache_valid = false;
    float cache_model[16] = {};         // world_from_model the cache was generated with
    hg_bin_buffers bins;                // binned camera raster scratch
};

// Learned shading surrogate (surrogate.cu): FP32 master parameters, Adam
// state, FP16 forward and transposed copies, training scratch.
struct hg_mlp {
    hg_ctx* ctx = nullptr;
    uint32_t arch = 0;         // HG_MLP_ARCH_*
    uint32_t n_params = 0;     // HG_MLP_PARAMS or HG_MLP_COMPACT_PARAMS
    float* params = nullptr;   // n_params floats
    float* grad = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    void* w16 = nullptr;       // __half[n_params], parameter layout
    void* wt16 = nullptr;      // __half[13312], W2^T W3^T W4^T W5^T (4 x 64 network only)
    float* loss = nullptr;     // device scalar
    void* scratch = nullptr;   // transposed activations and gradients, (16 + 4*64 + 4*64 + 16) x ld halves
    uint32_t ld_capacity = 0;
    uint64_t step = 0;
};

// Shade model 3's dual-scattering statistics (kDualTableFloat4 float4 on the
// device) and the material (albedo rgb, roughness, tilt) they were filled for.
struct hg_dual_table {
    float4* table = nullptr;
    float key[5] = {};
    bool valid = false;
};

struct hg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint32_t width = 0, height = 0, dom_w = 0, dom_h = 0;
    unsigned long long* center = nullptr;
    unsigned long long* cons = nullptr;
    uint32_t* beta = nullptr;
    uint32_t* dom = nullptr;
    float4* shaded = nullptr;
    float* shaded_depth = nullptr;
    float4* filtered = nullptr;
    float* filtered_depth = nullptr;
    float4* color = nullptr;
    float* depth = nullptr;
    uint32_t* hair_list = nullptr;  // pixels with hair (shade models 1 and 3), W*H
    uint32_t* hair_count = nullptr;
    hg_dual_table* dual_table = nullptr;  // shade model 3's dual-scattering table (shared by context copies)
    // Camera raster: per 8x8 pixel tile, the largest quantised depth held by
    // any of its G-buffer words (an upper bound once built, since the words
    // only decrease during the pass).
    uint32_t* tile_depth = nullptr;
    // Camera raster kind (hg_set_camera_raster): HG_CAMERA_RASTER_BINNED or _DIRECT.
    uint32_t camera_raster = HG_CAMERA_RASTER_DIRECT;
    // Asynchronous readback (hg_copy_out_async): copies run on copy_stream
    // behind ev_copy_src; ev_copy_done follows the last one.  pending_reads
    // has bit (1 << hg_buffer_id) set for buffers whose copy a later writer
    // has not yet been ordered after.
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copy_src = nullptr, ev_copy_done = nullptr;
    uint32_t pending_reads = 0;
    uint32_t* err = nullptr;       // device error word
    hg_light* lights = nullptr;    // device copy, HG_MAX_LIGHTS
    // Pinned staging ring for the light list; slot k is reused only after
    // the event recorded behind its last copy has completed.
    static constexpr int kLightSlots = 8;
    hg_light* lights_host = nullptr;  // kLightSlots * HG_MAX_LIGHTS
    cudaEvent_t light_events[kLightSlots] = {};
    int light_slot = 0;
    // Side stream and events for the frame's independent DOM half.
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_gen = nullptr, ev_join = nullptr;
    int sm_count = 0;
    hg_mlp* surrogate = nullptr;   // bound by hg_mlp_bind, used by shade_model 1
    // light probe (hg_env_set): RGB9E5 mip chains, six faces per level
    uint32_t* env_spec = nullptr;
    uint32_t* env_diff = nullptr;
    uint32_t env_spec_size = 0, env_spec_levels = 0, env_diff_size = 0, env_diff_levels = 0;
    float env_rot[4] = {0.0f, 0.0f, 0.0f, 1.0f};
    float env_intensity = 0.0f;
    // Bumped by every hg_env_set: a captured batch graph holds the probe's
    // device pointers, sizes and rotation by value and is re-captured when
    // this differs from the count it was captured at.
    uint64_t env_generation = 0;
    std::string last_error;
};

namespace hg {

// Dual-scattering table of shade model 3 (shade.cu): 64 uvw.z levels x 129
// view angles x 6 float4.
constexpr size_t kDualTableFloat4 = 64u * 129u * 6u;

// One view of a batched item (its camera view, or its deep-opacity view):
// uniforms, groom buffers and targets.  A device table of these is read in
// place by the batched kernels; the field names match the single-view
// argument structs so the same device functions serve both.
struct BatchView {
    hg_hair_params p;
    const hg_gpu_bundle* bundles;
    const float4* layers;
    const float4* style;
    hg_lod_record* lod;
    uint32_t* depth_key;
    uint32_t* offsets;
    uint32_t* indirect;
    hg_strand_ref* refs;
    // camera views: front-to-back draw order (as the single-view scan builds
    // it) and the per-8x8-tile depths between the two raster stages
    uint32_t* sorted;
    uint32_t* sorted_off;
    uint32_t* draw_order;
    uint32_t* order_meta;
    uint32_t* tile_depth;
    uint32_t tiles_x;
    float4* cache;                 // strand cache of the item's groom
    const uint32_t* strand_base;
    const uint32_t* strand_bundle;
    unsigned long long* center;
    unsigned long long* cons;
    uint32_t* beta;
    uint32_t* dom;                 // the item's deep opacity map (camera and DOM views)
    float4* shaded;
    float* shaded_depth;
    float4* filtered;
    float* filtered_depth;
    float4* color;
    float* depth;
    const float* scene;
    uint32_t* err;
    uint32_t bundle_count;         // bundles of the groom
    uint32_t count;                // bundles the view's lod/scan cover: min(pass_mode.y, bundle_count)
    uint32_t capacity;             // strand-ref capacity
    uint32_t strands;              // strands of the groom (the cache's extent)
    uint32_t width, height;        // this view's target size
    uint32_t dom_w, dom_h;
};

// Launch description of one batched frame: the view table (camera views
// first, then deep-opacity views), prefix tables over views, the contiguous
// target arenas and the tuning.
struct BatchDev {
    const BatchView* views = nullptr;
    uint32_t n_views = 0, n_cam = 0;
    const uint32_t* bundle_prefix = nullptr;  // n_views + 1, bundles covered by lod/scan
    const uint32_t* strand_prefix = nullptr;  // n_cam + 1, strands to generate
    const uint32_t* tile_prefix = nullptr;    // n_cam + 1, tile_w x tile_h pixel tiles
    const uint32_t* ftile_prefix = nullptr;   // n_cam + 1, filter tiles
    const uint32_t* dom_prefix = nullptr;     // n_cam + 1, DOM words (front + counters) per item
    const uint32_t* tdepth_prefix = nullptr;  // n_cam + 1, 8x8 tile-depth words per camera view
    uint32_t total_tdepth = 0;
    uint32_t total_bundles = 0, total_strands = 0, total_tiles = 0, total_ftiles = 0;
    uint64_t total_px = 0, total_dom_words = 0;
    unsigned long long* center = nullptr;     // arenas: every camera view's slice, concatenated
    unsigned long long* cons = nullptr;
    uint32_t* beta = nullptr;
    uint32_t* dom = nullptr;
    float4* color = nullptr;
    float* depth = nullptr;
    uint32_t* counters = nullptr;             // work counters of the three raster launches
    const hg_light* lights = nullptr;
    uint32_t n_lights = 0, ortho = 0;
    float exposure = 1.0f, depth_clear = 0.0f;
    uint32_t filter = 1, composite = 1;
    uint32_t gen_blocks = 1;                  // grid of the generate pass (occupancy x SMs)
    // tuning
    uint32_t raster_chunk = 4, raster_blocks_per_sm = 1, tile_w = 32, tile_h = 8, filter_tile = 0;
};

// raster.cu
// Once per device before the first shade launch: the dual-scattering angle table.
cudaError_t ensure_shade_setup(int device);
cudaError_t launch_clear(hg_ctx* ctx);
cudaError_t launch_clear_dom(hg_ctx* ctx);
cudaError_t launch_lod(hg_ctx* ctx, hg_groom* g, const hg_hair_params& p, int slot);
cudaError_t launch_scan(hg_ctx* ctx, hg_groom* g, const hg_hair_params& p, int slot);
cudaError_t launch_raster(hg_ctx* ctx, hg_groom* g, const hg_hair_params& p, int slot, const float* scene);
cudaError_t launch_generate(hg_ctx* ctx, hg_groom* g, const hg_hair_params& p);
void release_bins(hg_groom* g);  // frees the binned camera raster's scratch
constexpr uint32_t kStrandCacheCps = 65;

// Pixels per side of a tile of the camera pass's tile-depth buffer, as a
// shift, and the tile count of a w x h view.
constexpr uint32_t kTileShift = 3;
constexpr uint32_t tiles_along(uint32_t n) { return (n + (1u << kTileShift) - 1u) >> kTileShift; }

// shade.cu
cudaError_t launch_shade(hg_ctx* ctx, const hg_hair_params& p, uint32_t n_lights, uint32_t ortho, float exposure,
                         uint32_t model);
cudaError_t launch_karis_lobes(hg_ctx* ctx, const float* inputs, uint32_t n, float tilt, float* lobes);

// batched passes (raster.cu, shade.cu, filter.cu)
cudaError_t batch_occupancy(uint32_t* raster_per_sm, uint32_t* gen_per_sm);
cudaError_t launch_batch_setup(hg_ctx* ctx, const BatchDev& b);     // clears, lod, scan, generate
cudaError_t launch_batch_raster(hg_ctx* ctx, const BatchDev& b);    // camera + DOM depth, then DOM layers
cudaError_t launch_batch_shade(hg_ctx* ctx, const BatchDev& b);
cudaError_t launch_batch_filter_composite(hg_ctx* ctx, const BatchDev& b);
constexpr uint32_t kBatchMaxViews = 256;

// surrogate.cu
cudaError_t launch_mlp_infer(hg_mlp* m, const float* inputs, uint32_t n, float* lobes, float* net);
cudaError_t launch_mlp_infer_tc(hg_mlp* m, const float* inputs, uint32_t n, float* lobes, float* net);

// filter.cu
cudaError_t launch_filter(hg_ctx* ctx, const hg_hair_params& p);
cudaError_t launch_composite(hg_ctx* ctx, const hg_hair_params& p, uint32_t source_filtered);
cudaError_t launch_clear_color(hg_ctx* ctx, float depth_clear);

// receiver.cu
cudaError_t launch_visibility(hg_ctx* ctx, const hg_shadow_light& L, const float* points, uint32_t n, float* out);

}  // namespace hg
