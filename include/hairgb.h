/*
 * hairgb.h -- C ABI of the GB300 (sm_103a) strand-hair pipeline.
 *
 * This library replaces the compute passes that bevy_hair's render host
 * records per groom in `hair_pass` (src/render/pass.rs:259-657): clear, lod,
 * scan, raster (camera), clear_dom + lod + scan + raster (deep opacity map,
 * two modes), shade, filter and composite.  The host keeps the ECS glue
 * (extract/prepare) and the uniform math (make_params, light_fit) and calls
 * the entry points below instead of recording wgpu passes.
 *
 * Conventions
 *  - Every entry point returns hg_status.  No entry point aborts, traps or
 *    prints; hg_last_error() holds a one-line message for the last failure.
 *  - All GPU work of one context is ordered on one CUDA stream (the one given
 *    to hg_create, or a stream the context creates).  Calls enqueue work and
 *    return; hg_synchronize() waits and reports device-side error words.
 *  - Device memory is owned by the library.  Host arrays are read during the
 *    call only.  Pointers returned by hg_buffer() stay valid until the next
 *    hg_ensure_targets() that changes a size, or hg_destroy().
 *  - Struct layouts are the reference's std140/std430 layouts byte for byte
 *    (see the static asserts at the end of this header).
 */
#ifndef HAIRGB_H
#define HAIRGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HG_ABI_VERSION 1u

/* Layers per bundle cage; src/mesh.rs:10, common.wgsl:1. */
#define HG_LAYER_COUNT 16u
/* Style volume 8 x 8 x 16 texels per bundle; src/mesh.rs:11-14. */
#define HG_STYLE_TEXELS 1024u
/* Opacity slices behind each deep-opacity texel; src/render/pass.rs:24. */
#define HG_DOM_LAYERS 16u
/* Maximum lights in one shade call. */
#define HG_MAX_LIGHTS 256u

typedef enum hg_status {
    HG_OK = 0,
    HG_INVALID_ARG = 1,
    HG_OUT_OF_MEMORY = 2,
    HG_CUDA_ERROR = 3,
    HG_CAPACITY_EXCEEDED = 4,
    HG_DEVICE_TIMEOUT = 5,
    HG_NOT_READY = 6,
    HG_DEVICE_ERROR = 7
} hg_status;

/* HairParams uniform, 432 bytes (src/render/pass.rs:42-60,
 * src/render/shaders/common.wgsl:10-28).  Matrices are column-major
 * (glam to_cols_array_2d), so element [c*4 + r] is row r of column c. */
typedef struct hg_hair_params {
    float clip_from_world[16];
    float world_from_clip[16];
    float world_from_model[16];
    float light_clip_from_world[16];
    float camera_pos[4];
    float camera_forward[4];
    float screen[4];        /* width, height, near, far */
    float appearance[4];    /* roughness, tilt, lambda, center_diameter */
    float filter_params[4]; /* s_par, s_perp, dom_scale, dom_sigma */
    float albedo[4];
    uint32_t flags[4];      /* lod, filter, ambient_occlusion, deep_opacity */
    uint32_t pass_mode[4];  /* mode (0 camera, 1 DOM depth, 2 DOM layers), bundle_count, reverse_z, dom_lod */
    float light_eye[4];
    float light_forward[4];
    float dom_info[4];      /* dom_w, dom_h, light near, light far */
} hg_hair_params;

/* GpuBundle (src/render/pass.rs:71-78), 16 bytes. */
typedef struct hg_gpu_bundle {
    uint32_t layer_offset;
    uint32_t style_offset;
    uint32_t strand_count;
    uint32_t pad;
} hg_gpu_bundle;

/* GpuLayer (src/render/pass.rs:64-69), 32 bytes: position + baked AO, tangent. */
typedef struct hg_gpu_layer {
    float pos_ao[4];
    float tangent[4];
} hg_gpu_layer;

/* LodRecord (common.wgsl:42-47). */
typedef struct hg_lod_record {
    uint32_t n_lod;
    uint32_t control_points;
    uint32_t strand_count;
    uint32_t pad;
} hg_lod_record;

/* StrandRef (common.wgsl:49-54). */
typedef struct hg_strand_ref {
    uint32_t bundle;
    uint32_t strand;
    uint32_t n_lod;
    uint32_t control_points;
} hg_strand_ref;

/* Which LOD/refs/indirect set of a groom a pass uses.  A groom holds one set
 * for the camera view and one for the deep-opacity view, like GpuGroom's
 * camera_lod/camera_refs and dom_lod/dom_refs (src/render/pass.rs:80-96). */
typedef enum hg_view_slot {
    HG_SLOT_CAMERA = 0,
    HG_SLOT_DOM = 1
} hg_view_slot;

typedef enum hg_light_kind {
    HG_LIGHT_POINT = 0,
    HG_LIGHT_SPOT = 1,
    HG_LIGHT_DIRECTIONAL = 2,
    HG_LIGHT_RECT = 3
} hg_light_kind;

#define HG_LIGHT_CASTS_SHADOWS 1u

/* One light of the shade pass.  Replaces bevy_pbr's clustered light list,
 * directional list and rect-light list that shade.wesl:452-518 reads.
 *  point/spot: position, range (attenuation window), color = colour x intensity
 *  spot:       direction = unit axis pointing away from the light,
 *              spot[0..1] = angular scale/offset (cone mask clamp(cd*s+o,0,1)^2)
 *  directional: direction = unit vector toward the light (direction_to_light),
 *              color = colour x illuminance; CASTS_SHADOWS marks the light
 *              that receives the deep-opacity optical depth (the first such)
 *  rect:       position = centre, right/up = half axes, spot[0..1] = width,
 *              height, range
 * 112 bytes. */
typedef struct hg_light {
    uint32_t kind;
    uint32_t flags;
    float range;
    float pad0;
    float position[4];
    float color[4];
    float direction[4];
    float spot[4];
    float right[4];
    float up[4];
} hg_light;

/* What the shade pass reads besides HairParams and the G-buffer.  The
 * reference takes these from Bevy's view bind groups (shade.wesl:1-11). */
typedef struct hg_shade_desc {
    const hg_light* lights;   /* host array, light_count entries */
    uint32_t light_count;
    uint32_t ortho;           /* 1 when the camera projection is orthographic */
    float exposure;           /* view.exposure */
    uint32_t shade_model;     /* 0: Karis fit (shade.wesl); 1: learned 4 x 64 surrogate on tcgen05;
                                 2: the 4 x 64 surrogate on mma.sync (for comparison);
                                 3: the compact 2 x 32 surrogate on mma.sync */
} hg_shade_desc;

/* Buffers a context owns. */
typedef enum hg_buffer_id {
    HG_BUF_CENTER = 0,          /* u64[W*H] center-sample G-buffer */
    HG_BUF_CONSERVATIVE = 1,    /* u64[W*H] conservative G-buffer */
    HG_BUF_BETA = 2,            /* u32[W*H] (depth << 8 | beta8) side channel */
    HG_BUF_DOM = 3,             /* u32[DW*DH*(1+16)] front depths, then 16 counters per texel */
    HG_BUF_SHADED = 4,          /* float4[W*H] */
    HG_BUF_SHADED_DEPTH = 5,    /* float[W*H] view distance */
    HG_BUF_FILTERED = 6,        /* float4[W*H] */
    HG_BUF_FILTERED_DEPTH = 7,  /* float[W*H] */
    HG_BUF_COLOR = 8,           /* float4[W*H] composite target */
    HG_BUF_DEPTH = 9            /* float[W*H] composite depth attachment */
} hg_buffer_id;

/* Groom buffers held on the device. */
typedef enum hg_groom_buffer_id {
    HG_GBUF_LOD = 0,        /* hg_lod_record[bundle_count] of the slot */
    HG_GBUF_REFS = 1,       /* hg_strand_ref[max(strands,1)] of the slot */
    HG_GBUF_INDIRECT = 2,   /* u32[4]: (total refs, 1, 1, 0) of the slot */
    HG_GBUF_STRAND_CACHE = 3 /* float4[strands * 130] from hg_generate (slot ignored): per strand, in
                                upload order, 65 (world position, ao) then 65 (world tangent, w);
                                a null pointer and size 0 before the first hg_generate */
} hg_groom_buffer_id;

typedef struct hg_ctx hg_ctx;
typedef struct hg_groom hg_groom;

/* Per-groom frame description: the per-groom body of hair_pass
 * (src/render/pass.rs:375-643). */
typedef struct hg_frame_desc {
    const hg_hair_params* camera;       /* pass_mode.x == 0 */
    const hg_hair_params* dom;          /* pass_mode.x == 1; may be NULL when flags[3]==0 */
    const float* scene_depth;           /* device float[W*H] or NULL (no scene depth test) */
    hg_shade_desc shade;
    uint32_t composite;                 /* 1: blend into HG_BUF_COLOR/HG_BUF_DEPTH */
    uint32_t clear_color;               /* 1: reset HG_BUF_COLOR to 0 and HG_BUF_DEPTH to the
                                           far value of camera->pass_mode[2] before compositing */
} hg_frame_desc;

/* ---------------------------------------------------------------- context */

/* device: CUDA ordinal.  stream: a cudaStream_t, or NULL for a stream the
 * context creates and owns. */
hg_status hg_create(int device, void* stream, hg_ctx** out);
hg_status hg_destroy(hg_ctx* ctx);
const char* hg_status_string(hg_status status);
const char* hg_last_error(const hg_ctx* ctx);
uint32_t hg_abi_version(void);

/* Waits for the context's stream and reads the device error word.  Returns
 * HG_DEVICE_ERROR (with the word in *device_error) when a kernel reported a
 * bounds or capacity violation.  device_error may be NULL. */
hg_status hg_synchronize(hg_ctx* ctx, uint32_t* device_error);

/* Screen and deep-opacity targets; ensure_targets (src/render/pass.rs:789-815).
 * The reference fixes the map at 512x512 (pass.rs:22); here it is a parameter. */
hg_status hg_ensure_targets(hg_ctx* ctx, uint32_t width, uint32_t height,
                            uint32_t dom_width, uint32_t dom_height);
hg_status hg_buffer(hg_ctx* ctx, hg_buffer_id id, void** device_ptr, size_t* bytes);
/* Copies a context buffer to host memory (bytes must equal its size). */
hg_status hg_copy_out(hg_ctx* ctx, hg_buffer_id id, void* host, size_t bytes);
/* Enqueues the same copy on the context's copy stream, behind the work
 * enqueued so far, and returns at once.  host should be page-locked for the
 * copy to overlap later work; it must stay valid, and its contents are not
 * final, until hg_copy_wait returns.  Later passes that write the buffer wait
 * for the copy on the device, so the next frame can be enqueued right away.
 * (No reference counterpart: the reference never reads its targets back.) */
hg_status hg_copy_out_async(hg_ctx* ctx, hg_buffer_id id, void* host, size_t bytes);
/* Blocks until every hg_copy_out_async of the context has landed. */
hg_status hg_copy_wait(hg_ctx* ctx);
/* Copies host memory into a context buffer (used to feed a pass its inputs). */
hg_status hg_copy_in(hg_ctx* ctx, hg_buffer_id id, const void* host, size_t bytes);

/* ---------------------------------------------------------------- grooms */

/* GpuGroom::upload (src/render/pass.rs:98-167).  style is float4[style_count]
 * (xyz residual, w unused).  Offsets are validated: every bundle needs
 * layer_offset + 64 <= layer_count and style_offset + 1024 <= style_count. */
hg_status hg_groom_upload(hg_ctx* ctx,
                          const hg_gpu_bundle* bundles, uint32_t bundle_count,
                          const hg_gpu_layer* layers, uint32_t layer_count,
                          const float* style, uint32_t style_count,
                          hg_groom** out);
hg_status hg_groom_destroy(hg_ctx* ctx, hg_groom* groom);
hg_status hg_groom_buffer(hg_ctx* ctx, hg_groom* groom, hg_view_slot slot,
                          hg_groom_buffer_id id, void** device_ptr, size_t* bytes);
/* Copies a groom buffer of a slot to host memory (bytes must equal its size). */
hg_status hg_groom_copy_out(hg_ctx* ctx, hg_groom* groom, hg_view_slot slot,
                            hg_groom_buffer_id id, void* host, size_t bytes);

/* ---------------------------------------------------------------- passes */

/* clear.wgsl:7-16: center = conservative = ~0, beta = 0xffffffff. */
hg_status hg_clear(hg_ctx* ctx);
/* clear_dom.wgsl:8-21: front depths = 0xffffffff, counters = 0. */
hg_status hg_clear_dom(hg_ctx* ctx);
/* lod.wgsl:6-59 into the slot's LodRecords. */
hg_status hg_lod(hg_ctx* ctx, hg_groom* groom, const hg_hair_params* params, hg_view_slot slot);
/* scan.wgsl:6-24: LodRecords -> StrandRefs + indirect (total,1,1). */
hg_status hg_scan(hg_ctx* ctx, hg_groom* groom, const hg_hair_params* params, hg_view_slot slot);
/* raster.wgsl:225-337 over the slot's refs.  params->pass_mode[0] selects the
 * camera G-buffer (0) or the deep-opacity map (1 depth, 2 layers).
 * scene_depth: device float[W*H] scene depth (raster.wgsl:93-100) or NULL. */
hg_status hg_raster(hg_ctx* ctx, hg_groom* groom, const hg_hair_params* params,
                    hg_view_slot slot, const float* scene_depth);
/* How hg_raster draws the camera G-buffer.  Scheduling only: both give the
 * same words (every write is a commutative min).
 *  HG_CAMERA_RASTER_DIRECT (the default): every sample's atomicMin goes to
 *    global memory, after a read of the current word's high half, in two
 *    launches (the nearest quarter of the refs, then the rest, whose segments
 *    hidden behind per-8x8-tile depths are skipped).
 *  HG_CAMERA_RASTER_BINNED: every segment is listed under the 32x32 screen
 *    tiles its pixels can touch; a block per tile (and chunk of its list)
 *    resolves the tile's centre, conservative and beta words in shared memory,
 *    then issues one global atomicMin per word it lowered.  Segments whose
 *    pixels span more than 2x2 tiles are drawn with global atomics.  Its
 *    scratch (about 12.5 KiB per strand of the groom) is allocated on the
 *    groom's first binned raster.  Slower than the direct pass on the
 *    1920x1080 benchmark frame (1.08 vs 0.41 ms).
 * raster.wgsl (the reference) issues every sample's atomicMin directly; the
 * choice has no counterpart there. */
#define HG_CAMERA_RASTER_DIRECT 0u
#define HG_CAMERA_RASTER_BINNED 1u
hg_status hg_set_camera_raster(hg_ctx* ctx, uint32_t mode);
/* Strand cache: generates every strand of the groom at the full 65 control
 * points (control_points_for_lod(1.0)) in world space with
 * params->world_from_model -- the strand generation of raster.wgsl:231-317,
 * run once.  Later hg_raster calls whose params carry the same
 * world_from_model read refs drawn at 65 control points from the cache
 * instead of regenerating them; results are identical either way.  The
 * reference regenerates strands in every raster dispatch, so this pass has no
 * counterpart there.  The cache (2 KiB per strand) is allocated on first use. */
hg_status hg_generate(hg_ctx* ctx, hg_groom* groom, const hg_hair_params* params);
/* shade.wesl:523-593 (Karis model) over every pixel. */
hg_status hg_shade(hg_ctx* ctx, const hg_hair_params* params, const hg_shade_desc* desc);
/* filter.wgsl:20-135. */
hg_status hg_filter(hg_ctx* ctx, const hg_hair_params* params);
/* composite.wgsl:162-181 plus the ALPHA_BLENDING blend state and the depth
 * test of pipeline.rs:299-339, into HG_BUF_COLOR / HG_BUF_DEPTH.
 * source_filtered selects filtered (1) or shaded (0) colour. */
hg_status hg_composite(hg_ctx* ctx, const hg_hair_params* params, uint32_t source_filtered);
/* Fills HG_BUF_COLOR with 0 and HG_BUF_DEPTH with depth_clear. */
hg_status hg_clear_color(hg_ctx* ctx, float depth_clear);

/* The whole per-groom sequence of hair_pass: clear, lod, scan, raster; when
 * camera->flags[3] (deep_opacity): clear_dom, lod, scan, raster mode 1,
 * raster mode 2; shade; filter when camera->flags[1]; composite.  With the
 * deep opacity map on it also runs hg_generate once before the rasters. */
hg_status hg_groom_frame(hg_ctx* ctx, hg_groom* groom, const hg_frame_desc* desc);

/* ---------------------------------------------------------------- deep-opacity receivers */

/* ShadowLight (src/render/pass.rs:32-40), 112 bytes: the light view published
 * with the deep opacity map for other surfaces. depth = (near, far,
 * extinction per strand fragment, 1 once a map exists). */
typedef struct hg_shadow_light {
    float light_clip_from_world[16];
    float light_eye[4];
    float light_forward[4];
    float depth[4];
} hg_shadow_light;

/* The ShadowLight the reference publishes after the DOM passes
 * (src/render/pass.rs:574-579), from the DOM params (pass_mode.x == 1). */
hg_status hg_shadow_light_from(const hg_hair_params* dom_params, hg_shadow_light* out);

/* ---- Host-side per-view uniforms (no device work, no context) ----------- */

/* The camera of one view (ExtractedView: world_from_view, clip_from_view and
 * the optional clip_from_world override, src/render/pass.rs:342-348) and its
 * target size.  Matrices are column-major (glam to_cols_array). */
typedef struct hg_view_desc {
    float world_from_view[16];
    float clip_from_view[16];
    float clip_from_world[16]; /* used when has_clip_from_world != 0 */
    uint32_t has_clip_from_world;
    uint32_t width, height;
} hg_view_desc;

/* One groom's settings (HairGroom, src/lib.rs:32-63; albedo linear RGB + 1)
 * and its GPU asset's bounds and bundle count (GpuGroom). */
typedef struct hg_groom_desc {
    float world_from_model[16];
    float bounds_min[3];
    float bounds_max[3];
    uint32_t bundle_count;
    float roughness, tilt, lambda, center_diameter;
    float albedo[4];
    uint32_t lod, filter, ambient_occlusion, deep_opacity;
} hg_groom_desc;

/* A directional light as extract_hair records it (src/render/mod.rs:104-107). */
typedef struct hg_directional {
    float direction_to_light[3];
    uint32_t casts_shadows;
} hg_directional;

/* The camera (pass_mode.x = 0) and DOM depth (pass_mode.x = 1) HairParams of
 * one groom, as hair_pass builds them each frame (src/render/pass.rs:342-453:
 * camera position and forward, clip_from_world and its inverse, reverse-Z
 * detection :778-787, key_direction :711-719, world_extent :721-745,
 * light_fit :747-776, make_params :676-709).  The DOM layers params are the
 * DOM params with pass_mode.x = 2.  The DOM size is a parameter (the
 * reference fixes 512).  Pure host arithmetic in f32 (inverses in f64). */
hg_status hg_groom_params(const hg_view_desc* view, const hg_groom_desc* groom, const hg_directional* lights,
                          uint32_t light_count, uint32_t dom_w, uint32_t dom_h, hg_hair_params* camera,
                          hg_hair_params* dom);

/* hair_visibility (src/render/shaders/hair_shadow.wesl:30-75) for n world
 * points against the context's deep opacity map: the fraction of the key
 * light that reaches each point through the groom.  points: device float4[n]
 * (xyz used); visibility: device float[n].  The map's size is the context's
 * DOM size (the reference fixes 512x512). */
hg_status hg_hair_visibility(hg_ctx* ctx, const hg_shadow_light* light, const float* points, uint32_t n,
                             float* visibility);

/* ---------------------------------------------------------------- allocation-free scan */

/* Largest bundle_count hg_scan_noalloc accepts. */
#define HG_SCAN_NOALLOC_MAX_BUNDLES 65536u

/* The scan pass without any device allocation, for hosts that cannot call
 * cudaMalloc while they record a frame: an engine whose device memory all comes
 * from its own allocator or arena (every buffer handed out up front by its
 * render graph), or a real-time host whose fixed memory budget forbids
 * allocating inside the frame loop.  This entry point has no counterpart in
 * the reference; it computes the same StrandRefs and indirect words as hg_scan
 * (without hg_scan's front-to-back draw order, which needs more working
 * memory) and needs no context.
 *
 * lod:      device hg_lod_record[bundle_count] (input)
 * refs:     device hg_strand_ref[capacity] (output; entries past the total
 *           stay untouched)
 * indirect: device u32[4] (output: total, 1, 1, 0)
 * stream:   cudaStream_t to launch on (NULL: the legacy default stream)
 * Work goes on `stream` on the device current on the calling thread.
 *
 * The per-bundle offsets live in a fixed device array of
 * HG_SCAN_NOALLOC_MAX_BUNDLES + 1 words (256 KB) that every device holds while
 * the library is loaded; larger bundle counts return HG_CAPACITY_EXCEEDED.
 * The first call on a device looks up that array's device address (kept per
 * CUDA context: after a reset of the device's primary context, e.g. by
 * cudaDeviceReset, the next call looks it up again), so make the first call
 * on each device, and the first one after such a reset, before any stream
 * capture on it.  All calls share the one array: calls that can overlap on
 * the GPU (unordered streams) race and must be serialised by the caller.
 * Each call rewrites the offsets it reads, so nothing has to be cleared
 * between calls.  Returns HG_INVALID_ARG for null pointers or capacity 0,
 * and HG_CUDA_ERROR when a launch fails or when a CUDA error was already
 * pending on the calling thread (that error is left in place, and nothing is
 * launched). */
hg_status hg_scan_noalloc(const hg_lod_record* lod, uint32_t bundle_count, uint32_t capacity,
                          hg_strand_ref* refs, uint32_t* indirect, void* stream);

/* ---------------------------------------------------------------- environment light probe */

/* The light probe that shade.wesl's probe_radiance samples (shade.wesl:330-427,
 * the ENVIRONMENT_MAP specialization): a specular cubemap sampled trilinearly
 * at mip roughness x (levels - 1) along the R cone, and a diffuse irradiance
 * cubemap at mip 0 along the fibre normal.  Texels are RGB9E5
 * (VK_FORMAT_E5B9G9R9_UFLOAT_PACK32, the format of the reference's KTX2
 * probes); each array holds the mip levels from 0, each level the six faces
 * +X, -X, +Y, -Y, +Z, -Z of max(size >> level, 1)^2 texels, row-major.  The
 * face of a direction and its (s, t) follow the usual major-axis rule; within
 * a face the sampler is bilinear with clamp-to-edge (Bevy's GPU sampler also
 * filters across face edges, so colour parity with it is unpinned).
 * rotation is light_probes.view_rotation (x, y, z, w) and intensity
 * light_probes.intensity_for_view.  Without a probe (the default, or after
 * hg_env_set(ctx, NULL)) probe_radiance is zero, the reference's behaviour
 * without ENVIRONMENT_MAP. */
typedef struct hg_env_desc {
    const uint32_t* specular;    /* host, RGB9E5 */
    uint32_t specular_size, specular_levels;
    const uint32_t* diffuse;     /* host, RGB9E5 */
    uint32_t diffuse_size, diffuse_levels;
    float rotation[4];
    float intensity;
} hg_env_desc;

/* Upload (or, with NULL, drop) the context's light probe; every later shade
 * call adds probe_radiance x AO.  Sizes 1..4096, levels 1..1 + log2(size). */
hg_status hg_env_set(hg_ctx* ctx, const hg_env_desc* env);

/* ---------------------------------------------------------------- batched frames */

/* Many independent grooms, each with its own camera view and deep opacity
 * map, drawn as one batch: every pass runs as one launch over all items (the
 * camera and DOM-depth rasters of all items share one persistent launch whose
 * warps take strand refs from a global counter), and the whole frame is
 * captured once into a CUDA graph and replayed.  This has no counterpart in
 * the reference, which records one hair_pass per groom
 * (src/render/pass.rs:259-657); per item the results are those of
 * hg_groom_frame with the item's params: visibility bit for bit, colour to
 * the last bit of the same kernels' arithmetic.
 *
 * A batch owns every item's targets (one arena per buffer kind) and keeps a
 * pinned copy of the items' uniforms that the graph uploads at replay.  Each
 * groom may appear in one item only (its strand cache holds one transform). */
#define HG_BATCH_MAX_ITEMS 128u

typedef struct hg_batch hg_batch;

typedef struct hg_batch_item {
    hg_groom* groom;
    uint32_t width, height;   /* camera targets, 1..16384 */
    uint32_t dom_w, dom_h;    /* deep opacity map, 1..16384, or 0 x 0 for none */
} hg_batch_item;

/* Launch shapes the autotuner chooses among. */
typedef struct hg_batch_tuning {
    uint32_t raster_chunk;          /* strand refs a warp takes per grab, 1..64 */
    uint32_t raster_blocks_per_sm;  /* persistent raster grid = SMs x this, 1..resident limit */
    uint32_t tile_w, tile_h;        /* shade / composite pixel tile: tile_w in {16, 32, 64}, tile_w * tile_h == 256 */
    uint32_t filter_tile;           /* 0: 32 x 8, 1: 16 x 16 */
    float ms;                       /* output of hg_batch_tune: measured frame time of this shape */
} hg_batch_tuning;

typedef enum hg_batch_mode {
    HG_BATCH_GRAPH = 0,     /* replay the captured graph (recaptured when shapes or shade settings change) */
    HG_BATCH_LAUNCHES = 1,  /* the same batched launches issued directly */
    HG_BATCH_SEPARATE = 2   /* hg_groom_frame per item (the unbatched path, for comparison) */
} hg_batch_mode;

hg_status hg_batch_create(hg_ctx* ctx, const hg_batch_item* items, uint32_t count, hg_batch** out);
void hg_batch_destroy(hg_batch* batch);
/* Uniforms of one item: camera params (pass_mode.x 0, screen = the item's
 * size) and, when the item has a map, DOM params (pass_mode.x 1, screen and
 * dom_info = the map size; camera flags[3] must be 1).  All items must agree
 * on flags[1] (filter) and pass_mode.z (reverse Z).  Waits for the previous
 * frame to finish reading the pinned uniforms. */
hg_status hg_batch_set_params(hg_batch* batch, uint32_t item, const hg_hair_params* camera,
                              const hg_hair_params* dom);
/* One frame of every item: clear, lod, scan, generate, raster (camera + DOM
 * depth, then DOM layers), shade, filter, clear colour, composite.  shade:
 * lights as for hg_shade (shade_model 0 only).  Every item's params must have
 * been set. */
hg_status hg_batch_frame(hg_batch* batch, const hg_shade_desc* shade, hg_batch_mode mode);
/* One frame of batched launches with events between its phases: ms[0..4) =
 * setup (clears, lod, scan, generate), raster (camera + DOM depth, DOM
 * layers), shade, filter + colour clear + composite.  Synchronous. */
hg_status hg_batch_profile(hg_batch* batch, const hg_shade_desc* shade, float* ms);
/* Kernel launches one frame issues in `mode`. */
hg_status hg_batch_launches(hg_batch* batch, hg_batch_mode mode, uint32_t* launches);
/* Autotuner: times graph frames over a set of launch shapes (coordinate
 * search over raster chunk x grid, pixel tile, filter tile), keeps the
 * fastest, and reports every shape tried in results[0..*count) (up to
 * capacity). */
hg_status hg_batch_tune(hg_batch* batch, const hg_shade_desc* shade, hg_batch_tuning* results, uint32_t capacity,
                        uint32_t* count);
hg_status hg_batch_set_tuning(hg_batch* batch, const hg_batch_tuning* tuning);
hg_status hg_batch_get_tuning(hg_batch* batch, hg_batch_tuning* tuning);
/* An item's target (the hg_buffer_id kinds) as a device pointer and size. */
hg_status hg_batch_buffer(hg_batch* batch, uint32_t item, hg_buffer_id which, void** ptr, size_t* bytes);
/* Copy an item's target to host memory (bytes must equal its size); synchronous. */
hg_status hg_batch_copy_out(hg_batch* batch, uint32_t item, hg_buffer_id which, void* host, size_t bytes);
/* The same copy on the context's copy stream, returning at once (see
 * hg_copy_out_async; hg_copy_wait waits for it).  The next batched frame runs
 * its passes up to shading at once and waits for the copies only before it
 * writes the colour and depth targets. */
hg_status hg_batch_copy_out_async(hg_batch* batch, uint32_t item, hg_buffer_id which, void* host, size_t bytes);

/* ---------------------------------------------------------------- learned shading surrogate */

/* A small network that stands in for the Karis-fit lobes of shade.wesl:94-190
 * (no counterpart in the reference).  Inputs (10): sin theta_i, sin theta_o,
 * cos phi, sin phi, sigma_a (rgb), beta_m, beta_n, eta.  Outputs (12): the
 * lobes R, TT, TRT and the local back-scattering B, rgb each.  Architecture
 * 10 -> 64 -> 64 -> 64 -> 64 -> 12, ReLU, FP16 weights and activations with
 * FP32 accumulation; the network predicts log1p(lobe / 1e-3).  Parameters
 * are HG_MLP_PARAMS floats: W1[64][16] b1[64] W2[64][64] b2[64] W3[64][64]
 * b3[64] W4[64][64] b4[64] W5[16][64] b5[16] (W[out][in]; the padding
 * columns 10..15 of W1 and rows 12..15 of W5 and b5 stay zero).  A surrogate
 * works on its context's stream; destroy it before the context. */
#define HG_MLP_PARAMS 14608u
#define HG_MLP_INPUTS 10u
#define HG_MLP_OUTPUTS 12u
/* The compact network: 10 -> 32 -> 32 -> 3, the same inputs and roundings;
 * its 3 outputs are the per-light BSDF R + TT + TRT + 0.7 B (rgb) that the
 * shade pass adds at zero deep-opacity depth, as log1p(bsdf / 1e-3).
 * HG_MLP_COMPACT_PARAMS floats W1[32][16] b1[32] W2[32][32] b2[32] W3[16][32]
 * b3[16] (padding columns 10..15 of W1 and rows 3..15 of W3 and b3 stay
 * zero).  Trained on the same twelve-lobe targets, from which it forms the
 * three BSDF targets.  Shade model 3 evaluates it. */
#define HG_MLP_COMPACT_PARAMS 2128u
#define HG_MLP_ARCH_DEEP 0u     /* 4 x 64, HG_MLP_PARAMS */
#define HG_MLP_ARCH_COMPACT 1u  /* 2 x 32, HG_MLP_COMPACT_PARAMS */

typedef struct hg_mlp hg_mlp;

hg_status hg_mlp_create(hg_ctx* ctx, hg_mlp** out);   /* the 4 x 64 network; parameters start at zero */
/* A surrogate of the given HG_MLP_ARCH_*; parameters start at zero. */
hg_status hg_mlp_create_arch(hg_ctx* ctx, uint32_t arch, hg_mlp** out);
void hg_mlp_destroy(hg_mlp* mlp);
/* Number of parameters of the surrogate's architecture (0 for NULL). */
uint32_t hg_mlp_param_count(const hg_mlp* mlp);
/* Outputs per sample: 12 lobes (4 x 64 network) or 3 BSDF channels (compact). */
uint32_t hg_mlp_output_count(const hg_mlp* mlp);
/* Host float[count], count == hg_mlp_param_count; resets the optimiser state. */
hg_status hg_mlp_set_params(hg_mlp* mlp, const float* params, uint32_t count);
hg_status hg_mlp_get_params(hg_mlp* mlp, float* params, uint32_t count);
/* Training samples with FP64 lobes (Gauss-Legendre integration of the
 * Marschner/d'Eon azimuthal scattering, Zinke back-scattering) at the
 * longitudinal tilt `tilt`.  Sample k is a pure function of (seed, first + k).
 * Device buffers: inputs float[count][10]; targets float[count][12] =
 * log1p(lobe / 1e-3) (nullable); lobes double[count][12] (nullable). */
hg_status hg_mlp_samples(hg_ctx* ctx, uint64_t seed, uint64_t first, uint32_t count, float tilt, float* inputs,
                         float* targets, double* lobes);
/* Network evaluation.  Device buffers: inputs float[count][10]; lobes
 * float[count][k] (decoded, nullable); net float[count][k] (raw outputs,
 * nullable); k = hg_mlp_output_count. */
hg_status hg_mlp_infer(hg_mlp* mlp, const float* inputs, uint32_t count, float* lobes, float* net);
/* The same evaluation on the tcgen05 tensor cores: 128 rows per MMA,
 * accumulators in tensor memory, biases as two extra FP16 (high, low)
 * product columns.  Outputs match hg_mlp_infer to FP16 rounding.  4 x 64
 * network only (HG_INVALID_ARG for the compact one). */
hg_status hg_mlp_infer_tc(hg_mlp* mlp, const float* inputs, uint32_t count, float* lobes, float* net);
/* Gradient of the sum over samples and outputs of (net - target)^2 for one
 * batch (device inputs/targets), into host float[hg_mlp_param_count]; the loss sum
 * into *loss (nullable).  Parameters are unchanged.  Targets are always the
 * twelve transformed lobes of hg_mlp_samples (float[count][12]); the compact
 * network's targets are the three BSDF channels formed from them. */
hg_status hg_mlp_gradients(hg_mlp* mlp, const float* inputs, const float* targets, uint32_t count, float* grad,
                           float* loss);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the mean squared error
 * of one batch (device inputs/targets).  loss_sum: nullable device float that
 * receives the batch's sum of squared errors.  Asynchronous on the stream. */
hg_status hg_mlp_train_step(hg_mlp* mlp, const float* inputs, const float* targets, uint32_t count, float lr,
                            float* loss_sum);
/* The same 12 lobes from the Karis fits of shade.wesl:94-190 in FP32, as
 * shade model 0 evaluates them, for comparing the two models on one set of
 * inputs (device float[count][10] -> device float[count][12]; beta_n and eta
 * do not enter the fit). */
hg_status hg_karis_lobes(hg_ctx* ctx, const float* inputs, uint32_t count, float tilt, float* lobes);
/* Bind (or, with NULL, unbind) the surrogate that hg_shade_desc.shade_model
 * 1, 2 (4 x 64 network) or 3 (compact network) uses on this context. */
hg_status hg_mlp_bind(hg_ctx* ctx, hg_mlp* mlp);

#ifdef __cplusplus
} /* extern "C" */
#endif

#ifdef __cplusplus
static_assert(sizeof(hg_hair_params) == 432, "HairParams is 432 bytes (pipeline.rs:12)");
static_assert(sizeof(hg_gpu_bundle) == 16, "GpuBundle is 16 bytes");
static_assert(sizeof(hg_gpu_layer) == 32, "GpuLayer is 32 bytes");
static_assert(sizeof(hg_lod_record) == 16, "LodRecord is 16 bytes");
static_assert(sizeof(hg_strand_ref) == 16, "StrandRef is 16 bytes");
static_assert(sizeof(hg_light) == 112, "hg_light is 112 bytes");
static_assert(sizeof(hg_shadow_light) == 112, "ShadowLight is 112 bytes");
#else
_Static_assert(sizeof(hg_hair_params) == 432, "HairParams is 432 bytes (pipeline.rs:12)");
_Static_assert(sizeof(hg_gpu_bundle) == 16, "GpuBundle is 16 bytes");
_Static_assert(sizeof(hg_gpu_layer) == 32, "GpuLayer is 32 bytes");
_Static_assert(sizeof(hg_lod_record) == 16, "LodRecord is 16 bytes");
_Static_assert(sizeof(hg_strand_ref) == 16, "StrandRef is 16 bytes");
_Static_assert(sizeof(hg_light) == 112, "hg_light is 112 bytes");
_Static_assert(sizeof(hg_shadow_light) == 112, "ShadowLight is 112 bytes");
#endif

#endif /* HAIRGB_H */
