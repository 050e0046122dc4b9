/*
 * lucid_gb300 — C ABI of a GB300-native (sm_103a) replacement for LucidRaster's compute
 * rasterization passes (quad setup → bin counter → bin categorizer → bin dispatcher →
 * raster low/high with exact front-to-back OIT blending).
 *
 * Every entry point is plain C: plain pointers and sizes, no C++ or CUDA types in the
 * signatures. Streams are passed as `void*` holding a `cudaStream_t` (NULL = legacy default
 * stream). Geometry and output pointers are DEVICE pointers borrowed for the duration of the
 * call; the renderer owns every scratch buffer it needs (allocated once in lucid_create).
 *
 * All functions return lucid_status. Device-side capacity problems are not fatal: they are
 * recorded in lucid_info.error_code (read with lucid_get_info) and the affected bins are
 * painted red, as the reference paints overflowing high-load bins red
 * (data/shaders/raster_high.glsl:313-317).
 *
 * Reference interfaces replaced (paths are relative to the LucidRaster source tree):
 *   LucidRenderer::exConstruct   src/lucid_renderer.cpp:186-317   -> lucid_create
 *   LucidRenderer::render        src/lucid_renderer.cpp:319-350   -> lucid_render
 *   LucidRenderer::uploadInstances src/lucid_renderer.cpp:352-429 -> lucid_build_instances
 *   LucidRenderer::setupInputData src/lucid_renderer.cpp:431-451  -> (inside lucid_quad_setup)
 *   LucidRenderer::quadSetup     src/lucid_renderer.cpp:453-482   -> lucid_quad_setup
 *   LucidRenderer::computeBins   src/lucid_renderer.cpp:484-528   -> lucid_bin_count,
 *                                                                  lucid_bin_categorize,
 *                                                                  lucid_bin_dispatch
 *   LucidRenderer::rasterLow/High src/lucid_renderer.cpp:555-580  -> lucid_raster
 *   LucidRenderer::verifyInfo/getStats src/lucid_renderer.cpp:629-836 -> lucid_get_info
 *   FrustumInfo(const Camera&)   src/shading.cpp:46-74            -> lucid_make_config
 */
#ifndef LUCID_GB300_H
#define LUCID_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LUCID_ABI_VERSION 1

/* ---------------------------------------------------------------------------------------- */
/* Constants shared with the reference (data/shaders/shared/definitions.glsl:73-100)          */

#define LUCID_BIN_LEVELS_COUNT 5
#define LUCID_REJECTION_TYPE_COUNT 4
#define LUCID_TIMERS_COUNT 8
#define LUCID_STATS_COUNT 4
#define LUCID_INFO_MAX_DISPATCHES 256

#define LUCID_BIN_LEVEL_EMPTY 0
#define LUCID_BIN_LEVEL_MICRO 1
#define LUCID_BIN_LEVEL_LOW 2
#define LUCID_BIN_LEVEL_MEDIUM 3
#define LUCID_BIN_LEVEL_HIGH 4

/* InstanceData.flags bits (definitions.glsl:85-94, DrawCallOpt in src/lucid_base.h:140-142) */
#define LUCID_INST_HAS_VERTEX_COLORS 0x001u
#define LUCID_INST_HAS_VERTEX_TEX_COORDS 0x002u
#define LUCID_INST_HAS_VERTEX_NORMALS 0x004u
#define LUCID_INST_IS_OPAQUE 0x008u
#define LUCID_INST_TEX_OPAQUE 0x010u
#define LUCID_INST_HAS_UV_RECT 0x020u
#define LUCID_INST_HAS_ALBEDO_TEXTURE 0x040u
#define LUCID_INST_HAS_NORMAL_TEXTURE 0x080u
#define LUCID_INST_HAS_PBR_TEXTURE 0x100u
#define LUCID_INST_HAS_COLOR 0x200u

/* Rejection reasons (definitions.glsl:97-100) */
#define LUCID_REJECTION_TYPE_OTHER 0
#define LUCID_REJECTION_TYPE_BACKFACE 1
#define LUCID_REJECTION_TYPE_FRUSTUM 2
#define LUCID_REJECTION_TYPE_BETWEEN_SAMPLES 3

/* Largest instance the setup pass accepts (src/lucid_renderer.h:29 max_instance_quads). */
#define LUCID_MAX_INSTANCE_QUADS 1024

/* ---------------------------------------------------------------------------------------- */
/* Status codes                                                                              */

typedef enum lucid_status {
	LUCID_OK = 0,
	LUCID_INVALID_ARG = 1,
	LUCID_CAPACITY_EXCEEDED = 2,
	LUCID_CUDA_ERROR = 3,
	LUCID_TIMEOUT = 4,
	LUCID_NOT_SUPPORTED = 5,
	LUCID_OUT_OF_MEMORY = 6
} lucid_status;

/* lucid_info.error_code values (device-side, first error wins) */
#define LUCID_ERR_NONE 0u
#define LUCID_ERR_VISIBLE_QUADS 1u    /* more visible quads than options.max_visible_quads   */
#define LUCID_ERR_BIN_REFS 2u         /* bin quad/tri reference lists overflowed             */
#define LUCID_ERR_BAND_ENTRIES 3u     /* a 4-row band of a bin has too many triangle rows    */
#define LUCID_ERR_PIXEL_FRAGMENTS 4u  /* one pixel has more fragments than the sort capacity */
#define LUCID_ERR_INSTANCE_QUADS 5u   /* an instance has more than 1024 quads                */
#define LUCID_ERR_BIN_COUNT 6u        /* internal: bin work queue inconsistency              */
#define LUCID_ERR_VERTEX_INDEX 7u     /* a quad index is >= num_verts (quad rejected)        */

/* ---------------------------------------------------------------------------------------- */
/* Structures with the reference's memory layout                                             */

/* InstanceData (data/shaders/shared/structures.glsl:9-14): 16 bytes. */
typedef struct lucid_instance {
	int32_t index_offset;  /* offset (in u32 indices) of the instance's first quad in quads_ib */
	int32_t vertex_offset; /* added to every index of the instance                           */
	int32_t num_quads;     /* <= LUCID_MAX_INSTANCE_QUADS                                     */
	uint32_t flags;        /* LUCID_INST_* bits (low 16 bits used)                            */
} lucid_instance;

/* Frustum (structures.glsl:24-28), std140: 12 vec4 = 192 bytes. xyz used, w padding. */
typedef struct lucid_frustum {
	float ws_origins[4][4];
	float ws_dirs[4][4];
	float ws_origin0[4];
	float ws_dir0[4];
	float ws_dirx[4];
	float ws_diry[4];
} lucid_frustum;

/* Lighting (structures.glsl:16-21), std140: 64 bytes. */
typedef struct lucid_lighting {
	float ambient_color[4];
	float sun_color[4];
	float sun_dir[4];
	float sun_power, ambient_power;
	float _pad[2];
} lucid_lighting;

/* LucidConfig (structures.glsl:102-111), std140: 352 bytes.
 * view_proj_matrix is column-major (GLSL mat4: element [col][row] at index col*4+row). */
typedef struct lucid_config {
	lucid_frustum frustum;
	float view_proj_matrix[16];
	lucid_lighting lighting;
	float background_color[4];
	uint32_t enable_backface_culling;
	int32_t num_instances;
	int32_t instance_packet_size;
	uint32_t _pad;
} lucid_config;

/* LucidInfo (structures.glsl:70-99): identical layout for the first 1152 u32 words, followed
 * by 64 u32 words of GB300-specific status. In device memory the per-bin counter array
 * (10 * bin_count u32, definitions.glsl:117-129) follows this structure. */
typedef struct lucid_info {
	int32_t num_input_quads;
	int32_t num_visible_quads[2];
	int32_t num_counted_quads[2];
	int32_t bin_level_counts[LUCID_BIN_LEVELS_COUNT];

	uint32_t a_small_bins, a_high_bins;
	uint32_t a_setup_work_groups;
	uint32_t a_dummy_counter;

	uint32_t num_binning_dispatches[3];
	uint32_t bin_level_dispatches[LUCID_BIN_LEVELS_COUNT][3];

	uint32_t num_rejected_quads[LUCID_REJECTION_TYPE_COUNT];

	uint32_t setup_timers[LUCID_TIMERS_COUNT];
	uint32_t raster_timers[LUCID_TIMERS_COUNT];
	uint32_t bin_dispatcher_timers[LUCID_TIMERS_COUNT];

	/* stats[0]: fragments, stats[1]: half-block-tris, stats[2]: invalid pixels */
	uint32_t stats[LUCID_STATS_COUNT];

	int32_t dispatcher_first_batch[2][LUCID_INFO_MAX_DISPATCHES];
	int32_t dispatcher_num_batches[2][LUCID_INFO_MAX_DISPATCHES];

	int32_t temp[64];

	/* ---- GB300 extension (not in the reference) ---- */
	uint32_t error_code;      /* LUCID_ERR_*                                               */
	uint32_t error_detail[3]; /* e.g. bin id / count / capacity of the first error        */
	uint32_t raster_work_counter;
	uint32_t num_bin_quad_refs; /* sum of per-bin quad counts                             */
	uint32_t num_bin_tri_refs;  /* sum of per-bin tri counts                              */
	uint32_t max_pixel_fragments;
	uint64_t num_fragments;   /* 64-bit fragment count (stats[0] wraps above 2^32)        */
	uint64_t num_hblock_tris; /* 64-bit stats[1]                                          */
	uint32_t num_band_entries;
	uint32_t num_views;
	uint64_t raster_windows;          /* depth windows processed by the raster pass         */
	uint64_t raster_window_fragments; /* fragments sorted in those windows                  */
	uint32_t raster_radix_windows;    /* windows sorted by the block-wide radix fallback    */
	uint32_t raster_light_bins;       /* bins rastered by the light path (<= 32 fragments
	                                   * per pixel; one warp per row)                        */
	uint64_t raster_blended_fragments;/* fragments blended: each pixel's fragments up to the
	                                   * one that brings T to 0 (forward frames)             */
	uint32_t ext_reserved[42];
} lucid_info;

#define LUCID_INFO_REFERENCE_WORDS 1152
#define LUCID_INFO_WORDS 1216

/* ---------------------------------------------------------------------------------------- */
/* Renderer options (LucidRenderOpt in src/lucid_renderer.h:10-13 plus GB300 limits)          */

#define LUCID_OPT_TIMERS 0x01u            /* clock64 section timers into lucid_info.*_timers */
#define LUCID_OPT_ADDITIVE_BLENDING 0x02u /* out += rgb*a (shading.glsl:276-277)               */
#define LUCID_OPT_ALPHA_THRESHOLD 0x04u   /* stop a pixel once T < 1/128 (shading.glsl:62)     */
#define LUCID_OPT_VISUALIZE_ERRORS 0x08u  /* reference-order mode: depth-4 window, pixels whose
                                           * samples arrive too far out of order are red and
                                           * counted in lucid_info.stats[2] (shading.glsl:186-264) */
#define LUCID_OPT_REFERENCE_ORDER 0x20u   /* the reference's own order and blend instead of the
                                           * exact order: 22/18-bit block keys, 3-deep depth
                                           * window, lit sRGB RGBA8 shading (raster_low/high.glsl,
                                           * shading.glsl); not with ALPHA_THRESHOLD, gradients or
                                           * batches */
#define LUCID_OPT_SORTED_BIN_LISTS 0x40u  /* binning: sort every bin's quad and tri reference
                                           * lists by slot after the dispatcher, so that the
                                           * lists are reproducible bit for bit (the order
                                           * inside a bin otherwise follows the dispatcher's
                                           * atomics, as in the reference; the image does not
                                           * depend on it) */
#define LUCID_OPT_PIXEL_BLEND 0x10u       /* raster pass stores each pixel's sorted fragment
                                           * list; a pixel-parallel kernel shades and blends it
                                           * (same image bits; lucid_autotune picks it per scene) */

typedef struct lucid_options {
	uint32_t flags;            /* LUCID_OPT_*                                                  */
	int32_t bin_size;          /* 32 or 64 pixels (src/lucid_renderer.cpp:190: m_bin_size, whose
	                            * 64 option is commented out in the reference); 64-pixel bins
	                            * are rastered as four 32x32 tiles. The reference-order mode and
	                            * lucid_raster_dump_bins need 32. Buffers are sized for 32.  */
	int32_t max_input_quads;   /* capacity of the per-input-quad classification buffer        */
	int32_t max_visible_quads; /* MAX_VISIBLE_QUADS (definitions.glsl:54)                      */
	int32_t max_instances;     /* src/lucid_renderer.h:28 (64K)                                */
	int32_t low_high_threshold;/* bins with >= this many tris are HIGH (bin_categorizer.glsl:72)*/
	int32_t max_bin_refs;      /* capacity of each of the bin quad / bin tri lists             */
	int32_t band_capacity;     /* triangle rows per 4-row band of a bin (raster scratch)       */
	int32_t binning_ctas;      /* CTAs of bin_count / bin_dispatch (0 = 2 per SM)              */
	int32_t raster_ctas_per_sm;/* 0 = as many as fit                                           */
	int32_t max_views;         /* views of lucid_render_batch                                  */
	int32_t grad_store_fragments; /* fragment store of lucid_render_forward_grad: 0 = grows on
	                               * demand, > 0 = fixed capacity, < 0 = none (the backward pass
	                               * recomputes the fragment lists instead of reading them)      */
	int32_t slab_fragments;    /* raster: fragments per unfinished pixel a depth slab aims at
	                            * (0 = 165; a large value counts every key at once)            */
	int32_t light_max_pixel;   /* raster: a bin whose pixels have at most this many fragments
	                            * takes the light path (one warp per row, passes of the 32
	                            * nearest fragments per pixel, stop at T == 0); deeper bins take
	                            * the depth-window path. 0 = 64, < 0 = light path off          */
	int32_t reserved[2];
} lucid_options;

/* ---------------------------------------------------------------------------------------- */
/* Per-frame inputs (RenderContext, src/lucid_base.h:72-84, as used by
 * src/lucid_renderer.cpp:352-451). All array pointers are DEVICE pointers.                   */

#define LUCID_COLOR_RGBA8 0   /* u32 per vertex, R in the low byte (IColor)                   */
#define LUCID_COLOR_RGBA16F 1 /* 4 x IEEE half per vertex                                     */
#define LUCID_COLOR_RGBA32F 2 /* 4 x float per vertex                                         */

typedef struct lucid_frame_inputs {
	const float* positions;          /* float3 per vertex (world space)                         */
	const void* colors;              /* per-vertex colours, layout given by color_format        */
	int32_t color_format;            /* LUCID_COLOR_*                                           */
	int32_t num_verts;
	const uint32_t* quads_ib;        /* 4 u32 vertex indices per quad; a triangle is (a,b,c,c)  */
	int32_t num_quads;               /* total input quads = sum of instances' num_quads         */
	int32_t num_instances;
	const lucid_instance* instances; /* device array of num_instances                           */
	const uint32_t* instance_colors; /* RGBA8 per instance (used with LUCID_INST_HAS_COLOR)     */
	const float* tri_opacity;        /* optional: per input triangle (quad*2+second), may be 0  */
	const lucid_config* config;      /* HOST pointer, copied into the renderer's buffer         */
	/* optional shading inputs (shading.glsl:125-176; NULL when no instance uses them):        */
	const float* tex_coords;         /* float2 per vertex (LUCID_INST_HAS_ALBEDO_TEXTURE)       */
	const float* instance_uv_rects;  /* float4 per instance: uv min, uv size (LUCID_INST_HAS_UV_RECT) */
	const uint32_t* normals;         /* encoded normal per vertex (LUCID_INST_HAS_VERTEX_NORMALS:
	                                  * 10 bits per axis, (v - 512) / 511, funcs.glsl:61-66)    */
	const struct lucid_texture* opaque_texture;      /* HOST pointers to texture descriptors */
	const struct lucid_texture* transparent_texture;
} lucid_frame_inputs;

/* RGBA8 texture with its mip chain (the reference's opaque / transparent albedo atlases). texels:
 * device, the levels back to back, level l is max(1, width >> l) x max(1, height >> l) u32
 * (red in the low byte). Sampled trilinearly with repeat addressing. */
typedef struct lucid_texture {
	const uint32_t* texels;
	int32_t width, height;
	int32_t num_levels;
	int32_t _pad;
} lucid_texture;

/* Draw call of the host-side instance builder (SceneDrawCall, src/lucid_base.h:44-50). */
typedef struct lucid_draw_call {
	int32_t quad_offset;
	int32_t num_quads;
	uint32_t opts;          /* LUCID_INST_* bits of the draw call                                */
	uint32_t material_color;/* RGBA8; 0xffffffff means "no instance colour"                      */
} lucid_draw_call;

/* Simple perspective camera used to fill LucidConfig (stands in for libfwk Camera). The camera
 * looks down -Z of its own frame; pixel (x, y) maps to NDC (2x/W-1, 2y/H-1). */
typedef struct lucid_camera {
	float position[3];
	float right[3], up[3], forward[3]; /* orthonormal basis; forward is the view direction */
	float fov_y_radians;
	float near_plane, far_plane;
} lucid_camera;

/* View of a batched render (no reference counterpart). */
typedef struct lucid_view {
	int32_t width, height;
	lucid_frame_inputs inputs;
	float* out_rgba; /* device, width*height*4 floats */
} lucid_view;

typedef struct lucid_renderer lucid_renderer;

/* ---------------------------------------------------------------------------------------- */
/* Host-only helpers (no GPU needed)                                                         */

const char* lucid_status_string(lucid_status status);
/* Text of the last error raised on the calling thread (empty string if none). */
const char* lucid_last_error_string(void);
int lucid_abi_version(void);
lucid_status lucid_default_options(lucid_options* out);

/* Splits draw calls into instances of at most 1024 quads, as LucidRenderer::uploadInstances
 * does (src/lucid_renderer.cpp:352-429). Writes up to max_instances records and returns the
 * number written in *out_count (truncated like the reference, which resizes to max_instances).
 * out_colors receives one RGBA8 instance colour per instance (may be NULL). */
lucid_status lucid_build_instances(const lucid_draw_call* draw_calls, int32_t num_draw_calls,
								   lucid_instance* out_instances, uint32_t* out_colors,
								   int32_t max_instances, int32_t* out_count,
								   int32_t* out_num_quads);

/* Fills a LucidConfig from a camera, as FrustumInfo (src/shading.cpp:46-74) and
 * LucidRenderer::setupInputData (src/lucid_renderer.cpp:439-446) do. background_rgba may be
 * NULL (0,0,0,1). Lighting is set to SceneLighting::makeDefault (src/shading.cpp:26-34). */
lucid_status lucid_make_config(const lucid_camera* camera, int32_t width, int32_t height,
							   const float* background_rgba, int32_t backface_culling,
							   lucid_config* out);

/* ---------------------------------------------------------------------------------------- */
/* Renderer                                                                                  */

lucid_status lucid_create(const lucid_options* options, int32_t width, int32_t height,
						  lucid_renderer** out);
lucid_status lucid_destroy(lucid_renderer* renderer);

/* Whole frame: quad setup, bin count, categorize, dispatch, raster. Asynchronous on `stream`,
 * no host synchronisation, graph-capturable. out_rgba: device, width*height*4 floats, row y
 * of the image at offset y*width*4. */
lucid_status lucid_render(lucid_renderer* renderer, const lucid_frame_inputs* inputs,
						  float* out_rgba, void* stream);

/* Pass-level entry points (one per reference compute pass). They operate on the renderer's
 * buffers, so a caller can inspect intermediates between them. lucid_quad_setup also resets
 * the info block and uploads the config (setupInputData). */
lucid_status lucid_quad_setup(lucid_renderer* renderer, const lucid_frame_inputs* inputs,
							  void* stream);
lucid_status lucid_bin_count(lucid_renderer* renderer, void* stream);
lucid_status lucid_bin_categorize(lucid_renderer* renderer, void* stream);
lucid_status lucid_bin_dispatch(lucid_renderer* renderer, void* stream);
lucid_status lucid_raster(lucid_renderer* renderer, const lucid_frame_inputs* inputs,
						  float* out_rgba, void* stream);

/* Synchronises `stream` and copies the info block (and, if bin_counters is non-NULL, the
 * 10*bin_count per-bin counters) to host memory. */
lucid_status lucid_get_info(lucid_renderer* renderer, lucid_info* out_info,
							uint32_t* bin_counters, void* stream);

/* Read-only view of internal buffers, for parity tests and statistics. Synchronises `stream`
 * and copies min(bytes, buffer size) bytes of buffer `which` into host_dst. *out_bytes (may be
 * NULL) receives the buffer's size. */
#define LUCID_BUF_QUAD_AABBS 0    /* u32 per visible quad slot (MAX_VISIBLE_QUADS)             */
#define LUCID_BUF_TRI_BARY 1      /* uvec4 x2 per tri slot                                     */
#define LUCID_BUF_TRI_SCAN 2      /* uvec4 x2 per tri slot                                     */
#define LUCID_BUF_TRI_DEPTH 3     /* uvec4 per tri slot                                        */
#define LUCID_BUF_QUAD_COLORS 4   /* uvec4 per quad slot (RGBA8 vertex colours)                */
#define LUCID_BUF_TRI_NORMALS 5   /* u32 per tri slot                                          */
#define LUCID_BUF_QUAD_SOURCE 6   /* u32 per quad slot: input quad index                       */
#define LUCID_BUF_BIN_QUADS 7     /* u32 per bin quad reference                                */
#define LUCID_BUF_BIN_TRIS 8      /* u32 per bin tri reference                                 */
#define LUCID_BUF_QUAD_VERTS 9    /* uvec4 per quad slot: vertex indices                       */
lucid_status lucid_download_buffer(lucid_renderer* renderer, int32_t which, void* host_dst,
								   size_t bytes, size_t* out_bytes, void* stream);

/* Verification mode of the raster pass: renders like lucid_raster and also records, for each
 * pixel, the number of fragments and the input primitive ids (quad*2+second) of its first
 * max_per_pixel fragments in exact blend order (nearest first, ties by primitive id).
 * Host outputs: counts[width*height], prims[width*height*max_per_pixel]. Synchronous. */
lucid_status lucid_raster_dump(lucid_renderer* renderer, const lucid_frame_inputs* inputs,
							   float* out_rgba, int32_t max_per_pixel, int32_t* host_counts,
							   int32_t* host_prims, void* stream);

/* The same verification mode for full-size frames: renders the whole frame into out_rgba and
 * records the counts and first max_per_pixel prims of the pixels of the listed bins only
 * (bins: HOST array of num_bins distinct bin ids, bin = by * bins_x + bx). Host outputs:
 * host_counts[num_bins * 1024], host_prims[num_bins * 1024 * max_per_pixel]; bin k's local
 * pixel (x, y) is entry k * 1024 + y * 32 + x (pixels outside the viewport read as count 0,
 * prims -1; so do list entries past a pixel's count). Synchronous. Not in the reference-order mode. */
lucid_status lucid_raster_dump_bins(lucid_renderer* renderer, const lucid_frame_inputs* inputs,
									float* out_rgba, const int32_t* bins, int32_t num_bins,
									int32_t max_per_pixel, int32_t* host_counts, int32_t* host_prims,
									void* stream);

/* Differentiable forward (no reference counterpart): lucid_render that also records each
 * pixel's colour accumulated in FP64 and keeps the frame's bin lists for lucid_render_backward.
 * out_rgba (device, width*height*4 floats) receives clamp(FP64 colour rounded to FP32) with
 * alpha 1, the function whose gradient lucid_render_backward computes; it differs from
 * lucid_render's FP32 blend by the FP32 rounding of that blend (~1e-6). Front-to-back blend
 * only (LUCID_OPT_ADDITIVE_BLENDING and LUCID_OPT_ALPHA_THRESHOLD are rejected). */
lucid_status lucid_render_forward_grad(lucid_renderer* renderer, const lucid_frame_inputs* inputs,
									   float* out_rgba, void* stream);

/* Backward pass (no reference counterpart): given dL/dimage (device, width*height*4 floats,
 * alpha channel ignored) of the image of lucid_render_forward_grad, accumulates
 * dL/d(vertex RGBA) into dvertex_rgba (device, num_verts*4 floats, 16-byte aligned;
 * LUCID_COLOR_RGBA32F colours only) and dL/d(triangle opacity) into dtri_opacity (device, num_quads*2 floats;
 * requires inputs->tri_opacity). Either output may be NULL; gradients are ADDED. Channels whose
 * unclamped colour lies outside [0, 1] pass no gradient. Positions are not differentiated.
 * When the last pass on this renderer was lucid_render_forward_grad with an identical inputs
 * struct and config (same pointers, contents unchanged since), its bin lists and per-pixel
 * colours are reused; otherwise setup, binning and the FP64 colour pass are recomputed first. */
lucid_status lucid_render_backward(lucid_renderer* renderer, const lucid_frame_inputs* inputs,
								   const float* dl_dimage, float* dvertex_rgba,
								   float* dtri_opacity, void* stream);

/* Batched forward (no reference counterpart): renders num_views independent views (each with
 * its own size, geometry, colour format and config) with one launch per pass for all views:
 * setup and binning kernels whose CTA ranges map to views, and one persistent raster kernel
 * over the bins of every view (HIGH bins of all views first). Each view's image is bit-identical
 * to lucid_render of that view alone. views is a HOST array; num_views <= options.max_views
 * (at most 256); every view fits the renderer's width/height; the views' input quads together
 * fit options.max_visible_quads and max_input_quads; their bin references share
 * options.max_bin_refs. The frame is recorded once per batch topology (view count, sizes, quad
 * and instance counts) as a CUDA graph and replayed by later calls: the first call of a new
 * topology synchronises `stream` and allocates; later calls only stage changed view parameters
 * (pointers, configs) and launch the graph. Input contents may change freely between calls.
 * Must not be called while `stream` is being captured. Not re-entrant across streams.
 * Per-view device statistics and errors: lucid_get_batch_info. */
lucid_status lucid_render_batch(lucid_renderer* renderer, const lucid_view* views,
								int32_t num_views, void* stream);

/* Copies (synchronising `stream`) the lucid_info of view `view` of the last lucid_render_batch. */
lucid_status lucid_get_batch_info(lucid_renderer* renderer, int32_t view, lucid_info* out, void* stream);

/* Result of lucid_autotune. */
typedef struct lucid_tuning {
	uint32_t pixel_blend;       /* 1: LUCID_OPT_PIXEL_BLEND chosen                               */
	int32_t low_high_threshold; /* bins with >= this many tris are rastered first (HIGH)        */
	int32_t binning_ctas;       /* CTAs of the bin counter / dispatcher                         */
	int32_t num_candidates;     /* configurations timed                                         */
	float frame_ms;             /* median frame time of the winner                               */
	float default_ms;           /* median frame time of the renderer's options before tuning     */
	int32_t light_max_pixel;    /* deepest pixel of a bin rastered one warp per row (-1: none)  */
	int32_t bin_size;           /* bins of 32 or 64 pixels                                       */
} lucid_tuning;

/* Autotuner (no reference counterpart): times lucid_render of `inputs` into scratch_rgba
 * (device, width*height*4 floats) under candidate configurations, by coordinate descent over
 * the bin size (32 or 64 pixels; not in the reference-order mode), the blend strategy
 * (raster-pass blend or LUCID_OPT_PIXEL_BLEND; not for renderers with options.max_views > 1,
 * whose batches blend in the raster pass), the LOW/HIGH threshold (256, 1024, 4096), the
 * binning CTAs (1 or 2 per SM, within options.binning_ctas) and the per-bin raster path
 * (options.light_max_pixel: -1, 32, 64, 128, 256; bins up to that depth are rastered one warp
 * per row, deeper ones by CTA-wide depth windows); CUDA events on `stream`, median of 3 frames
 * after one warm-up frame each. The winner is stored in the renderer's options and returned in
 * *out (may be NULL). Synchronous. Raster CTAs are one per SM (shared memory). */
lucid_status lucid_autotune(lucid_renderer* renderer, const lucid_frame_inputs* inputs,
							float* scratch_rgba, lucid_tuning* out, void* stream);

/* Autotuner of batched frames (no reference counterpart): the same coordinate descent as
 * lucid_autotune (bin size, LOW/HIGH threshold, binning CTAs, per-bin raster path; not the
 * blend strategy), timing lucid_render_batch of `views` (which it renders into their
 * out_rgba). A batch's best options are not those of any one of its views: deep small views
 * and shallow large ones pull the per-bin raster path different ways. Synchronous. */
lucid_status lucid_autotune_batch(lucid_renderer* renderer, const lucid_view* views, int32_t num_views,
								  lucid_tuning* out, void* stream);

/* Quad generator (replaces triNeighbours / quadNodes / genQuads, src/quad_generator.cpp:18-201,
 * as used by Scene::generateQuads, src/scene.cpp:237-246): pairs triangles that share an edge
 * into quads, the quads_ib format of lucid_frame_inputs. positions: device, num_verts x float3;
 * tris: device, num_tris x 3 vertex indices; out_quads: device, capacity num_tris x 4 u32.
 * Writes, in tri order, each tri's selected quad {a, opposite, b, c}, nothing for the second
 * tri of a selected quad, or the degenerate quad (a, b, c, c); *out_num_quads (host) receives the
 * count, *out_num_degenerate (host, may be NULL) the degenerate ones. Quads are chosen by a greedy
 * independent set over score = conflicts - squareness * square_weight (the reference's weight is
 * 1.0, src/scene_convert.cpp:36) taken in the fixed order of the initial scores (ties by quad
 * index); the reference lowers scores as the greedy proceeds, which is sequential. Synchronous;
 * allocates its scratch. LUCID_INVALID_ARG for a vertex index outside [0, num_verts). */
lucid_status lucid_quad_generate(const float* positions, int32_t num_verts, const int32_t* tris,
								 int32_t num_tris, float square_weight, uint32_t* out_quads,
								 int32_t* out_num_quads, int32_t* out_num_degenerate, void* stream);

/* ---------------------------------------------------------------------------------------- */
/* Binning without allocation. No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc: a host whose allocator owns all device memory, or
 * code that records GPU work while allocating is not allowed. Runs the bin counter,
 * categorizer and dispatcher on caller-provided device buffers; their remaining scratch (the
 * counter's per-CTA bin histograms, the status block, the bin work list) is a static device
 * array of 1 MiB held by every GPU that loads the library.
 *
 * Inputs (device): quad_aabbs (max_visible_quads u32, layout of LUCID_BUF_QUAD_AABBS) and
 * tri_scan (2*max_visible_quads records of 8 u32, LUCID_BUF_TRI_SCAN, 16-byte aligned) of a
 * quad setup with num_small_quads / num_large_quads visible quads.
 * Outputs (device): bin_counters (10 * bin count u32, the g_counts layout), bin_quads and
 * bin_tris (max_bin_refs u32 each; every bin's references in slot order, as with
 * LUCID_OPT_SORTED_BIN_LISTS), optional info_out (one lucid_info: level counts, error code).
 * Limit: at most LUCID_NOALLOC_MAX_BINS 32x32 bins (e.g. 1920x1080 = 2040 bins); larger
 * viewports return LUCID_CAPACITY_EXCEEDED. All calls share the static scratch: calls whose
 * work overlaps on the GPU race; calls on one stream are ordered. The first call on each
 * device looks the scratch up with cudaGetSymbolAddress, so make it before any stream capture.
 * Calls no cudaMalloc or cudaFree. */
#define LUCID_NOALLOC_MAX_BINS 2048
lucid_status lucid_bin_noalloc(const uint32_t* quad_aabbs, const uint32_t* tri_scan,
							   int32_t num_small_quads, int32_t num_large_quads,
							   int32_t max_visible_quads, int32_t width, int32_t height,
							   int32_t low_high_threshold, uint32_t* bin_counters,
							   uint32_t* bin_quads, uint32_t* bin_tris, int32_t max_bin_refs,
							   lucid_info* info_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LUCID_GB300_H */
