/*
 * Scalar CPU oracle of LucidRaster's compute rasterization path.
 *
 * TEST INFRASTRUCTURE ONLY: this library is the checker for the CUDA path and the timed CPU
 * baseline. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 * Nothing in the lucid_gb300 package links, imports or calls it.
 *
 * Parity status: the reference runs only as Vulkan GLSL compute shaders on top of libfwk
 * (absent) and has no tests or golden vectors. Its setup, bin-counter and low-level row-span
 * functions are compiled as C++ from its shader sources (oracle/ref_build.py, oracle/_ref), and
 * this restatement's setup records, per-bin counts and per-pixel fragment counts are checked
 * bit for bit against them (tests/test_oracle_ref_pin.py). The exact per-pixel order and blend
 * (an extension of the reference's approximate window) are checked against hand-derived
 * known-answer cases, the FP64 blend and the reference's run-time invariants
 * (src/lucid_renderer.cpp:629-707 offset checks).
 *
 * Layout conventions shared with the CUDA path (both follow the reference):
 *   - quad slot k < num_visible[0] holds the k-th visible small quad in input order;
 *     slot MAX_VISIBLE_QUADS-1-k the k-th visible large quad (quad_setup.glsl:437-444),
 *   - tri slot = quad slot * 2 + second_tri,
 *   - records follow quad_setup.glsl:274-340 bit for bit.
 */
#ifndef LUCID_ORACLE_H
#define LUCID_ORACLE_H

#include <stdint.h>
#include "../include/lucid_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_inputs {
	int32_t width, height;
	int32_t max_visible_quads;
	int32_t low_high_threshold; /* 1024 in the reference */
	uint32_t flags;             /* LUCID_OPT_* (additive blending, alpha threshold)          */
	int32_t order_mode;         /* 0: exact per-pixel order, 1: reference 3-deep window      */
	const float* positions;
	const void* colors;
	int32_t color_format;
	int32_t num_verts;
	const uint32_t* quads_ib;
	int32_t num_quads;
	int32_t num_instances;
	const lucid_instance* instances;
	const uint32_t* instance_colors;
	const float* tri_opacity;
	const lucid_config* config;
	/* optional shading inputs as in lucid_frame_inputs (host memory; texture texels too) */
	const float* tex_coords;
	const float* instance_uv_rects;
	const uint32_t* normals;
	const lucid_texture* opaque_texture;
	const lucid_texture* transparent_texture;
	/* raster only these bins (ascending bin ids); NULL = all bins */
	const int32_t* bin_subset;
	int32_t num_bin_subset;
	int32_t num_threads; /* raster worker threads (>= 1) */
} oracle_inputs;

typedef struct oracle_outputs {
	/* ---- quad setup (sizes: MAX_VISIBLE_QUADS quads, 2*MAX_VISIBLE_QUADS tris) ---- */
	int32_t num_input_quads;
	int32_t num_visible[2];
	uint32_t rejected[LUCID_REJECTION_TYPE_COUNT];
	uint32_t error_code;
	uint32_t num_binning_dispatches;
	uint32_t* quad_aabbs;   /* [mvq]     may be NULL */
	uint32_t* quad_source;  /* [mvq]                 */
	uint32_t* quad_colors;  /* [mvq*4]               */
	uint32_t* quad_verts;   /* [mvq*4]               */
	uint32_t* tri_bary;     /* [2*mvq*8]             */
	uint32_t* tri_scan;     /* [2*mvq*8]             */
	uint32_t* tri_depth;    /* [2*mvq*4]             */
	uint32_t* tri_normals;  /* [2*mvq]               */
	/* ---- binning ---- */
	int32_t bin_count, bin_count_x, bin_count_y;
	uint32_t* bin_counters;    /* [10*bin_count] like g_counts (definitions.glsl:117-129)     */
	uint32_t* bin_quads;       /* [bin quad refs], per bin sorted by slot                     */
	uint32_t* bin_tris;        /* [bin tri refs], per bin sorted by slot                      */
	int64_t bin_refs_capacity; /* capacity of bin_quads / bin_tris arrays                     */
	int64_t num_bin_quads, num_bin_tris;
	int32_t bin_level_counts[LUCID_BIN_LEVELS_COUNT];
	/* ---- raster ---- */
	float* image;          /* [h*w*4] may be NULL                                           */
	double* image64;       /* [h*w*4] FP64 blend of the same ordered fragments, may be NULL */
	int32_t* frag_counts;  /* [h*w] may be NULL                                              */
	int32_t* frag_prims;   /* [h*w*max_per_pixel] may be NULL                                */
	int32_t max_per_pixel;
	uint64_t num_fragments;
	uint64_t num_hblock_tris;
	uint32_t max_pixel_fragments;
	uint64_t invalid_pixels; /* reference-order mode: pixels whose window overflowed */
	/* exact mode with bin_subset: frag_counts / frag_prims hold only the subset's bins, bin k
	 * of the subset at [k * 1024 + local pixel] (image and image64 stay full-frame)   */
	int32_t dump_by_subset;
} oracle_outputs;

/* Runs setup, binning and (if out->image or out->frag_counts is set) the raster pass.
 * Returns 0 on success, nonzero on invalid arguments. */
int oracle_run(const oracle_inputs* in, oracle_outputs* out);

int oracle_version(void);

/* ---- reference-order shading and reduction, one sample or one pixel at a time ----
 * Test entry points that pin the reference-order mode to the reference's own shadeSample,
 * reduceSample and finishReduceSamples (tests/test_oracle_ref_pin.py).
 * oracle_ref_shade: setup of `in`, then shadeRef of each (px[i], py[i], tris[i]): RGBA8 colour
 * and depth (inv_ray_pos). oracle_ref_reduce: one pixel's samples through RefReduce (3-deep
 * window) in segments seg[i] (non-decreasing; the colour is saturated at each segment's end),
 * then finish over background[0..3]. oracle_ref_pow: the pow of the sRGB conversions. */
int oracle_ref_shade(const oracle_inputs* in, int32_t n, const int32_t* px, const int32_t* py, const uint32_t* tris,
					 uint32_t* colors, float* depths);
int oracle_ref_reduce(const float* background, int32_t n, const uint32_t* colors, const float* depths,
					  const int32_t* seg, float* rgba);
float oracle_ref_pow(float x, float y);

/* ---- FP64 gradient model (checker of lucid_render_backward) ----
 * Builds the exact per-pixel fragment lists of the scene (coverage, order and barycentric
 * weights depend on positions only, which stay frozen) and evaluates, in FP64, the loss
 * L = sum over pixels and RGB of (clamp(C) - target)^2 as a function of the per-vertex RGBA
 * colours (num_verts*4 doubles) and the per-triangle opacities (num_quads*2 doubles, or NULL
 * when the scene has none). target: h*w*4 floats (alpha ignored). */
void* oracle_grad_build(const oracle_inputs* in);
void oracle_grad_free(void* ctx);
double oracle_grad_loss(void* ctx, const double* vcolors, const double* opacity, const float* target);
/* analytic gradient (back-to-front recursion in FP64); outputs may be NULL */
int oracle_grad_analytic(void* ctx, const double* vcolors, const double* opacity, const float* target,
						 double* dvcolors, double* dopacity);
/* adjoint alone: backpropagates a given upstream gradient dl_dimage (h*w*4 floats, alpha
 * ignored) through the FP64 blend; channels whose FP32 unclamped colour color32 (h*w*3 floats)
 * lies outside [0, 1] pass no gradient (the clamp) */
int oracle_grad_backprop(void* ctx, const double* vcolors, const double* opacity, const float* dl_dimage,
						 const float* color32, double* dvcolors, double* dopacity);
/* central difference (L(x+h) - L(x-h)) / 2h of one parameter: kind 0 = vertex colour
 * component index (vertex*4 + channel), kind 1 = triangle opacity index; only the pixels the
 * parameter touches are re-evaluated */
double oracle_grad_fd(void* ctx, const double* vcolors, const double* opacity, const float* target,
					  int kind, int index, double h);
uint64_t oracle_grad_num_fragments(void* ctx);

/* ---- quad generator (src/quad_generator.cpp) ----
 * Pairs triangles (num_tris x 3 vertex indices) that share an edge into quads; out_quads
 * (capacity num_tris x 4) receives, in tri order, each selected quad or a degenerate quad
 * (a, b, c, c). order 0: the reference's greedy (heap re-scoring removed quads' neighbours);
 * order 1: the same scores in synchronous rounds of local minima among the quads of the lowest
 * live conflict count (the CUDA path's). Returns 0, or
 * 1 for bad arguments, 2 for a vertex index out of range. */
int oracle_quadgen(const float* positions, int num_verts, const int32_t* tris, int num_tris,
				   float square_weight, int order, uint32_t* out_quads, int32_t* out_num_quads,
				   int32_t* out_num_degenerate);

#ifdef __cplusplus
}
#endif

#endif
