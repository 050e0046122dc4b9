// Shared device-side definitions of the lucid_gb300 CUDA path.
//
// Numerics: every file is compiled with --fmad=false, IEEE division and square root and no
// flush-to-zero, so each float expression below rounds exactly like the same expression on
// the CPU. Expressions keep the evaluation order of the reference GLSL (left to right).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lucid_gb300.h"

namespace lucid {

constexpr int kBinSize = 32;
constexpr int kBinShift = 5;
constexpr int kMaxDispatches = 256;      // LucidRenderer::m_max_dispatches for >= 4 GB
constexpr int kMaxBinCount = 16384;      // bins of one view (128 x 128 bins = 4096^2 pixels)
constexpr int kSetupThreads = 256;
constexpr int kBinningThreads = 1024;
constexpr int kRasterThreads = 512;
// uint4 per tri of the shading record: 4 with FP16 vertex colours, 3 otherwise
constexpr int kShadeRecWords = 4;
__host__ __device__ __forceinline__ int shadeRecWords(int color_format) {
	return color_format == LUCID_COLOR_RGBA16F ? 4 : 3;
}

// Per-view device parameters (passed by value to every kernel).
struct FrameParams {
	// ---- caller-owned inputs ----
	const float* positions;
	const void* colors;
	int color_format;
	int num_verts;
	const uint32_t* quads_ib;
	int num_quads;
	int num_instances;
	const lucid_instance* instances;
	const uint32_t* instance_colors;
	const float* tri_opacity;
	const float2* tex_coords;       // optional shading inputs
	const float4* instance_uv_rects;
	const uint32_t* normals;
	lucid_texture opaque_tex, trans_tex; // texels null when absent
	float* out_rgba;
	// ---- dimensions & limits ----
	int width, height;
	int bin_count_x, bin_count_y, bin_count;
	// bins are (1 << bin_shift) pixels square: 32 (5) or 64 (6). Setup's bin AABBs and the
	// raster tiles stay 32x32; a 64-pixel bin is rastered as its four 32x32 tiles.
	int bin_shift;
	int max_visible_quads;
	int max_bin_refs;
	int band_capacity;
	int low_high_threshold;
	int slab_target;      // fragments per unfinished pixel a depth slab aims at
	int light_max_pixel;  // bins whose pixels have at most this many fragments take the light path
	int num_setup_ctas;
	int num_binning_ctas;
	uint32_t flags;
	// LucidConfig by value: kernels read it from the parameter bank (no upload needed, so a
	// frame is graph-capturable without host staging buffers).
	lucid_config cfg;
	// ---- renderer-owned buffers ----
	lucid_info* info;
	uint32_t* counts;           // 10 * bin_count words after the info block
	int* inst_offsets;          // num_instances + 1
	uint4* quad_class;          // per input quad
	int4* setup_cta_counts;     // per setup CTA: small, large, (unused), (unused)
	int4* setup_cta_offsets;
	uint32_t* quad_aabbs;
	uint32_t* quad_source;
	uint4* quad_verts;
	uint4* quad_colors;
	uint4* quad_normals;  // encoded vertex normals per quad slot (STORAGE_QUAD_NORMAL)
	uint4* quad_tex;      // 2 per quad slot: tex0, tex1 - tex0, tex2 - tex0, tex3 - tex0
	uint4* tri_shade; // shadeRecWords(color_format) per tri: the two bary records (edge planes and
	                  // bary parameters, quad_setup.glsl:290-309), then the vertex
	                  // colours (RGBA8 or FP16, when the instance has them) and its instance
	                  // flags | id << 16 (ShadeRec in lucid_shade.cuh)
	uint4* tri_scan;  // 2 per tri
	uint4* tri_depth; // 1 per tri
	uint32_t* tri_normals;
	uint32_t* bin_quads;
	uint32_t* bin_tris;
	int* bin_batches;     // num_binning_ctas * 2 * bin_count histograms
	uint32_t* raster_work; // bin_count bin ids: HIGH, LOW, EMPTY
	uint2* band_scratch;  // per raster CTA: 8 * band_capacity entries
	uint2* band_keys;     // per raster CTA and band entry: depth-key range over the current group
	float4* band_planes;  // per raster CTA and band entry: the tri's depth plane (dx, dy, dz)
	int* dump_counts;     // verification mode (may be null)
	int* dump_prims;
	int dump_max;
	const int* dump_bin_slot; // per bin: slot in the dump arrays, -1 = not recorded (null: all)
	// gradient passes (kRasterStats / kRasterBackward)
	double* px_color64;   // per pixel: FP64 unclamped colour (3 doubles, stats pass output)
	float* px_color32;    // per pixel: FP32 unclamped colour (3 floats, clamp mask)
	const float* dl_dimage;
	float* dvertex_rgba;
	float* dtri_opacity;
	// batched frames: shared bump allocator of the bin reference lists (null for one view,
	// whose lists start at 0)
	uint32_t* ref_alloc; // [0] quad refs, [1] tri refs
	// fragment store of the differentiable forward (kRasterStore): every pixel's fragments as
	// tri slots in blend order
	uint32_t* grad_tris;
	uint32_t* grad_px_off;              // per pixel: first stored fragment
	uint32_t* grad_px_cnt;              // per pixel: stored fragments
	unsigned long long* grad_state;     // [0] overflow flag, [1] fragments allocated
	unsigned long long grad_capacity;   // fragments grad_tris holds
};

// ---------------------------------------------------------------------------------------------
// View sources of the pass kernels. A kernel is instantiated for one view (its FrameParams in
// the parameter bank) or for a batch of views (FrameParams in device memory; each CTA range
// belongs to one view, whose parameters the CTA copies to shared memory).

constexpr int kMaxBatchViews = 256;

struct OneView {
	FrameParams p;
	__device__ __forceinline__ const FrameParams& get(int& cta, int& ncta) const {
		cta = blockIdx.x, ncta = gridDim.x;
		return p;
	}
};

struct BatchViews {
	const FrameParams* views;
	int num_views;
	int cta_off[kMaxBatchViews + 1]; // CTAs [cta_off[v], cta_off[v + 1]) work on view v

	__device__ __forceinline__ const FrameParams& get(int& cta, int& ncta) const {
		__shared__ __align__(16) FrameParams s_view;
		const int c = int(blockIdx.x);
		int lo = 0, hi = num_views - 1;
		while(lo < hi) { // last view whose range starts at or before c (skips empty ranges)
			int mid = (lo + hi + 1) >> 1;
			if(cta_off[mid] <= c)
				lo = mid;
			else
				hi = mid - 1;
		}
		cta = c - cta_off[lo], ncta = cta_off[lo + 1] - cta_off[lo];
		const uint32_t* src = reinterpret_cast<const uint32_t*>(views + lo);
		uint32_t* dst = reinterpret_cast<uint32_t*>(&s_view);
		for(int i = threadIdx.x; i < int(sizeof(FrameParams) / 4); i += blockDim.x)
			dst[i] = src[i];
		__syncthreads();
		return s_view;
	}
};
static_assert(sizeof(FrameParams) % 4 == 0, "FrameParams is copied as 32-bit words");

// Raster kernel modes.
constexpr int kRasterForward = 0;  // image
constexpr int kRasterStats = 1;    // image + per-pixel FP64 colour for the backward pass
constexpr int kRasterBackward = 2; // gradients of vertex RGBA / triangle opacity
constexpr int kRasterStore = 3;    // each pixel's sorted fragments into the fragment store

// Offsets into the per-bin counter array (definitions.glsl:117-129)
__device__ __forceinline__ uint32_t& binQuadCounts(const FrameParams& p, int i) { return p.counts[p.bin_count * 0 + i]; }
__device__ __forceinline__ uint32_t& binQuadOffsets(const FrameParams& p, int i) { return p.counts[p.bin_count * 1 + i]; }
__device__ __forceinline__ uint32_t& binQuadOffsetsTemp(const FrameParams& p, int i) { return p.counts[p.bin_count * 2 + i]; }
__device__ __forceinline__ uint32_t& binTriCounts(const FrameParams& p, int i) { return p.counts[p.bin_count * 3 + i]; }
__device__ __forceinline__ uint32_t& binTriOffsets(const FrameParams& p, int i) { return p.counts[p.bin_count * 4 + i]; }
__device__ __forceinline__ uint32_t& binTriOffsetsTemp(const FrameParams& p, int i) { return p.counts[p.bin_count * 5 + i]; }
__device__ __forceinline__ uint32_t& lowLevelBins(const FrameParams& p, int i) { return p.counts[p.bin_count * 7 + i]; }
__device__ __forceinline__ uint32_t& highLevelBins(const FrameParams& p, int i) { return p.counts[p.bin_count * 9 + i]; }

// ---------------------------------------------------------------------------------------------
// Arithmetic helpers (identical evaluation order to the CPU oracle)

struct F3 {
	float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ bool feq(F3 a, F3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 cross3(F3 a, F3 b) {
	return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ F3 xyz4(const float* v) { return f3(v[0], v[1], v[2]); }

// GLSL int()/uint() of a float: truncation, saturating, NaN -> 0.
__device__ __forceinline__ int f2i(float x) {
	if(x != x)
		return 0;
	return __float2int_rz(x);
}
__device__ __forceinline__ uint32_t f2u(float x) {
	if(x != x || x <= 0.0f)
		return 0u;
	return __float2uint_rz(x);
}
__device__ __forceinline__ uint32_t fbits(float f) { return __float_as_uint(f); }
__device__ __forceinline__ float bitsf(uint32_t u) { return __uint_as_float(u); }

// Ascending sort key that puts the nearest fragment (largest inv_ray_pos) first.
// NaN depths (degenerate planes) use one canonical NaN so that CPU and GPU order them alike.
__device__ __forceinline__ uint32_t nearFirstKey(float inv_ray_pos) {
	uint32_t u = inv_ray_pos != inv_ray_pos ? 0x7fc00000u : fbits(inv_ray_pos);
	uint32_t asc = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
	return ~asc;
}
__device__ __forceinline__ float keyToDepth(uint32_t key) {
	uint32_t asc = ~key;
	uint32_t u = (asc & 0x80000000u) ? (asc & 0x7fffffffu) : ~asc;
	return bitsf(u);
}

// funcs.glsl:52-59
__device__ __forceinline__ uint32_t encodeAABB28(uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1) {
	return (x0 & 0x7fu) | ((y0 & 0x7fu) << 7) | ((x1 & 0x7fu) << 14) | ((y1 & 0x7fu) << 21);
}
__device__ __forceinline__ void decodeAABB28(uint32_t a, int& x0, int& y0, int& x1, int& y1) {
	x0 = int(a & 0x7fu), y0 = int((a >> 7) & 0x7fu), x1 = int((a >> 14) & 0x7fu),
	y1 = int((a >> 21) & 0x7fu);
}
// funcs.glsl:100-104
__device__ __forceinline__ float4 decodeRGBA8(uint32_t c) {
	const float s = 1.0f / 255.0f;
	return make_float4(float(c & 0xffu) * s, float((c >> 8) & 0xffu) * s,
					   float((c >> 16) & 0xffu) * s, float((c >> 24) & 0xffu) * s);
}

// First error wins; details recorded once.
__device__ __forceinline__ void raiseError(lucid_info* info, uint32_t code, uint32_t d0,
										   uint32_t d1, uint32_t d2) {
	if(atomicCAS(&info->error_code, 0u, code) == 0u) {
		info->error_detail[0] = d0;
		info->error_detail[1] = d1;
		info->error_detail[2] = d2;
	}
}

// ---------------------------------------------------------------------------------------------
// Block-wide scans

__device__ __forceinline__ uint32_t laneMaskLt() {
	uint32_t m;
	asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}

template <typename T> __device__ __forceinline__ T warpInclusiveScan(T v) {
	int lane = threadIdx.x & 31;
#pragma unroll
	for(int o = 1; o < 32; o <<= 1) {
		T t = __shfl_up_sync(0xffffffffu, v, o);
		if(lane >= o)
			v += t;
	}
	return v;
}

// Exclusive scan over the block; `smem` needs blockDim.x/32 + 1 elements. Returns the block
// total in *total. Must be called by all threads of the block.
template <typename T>
__device__ __forceinline__ T blockExclusiveScan(T v, T* smem, T* total) {
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	T inc = warpInclusiveScan(v);
	if(lane == 31)
		smem[warp] = inc;
	__syncthreads();
	if(warp == 0) {
		T w = lane < nw ? smem[lane] : T(0);
		T wi = warpInclusiveScan(w);
		if(lane < nw)
			smem[lane] = wi - w;
		if(lane == nw - 1)
			smem[nw] = wi;
	}
	__syncthreads();
	T res = smem[warp] + inc - v;
	if(total)
		*total = smem[nw];
	__syncthreads();
	return res;
}

} // namespace lucid
