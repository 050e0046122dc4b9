// C ABI of lucid_gb300: renderer object, buffer arena and pass orchestration.
//
// Mirrors LucidRenderer (src/lucid_renderer.h:21-96, src/lucid_renderer.cpp:186-580): the
// renderer owns every intermediate buffer; a frame is setup -> bin count -> categorize ->
// dispatch -> raster, all asynchronous on the caller's stream. Unlike the reference, grid
// sizes never depend on device-side counts (fixed or persistent grids read the counts on the
// device), so a frame needs no indirect dispatch and can be captured in a CUDA graph.

#include <algorithm>
#include <functional>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lucid_common.cuh"
#include "lucid_kernels.h"

namespace lucid {
cudaError_t configureRasterKernel();
cudaError_t configureRefKernel();
}

using namespace lucid;

static_assert(sizeof(lucid_instance) == 16, "InstanceData layout");
static_assert(sizeof(lucid_frustum) == 192, "Frustum layout");
static_assert(sizeof(lucid_lighting) == 64, "Lighting layout");
static_assert(sizeof(lucid_config) == 352, "LucidConfig layout");
static_assert(offsetof(lucid_config, view_proj_matrix) == 192, "LucidConfig layout");
static_assert(offsetof(lucid_config, lighting) == 256, "LucidConfig layout");
static_assert(offsetof(lucid_config, background_color) == 320, "LucidConfig layout");
static_assert(offsetof(lucid_config, enable_backface_culling) == 336, "LucidConfig layout");
static_assert(offsetof(lucid_info, temp) == (LUCID_INFO_REFERENCE_WORDS - 64) * 4, "LucidInfo layout");
static_assert(offsetof(lucid_info, error_code) == LUCID_INFO_REFERENCE_WORDS * 4, "LucidInfo layout");
static_assert(sizeof(lucid_info) == LUCID_INFO_WORDS * 4, "lucid_info size");
static_assert(offsetof(lucid_info, num_fragments) % 8 == 0, "64-bit counters alignment");
static_assert(offsetof(lucid_info, raster_blended_fragments) % 8 == 0, "64-bit counters alignment");

namespace {

thread_local std::string g_last_error;

lucid_status fail(lucid_status st, const std::string& msg) {
	g_last_error = msg;
	return st;
}

lucid_status cudaFail(cudaError_t err, const char* what) {
	return fail(LUCID_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(err));
}

#define LUCID_CUDA_TRY(call)                                                                       \
	do {                                                                                           \
		cudaError_t err__ = (call);                                                                \
		if(err__ != cudaSuccess)                                                                   \
			return cudaFail(err__, #call);                                                         \
	} while(0)

template <typename T> size_t bytesOf(size_t n) { return n * sizeof(T); }

} // namespace

void lucidSetLastError(const std::string& msg) { g_last_error = msg; }

struct lucid_renderer {
	lucid_options opts;
	int width, height;
	int bin_count_x, bin_count_y, bin_count;
	int device, num_sms;
	int raster_ctas;
	int setup_ctas_max;
	int binning_ctas_alloc; // CTAs the binning histogram scratch is sized for
	std::vector<void*> allocations;

	// buffers
	unsigned char* info_block = nullptr; // lucid_info + 10 * bin_count u32
	int* inst_offsets = nullptr;
	uint4* quad_class = nullptr;
	int4* setup_cta_counts = nullptr;
	int4* setup_cta_offsets = nullptr;
	uint32_t* quad_aabbs = nullptr;
	uint32_t* quad_source = nullptr;
	uint4* quad_verts = nullptr;
	uint4* quad_colors = nullptr;
	uint4* quad_normals = nullptr;
	uint4* quad_tex = nullptr;
	uint4* tri_shade = nullptr;
	uint4* tri_scan = nullptr;
	uint4* tri_depth = nullptr;
	uint32_t* tri_normals = nullptr;
	uint32_t* bin_quads = nullptr;
	uint32_t* bin_tris = nullptr;
	int* bin_batches = nullptr;
	uint32_t* raster_work = nullptr;
	uint2* band_scratch = nullptr;
	uint2* band_keys = nullptr;
	float4* band_planes = nullptr;
	uint8_t* ref_plan = nullptr; // reference-order mode: path of every bin

	FrameParams last{}; // parameters of the last quad setup (used by the later passes)
	bool have_frame = false;

	// gradient pass state, allocated on the first lucid_render_forward_grad / _backward
	double* px_color64 = nullptr;
	float* px_color32 = nullptr;
	float* stats_image = nullptr;
	uint32_t* grad_px_off = nullptr;
	uint32_t* grad_px_cnt = nullptr;
	unsigned long long* grad_state = nullptr;  // [0] store overflow, [1] fragments of the last frame
	uint32_t* grad_tris = nullptr;             // fragment store (own allocation, grows)
	size_t grad_capacity = 0;
	unsigned long long* grad_need_host = nullptr; // pinned copy of grad_state[1]
	cudaEvent_t grad_need_event = nullptr;
	bool grad_need_pending = false;
	// set by lucid_render_forward_grad, cleared by every other pass: the bin lists and the
	// per-pixel colours then belong to grad_inputs / grad_config
	bool grad_ready = false;
	lucid_frame_inputs grad_inputs{};
	lucid_config grad_config{};

	struct BatchPlan* batch = nullptr; // lucid_render_batch state (plan, buffers, graph)

	// bin_count_x / _y / bin_count are the 32-pixel grid the buffers are sized for; a frame
	// with 64-pixel bins (options.bin_size) uses the smaller grid of frameBins()
	size_t infoBytes() const { return sizeof(lucid_info) + size_t(10) * bin_count * 4; }
	lucid_info* info() const { return reinterpret_cast<lucid_info*>(info_block); }
	uint32_t* counts() const { return reinterpret_cast<uint32_t*>(info_block + sizeof(lucid_info)); }
};

namespace {

template <typename T> lucid_status allocate(lucid_renderer* r, T** ptr, size_t count) {
	void* p = nullptr;
	size_t bytes = std::max<size_t>(count * sizeof(T), 16);
	cudaError_t err = cudaMalloc(&p, bytes);
	if(err != cudaSuccess) {
		cudaGetLastError();
		return fail(LUCID_OUT_OF_MEMORY, std::string("cudaMalloc(") + std::to_string(bytes) +
											 " bytes): " + cudaGetErrorString(err));
	}
	r->allocations.push_back(p);
	*ptr = reinterpret_cast<T*>(p);
	return LUCID_OK;
}

void freeAll(lucid_renderer* r) {
	for(void* p : r->allocations)
		cudaFree(p);
	r->allocations.clear();
}

lucid_status validateInputs(const lucid_renderer* r, const lucid_frame_inputs* in) {
	if(!in)
		return fail(LUCID_INVALID_ARG, "inputs is NULL");
	if(!in->config)
		return fail(LUCID_INVALID_ARG, "inputs->config is NULL");
	if(in->num_quads < 0 || in->num_instances < 0 || in->num_verts < 0)
		return fail(LUCID_INVALID_ARG, "negative counts in inputs");
	if(in->num_quads > r->opts.max_input_quads)
		return fail(LUCID_CAPACITY_EXCEEDED,
					"num_quads " + std::to_string(in->num_quads) + " > options.max_input_quads " +
						std::to_string(r->opts.max_input_quads));
	if(in->num_instances > r->opts.max_instances)
		return fail(LUCID_CAPACITY_EXCEEDED, "num_instances > options.max_instances");
	if(in->num_quads > 0 && (!in->positions || !in->quads_ib || !in->instances))
		return fail(LUCID_INVALID_ARG, "positions, quads_ib and instances are required");
	if(in->num_quads > 0 && in->num_instances == 0)
		return fail(LUCID_INVALID_ARG, "num_quads > 0 but no instances");
	if(in->color_format < LUCID_COLOR_RGBA8 || in->color_format > LUCID_COLOR_RGBA32F)
		return fail(LUCID_INVALID_ARG, "unknown color_format");
	if(in->num_quads > 0 && !in->colors)
		return fail(LUCID_INVALID_ARG, "colors is NULL");
	for(const lucid_texture* t : {in->opaque_texture, in->transparent_texture})
		if(t && t->texels && (t->width <= 0 || t->height <= 0 || t->num_levels <= 0 || t->num_levels > 16))
			return fail(LUCID_INVALID_ARG, "texture size or level count out of range");
	return LUCID_OK;
}

void setShadingInputs(FrameParams& p, const lucid_frame_inputs* in) {
	p.tex_coords = reinterpret_cast<const float2*>(in->tex_coords);
	p.instance_uv_rects = reinterpret_cast<const float4*>(in->instance_uv_rects);
	p.normals = in->normals;
	p.opaque_tex = in->opaque_texture ? *in->opaque_texture : lucid_texture{};
	p.trans_tex = in->transparent_texture ? *in->transparent_texture : lucid_texture{};
}

// fragments per unfinished pixel that a depth slab of the raster aims at
int slabTarget(const lucid_renderer* r) { return r->opts.slab_fragments > 0 ? r->opts.slab_fragments : 165; }
// deepest pixel of a bin that takes the light raster path (-1: none)
int lightMaxPixel(const lucid_options* o) {
	return o->light_max_pixel == 0 ? 64 : (o->light_max_pixel < 0 ? -1 : o->light_max_pixel);
}
int lightMaxPixel(const lucid_renderer* r) { return lightMaxPixel(&r->opts); }
// bins of options.bin_size pixels (32 or 64): log2 of the size, the grid of a viewport, and the
// number of bins of the renderer's current frames
int binShift(const lucid_options& o) { return o.bin_size == 64 ? 6 : kBinShift; }
void binGrid(int w, int h, int bsh, int& bcx, int& bcy) {
	const int bs = 1 << bsh;
	bcx = (w + bs - 1) / bs, bcy = (h + bs - 1) / bs;
}
int frameBins(const lucid_renderer* r) {
	int bcx, bcy;
	binGrid(r->width, r->height, binShift(r->opts), bcx, bcy);
	return bcx * bcy;
}

FrameParams makeParams(lucid_renderer* r, const lucid_frame_inputs* in, float* out) {
	FrameParams p{};
	p.bin_shift = binShift(r->opts);
	binGrid(r->width, r->height, p.bin_shift, p.bin_count_x, p.bin_count_y);
	p.bin_count = p.bin_count_x * p.bin_count_y;
	p.positions = in->positions;
	p.colors = in->colors;
	p.color_format = in->color_format;
	p.num_verts = in->num_verts;
	p.quads_ib = in->quads_ib;
	p.num_quads = in->num_quads;
	p.num_instances = in->num_instances;
	p.instances = in->instances;
	p.instance_colors = in->instance_colors;
	p.tri_opacity = in->tri_opacity;
	setShadingInputs(p, in);
	p.out_rgba = out;
	p.cfg = *in->config;
	p.width = r->width, p.height = r->height;
	p.max_visible_quads = r->opts.max_visible_quads;
	p.max_bin_refs = r->opts.max_bin_refs;
	p.band_capacity = r->opts.band_capacity;
	p.low_high_threshold = r->opts.low_high_threshold;
	p.slab_target = slabTarget(r);
	p.light_max_pixel = lightMaxPixel(r);
	p.num_setup_ctas = (in->num_quads + kSetupThreads - 1) / kSetupThreads;
	p.num_binning_ctas = r->opts.binning_ctas;
	p.flags = r->opts.flags;
	p.info = r->info();
	p.counts = r->counts();
	p.inst_offsets = r->inst_offsets;
	p.quad_class = r->quad_class;
	p.setup_cta_counts = r->setup_cta_counts;
	p.setup_cta_offsets = r->setup_cta_offsets;
	p.quad_aabbs = r->quad_aabbs;
	p.quad_source = r->quad_source;
	p.quad_verts = r->quad_verts;
	p.quad_colors = r->quad_colors;
	p.quad_normals = r->quad_normals;
	p.quad_tex = r->quad_tex;
	p.tri_shade = r->tri_shade;
	p.tri_scan = r->tri_scan;
	p.tri_depth = r->tri_depth;
	p.tri_normals = r->tri_normals;
	p.bin_quads = r->bin_quads;
	p.bin_tris = r->bin_tris;
	p.bin_batches = r->bin_batches;
	p.raster_work = r->raster_work;
	p.band_scratch = r->band_scratch;
	p.band_keys = r->band_keys;
	p.band_planes = r->band_planes;
	return p;
}

lucid_status checkLaunch(const char* what) {
	cudaError_t err = cudaGetLastError();
	if(err != cudaSuccess)
		return cudaFail(err, what);
	return LUCID_OK;
}

lucid_status resetRasterCounters(lucid_renderer* r, cudaStream_t st) {
	lucid_info* info = r->info();
	LUCID_CUDA_TRY(cudaMemsetAsync(&info->raster_work_counter, 0, 4, st));
	LUCID_CUDA_TRY(cudaMemsetAsync(&info->stats[0], 0, 8, st));
	LUCID_CUDA_TRY(cudaMemsetAsync(&info->max_pixel_fragments, 0, 4, st));
	LUCID_CUDA_TRY(cudaMemsetAsync(&info->num_fragments, 0, 16, st));
	LUCID_CUDA_TRY(cudaMemsetAsync(info->raster_timers, 0, sizeof(info->raster_timers), st));
	LUCID_CUDA_TRY(cudaMemsetAsync(&info->raster_windows, 0,
								   offsetof(lucid_info, ext_reserved) - offsetof(lucid_info, raster_windows), st));
	return LUCID_OK;
}

} // namespace

// ---------------------------------------------------------------------------------------------
// Host-only helpers

extern "C" const char* lucid_status_string(lucid_status status) {
	switch(status) {
	case LUCID_OK: return "ok";
	case LUCID_INVALID_ARG: return "invalid argument";
	case LUCID_CAPACITY_EXCEEDED: return "capacity exceeded";
	case LUCID_CUDA_ERROR: return "CUDA error";
	case LUCID_TIMEOUT: return "timeout";
	case LUCID_NOT_SUPPORTED: return "not supported";
	case LUCID_OUT_OF_MEMORY: return "out of memory";
	}
	return "unknown status";
}

extern "C" const char* lucid_last_error_string(void) { return g_last_error.c_str(); }
extern "C" int lucid_abi_version(void) { return LUCID_ABI_VERSION; }

extern "C" lucid_status lucid_default_options(lucid_options* out) {
	if(!out)
		return fail(LUCID_INVALID_ARG, "out is NULL");
	memset(out, 0, sizeof(*out));
	out->flags = 0;
	out->bin_size = 32;
	out->max_input_quads = 1 << 22;
	out->max_visible_quads = 1 << 22;
	out->max_instances = 64 * 1024;
	out->low_high_threshold = 1024;
	out->max_bin_refs = 1 << 24;
	out->band_capacity = 16384;
	out->binning_ctas = 0;
	out->raster_ctas_per_sm = 0;
	out->max_views = 1;
	return LUCID_OK;
}

extern "C" lucid_status lucid_build_instances(const lucid_draw_call* dcs, int32_t num_dcs,
											  lucid_instance* out, uint32_t* out_colors,
											  int32_t max_instances, int32_t* out_count,
											  int32_t* out_num_quads) {
	if((num_dcs > 0 && !dcs) || !out || !out_count || max_instances < 0)
		return fail(LUCID_INVALID_ARG, "lucid_build_instances: bad arguments");
	int n = 0;
	int64_t total = 0;
	for(int d = 0; d < num_dcs; d++) {
		const lucid_draw_call& dc = dcs[d];
		if(dc.num_quads <= 0)
			continue;
		uint32_t opts = dc.opts;
		if(dc.material_color != 0xffffffffu)
			opts |= LUCID_INST_HAS_COLOR;
		for(int i = 0; i < dc.num_quads; i += LUCID_MAX_INSTANCE_QUADS) {
			if(n < max_instances) {
				out[n].index_offset = (dc.quad_offset + i) * 4;
				out[n].vertex_offset = 0;
				out[n].num_quads = std::min(LUCID_MAX_INSTANCE_QUADS, dc.num_quads - i);
				out[n].flags = opts & 0xffffu;
				if(out_colors)
					out_colors[n] = dc.material_color;
				total += out[n].num_quads;
			}
			n++;
		}
	}
	*out_count = std::min(n, max_instances);
	if(out_num_quads)
		*out_num_quads = int32_t(total);
	if(n > max_instances)
		return fail(LUCID_CAPACITY_EXCEEDED, "instance limit reached; list truncated");
	return LUCID_OK;
}

extern "C" lucid_status lucid_make_config(const lucid_camera* cam, int32_t width, int32_t height,
										  const float* background, int32_t backface_culling,
										  lucid_config* out) {
	if(!cam || !out || width <= 0 || height <= 0)
		return fail(LUCID_INVALID_ARG, "lucid_make_config: bad arguments");
	double p[3], r[3], u[3], f[3];
	for(int i = 0; i < 3; i++)
		p[i] = cam->position[i], r[i] = cam->right[i], u[i] = cam->up[i], f[i] = cam->forward[i];
	double ty = tan(double(cam->fov_y_radians) * 0.5);
	double tx = ty * (double(width) / double(height));
	double dirs[4][3];
	const double corners[4][2] = {{-1.0, -1.0}, {-1.0, 1.0}, {1.0, 1.0}, {1.0, -1.0}};
	for(int c = 0; c < 4; c++)
		for(int i = 0; i < 3; i++)
			dirs[c][i] = f[i] + r[i] * (corners[c][0] * tx) + u[i] * (corners[c][1] * ty);
	memset(out, 0, sizeof(*out));
	for(int c = 0; c < 4; c++)
		for(int i = 0; i < 3; i++) {
			out->frustum.ws_dirs[c][i] = float(dirs[c][i]);
			out->frustum.ws_origins[c][i] = float(p[i]);
		}
	for(int i = 0; i < 3; i++) {
		out->frustum.ws_origin0[i] = float(p[i]);
		out->frustum.ws_dir0[i] = float(dirs[0][i]);
		out->frustum.ws_dirx[i] = float((dirs[3][i] - dirs[0][i]) * (1.0 / double(width)));
		out->frustum.ws_diry[i] = float((dirs[1][i] - dirs[0][i]) * (1.0 / double(height)));
	}
	out->frustum.ws_origin0[3] = 1.0f;
	double zb[3] = {-f[0], -f[1], -f[2]};
	double view[4][4] = {{r[0], r[1], r[2], -(r[0] * p[0] + r[1] * p[1] + r[2] * p[2])},
						 {u[0], u[1], u[2], -(u[0] * p[0] + u[1] * p[1] + u[2] * p[2])},
						 {zb[0], zb[1], zb[2], -(zb[0] * p[0] + zb[1] * p[1] + zb[2] * p[2])},
						 {0.0, 0.0, 0.0, 1.0}};
	double n = cam->near_plane, fa = cam->far_plane;
	double proj[4][4] = {{1.0 / tx, 0.0, 0.0, 0.0},
						 {0.0, 1.0 / ty, 0.0, 0.0},
						 {0.0, 0.0, (fa + n) / (n - fa), (2.0 * fa * n) / (n - fa)},
						 {0.0, 0.0, -1.0, 0.0}};
	for(int row = 0; row < 4; row++)
		for(int col = 0; col < 4; col++) {
			double acc = 0.0;
			for(int k = 0; k < 4; k++)
				acc += proj[row][k] * view[k][col];
			out->view_proj_matrix[col * 4 + row] = float(acc);
		}
	// SceneLighting::makeDefault (src/shading.cpp:26-34)
	const float amb[4] = {0.8f, 0.8f, 0.6f, 1.0f}, sun[4] = {0.8f, 0.8f, 0.8f, 1.0f};
	const float sdir[4] = {0.842121f, -0.300567f, -0.447763f, 0.0f};
	for(int i = 0; i < 4; i++) {
		out->lighting.ambient_color[i] = amb[i];
		out->lighting.sun_color[i] = sun[i];
		out->lighting.sun_dir[i] = sdir[i];
		out->background_color[i] = background ? background[i] : (i == 3 ? 1.0f : 0.0f);
	}
	out->lighting.sun_power = 2.5f;
	out->lighting.ambient_power = 0.4f;
	out->enable_backface_culling = backface_culling ? 1u : 0u;
	out->num_instances = 0;
	out->instance_packet_size = 1;
	return LUCID_OK;
}

// ---------------------------------------------------------------------------------------------
// Renderer lifetime

extern "C" lucid_status lucid_create(const lucid_options* options, int32_t width, int32_t height,
									 lucid_renderer** out) {
	if(!out)
		return fail(LUCID_INVALID_ARG, "out is NULL");
	*out = nullptr;
	lucid_options o;
	if(options)
		o = *options;
	else
		lucid_default_options(&o);
	if(o.bin_size != 32 && o.bin_size != 64)
		return fail(LUCID_NOT_SUPPORTED, "bins must be 32x32 or 64x64 pixels");
	if(width <= 0 || height <= 0 || width > 4096 || height > 4096)
		return fail(LUCID_INVALID_ARG, "viewport must be within 1..4096 pixels per axis");
	if(o.max_visible_quads <= 0 || o.max_visible_quads > (1 << 23) || o.max_input_quads <= 0 ||
	   o.max_instances <= 0 || o.max_instances > 65536 || o.max_bin_refs <= 0 ||
	   o.band_capacity <= 0 || o.band_capacity > (1 << 21) || o.low_high_threshold <= 0)
		return fail(LUCID_INVALID_ARG, "options out of range");
	if(o.max_views < 1)
		o.max_views = 1;

	lucid_renderer* r = new lucid_renderer();
	r->opts = o;
	r->width = width, r->height = height;
	r->bin_count_x = (width + kBinSize - 1) / kBinSize;
	r->bin_count_y = (height + kBinSize - 1) / kBinSize;
	r->bin_count = r->bin_count_x * r->bin_count_y;
	auto bail = [&](lucid_status st) {
		freeAll(r);
		delete r;
		return st;
	};
	cudaError_t err = cudaGetDevice(&r->device);
	if(err != cudaSuccess)
		return bail(cudaFail(err, "cudaGetDevice"));
	err = cudaDeviceGetAttribute(&r->num_sms, cudaDevAttrMultiProcessorCount, r->device);
	if(err != cudaSuccess)
		return bail(cudaFail(err, "cudaDeviceGetAttribute"));
	if(r->opts.binning_ctas <= 0)
		r->opts.binning_ctas = 2 * r->num_sms;
	r->opts.binning_ctas = std::min(r->opts.binning_ctas, 4096);
	r->binning_ctas_alloc = r->opts.binning_ctas;
	err = configureRasterKernel();
	if(err == cudaSuccess)
		err = configureRefKernel();
	if(err == cudaSuccess)
		err = configureBinningKernels();
	if(err != cudaSuccess)
		return bail(cudaFail(err, "configure raster kernels"));
	int ctas_per_sm = r->opts.raster_ctas_per_sm > 0 ? r->opts.raster_ctas_per_sm : 1;
	r->raster_ctas = r->num_sms * ctas_per_sm;

	const size_t mvq = size_t(o.max_visible_quads);
	const size_t miq = size_t(o.max_input_quads);
	r->setup_ctas_max = int((miq + kSetupThreads - 1) / kSetupThreads);
	lucid_status st;
	if((st = allocate(r, &r->info_block, r->infoBytes())) != LUCID_OK ||
	   (st = allocate(r, &r->inst_offsets, size_t(o.max_instances) + 1)) != LUCID_OK ||
	   (st = allocate(r, &r->quad_class, miq)) != LUCID_OK ||
	   (st = allocate(r, &r->setup_cta_counts, size_t(r->setup_ctas_max))) != LUCID_OK ||
	   (st = allocate(r, &r->setup_cta_offsets, size_t(r->setup_ctas_max))) != LUCID_OK ||
	   (st = allocate(r, &r->quad_aabbs, mvq)) != LUCID_OK ||
	   (st = allocate(r, &r->quad_source, mvq)) != LUCID_OK ||
	   (st = allocate(r, &r->quad_verts, mvq)) != LUCID_OK ||
	   (st = allocate(r, &r->quad_colors, mvq)) != LUCID_OK ||
	   (st = allocate(r, &r->quad_normals, mvq)) != LUCID_OK ||
	   (st = allocate(r, &r->quad_tex, 2 * mvq)) != LUCID_OK ||
	   (st = allocate(r, &r->tri_shade, 2 * kShadeRecWords * mvq)) != LUCID_OK ||
	   (st = allocate(r, &r->tri_scan, 4 * mvq)) != LUCID_OK ||
	   (st = allocate(r, &r->tri_depth, 2 * mvq)) != LUCID_OK ||
	   (st = allocate(r, &r->tri_normals, 2 * mvq)) != LUCID_OK ||
	   (st = allocate(r, &r->bin_quads, size_t(o.max_bin_refs))) != LUCID_OK ||
	   (st = allocate(r, &r->bin_tris, size_t(o.max_bin_refs))) != LUCID_OK ||
	   (st = allocate(r, &r->bin_batches, size_t(r->opts.binning_ctas) * 2 * r->bin_count)) != LUCID_OK ||
	   (st = allocate(r, &r->raster_work, size_t(r->bin_count))) != LUCID_OK ||
	   (st = allocate(r, &r->band_scratch, size_t(r->raster_ctas) * 8 * o.band_capacity)) != LUCID_OK ||
	   (st = allocate(r, &r->band_keys, size_t(r->raster_ctas) * 8 * o.band_capacity)) != LUCID_OK ||
	   (st = allocate(r, &r->band_planes, size_t(r->raster_ctas) * 8 * o.band_capacity)) != LUCID_OK ||
	   (st = allocate(r, &r->ref_plan, size_t(r->bin_count))) != LUCID_OK)
		return bail(st);
	// zero the records once so that unused slots read as zero in parity dumps
	for(void* p : {(void*)r->quad_aabbs, (void*)r->quad_source})
		cudaMemset(p, 0, mvq * 4);
	cudaMemset(r->quad_verts, 0, mvq * 16);
	cudaMemset(r->quad_colors, 0, mvq * 16);
	cudaMemset(r->tri_shade, 0, mvq * 2 * kShadeRecWords * 16);
	cudaMemset(r->tri_scan, 0, mvq * 64);
	cudaMemset(r->tri_depth, 0, mvq * 32);
	cudaMemset(r->tri_normals, 0, mvq * 8);
	cudaMemset(r->info_block, 0, r->infoBytes());
	err = cudaDeviceSynchronize();
	if(err != cudaSuccess)
		return bail(cudaFail(err, "renderer initialisation"));
	*out = r;
	return LUCID_OK;
}

static void destroyBatchPlan(lucid_renderer* r);

extern "C" lucid_status lucid_destroy(lucid_renderer* r) {
	if(!r)
		return LUCID_OK;
	destroyBatchPlan(r);
	if(r->grad_need_event)
		cudaEventSynchronize(r->grad_need_event);
	if(r->grad_tris)
		cudaFree(r->grad_tris);
	if(r->grad_need_host)
		cudaFreeHost(r->grad_need_host);
	if(r->grad_need_event)
		cudaEventDestroy(r->grad_need_event);
	freeAll(r);
	delete r;
	return LUCID_OK;
}

// ---------------------------------------------------------------------------------------------
// Passes

extern "C" lucid_status lucid_quad_setup(lucid_renderer* r, const lucid_frame_inputs* in, void* stream) {
	if(!r)
		return fail(LUCID_INVALID_ARG, "renderer is NULL");
	lucid_status st = validateInputs(r, in);
	if(st != LUCID_OK)
		return st;
	cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
	// setupInputData (src/lucid_renderer.cpp:431-451): clear LucidInfo and the bin counters
	LUCID_CUDA_TRY(cudaMemsetAsync(r->info_block, 0, r->infoBytes(), s));
	r->last = makeParams(r, in, nullptr);
	r->have_frame = true;
	r->grad_ready = false;
	launchSetup(r->last, s);
	return checkLaunch("quad setup");
}

extern "C" lucid_status lucid_bin_count(lucid_renderer* r, void* stream) {
	if(!r || !r->have_frame)
		return fail(LUCID_INVALID_ARG, "lucid_bin_count needs a prior lucid_quad_setup");
	launchBinCount(r->last, reinterpret_cast<cudaStream_t>(stream));
	return checkLaunch("bin count");
}

extern "C" lucid_status lucid_bin_categorize(lucid_renderer* r, void* stream) {
	if(!r || !r->have_frame)
		return fail(LUCID_INVALID_ARG, "lucid_bin_categorize needs a prior lucid_quad_setup");
	launchBinCategorize(r->last, reinterpret_cast<cudaStream_t>(stream));
	return checkLaunch("bin categorize");
}

extern "C" lucid_status lucid_bin_dispatch(lucid_renderer* r, void* stream) {
	if(!r || !r->have_frame)
		return fail(LUCID_INVALID_ARG, "lucid_bin_dispatch needs a prior lucid_quad_setup");
	launchBinDispatch(r->last, reinterpret_cast<cudaStream_t>(stream));
	return checkLaunch("bin dispatch");
}

static lucid_status ensureGradStore(lucid_renderer* r, cudaStream_t s);
static lucid_status ensureStoreBuffers(lucid_renderer* r);

// The raster pass in store mode followed by the pixel-parallel blend; when the store cannot
// hold the frame, the raster pass's own blend runs instead (chosen on the device).
static lucid_status rasterPixelBlend(lucid_renderer* r, FrameParams p, cudaStream_t s) {
	lucid_status st;
	if((st = ensureStoreBuffers(r)) != LUCID_OK || (st = ensureGradStore(r, s)) != LUCID_OK)
		return st;
	p.grad_tris = r->grad_tris;
	p.grad_px_off = r->grad_px_off;
	p.grad_px_cnt = r->grad_px_cnt;
	p.grad_state = r->grad_state;
	p.grad_capacity = r->grad_capacity;
	LUCID_CUDA_TRY(cudaMemsetAsync(r->grad_state, 0, 16, s));
	if(r->grad_capacity == 0)
		LUCID_CUDA_TRY(cudaMemsetAsync(r->grad_state, 1, 8, s));
	LUCID_CUDA_TRY(cudaMemsetAsync(r->grad_px_cnt, 0, size_t(r->width) * r->height * 4, s));
	if((st = resetRasterCounters(r, s)) != LUCID_OK)
		return st;
	if(r->grad_capacity > 0) {
		launchRaster(p, r->raster_ctas, s, kRasterStore);
		if((st = checkLaunch("raster (store)")) != LUCID_OK)
			return st;
	}
	LUCID_CUDA_TRY(cudaMemsetAsync(&r->info()->raster_work_counter, 0, 4, s));
	launchRaster(p, r->raster_ctas, s, kRasterForward);
	if((st = checkLaunch("raster")) != LUCID_OK)
		return st;
	launchBlendPixels(p, s);
	if((st = checkLaunch("pixel blend")) != LUCID_OK)
		return st;
	if(r->grad_capacity > 0 && r->opts.grad_store_fragments == 0) {
		LUCID_CUDA_TRY(cudaMemcpyAsync(r->grad_need_host, &r->grad_state[1], 8, cudaMemcpyDeviceToHost, s));
		LUCID_CUDA_TRY(cudaEventRecord(r->grad_need_event, s));
		r->grad_need_pending = true;
	}
	return LUCID_OK;
}

static lucid_status rasterImpl(lucid_renderer* r, const lucid_frame_inputs* in, float* out,
							   int* dump_counts, int* dump_prims, int dump_max, cudaStream_t s,
							   const int* dump_bin_slot = nullptr) {
	if(!r || !r->have_frame)
		return fail(LUCID_INVALID_ARG, "lucid_raster needs a prior lucid_quad_setup");
	if(!out)
		return fail(LUCID_INVALID_ARG, "out_rgba is NULL");
	lucid_status st = validateInputs(r, in);
	if(st != LUCID_OK)
		return st;
	r->grad_ready = false;
	FrameParams p = r->last;
	p.slab_target = slabTarget(r);
	p.light_max_pixel = lightMaxPixel(r);
	p.colors = in->colors;
	p.color_format = in->color_format;
	p.instance_colors = in->instance_colors;
	p.tri_opacity = in->tri_opacity;
	setShadingInputs(p, in);
	p.cfg.background_color[0] = in->config->background_color[0];
	p.cfg.background_color[1] = in->config->background_color[1];
	p.cfg.background_color[2] = in->config->background_color[2];
	p.cfg.background_color[3] = in->config->background_color[3];
	p.out_rgba = out;
	p.dump_counts = dump_counts;
	p.dump_prims = dump_prims;
	p.dump_max = dump_max;
	p.dump_bin_slot = dump_bin_slot;
	if(r->opts.flags & LUCID_OPT_REFERENCE_ORDER) {
		if(r->opts.flags & LUCID_OPT_ALPHA_THRESHOLD)
			return fail(LUCID_NOT_SUPPORTED, "the reference-order mode has no alpha-threshold variant");
		if(r->opts.bin_size != 32)
			return fail(LUCID_NOT_SUPPORTED, "the reference-order mode needs 32x32 bins");
		if((st = resetRasterCounters(r, s)) != LUCID_OK)
			return st;
		LUCID_CUDA_TRY(cudaMemsetAsync(&r->info()->stats[2], 0, 4, s));
		launchRefRaster(p, r->ref_plan, s);
		return checkLaunch("raster (reference order)");
	}
	if((r->opts.flags & LUCID_OPT_PIXEL_BLEND) && !dump_counts)
		return rasterPixelBlend(r, p, s);
	if((st = resetRasterCounters(r, s)) != LUCID_OK)
		return st;
	launchRaster(p, r->raster_ctas, s);
	return checkLaunch("raster");
}

extern "C" lucid_status lucid_raster(lucid_renderer* r, const lucid_frame_inputs* in, float* out,
									 void* stream) {
	return rasterImpl(r, in, out, nullptr, nullptr, 0, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" lucid_status lucid_render(lucid_renderer* r, const lucid_frame_inputs* in, float* out,
									 void* stream) {
	lucid_status st;
	if((st = lucid_quad_setup(r, in, stream)) != LUCID_OK)
		return st;
	if((st = lucid_bin_count(r, stream)) != LUCID_OK)
		return st;
	if((st = lucid_bin_categorize(r, stream)) != LUCID_OK)
		return st;
	if((st = lucid_bin_dispatch(r, stream)) != LUCID_OK)
		return st;
	return lucid_raster(r, in, out, stream);
}

extern "C" lucid_status lucid_get_info(lucid_renderer* r, lucid_info* out, uint32_t* bin_counters,
									   void* stream) {
	if(!r || !out)
		return fail(LUCID_INVALID_ARG, "lucid_get_info: bad arguments");
	cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
	LUCID_CUDA_TRY(cudaStreamSynchronize(s));
	LUCID_CUDA_TRY(cudaMemcpy(out, r->info_block, sizeof(lucid_info), cudaMemcpyDeviceToHost));
	if(bin_counters)
		LUCID_CUDA_TRY(cudaMemcpy(bin_counters, r->counts(), size_t(10) * frameBins(r) * 4,
								  cudaMemcpyDeviceToHost));
	return LUCID_OK;
}

extern "C" lucid_status lucid_download_buffer(lucid_renderer* r, int32_t which, void* host_dst,
											  size_t bytes, size_t* out_bytes, void* stream) {
	if(!r)
		return fail(LUCID_INVALID_ARG, "renderer is NULL");
	const size_t mvq = size_t(r->opts.max_visible_quads);
	const void* src = nullptr;
	size_t size = 0;
	switch(which) {
	case LUCID_BUF_QUAD_AABBS: src = r->quad_aabbs, size = mvq * 4; break;
	case LUCID_BUF_TRI_BARY: // the first 32 bytes of every tri's shading record
		src = r->tri_shade, size = mvq * 64;
		break;
	case LUCID_BUF_TRI_SCAN: src = r->tri_scan, size = mvq * 64; break;
	case LUCID_BUF_TRI_DEPTH: src = r->tri_depth, size = mvq * 32; break;
	case LUCID_BUF_QUAD_COLORS: src = r->quad_colors, size = mvq * 16; break;
	case LUCID_BUF_TRI_NORMALS: src = r->tri_normals, size = mvq * 8; break;
	case LUCID_BUF_QUAD_SOURCE: src = r->quad_source, size = mvq * 4; break;
	case LUCID_BUF_BIN_QUADS: src = r->bin_quads, size = size_t(r->opts.max_bin_refs) * 4; break;
	case LUCID_BUF_BIN_TRIS: src = r->bin_tris, size = size_t(r->opts.max_bin_refs) * 4; break;
	case LUCID_BUF_QUAD_VERTS: src = r->quad_verts, size = mvq * 16; break;
	default: return fail(LUCID_INVALID_ARG, "unknown buffer id");
	}
	if(out_bytes)
		*out_bytes = size;
	if(host_dst && bytes) {
		LUCID_CUDA_TRY(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)));
		if(which == LUCID_BUF_TRI_BARY) {
			const size_t pitch = size_t(shadeRecWords(r->last.color_format)) * 16;
			const size_t rows = std::min(bytes, size) / 32;
			if(rows)
				LUCID_CUDA_TRY(cudaMemcpy2D(host_dst, 32, src, pitch, 32, rows, cudaMemcpyDeviceToHost));
		} else {
			LUCID_CUDA_TRY(cudaMemcpy(host_dst, src, std::min(bytes, size), cudaMemcpyDeviceToHost));
		}
	}
	return LUCID_OK;
}

// Verification dump over the whole frame (bins == NULL) or over a subset of bins.
static lucid_status rasterDump(lucid_renderer* r, const lucid_frame_inputs* in, float* out, int32_t max_per_pixel,
							   const int32_t* bins, int32_t num_bins, int32_t* host_counts, int32_t* host_prims,
							   void* stream) {
	if(!r || !host_counts || max_per_pixel < 0 || (max_per_pixel > 0 && !host_prims))
		return fail(LUCID_INVALID_ARG, "lucid_raster_dump: bad arguments");
	std::vector<int> slots;
	if(bins && (r->opts.flags & LUCID_OPT_REFERENCE_ORDER))
		return fail(LUCID_NOT_SUPPORTED, "lucid_raster_dump_bins: not in the reference-order mode");
	if(bins && r->opts.bin_size != 32)
		return fail(LUCID_NOT_SUPPORTED, "lucid_raster_dump_bins: needs 32x32 bins");
	if(bins) {
		if(num_bins <= 0 || num_bins > r->bin_count)
			return fail(LUCID_INVALID_ARG, "lucid_raster_dump_bins: num_bins out of range");
		slots.assign(size_t(r->bin_count), -1);
		for(int i = 0; i < num_bins; i++) {
			if(bins[i] < 0 || bins[i] >= r->bin_count || slots[size_t(bins[i])] >= 0)
				return fail(LUCID_INVALID_ARG, "lucid_raster_dump_bins: bin id out of range or repeated");
			slots[size_t(bins[i])] = i;
		}
	}
	cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
	const size_t npix = bins ? size_t(num_bins) * kBinSize * kBinSize : size_t(r->width) * r->height;
	int *dc = nullptr, *dp = nullptr, *dslot = nullptr;
	auto release = [&]() {
		if(dc)
			cudaFree(dc);
		if(dp)
			cudaFree(dp);
		if(dslot)
			cudaFree(dslot);
	};
	cudaError_t err = cudaMalloc(&dc, npix * 4);
	if(err == cudaSuccess && max_per_pixel > 0)
		err = cudaMalloc(&dp, npix * max_per_pixel * 4);
	if(err == cudaSuccess && bins)
		err = cudaMalloc(&dslot, slots.size() * 4);
	if(err == cudaSuccess && bins)
		err = cudaMemcpy(dslot, slots.data(), slots.size() * 4, cudaMemcpyHostToDevice);
	if(err == cudaSuccess && dp)
		err = cudaMemsetAsync(dp, 0xff, npix * max_per_pixel * 4, s);
	if(err == cudaSuccess)
		err = cudaMemsetAsync(dc, 0, npix * 4, s);
	if(err != cudaSuccess) {
		release();
		return cudaFail(err, "lucid_raster_dump buffers");
	}
	lucid_status st = lucid_quad_setup(r, in, stream);
	if(st == LUCID_OK)
		st = lucid_bin_count(r, stream);
	if(st == LUCID_OK)
		st = lucid_bin_categorize(r, stream);
	if(st == LUCID_OK)
		st = lucid_bin_dispatch(r, stream);
	if(st == LUCID_OK)
		st = rasterImpl(r, in, out, dc, dp, max_per_pixel, s, dslot);
	if(st == LUCID_OK) {
		err = cudaStreamSynchronize(s);
		if(err == cudaSuccess)
			err = cudaMemcpy(host_counts, dc, npix * 4, cudaMemcpyDeviceToHost);
		if(err == cudaSuccess && dp)
			err = cudaMemcpy(host_prims, dp, npix * max_per_pixel * 4, cudaMemcpyDeviceToHost);
		if(err != cudaSuccess)
			st = cudaFail(err, "lucid_raster_dump readback");
	}
	release();
	return st;
}

extern "C" lucid_status lucid_raster_dump(lucid_renderer* r, const lucid_frame_inputs* in, float* out,
										  int32_t max_per_pixel, int32_t* host_counts,
										  int32_t* host_prims, void* stream) {
	return rasterDump(r, in, out, max_per_pixel, nullptr, 0, host_counts, host_prims, stream);
}

extern "C" lucid_status lucid_raster_dump_bins(lucid_renderer* r, const lucid_frame_inputs* in, float* out,
											   const int32_t* bins, int32_t num_bins, int32_t max_per_pixel,
											   int32_t* host_counts, int32_t* host_prims, void* stream) {
	if(!bins)
		return fail(LUCID_INVALID_ARG, "lucid_raster_dump_bins: bins is NULL");
	return rasterDump(r, in, out, max_per_pixel, bins, num_bins, host_counts, host_prims, stream);
}

// Per-pixel offsets / counts and the state words of the fragment store (allocated once).
static lucid_status ensureStoreBuffers(lucid_renderer* r) {
	if(r->grad_state)
		return LUCID_OK;
	const size_t npix = size_t(r->width) * r->height;
	lucid_status st;
	if((st = allocate(r, &r->grad_px_off, npix)) != LUCID_OK || (st = allocate(r, &r->grad_px_cnt, npix)) != LUCID_OK)
		return st;
	cudaError_t err = cudaHostAlloc(reinterpret_cast<void**>(&r->grad_need_host), 8, cudaHostAllocDefault);
	if(err == cudaSuccess)
		err = cudaEventCreateWithFlags(&r->grad_need_event, cudaEventDisableTiming);
	if(err != cudaSuccess)
		return cudaFail(err, "fragment store host state");
	return allocate(r, &r->grad_state, 2);
}

static lucid_status checkGradInputs(lucid_renderer* r, const lucid_frame_inputs* in) {
	lucid_status st = validateInputs(r, in);
	if(st != LUCID_OK)
		return st;
	if(r->opts.flags & (LUCID_OPT_ADDITIVE_BLENDING | LUCID_OPT_ALPHA_THRESHOLD | LUCID_OPT_REFERENCE_ORDER))
		return fail(LUCID_NOT_SUPPORTED, "gradient passes support the exact-order front-to-back blend only");
	if(!r->px_color64) {
		const size_t npix = size_t(r->width) * r->height;
		if((st = allocate(r, &r->px_color64, npix * 3)) != LUCID_OK ||
		   (st = allocate(r, &r->px_color32, npix * 3)) != LUCID_OK ||
		   (st = allocate(r, &r->stats_image, npix * 4)) != LUCID_OK)
			return st;
	}
	return ensureStoreBuffers(r);
}

// Sizes the fragment store: a fixed capacity, none, or (automatic) at least 2^25 fragments and
// 1.25x the fragments of the last differentiable frame once that count is known on the host.
static lucid_status ensureGradStore(lucid_renderer* r, cudaStream_t s) {
	const int32_t opt = r->opts.grad_store_fragments;
	size_t want = r->grad_capacity;
	if(opt > 0) {
		want = size_t(opt);
	} else if(opt == 0) {
		want = std::max(want, size_t(1) << 25);
		if(r->grad_need_pending && cudaEventQuery(r->grad_need_event) == cudaSuccess) {
			r->grad_need_pending = false;
			const unsigned long long need = *r->grad_need_host;
			if(need > r->grad_capacity)
				want = std::max(want, size_t(need + need / 4));
		}
		cudaGetLastError(); // cudaEventQuery's cudaErrorNotReady
		want = std::min(want, size_t(0xffffffffu));
	} else {
		want = 0;
	}
	if(want == r->grad_capacity)
		return LUCID_OK;
	LUCID_CUDA_TRY(cudaStreamSynchronize(s));
	if(r->grad_tris) {
		cudaFree(r->grad_tris);
		r->grad_tris = nullptr;
		r->grad_capacity = 0;
	}
	if(want > 0) {
		cudaError_t err = cudaMalloc(&r->grad_tris, want * sizeof(uint32_t));
		if(err != cudaSuccess) {
			cudaGetLastError();
			r->grad_tris = nullptr; // no store: the raster pass recomputes the fragment lists
			return LUCID_OK;
		}
		r->grad_capacity = want;
	}
	return LUCID_OK;
}

namespace {

FrameParams gradParams(lucid_renderer* r) {
	FrameParams p = r->last;
	p.px_color64 = r->px_color64;
	p.px_color32 = r->px_color32;
	p.grad_tris = r->grad_tris;
	p.grad_px_off = r->grad_px_off;
	p.grad_px_cnt = r->grad_px_cnt;
	p.grad_state = r->grad_state;
	p.grad_capacity = r->grad_capacity;
	return p;
}

// Setup, binning and the differentiable forward: the raster pass in store mode and the
// pixel-parallel FP64 colour kernel, or, when the store cannot hold the frame, the raster
// pass's FP64 colour mode. Both alternatives are launched; each checks the store's overflow
// flag on the device and returns at once when it is not the one needed, so the host never
// waits for the outcome.
lucid_status gradForward(lucid_renderer* r, const lucid_frame_inputs* in, float* out, void* stream) {
	lucid_status st;
	cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
	if((st = ensureGradStore(r, s)) != LUCID_OK)
		return st;
	if((st = lucid_quad_setup(r, in, stream)) != LUCID_OK || (st = lucid_bin_count(r, stream)) != LUCID_OK ||
	   (st = lucid_bin_categorize(r, stream)) != LUCID_OK || (st = lucid_bin_dispatch(r, stream)) != LUCID_OK)
		return st;
	FrameParams p = gradParams(r);
	p.out_rgba = out;
	const size_t npix = size_t(r->width) * r->height;
	LUCID_CUDA_TRY(cudaMemsetAsync(r->grad_state, 0, 16, s));
	if(r->grad_capacity == 0)
		LUCID_CUDA_TRY(cudaMemsetAsync(r->grad_state, 1, 8, s)); // no store: flag it full
	LUCID_CUDA_TRY(cudaMemsetAsync(r->grad_px_cnt, 0, npix * 4, s));
	if((st = resetRasterCounters(r, s)) != LUCID_OK)
		return st;
	if(r->grad_capacity > 0) {
		launchRaster(p, r->raster_ctas, s, kRasterStore);
		if((st = checkLaunch("raster (store)")) != LUCID_OK)
			return st;
	}
	LUCID_CUDA_TRY(cudaMemsetAsync(&r->info()->raster_work_counter, 0, 4, s));
	launchRaster(p, r->raster_ctas, s, kRasterStats);
	if((st = checkLaunch("raster (FP64 colour)")) != LUCID_OK)
		return st;
	launchGradColor(p, s);
	if((st = checkLaunch("gradient colour")) != LUCID_OK)
		return st;
	if(r->grad_capacity > 0 && r->opts.grad_store_fragments == 0) {
		LUCID_CUDA_TRY(cudaMemcpyAsync(r->grad_need_host, &r->grad_state[1], 8, cudaMemcpyDeviceToHost, s));
		LUCID_CUDA_TRY(cudaEventRecord(r->grad_need_event, s));
		r->grad_need_pending = true;
	}
	r->grad_ready = true;
	r->grad_inputs = *in;
	r->grad_config = *in->config;
	return LUCID_OK;
}

} // namespace

extern "C" lucid_status lucid_render_forward_grad(lucid_renderer* r, const lucid_frame_inputs* in,
												  float* out_rgba, void* stream) {
	if(!r || !out_rgba)
		return fail(LUCID_INVALID_ARG, "lucid_render_forward_grad: renderer and out_rgba are required");
	lucid_status st = checkGradInputs(r, in);
	if(st != LUCID_OK)
		return st;
	return gradForward(r, in, out_rgba, stream);
}

extern "C" lucid_status lucid_render_backward(lucid_renderer* r, const lucid_frame_inputs* in,
											  const float* dl_dimage, float* dvertex_rgba,
											  float* dtri_opacity, void* stream) {
	if(!r || !dl_dimage)
		return fail(LUCID_INVALID_ARG, "lucid_render_backward: renderer and dl_dimage are required");
	lucid_status st = checkGradInputs(r, in);
	if(st != LUCID_OK)
		return st;
	if(dvertex_rgba && in->color_format != LUCID_COLOR_RGBA32F)
		return fail(LUCID_INVALID_ARG, "vertex colour gradients need LUCID_COLOR_RGBA32F colours");
	if(reinterpret_cast<uintptr_t>(dvertex_rgba) % 16 != 0)
		return fail(LUCID_INVALID_ARG, "dvertex_rgba must be 16-byte aligned");
	if(dtri_opacity && !in->tri_opacity)
		return fail(LUCID_INVALID_ARG, "opacity gradients need inputs->tri_opacity");
	// Reuse the forward pass's bin lists and per-pixel colours when the last pass on this
	// renderer was lucid_render_forward_grad of the same inputs; otherwise recompute them.
	lucid_frame_inputs cmp = *in;
	cmp.config = r->grad_inputs.config; // the config is compared by contents
	const bool reuse = r->grad_ready && memcmp(&r->grad_inputs, &cmp, sizeof(cmp)) == 0 &&
					   memcmp(&r->grad_config, in->config, sizeof(lucid_config)) == 0;
	if(!reuse && (st = gradForward(r, in, r->stats_image, stream)) != LUCID_OK)
		return st;
	// the pixel-parallel backward over the fragment store, or (store overflowed) the raster
	// pass's backward mode; each returns at once when it is not the one needed
	cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
	FrameParams p = gradParams(r);
	p.out_rgba = r->stats_image;
	p.dl_dimage = dl_dimage;
	p.dvertex_rgba = dvertex_rgba;
	p.dtri_opacity = dtri_opacity;
	launchGradBackward(p, s);
	if((st = checkLaunch("gradient backward")) != LUCID_OK)
		return st;
	LUCID_CUDA_TRY(cudaMemsetAsync(&r->info()->raster_work_counter, 0, 4, s));
	launchRaster(p, r->raster_ctas, s, kRasterBackward);
	return checkLaunch("raster (backward)");
}

// ---------------------------------------------------------------------------------------------
// Batched frames (no reference counterpart)
//
// A batch renders every view with one launch per pass: CTA ranges of the setup and binning
// kernels map to views, and one persistent raster kernel walks the (view, bin) work list of all
// views. Views take consecutive slices of the renderer's quad / tri record buffers (capacity =
// the view's input quads) and share the bin reference lists through a device bump allocator.
// The launch sequence of a batch topology (view count, sizes, quad and instance counts) is
// recorded once as a CUDA graph and replayed by later calls; the graph's first node copies the
// views' parameters (input pointers, configs) from a pinned staging block, rewritten only when
// they change.

struct BatchPlan {
	std::vector<int64_t> key;
	int num_views = 0;
	int max_bins = 0;
	std::vector<FrameParams> params; // what params_pinned holds
	std::vector<size_t> info_off;    // byte offset of each view's info block in `infos`
	std::vector<int> binning_ctas;   // per view, fixed when the plan's buffers are sized
	size_t info_bytes = 0;
	BatchViews per_view{}, setup_map{}, binning_map{}, bin_map{};
	std::vector<void*> allocations;
	FrameParams* params_dev = nullptr;
	FrameParams* params_pinned = nullptr;
	unsigned char* infos = nullptr;
	int* inst_offsets = nullptr;
	int4* setup_counts = nullptr;
	int4* setup_offsets = nullptr;
	int* bin_batches = nullptr;
	uint32_t* raster_work = nullptr;
	int* level_prefix = nullptr;
	uint32_t* counters = nullptr; // [0] quad refs, [1] tri refs, [2] raster work
	cudaStream_t capture_stream = nullptr;
	cudaEvent_t done = nullptr;
	cudaGraphExec_t exec = nullptr;
};

static void destroyBatchPlan(lucid_renderer* r) {
	BatchPlan* b = r->batch;
	if(!b)
		return;
	if(b->done)
		cudaEventSynchronize(b->done);
	if(b->exec)
		cudaGraphExecDestroy(b->exec);
	if(b->done)
		cudaEventDestroy(b->done);
	if(b->capture_stream)
		cudaStreamDestroy(b->capture_stream);
	if(b->params_pinned)
		cudaFreeHost(b->params_pinned);
	for(void* p : b->allocations)
		cudaFree(p);
	delete b;
	r->batch = nullptr;
}

namespace {

template <typename T> lucid_status batchAlloc(BatchPlan* b, T** ptr, size_t count) {
	void* p = nullptr;
	size_t bytes = std::max<size_t>(count * sizeof(T), 16);
	cudaError_t err = cudaMalloc(&p, bytes);
	if(err != cudaSuccess) {
		cudaGetLastError();
		return fail(LUCID_OUT_OF_MEMORY, std::string("batch cudaMalloc(") + std::to_string(bytes) +
											 " bytes): " + cudaGetErrorString(err));
	}
	b->allocations.push_back(p);
	*ptr = reinterpret_cast<T*>(p);
	return LUCID_OK;
}

int viewBins(int w, int h) { return ((w + kBinSize - 1) / kBinSize) * ((h + kBinSize - 1) / kBinSize); }
int viewSetupCtas(int nq) { return (nq + kSetupThreads - 1) / kSetupThreads; }
int viewBinningCtas(const lucid_renderer* r, int nq) {
	return std::max(1, std::min(r->opts.binning_ctas, (nq + 2047) / 2048));
}

std::vector<int64_t> batchKey(const lucid_renderer* r, const lucid_view* views, int n) {
	std::vector<int64_t> key;
	key.reserve(4 + 4 * size_t(n));
	key.push_back(n);
	// options the recorded graph bakes in (grid shapes, the sort pass)
	key.push_back(r->opts.bin_size);
	key.push_back(r->opts.binning_ctas);
	key.push_back(int64_t(r->opts.flags & LUCID_OPT_SORTED_BIN_LISTS));
	for(int v = 0; v < n; v++) {
		key.push_back(views[v].width);
		key.push_back(views[v].height);
		key.push_back(views[v].inputs.num_quads);
		key.push_back(views[v].inputs.num_instances);
	}
	return key;
}

// Parameters of every view, pointing into the plan's and the renderer's buffers.
void batchParams(lucid_renderer* r, BatchPlan* b, const lucid_view* views, std::vector<FrameParams>& out) {
	const int n = b->num_views;
	out.assign(size_t(n), FrameParams{});
	size_t qbase = 0, ibase = 0, sbase = 0, bbase = 0, rbase = 0;
	for(int v = 0; v < n; v++) {
		const lucid_view& vw = views[v];
		const lucid_frame_inputs& in = vw.inputs;
		FrameParams& p = out[size_t(v)];
		p.positions = in.positions;
		p.colors = in.colors;
		p.color_format = in.color_format;
		p.num_verts = in.num_verts;
		p.quads_ib = in.quads_ib;
		p.num_quads = in.num_quads;
		p.num_instances = in.num_instances;
		p.instances = in.instances;
		p.instance_colors = in.instance_colors;
		p.tri_opacity = in.tri_opacity;
		setShadingInputs(p, &in);
		p.out_rgba = vw.out_rgba;
		p.cfg = *in.config;
		p.width = vw.width, p.height = vw.height;
		p.bin_shift = binShift(r->opts);
		binGrid(vw.width, vw.height, p.bin_shift, p.bin_count_x, p.bin_count_y);
		p.bin_count = p.bin_count_x * p.bin_count_y;
		const int nq = in.num_quads;
		const int cap = std::max(nq, 1);
		p.max_visible_quads = cap;
		p.max_bin_refs = r->opts.max_bin_refs;
		p.band_capacity = r->opts.band_capacity;
		p.low_high_threshold = r->opts.low_high_threshold;
		p.slab_target = slabTarget(r);
		p.light_max_pixel = lightMaxPixel(r);
		p.num_setup_ctas = viewSetupCtas(nq);
		p.num_binning_ctas = b->binning_ctas[size_t(v)];
		p.flags = r->opts.flags & ~uint32_t(LUCID_OPT_TIMERS);
		p.info = reinterpret_cast<lucid_info*>(b->infos + b->info_off[size_t(v)]);
		p.counts = reinterpret_cast<uint32_t*>(b->infos + b->info_off[size_t(v)] + sizeof(lucid_info));
		p.inst_offsets = b->inst_offsets + ibase;
		p.quad_class = r->quad_class + qbase;
		p.setup_cta_counts = b->setup_counts + sbase;
		p.setup_cta_offsets = b->setup_offsets + sbase;
		p.quad_aabbs = r->quad_aabbs + qbase;
		p.quad_source = r->quad_source + qbase;
		p.quad_verts = r->quad_verts + qbase;
		p.quad_colors = r->quad_colors + qbase;
		p.quad_normals = r->quad_normals + qbase;
		p.quad_tex = r->quad_tex + 2 * qbase;
		p.tri_shade = r->tri_shade + 2 * kShadeRecWords * qbase;
		p.tri_scan = r->tri_scan + 4 * qbase;
		p.tri_depth = r->tri_depth + 2 * qbase;
		p.tri_normals = r->tri_normals + 2 * qbase;
		p.bin_quads = r->bin_quads;
		p.bin_tris = r->bin_tris;
		p.bin_batches = b->bin_batches + bbase;
		p.raster_work = b->raster_work + rbase;
		p.band_scratch = r->band_scratch;
		p.band_keys = r->band_keys;
		p.band_planes = r->band_planes;
		p.ref_alloc = b->counters;
		qbase += size_t(cap);
		ibase += size_t(in.num_instances) + 1;
		sbase += size_t(std::max(p.num_setup_ctas, 1));
		bbase += size_t(p.num_binning_ctas) * 2 * size_t(p.bin_count);
		rbase += size_t(p.bin_count);
	}
}

lucid_status buildBatchPlan(lucid_renderer* r, const lucid_view* views, int n, std::vector<int64_t> key,
							cudaStream_t user_stream) {
	// the previous plan's graph may still run on the caller's stream
	LUCID_CUDA_TRY(cudaStreamSynchronize(user_stream));
	destroyBatchPlan(r);
	BatchPlan* b = new BatchPlan();
	r->batch = b;
	b->key = std::move(key);
	b->num_views = n;
	size_t quads = 0, insts = 0, setup_ctas = 0, hist = 0, bins = 0;
	b->info_off.resize(size_t(n));
	b->binning_ctas.resize(size_t(n));
	for(int v = 0; v < n; v++) {
		const int nq = views[v].inputs.num_quads;
		const int vb = viewBins(views[v].width, views[v].height);
		b->max_bins = std::max(b->max_bins, vb);
		quads += size_t(std::max(nq, 1));
		insts += size_t(views[v].inputs.num_instances) + 1;
		setup_ctas += size_t(std::max(viewSetupCtas(nq), 1));
		b->binning_ctas[size_t(v)] = viewBinningCtas(r, nq);
		hist += size_t(b->binning_ctas[size_t(v)]) * 2 * size_t(vb);
		bins += size_t(vb);
		b->info_off[size_t(v)] = b->info_bytes;
		b->info_bytes += (sizeof(lucid_info) + size_t(10) * vb * 4 + 255) & ~size_t(255);
	}
	lucid_status st;
	if(quads > size_t(r->opts.max_visible_quads) || quads > size_t(r->opts.max_input_quads)) {
		destroyBatchPlan(r);
		return fail(LUCID_CAPACITY_EXCEEDED, "batch: total quads " + std::to_string(quads) +
												  " exceed options.max_visible_quads / max_input_quads");
	}
	auto bail = [&](lucid_status e) {
		destroyBatchPlan(r);
		return e;
	};
	if((st = batchAlloc(b, &b->params_dev, size_t(n))) != LUCID_OK ||
	   (st = batchAlloc(b, &b->infos, b->info_bytes)) != LUCID_OK ||
	   (st = batchAlloc(b, &b->inst_offsets, insts)) != LUCID_OK ||
	   (st = batchAlloc(b, &b->setup_counts, setup_ctas)) != LUCID_OK ||
	   (st = batchAlloc(b, &b->setup_offsets, setup_ctas)) != LUCID_OK ||
	   (st = batchAlloc(b, &b->bin_batches, hist)) != LUCID_OK ||
	   (st = batchAlloc(b, &b->raster_work, bins)) != LUCID_OK ||
	   (st = batchAlloc(b, &b->level_prefix, size_t(3) * (n + 1))) != LUCID_OK ||
	   (st = batchAlloc(b, &b->counters, 4)) != LUCID_OK)
		return bail(st);
	cudaError_t err = cudaHostAlloc(reinterpret_cast<void**>(&b->params_pinned), sizeof(FrameParams) * size_t(n),
									cudaHostAllocDefault);
	if(err != cudaSuccess)
		return bail(cudaFail(err, "cudaHostAlloc (batch parameters)"));
	if((err = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking)) != cudaSuccess ||
	   (err = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming)) != cudaSuccess)
		return bail(cudaFail(err, "batch stream / event"));

	// CTA maps of the passes
	BatchViews* maps[4] = {&b->per_view, &b->setup_map, &b->binning_map, &b->bin_map};
	for(BatchViews* m : maps) {
		m->views = b->params_dev;
		m->num_views = n;
		m->cta_off[0] = 0;
	}
	for(int v = 0; v < n; v++) {
		const int nq = views[v].inputs.num_quads;
		b->per_view.cta_off[v + 1] = v + 1;
		b->setup_map.cta_off[v + 1] = b->setup_map.cta_off[v] + viewSetupCtas(nq);
		b->binning_map.cta_off[v + 1] = b->binning_map.cta_off[v] + b->binning_ctas[size_t(v)];
		b->bin_map.cta_off[v + 1] = b->bin_map.cta_off[v] + viewBins(views[v].width, views[v].height);
	}

	// record the frame
	cudaStream_t cs = b->capture_stream;
	if((err = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
		return bail(cudaFail(err, "cudaStreamBeginCapture"));
	cudaMemcpyAsync(b->params_dev, b->params_pinned, sizeof(FrameParams) * size_t(n), cudaMemcpyHostToDevice, cs);
	cudaMemsetAsync(b->infos, 0, b->info_bytes, cs);
	cudaMemsetAsync(b->counters, 0, 16, cs);
	launchSetupBatch(b->per_view, b->setup_map, cs);
	launchBinningBatch(b->per_view, b->binning_map, b->bin_map, b->max_bins,
					   (r->opts.flags & LUCID_OPT_SORTED_BIN_LISTS) != 0, cs);
	launchRasterBatch(b->params_dev, n, b->level_prefix, b->counters + 2, r->raster_ctas, cs);
	cudaGraph_t graph = nullptr;
	cudaError_t cap_err = cudaStreamEndCapture(cs, &graph);
	cudaError_t launch_err = cudaGetLastError();
	if(cap_err != cudaSuccess || launch_err != cudaSuccess) {
		if(graph)
			cudaGraphDestroy(graph);
		return bail(cudaFail(cap_err != cudaSuccess ? cap_err : launch_err, "batch capture"));
	}
	err = cudaGraphInstantiate(&b->exec, graph, 0);
	cudaGraphDestroy(graph);
	if(err != cudaSuccess)
		return bail(cudaFail(err, "cudaGraphInstantiate"));
	return LUCID_OK;
}

} // namespace

extern "C" lucid_status lucid_render_batch(lucid_renderer* r, const lucid_view* views,
										   int32_t num_views, void* stream) {
	if(!r || !views || num_views <= 0)
		return fail(LUCID_INVALID_ARG, "lucid_render_batch: renderer, views and num_views > 0 are required");
	if(r->opts.flags & (LUCID_OPT_REFERENCE_ORDER | LUCID_OPT_PIXEL_BLEND))
		return fail(LUCID_NOT_SUPPORTED, "lucid_render_batch renders the exact order with the raster-pass blend");
	if(num_views > r->opts.max_views || num_views > kMaxBatchViews)
		return fail(LUCID_CAPACITY_EXCEEDED, "lucid_render_batch: num_views " + std::to_string(num_views) +
												  " > options.max_views (at most " + std::to_string(kMaxBatchViews) +
												  ")");
	for(int v = 0; v < num_views; v++) {
		const lucid_view& vw = views[v];
		if(vw.width <= 0 || vw.height <= 0 || vw.width > r->width || vw.height > r->height)
			return fail(LUCID_INVALID_ARG, "view " + std::to_string(v) + ": size must be within the renderer's");
		if(!vw.out_rgba)
			return fail(LUCID_INVALID_ARG, "view " + std::to_string(v) + ": out_rgba is NULL");
		lucid_status st = validateInputs(r, &vw.inputs);
		if(st != LUCID_OK)
			return fail(st, "view " + std::to_string(v) + ": " + g_last_error);
	}
	cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
	cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
	LUCID_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
	if(cap != cudaStreamCaptureStatusNone)
		return fail(LUCID_NOT_SUPPORTED, "lucid_render_batch records and replays its own CUDA graph; "
										 "call it outside stream capture");
	r->have_frame = false; // the single-view buffers are reused by the batch
	r->grad_ready = false;
	std::vector<int64_t> key = batchKey(r, views, num_views);
	lucid_status st;
	if(!r->batch || r->batch->key != key) {
		if((st = buildBatchPlan(r, views, num_views, std::move(key), s)) != LUCID_OK)
			return st;
	}
	BatchPlan* b = r->batch;
	std::vector<FrameParams> params;
	batchParams(r, b, views, params);
	const size_t bytes = sizeof(FrameParams) * params.size();
	if(b->params.size() != params.size() || memcmp(b->params.data(), params.data(), bytes) != 0) {
		// the previous replay's copy node must have read the staging block first
		LUCID_CUDA_TRY(cudaEventSynchronize(b->done));
		memcpy(b->params_pinned, params.data(), bytes);
		b->params.swap(params);
	}
	LUCID_CUDA_TRY(cudaGraphLaunch(b->exec, s));
	LUCID_CUDA_TRY(cudaEventRecord(b->done, s));
	return LUCID_OK;
}

extern "C" lucid_status lucid_quad_generate(const float* positions, int32_t num_verts, const int32_t* tris,
											int32_t num_tris, float square_weight, uint32_t* out_quads,
											int32_t* out_num_quads, int32_t* out_num_degenerate, void* stream) {
	if(!out_num_quads || num_tris < 0 || num_verts < 0 || (num_tris > 0 && (!positions || !tris || !out_quads)))
		return fail(LUCID_INVALID_ARG, "lucid_quad_generate: bad arguments");
	if(int64_t(num_tris) * 6 > int64_t(1) << 31)
		return fail(LUCID_CAPACITY_EXCEEDED, "lucid_quad_generate: too many triangles");
	std::string err;
	int nq = 0, nd = 0;
	const int rc = quadGenerate(positions, num_verts, tris, num_tris, square_weight, out_quads, &nq, &nd,
								reinterpret_cast<cudaStream_t>(stream), err);
	if(rc == 1)
		return fail(LUCID_INVALID_ARG, err);
	if(rc == 2)
		return fail(LUCID_OUT_OF_MEMORY, err);
	if(rc != 0)
		return fail(LUCID_CUDA_ERROR, err);
	*out_num_quads = nq;
	if(out_num_degenerate)
		*out_num_degenerate = nd;
	return LUCID_OK;
}

extern "C" lucid_status lucid_get_batch_info(lucid_renderer* r, int32_t view, lucid_info* out, void* stream) {
	if(!r || !out || !r->batch || view < 0 || view >= r->batch->num_views)
		return fail(LUCID_INVALID_ARG, "lucid_get_batch_info: no such view of the last batch");
	LUCID_CUDA_TRY(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)));
	LUCID_CUDA_TRY(cudaMemcpy(out, r->batch->infos + r->batch->info_off[size_t(view)], sizeof(lucid_info),
							  cudaMemcpyDeviceToHost));
	return LUCID_OK;
}

namespace {

// Coordinate descent over the renderer's options, timing `frame` (one lucid_render or one
// lucid_render_batch): CUDA events on `s`, median of 3 after a warm-up call per candidate. The
// winner stays in r->opts; on failure the options are restored.
lucid_status autotuneCore(lucid_renderer* r, cudaStream_t s, bool pixel_blend_candidate,
						  const std::function<lucid_status()>& frame, lucid_tuning* out) {
	cudaEvent_t e0, e1;
	LUCID_CUDA_TRY(cudaEventCreate(&e0));
	cudaError_t cerr = cudaEventCreate(&e1);
	if(cerr != cudaSuccess) {
		cudaEventDestroy(e0);
		return cudaFail(cerr, "cudaEventCreate");
	}
	const lucid_options saved = r->opts;
	int candidates = 0;
	auto timeFrame = [&](float& ms) -> lucid_status {
		float t[3];
		for(int i = 0; i < 4; i++) {
			cudaEventRecord(e0, s);
			lucid_status rs = frame();
			if(rs != LUCID_OK)
				return rs;
			cudaEventRecord(e1, s);
			cudaError_t err = cudaEventSynchronize(e1);
			if(err != cudaSuccess)
				return cudaFail(err, "autotune frame");
			if(i > 0)
				cudaEventElapsedTime(&t[i - 1], e0, e1);
		}
		std::sort(t, t + 3);
		ms = t[1];
		candidates++;
		return LUCID_OK;
	};
	float best_ms = 0.0f, default_ms = 0.0f;
	lucid_status st;
	if((st = timeFrame(default_ms)) == LUCID_OK) {
		best_ms = default_ms;
		lucid_options best = r->opts;
		auto tryOpts = [&](const lucid_options& o) -> lucid_status {
			r->opts = o;
			float ms = 0.0f;
			lucid_status rs = timeFrame(ms);
			if(rs == LUCID_OK && ms < best_ms)
				best_ms = ms, best = o;
			r->opts = best;
			return rs;
		};
		lucid_options o = best;
		// 0. bin size: 32 or 64 pixels (64-pixel bins are rastered as four 32x32 tiles: fewer
		// bin references and binning atomics, each tile scans its bin's whole lists)
		if(!(best.flags & LUCID_OPT_REFERENCE_ORDER)) {
			o.bin_size = best.bin_size == 64 ? 32 : 64;
			st = tryOpts(o);
		}
		// 1. blend strategy (not for batches: lucid_render_batch blends in the raster pass)
		o = best;
		o.flags ^= LUCID_OPT_PIXEL_BLEND;
		if(st == LUCID_OK && pixel_blend_candidate)
			st = tryOpts(o);
		// 2. LOW/HIGH threshold (raster work order)
		for(int th : {256, 1024, 4096}) {
			if(st != LUCID_OK || th == best.low_high_threshold)
				continue;
			o = best;
			o.low_high_threshold = th;
			st = tryOpts(o);
		}
		// 3. binning CTAs (within what the histogram scratch is sized for)
		for(int ctas : {r->num_sms, 2 * r->num_sms}) {
			if(st != LUCID_OK || ctas == best.binning_ctas || ctas > r->binning_ctas_alloc)
				continue;
			o = best;
			o.binning_ctas = ctas;
			st = tryOpts(o);
		}
		// 4. per-bin raster path: the deepest pixel of a bin that is rastered one warp per row
		// (light path) instead of by CTA-wide depth windows (-1: every bin by windows)
		for(int lm : {-1, 32, 64, 128, 256}) {
			if(st != LUCID_OK || lm == lightMaxPixel(&best))
				continue;
			o = best;
			o.light_max_pixel = lm;
			st = tryOpts(o);
		}
		r->opts = st == LUCID_OK ? best : saved;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if(st != LUCID_OK) {
		r->opts = saved;
		return st;
	}
	if(out) {
		memset(out, 0, sizeof(*out));
		out->pixel_blend = (r->opts.flags & LUCID_OPT_PIXEL_BLEND) ? 1u : 0u;
		out->low_high_threshold = r->opts.low_high_threshold;
		out->binning_ctas = r->opts.binning_ctas;
		out->light_max_pixel = lightMaxPixel(r);
		out->bin_size = r->opts.bin_size;
		out->num_candidates = candidates;
		out->frame_ms = best_ms;
		out->default_ms = default_ms;
	}
	return LUCID_OK;
}

} // namespace

extern "C" lucid_status lucid_autotune(lucid_renderer* r, const lucid_frame_inputs* in,
									   float* scratch_rgba, lucid_tuning* out, void* stream) {
	if(!r || !scratch_rgba)
		return fail(LUCID_INVALID_ARG, "lucid_autotune: renderer and scratch_rgba are required");
	lucid_status st = validateInputs(r, in);
	if(st != LUCID_OK)
		return st;
	return autotuneCore(r, reinterpret_cast<cudaStream_t>(stream), r->opts.max_views <= 1,
						[&]() { return lucid_render(r, in, scratch_rgba, stream); }, out);
}

extern "C" lucid_status lucid_autotune_batch(lucid_renderer* r, const lucid_view* views, int32_t num_views,
											 lucid_tuning* out, void* stream) {
	if(!r || !views || num_views <= 0)
		return fail(LUCID_INVALID_ARG, "lucid_autotune_batch: renderer, views and num_views > 0 are required");
	if(r->opts.flags & (LUCID_OPT_REFERENCE_ORDER | LUCID_OPT_PIXEL_BLEND))
		return fail(LUCID_NOT_SUPPORTED, "lucid_autotune_batch: batches render the exact order with the raster-pass blend");
	return autotuneCore(r, reinterpret_cast<cudaStream_t>(stream), false,
						[&]() { return lucid_render_batch(r, views, num_views, stream); }, out);
}
