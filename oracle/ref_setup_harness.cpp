/*
 * Harness of the reference's setup, bin-counter, row-span, shading and reduction functions
 * compiled as C++ (see oracle/ref_build.py).
 *
 * TEST INFRASTRUCTURE ONLY: tests/test_oracle_ref_pin.py compares its records with the oracle's
 * to pin the oracle's setup stage to the reference's own source. The functions that do the
 * arithmetic (processInputQuad, storeTri, storeQuad, addVisibleTri, addVisibleQuad and their
 * helpers) come from data/shaders/quad_setup.glsl and shared/funcs.glsl; this file only
 * provides their buffers and drives them in the order of the shader's main()
 * (quad_setup.glsl:374-489), one invocation at a time: shared-memory atomics become plain
 * increments, so every workgroup lists its visible quads in input order, as the oracle does.
 */
#include <cstdint>
#include <cstring>
#include <vector>

#include "glsl_shim.h"
#include "lucid_gb300.h"

namespace glsl {

// specialization constants (definitions.glsl:40-58); the bin size is 32 in every build
constexpr int BIN_SIZE = 32, BIN_SHIFT = 5;
// one invocation at a time: a subgroup of one (shading.glsl's shuffles pick lane `bit`)
#define SUBGROUP_SIZE 32
#define HALFGROUP_SIZE 32
int VIEWPORT_SIZE_X = 0, VIEWPORT_SIZE_Y = 0, MAX_VISIBLE_QUADS = 0, MAX_VISIBLE_TRIS = 0;
int BIN_COUNT_X = 0, BIN_COUNT_Y = 0, BIN_COUNT = 0;
struct {
	uint x;
} gl_WorkGroupID = {0u};

#include "ref_setup_gen.inc"

int* s_bins;
uvec2* g_scratch_64;
ivec2 s_bin_pos;

LucidConfig u_config;
float* g_verts;
vec2* g_tex_coords;
uint* g_colors;
uint* g_normals;
uint* g_quad_aabbs;
uvec4* g_uvec4_storage;
uint* g_normals_storage;
InstanceData* g_instances;
uint* g_instance_colors;
vec4* g_instance_uv_rects;
sampler2D opaque_texture, transparent_texture;
uint s_stats[STATS_COUNT];
float (*g_pow)(float, float) = nullptr;
int g_texture_calls = 0;

// the last ref_quad_setup's storage, read by ref_shade_samples
std::vector<uvec4> g_setup_storage;
std::vector<uint> g_setup_normals;

} // namespace glsl

using namespace glsl;

extern "C" {

typedef struct ref_setup_inputs {
	int32_t width, height, max_visible_quads;
	const float* positions;     /* float3 per vertex            */
	const uint32_t* colors;     /* RGBA8 per vertex (may be 0)  */
	const uint32_t* normals;    /* encoded per vertex (may be 0)*/
	const float* tex_coords;    /* float2 per vertex (may be 0) */
	const uint32_t* quads_ib;
	const lucid_instance* instances;
	int32_t num_instances;
	const lucid_config* config;
} ref_setup_inputs;

typedef struct ref_setup_outputs {
	uint32_t* quad_aabbs;  /* [mvq]          */
	uint32_t* tri_bary;    /* [2*mvq*8]      */
	uint32_t* tri_scan;    /* [2*mvq*8]      */
	uint32_t* tri_depth;   /* [2*mvq*4]      */
	uint32_t* tri_normals; /* [2*mvq]        */
	uint32_t* quad_colors; /* [mvq*4]        */
	int32_t num_input_quads;
	int32_t num_visible[2];
	uint32_t rejected[4];
} ref_setup_outputs;

static vec4 v4(const float* f) { return vec4(f[0], f[1], f[2], f[3]); }

int ref_quad_setup(const ref_setup_inputs* in, ref_setup_outputs* out) {
	const int mvq = in->max_visible_quads;
	VIEWPORT_SIZE_X = in->width, VIEWPORT_SIZE_Y = in->height;
	MAX_VISIBLE_QUADS = mvq;
	MAX_VISIBLE_TRIS = 2 * mvq;
	// LucidConfig by field (the C++ struct's layout is the shim's, not std140)
	const lucid_config& c = *in->config;
	for(int i = 0; i < 4; i++) {
		u_config.frustum.ws_origins[i] = v4(c.frustum.ws_origins[i]);
		u_config.frustum.ws_dirs[i] = v4(c.frustum.ws_dirs[i]);
		u_config.view_proj_matrix.col[i] = v4(c.view_proj_matrix + 4 * i);
	}
	u_config.frustum.ws_origin0 = v4(c.frustum.ws_origin0);
	u_config.frustum.ws_dir0 = v4(c.frustum.ws_dir0);
	u_config.frustum.ws_dirx = v4(c.frustum.ws_dirx);
	u_config.frustum.ws_diry = v4(c.frustum.ws_diry);
	u_config.enable_backface_culling = c.enable_backface_culling;
	u_config.num_instances = in->num_instances;
	u_config.instance_packet_size = c.instance_packet_size > 0 ? c.instance_packet_size : 1;

	std::vector<uvec4>& storage = g_setup_storage;
	std::vector<uint>& normals_storage = g_setup_normals;
	storage.assign(size_t(mvq) * 14, uvec4());
	normals_storage.assign(size_t(2) * mvq, 0u);
	std::vector<uint> quad_aabbs(mvq);
	std::vector<InstanceData> instances(size_t(in->num_instances));
	std::memcpy(instances.data(), in->instances, sizeof(lucid_instance) * size_t(in->num_instances));
	g_verts = const_cast<float*>(in->positions);
	g_colors = const_cast<uint*>(in->colors);
	g_normals = const_cast<uint*>(in->normals);
	g_tex_coords = reinterpret_cast<vec2*>(const_cast<float*>(in->tex_coords));
	g_quad_aabbs = quad_aabbs.data();
	g_uvec4_storage = storage.data();
	g_normals_storage = normals_storage.data();
	g_instances = instances.data();

	// main() (quad_setup.glsl:374-489) workgroup by workgroup, one invocation at a time
	const int packet = u_config.instance_packet_size;
	int num_input_quads = 0, num_visible[2] = {0, 0};
	uint rejected[4] = {0, 0, 0, 0};
	const int num_wgs = (in->num_instances + packet - 1) / packet;
	for(int wg = 0; wg < num_wgs; wg++) {
		for(int lix = 0; lix < packet; lix++) {
			const int instance_id = wg * packet + lix;
			if(instance_id < u_config.num_instances) {
				s_instances[lix] = g_instances[instance_id];
				s_quad_offset[lix] = atomicAdd(num_input_quads, s_instances[lix].num_quads);
				s_instance_id[lix] = instance_id;
			} else {
				s_instances[lix].num_quads = 0;
			}
		}
		for(int lix = 0; lix < packet * 2; lix++)
			s_num_visible[lix] = 0;
		for(int lix = 0; lix < 4; lix++)
			s_rejected_quads[lix] = 0;
		{
			const vec4 dxy = u_config.frustum.ws_dirx + u_config.frustum.ws_diry;
			s_ray_dir0 = vec3(u_config.frustum.ws_dir0.x, u_config.frustum.ws_dir0.y, u_config.frustum.ws_dir0.z) +
						 vec3(dxy.x, dxy.y, dxy.z) * 0.5f;
		}
		for(int i = 0; i < packet; i++) {
			for(int lix = 0; lix < s_instances[i].num_quads; lix++) {
				const int vertex_offset = s_instances[i].vertex_offset;
				const int index_offset = s_instances[i].index_offset + lix * 4;
				const uint v0 = in->quads_ib[index_offset + 0] + uint(vertex_offset);
				const uint v1 = in->quads_ib[index_offset + 1] + uint(vertex_offset);
				const uint v2 = in->quads_ib[index_offset + 2] + uint(vertex_offset);
				const uint v3 = in->quads_ib[index_offset + 3] + uint(vertex_offset);
				processInputQuad(uint(s_quad_offset[i] + lix), v0, v1, v2, v3, uint(i));
			}
			for(int lix = 0; lix < 2; lix++) {
				const int num_tris = s_num_visible[i * 2 + lix];
				const int offset = atomicAdd(num_visible[lix], num_tris);
				if(offset + num_tris > MAX_VISIBLE_TRIS)
					s_num_visible[i * 2 + lix] = std::max(0, MAX_VISIBLE_TRIS - offset);
				s_out_offset[lix] = offset;
			}
			const int num_small = s_num_visible[i * 2 + 0];
			const int num_large = s_num_visible[i * 2 + 1];
			const int num_tris = (num_small + num_large) * 2;
			const int instance_id = s_instance_id[i];
			const uint instance_flags_id = s_instances[i].flags | (uint(instance_id) << 16);
			for(int j = 0; j < num_tris; j++) {
				const int local_quad_idx = j >> 1, second_tri = j & 1;
				int quad_idx, src_idx;
				if(local_quad_idx < num_small) {
					src_idx = local_quad_idx;
					quad_idx = s_out_offset[0] + src_idx;
				} else {
					src_idx = local_quad_idx - num_small;
					quad_idx = (MAX_VISIBLE_QUADS - 1) - (s_out_offset[1] + src_idx);
					src_idx = (LSIZE - 1) - src_idx;
				}
				addVisibleTri(quad_idx, src_idx, instance_flags_id, second_tri);
			}
			for(int lix = 0; lix < LSIZE; lix++) {
				int quad_idx = -1, src_idx = 0;
				if(lix < num_small) {
					src_idx = lix;
					quad_idx = s_out_offset[0] + src_idx;
				} else if(lix - num_small < num_large) {
					src_idx = lix - num_small;
					quad_idx = (MAX_VISIBLE_QUADS - 1) - (s_out_offset[1] + src_idx);
					src_idx = (LSIZE - 1) - src_idx;
				}
				if(quad_idx != -1)
					addVisibleQuad(quad_idx, src_idx, instance_id);
			}
		}
		for(int lix = 0; lix < 4; lix++)
			rejected[lix] += s_rejected_quads[lix];
	}

	out->num_input_quads = num_input_quads;
	out->num_visible[0] = num_visible[0], out->num_visible[1] = num_visible[1];
	for(int k = 0; k < 4; k++)
		out->rejected[k] = rejected[k];
	std::memcpy(out->quad_aabbs, quad_aabbs.data(), size_t(mvq) * 4);
	std::memcpy(out->tri_bary, storage.data() + STORAGE_TRI_BARY_OFFSET, size_t(mvq) * 4 * 16);
	std::memcpy(out->tri_scan, storage.data() + STORAGE_TRI_SCAN_OFFSET, size_t(mvq) * 4 * 16);
	std::memcpy(out->tri_depth, storage.data() + STORAGE_TRI_DEPTH_OFFSET, size_t(mvq) * 2 * 16);
	std::memcpy(out->quad_colors, storage.data() + STORAGE_QUAD_COLOR_OFFSET, size_t(mvq) * 16);
	std::memcpy(out->tri_normals, normals_storage.data(), size_t(mvq) * 2 * 4);
	return 0;
}

// Tri records of the caller (oracle layout: 2 uvec4 per tri) in the reference's storage layout.
static std::vector<uvec4> scanStorage(const uint32_t* tri_scan, int mvq) {
	std::vector<uvec4> storage(size_t(mvq) * 14);
	std::memcpy(storage.data() + STORAGE_TRI_SCAN_OFFSET, tri_scan, size_t(mvq) * 4 * 16);
	return storage;
}

static void setView(int width, int height, int mvq) {
	VIEWPORT_SIZE_X = width, VIEWPORT_SIZE_Y = height;
	MAX_VISIBLE_QUADS = mvq;
	BIN_COUNT_X = (width + BIN_SIZE - 1) / BIN_SIZE, BIN_COUNT_Y = (height + BIN_SIZE - 1) / BIN_SIZE;
	BIN_COUNT = BIN_COUNT_X * BIN_COUNT_Y;
}

/* Per-bin quad and tri counts of the bin counter (bin_counter.glsl): countSmallQuadBins for every
 * visible small quad, countLargeTriBins for both tris of every visible large quad, then the
 * per-row prefix sum that closes the large tris' difference arrays (accumulateLargeTriCounts-
 * AcrossRows, whose scalar form the file keeps in a comment). Inputs: the setup records of
 * num_small / num_large visible quads in the oracle's layout. */
int ref_bin_counts(const uint32_t* quad_aabbs, const uint32_t* tri_scan, int32_t num_small, int32_t num_large,
				   int32_t max_visible_quads, int32_t width, int32_t height, uint32_t* quad_counts,
				   uint32_t* tri_counts) {
	setView(width, height, max_visible_quads);
	std::vector<uvec4> storage = scanStorage(tri_scan, max_visible_quads);
	std::vector<uint> aabbs(quad_aabbs, quad_aabbs + max_visible_quads);
	std::vector<int> bins(size_t(BIN_COUNT), 0);
	g_uvec4_storage = storage.data();
	g_quad_aabbs = aabbs.data();
	s_bins = bins.data();
	for(int k = 0; k < num_small; k++)
		countSmallQuadBins(uint(k));
	for(int i = 0; i < BIN_COUNT; i++)
		quad_counts[i] = uint32_t(bins[size_t(i)]), bins[size_t(i)] = 0;
	for(int k = 0; k < num_large; k++)
		for(int second = 0; second < 2; second++)
			countLargeTriBins((MAX_VISIBLE_QUADS - 1) - k, second);
	for(int by = 0; by < BIN_COUNT_Y; by++) {
		int accum = 0;
		for(int bx = 0; bx < BIN_COUNT_X; bx++)
			tri_counts[by * BIN_COUNT_X + bx] = uint32_t(accum += bins[size_t(by * BIN_COUNT_X + bx)]);
	}
	return 0;
}

/* Per-pixel fragment counts from the row spans of the low-level raster (raster_low.glsl):
 * generateRowTris of every visible tri in every bin of its bin AABB, one tri at a time, its
 * scratch entries decoded back into per-row spans (4 x 5-bit minima and maxima per 4 rows, the
 * empty row marked min 31 / max 0); pixels outside the viewport are not counted. */
int ref_coverage(const uint32_t* quad_aabbs, const uint32_t* tri_scan, int32_t num_small, int32_t num_large,
				 int32_t max_visible_quads, int32_t width, int32_t height, int32_t* counts) {
	setView(width, height, max_visible_quads);
	std::vector<uvec4> storage = scanStorage(tri_scan, max_visible_quads);
	std::vector<uvec2> scratch(size_t(1) << WORKGROUP_SCRATCH_SHIFT);
	g_uvec4_storage = storage.data();
	g_scratch_64 = scratch.data();
	std::memset(counts, 0, sizeof(int32_t) * size_t(width) * height);
	auto tri = [&](uint tri_idx, uint enc) {
		const ivec4 aabb = decodeAABB28(enc);
		for(int by = aabb[1]; by <= aabb[3]; by++)
			for(int bx = aabb[0]; bx <= aabb[2]; bx++) {
				s_bin_pos = ivec2(bx * BIN_SIZE, by * BIN_SIZE);
				for(int r = 0; r < BLOCK_ROWS; r++)
					s_block_row_tri_count[r] = 0;
				generateRowTris(tri_idx);
				for(int brow = 0; brow < BLOCK_ROWS; brow++) {
					if(s_block_row_tri_count[brow] == 0)
						continue;
					const uint off = scratchBlockRowOffset(0) + uint(brow) * (MAX_BLOCK_ROW_TRIS * 2);
					const uvec2 mins = g_scratch_64[off], maxs = g_scratch_64[off + MAX_BLOCK_ROW_TRIS];
					for(int r = 0; r < BLOCK_SIZE; r++) {
						const uint mn = ((r < 4 ? mins.x : mins.y) >> (5 * (r & 3))) & 31u;
						const uint mx = ((r < 4 ? maxs.x : maxs.y) >> (5 * (r & 3))) & 31u;
						const int py = by * BIN_SIZE + brow * BLOCK_SIZE + r;
						if(mn > mx || py >= height)
							continue;
						for(uint x = mn; x <= mx; x++) {
							const int px = bx * BIN_SIZE + int(x);
							if(px < width)
								counts[size_t(py) * width + px]++;
						}
					}
				}
			}
	};
	for(int k = 0; k < num_small; k++)
		for(uint second = 0; second < 2; second++)
			if(((quad_aabbs[k] >> (30 + second)) & 1u) == 0u)
				tri(uint(k) * 2 + second, quad_aabbs[k]);
	for(int k = 0; k < num_large; k++) {
		const int q = (max_visible_quads - 1) - k;
		for(uint second = 0; second < 2; second++)
			if(((quad_aabbs[q] >> (30 + second)) & 1u) == 0u)
				tri(uint(q) * 2 + second, quad_aabbs[q]);
	}
	return 0;
}

// shadeSample (shading.glsl:107-184) of the samples (px[i], py[i], tris[i]) on the last
// ref_quad_setup's records, with the scene's instance colours, lighting and background; RGBA8
// colour and depth (inv_ray_pos) per sample. pow_fn is GLSL's implementation-defined pow.
// Returns how many samples reached the texture stub (the tests' scenes have no textures: 0).
int ref_shade_samples(const lucid_config* cfg, const uint32_t* instance_colors, float (*pow_fn)(float, float),
					  int32_t n, const int32_t* px, const int32_t* py, const uint32_t* tris, uint32_t* colors,
					  float* depths) {
	g_uvec4_storage = g_setup_storage.data();
	g_normals_storage = g_setup_normals.data();
	g_instance_colors = const_cast<uint*>(instance_colors);
	g_pow = pow_fn;
	const lucid_lighting& L = cfg->lighting;
	u_config.lighting.ambient_color = v4(L.ambient_color);
	u_config.lighting.sun_color = v4(L.sun_color);
	u_config.lighting.sun_dir = v4(L.sun_dir);
	u_config.lighting.sun_power = L.sun_power;
	u_config.lighting.ambient_power = L.ambient_power;
	u_config.background_color = v4(cfg->background_color);
	g_texture_calls = 0;
	for(int i = 0; i < n; i++) {
		float depth = 0.0f;
		colors[i] = shadeSample(ivec2(px[i], py[i]), tris[i], depth);
		depths[i] = depth;
	}
	return g_texture_calls;
}

// One pixel's samples (RGBA8 colour, depth) through the 3-deep reduction window:
// initReduceSamples, reduceSample per sample, finishReduceSamples (shading.glsl:196-314). The
// samples come in segments (seg[i], non-decreasing), as shadeAndReduceSamples hands them over
// (raster.glsl:361-398): the colour a segment accumulates is saturated at its end.
int ref_reduce(const float* background, int32_t n, const uint32_t* colors, const float* depths, const int32_t* seg,
			   float* rgba) {
	u_config.background_color = v4(background);
	ReductionContext ctx;
	initReduceSamples(ctx);
	for(int i = 0; i < n;) {
		vec3 out_color = ctx.out_color;
		const int sg = seg[i];
		for(; i < n && seg[i] == sg; i++)
			reduceSample(ctx, out_color, uvec2(colors[i], floatBitsToUint(depths[i])), 1u);
		ctx.out_color = SATURATE(out_color);
	}
	const vec4 r = finishReduceSamples(ctx);
	for(int k = 0; k < 4; k++)
		rgba[k] = r[k];
	return 0;
}

} // extern "C"
