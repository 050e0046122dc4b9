// Scalar CPU oracle of LucidRaster's compute rasterization path (test infrastructure only).
//
// Each function restates one piece of the reference shaders (paths relative to the
// LucidRaster source tree) in plain single-threaded C++ with IEEE float arithmetic, no FMA
// contraction (built with -ffp-contract=off) and the float->int conversion rules of the GPU
// (saturating, NaN -> 0). Bin lists are produced in canonical order (per bin, by slot).
//
// Setup, binning counts and per-pixel coverage are pinned to the reference's own shader
// functions compiled as C++ (oracle/ref_build.py); the header says what pins the rest.

#include "lucid_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>
#include <unordered_map>
#include <set>

namespace {

// ---------------------------------------------------------------------------------------------
// Arithmetic helpers with explicit evaluation order

struct V3 {
	float x, y, z;
};
struct V4 {
	float x, y, z, w;
};

inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline bool eq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
// GLSL dot/cross evaluated left to right
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
	return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline V3 xyz(const float* v) { return v3(v[0], v[1], v[2]); }

// GLSL int(float): truncation; saturating with NaN -> 0 (PTX cvt.rzi.s32.f32 semantics)
inline int f2i(float x) {
	if(x != x)
		return 0;
	if(x >= 2147483648.0f)
		return 2147483647;
	if(x <= -2147483648.0f)
		return (-2147483647 - 1);
	return (int)x;
}
inline uint32_t f2u(float x) {
	if(x != x || x <= 0.0f)
		return 0u;
	if(x >= 4294967296.0f)
		return 0xffffffffu;
	return (uint32_t)x;
}
inline uint32_t fbits(float f) {
	uint32_t u;
	memcpy(&u, &f, 4);
	return u;
}
inline float bitsf(uint32_t u) {
	float f;
	memcpy(&f, &u, 4);
	return f;
}
// Ascending key of "nearest first": larger inv_ray_pos sorts first.
inline uint32_t nearFirstKey(float inv_ray_pos) {
	uint32_t u = inv_ray_pos != inv_ray_pos ? 0x7fc00000u : fbits(inv_ray_pos);
	uint32_t asc = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
	return ~asc;
}

// mat4 (column-major) * vec4(p, 1): ((c0*x + c1*y) + c2*z) + c3
inline V4 mulPoint(const float* m, V3 p) {
	V4 r;
	r.x = m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12];
	r.y = m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13];
	r.z = m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14];
	r.w = m[3] * p.x + m[7] * p.y + m[11] * p.z + m[15];
	return r;
}

// funcs.glsl:52-59
inline uint32_t encodeAABB28(uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1) {
	return (x0 & 0x7fu) | ((y0 & 0x7fu) << 7) | ((x1 & 0x7fu) << 14) | ((y1 & 0x7fu) << 21);
}
inline void decodeAABB28(uint32_t a, int& x0, int& y0, int& x1, int& y1) {
	x0 = int(a & 0x7fu), y0 = int((a >> 7) & 0x7fu), x1 = int((a >> 14) & 0x7fu),
	y1 = int((a >> 21) & 0x7fu);
}
// funcs.glsl:28-33
inline uint32_t encodeNormalUint(V3 n) {
	uint32_t x = f2u(512.0f + n.x * 511.0f) & 0x3ffu;
	uint32_t y = f2u(512.0f + n.y * 511.0f) & 0x3ffu;
	uint32_t z = f2u(512.0f + n.z * 511.0f) & 0x3ffu;
	return x | (y << 10) | (z << 20);
}
// funcs.glsl:100-104
inline void decodeRGBA8(uint32_t c, float out[4]) {
	const float s = 1.0f / 255.0f;
	out[0] = float(c & 0xffu) * s;
	out[1] = float((c >> 8) & 0xffu) * s;
	out[2] = float((c >> 16) & 0xffu) * s;
	out[3] = float((c >> 24) & 0xffu) * s;
}
inline float halfToFloat(uint16_t h) {
	uint32_t sign = uint32_t(h >> 15) << 31;
	uint32_t exp = (h >> 10) & 0x1f, man = h & 0x3ff;
	uint32_t bits;
	if(exp == 0) {
		if(man == 0)
			bits = sign;
		else { // subnormal half -> normal float
			int e = -1;
			do {
				man <<= 1;
				e++;
			} while(!(man & 0x400));
			man &= 0x3ff;
			bits = sign | (uint32_t(127 - 15 - e) << 23) | (man << 13);
		}
	} else if(exp == 31)
		bits = sign | 0x7f800000u | (man << 13);
	else
		bits = sign | ((exp + 112) << 23) | (man << 13);
	return bitsf(bits);
}

// ---------------------------------------------------------------------------------------------
// Pass state

constexpr int kBinSize = 32, kBinShift = 5;
constexpr int kMaxDispatches = 256;

struct QuadResult {
	int cls = -1; // -1 rejected, 0 small, 1 large
	int reason = 0;
	uint32_t enc_aabb = 0, y_aabb[2] = {0, 0};
	uint32_t v[4] = {0, 0, 0, 0};
	bool bad_index = false;
};

struct State {
	const oracle_inputs* in;
	int w, h, bcx, bcy, bins, mvq;
	V3 origin, dir0, dirx, diry, ray_dir0;
	// outputs of setup
	std::vector<uint32_t> quad_aabbs, quad_source, quad_colors, quad_verts, quad_normals, quad_tex;
	std::vector<uint32_t> tri_bary, tri_scan, tri_depth, tri_normals;
	std::vector<uint32_t> quad_inst; // instance id per quad slot
	int nvis[2] = {0, 0};
	// binning
	std::vector<std::vector<uint32_t>> bin_quads, bin_tris;
};

V3 vertexLoad(const State& s, uint32_t idx) {
	const float* p = s.in->positions + size_t(idx) * 3;
	return v3(p[0], p[1], p[2]);
}

// quad_setup.glsl:68-72
uint32_t vertexClipMask(V4 p) {
	return (p.x < -p.w ? 0x001u : 0u) | (p.x > p.w ? 0x002u : 0u) | (p.y < -p.w ? 0x004u : 0u) |
		   (p.y > p.w ? 0x008u : 0u) | (p.z < -p.w ? 0x010u : 0u) | (p.z > p.w ? 0x020u : 0u);
}

// quad_setup.glsl:77-128 (Blinn's clipped screen coverage)
void computeClippedAABB(const V4 vn[3], const float inv_w[3], uint32_t clipmask, float aabb[4]) {
	aabb[0] = 1.0f, aabb[1] = 1.0f, aabb[2] = -1.0f, aabb[3] = -1.0f;
	int any_vis = 0;
	uint32_t or_clipmask = clipmask | (clipmask >> 8) | (clipmask >> 16);
	for(int i = 0; i < 3; i++) {
		uint32_t cur = clipmask >> (i * 8);
		if((cur & 0x3u) == 0) {
			any_vis |= 0x1;
			if(vn[i].x - aabb[0] * vn[i].w < 0.0f)
				aabb[0] = vn[i].x * inv_w[i];
			if(vn[i].x - aabb[2] * vn[i].w > 0.0f)
				aabb[2] = vn[i].x * inv_w[i];
		}
		if((cur & 0xcu) == 0) {
			any_vis |= 0x10;
			if(vn[i].y - aabb[1] * vn[i].w < 0.0f)
				aabb[1] = vn[i].y * inv_w[i];
			if(vn[i].y - aabb[3] * vn[i].w > 0.0f)
				aabb[3] = vn[i].y * inv_w[i];
		}
	}
	if((any_vis & 0x0f) == 0) {
		aabb[0] = -1.0f, aabb[2] = 1.0f;
	} else if((or_clipmask & 0x3u) != 0) {
		for(int i = 0; i < 3; i++) {
			uint32_t cur = clipmask >> (i * 8);
			if((cur & 0x1u) != 0 && vn[i].x - aabb[0] * vn[i].w < 0.0f)
				aabb[0] = -1.0f;
			if((cur & 0x2u) != 0 && vn[i].x - aabb[2] * vn[i].w > 0.0f)
				aabb[2] = 1.0f;
		}
	}
	if((any_vis & 0xf0) == 0) {
		aabb[1] = -1.0f, aabb[3] = 1.0f;
	} else if((or_clipmask & 0xcu) != 0) {
		for(int i = 0; i < 3; i++) {
			uint32_t cur = clipmask >> (i * 8);
			if((cur & 0x4u) != 0 && vn[i].y - aabb[1] * vn[i].w < 0.0f)
				aabb[1] = -1.0f;
			if((cur & 0x8u) != 0 && vn[i].y - aabb[3] * vn[i].w > 0.0f)
				aabb[3] = 1.0f;
		}
	}
}

// quad_setup.glsl:136-254 (processInputQuad): cull tests, clipped AABB, bin AABB, class.
QuadResult processInputQuad(const State& s, const uint32_t v[4]) {
	QuadResult r;
	for(int i = 0; i < 4; i++)
		r.v[i] = v[i];
	const lucid_config& cfg = *s.in->config;
	bool cull0 = v[0] == v[1] || v[1] == v[2] || v[2] == v[0];
	bool cull1 = v[0] == v[2] || v[2] == v[3] || v[3] == v[0];
	if(cull0 && cull1) {
		r.reason = LUCID_REJECTION_TYPE_OTHER;
		return r;
	}
	uint32_t nv = uint32_t(s.in->num_verts);
	if(v[0] >= nv || v[1] >= nv || v[2] >= nv || v[3] >= nv) {
		r.reason = LUCID_REJECTION_TYPE_OTHER;
		r.bad_index = true;
		return r;
	}
	V3 vws[4] = {vertexLoad(s, v[0]), vertexLoad(s, v[1]), vertexLoad(s, v[2]),
				 vertexLoad(s, v[3])};
	cull0 = cull0 || eq(vws[0], vws[1]) || eq(vws[1], vws[2]) || eq(vws[2], vws[0]);
	cull1 = cull1 || eq(vws[0], vws[2]) || eq(vws[2], vws[3]) || eq(vws[3], vws[0]);

	if(cfg.enable_backface_culling != 0) {
		V3 o = s.origin;
		V3 p0 = sub(vws[0], o), p1 = sub(vws[1], o), p2 = sub(vws[2], o), p3 = sub(vws[3], o);
		V3 nrm0 = cross(p2, sub(p1, p2));
		V3 nrm1 = cross(p3, sub(p2, p3));
		float volume0 = dot(p0, nrm0);
		float volume1 = dot(p0, nrm1);
		cull0 = cull0 || volume0 <= 0.0f;
		cull1 = cull1 || volume1 <= 0.0f;
		if(cull0 && cull1) {
			r.reason = LUCID_REJECTION_TYPE_BACKFACE;
			return r;
		}
	}
	uint32_t cull_flags = (cull0 ? 1u : 0u) | (cull1 ? 2u : 0u);

	V4 vndc[4];
	for(int i = 0; i < 4; i++)
		vndc[i] = mulPoint(cfg.view_proj_matrix, vws[i]);
	uint32_t clipmask = vertexClipMask(vndc[0]) | (vertexClipMask(vndc[1]) << 8) |
						(vertexClipMask(vndc[2]) << 16) | (vertexClipMask(vndc[3]) << 24);
	uint32_t and_clipmask =
		clipmask & (clipmask >> 8) & (clipmask >> 16) & (clipmask >> 24) & 0xffu;
	uint32_t or_clipmask = clipmask | (clipmask >> 8) | (clipmask >> 16) | (clipmask >> 24);
	if(and_clipmask != 0) {
		r.reason = LUCID_REJECTION_TYPE_FRUSTUM;
		return r;
	}

	float aabb0[4], aabb1[4];
	float inv_w[4] = {1.0f / vndc[0].w, 1.0f / vndc[1].w, 1.0f / vndc[2].w, 1.0f / vndc[3].w};
	if((or_clipmask & 0x30u) != 0) {
		V4 t0[3] = {vndc[0], vndc[1], vndc[2]};
		float iw0[3] = {inv_w[0], inv_w[1], inv_w[2]};
		computeClippedAABB(t0, iw0, clipmask, aabb0);
		V4 t1[3] = {vndc[0], vndc[2], vndc[3]};
		float iw1[3] = {inv_w[0], inv_w[2], inv_w[3]};
		computeClippedAABB(t1, iw1, (clipmask & 0xffu) | ((clipmask & 0xffff0000u) >> 8), aabb1);
	}
	for(int i = 0; i < 4; i++) {
		vndc[i].x *= inv_w[i];
		vndc[i].y *= inv_w[i];
		vndc[i].z *= inv_w[i];
	}
	if((or_clipmask & 0x30u) == 0) {
		// computeAABB (quad_setup.glsl:131-134); min/max ignore NaN on both CPU and GPU
		aabb0[0] = fminf(fminf(vndc[0].x, vndc[1].x), vndc[2].x);
		aabb0[1] = fminf(fminf(vndc[0].y, vndc[1].y), vndc[2].y);
		aabb0[2] = fmaxf(fmaxf(vndc[0].x, vndc[1].x), vndc[2].x);
		aabb0[3] = fmaxf(fmaxf(vndc[0].y, vndc[1].y), vndc[2].y);
		aabb1[0] = fminf(fminf(vndc[0].x, vndc[2].x), vndc[3].x);
		aabb1[1] = fminf(fminf(vndc[0].y, vndc[2].y), vndc[3].y);
		aabb1[2] = fmaxf(fmaxf(vndc[0].x, vndc[2].x), vndc[3].x);
		aabb1[3] = fmaxf(fmaxf(vndc[0].y, vndc[2].y), vndc[3].y);
	}

	const float hx = float(s.w) * 0.5f, hy = float(s.h) * 0.5f;
	const float mx = float(s.w - 1), my = float(s.h - 1);
	float scale[4] = {hx, hy, hx, hy};
	for(int i = 0; i < 4; i++) {
		aabb0[i] = (aabb0[i] + 1.0f) * scale[i];
		aabb1[i] = (aabb1[i] + 1.0f) * scale[i];
	}
	float aabb[4] = {fminf(aabb0[0], aabb1[0]), fminf(aabb0[1], aabb1[1]),
					 fmaxf(aabb0[2], aabb1[2]), fmaxf(aabb0[3], aabb1[3])};

	// quad_setup.glsl:227-231 (quads falling between samples)
	if(ceilf(aabb[0] - 0.5001f) == floorf(aabb[2] + 0.5001f) ||
	   ceilf(aabb[1] - 0.5001f) == floorf(aabb[3] + 0.5001f)) {
		r.reason = LUCID_REJECTION_TYPE_BETWEEN_SAMPLES;
		return r;
	}

	const float adj[4] = {0.49f, 0.49f, -0.49f, -0.49f};
	const float hi[4] = {mx, my, mx, my};
	for(int i = 0; i < 4; i++) {
		aabb0[i] = fminf(fmaxf(aabb0[i] + adj[i], 0.0f), hi[i]);
		aabb1[i] = fminf(fmaxf(aabb1[i] + adj[i], 0.0f), hi[i]);
		aabb[i] = fminf(fmaxf(aabb[i] + adj[i], 0.0f), hi[i]);
	}
	uint32_t b[4];
	for(int i = 0; i < 4; i++)
		b[i] = f2u(aabb[i]) >> kBinShift;
	r.enc_aabb = encodeAABB28(b[0], b[1], b[2], b[3]) | (cull_flags << 30);
	uint32_t bw = b[2] - b[0] + 1, bh = b[3] - b[1] + 1;
	r.cls = bw * bh <= 4 ? 0 : 1;
	r.y_aabb[0] = f2u(aabb0[1]) | (f2u(aabb0[3]) << 16);
	r.y_aabb[1] = f2u(aabb1[1]) | (f2u(aabb1[3]) << 16);
	return r;
}

// quad_setup.glsl:274-340 (storeTri)
void storeTri(State& s, uint32_t tri_idx, uint32_t inst_flags_id, V3 tri0, V3 tri1, V3 tri2,
			  uint32_t y_aabb) {
	V3 normal = cross(sub(tri0, tri2), sub(tri1, tri0));
	float multiplier = 1.0f / sqrtf(dot(normal, normal));
	normal = mul(normal, multiplier);
	if((inst_flags_id & LUCID_INST_HAS_VERTEX_NORMALS) == 0)
		s.tri_normals[tri_idx] = encodeNormalUint(normal);

	V3 edge0 = mul(sub(tri0, tri2), multiplier);
	V3 edge1 = mul(sub(tri1, tri0), multiplier);
	float plane_dist = dot(normal, tri0);
	V3 nrm_tri0 = cross(tri0, normal);
	float param0 = dot(edge0, nrm_tri0);
	float param1 = dot(edge1, nrm_tri0);
	edge0 = cross(normal, edge0);
	edge1 = cross(normal, edge1);
	V3 e0 = v3(dot(edge0, s.dirx), dot(edge0, s.diry), dot(edge0, s.ray_dir0));
	V3 e1 = v3(dot(edge1, s.dirx), dot(edge1, s.diry), dot(edge1, s.ray_dir0));
	V3 pnormal = mul(normal, 1.0f / plane_dist);
	V3 deq = v3(dot(pnormal, s.dirx), dot(pnormal, s.diry), dot(pnormal, s.ray_dir0));

	uint32_t* d = &s.tri_depth[size_t(tri_idx) * 4];
	d[0] = fbits(deq.x), d[1] = fbits(deq.y), d[2] = fbits(deq.z), d[3] = inst_flags_id;
	uint32_t* bary = &s.tri_bary[size_t(tri_idx) * 8];
	bary[0] = fbits(e0.x), bary[1] = fbits(e0.y), bary[2] = fbits(e0.z), bary[3] = fbits(param0);
	bary[4] = fbits(e1.x), bary[5] = fbits(e1.y), bary[6] = fbits(e1.z), bary[7] = fbits(param1);

	V3 nrm0 = cross(tri2, sub(tri1, tri2));
	V3 nrm1 = cross(tri0, sub(tri2, tri0));
	V3 nrm2 = cross(tri1, sub(tri0, tri1));
	float volume = dot(tri0, nrm0);
	if(volume < 0.0f) {
		nrm0 = v3(-nrm0.x, -nrm0.y, -nrm0.z);
		nrm1 = v3(-nrm1.x, -nrm1.y, -nrm1.z);
		nrm2 = v3(-nrm2.x, -nrm2.y, -nrm2.z);
	}
	V3 edges[3] = {v3(dot(nrm0, s.dirx), dot(nrm0, s.diry), dot(nrm0, s.dir0)),
				   v3(dot(nrm1, s.dirx), dot(nrm1, s.diry), dot(nrm1, s.dir0)),
				   v3(dot(nrm2, s.dirx), dot(nrm2, s.diry), dot(nrm2, s.dir0))};
	float scan[3], step[3];
	uint32_t signs = 0;
	for(int i = 0; i < 3; i++) {
		float inv_ex = 1.0f / edges[i].x;
		float base = -(edges[i].z * inv_ex);
		step[i] = -(edges[i].y * inv_ex);
		// scan = scan_step * 0.5 + scan_base - (-0.5)
		scan[i] = (step[i] * 0.5f + base) - (-0.5f);
		signs |= (edges[i].x < 0.0f ? (1u << i) : 0u) | (edges[i].y < 0.0f ? (8u << i) : 0u);
	}
	uint32_t* sc = &s.tri_scan[size_t(tri_idx) * 8];
	sc[0] = fbits(scan[0]), sc[1] = fbits(scan[1]), sc[2] = fbits(scan[2]), sc[3] = y_aabb;
	sc[4] = fbits(step[0]), sc[5] = fbits(step[1]), sc[6] = fbits(step[2]), sc[7] = signs;
}

// quad_setup.glsl:374-489 with deterministic slot assignment in input order.
void quadSetup(State& s, oracle_outputs* out) {
	const oracle_inputs* in = s.in;
	int mvq = s.mvq;
	s.quad_aabbs.assign(mvq, 0);
	s.quad_source.assign(mvq, 0);
	s.quad_colors.assign(size_t(mvq) * 4, 0);
	s.quad_verts.assign(size_t(mvq) * 4, 0);
	s.quad_normals.assign(size_t(mvq) * 4, 0);
	s.quad_tex.assign(size_t(mvq) * 8, 0);
	s.quad_inst.assign(mvq, 0);
	s.tri_bary.assign(size_t(mvq) * 16, 0);
	s.tri_scan.assign(size_t(mvq) * 16, 0);
	s.tri_depth.assign(size_t(mvq) * 8, 0);
	s.tri_normals.assign(size_t(mvq) * 2, 0);
	int num_small = 0, num_large = 0;
	uint32_t rejected[4] = {0, 0, 0, 0};
	uint32_t input_quad = 0;
	for(int inst = 0; inst < in->num_instances; inst++) {
		const lucid_instance& id = in->instances[inst];
		if(id.num_quads > LUCID_MAX_INSTANCE_QUADS && out->error_code == 0)
			out->error_code = LUCID_ERR_INSTANCE_QUADS;
		for(int lq = 0; lq < id.num_quads; lq++, input_quad++) {
			size_t io = size_t(id.index_offset) + size_t(lq) * 4;
			uint32_t v[4];
			for(int k = 0; k < 4; k++)
				v[k] = in->quads_ib[io + k] + uint32_t(id.vertex_offset);
			QuadResult r = processInputQuad(s, v);
			if(r.cls < 0) {
				rejected[r.reason]++;
				if(r.bad_index && out->error_code == 0)
					out->error_code = LUCID_ERR_VERTEX_INDEX;
				continue;
			}
			if(num_small + num_large >= mvq) {
				if(out->error_code == 0)
					out->error_code = LUCID_ERR_VISIBLE_QUADS;
				continue;
			}
			int slot = r.cls == 0 ? num_small++ : (mvq - 1) - num_large++;
			s.quad_aabbs[slot] = r.enc_aabb;
			s.quad_source[slot] = input_quad;
			s.quad_inst[slot] = uint32_t(inst);
			for(int k = 0; k < 4; k++)
				s.quad_verts[size_t(slot) * 4 + k] = v[k];
			uint32_t flags = id.flags;
			// storeQuad (quad_setup.glsl:256-272): RGBA8 vertex colours, vertex normals, texture
			// coordinates relative to the first vertex
			if((flags & LUCID_INST_HAS_VERTEX_COLORS) && in->color_format == LUCID_COLOR_RGBA8) {
				const uint32_t* cols = (const uint32_t*)in->colors;
				for(int k = 0; k < 4; k++)
					s.quad_colors[size_t(slot) * 4 + k] = cols[v[k]];
			}
			if((flags & LUCID_INST_HAS_VERTEX_NORMALS) && in->normals)
				for(int k = 0; k < 4; k++)
					s.quad_normals[size_t(slot) * 4 + k] = in->normals[v[k]];
			if((flags & LUCID_INST_HAS_ALBEDO_TEXTURE) && in->tex_coords) {
				const float* tc = in->tex_coords;
				const float t0x = tc[size_t(v[0]) * 2], t0y = tc[size_t(v[0]) * 2 + 1];
				uint32_t* q = &s.quad_tex[size_t(slot) * 8];
				q[0] = fbits(t0x), q[1] = fbits(t0y);
				for(int k = 1; k < 4; k++) {
					q[2 * k] = fbits(tc[size_t(v[k]) * 2] - t0x);
					q[2 * k + 1] = fbits(tc[size_t(v[k]) * 2 + 1] - t0y);
				}
			}
			uint32_t inst_flags_id = (flags & 0xffffu) | (uint32_t(inst) << 16);
			for(int second = 0; second < 2; second++) {
				// addVisibleTri (quad_setup.glsl:356-372)
				if((r.enc_aabb >> (30 + second)) & 1u)
					continue;
				V3 t0 = sub(vertexLoad(s, v[0]), s.origin);
				V3 t1 = sub(vertexLoad(s, v[1 + second]), s.origin);
				V3 t2 = sub(vertexLoad(s, v[2 + second]), s.origin);
				storeTri(s, uint32_t(slot) * 2 + second, inst_flags_id, t0, t1, t2,
						 r.y_aabb[second]);
			}
		}
	}
	s.nvis[0] = num_small, s.nvis[1] = num_large;
	out->num_input_quads = int32_t(input_quad);
	out->num_visible[0] = num_small, out->num_visible[1] = num_large;
	for(int i = 0; i < 4; i++)
		out->rejected[i] = rejected[i];
	// quad_setup.glsl:471-485 (binning dispatch size)
	int small_batch = 1024 * 4, large_batch = 1024 / 2;
	int tasks = (num_small + small_batch - 1) / small_batch + (num_large + large_batch - 1) / large_batch;
	out->num_binning_dispatches = uint32_t(std::min(std::max(tasks, 4), kMaxDispatches));
}

// ---------------------------------------------------------------------------------------------
// Binning: bin_counter.glsl, bin_categorizer.glsl, bin_dispatcher.glsl

struct BinScan {
	float mn[3], mx[3], step[3];
};

// scanline.glsl:28-52 (loadScanlineParamsBin)
BinScan loadScanlineParamsBin(const uint32_t* sc, int& min_by, int& max_by) {
	BinScan p;
	float scan[3] = {bitsf(sc[0]), bitsf(sc[1]), bitsf(sc[2])};
	for(int i = 0; i < 3; i++)
		p.step[i] = bitsf(sc[4 + i]);
	min_by = int(sc[3] & 0xffffu) >> kBinShift;
	max_by = int(sc[3] >> 16) >> kBinShift;
	uint32_t sg = sc[7];
	const float offset = float(kBinSize) - 0.989f;
	const float start_x = 0.99f, start_y = float(min_by * kBinSize) - 0.01f;
	const float inf = INFINITY;
	for(int i = 0; i < 3; i++) {
		bool xneg = (sg >> i) & 1u, yneg = (sg >> (3 + i)) & 1u;
		float yoff = yneg ? 0.0f : offset, xoff = xneg ? 0.0f : offset;
		// scan += step * (yoffset + start.y) - (xoffset + start.x)
		scan[i] = scan[i] + (p.step[i] * (yoff + start_y) - (xoff + start_x));
		p.mn[i] = xneg ? -inf : scan[i];
		p.mx[i] = xneg ? scan[i] : inf;
		p.step[i] = p.step[i] * float(kBinSize);
	}
	return p;
}

// bin_counter.glsl:53-62 (scanlineStep)
void scanlineStep(BinScan& p, int& bmin, int& bmax) {
	float xmin = fmaxf(fmaxf(p.mn[0], p.mn[1]), p.mn[2]);
	float xmax = fminf(fminf(p.mx[0], p.mx[1]), p.mx[2]);
	for(int i = 0; i < 3; i++)
		p.mn[i] += p.step[i], p.mx[i] += p.step[i];
	bmin = f2i(xmin + 1.0f) >> kBinShift;
	bmax = f2i(xmax) >> kBinShift;
}

void binning(State& s, oracle_outputs* out) {
	int bins = s.bins;
	s.bin_quads.assign(bins, {});
	s.bin_tris.assign(bins, {});
	// Small quads (bin_counter.glsl:64-80, bin_dispatcher.glsl:66-80): every bin of the AABB
	for(int k = 0; k < s.nvis[0]; k++) {
		uint32_t enc = s.quad_aabbs[k];
		int x0, y0, x1, y1;
		decodeAABB28(enc, x0, y0, x1, y1);
		uint32_t entry = uint32_t(k) | (enc & 0xf0000000u);
		for(int by = y0; by <= y1; by++)
			for(int bx = x0; bx <= x1; bx++)
				s.bin_quads[by * s.bcx + bx].push_back(entry);
	}
	// Large tris (bin_counter.glsl:112-134, bin_dispatcher.glsl:89-114): bin rows by scanline
	for(int k = 0; k < s.nvis[1]; k++) {
		int quad_idx = (s.mvq - 1) - k;
		uint32_t enc = s.quad_aabbs[quad_idx];
		for(int second = 0; second < 2; second++) {
			if((enc >> (30 + second)) & 1u)
				continue;
			uint32_t tri_idx = uint32_t(quad_idx) * 2 + second;
			int x0, y0, x1, y1;
			decodeAABB28(enc, x0, y0, x1, y1);
			int bsy, bey;
			BinScan p = loadScanlineParamsBin(&s.tri_scan[size_t(tri_idx) * 8], bsy, bey);
			for(int by = bsy; by <= bey; by++) {
				int bmin, bmax;
				scanlineStep(p, bmin, bmax);
				bmin = std::max(bmin, x0), bmax = std::min(bmax, x1);
				for(int bx = bmin; bx <= bmax; bx++)
					s.bin_tris[by * s.bcx + bx].push_back(tri_idx);
			}
		}
	}
	// bin_categorizer.glsl:22-89: offsets (exclusive scan) and levels (LOW < threshold)
	std::vector<uint32_t> cnt(size_t(bins) * 10, 0);
	uint32_t qoff = 0, toff = 0;
	int level_counts[5] = {0, 0, 0, 0, 0};
	std::vector<uint32_t> low, high;
	for(int b = 0; b < bins; b++) {
		auto& q = s.bin_quads[b];
		auto& t = s.bin_tris[b];
		auto by_slot = [](uint32_t a, uint32_t b) { return (a & 0x0fffffffu) < (b & 0x0fffffffu); };
		std::sort(q.begin(), q.end(), by_slot);
		std::sort(t.begin(), t.end());
		uint32_t nq = uint32_t(q.size()), nt = uint32_t(t.size());
		cnt[bins * 0 + b] = nq;
		cnt[bins * 1 + b] = qoff;
		cnt[bins * 2 + b] = qoff + nq;
		cnt[bins * 3 + b] = nt;
		cnt[bins * 4 + b] = toff;
		cnt[bins * 5 + b] = toff + nt;
		qoff += nq, toff += nt;
		int64_t num_tris = int64_t(nt) + int64_t(nq) * 2;
		if(num_tris == 0)
			level_counts[LUCID_BIN_LEVEL_EMPTY]++;
		else if(num_tris < s.in->low_high_threshold)
			low.push_back(uint32_t(b)), level_counts[LUCID_BIN_LEVEL_LOW]++;
		else
			high.push_back(uint32_t(b)), level_counts[LUCID_BIN_LEVEL_HIGH]++;
	}
	for(size_t i = 0; i < low.size(); i++)
		cnt[size_t(bins) * 7 + i] = low[i];
	for(size_t i = 0; i < high.size(); i++)
		cnt[size_t(bins) * 9 + i] = high[i];
	for(int i = 0; i < 5; i++)
		out->bin_level_counts[i] = level_counts[i];
	out->num_bin_quads = qoff;
	out->num_bin_tris = toff;
	out->bin_count = bins, out->bin_count_x = s.bcx, out->bin_count_y = s.bcy;
	if(out->bin_counters)
		memcpy(out->bin_counters, cnt.data(), cnt.size() * 4);
	if(out->bin_quads && int64_t(qoff) <= out->bin_refs_capacity) {
		size_t o = 0;
		for(int b = 0; b < bins; b++)
			for(uint32_t e : s.bin_quads[b])
				out->bin_quads[o++] = e;
	}
	if(out->bin_tris && int64_t(toff) <= out->bin_refs_capacity) {
		size_t o = 0;
		for(int b = 0; b < bins; b++)
			for(uint32_t e : s.bin_tris[b])
				out->bin_tris[o++] = e;
	}
}

// ---------------------------------------------------------------------------------------------
// Raster (exact per-pixel order). Coverage follows raster_low.glsl:39-64 (generateRowTris):
// the scan starts at the tri's first 8-row block row inside the bin and steps one row at a
// time (rasterBinStep, raster.glsl:116-140). Depth and colour follow shading.glsl:107-165.

struct RowSpan {
	int lo, hi; // inclusive local x range, lo > hi means empty
};

// Per-row spans of one tri inside one bin; rows outside [row0, row1] are empty.
void triBinRows(const uint32_t* sc, int bin_x, int bin_y, RowSpan rows[32]) {
	for(int r = 0; r < 32; r++)
		rows[r] = RowSpan{31, 0};
	int ymin = int(sc[3] & 0xffffu) - bin_y, ymax = int(sc[3] >> 16) - bin_y;
	int min_by = std::min(std::max(ymin, 0), 31) >> 3;
	int max_by = std::min(std::max(ymax, 0), 31) >> 3;
	float sx = float(bin_x), sy = float(bin_y + min_by * 8);
	float mn[3], mx[3], step[3];
	uint32_t sg = sc[7];
	const float inf = INFINITY;
	for(int i = 0; i < 3; i++) {
		step[i] = bitsf(sc[4 + i]);
		// loadScanlineParamsRow (scanline.glsl:13-26): scan += step * start.y - start.x
		float scan = bitsf(sc[i]) + (step[i] * sy - sx);
		bool xneg = (sg >> i) & 1u;
		mn[i] = xneg ? -inf : scan;
		mx[i] = xneg ? scan : inf;
	}
	for(int row = min_by * 8; row < max_by * 8 + 8; row++) {
		float fl = fmaxf(fmaxf(mn[0], mn[1]), fmaxf(mn[2], 0.0f));
		float fh = fminf(fminf(mx[0], mx[1]), fminf(mx[2], float(kBinSize)));
		// Non-finite or out-of-range spans clamp to empty instead of wrapping.
		int lo = f2i(fminf(fl, 33.0f));
		int hi = f2i(fmaxf(fh, -1.0f)) - 1;
		if(lo > hi)
			lo = 31, hi = 0;
		for(int i = 0; i < 3; i++)
			mn[i] += step[i], mx[i] += step[i];
		rows[row] = RowSpan{lo, hi};
	}
}

struct Frag {
	uint32_t key;   // nearFirstKey(inv_ray_pos)
	uint32_t prim;  // input primitive id: input quad * 2 + second
	uint32_t tri;   // tri slot
	float depth;    // inv_ray_pos
};

// log2(x) for finite x > 0: exponent plus the series 2 atanh(t) = ln(m), t = (m - 1) / (m + 1),
// on the mantissa m in [sqrt(1/2), sqrt(2)) up to t^13; each operation rounds separately, as in
// the CUDA path. 0 gives -inf, +inf gives +inf, negative or NaN input NaN.
float seriesLog2(float x) {
	if(x != x || x < 0.0f)
		return NAN;
	if(x == 0.0f)
		return -INFINITY;
	if(x == INFINITY)
		return x;
	int e = 0;
	uint32_t b = fbits(x);
	if(((b >> 23) & 0xffu) == 0u) {
		x = x * 8388608.0f;
		b = fbits(x);
		e = -23;
	}
	e += int((b >> 23) & 0xffu) - 127;
	float m = bitsf((b & 0x7fffffu) | 0x3f800000u);
	if(m > 0x1.6a09e6p+0f) {
		m = m * 0.5f;
		e = e + 1;
	}
	const float t = (m - 1.0f) / (m + 1.0f);
	const float t2 = t * t;
	float sr = 0x1.3b13b2p-4f;      // 1/13
	sr = sr * t2 + 0x1.745d18p-4f; // 1/11
	sr = sr * t2 + 0x1.c71c72p-4f; // 1/9
	sr = sr * t2 + 0x1.24924ap-3f; // 1/7
	sr = sr * t2 + 0x1.99999ap-3f; // 1/5
	sr = sr * t2 + 0x1.555556p-2f; // 1/3
	sr = sr * t2 + 1.0f;
	const float ln_m = (2.0f * t) * sr;
	return float(e) + ln_m * 0x1.715476p+0f; // 1/ln 2
}

// Bilinear sample of one mip level (repeat addressing, texel centres at half integers).
void texSampleLevel(const lucid_texture& t, int level, float u, float v, float out[4]) {
	size_t off = 0;
	for(int l = 0; l < level; l++)
		off += size_t(std::max(1, t.width >> l)) * size_t(std::max(1, t.height >> l));
	const int w = std::max(1, t.width >> level), h = std::max(1, t.height >> level);
	u = u - floorf(u);
	v = v - floorf(v);
	if(u != u)
		u = 0.0f;
	if(v != v)
		v = 0.0f;
	const float fu = u * float(w) - 0.5f, fv = v * float(h) - 0.5f;
	const float xf = floorf(fu), yf = floorf(fv);
	const float a = fu - xf, b = fv - yf;
	const int x0 = int(xf), y0 = int(yf);
	auto texel = [&](int x, int y, float c[4]) {
		x = x < 0 ? x + w : (x >= w ? x - w : x);
		y = y < 0 ? y + h : (y >= h ? y - h : y);
		decodeRGBA8(t.texels[off + size_t(y) * w + x], c);
	};
	float c00[4], c10[4], c01[4], c11[4];
	texel(x0, y0, c00), texel(x0 + 1, y0, c10), texel(x0, y0 + 1, c01), texel(x0 + 1, y0 + 1, c11);
	const float wa = (1.0f - a) * (1.0f - b), wb = a * (1.0f - b), wc = (1.0f - a) * b, wd = a * b;
	for(int k = 0; k < 4; k++)
		out[k] = ((c00[k] * wa + c10[k] * wb) + c01[k] * wc) + c11[k] * wd;
}

// textureGrad, trilinear and repeat-addressed (the reference's sampler adds 16x anisotropy,
// src/lucid_base.h:30, the hardware's own footprint, not modelled)
void texSampleGrad(const lucid_texture* t, float u, float v, float dxu, float dxv, float dyu, float dyv,
				   float out[4]) {
	if(!t || !t->texels) {
		out[0] = out[1] = out[2] = out[3] = 1.0f;
		return;
	}
	const float W = float(t->width), H = float(t->height);
	const float ax = dxu * W, ay = dxv * H, bx = dyu * W, by = dyv * H;
	const float rho = fmaxf(sqrtf(ax * ax + ay * ay), sqrtf(bx * bx + by * by));
	float lambda = seriesLog2(rho);
	if(!(lambda > 0.0f))
		lambda = 0.0f;
	lambda = fminf(lambda, float(t->num_levels - 1));
	const float lf = floorf(lambda);
	const int l0 = int(lf);
	const float f = lambda - lf;
	texSampleLevel(*t, l0, u, v, out);
	if(f > 0.0f) {
		float c1[4];
		texSampleLevel(*t, l0 + 1, u, v, c1);
		const float g = 1.0f - f;
		for(int k = 0; k < 4; k++)
			out[k] = out[k] * g + c1[k] * f;
	}
}

// Everything shadeSample (shading.glsl:107-165) computes before lighting, in its float order.
struct ShadeCoreO {
	float col[4];    // colour with vertex colours and opacity
	float factor[4]; // instance colour x texture colour
	float b0, b1;
	uint32_t flags, inst;
};

ShadeCoreO shadeCore(const State& s, const Frag& f, int px, int py) {
	const oracle_inputs* in = s.in;
	ShadeCoreO o;
	const uint32_t* d = &s.tri_depth[size_t(f.tri) * 4];
	const uint32_t* b = &s.tri_bary[size_t(f.tri) * 8];
	const float fx = float(px), fy = float(py);
	const float ray_pos = 1.0f / f.depth;
	const float e0 = bitsf(b[0]) * fx + (bitsf(b[1]) * fy + bitsf(b[2]));
	const float e1 = bitsf(b[4]) * fx + (bitsf(b[5]) * fy + bitsf(b[6]));
	const float braw0 = e0 * ray_pos, braw1 = e1 * ray_pos;
	const float b0 = braw0 - bitsf(b[3]);
	const float b1 = braw1 - bitsf(b[7]);
	o.b0 = b0, o.b1 = b1;
	o.flags = d[3] & 0xffffu, o.inst = d[3] >> 16;
	const uint32_t quad = f.tri >> 1, second = f.tri & 1;
	float* col = o.col;
	col[0] = col[1] = col[2] = col[3] = 1.0f;
	if((o.flags & LUCID_INST_HAS_COLOR) && in->instance_colors)
		decodeRGBA8(in->instance_colors[o.inst], col);
	if(o.flags & LUCID_INST_HAS_ALBEDO_TEXTURE) {
		// shading.glsl:125-159: bary derivatives, texture coordinates, optional uv rect
		const float ray_posx = 1.0f / (f.depth + bitsf(d[0]));
		const float ray_posy = 1.0f / (f.depth + bitsf(d[1]));
		const float bdx0 = (e0 + bitsf(b[0])) * ray_posx - braw0, bdx1 = (e1 + bitsf(b[4])) * ray_posx - braw1;
		const float bdy0 = (e0 + bitsf(b[1])) * ray_posy - braw0, bdy1 = (e1 + bitsf(b[5])) * ray_posy - braw1;
		const uint32_t* q = &s.quad_tex[size_t(quad) * 8];
		const float t0x = bitsf(q[0]), t0y = bitsf(q[1]);
		const float t1x = bitsf(second ? q[4] : q[2]), t1y = bitsf(second ? q[5] : q[3]);
		const float t2x = bitsf(second ? q[6] : q[4]), t2y = bitsf(second ? q[7] : q[5]);
		float u = b0 * t1x + (b1 * t2x + t0x), v = b0 * t1y + (b1 * t2y + t0y);
		float dxu = bdx0 * t1x + bdx1 * t2x, dxv = bdx0 * t1y + bdx1 * t2y;
		float dyu = bdy0 * t1x + bdy1 * t2x, dyv = bdy0 * t1y + bdy1 * t2y;
		if((o.flags & LUCID_INST_HAS_UV_RECT) && in->instance_uv_rects) {
			const float* r = in->instance_uv_rects + size_t(o.inst) * 4;
			u = r[2] * (u - floorf(u)) + r[0];
			v = r[3] * (v - floorf(v)) + r[1];
			dxu = dxu * r[2], dxv = dxv * r[3], dyu = dyu * r[2], dyv = dyv * r[3];
		}
		float tc[4];
		if(o.flags & LUCID_INST_TEX_OPAQUE) {
			texSampleGrad(in->opaque_texture, u, v, dxu, dxv, dyu, dyv, tc);
			tc[3] = 1.0f;
		} else {
			texSampleGrad(in->transparent_texture, u, v, dxu, dxv, dyu, dyv, tc);
		}
		for(int k = 0; k < 4; k++)
			col[k] = col[k] * tc[k];
	}
	for(int k = 0; k < 4; k++)
		o.factor[k] = col[k];
	if(o.flags & LUCID_INST_HAS_VERTEX_COLORS) {
		float c[3][4];
		uint32_t vid[3] = {s.quad_verts[size_t(quad) * 4 + 0], s.quad_verts[size_t(quad) * 4 + 1 + second],
						   s.quad_verts[size_t(quad) * 4 + 2 + second]};
		for(int k = 0; k < 3; k++) {
			if(in->color_format == LUCID_COLOR_RGBA8) {
				decodeRGBA8(((const uint32_t*)in->colors)[vid[k]], c[k]);
			} else if(in->color_format == LUCID_COLOR_RGBA16F) {
				const uint16_t* hh = (const uint16_t*)in->colors + size_t(vid[k]) * 4;
				for(int j = 0; j < 4; j++)
					c[k][j] = halfToFloat(hh[j]);
			} else {
				const float* fc = (const float*)in->colors + size_t(vid[k]) * 4;
				for(int j = 0; j < 4; j++)
					c[k][j] = fc[j];
			}
		}
		const float wgt = (1.0f - b0) - b1;
		for(int j = 0; j < 4; j++)
			col[j] = col[j] * (wgt * c[0][j] + (b0 * c[1][j] + b1 * c[2][j]));
	}
	if(in->tri_opacity)
		col[3] = col[3] * in->tri_opacity[f.prim];
	return o;
}

void shadeFragment(const State& s, const Frag& f, int px, int py, float col[4]) {
	const ShadeCoreO o = shadeCore(s, f, px, py);
	for(int k = 0; k < 4; k++)
		col[k] = o.col[k];
}

// Fragments of every pixel of one bin (row-major 32x32 lists, unsorted); returns the count of
// (tri, half-block) pairs with a covered pixel.
uint64_t binFragments(const State& s, int bin, std::vector<std::vector<Frag>>& px) {
	uint64_t nhbt = 0;
	int bx = bin % s.bcx, by = bin / s.bcx;
	int bin_x = bx * kBinSize, bin_y = by * kBinSize;
	for(auto& v : px)
		v.clear();
	std::vector<uint32_t> tris;
	for(uint32_t e : s.bin_quads[bin]) {
		uint32_t quad = e & 0x0fffffffu;
		for(int second = 0; second < 2; second++)
			if(!((e >> (30 + second)) & 1u))
				tris.push_back(quad * 2 + second);
	}
	for(uint32_t t : s.bin_tris[bin])
		tris.push_back(t);
	RowSpan rows[32];
	for(uint32_t t : tris) {
		const uint32_t* sc = &s.tri_scan[size_t(t) * 8];
		triBinRows(sc, bin_x, bin_y, rows);
		const uint32_t* d = &s.tri_depth[size_t(t) * 4];
		float dx = bitsf(d[0]), dy = bitsf(d[1]), dz = bitsf(d[2]);
		uint32_t prim = s.quad_source[t >> 1] * 2 + (t & 1);
		for(int band = 0; band < 8; band++) {
			uint32_t colmask = 0;
			for(int r = band * 4; r < band * 4 + 4; r++) {
				RowSpan sp = rows[r];
				if(sp.lo > sp.hi)
					continue;
				colmask |= ((0xfu << (sp.lo >> 3)) & (0xfu >> (3 - (sp.hi >> 3))));
				int py = bin_y + r;
				if(py >= s.h)
					continue;
				for(int x = sp.lo; x <= sp.hi; x++) {
					int pxx = bin_x + x;
					if(pxx >= s.w)
						continue;
					// shading.glsl:116
					float inv_ray_pos = dx * float(pxx) + (dy * float(py) + dz);
					px[r * 32 + x].push_back(Frag{nearFirstKey(inv_ray_pos), prim, t, inv_ray_pos});
				}
			}
			nhbt += __builtin_popcount(colmask);
		}
	}
	return nhbt;
}

// Exact per-pixel order: nearest first (larger inv_ray_pos), ties by input primitive id.
inline bool fragLess(const Frag& a, const Frag& b) {
	return a.key != b.key ? a.key < b.key : a.prim < b.prim;
}

void rasterBin(const State& s, int bin, int slot, oracle_outputs* out, std::vector<std::vector<Frag>>& px,
			   uint64_t& nfrag, uint64_t& nhbt, uint32_t& maxfrag) {
	const oracle_inputs* in = s.in;
	int bx = bin % s.bcx, by = bin / s.bcx;
	int bin_x = bx * kBinSize, bin_y = by * kBinSize;
	nhbt += binFragments(s, bin, px);
	const float* bg = in->config->background_color;
	bool additive = (in->flags & LUCID_OPT_ADDITIVE_BLENDING) != 0;
	bool alpha_threshold = (in->flags & LUCID_OPT_ALPHA_THRESHOLD) != 0;
	const bool img64_requested = out->image64 != nullptr;
	for(int r = 0; r < 32; r++) {
		int py = bin_y + r;
		if(py >= s.h)
			break;
		for(int x = 0; x < 32; x++) {
			int pxx = bin_x + x;
			if(pxx >= s.w)
				break;
			auto& fr = px[r * 32 + x];
			std::sort(fr.begin(), fr.end(), fragLess);
			nfrag += fr.size();
			maxfrag = std::max(maxfrag, uint32_t(fr.size()));
			size_t pix = size_t(py) * s.w + pxx;
			// dump index: the whole frame, or (dump_by_subset) the bin's slot in the subset
			const size_t dpix = out->dump_by_subset ? size_t(slot) * 1024 + size_t(r * 32 + x) : pix;
			if(out->frag_counts)
				out->frag_counts[dpix] = int32_t(fr.size());
			if(out->frag_prims) {
				int32_t* dst = out->frag_prims + dpix * out->max_per_pixel;
				for(int i = 0; i < out->max_per_pixel; i++)
					dst[i] = i < int(fr.size()) ? int32_t(fr[i].prim) : -1;
			}
			// shading.glsl:279-280,312 in FP32 (and, when image64 is requested, FP64 over the
			// same FP32 colours). Without image64 the FP32 loop stops once T == 0: every later
			// fragment would add (c * a) * 0 = 0 and keep T at 0.
			const bool want64 = img64_requested;
			float oc[3] = {0.0f, 0.0f, 0.0f}, T = 1.0f;
			double oc64[3] = {0.0, 0.0, 0.0}, T64 = 1.0;
			for(const Frag& f : fr) {
				if(!want64 && !additive && T == 0.0f)
					break;
				float c[4];
				shadeFragment(s, f, pxx, py, c);
				if(additive) {
					for(int j = 0; j < 3; j++)
						oc[j] = oc[j] + c[j] * c[3];
					if(want64)
						for(int j = 0; j < 3; j++)
							oc64[j] = oc64[j] + double(c[j]) * double(c[3]);
				} else {
					for(int j = 0; j < 3; j++)
						oc[j] = oc[j] + (c[j] * c[3]) * T;
					T = T * (1.0f - c[3]);
					if(want64) {
						for(int j = 0; j < 3; j++)
							oc64[j] = oc64[j] + (double(c[j]) * double(c[3])) * T64;
						T64 = T64 * (1.0 - double(c[3]));
					}
					if(alpha_threshold && T < (1.0f / 128.0f))
						break;
				}
			}
			float* img = out->image ? out->image + pix * 4 : nullptr;
			double* img64 = out->image64 ? out->image64 + pix * 4 : nullptr;
			for(int j = 0; j < 3; j++) {
				float v = oc[j] + T * bg[j];
				double v64 = oc64[j] + T64 * double(bg[j]);
				if(img)
					img[j] = fminf(fmaxf(v, 0.0f), 1.0f);
				if(img64)
					img64[j] = std::min(std::max(v64, 0.0), 1.0);
			}
			if(img)
				img[3] = 1.0f;
			if(img64)
				img64[3] = 1.0;
		}
	}
}

// ---------------------------------------------------------------------------------------------
// Reference-order mode (order_mode 1): the reference's own per-pixel order and blend.
//
// LOW bins (raster_low.glsl): per 8x8 block, the tris whose row spans (scan started at the tri's
// first 8-row block row, generateRowTris :39-64) touch the block get a 22-bit key at their
// coverage centroid in the block (generateBlocks :101-131; rasterHalfBlockCentroid and
// rasterBlockDepth, raster.glsl:142-176) and are sorted when the block holds more than
// RC_COLOR_SIZE tris (:144-150). A block of more than 256 tris promotes the bin to the HIGH path
// (:93-103, :211-219).
// HIGH bins (raster_high.glsl): per 8x4 half-block (scan started at the tri's first half-block
// row, :60-81), an 18-bit key at the centroid (:168-186), always sorted; more than 16384 tris in
// a half-block row, or more than 4096 in one half-block by the range estimate of
// computeRBlockGroups (:114-147), paint the bin red (1, 0, 0, 0) (:297-301).
// Equal keys, which the reference leaves in shared-memory arrival order (not deterministic),
// are ordered by input primitive id; blocks of <= 3 tris (unsorted in the reference) are in
// primitive-id order.
// A pixel's samples are its block's sorted tris that cover it, shaded with the scene lighting
// and encoded RGBA8 (shadeSample, shading.glsl:107-184), then reduced through the 3-deep depth
// window (reduceSample / finishReduceSamples, shading.glsl:229-314); the accumulated colour is
// saturated at the end of every 256-fragment segment of the half-block (shadeAndReduceSamples,
// raster.glsl:361-398). The alpha-threshold variant (a subgroup vote in the reference) is not
// part of this mode.

// x^y for finite x > 0 as exp2(y * log2(x)): log2 of the mantissa m in [sqrt(1/2), sqrt(2)) from
// the series 2 atanh(t) = ln(m), t = (m - 1) / (m + 1), up to t^13; 2^f, f in [0, 1), from the
// Taylor series of e^(f ln 2) up to degree 10. The CUDA path evaluates the same float
// operations in the same order (no FMA on either side), so both round identically.
float refPow(float x, float y) {
	if(x != x)
		return x;
	if(x <= 0.0f)
		return x == 0.0f ? 0.0f : NAN;
	if(x == INFINITY)
		return y > 0.0f ? INFINITY : 0.0f;
	const float l2 = seriesLog2(x);
	const float z = y * l2;
	if(z >= 128.0f)
		return INFINITY;
	if(z < -149.0f)
		return 0.0f;
	const float k = floorf(z);
	const float u = (z - k) * 0x1.62e43p-1f; // ln 2
	float pe = 0x1.27e4fcp-22f;    // 1/10!
	pe = pe * u + 0x1.71de3ap-19f; // 1/9!
	pe = pe * u + 0x1.a01a02p-16f; // 1/8!
	pe = pe * u + 0x1.a01a02p-13f; // 1/7!
	pe = pe * u + 0x1.6c16c2p-10f; // 1/6!
	pe = pe * u + 0x1.111112p-7f;  // 1/5!
	pe = pe * u + 0x1.555556p-5f;  // 1/4!
	pe = pe * u + 0x1.555556p-3f;  // 1/3!
	pe = pe * u + 0.5f;
	pe = pe * u + 1.0f;
	pe = pe * u + 1.0f;
	int ki = int(k);
	if(ki < -126) { // scale in two steps to stay within normal exponents
		pe = pe * bitsf(uint32_t(ki + 126 + 127) << 23);
		ki = -126;
	}
	return pe * bitsf(uint32_t(ki + 127) << 23);
}

// funcs.glsl:61-66
inline V3 decodeNormalUint(uint32_t n) {
	const float s = 0x1.00804p-9f; // 1/511
	return v3((float((n >> 0) & 0x3ffu) - 512.0f) * s, (float((n >> 10) & 0x3ffu) - 512.0f) * s,
			  (float((n >> 20) & 0x3ffu) - 512.0f) * s);
}

// funcs.glsl:118-121
inline uint32_t encodeRGBA8(const float c[4]) {
	return f2u(c[0] * 255.0f) | (f2u(c[1] * 255.0f) << 8) | (f2u(c[2] * 255.0f) << 16) |
		   (f2u(c[3] * 255.0f) << 24);
}

inline float saturate(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// shadeSample (shading.glsl:107-184): colour as the exact mode's shading, then the flat tri
// normal, sun light and finalShading (funcs.glsl:153-164, 261-271), RGBA8; 0 when alpha is 0.
uint32_t shadeRef(const State& s, uint32_t tri, uint32_t prim, int px, int py, float& depth) {
	const uint32_t* d = &s.tri_depth[size_t(tri) * 4];
	const float inv_ray_pos = bitsf(d[0]) * float(px) + (bitsf(d[1]) * float(py) + bitsf(d[2]));
	depth = inv_ray_pos;
	const ShadeCoreO sc = shadeCore(s, Frag{0u, prim, tri, inv_ray_pos}, px, py);
	float c[4] = {sc.col[0], sc.col[1], sc.col[2], sc.col[3]};
	if(c[3] == 0.0f)
		return 0u;
	const lucid_lighting& L = s.in->config->lighting;
	V3 n;
	if((sc.flags & LUCID_INST_HAS_VERTEX_NORMALS) && s.in->normals) {
		// shading.glsl:168-174: normals interpolated with the perspective-correct barycentrics
		const uint32_t* qn = &s.quad_normals[size_t(tri >> 1) * 4];
		const uint32_t second = tri & 1;
		const V3 n0 = decodeNormalUint(qn[0]);
		const V3 n1 = sub(decodeNormalUint(qn[1 + second]), n0);
		const V3 n2 = sub(decodeNormalUint(qn[2 + second]), n0);
		n = v3(sc.b0 * n1.x + (sc.b1 * n2.x + n0.x), sc.b0 * n1.y + (sc.b1 * n2.y + n0.y),
			   sc.b0 * n1.z + (sc.b1 * n2.z + n0.z));
	} else {
		n = decodeNormalUint(s.tri_normals[tri]);
	}
	const float dn = (-L.sun_dir[0]) * n.x + (-L.sun_dir[1]) * n.y + (-L.sun_dir[2]) * n.z;
	const float light = fmaxf(0.0f, dn * 0x1.666666p-1f + 0x1.333334p-2f); // * 0.7 + 0.3
	for(int ch = 0; ch < 3; ch++) {
		const float cv = c[ch];
		const float lin = cv < 0x1.4b5dccp-5f ? 0x1.3d0722p-4f * cv // 0.04045, 1/12.92
											  : refPow((cv + 0x1.c28f5cp-5f) * 0x1.e54edep-1f, 0x1.333334p+1f);
		const float amb = L.ambient_color[ch] * L.ambient_power;
		const float dif = (L.sun_color[ch] * L.sun_power) * light;
		const float v = lin * (amb + dif);
		const float sr = v < 0x1.9a5c38p-9f ? 0x1.9d70a4p+3f * v // 0.0031308, 12.92
											: 0x1.0e147ap+0f * refPow(v, 0x1.aaaaaap-2f) - 0x1.c28f5cp-5f;
		c[ch] = saturate(sr);
	}
	return encodeRGBA8(c);
}

// ReductionContext (shading.glsl:196-227); depth slots 4 with LUCID_OPT_VISUALIZE_ERRORS
struct RefReduce {
	float depth[4];
	uint32_t col[3];
	float trans;
	float out[3];
	int depth_size;
	bool additive, invalid;

	void init(int dsize, bool add) {
		for(float& v : depth)
			v = 999999999.0f;
		col[0] = col[1] = col[2] = 0u;
		trans = 1.0f;
		out[0] = out[1] = out[2] = 0.0f;
		depth_size = dsize;
		additive = add;
		invalid = false;
	}
	void swapSlots(int a, int b) {
		std::swap(depth[a], depth[b]);
		if(a < 3 && b < 3)
			std::swap(col[a], col[b]);
	}
	void blend(uint32_t c) {
		float cur[4];
		decodeRGBA8(c, cur);
		if(additive) {
			for(int ch = 0; ch < 3; ch++)
				out[ch] = out[ch] + cur[ch] * cur[3];
		} else {
			for(int ch = 0; ch < 3; ch++)
				out[ch] = out[ch] + (cur[ch] * cur[3]) * trans;
			trans = trans * (1.0f - cur[3]);
		}
	}
	// reduceSample (shading.glsl:229-294) for one sample
	void sample(uint32_t color, float dep) {
		if(dep > depth[0]) {
			std::swap(color, col[0]);
			std::swap(dep, depth[0]);
			if(depth[0] > depth[1]) {
				swapSlots(0, 1);
				if(depth[1] > depth[2]) {
					swapSlots(1, 2);
					int i = 3;
					for(; i < depth_size && depth[i - 1] > depth[i]; i++)
						swapSlots(i - 1, i);
					if(depth_size == 4 && i == depth_size) {
						invalid = true;
						out[0] = 1.0f, out[1] = 0.0f, out[2] = 0.0f;
						trans = 0.0f;
						return;
					}
				}
			}
		}
		for(int i = depth_size - 1; i > 0; i--)
			depth[i] = depth[i - 1];
		depth[0] = dep;
		if(col[2] != 0u)
			blend(col[2]);
		col[2] = col[1], col[1] = col[0], col[0] = color;
	}
	void endSegment() {
		for(float& v : out)
			v = saturate(v);
	}
	// finishReduceSamples (shading.glsl:296-314)
	void finish(const float* bg, float rgba[4]) {
		for(int i = 2; i >= 0; i--)
			if(col[i] != 0u)
				blend(col[i]);
		for(int ch = 0; ch < 3; ch++)
			rgba[ch] = saturate(out[ch] + trans * bg[ch]);
		rgba[3] = 1.0f;
	}
};

struct RefTri {
	uint32_t tri, prim;
	RowSpan rows[32];
};

struct RefEntry {
	uint32_t key, prim;
	int t; // index into the bin's RefTri list
};

// Per-row spans of one tri inside one bin with the scan started at the tri's first row group
// of `group` rows (8: raster_low generateRowTris, 4: raster_high generateRowTris).
void triBinRowsFrom(const uint32_t* sc, int bin_x, int bin_y, int group, RowSpan rows[32]) {
	for(int r = 0; r < 32; r++)
		rows[r] = RowSpan{31, 0};
	const int shift = group == 8 ? 3 : 2;
	int ymin = int(sc[3] & 0xffffu) - bin_y, ymax = int(sc[3] >> 16) - bin_y;
	int min_g = std::min(std::max(ymin, 0), 31) >> shift;
	int max_g = std::min(std::max(ymax, 0), 31) >> shift;
	float sx = float(bin_x), sy = float(bin_y + min_g * group);
	float mn[3], mx[3], step[3];
	uint32_t sg = sc[7];
	for(int i = 0; i < 3; i++) {
		step[i] = bitsf(sc[4 + i]);
		float scan = bitsf(sc[i]) + (step[i] * sy - sx);
		bool xneg = (sg >> i) & 1u;
		mn[i] = xneg ? -INFINITY : scan;
		mx[i] = xneg ? scan : INFINITY;
	}
	for(int row = min_g * group; row < max_g * group + group; row++) {
		float fl = fmaxf(fmaxf(mn[0], mn[1]), fmaxf(mn[2], 0.0f));
		float fh = fminf(fminf(mx[0], mx[1]), fminf(mx[2], float(kBinSize)));
		int lo = f2i(fminf(fl, 33.0f));
		int hi = f2i(fmaxf(fh, -1.0f)) - 1;
		if(lo > hi)
			lo = 31, hi = 0;
		for(int i = 0; i < 3; i++)
			mn[i] += step[i], mx[i] += step[i];
		rows[row] = RowSpan{lo, hi};
	}
}

// 4-bit mask of the 8-pixel columns touched by rows [r0, r0 + 4) (BX_MASK_ROW, raster.glsl:123-127)
inline uint32_t rowGroupColumns(const RowSpan* rows, int r0) {
	uint32_t m = 0;
	for(int r = r0; r < r0 + 4; r++)
		if(rows[r].lo <= rows[r].hi)
			m |= ((0xfu << (rows[r].lo >> 3)) & (0xfu >> (3 - (rows[r].hi >> 3))));
	return m;
}

// rasterHalfBlockCentroid (raster.glsl:142-150) over rows [r0, r0 + 4) from column startx
inline void halfBlockCentroid(const RowSpan* rows, int r0, int startx, float& cx, float& cy, int& nfrag) {
	const float wy[4] = {1.0f, 3.0f, 5.0f, 7.0f};
	float px[4], py[4];
	nfrag = 0;
	for(int k = 0; k < 4; k++) {
		int xmin = std::max(rows[r0 + k].lo - startx, 0);
		int xmax = std::min(rows[r0 + k].hi - startx, 7);
		int count = std::max(xmax - xmin + 1, 0);
		px[k] = float(xmin * 2 + count) * float(count);
		py[k] = wy[k] * float(count);
		nfrag += count;
	}
	cx = px[0] + px[1] + px[2] + px[3];
	cy = py[0] + py[1] + py[2] + py[3];
}

// rasterBlockDepth (raster.glsl:170-176); inversesqrt = 1 / sqrt
inline uint32_t refBlockKey(const State& s, uint32_t tri, float cx, float cy, int nfrag, float bx, float by,
							float range) {
	const uint32_t* d = &s.tri_depth[size_t(tri) * 4];
	const float scale = 0.5f / float(nfrag);
	const float px = cx * scale + bx, py = cy * scale + by;
	const float ray_pos = bitsf(d[0]) * px + (bitsf(d[1]) * py + bitsf(d[2]));
	const float isq = 1.0f / sqrtf(ray_pos + 1.0f);
	return f2u(range * saturate(isq));
}

inline bool refLess(const RefEntry& a, const RefEntry& b) {
	return a.key != b.key ? a.key < b.key : a.prim < b.prim;
}

// Reduces the samples of every pixel of one half-block (8 x 4 pixels at local (hx*8, hy*4))
// from a list of tris in blend order; segments of 256 fragments in list order, pixels of a tri
// in row-major order (unpackSamples, raster.glsl:299-357).
void refReduceHalfBlock(const State& s, int bin_x, int bin_y, int hx, int hy, const std::vector<RefTri>& tris,
						const std::vector<RefEntry>& list, oracle_outputs* out, uint64_t& nfrag, uint64_t& ninvalid) {
	const oracle_inputs* in = s.in;
	const bool additive = (in->flags & LUCID_OPT_ADDITIVE_BLENDING) != 0;
	const bool visualize = (in->flags & LUCID_OPT_VISUALIZE_ERRORS) != 0;
	RefReduce ctx[32];
	int last_seg[32], nsamp[32];
	for(int i = 0; i < 32; i++) {
		ctx[i].init(visualize ? 4 : 3, additive);
		last_seg[i] = -1;
		nsamp[i] = 0;
	}
	const int startx = hx * 8, r0 = hy * 4;
	uint32_t offset = 0;
	for(const RefEntry& e : list) {
		const RefTri& t = tris[size_t(e.t)];
		uint32_t rank = 0;
		for(int k = 0; k < 4; k++) {
			const RowSpan sp = t.rows[r0 + k];
			int xmin = std::max(sp.lo - startx, 0), xmax = std::min(sp.hi - startx, 7);
			for(int x = xmin; x <= xmax; x++, rank++) {
				const int pl = k * 8 + x;
				const int seg = int((offset + rank) >> 8);
				if(last_seg[pl] >= 0 && seg != last_seg[pl])
					ctx[pl].endSegment();
				last_seg[pl] = seg;
				const int pxx = bin_x + startx + x, py = bin_y + r0 + k;
				float dep;
				const uint32_t color = shadeRef(s, t.tri, t.prim, pxx, py, dep);
				ctx[pl].sample(color, dep);
				if(pxx < s.w && py < s.h && out->frag_prims) {
					const size_t pix = size_t(py) * s.w + pxx;
					if(nsamp[pl] < out->max_per_pixel)
						out->frag_prims[pix * out->max_per_pixel + nsamp[pl]] = int32_t(t.prim);
				}
				nsamp[pl]++;
			}
		}
		offset += rank;
	}
	nfrag += offset;
	const float* bg = in->config->background_color;
	for(int pl = 0; pl < 32; pl++) {
		const int pxx = bin_x + startx + (pl & 7), py = bin_y + r0 + (pl >> 3);
		if(last_seg[pl] >= 0)
			ctx[pl].endSegment();
		if(pxx >= s.w || py >= s.h)
			continue;
		const size_t pix = size_t(py) * s.w + pxx;
		float rgba[4];
		ctx[pl].finish(bg, rgba);
		if(ctx[pl].invalid)
			ninvalid++;
		if(out->image)
			for(int ch = 0; ch < 4; ch++)
				out->image[pix * 4 + ch] = rgba[ch];
		if(out->frag_counts)
			out->frag_counts[pix] = nsamp[pl];
	}
}

void rasterBinRef(const State& s, int bin, oracle_outputs* out, uint64_t& nfrag, uint64_t& nhbt,
				  uint32_t& maxfrag, uint64_t& ninvalid) {
	const oracle_inputs* in = s.in;
	const int bx = bin % s.bcx, by = bin / s.bcx;
	const int bin_x = bx * kBinSize, bin_y = by * kBinSize;
	std::vector<std::pair<uint32_t, uint32_t>> tri_ids; // (tri slot, primitive id)
	for(uint32_t e : s.bin_quads[bin]) {
		const uint32_t quad = e & 0x0fffffffu;
		for(int second = 0; second < 2; second++)
			if(!((e >> (30 + second)) & 1u))
				tri_ids.push_back({quad * 2 + second, s.quad_source[quad] * 2 + second});
	}
	for(uint32_t t : s.bin_tris[bin])
		tri_ids.push_back({t, s.quad_source[t >> 1] * 2 + (t & 1)});
	const int64_t num_tris = int64_t(s.bin_tris[bin].size()) + 2 * int64_t(s.bin_quads[bin].size());
	std::vector<RefTri> tris(tri_ids.size());
	std::vector<std::vector<RefEntry>> lists;
	auto writeBackground = [&](const float* rgba4) {
		for(int r = 0; r < 32; r++)
			for(int x = 0; x < 32; x++) {
				const int pxx = bin_x + x, py = bin_y + r;
				if(pxx >= s.w || py >= s.h)
					continue;
				const size_t pix = size_t(py) * s.w + pxx;
				if(out->image)
					for(int ch = 0; ch < 4; ch++)
						out->image[pix * 4 + ch] = rgba4[ch];
				if(out->frag_counts)
					out->frag_counts[pix] = 0;
			}
	};
	if(num_tris == 0) { // EMPTY bins are not rastered; the image keeps the background
		const float* bg = in->config->background_color;
		const float rgba[4] = {saturate(bg[0]), saturate(bg[1]), saturate(bg[2]), 1.0f};
		writeBackground(rgba);
		return;
	}
	bool high = num_tris >= in->low_high_threshold;
	if(!high) {
		// raster_low: 8x8 blocks
		for(size_t i = 0; i < tris.size(); i++) {
			tris[i].tri = tri_ids[i].first, tris[i].prim = tri_ids[i].second;
			triBinRowsFrom(&s.tri_scan[size_t(tris[i].tri) * 8], bin_x, bin_y, 8, tris[i].rows);
		}
		lists.assign(16, {});
		for(size_t i = 0; i < tris.size(); i++)
			for(int brow = 0; brow < 4; brow++) {
				const uint32_t m = rowGroupColumns(tris[i].rows, brow * 8) | rowGroupColumns(tris[i].rows, brow * 8 + 4);
				for(int bcol = 0; bcol < 4; bcol++)
					if((m >> bcol) & 1u)
						lists[size_t(brow * 4 + bcol)].push_back(RefEntry{0u, tris[i].prim, int(i)});
			}
		for(auto& l : lists)
			if(l.size() > 256)
				high = true; // promoted (raster_low.glsl:211-219)
		if(!high) {
			for(int blk = 0; blk < 16; blk++) {
				const int brow = blk >> 2, bcol = blk & 3;
				auto& l = lists[size_t(blk)];
				for(RefEntry& e : l) {
					const RefTri& t = tris[size_t(e.t)];
					float cx0, cy0, cx1, cy1;
					int n0, n1;
					halfBlockCentroid(t.rows, brow * 8, bcol * 8, cx0, cy0, n0);
					halfBlockCentroid(t.rows, brow * 8 + 4, bcol * 8, cx1, cy1, n1);
					e.key = n0 + n1 > 0 ? refBlockKey(s, t.tri, cx0 + cx1, cy0 + cy1, n0 + n1, float(bin_x + bcol * 8),
													  float(bin_y + brow * 8), float(0x3ffffe))
										: 0u;
				}
				if(l.size() > 3)
					std::sort(l.begin(), l.end(), refLess);
				else
					std::sort(l.begin(), l.end(), [](const RefEntry& a, const RefEntry& b) { return a.prim < b.prim; });
				nhbt += 2 * l.size();
				refReduceHalfBlock(s, bin_x, bin_y, bcol, brow * 2, tris, l, out, nfrag, ninvalid);
				refReduceHalfBlock(s, bin_x, bin_y, bcol, brow * 2 + 1, tris, l, out, nfrag, ninvalid);
			}
		}
	}
	if(high) {
		// raster_high: 8x4 half-blocks, scan started at the half-block row
		for(size_t i = 0; i < tris.size(); i++) {
			tris[i].tri = tri_ids[i].first, tris[i].prim = tri_ids[i].second;
			triBinRowsFrom(&s.tri_scan[size_t(tris[i].tri) * 8], bin_x, bin_y, 4, tris[i].rows);
		}
		lists.assign(32, {});
		int row_count[8] = {0, 0, 0, 0, 0, 0, 0, 0}, estimate[32];
		for(int& v : estimate)
			v = 0;
		for(size_t i = 0; i < tris.size(); i++)
			for(int hrow = 0; hrow < 8; hrow++) {
				const uint32_t m = rowGroupColumns(tris[i].rows, hrow * 4);
				if(m == 0)
					continue;
				row_count[hrow]++;
				const int lo = __builtin_ctz(m), hi = 31 - __builtin_clz(m);
				for(int c = lo; c <= hi; c++)
					estimate[hrow * 4 + c]++;
				for(int c = 0; c < 4; c++)
					if((m >> c) & 1u)
						lists[size_t(hrow * 4 + c)].push_back(RefEntry{0u, tris[i].prim, int(i)});
			}
		bool error = false;
		for(int r = 0; r < 8; r++)
			error |= row_count[r] > 16384;
		for(int v : estimate)
			error |= v > 4096;
		if(error) {
			const float red[4] = {1.0f, 0.0f, 0.0f, 0.0f};
			writeBackground(red);
			return;
		}
		for(int hb = 0; hb < 32; hb++) {
			const int hrow = hb >> 2, hcol = hb & 3;
			auto& l = lists[size_t(hb)];
			for(RefEntry& e : l) {
				const RefTri& t = tris[size_t(e.t)];
				float cx, cy;
				int n;
				halfBlockCentroid(t.rows, hrow * 4, hcol * 8, cx, cy, n);
				e.key = n > 0 ? refBlockKey(s, t.tri, cx, cy, n, float(bin_x + hcol * 8), float(bin_y + hrow * 4),
											float(0x7fffe))
							  : 0u;
			}
			std::sort(l.begin(), l.end(), refLess);
			nhbt += l.size();
			refReduceHalfBlock(s, bin_x, bin_y, hcol, hrow, tris, l, out, nfrag, ninvalid);
		}
	}
	if(out->frag_counts)
		for(int r = 0; r < 32; r++)
			for(int x = 0; x < 32; x++) {
				const int pxx = bin_x + x, py = bin_y + r;
				if(pxx < s.w && py < s.h)
					maxfrag = std::max(maxfrag, uint32_t(out->frag_counts[size_t(py) * s.w + pxx]));
			}
}

void raster(State& s, oracle_outputs* out) {
	const oracle_inputs* in = s.in;
	std::vector<int> bins;
	if(in->bin_subset) {
		for(int i = 0; i < in->num_bin_subset; i++)
			if(in->bin_subset[i] >= 0 && in->bin_subset[i] < s.bins)
				bins.push_back(in->bin_subset[i]);
	} else {
		for(int b = 0; b < s.bins; b++)
			bins.push_back(b);
	}
	int nt = std::max(1, in->num_threads);
	std::atomic<size_t> next{0};
	std::vector<uint64_t> nf(nt, 0), nh(nt, 0), ni(nt, 0);
	std::vector<uint32_t> mf(nt, 0);
	auto worker = [&](int tid) {
		std::vector<std::vector<Frag>> px(1024);
		while(true) {
			size_t i = next.fetch_add(1);
			if(i >= bins.size())
				break;
			if(in->order_mode == 1)
				rasterBinRef(s, bins[i], out, nf[tid], nh[tid], mf[tid], ni[tid]);
			else
				rasterBin(s, bins[i], int(i), out, px, nf[tid], nh[tid], mf[tid]);
		}
	};
	if(nt == 1)
		worker(0);
	else {
		std::vector<std::thread> th;
		for(int t = 0; t < nt; t++)
			th.emplace_back(worker, t);
		for(auto& t : th)
			t.join();
	}
	out->num_fragments = 0, out->num_hblock_tris = 0, out->max_pixel_fragments = 0, out->invalid_pixels = 0;
	for(int t = 0; t < nt; t++) {
		out->invalid_pixels += ni[t];
		out->num_fragments += nf[t];
		out->num_hblock_tris += nh[t];
		out->max_pixel_fragments = std::max(out->max_pixel_fragments, mf[t]);
	}
}

void initState(State& s, const oracle_inputs* in) {
	s.in = in;
	s.w = in->width, s.h = in->height;
	s.bcx = (s.w + kBinSize - 1) / kBinSize;
	s.bcy = (s.h + kBinSize - 1) / kBinSize;
	s.bins = s.bcx * s.bcy;
	s.mvq = in->max_visible_quads;
	const lucid_frustum& fr = in->config->frustum;
	s.origin = xyz(fr.ws_origin0);
	s.dir0 = xyz(fr.ws_dir0);
	s.dirx = xyz(fr.ws_dirx);
	s.diry = xyz(fr.ws_diry);
	// quad_setup.glsl:397-398: ray through the centre of pixel (0, 0)
	V3 dxy = add(s.dirx, s.diry);
	s.ray_dir0 = add(s.dir0, mul(dxy, 0.5f));
}

// ---------------------------------------------------------------------------------------------
// FP64 gradient model. Positions are frozen, so coverage, per-pixel order and the barycentric
// weights (computed in FP32 exactly as the shader does, shading.glsl:116-133) are constants;
// colours and alphas are FP64 functions of the vertex colours and triangle opacities.

struct GFrag {
	uint32_t vid[3];
	uint32_t prim;
	double wgt[3];
	double inst[4];
	bool has_vc;
};

struct GradCtx {
	int w, h;
	double bg[3];
	bool has_opacity;
	std::vector<uint32_t> pix_off; // fragments of pixel i: [pix_off[i], pix_off[i+1])
	std::vector<GFrag> frags;
	std::vector<std::vector<uint32_t>> vert_pixels, prim_pixels;
};

void pixelColor64(const GradCtx& g, uint32_t pix, const double* vc, const double* op, double C[3]) {
	double T = 1.0;
	C[0] = C[1] = C[2] = 0.0;
	for(uint32_t i = g.pix_off[pix]; i < g.pix_off[pix + 1]; i++) {
		const GFrag& f = g.frags[i];
		double col[4] = {f.inst[0], f.inst[1], f.inst[2], f.inst[3]};
		if(f.has_vc)
			for(int ch = 0; ch < 4; ch++)
				col[ch] *= f.wgt[0] * vc[size_t(f.vid[0]) * 4 + ch] + f.wgt[1] * vc[size_t(f.vid[1]) * 4 + ch] +
						   f.wgt[2] * vc[size_t(f.vid[2]) * 4 + ch];
		double a = col[3] * (op ? op[f.prim] : 1.0);
		for(int ch = 0; ch < 3; ch++)
			C[ch] += col[ch] * a * T;
		T *= 1.0 - a;
	}
	for(int ch = 0; ch < 3; ch++)
		C[ch] += T * g.bg[ch];
}

double pixelLoss64(const GradCtx& g, uint32_t pix, const double* vc, const double* op, const float* target) {
	double C[3];
	pixelColor64(g, pix, vc, op, C);
	double l = 0.0;
	for(int ch = 0; ch < 3; ch++) {
		double d = std::min(std::max(C[ch], 0.0), 1.0) - double(target[size_t(pix) * 4 + ch]);
		l += d * d;
	}
	return l;
}

extern "C" int oracle_ref_shade(const oracle_inputs* in, int32_t n, const int32_t* px, const int32_t* py,
								const uint32_t* tris, uint32_t* colors, float* depths) {
	if(!in || !in->config || in->width <= 0 || in->height <= 0 || in->max_visible_quads <= 0 || n < 0 ||
	   (n > 0 && (!px || !py || !tris || !colors || !depths)))
		return 1;
	if(in->num_quads > 0 && (!in->positions || !in->quads_ib || !in->instances))
		return 1;
	State s;
	initState(s, in);
	oracle_outputs dummy;
	memset(&dummy, 0, sizeof(dummy));
	quadSetup(s, &dummy);
	for(int i = 0; i < n; i++) {
		const uint32_t tri = tris[i];
		if(tri >= 2u * uint32_t(in->max_visible_quads))
			return 1;
		const uint32_t prim = s.quad_source[tri >> 1] * 2 + (tri & 1);
		float depth = 0.0f;
		colors[i] = shadeRef(s, tri, prim, px[i], py[i], depth);
		depths[i] = depth;
	}
	return 0;
}

extern "C" int oracle_ref_reduce(const float* background, int32_t n, const uint32_t* colors, const float* depths,
								 const int32_t* seg, float* rgba) {
	if(!background || !rgba || n < 0 || (n > 0 && (!colors || !depths || !seg)))
		return 1;
	RefReduce r;
	r.init(3, false);
	for(int i = 0; i < n; i++) {
		if(i > 0 && seg[i] != seg[i - 1])
			r.endSegment();
		r.sample(colors[i], depths[i]);
	}
	if(n > 0)
		r.endSegment();
	r.finish(background, rgba);
	return 0;
}

extern "C" float oracle_ref_pow(float x, float y) { return refPow(x, y); }

} // namespace

extern "C" int oracle_version(void) { return 1; }

extern "C" void* oracle_grad_build(const oracle_inputs* in) {
	if(!in || !in->config || in->order_mode != 0)
		return nullptr;
	State s;
	initState(s, in);
	oracle_outputs dummy;
	memset(&dummy, 0, sizeof(dummy));
	quadSetup(s, &dummy);
	binning(s, &dummy);
	GradCtx* g = new GradCtx();
	g->w = s.w, g->h = s.h;
	for(int ch = 0; ch < 3; ch++)
		g->bg[ch] = in->config->background_color[ch];
	g->has_opacity = in->tri_opacity != nullptr;
	const size_t npix = size_t(s.w) * s.h;
	std::vector<std::vector<GFrag>> per_pix(npix);
	std::vector<std::vector<Frag>> px(1024);
	for(int bin = 0; bin < s.bins; bin++) {
		binFragments(s, bin, px);
		int bin_x = (bin % s.bcx) * kBinSize, bin_y = (bin / s.bcx) * kBinSize;
		for(int i = 0; i < 1024; i++) {
			auto& fr = px[i];
			if(fr.empty())
				continue;
			std::sort(fr.begin(), fr.end(), fragLess);
			int pxx = bin_x + (i & 31), py = bin_y + (i >> 5);
			auto& out = per_pix[size_t(py) * s.w + pxx];
			for(const Frag& f : fr) {
				// barycentric weights exactly as shadeFragment computes them
				const uint32_t* d = &s.tri_depth[size_t(f.tri) * 4];
				const uint32_t* b = &s.tri_bary[size_t(f.tri) * 8];
				float fx = float(pxx), fy = float(py);
				float ray_pos = 1.0f / f.depth;
				float e0 = bitsf(b[0]) * fx + (bitsf(b[1]) * fy + bitsf(b[2]));
				float e1 = bitsf(b[4]) * fx + (bitsf(b[5]) * fy + bitsf(b[6]));
				float b0 = e0 * ray_pos - bitsf(b[3]), b1 = e1 * ray_pos - bitsf(b[7]);
				float wgt = (1.0f - b0) - b1;
				uint32_t flags = d[3] & 0xffffu, inst = d[3] >> 16;
				uint32_t quad = f.tri >> 1, second = f.tri & 1;
				GFrag gf;
				gf.vid[0] = s.quad_verts[size_t(quad) * 4];
				gf.vid[1] = s.quad_verts[size_t(quad) * 4 + 1 + second];
				gf.vid[2] = s.quad_verts[size_t(quad) * 4 + 2 + second];
				gf.prim = f.prim;
				gf.wgt[0] = wgt, gf.wgt[1] = b0, gf.wgt[2] = b1;
				// instance colour x texture colour: the factor of the vertex colours
				const ShadeCoreO core = shadeCore(s, f, pxx, py);
				(void)inst;
				for(int ch = 0; ch < 4; ch++)
					gf.inst[ch] = core.factor[ch];
				gf.has_vc = (flags & LUCID_INST_HAS_VERTEX_COLORS) != 0;
				out.push_back(gf);
			}
		}
	}
	g->pix_off.resize(npix + 1, 0);
	for(size_t i = 0; i < npix; i++)
		g->pix_off[i + 1] = g->pix_off[i] + uint32_t(per_pix[i].size());
	g->frags.reserve(g->pix_off[npix]);
	g->vert_pixels.assign(size_t(in->num_verts), {});
	g->prim_pixels.assign(size_t(in->num_quads) * 2, {});
	for(size_t i = 0; i < npix; i++) {
		for(const GFrag& f : per_pix[i]) {
			g->frags.push_back(f);
			for(int k = 0; k < 3; k++)
				if(g->vert_pixels[f.vid[k]].empty() || g->vert_pixels[f.vid[k]].back() != i)
					g->vert_pixels[f.vid[k]].push_back(uint32_t(i));
			if(f.prim < g->prim_pixels.size())
				g->prim_pixels[f.prim].push_back(uint32_t(i));
		}
		std::vector<GFrag>().swap(per_pix[i]);
	}
	return g;
}

extern "C" void oracle_grad_free(void* ctx) { delete static_cast<GradCtx*>(ctx); }

extern "C" uint64_t oracle_grad_num_fragments(void* ctx) {
	return static_cast<GradCtx*>(ctx)->frags.size();
}

extern "C" double oracle_grad_loss(void* ctx, const double* vc, const double* op, const float* target) {
	const GradCtx& g = *static_cast<GradCtx*>(ctx);
	double l = 0.0;
	for(uint32_t i = 0; i + 1 < g.pix_off.size(); i++)
		l += pixelLoss64(g, i, vc, g.has_opacity ? op : nullptr, target);
	return l;
}

namespace {
// Backpropagates per-pixel upstream gradients through the FP64 blend. With target != NULL the
// upstream gradient is that of the squared-error loss on the FP64 colour; otherwise it is
// dl_dimage (h*w*4 floats), masked where color32 (h*w*3 floats, the unclamped colour of the
// FP32 forward pass) lies outside [0, 1].
int gradBackprop(const GradCtx& g, const double* vc, const double* op, const float* target,
				 const float* dl_dimage, const float* color32, double* dvc, double* dop) {
	const double* opp = g.has_opacity ? op : nullptr;
	std::vector<double> col, alpha, T;
	for(uint32_t pix = 0; pix + 1 < g.pix_off.size(); pix++) {
		uint32_t beg = g.pix_off[pix], end = g.pix_off[pix + 1];
		if(beg == end)
			continue;
		size_t n = end - beg;
		col.resize(n * 4), alpha.resize(n), T.resize(n + 1);
		double C[3] = {0.0, 0.0, 0.0};
		T[0] = 1.0;
		for(size_t i = 0; i < n; i++) {
			const GFrag& f = g.frags[beg + i];
			for(int ch = 0; ch < 4; ch++) {
				double v = f.inst[ch];
				if(f.has_vc)
					v *= f.wgt[0] * vc[size_t(f.vid[0]) * 4 + ch] + f.wgt[1] * vc[size_t(f.vid[1]) * 4 + ch] +
						 f.wgt[2] * vc[size_t(f.vid[2]) * 4 + ch];
				col[i * 4 + ch] = v;
			}
			alpha[i] = col[i * 4 + 3] * (opp ? opp[f.prim] : 1.0);
			for(int ch = 0; ch < 3; ch++)
				C[ch] += col[i * 4 + ch] * alpha[i] * T[i];
			T[i + 1] = T[i] * (1.0 - alpha[i]);
		}
		double gch[3];
		for(int ch = 0; ch < 3; ch++) {
			C[ch] += T[n] * g.bg[ch];
			double out = std::min(std::max(C[ch], 0.0), 1.0);
			// torch-style clamp gradient: passes where min <= C <= max
			if(target)
				gch[ch] = (C[ch] >= 0.0 && C[ch] <= 1.0) ? 2.0 * (out - double(target[size_t(pix) * 4 + ch])) : 0.0;
			else {
				float cf = color32[size_t(pix) * 3 + ch];
				gch[ch] = (cf >= 0.0f && cf <= 1.0f) ? double(dl_dimage[size_t(pix) * 4 + ch]) : 0.0;
			}
		}
		// back to front: B = colour behind fragment i+1; dC/da_i = T_i (c_i - B)
		double B[3] = {g.bg[0], g.bg[1], g.bg[2]};
		for(size_t ii = n; ii-- > 0;) {
			const GFrag& f = g.frags[beg + ii];
			double dcol[4] = {0.0, 0.0, 0.0, 0.0}, da = 0.0;
			for(int ch = 0; ch < 3; ch++) {
				dcol[ch] = gch[ch] * alpha[ii] * T[ii];
				da += gch[ch] * T[ii] * (col[ii * 4 + ch] - B[ch]);
			}
			double opv = opp ? opp[f.prim] : 1.0;
			dcol[3] = da * opv;
			if(dvc && f.has_vc)
				for(int k = 0; k < 3; k++)
					for(int ch = 0; ch < 4; ch++)
						dvc[size_t(f.vid[k]) * 4 + ch] += f.inst[ch] * f.wgt[k] * dcol[ch];
			if(dop && opp)
				dop[f.prim] += da * col[ii * 4 + 3];
			for(int ch = 0; ch < 3; ch++)
				B[ch] = col[ii * 4 + ch] * alpha[ii] + (1.0 - alpha[ii]) * B[ch];
		}
	}
	return 0;
}
} // namespace

extern "C" int oracle_grad_analytic(void* ctx, const double* vc, const double* op, const float* target,
									double* dvc, double* dop) {
	const GradCtx& g = *static_cast<GradCtx*>(ctx);
	return gradBackprop(g, vc, g.has_opacity ? op : nullptr, target, nullptr, nullptr, dvc, dop);
}

extern "C" int oracle_grad_backprop(void* ctx, const double* vc, const double* op, const float* dl_dimage,
									const float* color32, double* dvc, double* dop) {
	const GradCtx& g = *static_cast<GradCtx*>(ctx);
	if(!dl_dimage || !color32)
		return 1;
	return gradBackprop(g, vc, g.has_opacity ? op : nullptr, nullptr, dl_dimage, color32, dvc, dop);
}

extern "C" double oracle_grad_fd(void* ctx, const double* vc, const double* op, const float* target,
								 int kind, int index, double h) {
	const GradCtx& g = *static_cast<GradCtx*>(ctx);
	const std::vector<uint32_t>& pixels = kind == 0 ? g.vert_pixels[size_t(index) / 4] : g.prim_pixels[index];
	std::vector<double> v(vc, vc + g.vert_pixels.size() * 4);
	std::vector<double> o;
	if(g.has_opacity)
		o.assign(op, op + g.prim_pixels.size());
	double* param = kind == 0 ? &v[index] : &o[index];
	const double x = *param;
	double lp = 0.0, lm = 0.0;
	*param = x + h;
	for(uint32_t pix : pixels)
		lp += pixelLoss64(g, pix, v.data(), g.has_opacity ? o.data() : nullptr, target);
	*param = x - h;
	for(uint32_t pix : pixels)
		lm += pixelLoss64(g, pix, v.data(), g.has_opacity ? o.data() : nullptr, target);
	return (lp - lm) / (2.0 * h);
}

// ---------------------------------------------------------------------------------------------
// Quad generator (src/quad_generator.cpp): pairs triangles that share an edge into quads.
//
// triNeighbours (:18-44): neighbour across edge j of tri i is the first tri (lowest index) that
// holds the reversed directed edge, unless that is tri i itself. quadNodes (:55-120): for every
// tri in order and edge i whose neighbour also lists it, with a vertex not in the tri, one quad
// {tri[i], opposite, tri[i+1], tri[i+2]} (created by the lower-index tri of the pair), its
// squareness (:8-16) and conflicts with the other quads of both tris. genQuads (:122-201): a
// greedy independent set by score = conflicts - squareness * square_weight, then every tri in
// order gives its selected quad, or a degenerate quad (a, b, c, c); the second tri of a selected
// quad gives nothing.
// Two greedy variants: order 0 is the reference's (a heap that lowers the score of quads whose
// conflicts are removed, :154-171; equal scores by quad index, fwk's heap order being unknown);
// order 1 takes the same scores in synchronous rounds: the candidates are the undecided quads
// with the lowest number of undecided conflicts (the heap's leading term), and every candidate
// whose (score on the undecided conflicts, index) is below that of each conflicting candidate is
// selected at once. The CUDA path computes it in parallel; on the test meshes it leaves as few
// tris unpaired as the reference's order. normalize(v) = v / |v|; a NaN squareness counts as 0.

namespace {

struct QNode {
	int tris[2];
	int verts[4];
	int conflicts[4];
	float squareness;
	int degree() const {
		int d = 0;
		for(int c : conflicts)
			d += c != -1;
		return d;
	}
	void addConflict(int idx) {
		for(int c : conflicts)
			if(c == idx)
				return;
		for(int& c : conflicts)
			if(c == -1) {
				c = idx;
				return;
			}
	}
};

V3 normalize3(V3 v) {
	const float l = sqrtf(dot(v, v));
	return v3(v.x / l, v.y / l, v.z / l);
}

float quadSquareness(const V3 c[4]) {
	V3 e[4];
	for(int i = 0; i < 4; i++)
		e[i] = normalize3(sub(c[(i + 1) & 3], c[i]));
	float out = 0.0f;
	for(int i = 0; i < 4; i++)
		out += fabsf(dot(e[i], e[(i + 1) & 3]));
	const float sq = (4.0f - out) * 0.25f;
	return sq == sq ? sq : 0.0f;
}

} // namespace

extern "C" int oracle_quadgen(const float* positions, int num_verts, const int32_t* tris, int num_tris,
							  float square_weight, int order, uint32_t* out_quads, int32_t* out_num_quads,
							  int32_t* out_num_degenerate) {
	if(num_tris < 0 || (num_tris > 0 && (!tris || !positions || !out_quads)) || order < 0 || order > 1)
		return 1;
	for(int i = 0; i < 3 * num_tris; i++)
		if(tris[i] < 0 || tris[i] >= num_verts)
			return 2;
	const size_t nt = size_t(num_tris);
	// triNeighbours
	std::unordered_map<uint64_t, int> edge_tri;
	edge_tri.reserve(nt * 4);
	auto ekey = [](int a, int b) { return (uint64_t(uint32_t(a)) << 32) | uint32_t(b); };
	for(size_t i = 0; i < nt; i++)
		for(int j = 0; j < 3; j++)
			edge_tri.emplace(ekey(tris[i * 3 + j], tris[i * 3 + (j == 2 ? 0 : j + 1)]), int(i));
	std::vector<int> nb(nt * 3, -1);
	for(size_t i = 0; i < nt; i++)
		for(int j = 0; j < 3; j++) {
			auto it = edge_tri.find(ekey(tris[i * 3 + (j == 2 ? 0 : j + 1)], tris[i * 3 + j]));
			if(it != edge_tri.end() && it->second != int(i))
				nb[i * 3 + j] = it->second;
		}
	// quadNodes
	std::vector<QNode> quads;
	std::vector<int> tri_quads(nt * 3, -1);
	auto vpos = [&](int v) { return xyz(positions + size_t(v) * 3); };
	for(size_t i0 = 0; i0 < nt; i0++) {
		const int* t0 = tris + i0 * 3;
		for(int i = 0; i < 3; i++) {
			const int i1 = nb[i0 * 3 + i];
			if(i1 == -1 || tri_quads[i0 * 3 + i] != -1)
				continue;
			int j = -1;
			for(int k = 0; k < 3; k++)
				if(nb[size_t(i1) * 3 + k] == int(i0)) {
					j = k;
					break;
				}
			if(j == -1)
				continue;
			int opposite = -1;
			for(int k = 0; k < 3; k++) {
				const int ov = tris[size_t(i1) * 3 + k];
				if(ov != t0[0] && ov != t0[1] && ov != t0[2]) {
					opposite = ov;
					break;
				}
			}
			if(opposite == -1)
				continue;
			QNode q;
			q.tris[0] = int(i0), q.tris[1] = i1;
			q.verts[0] = t0[i], q.verts[1] = opposite, q.verts[2] = t0[(i + 1) % 3], q.verts[3] = t0[(i + 2) % 3];
			for(int& c : q.conflicts)
				c = -1;
			V3 pts[4];
			for(int k = 0; k < 4; k++)
				pts[k] = vpos(q.verts[k]);
			q.squareness = quadSquareness(pts);
			const int qi = int(quads.size());
			quads.push_back(q);
			tri_quads[i0 * 3 + i] = qi;
			tri_quads[size_t(i1) * 3 + j] = qi;
		}
	}
	for(size_t t = 0; t < nt; t++)
		for(int i = 0; i < 3; i++) {
			const int q0 = tri_quads[t * 3 + i], q1 = tri_quads[t * 3 + (i == 2 ? 0 : i + 1)];
			if(q0 != -1 && q1 != -1) {
				quads[size_t(q0)].addConflict(q1);
				quads[size_t(q1)].addConflict(q0);
			}
		}
	// genQuads: greedy independent set
	const size_t nq = quads.size();
	std::vector<uint8_t> state(nq, 0); // 2 selected, 1 removed
	std::vector<bool> second_tri(nt, false);
	std::vector<int> degree(nq);
	for(size_t q = 0; q < nq; q++)
		degree[q] = quads[q].degree();
	auto score = [&](size_t q) { return float(degree[q]) - quads[q].squareness * square_weight; };
	auto select = [&](size_t q) {
		state[q] = 2;
		second_tri[size_t(quads[q].tris[1])] = true;
	};
	if(order == 1) {
		// synchronous rounds: every undecided quad scores its undecided conflicts; the candidates
		// are the undecided quads of the lowest live conflict count, and every candidate whose
		// (score, index) is below that of each conflicting candidate is selected at once, its
		// conflicts removed
		std::vector<std::pair<float, int>> key(nq);
		std::vector<int> live_deg(nq, 0);
		std::vector<size_t> picked;
		size_t undecided = nq;
		while(undecided > 0) {
			int min_deg = 5;
			for(size_t q = 0; q < nq; q++) {
				if(state[q])
					continue;
				int live = 0;
				for(int c : quads[q].conflicts)
					live += c != -1 && !state[size_t(c)];
				live_deg[q] = live;
				min_deg = std::min(min_deg, live);
				float sc = float(live) - quads[q].squareness * square_weight;
				key[q] = {sc == 0.0f ? 0.0f : sc, int(q)};
			}
			auto candidate = [&](size_t q) { return !state[q] && live_deg[q] == min_deg; };
			picked.clear();
			for(size_t q = 0; q < nq; q++) {
				if(!candidate(q))
					continue;
				bool local_min = true;
				for(int c : quads[q].conflicts)
					if(c != -1 && candidate(size_t(c)) && !(key[q] < key[size_t(c)]))
						local_min = false;
				if(local_min)
					picked.push_back(q);
			}
			for(size_t q : picked) {
				select(q);
				for(int c : quads[q].conflicts)
					if(c != -1)
						state[size_t(c)] = 1;
			}
			undecided = 0;
			for(size_t q = 0; q < nq; q++)
				undecided += state[q] == 0;
		}
	} else {
		std::set<std::pair<float, int>> heap;
		std::vector<float> key(nq);
		for(size_t q = 0; q < nq; q++) {
			key[q] = score(q);
			heap.insert({key[q], int(q)});
		}
		while(!heap.empty()) {
			const size_t q = size_t(heap.begin()->second);
			heap.erase(heap.begin());
			if(state[q])
				continue;
			select(q);
			for(int c : quads[q].conflicts) {
				if(c == -1)
					continue;
				state[size_t(c)] = 1;
				for(int c2 : quads[size_t(c)].conflicts)
					if(c2 != -1 && !state[size_t(c2)]) {
						degree[size_t(c2)]--;
						heap.erase({key[size_t(c2)], c2});
						key[size_t(c2)] = score(size_t(c2));
						heap.insert({key[size_t(c2)], c2});
					}
			}
		}
	}
	// output in tri order
	int nout = 0, ndeg = 0;
	for(size_t t = 0; t < nt; t++) {
		if(second_tri[t])
			continue;
		int sel = -1;
		for(int i = 0; i < 3; i++) {
			const int q = tri_quads[t * 3 + i];
			if(q != -1 && state[size_t(q)] == 2) {
				sel = q;
				break;
			}
		}
		uint32_t* o = out_quads + size_t(nout) * 4;
		if(sel == -1) {
			o[0] = uint32_t(tris[t * 3]), o[1] = uint32_t(tris[t * 3 + 1]);
			o[2] = uint32_t(tris[t * 3 + 2]), o[3] = uint32_t(tris[t * 3 + 2]);
			ndeg++;
		} else {
			for(int k = 0; k < 4; k++)
				o[k] = uint32_t(quads[size_t(sel)].verts[k]);
		}
		nout++;
	}
	*out_num_quads = nout;
	if(out_num_degenerate)
		*out_num_degenerate = ndeg;
	return 0;
}

extern "C" int oracle_run(const oracle_inputs* in, oracle_outputs* out) {
	if(!in || !out || !in->config || in->width <= 0 || in->height <= 0 ||
	   in->max_visible_quads <= 0 || in->order_mode < 0 || in->order_mode > 1)
		return 1;
	if(in->order_mode == 1 && (in->flags & LUCID_OPT_ALPHA_THRESHOLD))
		return 1; // a subgroup vote in the reference; not part of the reference-order mode
	if(in->num_quads > 0 && (!in->positions || !in->quads_ib || !in->instances))
		return 1;
	State s;
	initState(s, in);
	out->error_code = 0;
	quadSetup(s, out);
	binning(s, out);
	auto copy = [](uint32_t* dst, const std::vector<uint32_t>& src) {
		if(dst)
			memcpy(dst, src.data(), src.size() * 4);
	};
	copy(out->quad_aabbs, s.quad_aabbs);
	copy(out->quad_source, s.quad_source);
	copy(out->quad_colors, s.quad_colors);
	copy(out->quad_verts, s.quad_verts);
	copy(out->tri_bary, s.tri_bary);
	copy(out->tri_scan, s.tri_scan);
	copy(out->tri_depth, s.tri_depth);
	copy(out->tri_normals, s.tri_normals);
	if(out->image || out->frag_counts || out->image64 || out->frag_prims)
		raster(s, out);
	return 0;
}
