// Quad setup pass (data/shaders/quad_setup.glsl) as three deterministic kernels:
//
//   setupPrepKernel     instance quad offsets (exclusive scan of InstanceData.num_quads)
//   setupClassifyKernel one thread per input quad: culling, clipped AABB, bin AABB, small/large
//   setupScanKernel     exclusive scan of the per-CTA small/large counts
//   setupStoreKernel    writes quad and triangle records at slots given by the scans
//
// The reference allocates output slots with atomics per work-group (quad_setup.glsl:415-422),
// which makes the record order nondeterministic. Here slot k < num_visible[0] holds the k-th
// visible small quad in input order, slot MAX_VISIBLE_QUADS-1-k the k-th visible large quad:
// the reference's layout (quad_setup.glsl:437-444) in a canonical order.

#include "lucid_common.cuh"
#include "lucid_kernels.h"

namespace lucid {

// ---------------------------------------------------------------------------------------------
// Per-quad math (quad_setup.glsl:64-254)

struct QuadClass {
	int cls; // -1 rejected, 0 small, 1 large
	int reason;
	uint32_t enc_aabb, y_aabb0, y_aabb1;
};

struct F4 {
	float x, y, z, w;
};

__device__ __forceinline__ F3 loadVertex(const float* pos, uint32_t idx) {
	const float* p = pos + size_t(idx) * 3;
	return f3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

__device__ __forceinline__ F4 mulPoint(const float* m, F3 p) {
	F4 r;
	r.x = m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12];
	r.y = m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13];
	r.z = m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14];
	r.w = m[3] * p.x + m[7] * p.y + m[11] * p.z + m[15];
	return r;
}

__device__ __forceinline__ uint32_t vertexClipMask(F4 p) {
	return (p.x < -p.w ? 0x001u : 0u) | (p.x > p.w ? 0x002u : 0u) | (p.y < -p.w ? 0x004u : 0u) |
		   (p.y > p.w ? 0x008u : 0u) | (p.z < -p.w ? 0x010u : 0u) | (p.z > p.w ? 0x020u : 0u);
}

// Blinn's clipped screen coverage (quad_setup.glsl:77-128)
__device__ __forceinline__ void computeClippedAABB(F4 v0, F4 v1, F4 v2, float iw0, float iw1, float iw2,
								   uint32_t clipmask, float aabb[4]) {
	F4 vn[3] = {v0, v1, v2};
	float inv_w[3] = {iw0, iw1, iw2};
	aabb[0] = 1.0f, aabb[1] = 1.0f, aabb[2] = -1.0f, aabb[3] = -1.0f;
	int any_vis = 0;
	uint32_t or_clipmask = clipmask | (clipmask >> 8) | (clipmask >> 16);
#pragma unroll
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
#pragma unroll
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
#pragma unroll
		for(int i = 0; i < 3; i++) {
			uint32_t cur = clipmask >> (i * 8);
			if((cur & 0x4u) != 0 && vn[i].y - aabb[1] * vn[i].w < 0.0f)
				aabb[1] = -1.0f;
			if((cur & 0x8u) != 0 && vn[i].y - aabb[3] * vn[i].w > 0.0f)
				aabb[3] = 1.0f;
		}
	}
}

__device__ __forceinline__ QuadClass processInputQuad(const FrameParams& p, const lucid_config& cfg,
									  const uint32_t v[4]) {
	QuadClass r;
	r.cls = -1, r.reason = LUCID_REJECTION_TYPE_OTHER;
	r.enc_aabb = r.y_aabb0 = r.y_aabb1 = 0;
	bool cull0 = v[0] == v[1] || v[1] == v[2] || v[2] == v[0];
	bool cull1 = v[0] == v[2] || v[2] == v[3] || v[3] == v[0];
	if(cull0 && cull1)
		return r;
	// Indices past the vertex array are rejected instead of read (no reference counterpart).
	uint32_t nv = uint32_t(p.num_verts);
	if(v[0] >= nv || v[1] >= nv || v[2] >= nv || v[3] >= nv) {
		raiseError(p.info, LUCID_ERR_VERTEX_INDEX, max(max(v[0], v[1]), max(v[2], v[3])), nv, 0);
		return r;
	}
	F3 vws[4] = {loadVertex(p.positions, v[0]), loadVertex(p.positions, v[1]),
				 loadVertex(p.positions, v[2]), loadVertex(p.positions, v[3])};
	cull0 = cull0 || feq(vws[0], vws[1]) || feq(vws[1], vws[2]) || feq(vws[2], vws[0]);
	cull1 = cull1 || feq(vws[0], vws[2]) || feq(vws[2], vws[3]) || feq(vws[3], vws[0]);

	if(cfg.enable_backface_culling != 0) {
		F3 o = xyz4(cfg.frustum.ws_origin0);
		F3 p0 = vws[0] - o, p1 = vws[1] - o, p2 = vws[2] - o, p3 = vws[3] - o;
		F3 nrm0 = cross3(p2, p1 - p2);
		F3 nrm1 = cross3(p3, p2 - p3);
		float volume0 = dot3(p0, nrm0);
		float volume1 = dot3(p0, nrm1);
		cull0 = cull0 || volume0 <= 0.0f;
		cull1 = cull1 || volume1 <= 0.0f;
		if(cull0 && cull1) {
			r.reason = LUCID_REJECTION_TYPE_BACKFACE;
			return r;
		}
	}
	uint32_t cull_flags = (cull0 ? 1u : 0u) | (cull1 ? 2u : 0u);

	F4 vndc[4];
#pragma unroll
	for(int i = 0; i < 4; i++)
		vndc[i] = mulPoint(cfg.view_proj_matrix, vws[i]);
	uint32_t clipmask = vertexClipMask(vndc[0]) | (vertexClipMask(vndc[1]) << 8) |
						(vertexClipMask(vndc[2]) << 16) | (vertexClipMask(vndc[3]) << 24);
	uint32_t and_clipmask = clipmask & (clipmask >> 8) & (clipmask >> 16) & (clipmask >> 24) & 0xffu;
	uint32_t or_clipmask = clipmask | (clipmask >> 8) | (clipmask >> 16) | (clipmask >> 24);
	if(and_clipmask != 0) {
		r.reason = LUCID_REJECTION_TYPE_FRUSTUM;
		return r;
	}

	float aabb0[4], aabb1[4];
	float inv_w[4] = {1.0f / vndc[0].w, 1.0f / vndc[1].w, 1.0f / vndc[2].w, 1.0f / vndc[3].w};
	if((or_clipmask & 0x30u) != 0) {
		computeClippedAABB(vndc[0], vndc[1], vndc[2], inv_w[0], inv_w[1], inv_w[2], clipmask, aabb0);
		computeClippedAABB(vndc[0], vndc[2], vndc[3], inv_w[0], inv_w[2], inv_w[3],
						   (clipmask & 0xffu) | ((clipmask & 0xffff0000u) >> 8), aabb1);
	}
#pragma unroll
	for(int i = 0; i < 4; i++) {
		vndc[i].x *= inv_w[i];
		vndc[i].y *= inv_w[i];
		vndc[i].z *= inv_w[i];
	}
	if((or_clipmask & 0x30u) == 0) {
		aabb0[0] = fminf(fminf(vndc[0].x, vndc[1].x), vndc[2].x);
		aabb0[1] = fminf(fminf(vndc[0].y, vndc[1].y), vndc[2].y);
		aabb0[2] = fmaxf(fmaxf(vndc[0].x, vndc[1].x), vndc[2].x);
		aabb0[3] = fmaxf(fmaxf(vndc[0].y, vndc[1].y), vndc[2].y);
		aabb1[0] = fminf(fminf(vndc[0].x, vndc[2].x), vndc[3].x);
		aabb1[1] = fminf(fminf(vndc[0].y, vndc[2].y), vndc[3].y);
		aabb1[2] = fmaxf(fmaxf(vndc[0].x, vndc[2].x), vndc[3].x);
		aabb1[3] = fmaxf(fmaxf(vndc[0].y, vndc[2].y), vndc[3].y);
	}

	const float hx = float(p.width) * 0.5f, hy = float(p.height) * 0.5f;
	const float mx = float(p.width - 1), my = float(p.height - 1);
	const float scale[4] = {hx, hy, hx, hy};
#pragma unroll
	for(int i = 0; i < 4; i++) {
		aabb0[i] = (aabb0[i] + 1.0f) * scale[i];
		aabb1[i] = (aabb1[i] + 1.0f) * scale[i];
	}
	float aabb[4] = {fminf(aabb0[0], aabb1[0]), fminf(aabb0[1], aabb1[1]),
					 fmaxf(aabb0[2], aabb1[2]), fmaxf(aabb0[3], aabb1[3])};
	if(ceilf(aabb[0] - 0.5001f) == floorf(aabb[2] + 0.5001f) ||
	   ceilf(aabb[1] - 0.5001f) == floorf(aabb[3] + 0.5001f)) {
		r.reason = LUCID_REJECTION_TYPE_BETWEEN_SAMPLES;
		return r;
	}
	const float adj[4] = {0.49f, 0.49f, -0.49f, -0.49f};
	const float hi[4] = {mx, my, mx, my};
#pragma unroll
	for(int i = 0; i < 4; i++) {
		aabb0[i] = fminf(fmaxf(aabb0[i] + adj[i], 0.0f), hi[i]);
		aabb1[i] = fminf(fmaxf(aabb1[i] + adj[i], 0.0f), hi[i]);
		aabb[i] = fminf(fmaxf(aabb[i] + adj[i], 0.0f), hi[i]);
	}
	uint32_t b0 = f2u(aabb[0]) >> kBinShift, b1 = f2u(aabb[1]) >> kBinShift;
	uint32_t b2 = f2u(aabb[2]) >> kBinShift, b3 = f2u(aabb[3]) >> kBinShift;
	r.enc_aabb = encodeAABB28(b0, b1, b2, b3) | (cull_flags << 30);
	uint32_t bw = b2 - b0 + 1, bh = b3 - b1 + 1;
	r.cls = bw * bh <= 4u ? 0 : 1;
	r.y_aabb0 = f2u(aabb0[1]) | (f2u(aabb0[3]) << 16);
	r.y_aabb1 = f2u(aabb1[1]) | (f2u(aabb1[3]) << 16);
	return r;
}

// storeTri (quad_setup.glsl:274-340)
__device__ __forceinline__ void storeTri(const FrameParams& p, const lucid_config& cfg, F3 ray_dir0,
						 uint32_t tri_idx, uint32_t inst_flags_id, F3 tri0, F3 tri1, F3 tri2,
						 uint32_t y_aabb, uint3 colors, const uint2* half_colors) {
	F3 dirx = xyz4(cfg.frustum.ws_dirx), diry = xyz4(cfg.frustum.ws_diry);
	F3 dir0 = xyz4(cfg.frustum.ws_dir0);
	F3 normal = cross3(tri0 - tri2, tri1 - tri0);
	float multiplier = 1.0f / sqrtf(dot3(normal, normal));
	normal = normal * multiplier;
	if((inst_flags_id & LUCID_INST_HAS_VERTEX_NORMALS) == 0) {
		uint32_t nx = f2u(512.0f + normal.x * 511.0f) & 0x3ffu;
		uint32_t ny = f2u(512.0f + normal.y * 511.0f) & 0x3ffu;
		uint32_t nz = f2u(512.0f + normal.z * 511.0f) & 0x3ffu;
		p.tri_normals[tri_idx] = nx | (ny << 10) | (nz << 20);
	}
	F3 edge0 = (tri0 - tri2) * multiplier;
	F3 edge1 = (tri1 - tri0) * multiplier;
	float plane_dist = dot3(normal, tri0);
	F3 nrm_tri0 = cross3(tri0, normal);
	float param0 = dot3(edge0, nrm_tri0);
	float param1 = dot3(edge1, nrm_tri0);
	edge0 = cross3(normal, edge0);
	edge1 = cross3(normal, edge1);
	F3 e0 = f3(dot3(edge0, dirx), dot3(edge0, diry), dot3(edge0, ray_dir0));
	F3 e1 = f3(dot3(edge1, dirx), dot3(edge1, diry), dot3(edge1, ray_dir0));
	F3 pnormal = normal * (1.0f / plane_dist);
	F3 deq = f3(dot3(pnormal, dirx), dot3(pnormal, diry), dot3(pnormal, ray_dir0));
	p.tri_depth[tri_idx] = make_uint4(fbits(deq.x), fbits(deq.y), fbits(deq.z), inst_flags_id);
	const uint4 bary0 = make_uint4(fbits(e0.x), fbits(e0.y), fbits(e0.z), fbits(param0));
	const uint4 bary1 = make_uint4(fbits(e1.x), fbits(e1.y), fbits(e1.z), fbits(param1));
	// the shading record: what a fragment of the tri reads, in 48 (64 with FP16 colours)
	// contiguous bytes (layout: ShadeRec in lucid_shade.cuh)
	uint4* rec = p.tri_shade + size_t(tri_idx) * shadeRecWords(p.color_format);
	rec[0] = bary0;
	rec[1] = bary1;
	if(half_colors) {
		rec[2] = make_uint4(half_colors[0].x, half_colors[0].y, half_colors[1].x, inst_flags_id);
		rec[3] = make_uint4(half_colors[1].y, half_colors[2].x, half_colors[2].y, 0u);
	} else {
		rec[2] = make_uint4(colors.x, colors.y, colors.z, inst_flags_id);
	}

	F3 nrm0 = cross3(tri2, tri1 - tri2);
	F3 nrm1 = cross3(tri0, tri2 - tri0);
	F3 nrm2 = cross3(tri1, tri0 - tri1);
	float volume = dot3(tri0, nrm0);
	if(volume < 0.0f) {
		nrm0 = f3(-nrm0.x, -nrm0.y, -nrm0.z);
		nrm1 = f3(-nrm1.x, -nrm1.y, -nrm1.z);
		nrm2 = f3(-nrm2.x, -nrm2.y, -nrm2.z);
	}
	F3 edges[3] = {f3(dot3(nrm0, dirx), dot3(nrm0, diry), dot3(nrm0, dir0)),
				   f3(dot3(nrm1, dirx), dot3(nrm1, diry), dot3(nrm1, dir0)),
				   f3(dot3(nrm2, dirx), dot3(nrm2, diry), dot3(nrm2, dir0))};
	float scan[3], step[3];
	uint32_t signs = 0;
#pragma unroll
	for(int i = 0; i < 3; i++) {
		float inv_ex = 1.0f / edges[i].x;
		float base = -(edges[i].z * inv_ex);
		step[i] = -(edges[i].y * inv_ex);
		scan[i] = (step[i] * 0.5f + base) - (-0.5f);
		signs |= (edges[i].x < 0.0f ? (1u << i) : 0u) | (edges[i].y < 0.0f ? (8u << i) : 0u);
	}
	p.tri_scan[size_t(tri_idx) * 2 + 0] =
		make_uint4(fbits(scan[0]), fbits(scan[1]), fbits(scan[2]), y_aabb);
	p.tri_scan[size_t(tri_idx) * 2 + 1] =
		make_uint4(fbits(step[0]), fbits(step[1]), fbits(step[2]), signs);
}

// Instance of input quad q: largest i with inst_offsets[i] <= q (binary search).
__device__ __forceinline__ int findInstance(const int* offs, int n, int q) {
	int lo = 0, hi = n; // offs[lo] <= q < offs[hi]
	while(hi - lo > 1) {
		int mid = (lo + hi) >> 1;
		if(__ldg(offs + mid) <= q)
			lo = mid;
		else
			hi = mid;
	}
	return lo;
}

__device__ __forceinline__ void loadQuadIndices(const FrameParams& p, int inst, int local,
												uint32_t v[4]) {
	lucid_instance id = p.instances[inst];
	const uint32_t* src = p.quads_ib + size_t(id.index_offset) + size_t(local) * 4;
	if((reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
		uint4 q = __ldg(reinterpret_cast<const uint4*>(src));
		v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
	} else {
		v[0] = __ldg(src), v[1] = __ldg(src + 1), v[2] = __ldg(src + 2), v[3] = __ldg(src + 3);
	}
	uint32_t vo = uint32_t(id.vertex_offset);
	v[0] += vo, v[1] += vo, v[2] += vo, v[3] += vo;
}

// ---------------------------------------------------------------------------------------------
// Kernels

template <class Src> __global__ void __launch_bounds__(1024) setupPrepKernel(Src src) {
	__shared__ int s_scan[33];
	int cta, ncta;
	const FrameParams& p = src.get(cta, ncta);
	int n = p.num_instances;
	int per = (n + blockDim.x - 1) / blockDim.x;
	int beg = min(n, int(threadIdx.x) * per), end = min(n, beg + per);
	int local = 0;
	bool bad = false;
	for(int i = beg; i < end; i++) {
		int nq = p.instances[i].num_quads;
		bad |= nq < 0 || nq > LUCID_MAX_INSTANCE_QUADS;
		local += max(nq, 0);
	}
	int total;
	int off = blockExclusiveScan(local, s_scan, &total);
	for(int i = beg; i < end; i++) {
		p.inst_offsets[i] = off;
		off += max(p.instances[i].num_quads, 0);
	}
	if(threadIdx.x == 0) {
		p.inst_offsets[n] = total;
		p.info->num_input_quads = total;
		if(total != p.num_quads)
			raiseError(p.info, LUCID_ERR_INSTANCE_QUADS, uint32_t(total), uint32_t(p.num_quads), 0);
	}
	if(bad)
		raiseError(p.info, LUCID_ERR_INSTANCE_QUADS, 0, 0, 1);
}

template <class Src> __global__ void __launch_bounds__(kSetupThreads) setupClassifyKernel(Src src) {
	__shared__ int s_counts[2 + LUCID_REJECTION_TYPE_COUNT];
	int cta, ncta;
	const FrameParams& p = src.get(cta, ncta);
	if(threadIdx.x < 2 + LUCID_REJECTION_TYPE_COUNT)
		s_counts[threadIdx.x] = 0;
	__syncthreads();
	int q = cta * blockDim.x + threadIdx.x;
	int cls = -1;
	if(q < p.num_quads) {
		int inst = findInstance(p.inst_offsets, p.num_instances, q);
		uint32_t v[4];
		loadQuadIndices(p, inst, q - __ldg(p.inst_offsets + inst), v);
		QuadClass r = processInputQuad(p, p.cfg, v);
		cls = r.cls;
		p.quad_class[q] = make_uint4(r.enc_aabb, r.y_aabb0, r.y_aabb1,
									 uint32_t(r.cls + 1) | (uint32_t(r.reason) << 8));
		if(r.cls < 0)
			atomicAdd(&s_counts[2 + r.reason], 1);
	}
	int nsmall = __syncthreads_count(cls == 0);
	int nlarge = __syncthreads_count(cls == 1);
	if(threadIdx.x == 0)
		p.setup_cta_counts[cta] = make_int4(nsmall, nlarge, 0, 0);
	if(threadIdx.x < LUCID_REJECTION_TYPE_COUNT && s_counts[2 + threadIdx.x] > 0)
		atomicAdd(&p.info->num_rejected_quads[threadIdx.x], uint32_t(s_counts[2 + threadIdx.x]));
}

template <class Src> __global__ void __launch_bounds__(1024) setupScanKernel(Src src) {
	__shared__ int s_scan[33];
	int cta, ncta;
	const FrameParams& p = src.get(cta, ncta);
	int n = p.num_setup_ctas;
	int per = (n + blockDim.x - 1) / blockDim.x;
	int beg = min(n, int(threadIdx.x) * per), end = min(n, beg + per);
	int ls = 0, ll = 0;
	for(int i = beg; i < end; i++) {
		int4 c = p.setup_cta_counts[i];
		ls += c.x, ll += c.y;
	}
	int ts, tl;
	int os = blockExclusiveScan(ls, s_scan, &ts);
	int ol = blockExclusiveScan(ll, s_scan, &tl);
	for(int i = beg; i < end; i++) {
		int4 c = p.setup_cta_counts[i];
		p.setup_cta_offsets[i] = make_int4(os, ol, 0, 0);
		os += c.x, ol += c.y;
	}
	if(threadIdx.x == 0) {
		// If everything fits these are final; otherwise setupStoreKernel overwrites them at
		// the capacity cut.
		if(int64_t(ts) + int64_t(tl) <= int64_t(p.max_visible_quads)) {
			p.info->num_visible_quads[0] = ts;
			p.info->num_visible_quads[1] = tl;
		}
	}
}

template <class Src> __global__ void __launch_bounds__(kSetupThreads) setupStoreKernel(Src src) {
	__shared__ int s_scan[kSetupThreads / 32 + 1];
	int cta, ncta;
	const FrameParams& p = src.get(cta, ncta);
	int q = cta * blockDim.x + threadIdx.x;
	uint4 rec = make_uint4(0, 0, 0, 0);
	if(q < p.num_quads)
		rec = p.quad_class[q];
	int cls = int(rec.w & 0xffu) - 1;
	int4 base = p.setup_cta_offsets[cta];
	int rs = blockExclusiveScan(cls == 0 ? 1 : 0, s_scan, (int*)nullptr);
	int rl = blockExclusiveScan(cls == 1 ? 1 : 0, s_scan, (int*)nullptr);
	if(cls < 0)
		return;
	int small_rank = base.x + rs, large_rank = base.y + rl;
	int64_t rank_all = int64_t(small_rank) + large_rank;
	int mvq = p.max_visible_quads;
	if(rank_all >= mvq) {
		if(rank_all == mvq)
			raiseError(p.info, LUCID_ERR_VISIBLE_QUADS, uint32_t(mvq), 0, 0);
		return;
	}
	if(rank_all == mvq - 1) {
		// Last quad that fits: visible counts are the kept quads of each class.
		p.info->num_visible_quads[0] = small_rank + (cls == 0 ? 1 : 0);
		p.info->num_visible_quads[1] = large_rank + (cls == 1 ? 1 : 0);
	}
	int slot = cls == 0 ? small_rank : (mvq - 1) - large_rank;
	int inst = findInstance(p.inst_offsets, p.num_instances, q);
	uint32_t v[4];
	loadQuadIndices(p, inst, q - __ldg(p.inst_offsets + inst), v);
	p.quad_aabbs[slot] = rec.x;
	p.quad_source[slot] = uint32_t(q);
	p.quad_verts[slot] = make_uint4(v[0], v[1], v[2], v[3]);
	uint32_t flags = uint32_t(p.instances[inst].flags);
	uint4 qc = make_uint4(0u, 0u, 0u, 0u);
	if((flags & LUCID_INST_HAS_VERTEX_COLORS) && p.color_format == LUCID_COLOR_RGBA8) {
		const uint32_t* cols = reinterpret_cast<const uint32_t*>(p.colors);
		qc = make_uint4(__ldg(cols + v[0]), __ldg(cols + v[1]), __ldg(cols + v[2]), __ldg(cols + v[3]));
		p.quad_colors[slot] = qc;
	}
	uint2 hq[4]; // FP16 vertex colours of the quad (into the tris' shading records)
	const bool half_vc = (flags & LUCID_INST_HAS_VERTEX_COLORS) && p.color_format == LUCID_COLOR_RGBA16F;
	if(half_vc) {
		const uint2* hc = reinterpret_cast<const uint2*>(p.colors);
#pragma unroll
		for(int i = 0; i < 4; i++)
			hq[i] = __ldg(hc + v[i]);
	}
	// storeQuad (quad_setup.glsl:256-272): vertex normals, texture coordinates relative to the
	// first vertex
	if((flags & LUCID_INST_HAS_VERTEX_NORMALS) && p.normals)
		p.quad_normals[slot] =
			make_uint4(__ldg(p.normals + v[0]), __ldg(p.normals + v[1]), __ldg(p.normals + v[2]), __ldg(p.normals + v[3]));
	if((flags & LUCID_INST_HAS_ALBEDO_TEXTURE) && p.tex_coords) {
		const float2 t0 = __ldg(p.tex_coords + v[0]), a = __ldg(p.tex_coords + v[1]);
		const float2 b = __ldg(p.tex_coords + v[2]), c = __ldg(p.tex_coords + v[3]);
		p.quad_tex[size_t(slot) * 2] = make_uint4(fbits(t0.x), fbits(t0.y), fbits(a.x - t0.x), fbits(a.y - t0.y));
		p.quad_tex[size_t(slot) * 2 + 1] =
			make_uint4(fbits(b.x - t0.x), fbits(b.y - t0.y), fbits(c.x - t0.x), fbits(c.y - t0.y));
	}
	uint32_t inst_flags_id = (flags & 0xffffu) | (uint32_t(inst) << 16);
	const lucid_config& cfg = p.cfg;
	F3 origin = xyz4(cfg.frustum.ws_origin0);
	F3 dir0 = xyz4(cfg.frustum.ws_dir0);
	F3 dxy = xyz4(cfg.frustum.ws_dirx) + xyz4(cfg.frustum.ws_diry);
	F3 ray_dir0 = dir0 + dxy * 0.5f;
#pragma unroll
	for(int second = 0; second < 2; second++) {
		if((rec.x >> (30 + second)) & 1u)
			continue;
		F3 t0 = loadVertex(p.positions, v[0]) - origin;
		F3 t1 = loadVertex(p.positions, v[1 + second]) - origin;
		F3 t2 = loadVertex(p.positions, v[2 + second]) - origin;
		const uint2 ht[3] = {hq[0], second ? hq[2] : hq[1], second ? hq[3] : hq[2]};
		storeTri(p, cfg, ray_dir0, uint32_t(slot) * 2 + second, inst_flags_id, t0, t1, t2,
				 second ? rec.z : rec.y, make_uint3(qc.x, second ? qc.z : qc.y, second ? qc.w : qc.z),
				 half_vc ? ht : nullptr);
	}
}

// ---------------------------------------------------------------------------------------------
// Launchers

void launchSetup(const FrameParams& p, cudaStream_t stream) {
	const OneView v{p};
	setupPrepKernel<<<1, 1024, 0, stream>>>(v);
	if(p.num_quads > 0) {
		setupClassifyKernel<<<p.num_setup_ctas, kSetupThreads, 0, stream>>>(v);
		setupScanKernel<<<1, 1024, 0, stream>>>(v);
		setupStoreKernel<<<p.num_setup_ctas, kSetupThreads, 0, stream>>>(v);
	}
}

void launchSetupBatch(const BatchViews& per_view, const BatchViews& setup_ctas, cudaStream_t stream) {
	setupPrepKernel<<<per_view.num_views, 1024, 0, stream>>>(per_view);
	const int n = setup_ctas.cta_off[setup_ctas.num_views];
	if(n > 0)
		setupClassifyKernel<<<n, kSetupThreads, 0, stream>>>(setup_ctas);
	setupScanKernel<<<per_view.num_views, 1024, 0, stream>>>(per_view);
	if(n > 0)
		setupStoreKernel<<<n, kSetupThreads, 0, stream>>>(setup_ctas);
}

} // namespace lucid
