// Reference-order mode of the raster pass (LUCID_OPT_REFERENCE_ORDER): the reference's own
// per-pixel order and blend instead of the exact order.
//
// refPlanKernel       one CTA per bin: the bin's path. LOW bins (< low_high_threshold tris,
//                     bin_categorizer.glsl:72) use 8x8 blocks unless a block holds more than 256
//                     tris, which promotes the bin to the HIGH path (raster_low.glsl:93-103,
//                     211-219); HIGH bins use 8x4 half-blocks and are painted red when a
//                     half-block row holds more than 16384 tris or the range estimate of one
//                     half-block exceeds 4096 (raster_high.glsl:77-81, 114-147, 297-301).
// refHalfBlockKernel  one CTA per (bin, 8x4 half-block): the list of tris whose spans touch the
//                     block (LOW: the 8x8 block, scan started at the tri's first 8-row block row,
//                     raster_low.glsl:39-64) or the half-block (HIGH: scan started at the first
//                     4-row half-block row, raster_high.glsl:60-81), each with a 22-bit (LOW) or
//                     18-bit (HIGH) key at its coverage centroid (rasterHalfBlockCentroid /
//                     rasterBlockDepth, raster.glsl:142-176), sorted by (key, primitive id) —
//                     LOW blocks of <= 3 tris by primitive id (the reference leaves both in
//                     shared-memory arrival order, which is not deterministic). The half-block's
//                     fragments, in list order and row-major within a tri, form 256-fragment
//                     segments (unpackSamples, raster.glsl:299-357). One thread per pixel then
//                     walks the list: shadeSampleRef (lit, RGBA8) and the 3-deep depth window
//                     (reduceSample / finishReduceSamples, shading.glsl:229-314), saturating the
//                     accumulated colour at the end of every segment (raster.glsl:361-398);
//                     LUCID_OPT_VISUALIZE_ERRORS uses the depth-4 window that marks pixels whose
//                     samples arrive too far out of order (shading.glsl:186-191, 258-264).

#include "lucid_common.cuh"
#include "lucid_kernels.h"
#include "lucid_shade.cuh"

namespace lucid {

constexpr int kRefThreads = 128;
constexpr int kRefMaxList = 4096;        // tris of one half-block list (raster_high.glsl:23-30)
constexpr int kRefLowBlockTris = 256;    // raster_low.glsl:17
constexpr int kRefHighRowTris = 16384;   // raster_high.glsl:32
constexpr uint8_t kRefEmpty = 0, kRefLow = 1, kRefHigh = 2, kRefError = 3;

struct RefSmem {
	unsigned long long sort_key[kRefMaxList]; // (key << 36) | (prim << 12) | entry
	uint32_t tri[kRefMaxList];
	uint32_t prim[kRefMaxList];
	uint32_t lo4[kRefMaxList];  // the half-block's 4 row spans: 8-bit lo / hi per row
	uint32_t hi4[kRefMaxList];
	uint32_t offset[kRefMaxList]; // first fragment of sorted entry j in the half-block
	int count;
	int scan[kRefThreads / 32 + 1];
};

// Row spans [r0, r0 + n) of one tri in a bin, with the scan started at the tri's first group of
// `group` rows (8 or 4) and stepped one row at a time (triBinRowsFrom of the oracle; rows
// outside the tri's groups are empty: lo 31, hi 0).
__device__ __forceinline__ void refRows(const FrameParams& p, uint32_t tri, int bin_x, int bin_y, int group,
										int r0, int n, int* lo, int* hi) {
	for(int i = 0; i < n; i++)
		lo[i] = 31, hi[i] = 0;
	const uint4 a = __ldg(p.tri_scan + size_t(tri) * 2), b = __ldg(p.tri_scan + size_t(tri) * 2 + 1);
	const int shift = group == 8 ? 3 : 2;
	const int ymin = int(a.w & 0xffffu) - bin_y, ymax = int(a.w >> 16) - bin_y;
	const int min_g = min(max(ymin, 0), 31) >> shift, max_g = min(max(ymax, 0), 31) >> shift;
	const int start = min_g * group, end = max_g * group + group;
	if(r0 + n <= start || r0 >= end)
		return;
	const float inf = __int_as_float(0x7f800000);
	const float sx = float(bin_x), sy = float(bin_y + start);
	const float step[3] = {bitsf(b.x), bitsf(b.y), bitsf(b.z)};
	const float scan0[3] = {bitsf(a.x), bitsf(a.y), bitsf(a.z)};
	float mn[3], mx[3];
	for(int k = 0; k < 3; k++) {
		const float sc = scan0[k] + (step[k] * sy - sx);
		const bool xneg = (b.w >> k) & 1u;
		mn[k] = xneg ? -inf : sc;
		mx[k] = xneg ? sc : inf;
	}
	const int stop = min(end, r0 + n);
	for(int row = start; row < stop; row++) {
		if(row >= r0) {
			const float fl = fmaxf(fmaxf(mn[0], mn[1]), fmaxf(mn[2], 0.0f));
			const float fh = fminf(fminf(mx[0], mx[1]), fminf(mx[2], float(kBinSize)));
			int l = f2i(fminf(fl, 33.0f));
			int h = f2i(fmaxf(fh, -1.0f)) - 1;
			if(l > h)
				l = 31, h = 0;
			lo[row - r0] = l, hi[row - r0] = h;
		}
		for(int k = 0; k < 3; k++)
			mn[k] += step[k], mx[k] += step[k];
	}
}

// 8-pixel columns touched by 4 rows (BX_MASK_ROW, raster.glsl:123-127)
__device__ __forceinline__ uint32_t refColumns(const int* lo, const int* hi) {
	uint32_t m = 0;
	for(int r = 0; r < 4; r++)
		if(lo[r] <= hi[r])
			m |= ((0xfu << (lo[r] >> 3)) & (0xfu >> (3 - (hi[r] >> 3))));
	return m;
}

// rasterHalfBlockCentroid (raster.glsl:142-150)
__device__ __forceinline__ void refCentroid(const int* lo, const int* hi, int startx, float& cx, float& cy, int& n) {
	const float wy[4] = {1.0f, 3.0f, 5.0f, 7.0f};
	float px[4], py[4];
	n = 0;
	for(int k = 0; k < 4; k++) {
		const int xmin = max(lo[k] - startx, 0), xmax = min(hi[k] - startx, 7);
		const int c = max(xmax - xmin + 1, 0);
		px[k] = float(xmin * 2 + c) * float(c);
		py[k] = wy[k] * float(c);
		n += c;
	}
	cx = px[0] + px[1] + px[2] + px[3];
	cy = py[0] + py[1] + py[2] + py[3];
}

// rasterBlockDepth (raster.glsl:170-176); inversesqrt = 1 / sqrt
__device__ __forceinline__ uint32_t refKey(const FrameParams& p, uint32_t tri, float cx, float cy, int n, float bx,
										   float by, float range) {
	if(n == 0)
		return 0u;
	const uint4 d = __ldg(p.tri_depth + tri);
	const float scale = 0.5f / float(n);
	const float px = cx * scale + bx, py = cy * scale + by;
	const float ray_pos = bitsf(d.x) * px + (bitsf(d.y) * py + bitsf(d.z));
	const float isq = 1.0f / sqrtf(ray_pos + 1.0f);
	return f2u(range * saturatef(isq));
}

__device__ __forceinline__ void refBinTri(const FrameParams& p, int bin, int i, int qc, uint32_t qoff, uint32_t toff,
										  uint32_t& tri, bool& valid) {
	valid = true;
	if(i < 2 * qc) {
		const uint32_t e = p.bin_quads[qoff + (i >> 1)];
		const int second = i & 1;
		valid = !((e >> (30 + second)) & 1u);
		tri = (e & 0x0fffffffu) * 2 + second;
	} else {
		tri = p.bin_tris[toff + (i - 2 * qc)];
	}
}

__global__ void __launch_bounds__(256) refPlanKernel(FrameParams p, uint8_t* plan) {
	__shared__ int cnt[32], rows[8];
	const int bin = blockIdx.x;
	const int bin_x = (bin % p.bin_count_x) * kBinSize, bin_y = (bin / p.bin_count_x) * kBinSize;
	const int qc = int(binQuadCounts(p, bin)), tc = int(binTriCounts(p, bin));
	const uint32_t qoff = binQuadOffsets(p, bin), toff = binTriOffsets(p, bin);
	const int64_t num_tris = int64_t(tc) + 2 * int64_t(qc);
	if(num_tris == 0) {
		if(threadIdx.x == 0)
			plan[bin] = kRefEmpty;
		return;
	}
	const bool lists_ok = uint64_t(qoff) + qc <= uint64_t(p.max_bin_refs) && uint64_t(toff) + tc <= uint64_t(p.max_bin_refs);
	if(!lists_ok) {
		if(threadIdx.x == 0)
			plan[bin] = kRefError;
		return;
	}
	bool high = num_tris >= p.low_high_threshold;
	int lo[32], hi[32];
	if(!high) {
		if(threadIdx.x < 32)
			cnt[threadIdx.x] = 0;
		__syncthreads();
		for(int i = threadIdx.x; i < 2 * qc + tc; i += blockDim.x) {
			uint32_t tri;
			bool valid;
			refBinTri(p, bin, i, qc, qoff, toff, tri, valid);
			if(!valid)
				continue;
			refRows(p, tri, bin_x, bin_y, 8, 0, 32, lo, hi);
			for(int brow = 0; brow < 4; brow++) {
				const uint32_t m = refColumns(lo + brow * 8, hi + brow * 8) | refColumns(lo + brow * 8 + 4, hi + brow * 8 + 4);
				for(int c = 0; c < 4; c++)
					if((m >> c) & 1u)
						atomicAdd(&cnt[brow * 4 + c], 1);
			}
		}
		__syncthreads();
		high = __syncthreads_or(threadIdx.x < 16 && cnt[threadIdx.x] > kRefLowBlockTris);
	}
	if(high) {
		if(threadIdx.x < 32)
			cnt[threadIdx.x] = 0;
		if(threadIdx.x < 8)
			rows[threadIdx.x] = 0;
		__syncthreads();
		for(int i = threadIdx.x; i < 2 * qc + tc; i += blockDim.x) {
			uint32_t tri;
			bool valid;
			refBinTri(p, bin, i, qc, qoff, toff, tri, valid);
			if(!valid)
				continue;
			refRows(p, tri, bin_x, bin_y, 4, 0, 32, lo, hi);
			for(int hrow = 0; hrow < 8; hrow++) {
				const uint32_t m = refColumns(lo + hrow * 4, hi + hrow * 4);
				if(m == 0)
					continue;
				atomicAdd(&rows[hrow], 1);
				const int c0 = __ffs(m) - 1, c1 = 31 - __clz(m);
				for(int c = c0; c <= c1; c++)
					atomicAdd(&cnt[hrow * 4 + c], 1);
			}
		}
		__syncthreads();
		const bool err = (threadIdx.x < 8 && rows[threadIdx.x] > kRefHighRowTris) ||
						 (threadIdx.x < 32 && cnt[threadIdx.x] > kRefMaxList);
		const bool any_err = __syncthreads_or(err);
		if(threadIdx.x == 0)
			plan[bin] = any_err ? kRefError : kRefHigh;
	} else if(threadIdx.x == 0) {
		plan[bin] = kRefLow;
	}
}

// ReductionContext (shading.glsl:196-314) of one pixel, in registers
struct RefWindow {
	float depth[4];
	uint32_t col[3];
	float trans;
	float out[3];
	bool invalid;

	__device__ void init() {
		for(int i = 0; i < 4; i++)
			depth[i] = 999999999.0f;
		col[0] = col[1] = col[2] = 0u;
		trans = 1.0f;
		out[0] = out[1] = out[2] = 0.0f;
		invalid = false;
	}
	__device__ void swapSlots(int a, int b) {
		float t = depth[a];
		depth[a] = depth[b], depth[b] = t;
		if(a < 3 && b < 3) {
			uint32_t c = col[a];
			col[a] = col[b], col[b] = c;
		}
	}
	__device__ void blend(uint32_t c, bool additive) {
		const float4 cur = decodeRGBA8(c);
		const float rgb[3] = {cur.x, cur.y, cur.z};
		if(additive) {
			for(int ch = 0; ch < 3; ch++)
				out[ch] = out[ch] + rgb[ch] * cur.w;
		} else {
			for(int ch = 0; ch < 3; ch++)
				out[ch] = out[ch] + (rgb[ch] * cur.w) * trans;
			trans = trans * (1.0f - cur.w);
		}
	}
	__device__ void sample(uint32_t color, float dep, int dsize, bool additive) {
		if(dep > depth[0]) {
			uint32_t c = col[0];
			col[0] = color, color = c;
			float d = depth[0];
			depth[0] = dep, dep = d;
			if(depth[0] > depth[1]) {
				swapSlots(0, 1);
				if(depth[1] > depth[2]) {
					swapSlots(1, 2);
					int i = 3;
					for(; i < dsize && depth[i - 1] > depth[i]; i++)
						swapSlots(i - 1, i);
					if(dsize == 4 && i == dsize) {
						invalid = true;
						out[0] = 1.0f, out[1] = 0.0f, out[2] = 0.0f;
						trans = 0.0f;
						return;
					}
				}
			}
		}
		for(int i = dsize - 1; i > 0; i--)
			depth[i] = depth[i - 1];
		depth[0] = dep;
		if(col[2] != 0u)
			blend(col[2], additive);
		col[2] = col[1], col[1] = col[0], col[0] = color;
	}
	__device__ void endSegment() {
		for(int ch = 0; ch < 3; ch++)
			out[ch] = saturatef(out[ch]);
	}
};

__global__ void __launch_bounds__(kRefThreads) refHalfBlockKernel(FrameParams p, const uint8_t* plan) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	RefSmem& s = *reinterpret_cast<RefSmem*>(smem_raw);
	const int bin = blockIdx.x, hb = blockIdx.y;
	const int hx = hb & 3, hy = hb >> 2; // half-block column (8 px) and row (4 px) in the bin
	const int bin_x = (bin % p.bin_count_x) * kBinSize, bin_y = (bin / p.bin_count_x) * kBinSize;
	const int t = threadIdx.x;
	const int lx = t & 7, ly = t >> 3; // pixel of thread t < 32 in the half-block
	const int px = bin_x + hx * 8 + lx, py = bin_y + hy * 4 + ly;
	const bool pix_thread = t < 32 && px < p.width && py < p.height;
	const size_t pix = size_t(py) * p.width + px;
	const uint8_t path = plan[bin];
	if(path == kRefEmpty || path == kRefError) {
		if(pix_thread) {
			const float* bg = p.cfg.background_color;
			const float4 o = path == kRefEmpty ? make_float4(saturatef(bg[0]), saturatef(bg[1]), saturatef(bg[2]), 1.0f)
											   : make_float4(1.0f, 0.0f, 0.0f, 0.0f);
			reinterpret_cast<float4*>(p.out_rgba)[pix] = o;
			if(p.dump_counts)
				p.dump_counts[pix] = 0;
		}
		return;
	}
	const bool low = path == kRefLow;
	const int qc = int(binQuadCounts(p, bin)), tc = int(binTriCounts(p, bin));
	const uint32_t qoff = binQuadOffsets(p, bin), toff = binTriOffsets(p, bin);
	if(t == 0)
		s.count = 0;
	__syncthreads();

	// the block's (LOW) or half-block's (HIGH) list with keys and this half-block's spans
	for(int i = t; i < 2 * qc + tc; i += kRefThreads) {
		uint32_t tri;
		bool valid;
		refBinTri(p, bin, i, qc, qoff, toff, tri, valid);
		if(!valid)
			continue;
		int lo[8], hi[8];
		uint32_t key;
		const int* hlo;
		const int* hhi;
		if(low) {
			const int brow = hy >> 1;
			refRows(p, tri, bin_x, bin_y, 8, brow * 8, 8, lo, hi);
			const uint32_t m = refColumns(lo, hi) | refColumns(lo + 4, hi + 4);
			if(!((m >> hx) & 1u))
				continue;
			float cx0, cy0, cx1, cy1;
			int n0, n1;
			refCentroid(lo, hi, hx * 8, cx0, cy0, n0);
			refCentroid(lo + 4, hi + 4, hx * 8, cx1, cy1, n1);
			key = refKey(p, tri, cx0 + cx1, cy0 + cy1, n0 + n1, float(bin_x + hx * 8), float(bin_y + brow * 8),
						 float(0x3ffffe));
			hlo = lo + (hy & 1) * 4, hhi = hi + (hy & 1) * 4;
		} else {
			refRows(p, tri, bin_x, bin_y, 4, hy * 4, 4, lo, hi);
			const uint32_t m = refColumns(lo, hi);
			if(!((m >> hx) & 1u))
				continue;
			float cx, cy;
			int n;
			refCentroid(lo, hi, hx * 8, cx, cy, n);
			key = refKey(p, tri, cx, cy, n, float(bin_x + hx * 8), float(bin_y + hy * 4), float(0x7fffe));
			hlo = lo, hhi = hi;
		}
		const int slot = atomicAdd(&s.count, 1);
		if(slot < kRefMaxList) {
			const uint32_t prim = __ldg(p.quad_source + (tri >> 1)) * 2 + (tri & 1);
			s.tri[slot] = tri;
			s.prim[slot] = prim;
			s.lo4[slot] = uint32_t(hlo[0]) | (uint32_t(hlo[1]) << 8) | (uint32_t(hlo[2]) << 16) | (uint32_t(hlo[3]) << 24);
			s.hi4[slot] = uint32_t(hhi[0]) | (uint32_t(hhi[1]) << 8) | (uint32_t(hhi[2]) << 16) | (uint32_t(hhi[3]) << 24);
			s.sort_key[slot] = (static_cast<unsigned long long>(key) << 36) | (static_cast<unsigned long long>(prim) << 12);
		}
	}
	__syncthreads();
	const int n = s.count;
	if(n > kRefMaxList) { // the plan kernel's bounds make this unreachable
		if(t == 0)
			raiseError(p.info, LUCID_ERR_BAND_ENTRIES, uint32_t(bin), uint32_t(n), uint32_t(kRefMaxList));
		return;
	}
	// sort keys: (key, primitive id), or primitive id alone for LOW blocks of <= 3 tris
	const bool by_prim = low && n <= 3;
	int npow = 1;
	while(npow < n)
		npow <<= 1;
	for(int i = t; i < npow; i += kRefThreads) {
		if(i < n) {
			unsigned long long k = s.sort_key[i];
			if(by_prim)
				k &= (1ull << 36) - 1;
			s.sort_key[i] = k | static_cast<unsigned long long>(i);
		} else {
			s.sort_key[i] = ~0ull;
		}
	}
	__syncthreads();
	for(int k = 2; k <= npow; k <<= 1)
		for(int j = k >> 1; j > 0; j >>= 1) {
			for(int i = t; i < npow; i += kRefThreads) {
				const int l = i ^ j;
				if(l > i) {
					const unsigned long long a = s.sort_key[i], b = s.sort_key[l];
					const bool up = (i & k) == 0;
					if((a > b) == up)
						s.sort_key[i] = b, s.sort_key[l] = a;
				}
			}
			__syncthreads();
		}

	// fragment offsets of the sorted entries in the half-block (segments of 256)
	const int startx = hx * 8;
	auto entryFrags = [&](int e) {
		int c = 0;
		for(int r = 0; r < 4; r++) {
			const int l = int((s.lo4[e] >> (8 * r)) & 0xffu), h = int((s.hi4[e] >> (8 * r)) & 0xffu);
			c += max(min(h - startx, 7) - max(l - startx, 0) + 1, 0);
		}
		return c;
	};
	const int per = (n + kRefThreads - 1) / kRefThreads;
	const int beg = min(n, t * per), end = min(n, beg + per);
	int local = 0;
	for(int j = beg; j < end; j++)
		local += entryFrags(int(s.sort_key[j] & 0xfffu));
	int total;
	int off = blockExclusiveScan(local, s.scan, &total);
	for(int j = beg; j < end; j++) {
		s.offset[j] = uint32_t(off);
		off += entryFrags(int(s.sort_key[j] & 0xfffu));
	}
	if(t == 0) {
		atomicAdd(reinterpret_cast<unsigned long long*>(&p.info->num_fragments), (unsigned long long)total);
		atomicAdd(reinterpret_cast<unsigned long long*>(&p.info->num_hblock_tris), (unsigned long long)n);
		atomicAdd(&p.info->stats[0], uint32_t(total));
		atomicAdd(&p.info->stats[1], uint32_t(n));
	}
	__syncthreads();
	if(t >= 32)
		return;

	// one thread per pixel: samples in list order through the window
	const bool additive = (p.flags & LUCID_OPT_ADDITIVE_BLENDING) != 0;
	const int dsize = (p.flags & LUCID_OPT_VISUALIZE_ERRORS) ? 4 : 3;
	RefWindow w;
	w.init();
	int last_seg = -1, nsamp = 0;
	for(int j = 0; j < n; j++) {
		const int e = int(s.sort_key[j] & 0xfffu);
		const int l = int((s.lo4[e] >> (8 * ly)) & 0xffu), h = int((s.hi4[e] >> (8 * ly)) & 0xffu);
		const int xmin = max(l - startx, 0), xmax = min(h - startx, 7);
		if(lx < xmin || lx > xmax)
			continue;
		int rank = lx - xmin;
		for(int r = 0; r < ly; r++) {
			const int lr = int((s.lo4[e] >> (8 * r)) & 0xffu), hr = int((s.hi4[e] >> (8 * r)) & 0xffu);
			rank += max(min(hr - startx, 7) - max(lr - startx, 0) + 1, 0);
		}
		const int seg = int((s.offset[j] + uint32_t(rank)) >> 8);
		if(last_seg >= 0 && seg != last_seg)
			w.endSegment();
		last_seg = seg;
		float dep;
		const uint32_t color = shadeSampleRef(p, s.tri[e], px, py, dep);
		w.sample(color, dep, dsize, additive);
		if(p.dump_prims && pix_thread && nsamp < p.dump_max)
			p.dump_prims[pix * p.dump_max + nsamp] = int(s.prim[e]);
		nsamp++;
	}
	if(last_seg >= 0)
		w.endSegment();
	for(int i = 2; i >= 0; i--)
		if(w.col[i] != 0u)
			w.blend(w.col[i], additive);
	if(pix_thread) {
		const float* bg = p.cfg.background_color;
		float4 o;
		o.x = saturatef(w.out[0] + w.trans * bg[0]);
		o.y = saturatef(w.out[1] + w.trans * bg[1]);
		o.z = saturatef(w.out[2] + w.trans * bg[2]);
		o.w = 1.0f;
		reinterpret_cast<float4*>(p.out_rgba)[pix] = o;
		if(p.dump_counts)
			p.dump_counts[pix] = nsamp;
		if(nsamp > 0)
			atomicMax(&p.info->max_pixel_fragments, uint32_t(nsamp));
		if(w.invalid)
			atomicAdd(&p.info->stats[2], 1u);
	}
}

size_t refSmemBytes() { return sizeof(RefSmem); }

cudaError_t configureRefKernel() {
	return cudaFuncSetAttribute(refHalfBlockKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(RefSmem)));
}

void launchRefRaster(const FrameParams& p, uint8_t* plan, cudaStream_t stream) {
	refPlanKernel<<<p.bin_count, 256, 0, stream>>>(p, plan);
	refHalfBlockKernel<<<dim3(p.bin_count, 32), kRefThreads, sizeof(RefSmem), stream>>>(p, plan);
}

} // namespace lucid
