// Raster pass in exact per-pixel order (replaces data/shaders/raster_low.glsl and
// raster_high.glsl; see shared/raster.glsl and shared/shading.glsl).
//
// One persistent CTA per SM walks the bin work list (HIGH bins, then LOW, then EMPTY) through
// an atomic counter. Per 32x32 bin:
//
//  A. Row spans. Each thread takes triangles of the bin's quad / tri lists and steps the
//     reference scanline one row at a time from the triangle's first 8-row block row inside
//     the bin (raster_low.glsl:39-64 with rasterBinStep, raster.glsl:116-140). Every non-empty
//     4-row band becomes an 8-byte entry (four 5-bit [min,max] spans + 24-bit tri slot, the
//     layout of raster_high.glsl:85-88) in this CTA's band scratch; spans are clipped to the
//     viewport. A shared +1/-1 difference array per row counts fragments per pixel.
//  B. Pixel groups. The bin's pixels (row-major) are cut into groups of at most 256 pixels
//     and kGroupCap fragments using the per-pixel prefix sum.
//  C. Per group: fragments (32-bit nearest-first depth key, 32-bit payload = pixel | entry)
//     are generated in shared memory, then sorted by a stable LSD radix sort on the depth key
//     followed by the pixel index (5 passes of 8 bits, warp-match ranking); runs of equal
//     depth are put in primitive-id order. Shading runs in parallel batches of 16 fragments
//     per pixel; one thread per pixel blends front to back in FP32
//     (out += rgb*a*T; T *= 1-a, shading.glsl:279-280) and stops once T == 0, after which no
//     later fragment can change the result. Background is added last (shading.glsl:312).

#include "lucid_common.cuh"
#include "lucid_kernels.h"

namespace lucid {

constexpr int RT = kRasterThreads;
constexpr int NW = RT / 32;
constexpr int kGroupCap = 8192;     // fragments per pixel group (shared-memory sort capacity)
constexpr int kGroupPixels = 256;   // pixels per group (8-bit pixel index in the payload)
constexpr int kShadeBatch = 16;     // fragments per pixel per shading round

struct RasterSmem {
	// kv[b][0] = keys, kv[b][1] = payloads of buffer b; the buffer not holding the sorted
	// fragments doubles as the 64 KB shading stage (kGroupPixels * kShadeBatch float4).
	uint32_t kv[2][2][kGroupCap];
	uint32_t radix[256 * NW];
	int pix_prefix[1025];
	int row_diff[32 * 33];
	float px_T[kGroupPixels];
	float px_c[kGroupPixels][3];
	int px_cursor[kGroupPixels];
	int band_count[8];
	int scan_tmp[NW + 1];
	uint32_t scan_tmpu[NW + 1];
	unsigned long long stat_hbt;
	int bin;
	int group_end;
	int flag;
	int single_digit;
};

size_t rasterSmemBytes() { return sizeof(RasterSmem); }
int rasterThreads() { return RT; }

__device__ __forceinline__ uint32_t entryTri(uint2 e) { return (e.x >> 20) | ((e.y >> 20) << 12); }

// Fragment colour (shading.glsl:107-165 without lighting/texturing; exact-mode FP32 colours).
__device__ __forceinline__ float4 shadeFragment(const FrameParams& p, uint32_t tri, float inv_ray_pos,
												int px, int py) {
	uint4 b0r = __ldg(p.tri_bary + size_t(tri) * 2);
	uint4 b1r = __ldg(p.tri_bary + size_t(tri) * 2 + 1);
	uint32_t fid = __ldg(&p.tri_depth[tri].w);
	float fx = float(px), fy = float(py);
	float ray_pos = 1.0f / inv_ray_pos;
	float e0 = bitsf(b0r.x) * fx + (bitsf(b0r.y) * fy + bitsf(b0r.z));
	float e1 = bitsf(b1r.x) * fx + (bitsf(b1r.y) * fy + bitsf(b1r.z));
	float b0 = e0 * ray_pos, b1 = e1 * ray_pos;
	b0 = b0 - bitsf(b0r.w);
	b1 = b1 - bitsf(b1r.w);
	uint32_t flags = fid & 0xffffu, inst = fid >> 16;
	float4 col = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
	if((flags & LUCID_INST_HAS_COLOR) && p.instance_colors)
		col = decodeRGBA8(__ldg(p.instance_colors + inst));
	if(flags & LUCID_INST_HAS_VERTEX_COLORS) {
		uint32_t quad = tri >> 1, second = tri & 1;
		uint4 qv = __ldg(p.quad_verts + quad);
		uint32_t v1 = second ? qv.z : qv.y, v2 = second ? qv.w : qv.z;
		float4 c0, c1, c2;
		if(p.color_format == LUCID_COLOR_RGBA8) {
			uint4 qc = __ldg(p.quad_colors + quad);
			c0 = decodeRGBA8(qc.x);
			c1 = decodeRGBA8(second ? qc.z : qc.y);
			c2 = decodeRGBA8(second ? qc.w : qc.z);
		} else if(p.color_format == LUCID_COLOR_RGBA16F) {
			const uint2* hc = reinterpret_cast<const uint2*>(p.colors);
			uint2 h0 = __ldg(hc + qv.x), h1 = __ldg(hc + v1), h2 = __ldg(hc + v2);
			auto cvt = [](uint2 h) {
				__half2 a = *reinterpret_cast<__half2*>(&h.x), b = *reinterpret_cast<__half2*>(&h.y);
				float2 fa = __half22float2(a), fb = __half22float2(b);
				return make_float4(fa.x, fa.y, fb.x, fb.y);
			};
			c0 = cvt(h0), c1 = cvt(h1), c2 = cvt(h2);
		} else {
			const float4* fc = reinterpret_cast<const float4*>(p.colors);
			c0 = __ldg(fc + qv.x), c1 = __ldg(fc + v1), c2 = __ldg(fc + v2);
		}
		float w = (1.0f - b0) - b1;
		col.x = col.x * (w * c0.x + (b0 * c1.x + b1 * c2.x));
		col.y = col.y * (w * c0.y + (b0 * c1.y + b1 * c2.y));
		col.z = col.z * (w * c0.z + (b0 * c1.z + b1 * c2.z));
		col.w = col.w * (w * c0.w + (b0 * c1.w + b1 * c2.w));
	}
	if(p.tri_opacity) {
		uint32_t prim = __ldg(p.quad_source + (tri >> 1)) * 2 + (tri & 1);
		col.w = col.w * __ldg(p.tri_opacity + prim);
	}
	return col;
}

__device__ __forceinline__ uint32_t fragPrim(const FrameParams& p, const uint2* scratch, int band_cap,
											 uint32_t val) {
	uint32_t band = (val >> 8) & 7u, slot = val >> 11;
	uint32_t tri = entryTri(scratch[size_t(band) * band_cap + slot]);
	return __ldg(p.quad_source + (tri >> 1)) * 2 + (tri & 1);
}

// One stable LSD pass on 8-bit digits. Returns false (and leaves the data in place) when all
// elements share the digit.
__device__ bool radixPass(RasterSmem& s, int src, int n, int shift, bool pixel_digit) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t* kin = s.kv[src][0];
	const uint32_t* vin = s.kv[src][1];
	uint32_t* kout = s.kv[src ^ 1][0];
	uint32_t* vout = s.kv[src ^ 1][1];
	int chunk = (((n + NW - 1) / NW) + 31) & ~31;
	int beg = min(n, warp * chunk), end = min(n, beg + chunk);
	for(int i = threadIdx.x; i < 256 * NW; i += RT)
		s.radix[i] = 0;
	if(threadIdx.x == 0)
		s.single_digit = 0;
	__syncthreads();
	for(int base = beg; base < end; base += 32) {
		int i = base + lane;
		bool valid = i < end;
		uint32_t d = 0;
		if(valid)
			d = pixel_digit ? (vin[i] & 0xffu) : ((kin[i] >> shift) & 0xffu);
		uint32_t act = __ballot_sync(0xffffffffu, valid);
		if(valid) {
			uint32_t peers = __match_any_sync(act, d);
			if(lane == __ffs(peers) - 1)
				s.radix[d * NW + warp] += __popc(peers);
		}
	}
	__syncthreads();
	// exclusive scan of radix[] in (digit, warp) order; 8 counters per thread
	{
		uint32_t loc[8], sum = 0;
#pragma unroll
		for(int j = 0; j < 8; j++) {
			loc[j] = s.radix[threadIdx.x * 8 + j];
			sum += loc[j];
		}
		uint32_t tot;
		uint32_t off = blockExclusiveScan(sum, s.scan_tmpu, &tot);
#pragma unroll
		for(int j = 0; j < 8; j++) {
			s.radix[threadIdx.x * 8 + j] = off;
			off += loc[j];
		}
	}
	__syncthreads();
	if(threadIdx.x < 256) {
		uint32_t d = threadIdx.x;
		uint32_t next = d < 255 ? s.radix[(d + 1) * NW] : uint32_t(n);
		if(next - s.radix[d * NW] == uint32_t(n))
			s.single_digit = 1;
	}
	__syncthreads();
	if(s.single_digit) {
		__syncthreads();
		return false;
	}
	for(int base = beg; base < end; base += 32) {
		int i = base + lane;
		bool valid = i < end;
		uint32_t k = 0, v = 0, d = 0;
		if(valid) {
			k = kin[i], v = vin[i];
			d = pixel_digit ? (v & 0xffu) : ((k >> shift) & 0xffu);
		}
		uint32_t act = __ballot_sync(0xffffffffu, valid);
		if(valid) {
			uint32_t peers = __match_any_sync(act, d);
			uint32_t pos = s.radix[d * NW + warp] + __popc(peers & laneMaskLt());
			__syncwarp(act);
			if(lane == __ffs(peers) - 1)
				s.radix[d * NW + warp] += __popc(peers);
			if(pos < uint32_t(n)) {
				kout[pos] = k;
				vout[pos] = v;
			}
		}
		__syncwarp();
	}
	__syncthreads();
	return true;
}

__device__ void writePixel(const FrameParams& p, int px, int py, float4 c) {
	if(px < p.width && py < p.height)
		reinterpret_cast<float4*>(p.out_rgba)[size_t(py) * p.width + px] = c;
}

__global__ void __launch_bounds__(RT, 1) rasterKernel(FrameParams p) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	RasterSmem& s = *reinterpret_cast<RasterSmem*>(smem_raw);
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int band_cap = p.band_capacity;
	uint2* scratch = p.band_scratch + size_t(blockIdx.x) * 8 * band_cap;
	const float4 bg = make_float4(p.cfg.background_color[0], p.cfg.background_color[1],
								  p.cfg.background_color[2], p.cfg.background_color[3]);
	const bool additive = (p.flags & LUCID_OPT_ADDITIVE_BLENDING) != 0;
	const bool alpha_threshold = (p.flags & LUCID_OPT_ALPHA_THRESHOLD) != 0;
	const bool dump = p.dump_counts != nullptr;

	while(true) {
		if(tid == 0) {
			uint32_t w = atomicAdd(&p.info->raster_work_counter, 1u);
			s.bin = w < uint32_t(p.bin_count) ? int(p.raster_work[w]) : -1;
			s.flag = 0;
			s.stat_hbt = 0;
		}
		if(tid < 8)
			s.band_count[tid] = 0;
		for(int i = tid; i < 32 * 33; i += RT)
			s.row_diff[i] = 0;
		__syncthreads();
		const int bin = s.bin;
		if(bin < 0)
			break;
		const int bx = bin % p.bin_count_x, by = bin / p.bin_count_x;
		const int bin_x = bx * kBinSize, bin_y = by * kBinSize;
		const int vis_w = p.width - bin_x, vis_h = p.height - bin_y;
		const int qc = int(binQuadCounts(p, bin)), tc = int(binTriCounts(p, bin));
		const uint32_t qoff = binQuadOffsets(p, bin), toff = binTriOffsets(p, bin);
		bool lists_ok = uint64_t(qoff) + qc <= uint64_t(p.max_bin_refs) &&
						uint64_t(toff) + tc <= uint64_t(p.max_bin_refs);

		// ---- A. row spans -> band entries + per-row fragment difference arrays
		unsigned long long hbt = 0;
		const int ntris = lists_ok ? 2 * qc + tc : 0;
		for(int i = tid; i < ntris; i += RT) {
			uint32_t tri;
			if(i < 2 * qc) {
				uint32_t e = p.bin_quads[qoff + (i >> 1)];
				int second = i & 1;
				if((e >> (30 + second)) & 1u)
					continue;
				tri = (e & 0x0fffffffu) * 2 + second;
			} else {
				tri = p.bin_tris[toff + (i - 2 * qc)];
			}
			uint4 r0 = __ldg(p.tri_scan + size_t(tri) * 2);
			uint4 r1 = __ldg(p.tri_scan + size_t(tri) * 2 + 1);
			int ymin = int(r0.w & 0xffffu) - bin_y, ymax = int(r0.w >> 16) - bin_y;
			int min_by = min(max(ymin, 0), 31) >> 3, max_by = min(max(ymax, 0), 31) >> 3;
			float sx = float(bin_x), sy = float(bin_y + min_by * 8);
			float step[3] = {bitsf(r1.x), bitsf(r1.y), bitsf(r1.z)};
			float scan0[3] = {bitsf(r0.x), bitsf(r0.y), bitsf(r0.z)};
			float mn[3], mx[3];
#pragma unroll
			for(int k = 0; k < 3; k++) {
				float sc = scan0[k] + (step[k] * sy - sx);
				bool xneg = (r1.w >> k) & 1u;
				mn[k] = xneg ? -INFINITY : sc;
				mx[k] = xneg ? sc : INFINITY;
			}
			for(int band = min_by * 2; band < max_by * 2 + 2; band++) {
				uint32_t minb = 0, maxb = 0, colmask = 0;
				bool nonempty = false;
#pragma unroll
				for(int r = 0; r < 4; r++) {
					int row = band * 4 + r;
					float fl = fmaxf(fmaxf(mn[0], mn[1]), fmaxf(mn[2], 0.0f));
					float fh = fminf(fminf(mx[0], mx[1]), fminf(mx[2], float(kBinSize)));
					int lo = f2i(fminf(fl, 33.0f));
					int hi = f2i(fmaxf(fh, -1.0f)) - 1;
#pragma unroll
					for(int k = 0; k < 3; k++)
						mn[k] += step[k], mx[k] += step[k];
					if(lo <= hi)
						colmask |= ((0xfu << (lo >> 3)) & (0xfu >> (3 - (hi >> 3))));
					int chi = min(hi, vis_w - 1);
					if(row >= vis_h)
						chi = -1;
					if(lo <= chi) {
						nonempty = true;
						atomicAdd(&s.row_diff[row * 33 + lo], 1);
						atomicAdd(&s.row_diff[row * 33 + chi + 1], -1);
					} else {
						lo = 31, chi = 0;
					}
					minb |= uint32_t(lo) << (5 * r);
					maxb |= uint32_t(chi) << (5 * r);
				}
				hbt += __popc(colmask);
				if(nonempty) {
					int slot = atomicAdd(&s.band_count[band], 1);
					if(slot < band_cap)
						scratch[size_t(band) * band_cap + slot] =
							make_uint2(minb | ((tri & 0xfffu) << 20), maxb | ((tri >> 12) << 20));
				}
			}
		}
		// reduce half-block-tri counts
#pragma unroll
		for(int o = 16; o > 0; o >>= 1)
			hbt += __shfl_xor_sync(0xffffffffu, hbt, o);
		if(lane == 0 && hbt)
			atomicAdd(&s.stat_hbt, hbt);
		__syncthreads();
		bool overflow = !lists_ok;
		for(int b = 0; b < 8; b++)
			overflow |= s.band_count[b] > band_cap;
		if(overflow) {
			if(tid == 0) {
				if(lists_ok)
					raiseError(p.info, LUCID_ERR_BAND_ENTRIES, uint32_t(bin), 0, uint32_t(band_cap));
			}
			for(int i = tid; i < 1024; i += RT)
				writePixel(p, bin_x + (i & 31), bin_y + (i >> 5), make_float4(1.0f, 0.0f, 0.0f, 1.0f));
			__syncthreads();
			continue;
		}

		// ---- B. per-pixel counts and their prefix over the bin (row-major)
		for(int row = warp; row < 32; row += NW) {
			int v = s.row_diff[row * 33 + lane];
			s.row_diff[row * 33 + lane] = warpInclusiveScan(v);
		}
		__syncthreads();
		{
			int c0 = s.row_diff[(2 * tid >> 5) * 33 + (2 * tid & 31)];
			int c1 = s.row_diff[((2 * tid + 1) >> 5) * 33 + ((2 * tid + 1) & 31)];
			int total;
			int off = blockExclusiveScan(c0 + c1, s.scan_tmp, &total);
			s.pix_prefix[2 * tid] = off;
			s.pix_prefix[2 * tid + 1] = off + c0;
			if(tid == 0)
				s.pix_prefix[1024] = total;
			int mx = max(c0, c1);
#pragma unroll
			for(int o = 16; o > 0; o >>= 1)
				mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
			if(lane == 0 && mx > 0)
				atomicMax(&p.info->max_pixel_fragments, uint32_t(mx));
			if(tid == 0) {
				unsigned long long hb = s.stat_hbt;
				atomicAdd((unsigned long long*)&p.info->num_fragments, (unsigned long long)total);
				atomicAdd((unsigned long long*)&p.info->num_hblock_tris, hb);
				atomicAdd(&p.info->stats[0], uint32_t(total));
				atomicAdd(&p.info->stats[1], uint32_t(hb));
			}
		}
		__syncthreads();

		// ---- C. pixel groups
		int p0 = 0;
		while(p0 < 1024) {
			if(tid == 0) {
				int base = s.pix_prefix[p0];
				int limit = min(p0 + kGroupPixels, 1024);
				int p1;
				if(s.pix_prefix[p0 + 1] - base > kGroupCap) {
					p1 = -(p0 + 1); // single pixel beyond capacity
				} else {
					int lo = p0 + 1, hi = limit; // largest p1 in [lo, hi] with count <= cap
					while(lo < hi) {
						int mid = (lo + hi + 1) >> 1;
						if(s.pix_prefix[mid] - base <= kGroupCap)
							lo = mid;
						else
							hi = mid - 1;
					}
					p1 = lo;
				}
				s.group_end = p1;
			}
			__syncthreads();
			int p1 = s.group_end;
			if(p1 < 0) {
				p1 = -p1;
				if(tid == 0) {
					raiseError(p.info, LUCID_ERR_PIXEL_FRAGMENTS, uint32_t(bin), uint32_t(p0),
							   uint32_t(s.pix_prefix[p0 + 1] - s.pix_prefix[p0]));
					writePixel(p, bin_x + (p0 & 31), bin_y + (p0 >> 5), make_float4(1.0f, 0.0f, 0.0f, 1.0f));
				}
				__syncthreads();
				p0 = p1;
				continue;
			}
			const int npix = p1 - p0;
			const int gbase = s.pix_prefix[p0];
			const int n = s.pix_prefix[p1] - gbase;
			const int r0 = p0 >> 5, r1 = (p1 - 1) >> 5;

			// C1. fragment generation
			int running = 0;
			for(int b = r0 >> 2; b <= (r1 >> 2); b++) {
				int ne = s.band_count[b];
				for(int base = 0; base < ne; base += RT) {
					int j = base + tid;
					int cnt = 0;
					uint2 e = make_uint2(0, 0);
					if(j < ne) {
						e = scratch[size_t(b) * band_cap + j];
#pragma unroll
						for(int r = 0; r < 4; r++) {
							int row = b * 4 + r;
							if(row < r0 || row > r1)
								continue;
							int lo = (e.x >> (5 * r)) & 31, hi = (e.y >> (5 * r)) & 31;
							int xlo = max(lo, p0 - 32 * row), xhi = min(hi, p1 - 1 - 32 * row);
							cnt += max(0, xhi - xlo + 1);
						}
					}
					int total;
					int pos = blockExclusiveScan(cnt, s.scan_tmp, &total) + running;
					if(cnt > 0) {
						uint32_t tri = entryTri(e);
						uint4 d = __ldg(p.tri_depth + tri);
						float dx = bitsf(d.x), dy = bitsf(d.y), dz = bitsf(d.z);
						uint32_t vbase = (uint32_t(b) << 8) | (uint32_t(j) << 11);
#pragma unroll
						for(int r = 0; r < 4; r++) {
							int row = b * 4 + r;
							if(row < r0 || row > r1)
								continue;
							int lo = (e.x >> (5 * r)) & 31, hi = (e.y >> (5 * r)) & 31;
							int xlo = max(lo, p0 - 32 * row), xhi = min(hi, p1 - 1 - 32 * row);
							float fy = float(bin_y + row);
							float ty = dy * fy + dz;
							for(int x = xlo; x <= xhi; x++) {
								float inv_ray_pos = dx * float(bin_x + x) + ty;
								if(pos < n) { // n <= kGroupCap; counts and spans agree by construction
									s.kv[0][0][pos] = nearFirstKey(inv_ray_pos);
									s.kv[0][1][pos] = vbase | uint32_t(row * 32 + x - p0);
								}
								pos++;
							}
						}
					}
					running += total;
				}
			}
			__syncthreads();

			// C2. stable radix sort: depth key bytes 0..3, then pixel
			int cur = 0;
			if(n > 1) {
				for(int pass = 0; pass < 4; pass++)
					if(radixPass(s, cur, n, pass * 8, false))
						cur ^= 1;
				if(radixPass(s, cur, n, 0, true))
					cur ^= 1;
			}
			uint32_t* K = s.kv[cur][0];
			uint32_t* V = s.kv[cur][1];

			// C3. equal-depth runs in primitive order
			for(int i = tid; i < n; i += RT) {
				bool same_prev = i > 0 && K[i - 1] == K[i] && ((V[i - 1] ^ V[i]) & 0xffu) == 0;
				bool same_next = i + 1 < n && K[i + 1] == K[i] && ((V[i + 1] ^ V[i]) & 0xffu) == 0;
				if(!same_prev && same_next) {
					int e = i + 1;
					while(e < n && K[e] == K[i] && ((V[e] ^ V[i]) & 0xffu) == 0)
						e++;
					for(int a = i + 1; a < e; a++) { // insertion sort by primitive id
						uint32_t va = V[a], pa = fragPrim(p, scratch, band_cap, va);
						int c = a - 1;
						while(c >= i && fragPrim(p, scratch, band_cap, V[c]) > pa) {
							V[c + 1] = V[c];
							c--;
						}
						V[c + 1] = va;
					}
				}
			}
			for(int t = tid; t < npix; t += RT) {
				s.px_T[t] = 1.0f;
				s.px_c[t][0] = s.px_c[t][1] = s.px_c[t][2] = 0.0f;
				s.px_cursor[t] = s.pix_prefix[p0 + t] - gbase;
			}
			__syncthreads();

			// C4. shade in batches, blend sequentially per pixel
			float4* stage = reinterpret_cast<float4*>(&s.kv[cur ^ 1][0][0]);
			while(true) {
				for(int slot = tid; slot < npix * kShadeBatch; slot += RT) {
					int t = slot / kShadeBatch, j = slot % kShadeBatch;
					int f = s.px_cursor[t] + j;
					int fend = s.pix_prefix[p0 + t + 1] - gbase;
					if(f < fend && (s.px_T[t] != 0.0f || dump)) {
						uint32_t v = V[f];
						uint32_t band = (v >> 8) & 7u, eslot = v >> 11;
						uint32_t tri = entryTri(scratch[size_t(band) * band_cap + eslot]);
						int pl = p0 + int(v & 0xffu);
						stage[slot] = shadeFragment(p, tri, keyToDepth(K[f]), bin_x + (pl & 31),
													bin_y + (pl >> 5));
					}
				}
				__syncthreads();
				bool active = false;
				for(int t = tid; t < npix; t += RT) {
					int f = s.px_cursor[t];
					int fend = s.pix_prefix[p0 + t + 1] - gbase;
					int fbeg = s.pix_prefix[p0 + t] - gbase;
					float T = s.px_T[t];
					float c0 = s.px_c[t][0], c1 = s.px_c[t][1], c2 = s.px_c[t][2];
					int j = 0;
					for(; j < kShadeBatch && f < fend; j++, f++) {
						if(T == 0.0f && !dump)
							break;
						float4 c = stage[t * kShadeBatch + j];
						if(dump) {
							int idx = f - fbeg;
							if(idx < p.dump_max) {
								int pl = p0 + t;
								int px = bin_x + (pl & 31), py = bin_y + (pl >> 5);
								if(px < p.width && py < p.height)
									p.dump_prims[(size_t(py) * p.width + px) * p.dump_max + idx] =
										int(fragPrim(p, scratch, band_cap, V[f]));
							}
						}
						if(additive) {
							c0 = c0 + c.x * c.w;
							c1 = c1 + c.y * c.w;
							c2 = c2 + c.z * c.w;
						} else {
							c0 = c0 + (c.x * c.w) * T;
							c1 = c1 + (c.y * c.w) * T;
							c2 = c2 + (c.z * c.w) * T;
							T = T * (1.0f - c.w);
							if(alpha_threshold && T < (1.0f / 128.0f)) {
								f = fend; // done with this pixel
								break;
							}
						}
					}
					s.px_cursor[t] = f;
					s.px_T[t] = T;
					s.px_c[t][0] = c0, s.px_c[t][1] = c1, s.px_c[t][2] = c2;
					active |= f < fend && (T != 0.0f || dump);
				}
				if(!__syncthreads_or(active))
					break;
			}
			for(int t = tid; t < npix; t += RT) {
				int pl = p0 + t;
				int px = bin_x + (pl & 31), py = bin_y + (pl >> 5);
				float T = s.px_T[t];
				float4 o;
				o.x = fminf(fmaxf(s.px_c[t][0] + T * bg.x, 0.0f), 1.0f);
				o.y = fminf(fmaxf(s.px_c[t][1] + T * bg.y, 0.0f), 1.0f);
				o.z = fminf(fmaxf(s.px_c[t][2] + T * bg.z, 0.0f), 1.0f);
				o.w = 1.0f;
				writePixel(p, px, py, o);
				if(dump && px < p.width && py < p.height)
					p.dump_counts[size_t(py) * p.width + px] = s.pix_prefix[pl + 1] - s.pix_prefix[pl];
			}
			if(tid == 0 && running != n)
				raiseError(p.info, LUCID_ERR_BIN_COUNT, uint32_t(bin), uint32_t(running), uint32_t(n));
			__syncthreads();
			p0 = p1;
		}
	}
}

void launchRaster(const FrameParams& p, int num_ctas, cudaStream_t stream) {
	rasterKernel<<<num_ctas, RT, sizeof(RasterSmem), stream>>>(p);
}

cudaError_t configureRasterKernel() {
	return cudaFuncSetAttribute(rasterKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
								int(sizeof(RasterSmem)));
}

} // namespace lucid
