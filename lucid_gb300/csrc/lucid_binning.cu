// Binning passes: data/shaders/bin_counter.glsl, bin_categorizer.glsl, bin_dispatcher.glsl.
//
// binCountKernel      fixed grid of CTAs; CTA c owns a contiguous range of the visible small
//                     quads and of the visible large quads. Shared-memory histogram per bin,
//                     written to the CTA's row of bin_batches (the reference keeps the same
//                     per-work-group histograms, bin_counter.glsl:184-190) and added to the
//                     global BIN_QUAD_COUNTS / BIN_TRI_COUNTS.
//                     Small quads count every bin of their AABB; large triangles count bin
//                     rows by the conservative bin scanline (scanline.glsl:28-52) as a +1/-1
//                     difference array closed by a warp prefix scan per row.
// binCategorizeKernel one CTA: exclusive scans of the counts (offsets), LOW/HIGH bin lists in
//                     bin order, level counts and the raster work list (HIGH, LOW, EMPTY).
// binDispatchKernel   same CTA ranges as the counter; each CTA reserves its slice of every bin
//                     once (atomicAdd on *_OFFSETS_TEMP) and scatters quad / tri references.
//
// binSortKernel       (LUCID_OPT_SORTED_BIN_LISTS) one CTA per bin: each bin's quad and tri
//                     reference lists in slot order, so that a frame's bin lists are
//                     reproducible bit for bit. Without it the order inside a bin depends on
//                     the CTAs' reservations (atomics, as in the reference); no later pass
//                     depends on it.
//
// For small quads (at most 4 bins each) the counter and dispatcher aggregate per warp with
// __match_any_sync: lanes whose quad touches the same bin add to it with one shared atomic and
// take consecutive slots of it. Large tris cover very different numbers of rows and bins, so
// each lane walks its own tri.

#include "lucid_common.cuh"
#include "lucid_kernels.h"

namespace lucid {

struct BinScan {
	float mn[3], mx[3], step[3];
};

// scanline.glsl:28-52 (loadScanlineParamsBin) for bins of 1 << bsh pixels (BIN_SIZE, BIN_SHIFT)
__device__ __forceinline__ BinScan loadScanlineParamsBin(uint4 r0, uint4 r1, int& min_by,
														 int& max_by, int bsh) {
	BinScan s;
	float scan[3] = {bitsf(r0.x), bitsf(r0.y), bitsf(r0.z)};
	s.step[0] = bitsf(r1.x), s.step[1] = bitsf(r1.y), s.step[2] = bitsf(r1.z);
	min_by = int(r0.w & 0xffffu) >> bsh;
	max_by = int(r0.w >> 16) >> bsh;
	const float bin_size = float(1 << bsh);
	const float offset = bin_size - 0.989f;
	const float start_x = 0.99f, start_y = float(min_by << bsh) - 0.01f;
#pragma unroll
	for(int i = 0; i < 3; i++) {
		bool xneg = (r1.w >> i) & 1u, yneg = (r1.w >> (3 + i)) & 1u;
		float yoff = yneg ? 0.0f : offset, xoff = xneg ? 0.0f : offset;
		scan[i] = scan[i] + (s.step[i] * (yoff + start_y) - (xoff + start_x));
		s.mn[i] = xneg ? -INFINITY : scan[i];
		s.mx[i] = xneg ? scan[i] : INFINITY;
		s.step[i] = s.step[i] * bin_size;
	}
	return s;
}

// bin_counter.glsl:53-62 (scanlineStep)
__device__ __forceinline__ void scanlineStep(BinScan& s, int& bmin, int& bmax, int bsh) {
	float xmin = fmaxf(fmaxf(s.mn[0], s.mn[1]), s.mn[2]);
	float xmax = fminf(fminf(s.mx[0], s.mx[1]), s.mx[2]);
#pragma unroll
	for(int i = 0; i < 3; i++)
		s.mn[i] += s.step[i], s.mx[i] += s.step[i];
	bmin = f2i(xmin + 1.0f) >> bsh;
	bmax = f2i(xmax) >> bsh;
}

__device__ __forceinline__ void ctaRange(int n, int cta, int ncta, int& beg, int& end) {
	beg = int((int64_t(n) * cta) / ncta);
	end = int((int64_t(n) * (cta + 1)) / ncta);
}

// ---------------------------------------------------------------------------------------------
// Warp aggregation: lanes holding the same bin (key >= 0) add their count with one shared atomic
// by the group's lowest lane. Every lane of the warp must call these.

__device__ __forceinline__ void warpAddBin(int* s_bins, int key, int sign) {
	const uint32_t peers = __match_any_sync(0xffffffffu, key);
	if(key >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1)
		atomicAdd(&s_bins[key], sign * __popc(peers));
}

// Slot of this lane's reference to bin `key` (>= 0): the group's lowest lane reserves the group's
// slots with one shared atomic; lanes take them in lane order.
__device__ __forceinline__ uint32_t warpBinSlot(int* s_bins, int key) {
	const uint32_t peers = __match_any_sync(0xffffffffu, key);
	const int leader = __ffs(peers) - 1;
	int base = 0;
	if(key >= 0 && (threadIdx.x & 31) == leader)
		base = atomicAdd(&s_bins[key], __popc(peers));
	base = __shfl_sync(0xffffffffu, base, leader);
	return uint32_t(base + __popc(peers & laneMaskLt()));
}

// The bins of an encoded AABB (setup encodes it in 32-pixel bins, 7 bits per coordinate) in the
// frame's bins of 1 << bin_shift pixels; an empty AABB stays empty.
__device__ __forceinline__ void decodeBinAABB(const FrameParams& p, uint32_t enc, int& x0, int& y0, int& x1, int& y1) {
	decodeAABB28(enc, x0, y0, x1, y1);
	const int sh = p.bin_shift - kBinShift;
	x0 >>= sh, y0 >>= sh, x1 >>= sh, y1 >>= sh;
}

// Bin j (0..3) of a small quad's bin AABB (at most 4 bins, bin_counter.glsl:64-80), -1 if none.
__device__ __forceinline__ int smallQuadBin(int x0, int y0, int x1, int y1, int bcx, int j) {
	const int w = x1 - x0 + 1, n = w * (y1 - y0 + 1);
	if(j >= n)
		return -1;
	return (y0 + j / w) * bcx + x0 + j % w;
}

// A large quad's tri of work item `it` (2 per quad, large quads counted from the top slot down):
// its slot and encoded AABB; false when the tri is culled.
__device__ __forceinline__ bool largeTri(const FrameParams& p, int lbeg, int it, uint32_t& tri, uint32_t& enc) {
	const int k = lbeg + (it >> 1), second = it & 1;
	const int quad_idx = (p.max_visible_quads - 1) - k;
	enc = p.quad_aabbs[quad_idx];
	tri = uint32_t(quad_idx) * 2 + second;
	return ((enc >> (30 + second)) & 1u) == 0u;
}

// ---------------------------------------------------------------------------------------------

template <class Src> __global__ void __launch_bounds__(kBinningThreads, 1) binCountKernel(Src src) {
	extern __shared__ int s_bins[];
	int cta, ncta;
	const FrameParams& p = src.get(cta, ncta);
	const int bins = p.bin_count, bcx = p.bin_count_x, bcy = p.bin_count_y;
	const int nsmall = p.info->num_visible_quads[0], nlarge = p.info->num_visible_quads[1];
	int* hist = p.bin_batches + size_t(cta) * 2 * bins;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

	// ---- small quads: every bin of the AABB (bin_counter.glsl:64-80), one shared atomic per
	// distinct bin of a warp
	for(int i = threadIdx.x; i < bins; i += blockDim.x)
		s_bins[i] = 0;
	__syncthreads();
	int sbeg, send;
	ctaRange(nsmall, cta, ncta, sbeg, send);
	for(int base = sbeg + warp * 32; base < send; base += blockDim.x) {
		const int k = base + lane;
		int x0 = 0, y0 = 0, x1 = -1, y1 = -1;
		if(k < send)
			decodeBinAABB(p, p.quad_aabbs[k], x0, y0, x1, y1);
		const int nb = __reduce_max_sync(0xffffffffu, (x1 - x0 + 1) * (y1 - y0 + 1));
		for(int j = 0; j < nb; j++)
			warpAddBin(s_bins, k < send ? smallQuadBin(x0, y0, x1, y1, bcx, j) : -1, 1);
	}
	__syncthreads();
	for(int i = threadIdx.x; i < bins; i += blockDim.x) {
		int v = s_bins[i];
		hist[i] = v;
		if(v > 0)
			atomicAdd(&binQuadCounts(p, i), uint32_t(v));
	}
	__syncthreads();

	// ---- large tris: bin rows by scanline (bin_counter.glsl:112-134) as +1 / -1 difference
	// arrays (rows per tri vary widely: one lane per tri, shared atomics)
	for(int i = threadIdx.x; i < bins; i += blockDim.x)
		s_bins[i] = 0;
	__syncthreads();
	int lbeg, lend;
	ctaRange(nlarge, cta, ncta, lbeg, lend);
	const int items = 2 * (lend - lbeg);
	for(int it = threadIdx.x; it < items; it += blockDim.x) {
		uint32_t tri, enc;
		if(!largeTri(p, lbeg, it, tri, enc))
			continue;
		int x0, y0, x1, y1;
		decodeBinAABB(p, enc, x0, y0, x1, y1);
		int bsy, bey;
		BinScan sc = loadScanlineParamsBin(p.tri_scan[size_t(tri) * 2], p.tri_scan[size_t(tri) * 2 + 1], bsy, bey,
										   p.bin_shift);
		for(int by = bsy; by <= bey; by++) {
			int bmin, bmax;
			scanlineStep(sc, bmin, bmax, p.bin_shift);
			bmin = max(bmin, x0), bmax = min(bmax, x1);
			if(bmax >= bmin) {
				atomicAdd(&s_bins[bmin + by * bcx], 1);
				if(bmax + 1 < bcx)
					atomicAdd(&s_bins[bmax + 1 + by * bcx], -1);
			}
		}
	}
	__syncthreads();
	// close the difference arrays: one warp per bin row (bin_counter.glsl:82-103)
	{
		const int nw = blockDim.x >> 5;
		for(int by = warp; by < bcy; by += nw) {
			int prev = 0;
			for(int base = 0; base < bcx; base += 32) {
				int bx = base + lane;
				int v = bx < bcx ? s_bins[by * bcx + bx] : 0;
				int acc = prev + warpInclusiveScan(v);
				if(bx < bcx)
					s_bins[by * bcx + bx] = acc;
				prev = __shfl_sync(0xffffffffu, acc, 31);
			}
		}
	}
	__syncthreads();
	for(int i = threadIdx.x; i < bins; i += blockDim.x) {
		int v = s_bins[i];
		hist[bins + i] = v;
		if(v > 0)
			atomicAdd(&binTriCounts(p, i), uint32_t(v));
	}
	if(threadIdx.x < 2 && cta < LUCID_INFO_MAX_DISPATCHES) {
		int batch = threadIdx.x == 0 ? 4096 : 512;
		int beg = threadIdx.x == 0 ? sbeg : lbeg, end = threadIdx.x == 0 ? send : lend;
		p.info->dispatcher_first_batch[threadIdx.x][cta] = end > beg ? beg / batch : -1;
		p.info->dispatcher_num_batches[threadIdx.x][cta] = (end - beg + batch - 1) / batch;
	}
	if(cta == 0 && threadIdx.x == 0) {
		// quad_setup.glsl:471-485
		int tasks = (nsmall + 4095) / 4096 + (nlarge + 511) / 512;
		p.info->num_binning_dispatches[0] = uint32_t(min(max(tasks, 4), kMaxDispatches));
		p.info->num_binning_dispatches[1] = 1;
		p.info->num_binning_dispatches[2] = 1;
		p.info->num_counted_quads[0] = nsmall;
		p.info->num_counted_quads[1] = nlarge;
	}
}

// ---------------------------------------------------------------------------------------------

template <class Src> __global__ void __launch_bounds__(1024) binCategorizeKernel(Src src) {
	__shared__ uint32_t s_scan[33];
	__shared__ int s_iscan[33];
	__shared__ uint32_t s_base[2];
	int cta, ncta;
	const FrameParams& p = src.get(cta, ncta);
	const int bins = p.bin_count;
	const int per = (bins + blockDim.x - 1) / blockDim.x;
	const int beg = min(bins, int(threadIdx.x) * per), end = min(bins, beg + per);

	// bin_categorizer.glsl:22-53: exclusive scans into *_OFFSETS and *_OFFSETS_TEMP
	uint32_t lq = 0, lt = 0;
	int nlow = 0, nhigh = 0, nempty = 0;
	for(int i = beg; i < end; i++) {
		uint32_t q = binQuadCounts(p, i), t = binTriCounts(p, i);
		lq += q, lt += t;
		int64_t num_tris = int64_t(t) + int64_t(q) * 2;
		if(num_tris == 0)
			nempty++;
		else if(num_tris < p.low_high_threshold)
			nlow++;
		else
			nhigh++;
	}
	uint32_t tq, tt;
	uint32_t oq = blockExclusiveScan(lq, s_scan, &tq);
	uint32_t ot = blockExclusiveScan(lt, s_scan, &tt);
	// views of a batch take their lists from the shared reference buffers
	if(threadIdx.x == 0) {
		s_base[0] = p.ref_alloc ? atomicAdd(&p.ref_alloc[0], tq) : 0u;
		s_base[1] = p.ref_alloc ? atomicAdd(&p.ref_alloc[1], tt) : 0u;
	}
	__syncthreads();
	const uint32_t base_q = s_base[0], base_t = s_base[1];
	oq += base_q, ot += base_t;
	int tlow, thigh, tempty;
	int olow = blockExclusiveScan(nlow, s_iscan, &tlow);
	int ohigh = blockExclusiveScan(nhigh, s_iscan, &thigh);
	int oempty = blockExclusiveScan(nempty, s_iscan, &tempty);
	// bin_categorizer.glsl:57-89: levels (EMPTY, LOW < threshold, HIGH), lists in bin order
	for(int i = beg; i < end; i++) {
		uint32_t q = binQuadCounts(p, i), t = binTriCounts(p, i);
		binQuadOffsets(p, i) = oq;
		binQuadOffsetsTemp(p, i) = oq;
		binTriOffsets(p, i) = ot;
		binTriOffsetsTemp(p, i) = ot;
		oq += q, ot += t;
		int64_t num_tris = int64_t(t) + int64_t(q) * 2;
		if(num_tris == 0) {
			p.raster_work[thigh + tlow + oempty++] = uint32_t(i);
		} else if(num_tris < p.low_high_threshold) {
			lowLevelBins(p, olow) = uint32_t(i);
			p.raster_work[thigh + olow] = uint32_t(i);
			olow++;
		} else {
			highLevelBins(p, ohigh) = uint32_t(i);
			p.raster_work[ohigh] = uint32_t(i);
			ohigh++;
		}
	}
	if(threadIdx.x < LUCID_BIN_LEVELS_COUNT) {
		int lv = threadIdx.x;
		int cnt = lv == LUCID_BIN_LEVEL_EMPTY ? tempty
				  : lv == LUCID_BIN_LEVEL_LOW ? tlow
				  : lv == LUCID_BIN_LEVEL_HIGH ? thigh
											  : 0;
		p.info->bin_level_counts[lv] = cnt;
		int maxd = kMaxDispatches >> (lv == LUCID_BIN_LEVEL_HIGH ? 1 : 0);
		p.info->bin_level_dispatches[lv][0] = uint32_t(min(cnt, maxd));
		p.info->bin_level_dispatches[lv][1] = 1;
		p.info->bin_level_dispatches[lv][2] = 1;
	}
	if(threadIdx.x == 0) {
		p.info->num_bin_quad_refs = tq;
		p.info->num_bin_tri_refs = tt;
		if(uint64_t(base_q) + tq > uint64_t(p.max_bin_refs) || uint64_t(base_t) + tt > uint64_t(p.max_bin_refs))
			raiseError(p.info, LUCID_ERR_BIN_REFS, base_q + tq, base_t + tt, uint32_t(p.max_bin_refs));
	}
}

// ---------------------------------------------------------------------------------------------

template <class Src> __global__ void __launch_bounds__(kBinningThreads, 1) binDispatchKernel(Src src) {
	extern __shared__ int s_bins[];
	int cta, ncta;
	const FrameParams& p = src.get(cta, ncta);
	const int bins = p.bin_count, bcx = p.bin_count_x;
	const uint32_t cap = uint32_t(p.max_bin_refs);
	const int nsmall = p.info->num_visible_quads[0], nlarge = p.info->num_visible_quads[1];
	const int* hist = p.bin_batches + size_t(cta) * 2 * bins;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

	// ---- small quads (bin_dispatcher.glsl:66-80, 202-232): the CTA reserves its slice of every
	// bin once; a warp's references to one bin take consecutive slots of it
	for(int i = threadIdx.x; i < bins; i += blockDim.x) {
		int v = hist[i];
		s_bins[i] = v > 0 ? int(atomicAdd(&binQuadOffsetsTemp(p, i), uint32_t(v))) : 0;
	}
	__syncthreads();
	int sbeg, send;
	ctaRange(nsmall, cta, ncta, sbeg, send);
	for(int base = sbeg + warp * 32; base < send; base += blockDim.x) {
		const int k = base + lane;
		int x0 = 0, y0 = 0, x1 = -1, y1 = -1;
		uint32_t entry = 0u;
		if(k < send) {
			const uint32_t enc = p.quad_aabbs[k];
			entry = uint32_t(k) | (enc & 0xf0000000u);
			decodeBinAABB(p, enc, x0, y0, x1, y1);
		}
		const int nb = __reduce_max_sync(0xffffffffu, (x1 - x0 + 1) * (y1 - y0 + 1));
		for(int j = 0; j < nb; j++) {
			const int key = k < send ? smallQuadBin(x0, y0, x1, y1, bcx, j) : -1;
			const uint32_t slot = warpBinSlot(s_bins, key);
			if(key >= 0 && slot < cap)
				p.bin_quads[slot] = entry;
		}
	}
	__syncthreads();

	// ---- large tris (bin_dispatcher.glsl:89-114, 234-258): one lane per tri (rows and spans vary
	// widely), a shared atomic per reference
	for(int i = threadIdx.x; i < bins; i += blockDim.x) {
		int v = hist[bins + i];
		s_bins[i] = v > 0 ? int(atomicAdd(&binTriOffsetsTemp(p, i), uint32_t(v))) : 0;
	}
	__syncthreads();
	int lbeg, lend;
	ctaRange(nlarge, cta, ncta, lbeg, lend);
	const int items = 2 * (lend - lbeg);
	for(int it = threadIdx.x; it < items; it += blockDim.x) {
		uint32_t tri, enc;
		if(!largeTri(p, lbeg, it, tri, enc))
			continue;
		int x0, y0, x1, y1;
		decodeBinAABB(p, enc, x0, y0, x1, y1);
		int bsy, bey;
		BinScan sc = loadScanlineParamsBin(p.tri_scan[size_t(tri) * 2], p.tri_scan[size_t(tri) * 2 + 1], bsy, bey,
										   p.bin_shift);
		for(int by = bsy; by <= bey; by++) {
			int bmin, bmax;
			scanlineStep(sc, bmin, bmax, p.bin_shift);
			bmin = max(bmin, x0), bmax = min(bmax, x1);
			for(int bx = bmin; bx <= bmax; bx++) {
				uint32_t slot = uint32_t(atomicAdd(&s_bins[by * bcx + bx], 1));
				if(slot < cap)
					p.bin_tris[slot] = tri;
			}
		}
	}
}

// ---------------------------------------------------------------------------------------------
// Canonical order of the bin reference lists: the dispatcher's slices come in the order the CTAs
// reserved them (atomics, as in the reference), so each bin's quad and tri lists are sorted here
// by slot (quad references by their low 28 bits; the cull flags ride along). Every later pass is
// order-independent; the sorted lists make a frame's binning bit-reproducible. One CTA per bin:
// up to 32 references by one warp in registers, up to kSortCap in shared memory, longer lists in
// place in global memory; all by the same bitonic network whose every step moves the smaller
// element to the lower index, so indices past the list's end act as +infinity and are skipped.

constexpr int kSortThreads = 256;
constexpr int kSortCap = 4096;

__device__ __forceinline__ uint32_t refKey(uint32_t v) { return v & 0x0fffffffu; }

// Partner of index i in step (k, j) of the network (merge size k, stride j): the first step of
// each merge pairs i with its mirror in the k-block, the later ones with i ^ j.
__device__ __forceinline__ int bitonicPartner(int i, int k, int j) { return j == (k >> 1) ? i ^ (k - 1) : i ^ j; }

template <class Src> __global__ void __launch_bounds__(kSortThreads, 4) binSortKernel(Src src) {
	__shared__ uint32_t s_v[kSortCap];
	int cta, ncta;
	const FrameParams& p = src.get(cta, ncta);
	const int lane = threadIdx.x & 31;
	for(int bin = cta; bin < p.bin_count; bin += ncta) {
		for(int list = 0; list < 2; list++) {
			const uint32_t n = list == 0 ? binQuadCounts(p, bin) : binTriCounts(p, bin);
			const uint32_t off = list == 0 ? binQuadOffsets(p, bin) : binTriOffsets(p, bin);
			if(n <= 1u || uint64_t(off) + n > uint64_t(p.max_bin_refs))
				continue; // nothing to order, or the lists overflowed (error raised)
			uint32_t* d = (list == 0 ? p.bin_quads : p.bin_tris) + off;
			const int cnt = int(n);
			if(cnt <= 32) {
				if(threadIdx.x < 32) {
					uint32_t v = lane < cnt ? d[lane] : 0xffffffffu;
					for(int k = 2; k <= 32; k <<= 1)
						for(int j = k >> 1; j > 0; j >>= 1) {
							const int q = bitonicPartner(lane, k, j);
							const uint32_t o = __shfl_sync(0xffffffffu, v, q);
							const bool lower = lane < q;
							const bool swap = lower ? refKey(o) < refKey(v) : refKey(v) < refKey(o);
							v = swap ? o : v;
						}
					if(lane < cnt)
						d[lane] = v;
				}
			} else if(cnt <= kSortCap) {
				int P = 64;
				while(P < cnt)
					P <<= 1;
				for(int i = threadIdx.x; i < P; i += kSortThreads)
					s_v[i] = i < cnt ? d[i] : 0xffffffffu;
				__syncthreads();
				for(int k = 2; k <= P; k <<= 1)
					for(int j = k >> 1; j > 0; j >>= 1) {
						for(int i = threadIdx.x; i < P; i += kSortThreads) {
							const int q = bitonicPartner(i, k, j);
							if(q > i) {
								const uint32_t a = s_v[i], b = s_v[q];
								if(refKey(b) < refKey(a))
									s_v[i] = b, s_v[q] = a;
							}
						}
						__syncthreads();
					}
				for(int i = threadIdx.x; i < cnt; i += kSortThreads)
					d[i] = s_v[i];
			} else {
				int P = 1;
				while(P < cnt)
					P <<= 1;
				for(int k = 2; k <= P; k <<= 1)
					for(int j = k >> 1; j > 0; j >>= 1) {
						for(int i = threadIdx.x; i < cnt; i += kSortThreads) {
							const int q = bitonicPartner(i, k, j);
							if(q > i && q < cnt) {
								const uint32_t a = d[i], b = d[q];
								if(refKey(b) < refKey(a))
									d[i] = b, d[q] = a;
							}
						}
						__syncthreads();
					}
			}
			__syncthreads();
		}
	}
}

// ---------------------------------------------------------------------------------------------

cudaError_t configureBinningKernels() {
	// the counter and dispatcher keep one int per bin of the view in shared memory
	const int bytes = kMaxBinCount * int(sizeof(int));
	cudaError_t err;
	if((err = cudaFuncSetAttribute(binCountKernel<OneView>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) !=
		   cudaSuccess ||
	   (err = cudaFuncSetAttribute(binDispatchKernel<OneView>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) !=
		   cudaSuccess ||
	   (err = cudaFuncSetAttribute(binCountKernel<BatchViews>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) !=
		   cudaSuccess)
		return err;
	return cudaFuncSetAttribute(binDispatchKernel<BatchViews>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

void launchBinCount(const FrameParams& p, cudaStream_t stream) {
	binCountKernel<<<p.num_binning_ctas, kBinningThreads, p.bin_count * sizeof(int), stream>>>(OneView{p});
}
void launchBinCategorize(const FrameParams& p, cudaStream_t stream) {
	binCategorizeKernel<<<1, 1024, 0, stream>>>(OneView{p});
}
void launchBinDispatch(const FrameParams& p, cudaStream_t stream) {
	binDispatchKernel<<<p.num_binning_ctas, kBinningThreads, p.bin_count * sizeof(int), stream>>>(OneView{p});
	if(p.flags & LUCID_OPT_SORTED_BIN_LISTS)
		binSortKernel<<<p.bin_count, kSortThreads, 0, stream>>>(OneView{p});
}

void launchBinningBatch(const BatchViews& per_view, const BatchViews& binning_ctas, const BatchViews& bin_ctas,
						int max_bins, bool sorted_lists, cudaStream_t stream) {
	const int n = binning_ctas.cta_off[binning_ctas.num_views];
	const size_t smem = size_t(max_bins) * sizeof(int);
	binCountKernel<<<n, kBinningThreads, smem, stream>>>(binning_ctas);
	binCategorizeKernel<<<per_view.num_views, 1024, 0, stream>>>(per_view);
	binDispatchKernel<<<n, kBinningThreads, smem, stream>>>(binning_ctas);
	if(sorted_lists)
		binSortKernel<<<bin_ctas.cta_off[bin_ctas.num_views], kSortThreads, 0, stream>>>(bin_ctas);
}

} // namespace lucid
