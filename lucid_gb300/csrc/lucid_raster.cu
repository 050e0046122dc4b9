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
//     whose fragments, each pixel counted up to kWindow, fit kGroupBudget; a group ends at a
//     row boundary when it holds one.
//  C. Depth windows. A group whose pixels all have <= kHeavyPixel fragments is one window. In
//     a heavier group every pixel gets a coarse histogram of its depth keys (buckets of one
//     depth slab of the group's key range); a pixel's window is the run of buckets, from the
//     first one it has not processed, that holds >= kWindow fragments. Buckets split the key
//     space in order, so windows visit each pixel's fragments strictly front to back. A slab
//     covers about slab_target fragments per unfinished pixel (from an estimate gathered with
//     the group's key range); the next slab is counted only if a pixel needs it. The first
//     slab is generated directly: one pass over the band entries appends its fragments to
//     per-pixel regions of the idle sort buffer and counts each in its pixel's histogram, and
//     the first window is scattered from the regions (no second pass over the entries).
//  D. Per window: fragments (32-bit nearest-first depth key, 32-bit payload = pixel | tri) are
//     generated by one warp per pixel row (lane = pixel, band entries broadcast by shuffle) and
//     written to their pixel's segment, in a heavy group to the sub-segment of their depth
//     bucket. Sub-segments are sorted by key (one thread per small sub-segment with a register
//     network, grouped by size; one warp per larger one with a bitonic network; a block-wide
//     radix sort when one exceeds 256). Runs of equal depth are put in primitive-id order.
//     Shading runs in parallel batches from each tri's 48-byte shading record; one thread per
//     pixel blends front to back in FP32 (out += rgb*a*T; T *= 1-a, shading.glsl:279-280) and
//     stops once T == 0: no later fragment can change the pixel (it adds rgb*a*0). Background
//     is added last (shading.glsl:312).

#include "lucid_common.cuh"
#include "lucid_kernels.h"
#include "lucid_shade.cuh"

namespace lucid {

// Work counters of the depth-window path (diagnostics, off by default): built with
// LUCID_RASTER_COUNTERS=1 (lucid_gb300/build.py --counters) and run with LUCID_OPT_TIMERS, the
// kernel adds 24 64-bit counts into lucid_info.temp (read by lucid_gb300/profile_raster.py):
//  0 key-range entry visits      1 / 2 slab-histogram fragments evaluated / counted
//  3 / 4 window-generation fragments evaluated / kept   5 / 6 entries broadcast by 1-2 / 3-4
//  7 slabs built                 8 depth-window groups     9 direct slabs sent to the histogram
// 10 fragments shaded           11 windows               12 cycles of window selection (thread 0)
// 13 cycles of window generation (thread 0)              14 cycles of key ranges (thread 0)
// 15 cycles of the walk (thread 0)                       16 / 17 direct append: warp cycles
//    summed over warps / wall cycles (thread 0)          18 / 19 walk: warp cycles / wall cycles
#ifndef LUCID_RASTER_COUNTERS
#define LUCID_RASTER_COUNTERS 0
#endif
#if LUCID_RASTER_COUNTERS
#define RCOUNT(i, v) (rc[i] += (unsigned long long)(v))
#else
#define RCOUNT(i, v) ((void)0)
#endif

constexpr int RT = kRasterThreads;
constexpr int NW = RT / 32;
constexpr int kGroupCap = 8192;     // fragments per window (shared-memory sort capacity)
constexpr int kGroupPixels = 256;   // pixels per group (8-bit pixel index in the payload)
constexpr int kStage = 4096;        // shaded fragments per shading round (64 KB of float4)
constexpr int kShadeFirst = 128;    // fragments per pixel in a window's first shading round
constexpr int kShadeNext = 32;      // ... and in its later rounds
constexpr int kWindow = 160;        // target fragments per pixel per depth window
// a group with a pixel of more fragments is processed in depth windows: the histogram buckets
// split its pixels' lists into small sub-segments (cheap thread sorts instead of warp sorts of
// whole lists)
constexpr int kHeavyPixel = 32;
constexpr int kGroupBudget = 7680;  // sum over a group's pixels of min(count, kWindow)
constexpr int kHistWords = 8192;    // per-group depth histogram (pixels x buckets)
constexpr int kCoarseShift = 20;    // fragment estimate bins: depth keys >> 20 (4096 bins)
constexpr int kCoarseBins = 1 << (32 - kCoarseShift);
constexpr int kMaxSlabs = 64;       // depth slabs of one group at most
// light bins: each pass of a row keeps at most kLightPixel fragments per pixel, so they fit a
// warp's kLightPool-entry slice of the sort buffers
constexpr int kLightPixel = 32;
constexpr int kLightPool = 32 * kLightPixel;

struct RasterSmem {
	// kv[b][0] = keys, kv[b][1] = payloads of buffer b; the buffer not holding the sorted
	// fragments doubles as the 64 KB shading stage.
	uint32_t kv[2][2][kGroupCap];
	// per-(pixel, bucket) fragment counts; inside a window the counts of its buckets become
	// the sub-segment cursors
	uint32_t hist[kHistWords];
	uint32_t radix[256 * NW];
	int pix_count[1024];
	int eff_prefix[1025];
	int row_diff[32 * 33];
	float px_T[kGroupPixels];
	float px_c[kGroupPixels][3];
	int px_lo[kGroupPixels];     // first bucket not yet processed
	int px_cut[kGroupPixels];    // last bucket of the current window (-1: not in the window)
	int px_wbase[kGroupPixels];  // window segment start in the sort buffer
	int px_wend[kGroupPixels];   // window segment end (generation cursor of light groups)
	int px_wcnt[kGroupPixels];   // fragments of the pixel in the current window
	int px_bcur[kGroupPixels];   // blend cursor
	int px_done[kGroupPixels];   // fragments already processed (verification dump index)
	int px_state[kGroupPixels];  // 0 active, 1 finished
	int px_rend[kGroupPixels];   // fragments of the pixel's region of a directly generated slab
	int px_slot[kGroupPixels];   // shading round: blend cursor | fragments to shade << 16
	// sub-segments of the current window that need sorting, as (start << 16 | count):
	// counts 2..16 are sorted by one thread, by size class (2, 3-4, 5-8, 9-16; class 0 from the
	// front and class 2 from the back of sub_small, classes 1 and 3 likewise in `radix`, which
	// the window does not need unless it is radix sorted), 17..256 by one warp
	uint32_t sub_small[kGroupCap / 2];
	uint32_t sub_large[kGroupCap / 17 + 1];
	unsigned long long n_cls; // counts of the four size classes, 16 bits each
	int n_large;
	int band_count[8];
	int scan_tmp[NW + 1];
	uint32_t scan_tmpu[NW + 1];
	unsigned long long stat_hbt;
	unsigned long long store_base; // kRasterStore: first store slot of the bin
	uint32_t kmin, kmax;
	uint32_t group_frags;      // fragments of the current group's pixels
	uint32_t slab_lo, slab_hi; // depth slab whose keys the histogram holds
	int slab_next;             // index of the next slab
	int slab_first[kMaxSlabs]; // first estimate bin of every slab (INT_MAX: no such slab)
	int bin;
	int tile;        // 32x32 tile of a 64-pixel bin (0..3: x = tile & 1, y = tile >> 1)
	int group_end;
	int single_digit;
	int any_big;
	int bin_maxpx;   // most fragments of one pixel of the bin
	int view;        // view of the current bin (batched frames)
	int loaded_view; // view whose parameters view_params holds
	int store_ok;    // kRasterStore: the bin's fragments fit the store
	FrameParams view_params;
};

static_assert(sizeof(RasterSmem) <= 227 * 1024, "raster shared memory exceeds one SM");
static_assert(256 * NW == kGroupCap / 2, "the small sub-segment lists share the radix histograms' size");
static_assert(2 * NW * kLightPool <= 4 * kGroupCap, "the light path's row pools live in the sort buffers");

// Depth histogram slot of pixel t's bucket bk (2^nb_log >= 32 buckets per pixel). The bucket is
// XOR-swizzled by the pixel's lane so that the 32 pixels of a row, which mostly hit the same
// bucket of a planar triangle, fall into 32 different shared-memory banks.
// With 2^nb_log = 32 << g buckets per pixel, lane l of a pixel's warp owns buckets
// [l << g, (l + 1) << g): bucket bk sits in plane (bk & (2^g - 1)) of 32 words at column
// (bk >> g) ^ (t & 31), so a lane's buckets are conflict-free loads across the warp and the 32
// pixels of a row that hit one bucket still use 32 different banks.
__device__ __forceinline__ int histIdx(int t, int bk, int nb_log) {
	const int g = nb_log - 5;
	return (t << nb_log) | ((bk & ((1 << g) - 1)) << 5) | ((bk >> g) ^ (t & 31));
}

// A sub-segment of a window to sort: start relative to its pixel's window (13 bits), count
// (9 bits) and pixel of the group (8 bits).
__device__ __forceinline__ uint32_t segEntry(int rel, int cnt, int tp) {
	return uint32_t(rel) | uint32_t(cnt) << 13 | uint32_t(tp) << 22;
}
__device__ __forceinline__ int segCount(uint32_t e) { return int((e >> 13) & 0x1ffu); }
__device__ __forceinline__ int segPixel(uint32_t e) { return int(e >> 22); }
static_assert(kCoarseBins <= kHistWords, "the fragment estimate lives in the depth histogram");

size_t rasterSmemBytes() { return sizeof(RasterSmem); }
int rasterThreads() { return RT; }

__device__ __forceinline__ uint32_t entryTri(uint2 e) { return (e.x >> 20) | ((e.y >> 20) << 12); }

// A window fragment's payload: pixel of the group (8 bits) and tri (24 bits, the band entries'
// tri field).
__device__ __forceinline__ uint32_t fragPayload(int tp, uint32_t tri) { return uint32_t(tp) | (tri << 8); }
__device__ __forceinline__ uint32_t payloadTri(uint32_t val) { return val >> 8; }

// Verification dump: index of pixel (px, py), local pixel pl of `bin`, in the dump arrays, or
// -1 when it is not recorded. Whole frame: y * width + x; bin subset: slot * 1024 + pl.
__device__ __forceinline__ long long dumpPixel(const FrameParams& p, int bin, int pl, int px, int py) {
	if(px >= p.width || py >= p.height)
		return -1;
	if(p.dump_bin_slot) {
		const int slot = p.dump_bin_slot[bin];
		return slot < 0 ? -1 : (long long)slot * 1024 + pl;
	}
	return (long long)py * p.width + px;
}

__device__ __forceinline__ uint32_t fragPrim(const FrameParams& p, uint32_t val) {
	const uint32_t tri = payloadTri(val);
	return __ldg(p.quad_source + (tri >> 1)) * 2 + (tri & 1);
}

// Lanes of the warp (within `act`) whose 8-bit digit equals this lane's: 8 ballots, one per bit.
// Every lane of the warp must call it.
__device__ __forceinline__ uint32_t digitPeers(uint32_t d, uint32_t act) {
	uint32_t peers = act;
#pragma unroll
	for(int b = 0; b < 8; b++) {
		bool bit = (d >> b) & 1u;
		uint32_t m = __ballot_sync(0xffffffffu, bit);
		peers &= bit ? m : ~m;
	}
	return peers;
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
		uint32_t peers = digitPeers(d, act);
		if(valid && lane == __ffs(peers) - 1)
			s.radix[d * NW + warp] += __popc(peers);
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
		uint32_t peers = digitPeers(d, act);
		uint32_t pos = 0;
		if(valid)
			pos = s.radix[d * NW + warp] + __popc(peers & laneMaskLt());
		__syncwarp();
		if(valid && lane == __ffs(peers) - 1)
			s.radix[d * NW + warp] += __popc(peers);
		if(valid && pos < uint32_t(n)) {
			kout[pos] = k;
			vout[pos] = v;
		}
		__syncwarp();
	}
	__syncthreads();
	return true;
}

// Sorts (key, payload) pairs [base, base+n) of shared memory ascending by key with one warp:
// a bitonic network over 32*E registers (element i = e*32 + lane), padded with key 0xffffffff
// (never produced by nearFirstKey). Equal keys keep no particular order. Called by all lanes.
template <int E>
__device__ __forceinline__ void warpSortSegment(uint32_t* K, uint32_t* V, int base, int n) {
	const int lane = threadIdx.x & 31;
	uint32_t k[E], v[E];
#pragma unroll
	for(int e = 0; e < E; e++) {
		int i = e * 32 + lane;
		k[e] = i < n ? K[base + i] : 0xffffffffu;
		v[e] = i < n ? V[base + i] : 0u;
	}
#pragma unroll
	for(int kk = 2; kk <= 32 * E; kk <<= 1) {
#pragma unroll
		for(int j = kk >> 1; j > 0; j >>= 1) {
			if(j >= 32) {
#pragma unroll
				for(int e = 0; e < E; e++) {
					int e2 = e ^ (j >> 5);
					if(e2 > e) {
						bool up = ((e * 32 + lane) & kk) == 0;
						bool sw = up ? (k[e] > k[e2]) : (k[e] < k[e2]);
						uint32_t tk = sw ? k[e2] : k[e], tv = sw ? v[e2] : v[e];
						k[e2] = sw ? k[e] : k[e2], v[e2] = sw ? v[e] : v[e2];
						k[e] = tk, v[e] = tv;
					}
				}
			} else {
				const bool lower = (lane & j) == 0;
#pragma unroll
				for(int e = 0; e < E; e++) {
					uint32_t ok = __shfl_xor_sync(0xffffffffu, k[e], j);
					uint32_t ov = __shfl_xor_sync(0xffffffffu, v[e], j);
					bool up = ((e * 32 + lane) & kk) == 0;
					bool take = lower == up ? ok < k[e] : ok > k[e];
					k[e] = take ? ok : k[e];
					v[e] = take ? ov : v[e];
				}
			}
		}
	}
#pragma unroll
	for(int e = 0; e < E; e++) {
		int i = e * 32 + lane;
		if(i < n) {
			K[base + i] = k[e];
			V[base + i] = v[e];
		}
	}
}

// Sorts a small segment [base, base+n), n <= N, by one thread: bitonic network in registers.
template <int N>
__device__ __forceinline__ void threadSortSegment(uint32_t* K, uint32_t* V, int base, int n) {
	uint32_t k[N], v[N];
#pragma unroll
	for(int i = 0; i < N; i++) {
		k[i] = i < n ? K[base + i] : 0xffffffffu;
		v[i] = i < n ? V[base + i] : 0u;
	}
#pragma unroll
	for(int kk = 2; kk <= N; kk <<= 1) {
#pragma unroll
		for(int j = kk >> 1; j > 0; j >>= 1) {
#pragma unroll
			for(int i = 0; i < N; i++) {
				int l = i ^ j;
				if(l > i) {
					bool up = (i & kk) == 0;
					bool sw = up ? (k[i] > k[l]) : (k[i] < k[l]);
					uint32_t tk = sw ? k[l] : k[i], tv = sw ? v[l] : v[i];
					k[l] = sw ? k[i] : k[l], v[l] = sw ? v[i] : v[l];
					k[i] = tk, v[i] = tv;
				}
			}
		}
	}
#pragma unroll
	for(int i = 0; i < N; i++)
		if(i < n) {
			K[base + i] = k[i];
			V[base + i] = v[i];
		}
}

__device__ void writePixel(const FrameParams& p, int px, int py, float4 c) {
	if(px < p.width && py < p.height)
		reinterpret_cast<float4*>(p.out_rgba)[size_t(py) * p.width + px] = c;
}

// ne * k / d for 0 <= k <= d <= 16 (a warp's slice of a band's entries) in 32-bit arithmetic
// while ne * k fits, instead of a 64-bit division
__device__ __forceinline__ int sliceBound(int ne, int k, int d) {
	return ne < (1 << 28) ? int((uint32_t(ne) * uint32_t(k)) / uint32_t(d)) : int((int64_t(ne) * k) / d);
}

// Visits every fragment of pixels [p0, p1) of the bin: fn(t, key, tri) with t the pixel
// index inside the group, called by the lane owning pixel t. Warps are assigned to the group's
// rows (lane = pixel column) and split a row's band entries; entries are loaded 32 at a time
// (one per lane) and broadcast by shuffle. The key is evaluated exactly as in the oracle
// (shading.glsl:116): dx * px + (dy * py + dz).
//
// With `ekeys` (the entries' depth-key ranges over the group, written by the histogram pass)
// only entries whose range meets the current window of some pixel of the row are visited; the
// window of pixel t holds the keys of its buckets [px_lo, px_cut] (bucket = (key - kmin) >> shift).
// With `ekeys` and flo <= fhi, entries are culled against the fixed key range [flo, fhi] instead.
template <bool kQuad = false, int U = 4, typename Fn>
__device__ __forceinline__ void forEachGroupFragment(const FrameParams& p, const RasterSmem& s,
													  const uint2* scratch, const float4* planes, int band_cap, int bin_x,
													  int bin_y, int p0, int p1, Fn fn,
													  const uint2* ekeys = nullptr, uint32_t kmin = 0u,
													  int shift = 0, uint32_t flo = 1u, uint32_t fhi = 0u,
													  unsigned long long* ecount = nullptr) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int r0 = p0 >> 5, r1 = (p1 - 1) >> 5;
	const int nrows = r1 - r0 + 1;
	const int per_row = NW / nrows; // >= 1: a group spans at most 9 rows
	if(warp >= per_row * nrows)
		return;
	const int row = r0 + warp / per_row, slice = warp % per_row;
	const int b = row >> 2, rshift = 5 * (row & 3);
	const int ne = s.band_count[b];
	const int jbeg = sliceBound(ne, slice, per_row), jend = sliceBound(ne, slice + 1, per_row);
	const int pix = row * 32 + lane;
	const bool in_group = pix >= p0 && pix < p1;
	const int t = pix - p0;
	const float fx = float(bin_x + lane), fy = float(bin_y + row);
	uint32_t wlo = 0u, whi = 0xffffffffu;
	if(ekeys && flo <= fhi) {
		wlo = flo, whi = fhi;
	} else if(ekeys) {
		uint32_t lo_k = 0xffffffffu, hi_k = 0u;
		if(in_group && s.px_cut[t] >= 0) {
			const unsigned long long a = (unsigned long long)kmin + ((unsigned long long)s.px_lo[t] << shift);
			const unsigned long long z = (unsigned long long)kmin + ((unsigned long long)(s.px_cut[t] + 1) << shift) - 1ull;
			lo_k = uint32_t(a < 0xffffffffull ? a : 0xffffffffull);
			hi_k = uint32_t(z < 0xffffffffull ? z : 0xffffffffull);
		}
#pragma unroll
		for(int o = 16; o > 0; o >>= 1) {
			lo_k = min(lo_k, __shfl_xor_sync(0xffffffffu, lo_k, o));
			hi_k = max(hi_k, __shfl_xor_sync(0xffffffffu, hi_k, o));
		}
		if(lo_k > hi_k)
			return; // no pixel of this row takes part in the window
		wlo = lo_k, whi = hi_k;
	}
	// the group's columns in this row
	const int glo = max(0, p0 - 32 * row), ghi = min(31, p1 - 1 - 32 * row);
	// lane j's entry, its key range and plane are loaded together, and the next chunk's while
	// this one is processed
	const size_t bbase = size_t(b) * band_cap;
	uint2 n_e = make_uint2(0u, 0u), n_kr = make_uint2(0u, 0xffffffffu);
	float4 n_d = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	if(jbeg + lane < jend) {
		n_e = scratch[bbase + jbeg + lane];
		n_d = planes[bbase + jbeg + lane];
		if(ekeys)
			n_kr = ekeys[bbase + jbeg + lane];
	}
	for(int j0 = jbeg; j0 < jend; j0 += 32) {
		// lane j's entry: its span in this row, its tri and the row's part of its plane
		// (dy * py + dz, the same for every pixel of the row); only entries whose span meets
		// the group's columns take part
		const int j = j0 + lane;
		bool rel = j < jend;
		const uint2 e = n_e, kr = n_kr;
		const float4 d = n_d;
		if(j + 32 < jend) {
			n_e = scratch[bbase + j + 32];
			n_d = planes[bbase + j + 32];
			if(ekeys)
				n_kr = ekeys[bbase + j + 32];
		}
		if(rel && ekeys)
			rel = kr.y >= wlo && kr.x <= whi;
		uint32_t span = 0u, tri = 0u;
		float dx = 0.0f, ty = 0.0f;
		if(rel) {
			const int lo = (e.x >> rshift) & 31, hi = (e.y >> rshift) & 31;
			rel = max(lo, glo) <= min(hi, ghi);
			if(rel) {
				tri = entryTri(e);
				dx = d.x;
				ty = d.y * fy + d.z;
				span = uint32_t(lo) | uint32_t(hi) << 5;
			}
		}
		// up to four entries per step (in lane order), so that their shuffles, key evaluations and
		// the callbacks' shared-memory round trips overlap
		uint32_t todo = __ballot_sync(0xffffffffu, rel);
		if(LUCID_RASTER_COUNTERS && ecount && lane == 0)
			*ecount += __popc(todo);
		while(todo != 0u) {
			int k[U];
			bool has[U];
#pragma unroll
			for(int u = 0; u < U; u++) {
				has[u] = todo != 0u;
				k[u] = has[u] ? __ffs(todo) - 1 : 0;
				if(has[u])
					todo &= todo - 1u;
			}
			uint32_t sp[U], tr[U], key[U];
			float kdx[U], kty[U];
#pragma unroll
			for(int u = 0; u < U; u++) {
				sp[u] = __shfl_sync(0xffffffffu, span, k[u]);
				kdx[u] = __shfl_sync(0xffffffffu, dx, k[u]);
				kty[u] = __shfl_sync(0xffffffffu, ty, k[u]);
				tr[u] = __shfl_sync(0xffffffffu, tri, k[u]);
			}
#pragma unroll
			for(int u = 0; u < U; u++)
				key[u] = nearFirstKey(kdx[u] * fx + kty[u]);
			if constexpr(kQuad) {
				// the U entries' fragments of this lane in one call (the callback can issue
				// their shared-memory atomics back to back)
				bool on[U];
#pragma unroll
				for(int u = 0; u < U; u++)
					on[u] = has[u] && in_group && lane >= int(sp[u] & 31u) && lane <= int(sp[u] >> 5);
				fn(t, on, key, tr);
			} else {
#pragma unroll
				for(int u = 0; u < U; u++)
					if(has[u] && in_group && lane >= int(sp[u] & 31u) && lane <= int(sp[u] >> 5))
						fn(t, key[u], tr[u]);
			}
		}
	}
}

// forEachGroupFragment's four-entry mode with the row's relevant entries staged in shared memory:
// a warp compacts the entries of its slice that take part (span in the group's columns, key range
// meeting [flo, fhi] when `ekeys` is given) into its kStageEntries-entry area of `stage`, up to
// kStageEntries at a time, then every lane reads them four per step with broadcast loads (one
// 16-byte load per entry instead of four shuffles). fn(t, on[4], key[4], tri[4]).
constexpr int kStageEntries = 256;
static_assert(NW * kStageEntries * 16 <= 2 * kGroupCap * 4, "the staged entries live in one sort buffer");
template <typename Fn>
__device__ __forceinline__ void forEachGroupFragmentStaged(const FrameParams& p, const RasterSmem& s,
														   const uint2* scratch, const float4* planes, int band_cap,
														   int bin_x, int bin_y, int p0, int p1, Fn fn, uint4* stage,
														   const uint2* ekeys, uint32_t flo, uint32_t fhi) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int r0 = p0 >> 5, r1 = (p1 - 1) >> 5;
	const int nrows = r1 - r0 + 1;
	const int per_row = NW / nrows;
	if(warp >= per_row * nrows)
		return;
	const int row = r0 + warp / per_row, slice = warp % per_row;
	const int b = row >> 2, rshift = 5 * (row & 3);
	const int ne = s.band_count[b];
	const int jbeg = sliceBound(ne, slice, per_row), jend = sliceBound(ne, slice + 1, per_row);
	const int pix = row * 32 + lane;
	const bool in_group = pix >= p0 && pix < p1;
	const int t = pix - p0;
	const float fx = float(bin_x + lane), fy = float(bin_y + row);
	const int glo = max(0, p0 - 32 * row), ghi = min(31, p1 - 1 - 32 * row);
	const uint32_t lt = laneMaskLt();
	uint4* ws = stage + warp * kStageEntries;
	const size_t bbase = size_t(b) * band_cap;
	uint2 n_e = make_uint2(0u, 0u), n_kr = make_uint2(0u, 0xffffffffu);
	float4 n_d = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	if(jbeg + lane < jend) {
		n_e = scratch[bbase + jbeg + lane];
		n_d = planes[bbase + jbeg + lane];
		if(ekeys)
			n_kr = ekeys[bbase + jbeg + lane];
	}
	for(int s0 = jbeg; s0 < jend; s0 += kStageEntries) {
		const int s1 = min(s0 + kStageEntries, jend);
		int n = 0;
		for(int j0 = s0; j0 < s1; j0 += 32) {
			const int j = j0 + lane;
			bool rel = j < s1;
			const uint2 e = n_e, kr = n_kr;
			const float4 d = n_d;
			if(j + 32 < jend) {
				n_e = scratch[bbase + j + 32];
				n_d = planes[bbase + j + 32];
				if(ekeys)
					n_kr = ekeys[bbase + j + 32];
			}
			if(rel && ekeys)
				rel = kr.y >= flo && kr.x <= fhi;
			const int lo = (e.x >> rshift) & 31, hi = (e.y >> rshift) & 31;
			rel = rel && max(lo, glo) <= min(hi, ghi);
			const uint32_t m = __ballot_sync(0xffffffffu, rel);
			if(rel)
				ws[n + __popc(m & lt)] = make_uint4(uint32_t(lo) | uint32_t(hi) << 5, entryTri(e),
													__float_as_uint(d.x), __float_as_uint(d.y * fy + d.z));
			n += __popc(m);
		}
		__syncwarp();
		for(int i = 0; i < n; i += 4) {
			bool on[4];
			uint32_t key[4], tr[4];
#pragma unroll
			for(int u = 0; u < 4; u++) {
				const bool has = i + u < n;
				const uint4 q = ws[has ? i + u : i];
				key[u] = nearFirstKey(__uint_as_float(q.z) * fx + __uint_as_float(q.w));
				tr[u] = q.y;
				on[u] = has && in_group && lane >= int(q.x & 31u) && lane <= int(q.x >> 5);
			}
			fn(t, on, key, tr);
		}
		__syncwarp();
	}
}

// Input primitive id of a tri slot (ties between equal depth keys go by it).
__device__ __forceinline__ uint32_t triPrim(const FrameParams& p, uint32_t tri) {
	return __ldg(p.quad_source + (tri >> 1)) * 2 + (tri & 1);
}

// (key, prim) order of two fragments of one pixel: nearest first, equal keys by input primitive
// id (looked up only for equal keys; a tri covers a pixel once, so the order is strict).
__device__ __forceinline__ bool fragBefore(const FrameParams& p, uint32_t ka, uint32_t ta, uint32_t kb, uint32_t tb) {
	return ka < kb || (ka == kb && triPrim(p, ta) < triPrim(p, tb));
}

// One row of a light bin, by one warp (lane = pixel column). In each pass every lane gathers,
// from the band entries of the row, the nearest min(count, kLightPixel) fragments of its pixel
// behind the last fragment it has blended (all of them when the pixel has no more) into its
// slots of the warp's pool (K: depth keys, V: tri slots), then blends them front to back,
// taking the nearest remaining one each step, and stops once T == 0: nothing behind that point
// is ordered or shaded. A pixel with more fragments than slots whose T is still above 0 takes
// another pass. Keys, shading and blend are the FP32 expressions of the group path
// (shading.glsl:116, :279-280, :312). Returns the fragments the lane blended.
// A row whose pixels all fit their slots (the common case) is gathered with lane = band entry
// instead: each lane walks its entry's span in the row and appends the fragments to their
// pixels through per-pixel cursors (`cursor`, 32 ints of the warp), so that every lane does
// useful work; the order inside a pixel's slots does not matter, the blend selects by
// (key, prim).
__device__ unsigned long long lightRow(const FrameParams& p, const RasterSmem& s, const uint2* scratch,
									   const float4* planes, int band_cap, int bin, int bin_x, int bin_y, int row,
									   uint32_t* K, uint32_t* V, int* cursor, float4 bg, bool additive,
									   bool alpha_threshold, bool dump, long long* tacc) {
	const int lane = threadIdx.x & 31;
	long long t0 = tacc ? clock64() : 0;
	const int pl = row * 32 + lane;
	const int cnt = s.pix_count[pl];
	const int cap = min(cnt, kLightPixel);
	const int off = warpInclusiveScan(cap) - cap;
	const int px = bin_x + lane, py = bin_y + row;
	const float fx = float(px), fy = float(py);
	const int b = row >> 2, rshift = 5 * (row & 3);
	const int ne = s.band_count[b];
	float T = 1.0f, c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
	int k = 0, remaining = cnt;
	bool have_thr = false; // the last blended fragment: later passes gather what lies behind it
	uint32_t thr_key = 0u, thr_tri = 0u;
	bool done = cnt == 0;
	const long long dbase = dump ? dumpPixel(p, bin, pl, px, py) : -1;
	int row_max = cnt;
#pragma unroll
	for(int o = 16; o > 0; o >>= 1)
		row_max = max(row_max, __shfl_xor_sync(0xffffffffu, row_max, o));
	bool single = row_max <= kLightPixel; // one pass gathers every fragment of the row
	while(__any_sync(0xffffffffu, !done)) {
		// A. the pass's fragments from the band entries (spans already clipped to the viewport)
		const bool want = !done;
		const bool bounded = remaining > cap; // keep only the nearest `cap`
		int size = 0, maxi = 0;
		uint32_t maxk = 0u, maxt = 0u;
		if(single) {
			cursor[lane] = off;
			__syncwarp();
			for(int j = lane; j < ne; j += 32) {
				const uint2 e = scratch[size_t(b) * band_cap + j];
				const int lo = (e.x >> rshift) & 31, hi = (e.y >> rshift) & 31;
				if(lo > hi)
					continue;
				const float4 d = planes[size_t(b) * band_cap + j];
				const uint32_t t = entryTri(e);
				const float ty = d.y * fy + d.z;
				int x = lo;
				// four cursors reserved before any of their stores: the atomics' latencies overlap
				for(; x + 3 <= hi; x += 4) {
					uint32_t key[4];
					int pos[4];
#pragma unroll
					for(int u = 0; u < 4; u++)
						key[u] = nearFirstKey(d.x * float(bin_x + x + u) + ty);
#pragma unroll
					for(int u = 0; u < 4; u++)
						pos[u] = atomicAdd(&cursor[x + u], 1);
#pragma unroll
					for(int u = 0; u < 4; u++)
						if(pos[u] < kLightPool) {
							K[pos[u]] = key[u];
							V[pos[u]] = t;
						}
				}
				for(; x <= hi; x++) {
					const uint32_t key = nearFirstKey(d.x * float(bin_x + x) + ty);
					const int pos = atomicAdd(&cursor[x], 1);
					if(pos < kLightPool) {
						K[pos] = key;
						V[pos] = t;
					}
				}
			}
			__syncwarp();
			size = cursor[lane] - off;
			__syncwarp();
			single = false;
		} else
		for(int j0 = 0; j0 < ne; j0 += 32) {
			const int j = j0 + lane;
			bool rel = j < ne;
			uint32_t span = 0u, tri = 0u;
			float dx = 0.0f, ty = 0.0f;
			if(rel) {
				const uint2 e = scratch[size_t(b) * band_cap + j];
				const int lo = (e.x >> rshift) & 31, hi = (e.y >> rshift) & 31;
				rel = lo <= hi;
				if(rel) {
					const float4 d = planes[size_t(b) * band_cap + j];
					tri = entryTri(e);
					dx = d.x;
					ty = d.y * fy + d.z;
					span = uint32_t(lo) | uint32_t(hi) << 5;
				}
			}
			uint32_t todo = __ballot_sync(0xffffffffu, rel);
			while(todo != 0u) {
				int kk[4];
				bool has[4];
#pragma unroll
				for(int u = 0; u < 4; u++) {
					has[u] = todo != 0u;
					kk[u] = has[u] ? __ffs(todo) - 1 : 0;
					if(has[u])
						todo &= todo - 1u;
				}
				uint32_t sp[4], tr[4];
				float kdx[4], kty[4];
#pragma unroll
				for(int u = 0; u < 4; u++) {
					sp[u] = __shfl_sync(0xffffffffu, span, kk[u]);
					kdx[u] = __shfl_sync(0xffffffffu, dx, kk[u]);
					kty[u] = __shfl_sync(0xffffffffu, ty, kk[u]);
					tr[u] = __shfl_sync(0xffffffffu, tri, kk[u]);
				}
#pragma unroll
				for(int u = 0; u < 4; u++) {
					if(!(want && has[u] && lane >= int(sp[u] & 31u) && lane <= int(sp[u] >> 5)))
						continue;
					const uint32_t key = nearFirstKey(kdx[u] * fx + kty[u]), t = tr[u];
					if(have_thr && !fragBefore(p, thr_key, thr_tri, key, t))
						continue; // blended in an earlier pass
					if(size < cap) {
						K[off + size] = key;
						V[off + size] = t;
						if(bounded && (size == 0 || fragBefore(p, maxk, maxt, key, t)))
							maxk = key, maxt = t, maxi = size;
						size++;
					} else if(fragBefore(p, key, t, maxk, maxt)) {
						// full: the new fragment replaces the farthest one kept
						K[off + maxi] = key;
						V[off + maxi] = t;
						// the farthest kept fragment: the largest key without a branch per element,
						// equal keys (rare) by the larger input primitive id in a second scan
						maxi = 0, maxk = K[off];
						bool tie = false;
						for(int i = 1; i < cap; i++) {
							const uint32_t ki = K[off + i];
							const bool gt = ki > maxk;
							tie = gt ? false : (tie || ki == maxk);
							maxi = gt ? i : maxi;
							maxk = gt ? ki : maxk;
						}
						maxt = V[off + maxi];
						if(tie) {
							uint32_t bp = triPrim(p, maxt);
							for(int i = 0; i < cap; i++)
								if(K[off + i] == maxk && i != maxi) {
									const uint32_t pi = triPrim(p, V[off + i]);
									if(pi > bp)
										maxi = i, bp = pi, maxt = V[off + i];
								}
						}
					}
				}
			}
		}
		__syncwarp();
		if(tacc && lane == 0) {
			const long long t1 = clock64();
			tacc[3] += t1 - t0;
			t0 = t1;
		}
		if(want && size != min(remaining, cap)) {
			raiseError(p.info, LUCID_ERR_BIN_COUNT, uint32_t(bin), uint32_t(pl), uint32_t(size));
			done = true;
		}
		// B. front-to-back blend by selection; the next fragment's shading record is loaded while
		// the current one is shaded
		int n = want && !done ? size : 0;
		auto take = [&](uint32_t& key, uint32_t& tri) {
			int bi = off;
			key = K[off];
			// the nearest key without a branch per element; equal keys (rare) are then ordered by
			// input primitive id in a second scan
			bool tie = false;
			for(int i = off + 1; i < off + n; i++) {
				const uint32_t ki = K[i];
				const bool lt = ki < key;
				tie = lt ? false : (tie || ki == key);
				bi = lt ? i : bi;
				key = lt ? ki : key;
			}
			if(tie) {
				uint32_t bp = triPrim(p, V[bi]);
				for(int i = off; i < off + n; i++)
					if(K[i] == key && i != bi) {
						const uint32_t pi = triPrim(p, V[i]);
						if(pi < bp)
							bi = i, bp = pi;
					}
			}
			tri = V[bi];
			K[bi] = K[off + n - 1];
			V[bi] = V[off + n - 1];
			n--;
		};
		bool stop = false;
		if(n > 0) {
			uint32_t ck, ct;
			take(ck, ct);
			ShadeRec cr = loadShadeRec(p, ct);
			while(true) {
				uint32_t nk = 0u, nt = 0u;
				ShadeRec nr;
				const bool more = n > 0;
				if(more) {
					take(nk, nt);
					nr = loadShadeRec(p, nt);
				}
				const float4 c = shadeCoreRec(p, ct, cr, keyToDepth(ck), px, py).col;
				if(dbase >= 0 && k < p.dump_max)
					p.dump_prims[size_t(dbase) * p.dump_max + k] = int(triPrim(p, ct));
				k++;
				remaining--;
				have_thr = true, thr_key = ck, thr_tri = ct;
				const float qx = c.x * c.w, qy = c.y * c.w, qz = c.z * c.w;
				if(additive) {
					c0 = c0 + qx;
					c1 = c1 + qy;
					c2 = c2 + qz;
				} else {
					c0 = c0 + qx * T;
					c1 = c1 + qy * T;
					c2 = c2 + qz * T;
					T = T * (1.0f - c.w);
					if((T == 0.0f && !dump) || (alpha_threshold && T < (1.0f / 128.0f))) {
						stop = true;
						break;
					}
				}
				if(!more)
					break;
				ck = nk, ct = nt, cr = nr;
			}
		}
		if(want)
			done = done || stop || remaining == 0;
		if(tacc && lane == 0) {
			const long long t1 = clock64();
			tacc[5] += t1 - t0;
			t0 = t1;
		}
	}
	float4 o;
	o.x = fminf(fmaxf(c0 + T * bg.x, 0.0f), 1.0f);
	o.y = fminf(fmaxf(c1 + T * bg.y, 0.0f), 1.0f);
	o.z = fminf(fmaxf(c2 + T * bg.z, 0.0f), 1.0f);
	o.w = 1.0f;
	writePixel(p, px, py, o);
	if(dbase >= 0)
		p.dump_counts[dbase] = cnt;
	__syncwarp();
	return (unsigned long long)k;
}

// Work sources of the raster kernel: the bins of one frame, or the bins of every view of a
// batched frame.
struct OneViewWork {
	FrameParams p;
	__device__ __forceinline__ const FrameParams& first() const { return p; }
	__device__ __forceinline__ lucid_info* timerInfo() const { return p.info; }
	// thread 0: next tile of the work list (the bins HIGH, LOW, EMPTY, each as its tiles: one
	// for 32-pixel bins, four for 64-pixel bins), bin -1 when done
	__device__ __forceinline__ void next(RasterSmem& s) const {
		const int tsh = 2 * (p.bin_shift - kBinShift);
		const uint32_t w = atomicAdd(&p.info->raster_work_counter, 1u);
		s.bin = w < (uint32_t(p.bin_count) << tsh) ? int(p.raster_work[w >> tsh]) : -1;
		s.tile = int(w & ((1u << tsh) - 1u));
		s.view = 0;
	}
	__device__ __forceinline__ const FrameParams& view(RasterSmem&) const { return p; }
};

// All views' HIGH bins are handed out first (view by view), then the LOW bins, then the EMPTY
// ones, so the heaviest bins of every view start early.
struct BatchWork {
	const FrameParams* views;
	int num_views;
	uint32_t* counter;       // work items handed out
	const int* level_prefix; // [3][num_views + 1] bins of each level (HIGH, LOW, EMPTY) before view v
	__device__ __forceinline__ const FrameParams& first() const { return views[0]; }
	__device__ __forceinline__ lucid_info* timerInfo() const { return nullptr; }
	__device__ __forceinline__ void next(RasterSmem& s) const {
		const int w = int(atomicAdd(counter, 1u));
		const int nv1 = num_views + 1;
		int bin = -1, view = -1, tile = 0, base = 0;
		for(int L = 0; L < 3; L++) {
			const int* pre = level_prefix + L * nv1;
			const int n = pre[num_views];
			if(w < base + n) {
				const int j = w - base;
				int lo = 0, hi = num_views - 1;
				while(lo < hi) {
					int mid = (lo + hi + 1) >> 1;
					if(pre[mid] <= j)
						lo = mid;
					else
						hi = mid - 1;
				}
				// the prefixes count tiles (1 or 4 per bin of the view)
				const int tsh = 2 * (views[lo].bin_shift - kBinShift);
				const int* ph = level_prefix, *pl = level_prefix + nv1;
				const int nhigh = (ph[lo + 1] - ph[lo]) >> tsh, nlow = (pl[lo + 1] - pl[lo]) >> tsh;
				const int k = j - pre[lo];
				const int kb = k >> tsh;
				const int pos = L == 0 ? kb : L == 1 ? nhigh + kb : nhigh + nlow + kb;
				view = lo;
				tile = k & ((1 << tsh) - 1);
				bin = int(views[lo].raster_work[pos]);
				break;
			}
			base += n;
		}
		s.bin = bin;
		s.tile = tile;
		s.view = view;
	}
	// called by every thread after the barrier that follows next()
	__device__ __forceinline__ const FrameParams& view(RasterSmem& s) const {
		if(s.view != s.loaded_view) {
			const uint32_t* src = reinterpret_cast<const uint32_t*>(views + s.view);
			uint32_t* dst = reinterpret_cast<uint32_t*>(&s.view_params);
			for(int i = threadIdx.x; i < int(sizeof(FrameParams) / 4); i += blockDim.x)
				dst[i] = src[i];
			__syncthreads();
			if(threadIdx.x == 0)
				s.loaded_view = s.view;
		}
		return s.view_params;
	}
};

template <int MODE, class Work>
__global__ void __launch_bounds__(RT, 1) rasterKernel(Work work) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	RasterSmem& s = *reinterpret_cast<RasterSmem*>(smem_raw);
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	// band scratch, its capacity and the option flags are the renderer's, shared by all views
	const FrameParams& p_first = work.first();
	const int band_cap = p_first.band_capacity;
	uint2* scratch = p_first.band_scratch + size_t(blockIdx.x) * 8 * band_cap;
	uint2* ekeys = p_first.band_keys + size_t(blockIdx.x) * 8 * band_cap;
	float4* planes = p_first.band_planes + size_t(blockIdx.x) * 8 * band_cap;
	const uint32_t opt_flags = p_first.flags;
	const bool additive = (opt_flags & LUCID_OPT_ADDITIVE_BLENDING) != 0;
	const bool alpha_threshold = (opt_flags & LUCID_OPT_ALPHA_THRESHOLD) != 0;
	if(tid == 0)
		s.loaded_view = -1;
	// with a fragment store (differentiable frames, pixel-parallel blend) the other modes run
	// only when the store overflowed; otherwise the pixel-parallel kernels do the work
	if constexpr(MODE != kRasterStore) {
		if(p_first.grad_state && *reinterpret_cast<volatile unsigned long long*>(p_first.grad_state) == 0ull)
			return;
	}
	// Section timers (timers.glsl:9-39): thread 0 accumulates clock64 deltas between the
	// CTA-wide barriers that separate the phases; units of 256 cycles in lucid_info.raster_timers:
	// 0 row spans, 1 counts, 2 depth histograms, 3 window fragments, 4 sort, 5 shading,
	// 6 blending, 7 output and bin fetch. Light bins: 3 fragments and 5 blend of warp 0's rows,
	// 6 the wait for the other warps.
	lucid_info* const timer_info = work.timerInfo();
	const bool timers = (opt_flags & LUCID_OPT_TIMERS) != 0 && timer_info != nullptr;
	long long tacc[8] = {0, 0, 0, 0, 0, 0, 0, 0}, tlast = timers ? clock64() : 0;
#if LUCID_RASTER_COUNTERS
	unsigned long long rc[24] = {};
	long long tc2 = 0;
#endif
#define RASTER_TIMER(i)                                                                            \
	do {                                                                                           \
		if(timers && tid == 0) {                                                                   \
			long long now__ = clock64();                                                           \
			tacc[i] += now__ - tlast;                                                              \
			tlast = now__;                                                                         \
		}                                                                                          \
	} while(0)

	while(true) {
		if(tid == 0) {
			work.next(s);
			s.stat_hbt = 0;
			s.bin_maxpx = 0;
		}
		if(tid < 8)
			s.band_count[tid] = 0;
		for(int i = tid; i < 32 * 33; i += RT)
			s.row_diff[i] = 0;
		__syncthreads();
		RASTER_TIMER(7);
		const int bin = s.bin;
		if(bin < 0)
			break;
		const FrameParams& p = work.view(s);
		const float4 bg = make_float4(p.cfg.background_color[0], p.cfg.background_color[1],
									  p.cfg.background_color[2], p.cfg.background_color[3]);
		const bool dump = p.dump_counts != nullptr;
		// the tile's origin: bins of 1 << bin_shift pixels, rastered as 32x32 tiles
		const int bx = bin % p.bin_count_x, by = bin / p.bin_count_x;
		const int tiled = p.bin_shift > kBinShift;
		const int bin_x = (bx << p.bin_shift) + (s.tile & 1) * kBinSize;
		const int bin_y = (by << p.bin_shift) + (s.tile >> 1) * kBinSize;
		const int vis_w = p.width - bin_x, vis_h = p.height - bin_y;
		if(vis_w <= 0 || vis_h <= 0) {
			__syncthreads(); // every thread has read this item before thread 0 fetches the next
			continue;
		}
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
			if(tiled) {
				// a 64-pixel bin's lists hold tris of all four tiles: keep those whose quad's
				// 32-pixel bin AABB (setup's) holds this tile
				int x0, y0, x1, y1;
				decodeAABB28(__ldg(p.quad_aabbs + (tri >> 1)), x0, y0, x1, y1);
				const int tx = bin_x >> kBinShift, ty = bin_y >> kBinShift;
				if(tx < x0 || tx > x1 || ty < y0 || ty > y1)
					continue;
			}
			uint4 r0 = __ldg(p.tri_scan + size_t(tri) * 2);
			uint4 r1 = __ldg(p.tri_scan + size_t(tri) * 2 + 1);
			const uint4 dq = __ldg(p.tri_depth + tri);
			const float4 plane = make_float4(bitsf(dq.x), bitsf(dq.y), bitsf(dq.z), 0.0f);
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
					if(slot < band_cap) {
						scratch[size_t(band) * band_cap + slot] =
							make_uint2(minb | ((tri & 0xfffu) << 20), maxb | ((tri >> 12) << 20));
						planes[size_t(band) * band_cap + slot] = plane;
					}
				}
			}
		}
#pragma unroll
		for(int o = 16; o > 0; o >>= 1)
			hbt += __shfl_xor_sync(0xffffffffu, hbt, o);
		if(lane == 0 && hbt)
			atomicAdd(&s.stat_hbt, hbt);
		__syncthreads();
		RASTER_TIMER(0);
		bool overflow = !lists_ok;
		for(int b = 0; b < 8; b++)
			overflow |= s.band_count[b] > band_cap;
		if(overflow) {
			if(tid == 0 && lists_ok)
				raiseError(p.info, LUCID_ERR_BAND_ENTRIES, uint32_t(bin), 0, uint32_t(band_cap));
			for(int i = tid; i < 1024; i += RT)
				writePixel(p, bin_x + (i & 31), bin_y + (i >> 5), make_float4(1.0f, 0.0f, 0.0f, 1.0f));
			__syncthreads();
			continue;
		}

		// ---- B. per-pixel counts; prefix of min(count, kWindow) for the groups
		for(int row = warp; row < 32; row += NW) {
			int v = s.row_diff[row * 33 + lane];
			s.pix_count[row * 32 + lane] = warpInclusiveScan(v);
		}
		__syncthreads();
		{
			int c0 = s.pix_count[2 * tid], c1 = s.pix_count[2 * tid + 1];
			int e0 = min(c0, kWindow), e1 = min(c1, kWindow);
			int total;
			int off = blockExclusiveScan(e0 + e1, s.scan_tmp, &total);
			s.eff_prefix[2 * tid] = off;
			s.eff_prefix[2 * tid + 1] = off + e0;
			if(tid == 0)
				s.eff_prefix[1024] = total;
			int frags;
			const int foff = blockExclusiveScan(c0 + c1, s.scan_tmp, &frags);
			if constexpr(MODE == kRasterStore) {
				// the bin's slice of the fragment store; per pixel its offset and count
				if(tid == 0) {
					unsigned long long base = atomicAdd(&p.grad_state[1], (unsigned long long)frags);
					s.store_ok = base + (unsigned long long)frags <= p.grad_capacity;
					if(!s.store_ok)
						atomicExch(&p.grad_state[0], 1ull);
					s.store_base = base;
				}
				__syncthreads();
				if(s.store_ok) {
					const uint32_t base = uint32_t(s.store_base);
					const int cs[2] = {c0, c1};
					for(int k = 0; k < 2; k++) {
						const int pl = 2 * tid + k;
						const int px = bin_x + (pl & 31), py = bin_y + (pl >> 5);
						if(px < p.width && py < p.height) {
							p.grad_px_off[size_t(py) * p.width + px] = base + uint32_t(foff + (k ? c0 : 0));
							p.grad_px_cnt[size_t(py) * p.width + px] = uint32_t(cs[k]);
						}
					}
				}
			}
			int mx = max(c0, c1);
#pragma unroll
			for(int o = 16; o > 0; o >>= 1)
				mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
			if(lane == 0 && mx > 0) {
				atomicMax(&p.info->max_pixel_fragments, uint32_t(mx));
				atomicMax(&s.bin_maxpx, mx);
			}
			if(tid == 0) {
				unsigned long long hb = s.stat_hbt;
				atomicAdd((unsigned long long*)&p.info->num_fragments, (unsigned long long)frags);
				atomicAdd((unsigned long long*)&p.info->num_hblock_tris, hb);
				atomicAdd(&p.info->stats[0], uint32_t(frags));
				atomicAdd(&p.info->stats[1], uint32_t(hb));
			}
		}
		__syncthreads();
		RASTER_TIMER(1);

		// ---- L. light bins (every pixel has at most kLightPixel fragments): one warp per row,
		// no CTA barrier until the bin is done
		if constexpr(MODE == kRasterForward) {
			if(s.bin_maxpx <= p.light_max_pixel) {
				uint32_t* K = &s.kv[0][0][0] + warp * kLightPool;
				uint32_t* V = &s.kv[0][0][0] + NW * kLightPool + warp * kLightPool;
				unsigned long long blended = 0;
				// timers: warp 0's rows split into generation (3) and blend (5); the wait for the
				// other warps at the end of the bin goes to 6
				long long* ta = timers && tid == 0 ? tacc : nullptr;
				int* cursor = &s.eff_prefix[warp * 32];
				for(int row = warp; row < 32; row += NW)
					blended += lightRow(p, s, scratch, planes, band_cap, bin, bin_x, bin_y, row, K, V, cursor, bg,
										additive, alpha_threshold, dump, ta);
				if(ta)
					tlast = clock64();
#pragma unroll
				for(int o = 16; o > 0; o >>= 1)
					blended += __shfl_xor_sync(0xffffffffu, blended, o);
				if(lane == 0 && blended)
					atomicAdd((unsigned long long*)&p.info->raster_blended_fragments, blended);
				if(tid == 0)
					atomicAdd(&p.info->raster_light_bins, 1u);
				__syncthreads();
				RASTER_TIMER(6);
				continue;
			}
		}

		// ---- C. pixel groups
		int p0 = 0;
		unsigned long long nblend = 0; // fragments this thread's pixels blended (forward mode)
		while(p0 < 1024) {
			if(tid == 0) {
				int base = s.eff_prefix[p0];
				int lo = p0 + 1, hi = min(p0 + kGroupPixels, 1024); // largest p1 within budget
				while(lo < hi) {
					int mid = (lo + hi + 1) >> 1;
					if(s.eff_prefix[mid] - base <= kGroupBudget)
						lo = mid;
					else
						hi = mid - 1;
				}
				// end the group at a row boundary when it holds one: a group's passes visit the band
				// entries of every row it touches, and a row split between two groups is visited twice
				if((lo & 31) != 0 && (lo & ~31) > p0)
					lo &= ~31;
				s.group_end = lo;
				s.kmin = 0xffffffffu;
				s.kmax = 0u;
				s.group_frags = 0u;
				s.n_cls = 0ull, s.n_large = 0;
			}
			__syncthreads();
			const int p1 = s.group_end;
			const int npix = p1 - p0;
			const int t = tid; // thread of pixel t (npix <= 256 < RT)
			// gradient passes: per-pixel state kept in the registers of thread t
			double acc64[3] = {0.0, 0.0, 0.0}, c64[3] = {0.0, 0.0, 0.0}, T64 = 1.0;
			float grad[3] = {0.0f, 0.0f, 0.0f};
			bool heavy = false;
			{
				uint32_t c = t < npix ? uint32_t(s.pix_count[p0 + t]) : 0u;
#pragma unroll
				for(int o = 16; o > 0; o >>= 1)
					c += __shfl_xor_sync(0xffffffffu, c, o);
				if(lane == 0 && c)
					atomicAdd(&s.group_frags, c);
			}
			if(t < npix) {
				int c = s.pix_count[p0 + t];
				heavy = c > kHeavyPixel;
				s.px_T[t] = 1.0f;
				s.px_c[t][0] = s.px_c[t][1] = s.px_c[t][2] = 0.0f;
				s.px_lo[t] = 0;
				s.px_done[t] = 0;
				s.px_state[t] = c == 0 ? 1 : 0;
				if constexpr(MODE == kRasterBackward) {
					// dL/dout through the clamp of the forward output (gradient passes where
					// 0 <= C <= 1), and the FP64 colour of the stats pass
					int pl = p0 + t;
					int px = bin_x + (pl & 31), py = bin_y + (pl >> 5);
					bool any = false;
					if(px < p.width && py < p.height) {
						size_t pix = size_t(py) * p.width + px;
						for(int ch = 0; ch < 3; ch++) {
							float cf = p.px_color32[pix * 3 + ch];
							float gch = p.dl_dimage[pix * 4 + ch];
							grad[ch] = (cf >= 0.0f && cf <= 1.0f) ? gch : 0.0f;
							c64[ch] = p.px_color64[pix * 3 + ch];
							any |= grad[ch] != 0.0f;
						}
					}
					if(!any)
						s.px_state[t] = 1;
				}
			}
			const bool windowed = __syncthreads_or(heavy);

			// C1. key range, fragment estimate and per-pixel depth histograms of a heavy group
			int nb_log = 0, shift = 0;
			bool slabs_on = false; // slab 0 is narrower than the group's key range
#if LUCID_RASTER_COUNTERS
			if(tid == 0)
				tc2 = clock64();
#endif
			if(windowed) {
				const int r0 = p0 >> 5, r1 = (p1 - 1) >> 5;
				// slabs only when the group holds more than two slabs' fragments (a second pass over
				// the entries costs more than it saves on shallower groups)
				const int n_active0 = __syncthreads_count(t < npix && s.px_state[t] != 1);
				const bool slabs = (unsigned long long)s.group_frags >
								   2ull * (unsigned long long)max(1, p.slab_target) * (unsigned long long)max(1, n_active0);
				slabs_on = slabs;
				if(slabs)
					for(int i = tid; i < kCoarseBins; i += RT)
						s.hist[i] = 0u;
				if(tid < kMaxSlabs)
					s.slab_first[tid] = 0x7fffffff;
				__syncthreads();
				uint32_t kmn = 0xffffffffu, kmx = 0u;
				for(int b = r0 >> 2; b <= (r1 >> 2); b++) {
					const int ne = s.band_count[b];
					for(int j = tid; j < ne; j += RT) {
						uint2 e = scratch[size_t(b) * band_cap + j];
						const float4 d = planes[size_t(b) * band_cap + j];
						RCOUNT(0, 1);
						float dx = d.x, dy = d.y, dz = d.z;
						uint32_t emn = 0xffffffffu, emx = 0u;
						int wsum = 0;
						auto rowRange = [&](int r, int row) {
							int lo = (e.x >> (5 * r)) & 31, hi = (e.y >> (5 * r)) & 31;
							int xlo = max(lo, p0 - 32 * row), xhi = min(hi, p1 - 1 - 32 * row);
							if(xlo > xhi)
								return;
							wsum += xhi - xlo + 1;
							// the evaluation is monotone in x, so the row's extremes are its ends
							float ty = dy * float(bin_y + row) + dz;
							uint32_t ka = nearFirstKey(dx * float(bin_x + xlo) + ty);
							uint32_t kb = nearFirstKey(dx * float(bin_x + xhi) + ty);
							emn = min(emn, min(ka, kb));
							emx = max(emx, max(ka, kb));
						};
						if(r0 == r1) { // a one-row group (the common case): its band's row only
							rowRange(r0 & 3, r0);
						} else {
#pragma unroll
							for(int r = 0; r < 4; r++) {
								int row = b * 4 + r;
								if(row >= r0 && row <= r1)
									rowRange(r, row);
							}
						}
						kmn = min(kmn, emn);
						kmx = max(kmx, emx);
						// fragment estimate: the entry's covered pixels at the midpoint of its keys
						if(slabs && wsum > 0) {
							const uint32_t mid = (emn >> 1) + (emx >> 1) + (emn & emx & 1u);
							atomicAdd(&s.hist[mid >> kCoarseShift], uint32_t(wsum));
						}
						// the entry's key range over the group, for the windows' entry culling;
						// planes that could evaluate to NaN somewhere keep the full range
						const float lim = 1e30f;
						if(!(fabsf(dx) < lim && fabsf(dy) < lim && fabsf(dz) < lim))
							emn = 0u, emx = 0xffffffffu;
						ekeys[size_t(b) * band_cap + j] = make_uint2(emn, emx);
					}
				}
#pragma unroll
				for(int o = 16; o > 0; o >>= 1) {
					kmn = min(kmn, __shfl_xor_sync(0xffffffffu, kmn, o));
					kmx = max(kmx, __shfl_xor_sync(0xffffffffu, kmx, o));
				}
				if(lane == 0) {
					atomicMin(&s.kmin, kmn);
					atomicMax(&s.kmax, kmx);
				}
				// buckets per pixel = 2^nb_log, at most 128: finer buckets make the window walks
				// longer than the sorts they save
				nb_log = 31 - __clz(max(1, min(128, kHistWords / npix)));
				// slabs of about p.slab_target fragments per unfinished pixel: slab k starts at the
				// first estimate bin whose preceding fragments reach k times that (the bins'
				// exclusive prefix sum, 8 bins per thread)
				__syncthreads();
				if(slabs) {
					constexpr int per = kCoarseBins / RT;
					uint32_t v[per], sum = 0u;
#pragma unroll
					for(int k = 0; k < per; k++) {
						v[k] = s.hist[tid * per + k];
						sum += v[k];
					}
					uint32_t acc = blockExclusiveScan(sum, s.scan_tmpu, (uint32_t*)nullptr);
					const unsigned long long slab_size =
						(unsigned long long)max(1, p.slab_target) * (unsigned long long)max(1, n_active0);
					const int bin_lo = int(s.kmin >> kCoarseShift), bin_hi = int(s.kmax >> kCoarseShift);
#pragma unroll
					for(int k = 0; k < per; k++) {
						const int bin = tid * per + k;
						if(bin >= bin_lo && bin <= bin_hi) {
							const int id = bin == bin_lo ? 0 : int(min(acc / slab_size, (unsigned long long)(kMaxSlabs - 1)));
							atomicMin(&s.slab_first[id], bin);
						}
						acc += v[k];
					}
				}
				__syncthreads();
			}
			const int nbuckets = 1 << nb_log;
			// Depth slabs: the histogram holds the keys of one slab [slab_lo, slab_hi] of the
			// group's key range, sized by the coarse estimate for about p.slab_target fragments per
			// unfinished pixel; the next slab is counted only when an unfinished pixel has used up
			// the current one. Pixels whose transmittance reaches 0 early never pay for the keys
			// behind them.
			uint32_t slab_lo = 0u, slab_hi = 0xffffffffu;
			auto buildSlab = [&](int slab) {
				if(tid == 0) {
					// the slab's keys: from its first bin (the group's kmin for slab 0) to the key
					// before the next slab's first bin (the group's kmax for the last)
					int next = slab + 1;
					while(next < kMaxSlabs && s.slab_first[next] == 0x7fffffff)
						next++;
					s.slab_lo = slab == 0 ? s.kmin : uint32_t(s.slab_first[slab]) << kCoarseShift;
					s.slab_hi = next >= kMaxSlabs ? s.kmax : (uint32_t(s.slab_first[next]) << kCoarseShift) - 1u;
					s.slab_next = next;
				}
				for(int i = tid; i < (npix << nb_log); i += RT)
					s.hist[i] = 0;
				__syncthreads();
				slab_lo = s.slab_lo, slab_hi = s.slab_hi;
				const uint32_t range = slab_hi - slab_lo;
				const int bits = range ? 32 - __clz(range) : 0;
				shift = max(0, bits - nb_log);
				const uint32_t lo_k = slab_lo, hi_k = slab_hi;
				const int sh = shift;
				// entries are culled against the slab only when it is narrower than the group's keys
				const bool cull = lo_k > s.kmin || hi_k < s.kmax;
				RCOUNT(7, tid == 0);
#if LUCID_RASTER_COUNTERS
				unsigned long long* ec5 = &rc[5];
#else
				unsigned long long* ec5 = nullptr;
#endif
				if(cull)
					forEachGroupFragment(p, s, scratch, planes, band_cap, bin_x, bin_y, p0, p1,
										 [&](int tp, uint32_t key, uint32_t) {
											 RCOUNT(1, 1);
											 if(key >= lo_k && key <= hi_k) {
												 RCOUNT(2, 1);
												 atomicAdd(&s.hist[histIdx(tp, int((key - lo_k) >> sh), nb_log)], 1u);
											 }
										 },
										 ekeys, 0u, 0, lo_k, hi_k, ec5);
				else // the whole key range: no test per fragment
					forEachGroupFragment(p, s, scratch, planes, band_cap, bin_x, bin_y, p0, p1,
										 [&](int tp, uint32_t key, uint32_t) {
											 RCOUNT(1, 1);
											 RCOUNT(2, 1);
											 atomicAdd(&s.hist[histIdx(tp, int((key - lo_k) >> sh), nb_log)], 1u);
										 }, nullptr, 0u, 0, 1u, 0u, ec5);
				__syncthreads();
				if(t < npix && s.px_state[t] != 1) {
					s.px_state[t] = 0;
					s.px_lo[t] = 0;
				}
				__syncthreads();
			};
#if LUCID_RASTER_COUNTERS
			if(tid == 0)
				rc[14] += clock64() - tc2;
#endif
			// Direct slab 0: one pass over the band entries appends every fragment of the slab to
			// its pixel's region of the idle sort buffer (kGroupCap / npix fragments per pixel)
			// and counts it in its pixel's bucket, and the first window is scattered from the
			// regions instead of generated from the entries again. A pixel whose slab overflows
			// its region sends the group to the histogram pass over the entries (which counts
			// the buckets afresh).
			// odd region stride: the pixels of a row append at similar cursors, so that their
			// stores fall into different banks
			const int rcap = ((kGroupCap / max(npix, 1)) - 1) | 1;
			bool direct_src = false;
			auto buildSlabDirect = [&]() -> bool {
				if(rcap < 64)
					return false;
				// a pixel with more fragments than its region fits only if slab 0 is narrower
				// than the group's keys
				if(!slabs_on && __syncthreads_or(t < npix && s.pix_count[p0 + t] > rcap))
					return false;
				if(tid == 0) {
					int next = 1;
					while(next < kMaxSlabs && s.slab_first[next] == 0x7fffffff)
						next++;
					s.slab_lo = s.kmin;
					s.slab_hi = next >= kMaxSlabs ? s.kmax : (uint32_t(s.slab_first[next]) << kCoarseShift) - 1u;
					s.slab_next = next;
				}
				if(t < npix)
					s.px_wend[t] = t * rcap;
				for(int i = tid; i < (npix << nb_log); i += RT)
					s.hist[i] = 0;
				__syncthreads();
				slab_lo = s.slab_lo, slab_hi = s.slab_hi;
				const uint32_t range = slab_hi - slab_lo;
				const int bits = range ? 32 - __clz(range) : 0;
				shift = max(0, bits - nb_log);
				const uint32_t lo_k = slab_lo, hi_k = slab_hi;
				const int sh = shift;
				const bool cull = lo_k > s.kmin || hi_k < s.kmax;
#if LUCID_RASTER_COUNTERS
				const long long tw0 = clock64();
#endif
				constexpr int AU = 4; // entries per step (8 measured slower than 4)
				auto append = [&](int tp, const bool* on, const uint32_t* key, const uint32_t* tri) {
					const int end = (tp + 1) * rcap;
					int pos[AU];
#pragma unroll
					for(int u = 0; u < AU; u++)
						pos[u] = on[u] && key[u] >= lo_k && key[u] <= hi_k ? atomicAdd(&s.px_wend[tp], 1) : end;
#pragma unroll
					for(int u = 0; u < AU; u++)
						if(pos[u] < end) {
							s.kv[1][0][pos[u]] = key[u];
							s.kv[1][1][pos[u]] = fragPayload(tp, tri[u]);
							atomicAdd(&s.hist[histIdx(tp, int((key[u] - lo_k) >> sh), nb_log)], 1u);
						}
				};
				// the idle window buffer holds the warps' staged entries
				forEachGroupFragmentStaged(p, s, scratch, planes, band_cap, bin_x, bin_y, p0, p1, append,
										   reinterpret_cast<uint4*>(&s.kv[0][0][0]), cull ? ekeys : nullptr,
										   cull ? lo_k : 0u, cull ? hi_k : 0xffffffffu);
#if LUCID_RASTER_COUNTERS
				if(lane == 0)
					rc[16] += clock64() - tw0;
#endif
				__syncthreads(); // every append is done before a pixel's cursor is tested below
#if LUCID_RASTER_COUNTERS
				if(tid == 0)
					rc[17] += clock64() - tw0;
#endif
				if(__syncthreads_or(t < npix && s.px_wend[t] > (t + 1) * rcap)) {
					RCOUNT(9, tid == 0);
					return false;
				}
				if(t < npix)
					s.px_rend[t] = s.px_wend[t] - t * rcap;
				if(t < npix && s.px_state[t] != 1) {
					s.px_state[t] = 0;
					s.px_lo[t] = 0;
				}
				__syncthreads();
				RCOUNT(7, tid == 0);
				return true;
			};
			if(windowed) {
				direct_src = buildSlabDirect();
				if(!direct_src)
					buildSlab(0);
			}
			RCOUNT(8, tid == 0 && windowed);
			RASTER_TIMER(2);

			// C2. windows
			while(true) {
#if LUCID_RASTER_COUNTERS
				if(tid == 0)
					tc2 = clock64();
#endif
				// this round's window of every active pixel and the window's sub-segments that need
				// sorting: one per bucket of the window (heavy group) or one per pixel (light group).
				// Positions are relative to the pixel's window start until the block scan places
				// the windows: a heavy pixel's warp walks its buckets 32 at a time to the first cut
				// holding >= kWindow fragments and turns the bucket counts into relative cursors.
				// List slots come from warp-aggregated counters; an entry is
				// (relative start, count, pixel), see segEntry.
				// one sub-segment per lane of each of two pixels A and B: class masks by ballot, one
				// packed atomic for the slots of both (A's entries first)
				auto addSegments2 = [&](bool inA, int begA, int cA, int tpA, bool inB, int begB, int cB, int tpB) {
					constexpr int kList = kGroupCap / 2;
					const uint32_t lt = laneMaskLt();
					const bool smA = inA && cA >= 2 && cA <= 16, lgA = inA && cA > 16 && cA <= 256;
					const bool smB = inB && cB >= 2 && cB <= 16, lgB = inB && cB > 16 && cB <= 256;
					const uint32_t msmA = __ballot_sync(0xffffffffu, smA), mlgA = __ballot_sync(0xffffffffu, lgA);
					const uint32_t msmB = __ballot_sync(0xffffffffu, smB), mlgB = __ballot_sync(0xffffffffu, lgB);
					if(msmA | mlgA | msmB | mlgB) {
						const int clsA = cA <= 2 ? 0 : cA <= 4 ? 1 : cA <= 8 ? 2 : 3;
						const int clsB = cB <= 2 ? 0 : cB <= 4 ? 1 : cB <= 8 ? 2 : 3;
						const uint32_t a0 = __ballot_sync(0xffffffffu, clsA & 1), a1 = __ballot_sync(0xffffffffu, clsA & 2);
						const uint32_t b0 = __ballot_sync(0xffffffffu, clsB & 1), b1 = __ballot_sync(0xffffffffu, clsB & 2);
						const uint32_t mA[4] = {msmA & ~a0 & ~a1, msmA & a0 & ~a1, msmA & ~a0 & a1, msmA & a0 & a1};
						const uint32_t mB[4] = {msmB & ~b0 & ~b1, msmB & b0 & ~b1, msmB & ~b0 & b1, msmB & b0 & b1};
						unsigned long long add = 0ull;
#pragma unroll
						for(int k = 0; k < 4; k++)
							add |= (unsigned long long)(__popc(mA[k]) + __popc(mB[k])) << (16 * k);
						unsigned long long base = 0ull;
						int lbase = 0;
						if(lane == 0) {
							if(add)
							{
								// two 32-bit atomics: classes 0-1 and 2-3 (no field carries across)
								uint32_t* nc32 = reinterpret_cast<uint32_t*>(&s.n_cls);
								const uint32_t b0 = atomicAdd(nc32, uint32_t(add)), b1 = atomicAdd(nc32 + 1, uint32_t(add >> 32));
								base = (unsigned long long)b0 | ((unsigned long long)b1 << 32);
							}
							if(mlgA | mlgB)
								lbase = atomicAdd(&s.n_large, __popc(mlgA) + __popc(mlgB));
						}
						base = __shfl_sync(0xffffffffu, base, 0);
						lbase = __shfl_sync(0xffffffffu, lbase, 0);
						auto put = [&](int cls, int pos, uint32_t entry) {
							if(pos >= kList) // lists overflow: the window is radix sorted
								return;
							if(cls == 0)
								s.sub_small[pos] = entry;
							else if(cls == 1)
								s.radix[pos] = entry;
							else if(cls == 2)
								s.sub_small[kList - 1 - pos] = entry;
							else
								s.radix[kList - 1 - pos] = entry;
						};
#pragma unroll
						for(int k = 0; k < 4; k++) {
							const int bk = int((base >> (16 * k)) & 0xffffu);
							if(smA && clsA == k)
								put(k, bk + __popc(mA[k] & lt), segEntry(begA, cA, tpA));
							if(smB && clsB == k)
								put(k, bk + __popc(mA[k]) + __popc(mB[k] & lt), segEntry(begB, cB, tpB));
						}
						constexpr int kLarge = kGroupCap / 17 + 1;
						if(lgA && lbase + __popc(mlgA & lt) < kLarge)
							s.sub_large[lbase + __popc(mlgA & lt)] = segEntry(begA, cA, tpA);
						if(lgB && lbase + __popc(mlgA) + __popc(mlgB & lt) < kLarge)
							s.sub_large[lbase + __popc(mlgA) + __popc(mlgB & lt)] = segEntry(begB, cB, tpB);
					}
					return (inA && cA > 256) || (inB && cB > 256);
				};
				auto addSegments = [&](bool in, int beg, int c, int tp) {
					return addSegments2(in, beg, c, tp, false, 0, 0, 0);
				};
				bool big = false;
#if LUCID_RASTER_COUNTERS
				const long long tk0 = clock64();
#endif
				if(windowed) {
					// one warp step per pixel: lane l sums its 2^g buckets from the pixel's first
					// unprocessed one, a warp scan finds the lane holding the cut, and the lane's
					// running sum the cut bucket. Two pixels per warp at a time; the sub-segments
					// of both take their list slots with one packed warp scan and one atomic.
					constexpr int kList = kGroupCap / 2;
					const int g = nb_log - 5, G = 1 << g;
					for(int tp0 = warp; tp0 < npix; tp0 += 2 * NW) {
						int tpq[2] = {tp0, tp0 + NW};
						bool act[2];
						int lsum[2], cntq[2][4], lo[2];
#pragma unroll
						for(int q = 0; q < 2; q++) {
							act[q] = tpq[q] < npix && s.px_state[tpq[q]] == 0;
							lo[q] = act[q] ? s.px_lo[tpq[q]] : nbuckets;
							lsum[q] = 0;
#pragma unroll
							for(int k = 0; k < 4; k++) {
								const int bk = (lane << g) + k;
								const int v = (k < G && act[q] && bk >= lo[q]) ? int(s.hist[histIdx(tpq[q], bk, nb_log)]) : 0;
								cntq[q][k] = v;
								lsum[q] += v;
							}
						}
						int incl[2], excl[2], cutq[2], accq[2];
#pragma unroll
						for(int q = 0; q < 2; q++) {
							incl[q] = warpInclusiveScan(lsum[q]);
							excl[q] = incl[q] - lsum[q];
						}
						// per lane: included buckets (k <= lastk) and the packed class counts
						// this lane's sub-segments per size class, 16 bits each: classes 0-1 and 2-3
						// (no field carries into the next)
						uint32_t cc01 = 0u, cc23 = 0u;
						int lcount = 0, lastk[2];
#pragma unroll
						for(int q = 0; q < 2; q++) {
							const uint32_t hit = __ballot_sync(0xffffffffu, act[q] && incl[q] >= kWindow);
							const int cl = hit ? __ffs(hit) - 1 : 32;
							int myk = G - 1, run = excl[q];
							if(lane == cl) {
								myk = -1;
#pragma unroll
								for(int k = 0; k < 4; k++) {
									if(k < G && myk < 0) {
										run += cntq[q][k];
										if(run >= kWindow)
											myk = k;
									}
								}
							}
							lastk[q] = !act[q] || lane > cl ? -1 : lane < cl ? G - 1 : myk;
							const int kc = __shfl_sync(0xffffffffu, myk, cl & 31);
							cutq[q] = hit ? (cl << g) + kc : nbuckets - 1;
							// the window's fragments: everything up to the cut
							const int upto = hit ? __shfl_sync(0xffffffffu, run, cl & 31) : __shfl_sync(0xffffffffu, incl[q], 31);
							accq[q] = upto;
#pragma unroll
							for(int k = 0; k < 4; k++) {
								const int c = cntq[q][k];
								if(k <= lastk[q] && c >= 2) {
									if(c <= 16) {
										const int cls = 31 - __clz(c - 1);
										const uint32_t inc = 1u << ((cls & 1) << 4);
										cc01 += cls < 2 ? inc : 0u;
										cc23 += cls < 2 ? 0u : inc;
									} else if(c <= 256)
										lcount++;
									else
										big = true;
								}
							}
						}
						const uint32_t ci01 = warpInclusiveScan(cc01), ci23 = warpInclusiveScan(cc23);
						const int lincl = warpInclusiveScan(lcount);
						uint32_t b01 = 0u, b23 = 0u;
						int lbase = 0;
						if(lane == 31) {
							// the two 32-bit halves of the packed class counts
							uint32_t* nc32 = reinterpret_cast<uint32_t*>(&s.n_cls);
							if(ci01)
								b01 = atomicAdd(nc32, ci01);
							if(ci23)
								b23 = atomicAdd(nc32 + 1, ci23);
							if(lincl)
								lbase = atomicAdd(&s.n_large, lincl);
						}
						b01 = __shfl_sync(0xffffffffu, b01, 31);
						b23 = __shfl_sync(0xffffffffu, b23, 31);
						lbase = __shfl_sync(0xffffffffu, lbase, 31);
						// this lane's first slot per class
						uint32_t cp01 = b01 + ci01 - cc01, cp23 = b23 + ci23 - cc23;
						int lpos = lbase + lincl - lcount;
#pragma unroll
						for(int q = 0; q < 2; q++) {
							int rel = excl[q];
#pragma unroll
							for(int k = 0; k < 4; k++) {
								const int c = cntq[q][k];
								if(k <= lastk[q]) {
									const int bk = (lane << g) + k;
									if(bk >= lo[q]) {
										s.hist[histIdx(tpq[q], bk, nb_log)] = uint32_t(rel);
										if(c >= 2 && c <= 16) {
											const int cls = 31 - __clz(c - 1); // 2 -> 0, 3-4 -> 1, 5-8 -> 2, 9-16 -> 3
											const bool back = cls >= 2;        // classes 2 and 3 fill their lists from the back
											const uint32_t sh16 = uint32_t(cls & 1) << 4;
											const int pos = int(((back ? cp23 : cp01) >> sh16) & 0xffffu);
											cp01 += back ? 0u : 1u << sh16;
											cp23 += back ? 1u << sh16 : 0u;
											const uint32_t entry = segEntry(rel, c, tpq[q]);
											const int idx = back ? kList - 1 - pos : pos;
											if(pos < kList) { // lists overflow: the window is radix sorted
												if(cls & 1)
													s.radix[idx] = entry;
												else
													s.sub_small[idx] = entry;
											}
										} else if(c > 16 && c <= 256) {
											if(lpos < kGroupCap / 17 + 1)
												s.sub_large[lpos] = segEntry(rel, c, tpq[q]);
											lpos++;
										}
									}
								}
								rel += c;
							}
						}
						if(lane == 0) {
#pragma unroll
							for(int q = 0; q < 2; q++) {
								if(!act[q])
									continue;
								const int tp = tpq[q];
								s.px_cut[tp] = cutq[q];
								s.px_wcnt[tp] = accq[q];
								if(accq[q] == 0)
									s.px_state[tp] = (s.px_done[tp] < s.pix_count[p0 + tp] && s.slab_hi < s.kmax) ? 2 : 1;
							}
						}
					}
				} else {
					const bool in = t < npix && s.px_state[t] == 0;
					const int c = in ? s.pix_count[p0 + t] : 0;
					if(in) {
						s.px_cut[t] = 0;
						s.px_wcnt[t] = c;
					}
					big = addSegments(in, 0, c, t);
				}
#if LUCID_RASTER_COUNTERS
				if(tid == 0)
					rc[15] += clock64() - tc2;
				if(lane == 0)
					rc[18] += clock64() - tk0;
#endif
				__syncthreads();
#if LUCID_RASTER_COUNTERS
				if(tid == 0)
					rc[19] += clock64() - tk0;
#endif
				int wcount = t < npix && s.px_state[t] == 0 ? s.px_wcnt[t] : 0;
				int total;
				int wbase = blockExclusiveScan(wcount, s.scan_tmp, &total);
				const bool over = total > kGroupCap;
				bool deferred = false;
				if(over) {
					// defer the pixels that do not fit this round (their window stays)
					bool fits = wbase + wcount <= kGroupCap;
					deferred = !fits && wcount > 0;
					if(!fits)
						wcount = 0;
					if(t < npix && s.px_state[t] == 0 && wbase == 0 && !fits) {
						// the first pending pixel alone exceeds the capacity
						raiseError(p.info, LUCID_ERR_PIXEL_FRAGMENTS, uint32_t(bin), uint32_t(p0 + t), uint32_t(total));
						if constexpr(MODE == kRasterStore) {
							// the store holds only the fragments written so far
							const int pl = p0 + t, px = bin_x + (pl & 31), py = bin_y + (pl >> 5);
							if(s.store_ok && px < p.width && py < p.height)
								p.grad_px_cnt[size_t(py) * p.width + px] = uint32_t(s.px_done[t]);
						}
						s.px_state[t] = 1;
						s.px_T[t] = 0.0f;
						s.px_c[t][0] = 1.0f, s.px_c[t][1] = 0.0f, s.px_c[t][2] = 0.0f;
						deferred = false;
					}
					wbase = blockExclusiveScan(wcount, s.scan_tmp, &total);
				}
				if(t < npix) {
					s.px_wbase[t] = wbase;
					s.px_wend[t] = wbase;
					s.px_bcur[t] = wbase;
					if(deferred) {
						s.px_cut[t] = -2 - s.px_cut[t]; // keeps the cut for the restore below
					} else {
						s.px_wcnt[t] = wcount;
						if(wcount == 0)
							s.px_cut[t] = -1; // not in this window (finished, empty or deferred)
					}
				}
				if(over && windowed) {
					// a deferred heavy pixel gets its bucket counts back from the cursors
					__syncthreads();
					for(int tp = warp; tp < npix; tp += NW) {
						const int enc = s.px_cut[tp];
						if(enc > -2)
							continue;
						const int cut = -2 - enc, wc = s.px_wcnt[tp];
						for(int c0 = s.px_lo[tp]; c0 <= cut; c0 += 32) {
							const int bk = c0 + lane;
							const bool in = bk <= cut;
							const int off = in ? int(s.hist[histIdx(tp, bk, nb_log)]) : 0;
							const int nxt = in ? (bk < cut ? int(s.hist[histIdx(tp, bk + 1, nb_log)]) : wc) : 0;
							__syncwarp();
							if(in)
								s.hist[histIdx(tp, bk, nb_log)] = uint32_t(nxt - off);
							__syncwarp();
						}
						if(lane == 0)
							s.px_cut[tp] = -1, s.px_wcnt[tp] = 0;
					}
				}
				if(tid == 0) {
					// sub-segment lists longer than their arrays (a window of many equal-depth
					// runs) send the window to the radix sort
					const unsigned long long nc = s.n_cls;
					constexpr int kList = kGroupCap / 2;
					const int n0 = int(nc & 0xffffu), n1 = int((nc >> 16) & 0xffffu);
					const int n2 = int((nc >> 32) & 0xffffu), n3 = int(nc >> 48);
					if(n0 + n2 > kList || n1 + n3 > kList || s.n_large > kGroupCap / 17 + 1)
						big = true;
				}
				const bool any_big = __syncthreads_or(big);
				if(!__syncthreads_or(wcount > 0)) {
					if(windowed && __syncthreads_or(t < npix && s.px_state[t] == 2)) {
						direct_src = false;
						buildSlab(s.slab_next); // a waiting pixel implies slab_hi < kmax
						continue;
					}
					break;
				}
				const int n = total;
#if LUCID_RASTER_COUNTERS
				if(tid == 0) {
					const long long now = clock64();
					rc[12] += now - tc2;
					tc2 = now;
				}
				RCOUNT(11, tid == 0);
				unsigned long long* ec6 = &rc[6];
#else
				unsigned long long* ec6 = nullptr;
#endif

				// C3. window fragments into their sub-segments. A lane always visits the same pixel,
				// so its window (as a key range), cursor base and end are read once.
				if(windowed && direct_src) {
					// the first window of a direct slab: from the pixels' regions
					direct_src = false;
					for(int tp = warp; tp < npix; tp += NW) {
						const int cut = s.px_cut[tp];
						if(cut < 0)
							continue;
						const uint32_t w_lo = uint32_t((unsigned long long)slab_lo + ((unsigned long long)s.px_lo[tp] << shift));
						const unsigned long long z = (unsigned long long)slab_lo + ((unsigned long long)(cut + 1) << shift) - 1ull;
						const uint32_t w_hi = uint32_t(z < (unsigned long long)slab_hi ? z : (unsigned long long)slab_hi);
						const int base = s.px_wbase[tp], end = base + s.px_wcnt[tp];
						const int beg = tp * rcap, n = s.px_rend[tp];
						for(int k = lane; k < n; k += 32) {
							const uint32_t key = s.kv[1][0][beg + k];
							if(key < w_lo || key > w_hi)
								continue;
							const int pos = base + int(atomicAdd(&s.hist[histIdx(tp, int((key - slab_lo) >> shift), nb_log)], 1u));
							if(pos < end) {
								s.kv[0][0][pos] = key;
								s.kv[0][1][pos] = s.kv[1][1][beg + k];
							}
						}
					}
				} else
				if(windowed) {
					int c_tp = -1, c_base = 0, c_end = 0;
					uint32_t c_klo = 1u, c_khi = 0u;
					forEachGroupFragment<true>(p, s, scratch, planes, band_cap, bin_x, bin_y, p0, p1,
										 [&](int tp, const bool* on, const uint32_t* key, const uint32_t* tri) {
											 if(tp != c_tp) {
												 c_tp = tp;
												 const int cut = s.px_cut[tp];
												 c_klo = 1u, c_khi = 0u;
												 if(cut >= 0) {
													 const unsigned long long a = (unsigned long long)slab_lo +
																				  ((unsigned long long)s.px_lo[tp] << shift);
													 const unsigned long long z = (unsigned long long)slab_lo +
																				  ((unsigned long long)(cut + 1) << shift) - 1ull;
													 c_klo = uint32_t(a);
													 c_khi = uint32_t(z < (unsigned long long)slab_hi ? z : (unsigned long long)slab_hi);
												 }
												 c_base = s.px_wbase[tp];
												 c_end = c_base + s.px_wcnt[tp];
											 }
											 bool w[4];
											 int pos[4];
#pragma unroll
											 for(int u = 0; u < 4; u++) {
												 w[u] = on[u] && key[u] >= c_klo && key[u] <= c_khi;
												 RCOUNT(3, on[u]);
												 RCOUNT(4, w[u]);
											 }
#pragma unroll
											 for(int u = 0; u < 4; u++)
												 pos[u] = w[u] ? c_base + int(atomicAdd(&s.hist[histIdx(tp, int((key[u] - slab_lo) >> shift), nb_log)], 1u)) : c_end;
#pragma unroll
											 for(int u = 0; u < 4; u++)
												 if(pos[u] < c_end) {
													 s.kv[0][0][pos[u]] = key[u];
													 s.kv[0][1][pos[u]] = fragPayload(tp, tri[u]);
												 }
										 },
										 ekeys, slab_lo, shift, 1u, 0u, ec6);
				} else {
					forEachGroupFragment(p, s, scratch, planes, band_cap, bin_x, bin_y, p0, p1,
										 [&](int tp, uint32_t key, uint32_t tri) {
											 if(s.px_cut[tp] < 0)
												 return;
											 const int pos = atomicAdd(&s.px_wend[tp], 1);
											 if(pos < s.px_wbase[tp] + s.px_wcnt[tp]) {
												 s.kv[0][0][pos] = key;
												 s.kv[0][1][pos] = fragPayload(tp, tri);
											 }
										 });
				}
				__syncthreads();
				// every window segment must be exactly full (histogram and generation evaluate the
				// same keys); anything else is an internal error
				if(t < npix && s.px_cut[t] >= 0) {
					int filled = windowed ? s.px_wbase[t] + int(s.hist[histIdx(t, s.px_cut[t], nb_log)]) : s.px_wend[t];
					int want = s.px_wbase[t] + s.px_wcnt[t];
					if(filled != want)
						raiseError(p.info, LUCID_ERR_BIN_COUNT, uint32_t(bin), uint32_t(p0 + t),
								   uint32_t(filled - s.px_wbase[t]));
					s.px_wend[t] = want;
				}
				// no barrier: the sorts below read neither px_wend nor the cursors, and thread t
				// alone reads px_wend[t] until the next barrier
#if LUCID_RASTER_COUNTERS
				if(tid == 0)
					rc[13] += clock64() - tc2;
#endif
				RASTER_TIMER(3);

				// C4. sort every sub-segment by key: small ones by one thread, larger ones (<= 256)
				// by one warp; any larger one sends the whole window to the block-wide radix sort
				if(!any_big) {
					uint32_t* K0 = s.kv[0][0];
					uint32_t* V0 = s.kv[0][1];
					// one index space over the four size classes, in class order, so that the
					// lanes of a warp mostly run the same network
					constexpr int kList = kGroupCap / 2;
					const unsigned long long nc = s.n_cls;
					const int e0 = int(nc & 0xffffu), e1 = e0 + int((nc >> 16) & 0xffffu);
					const int e2 = e1 + int((nc >> 32) & 0xffffu), ns = e2 + int(nc >> 48), nl = s.n_large;
					// entries of deferred pixels (not in this window) are skipped
					for(int i = tid; i < ns; i += RT) {
						const uint32_t e = i < e0 ? s.sub_small[i]
										 : i < e1 ? s.radix[i - e0]
										 : i < e2 ? s.sub_small[kList - 1 - (i - e1)]
												  : s.radix[kList - 1 - (i - e2)];
						const int tp = segPixel(e);
						if(s.px_cut[tp] < 0)
							continue;
						const int beg = s.px_wbase[tp] + int(e & 0x1fffu), cnt = segCount(e);
						if(i < e0)
							threadSortSegment<2>(K0, V0, beg, cnt);
						else if(i < e1)
							threadSortSegment<4>(K0, V0, beg, cnt);
						else if(i < e2)
							threadSortSegment<8>(K0, V0, beg, cnt);
						else
							threadSortSegment<16>(K0, V0, beg, cnt);
					}
					for(int i = warp; i < nl; i += NW) {
						const uint32_t e = s.sub_large[i];
						const int tp = segPixel(e);
						if(s.px_cut[tp] < 0)
							continue;
						const int beg = s.px_wbase[tp] + int(e & 0x1fffu), cnt = segCount(e);
						if(cnt <= 32)
							warpSortSegment<1>(K0, V0, beg, cnt);
						else if(cnt <= 64)
							warpSortSegment<2>(K0, V0, beg, cnt);
						else if(cnt <= 128)
							warpSortSegment<4>(K0, V0, beg, cnt);
						else
							warpSortSegment<8>(K0, V0, beg, cnt);
					}
				}
				__syncthreads();
				// the lists are consumed: the next window's start empty (read again only by the next
				// window's selection, after further barriers)
				if(tid == 0)
					s.n_cls = 0ull, s.n_large = 0;
				RASTER_TIMER(4);
				const bool use_radix = any_big && n > 1;
				if(tid == 0) {
					atomicAdd((unsigned long long*)&p.info->raster_windows, 1ull);
					atomicAdd((unsigned long long*)&p.info->raster_window_fragments, (unsigned long long)n);
					if(use_radix)
						atomicAdd(&p.info->raster_radix_windows, 1u);
				}
				int cur = 0;
				if(use_radix) {
					for(int pass = 0; pass < 4; pass++)
						if(radixPass(s, cur, n, pass * 8, false))
							cur ^= 1;
					if(radixPass(s, cur, n, 0, true))
						cur ^= 1;
				}
				uint32_t* K = s.kv[cur][0];
				uint32_t* V = s.kv[cur][1];

				// C5. equal-depth runs in primitive order (a run starts where the next fragment has
				// the same key and pixel and the previous one does not; equal neighbouring keys are
				// rare, so most elements read two keys and nothing else)
				for(int i = tid; i < n; i += RT) {
					const uint32_t ki = K[i];
					if(i + 1 >= n || K[i + 1] != ki)
						continue;
					const uint32_t vi = V[i];
					const bool same_prev = i > 0 && K[i - 1] == ki && ((V[i - 1] ^ vi) & 0xffu) == 0;
					const bool same_next = ((V[i + 1] ^ vi) & 0xffu) == 0;
					if(!same_prev && same_next) {
						int e = i + 1;
						while(e < n && K[e] == K[i] && ((V[e] ^ V[i]) & 0xffu) == 0)
							e++;
						for(int a = i + 1; a < e; a++) {
							uint32_t va = V[a], pa = fragPrim(p, va);
							int c = a - 1;
							while(c >= i && fragPrim(p, V[c]) > pa) {
								V[c + 1] = V[c];
								c--;
							}
							V[c + 1] = va;
						}
					}
				}
				__syncthreads();
				RASTER_TIMER(1);

				// C6. shade in batches, blend sequentially per pixel (store mode: copy the sorted
				// window to the pixel's store slice, one warp per pixel)
				float4* stage = reinterpret_cast<float4*>(&s.kv[cur ^ 1][0][0]);
				if constexpr(MODE == kRasterStore) {
					if(s.store_ok) {
						for(int tp = warp; tp < npix; tp += NW) {
							if(s.px_state[tp] != 0 || s.px_cut[tp] < 0)
								continue;
							const int pl = p0 + tp;
							const int px = bin_x + (pl & 31), py = bin_y + (pl >> 5);
							if(px >= p.width || py >= p.height)
								continue;
							const uint32_t dst = p.grad_px_off[size_t(py) * p.width + px] + uint32_t(s.px_done[tp]);
							const int wb = s.px_wbase[tp], wc = s.px_wcnt[tp];
							for(int k = lane; k < wc; k += 32) {
								const uint32_t tri = payloadTri(V[wb + k]);
								p.grad_tris[dst + k] = tri < 2u * uint32_t(p.max_visible_quads) ? tri : 0xffffffffu;
							}
						}
					}
					__syncthreads();
				}
				for(int round = 0; MODE != kRasterStore; round++) {
					// fragments shaded per pixel in this round: the first round's batch covers
					// what most pixels need to reach T == 0, later ones are shorter so that
					// little is shaded behind that point; odd, so that the pixels' staging rows
					// start in different shared-memory banks
					const int batch = (min(round == 0 ? kShadeFirst : kShadeNext, kStage / max(npix, 1)) - 1) | 1;
					if constexpr(MODE != kRasterBackward) {
						// per pixel: the blend cursor (< kGroupCap) and the fragments to shade in
						// this round (<= batch), read by every slot of the pixel with one load
						if(t < npix) {
							const int b = s.px_bcur[t];
							const int m = s.px_state[t] == 0 ? max(0, min(batch, s.px_wend[t] - b)) : 0;
							s.px_slot[t] = b | (m << 16);
						}
						__syncthreads();
						// slot / batch by multiply and shift (exact for odd batch in [15, 255] and
						// slot < 4096)
						const uint32_t bmul = (1u << 20) / uint32_t(batch) + 1u;
						// two slots per thread per step: both fragments' payloads and keys are read
						// before either is shaded, so that their record loads and FP32 chains overlap
						const int nslots = npix * batch;
						for(int slot0 = tid; slot0 < nslots; slot0 += 2 * RT) {
							int fq[2], tq[2];
							bool okq[2];
							uint32_t vq[2], kq[2];
#pragma unroll
							for(int q = 0; q < 2; q++) {
								const int slot = slot0 + q * RT;
								tq[q] = int((uint32_t(slot) * bmul) >> 20);
								const int ps = s.px_slot[min(tq[q], npix - 1)];
								const int j = slot - tq[q] * batch;
								fq[q] = (ps & 0xffff) + j;
								okq[q] = slot < nslots && j < (ps >> 16);
								vq[q] = okq[q] ? V[fq[q]] : 0u;
								kq[q] = okq[q] ? K[fq[q]] : 0u;
							}
							float4 cq[2];
#pragma unroll
							for(int q = 0; q < 2; q++) {
								const int pl = p0 + int(vq[q] & 0xffu);
								cq[q] = okq[q] ? shadeFragment(p, payloadTri(vq[q]), keyToDepth(kq[q]), bin_x + (pl & 31), bin_y + (pl >> 5))
											   : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
								if constexpr(MODE == kRasterForward)
									cq[q] = make_float4(cq[q].x * cq[q].w, cq[q].y * cq[q].w, cq[q].z * cq[q].w, 1.0f - cq[q].w);
							}
#pragma unroll
							for(int q = 0; q < 2; q++)
								if(okq[q]) {
									RCOUNT(10, 1);
									stage[slot0 + q * RT] = cq[q];
								}
						}
					}
					__syncthreads();
					RASTER_TIMER(5);
					bool active = false;
					if(t < npix && s.px_state[t] == 0) {
						int f = s.px_bcur[t];
						const int fend = s.px_wend[t], fbeg = s.px_wbase[t];
						float T = s.px_T[t];
						float c0 = s.px_c[t][0], c1 = s.px_c[t][1], c2 = s.px_c[t][2];
						bool finished = false;
						if(MODE == kRasterForward && !dump && !additive && !alpha_threshold) {
							// the plain forward blend without a branch per fragment: once T is 0 the
							// remaining steps of a run of 8 add -0 (the identity of FP32 addition)
							// and keep T, so the colour is that of the front-to-back loop that stops
							// at T == 0 (the same FP32 operations in the same order). A finished
							// pixel's cursor is not read again.
							const float4* sp = stage + t * batch;
							const int n = min(batch, fend - f);
							int on_steps = 0; // fragments blended (before T reached 0)
							auto step = [&](float4 q) {
								const bool on = T != 0.0f;
								on_steps += on ? 1 : 0;
								c0 = c0 + (on ? q.x * T : -0.0f);
								c1 = c1 + (on ? q.y * T : -0.0f);
								c2 = c2 + (on ? q.z * T : -0.0f);
								T = T * (on ? q.w : 1.0f);
							};
							int j = 0;
							for(; j + 8 <= n; j += 8) {
								float4 q[8];
#pragma unroll
								for(int u = 0; u < 8; u++)
									q[u] = sp[j + u];
#pragma unroll
								for(int u = 0; u < 8; u++)
									step(q[u]);
								if(T == 0.0f)
									break;
							}
							for(; T != 0.0f && j < n; j++)
								step(sp[j]);
							finished = T == 0.0f;
							if constexpr(MODE == kRasterForward)
								nblend += (unsigned long long)on_steps - (unsigned long long)j; // j is added below
							f += j;
						} else
						for(int j = 0; j < batch && f < fend; j++, f++) {
							float4 c;
							if constexpr(MODE == kRasterBackward) {
								// recompute the fragment's shading and route dL/dC to its inputs:
								// dC/dc = a*T, dC/da = c*T - S/(1-a) with S the colour behind it,
								// S = C - (colour accumulated up to and including it) in FP64
								uint32_t tri = payloadTri(V[f]);
								int pl = p0 + t;
								FragmentShade fs = shadeFragmentFull(p, tri, keyToDepth(K[f]),
																	 bin_x + (pl & 31), bin_y + (pl >> 5));
								c = fs.col;
								// the gradient terms use an FP64 transmittance (the FP32 one of
								// the image drifts by ~n ulp and c - B cancels)
								const float a = c.w;
								const float ca[3] = {c.x * a, c.y * a, c.z * a};
								const float cc[3] = {c.x, c.y, c.z};
								double da = 0.0;
								float dc[3];
								const double inv = 1.0 - double(a); // exact: a has a 24-bit mantissa
								const double rinv = inv != 0.0 ? 1.0 / inv : 0.0;
								for(int ch = 0; ch < 3; ch++) {
									acc64[ch] += double(ca[ch]) * T64;
									double behind = c64[ch] - acc64[ch];
									dc[ch] = float(double(grad[ch]) * double(a) * T64);
									double term = double(cc[ch]) * T64 - behind * rinv;
									da += double(grad[ch]) * term;
								}
								T64 *= inv;
								if(p.dvertex_rgba && fs.has_vc && p.color_format == LUCID_COLOR_RGBA32F) {
									// one vector reduction per vertex (RGBA rows are 16-byte aligned)
									const float dalpha = float(da) * fs.opacity;
									for(int k = 0; k < 3; k++) {
										float4* dst = reinterpret_cast<float4*>(p.dvertex_rgba) + fs.vid[k];
										atomicAdd(dst, make_float4(fs.inst.x * fs.wgt[k] * dc[0],
																   fs.inst.y * fs.wgt[k] * dc[1],
																   fs.inst.z * fs.wgt[k] * dc[2],
																   fs.inst.w * fs.wgt[k] * dalpha));
									}
								}
								if(p.dtri_opacity && p.tri_opacity)
									atomicAdd(p.dtri_opacity + fs.prim, float(da) * fs.alpha_pre);
							} else {
								c = stage[t * batch + j];
							}
							if constexpr(MODE == kRasterStats) {
								acc64[0] += double(c.x * c.w) * T64;
								acc64[1] += double(c.y * c.w) * T64;
								acc64[2] += double(c.z * c.w) * T64;
								T64 *= 1.0 - double(c.w);
							}
							if(dump) {
								int idx = s.px_done[t] + (f - fbeg);
								if(idx < p.dump_max) {
									int pl = p0 + t;
									long long di = dumpPixel(p, bin, pl, bin_x + (pl & 31), bin_y + (pl >> 5));
									if(di >= 0)
										p.dump_prims[size_t(di) * p.dump_max + idx] = int(fragPrim(p, V[f]));
								}
							}
							if constexpr(MODE == kRasterForward) {
								// c = (premultiplied rgb, 1 - alpha)
								if(additive) {
									c0 = c0 + c.x;
									c1 = c1 + c.y;
									c2 = c2 + c.z;
								} else {
									c0 = c0 + c.x * T;
									c1 = c1 + c.y * T;
									c2 = c2 + c.z * T;
									T = T * c.w;
									if((T == 0.0f && !dump) || (alpha_threshold && T < (1.0f / 128.0f))) {
										finished = true;
										f++;
										break;
									}
								}
							} else if(additive) {
								c0 = c0 + c.x * c.w;
								c1 = c1 + c.y * c.w;
								c2 = c2 + c.z * c.w;
							} else {
								c0 = c0 + (c.x * c.w) * T;
								c1 = c1 + (c.y * c.w) * T;
								c2 = c2 + (c.z * c.w) * T;
								T = T * (1.0f - c.w);
								if((T == 0.0f && !dump) || (alpha_threshold && T < (1.0f / 128.0f))) {
									finished = true;
									f++;
									break;
								}
							}
						}
						if constexpr(MODE == kRasterForward)
							nblend += (unsigned long long)(f - s.px_bcur[t]);
						s.px_bcur[t] = f;
						s.px_T[t] = T;
						s.px_c[t][0] = c0, s.px_c[t][1] = c1, s.px_c[t][2] = c2;
						if(finished)
							s.px_state[t] = 1;
						else
							active = f < fend;
					}
					const bool any_active = __syncthreads_or(active);
					RASTER_TIMER(6);
					if(!any_active)
						break;
				}
				// advance every pixel that took part in this window
				if(t < npix && s.px_state[t] == 0 && s.px_cut[t] >= 0) {
					s.px_done[t] += s.px_wcnt[t];
					int next = s.px_cut[t] + 1;
					s.px_lo[t] = next;
					if(!windowed || s.px_done[t] >= s.pix_count[p0 + t]) // every fragment is processed
						s.px_state[t] = 1;
					else if(next >= nbuckets) // the slab is used up: wait for the next one, or done
						s.px_state[t] = slab_hi < s.kmax ? 2 : 1;
				}
				// every pixel finished: no further selection round
				if(!__syncthreads_or(t < npix && s.px_state[t] != 1))
					break;
			}

			// C7. output
			if(t < npix && MODE != kRasterBackward && MODE != kRasterStore) {
				int pl = p0 + t;
				int px = bin_x + (pl & 31), py = bin_y + (pl >> 5);
				float T = s.px_T[t];
				float un[3] = {s.px_c[t][0] + T * bg.x, s.px_c[t][1] + T * bg.y, s.px_c[t][2] + T * bg.z};
				if constexpr(MODE == kRasterStats) {
					// the differentiable forward returns the FP64 colour rounded to FP32, the
					// function whose gradient the backward pass computes
					const float bgc[3] = {bg.x, bg.y, bg.z};
					for(int ch = 0; ch < 3; ch++) {
						acc64[ch] += T64 * double(bgc[ch]);
						un[ch] = float(acc64[ch]);
					}
				}
				float4 o;
				o.x = fminf(fmaxf(un[0], 0.0f), 1.0f);
				o.y = fminf(fmaxf(un[1], 0.0f), 1.0f);
				o.z = fminf(fmaxf(un[2], 0.0f), 1.0f);
				o.w = 1.0f;
				writePixel(p, px, py, o);
				if(dump) {
					long long di = dumpPixel(p, bin, pl, px, py);
					if(di >= 0)
						p.dump_counts[di] = s.pix_count[pl];
				}
				if constexpr(MODE == kRasterStats) {
					if(px < p.width && py < p.height) {
						size_t pix = size_t(py) * p.width + px;
						for(int ch = 0; ch < 3; ch++) {
							p.px_color64[pix * 3 + ch] = acc64[ch];
							p.px_color32[pix * 3 + ch] = un[ch];
						}
					}
				}
			}
			__syncthreads();
			RASTER_TIMER(7);
			p0 = p1;
		}
		if constexpr(MODE == kRasterForward) {
#pragma unroll
			for(int o = 16; o > 0; o >>= 1)
				nblend += __shfl_xor_sync(0xffffffffu, nblend, o);
			if(lane == 0 && nblend)
				atomicAdd((unsigned long long*)&p.info->raster_blended_fragments, nblend);
		}
	}
	if(timers && tid == 0)
		for(int i = 0; i < 8; i++)
			atomicAdd(&timer_info->raster_timers[i], uint32_t(tacc[i] >> 8));
#if LUCID_RASTER_COUNTERS
	if(timers)
		for(int i = 0; i < 24; i++) {
			unsigned long long v = rc[i];
#pragma unroll
			for(int o = 16; o > 0; o >>= 1)
				v += __shfl_xor_sync(0xffffffffu, v, o);
			if(lane == 0 && v)
				atomicAdd(reinterpret_cast<unsigned long long*>(timer_info->temp) + i, v);
		}
#endif
#undef RASTER_TIMER
}

void launchRaster(const FrameParams& p, int num_ctas, cudaStream_t stream, int mode) {
	const OneViewWork w{p};
	if(mode == kRasterStore)
		rasterKernel<kRasterStore><<<num_ctas, RT, sizeof(RasterSmem), stream>>>(w);
	else if(mode == kRasterStats)
		rasterKernel<kRasterStats><<<num_ctas, RT, sizeof(RasterSmem), stream>>>(w);
	else if(mode == kRasterBackward)
		rasterKernel<kRasterBackward><<<num_ctas, RT, sizeof(RasterSmem), stream>>>(w);
	else
		rasterKernel<kRasterForward><<<num_ctas, RT, sizeof(RasterSmem), stream>>>(w);
}

// One CTA: bins of each level per view (from the categorizer's counts) as prefix sums over
// the views, and the work counter of the batched raster pass reset.
__global__ void __launch_bounds__(kMaxBatchViews) batchPlanKernel(const FrameParams* views, int num_views,
																   int* level_prefix, uint32_t* counter) {
	__shared__ int s_scan[kMaxBatchViews / 32 + 1];
	const int v = threadIdx.x;
	const int levels[3] = {LUCID_BIN_LEVEL_HIGH, LUCID_BIN_LEVEL_LOW, LUCID_BIN_LEVEL_EMPTY};
	for(int L = 0; L < 3; L++) {
		// tiles: 1 per 32-pixel bin, 4 per 64-pixel bin
		int n = v < num_views ? int(views[v].info->bin_level_counts[levels[L]]) << (2 * (views[v].bin_shift - kBinShift)) : 0;
		int total;
		int off = blockExclusiveScan(n, s_scan, &total);
		if(v < num_views)
			level_prefix[L * (num_views + 1) + v] = off;
		if(v == 0)
			level_prefix[L * (num_views + 1) + num_views] = total;
	}
	if(v == 0)
		*counter = 0;
}

void launchRasterBatch(const FrameParams* views_dev, int num_views, int* level_prefix, uint32_t* counter,
					   int num_ctas, cudaStream_t stream) {
	batchPlanKernel<<<1, kMaxBatchViews, 0, stream>>>(views_dev, num_views, level_prefix, counter);
	const BatchWork w{views_dev, num_views, counter, level_prefix};
	rasterKernel<kRasterForward><<<num_ctas, RT, sizeof(RasterSmem), stream>>>(w);
}

cudaError_t configureRasterKernel() {
	cudaError_t err;
	const int bytes = int(sizeof(RasterSmem));
	if((err = cudaFuncSetAttribute(rasterKernel<kRasterForward, OneViewWork>,
								   cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) != cudaSuccess)
		return err;
	if((err = cudaFuncSetAttribute(rasterKernel<kRasterStats, OneViewWork>,
								   cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) != cudaSuccess)
		return err;
	if((err = cudaFuncSetAttribute(rasterKernel<kRasterBackward, OneViewWork>,
								   cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) != cudaSuccess)
		return err;
	if((err = cudaFuncSetAttribute(rasterKernel<kRasterStore, OneViewWork>,
								   cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) != cudaSuccess)
		return err;
	return cudaFuncSetAttribute(rasterKernel<kRasterForward, BatchWork>,
								cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

} // namespace lucid
