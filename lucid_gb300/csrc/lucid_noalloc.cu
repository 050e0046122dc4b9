// Binning entry point that allocates nothing (no counterpart in the reference).
//
// Who needs it: code that must not call cudaMalloc/cudaFree, for example a host that hands
// all device memory to its own allocator up front, or a caller that records work while
// allocation is not permitted. lucid_bin_noalloc runs the bin counter, categorizer and
// dispatcher kernels of lucid_binning.cu, and the sort that puts each bin's reference lists in
// slot order (in place, no scratch), on caller-provided inputs and outputs; the only
// memory they need beyond those — the counter kernel's per-CTA bin histograms, the status
// block and the bin work list — lives in the fixed-size static device array below.
//
// Limits and sharing:
//  * at most LUCID_NOALLOC_MAX_BINS bins (32x32-pixel bins of the viewport) and
//    kNoAllocCtas histogram rows: 1 MiB of device memory held by every GPU that loads the
//    library, for the life of the process;
//  * every call on a device uses the same array: two calls whose kernels overlap on the GPU
//    (e.g. on two streams without ordering) race and corrupt each other's results. Calls on
//    one stream are ordered and safe. The status block is cleared by each call; the
//    histogram rows are fully rewritten by each call before they are read.
//  * the first call on each device looks up the array's device address with
//    cudaGetSymbolAddress; make that first call before any stream capture.

#include <mutex>
#include <string>

#include "lucid_common.cuh"
#include "lucid_kernels.h"

namespace lucid {

constexpr int kNoAllocCtas = 64;
constexpr int kNoAllocMaxBins = LUCID_NOALLOC_MAX_BINS;
constexpr size_t kNoAllocInfoBytes = (sizeof(lucid_info) + 255) & ~size_t(255);
constexpr size_t kNoAllocWorkBytes = size_t(kNoAllocMaxBins) * 4;
constexpr size_t kNoAllocHistBytes = size_t(kNoAllocCtas) * 2 * kNoAllocMaxBins * 4;
constexpr size_t kNoAllocScratchBytes = kNoAllocInfoBytes + kNoAllocWorkBytes + kNoAllocHistBytes;

// The scratch: [status block | bin work list | per-CTA histograms].
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

__global__ void noallocSetVisibleCounts(lucid_info* info, int num_small, int num_large) {
	info->num_visible_quads[0] = num_small;
	info->num_visible_quads[1] = num_large;
}

} // namespace lucid

using namespace lucid;

// Message for lucid_last_error_string (defined in lucid_host.cu).
void lucidSetLastError(const std::string& msg);

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
unsigned char* g_noalloc_ptr[kMaxDevices] = {};

lucid_status noallocFail(lucid_status st, const std::string& msg) {
	lucidSetLastError(msg);
	return st;
}

} // namespace

extern "C" lucid_status lucid_bin_noalloc(const uint32_t* quad_aabbs, const uint32_t* tri_scan,
										  int32_t num_small_quads, int32_t num_large_quads,
										  int32_t max_visible_quads, int32_t width, int32_t height,
										  int32_t low_high_threshold, uint32_t* bin_counters,
										  uint32_t* bin_quads, uint32_t* bin_tris,
										  int32_t max_bin_refs, lucid_info* info_out,
										  void* stream) {
	if(width <= 0 || height <= 0 || width > 4096 || height > 4096)
		return noallocFail(LUCID_INVALID_ARG, "lucid_bin_noalloc: viewport must be 1..4096 pixels per axis");
	const int bcx = (width + kBinSize - 1) / kBinSize, bcy = (height + kBinSize - 1) / kBinSize;
	if(bcx * bcy > kNoAllocMaxBins)
		return noallocFail(LUCID_CAPACITY_EXCEEDED,
						   "lucid_bin_noalloc: " + std::to_string(bcx * bcy) + " bins exceed the static scratch limit of " +
							   std::to_string(kNoAllocMaxBins) + " (LUCID_NOALLOC_MAX_BINS)");
	if(max_visible_quads <= 0 || num_small_quads < 0 || num_large_quads < 0 ||
	   int64_t(num_small_quads) + num_large_quads > max_visible_quads || max_bin_refs < 0 ||
	   low_high_threshold <= 0)
		return noallocFail(LUCID_INVALID_ARG, "lucid_bin_noalloc: inconsistent counts or limits");
	if(!quad_aabbs || !tri_scan || !bin_counters || !bin_quads || !bin_tris)
		return noallocFail(LUCID_INVALID_ARG, "lucid_bin_noalloc: NULL input or output pointer");
	if(reinterpret_cast<uintptr_t>(tri_scan) & 15u)
		return noallocFail(LUCID_INVALID_ARG, "lucid_bin_noalloc: tri_scan must be 16-byte aligned");

	int dev = 0;
	cudaError_t err = cudaGetDevice(&dev);
	if(err != cudaSuccess)
		return noallocFail(LUCID_CUDA_ERROR, std::string("cudaGetDevice: ") + cudaGetErrorString(err));
	if(dev < 0 || dev >= kMaxDevices)
		return noallocFail(LUCID_NOT_SUPPORTED, "lucid_bin_noalloc: device index out of range");
	unsigned char* base;
	{
		std::lock_guard<std::mutex> lock(g_noalloc_mutex);
		if(!g_noalloc_ptr[dev]) {
			void* ptr = nullptr;
			err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
			if(err != cudaSuccess || !ptr)
				return noallocFail(LUCID_CUDA_ERROR, std::string("cudaGetSymbolAddress(scratch): ") +
														 cudaGetErrorString(err));
			g_noalloc_ptr[dev] = static_cast<unsigned char*>(ptr);
		}
		base = g_noalloc_ptr[dev];
	}
	cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
	lucid_info* info = reinterpret_cast<lucid_info*>(base);

	FrameParams p{};
	p.width = width, p.height = height;
	p.bin_count_x = bcx, p.bin_count_y = bcy, p.bin_count = bcx * bcy;
	p.bin_shift = kBinShift; // 32x32 bins
	p.max_visible_quads = max_visible_quads;
	p.max_bin_refs = max_bin_refs;
	p.low_high_threshold = low_high_threshold;
	p.num_binning_ctas = kNoAllocCtas;
	p.flags = LUCID_OPT_SORTED_BIN_LISTS; // reference lists in slot order (sorted in place)
	p.info = info;
	p.counts = bin_counters;
	p.quad_aabbs = const_cast<uint32_t*>(quad_aabbs);
	p.tri_scan = reinterpret_cast<uint4*>(const_cast<uint32_t*>(tri_scan));
	p.bin_quads = bin_quads;
	p.bin_tris = bin_tris;
	p.raster_work = reinterpret_cast<uint32_t*>(base + kNoAllocInfoBytes);
	p.bin_batches = reinterpret_cast<int*>(base + kNoAllocInfoBytes + kNoAllocWorkBytes);

	// What must start at zero: the status block and the caller's counters (the histogram
	// rows are fully written by the counter kernel before the dispatcher reads them).
	if((err = cudaMemsetAsync(info, 0, sizeof(lucid_info), s)) != cudaSuccess ||
	   (err = cudaMemsetAsync(bin_counters, 0, size_t(10) * p.bin_count * 4, s)) != cudaSuccess)
		return noallocFail(LUCID_CUDA_ERROR, std::string("cudaMemsetAsync: ") + cudaGetErrorString(err));
	noallocSetVisibleCounts<<<1, 1, 0, s>>>(info, num_small_quads, num_large_quads);
	launchBinCount(p, s);
	launchBinCategorize(p, s);
	launchBinDispatch(p, s);
	if(info_out) {
		err = cudaMemcpyAsync(info_out, info, sizeof(lucid_info), cudaMemcpyDeviceToDevice, s);
		if(err != cudaSuccess) {
			cudaGetLastError();
			return noallocFail(LUCID_CUDA_ERROR, std::string("lucid_bin_noalloc: copy to info_out: ") +
													 cudaGetErrorString(err));
		}
	}
	err = cudaGetLastError();
	if(err != cudaSuccess)
		return noallocFail(LUCID_CUDA_ERROR, std::string("lucid_bin_noalloc launch: ") + cudaGetErrorString(err));
	return LUCID_OK;
}
