// Launchers of the lucid_gb300 kernels (one per reference compute pass).
#pragma once

#include <string>

#include "lucid_common.cuh"

namespace lucid {

void launchSetup(const FrameParams& p, cudaStream_t stream);
void launchBinCount(const FrameParams& p, cudaStream_t stream);
void launchBinCategorize(const FrameParams& p, cudaStream_t stream);
void launchBinDispatch(const FrameParams& p, cudaStream_t stream);
void launchRaster(const FrameParams& p, int num_ctas, cudaStream_t stream, int mode = kRasterForward);
// Batched frames: one launch per pass for every view (CTA ranges per view in the maps).
void launchSetupBatch(const BatchViews& per_view, const BatchViews& setup_ctas, cudaStream_t stream);
void launchBinningBatch(const BatchViews& per_view, const BatchViews& binning_ctas, const BatchViews& bin_ctas,
						int max_bins, bool sorted_lists, cudaStream_t stream);
void launchRasterBatch(const FrameParams* views_dev, int num_views, int* level_prefix, uint32_t* counter,
					   int num_ctas, cudaStream_t stream);
// Pixel-parallel kernels over the fragment store: the plain blend and the differentiable
// frame's FP64 colour and backward pass.
void launchBlendPixels(const FrameParams& p, cudaStream_t stream);
void launchGradColor(const FrameParams& p, cudaStream_t stream);
void launchGradBackward(const FrameParams& p, cudaStream_t stream);
// Reference-order mode: per-bin path, then one CTA per (bin, 8x4 half-block).
void launchRefRaster(const FrameParams& p, uint8_t* plan, cudaStream_t stream);
// Quad generator (synchronous on `stream`): 0 ok, 1 bad vertex index, 2 out of memory, 3 CUDA error.
int quadGenerate(const float* positions, int num_verts, const int32_t* tris, int num_tris, float square_weight,
				 uint32_t* out_quads, int* out_num_quads, int* out_num_degenerate, cudaStream_t stream,
				 std::string& err);
cudaError_t configureBinningKernels();
size_t rasterSmemBytes();
int rasterThreads();

} // namespace lucid
