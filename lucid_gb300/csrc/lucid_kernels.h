// Launchers of the lucid_gb300 kernels (one per reference compute pass).
#pragma once

#include "lucid_common.cuh"

namespace lucid {

void launchSetup(const FrameParams& p, cudaStream_t stream);
void launchBinCount(const FrameParams& p, cudaStream_t stream);
void launchBinCategorize(const FrameParams& p, cudaStream_t stream);
void launchBinDispatch(const FrameParams& p, cudaStream_t stream);
void launchRaster(const FrameParams& p, int num_ctas, cudaStream_t stream, int mode = kRasterForward);
size_t rasterSmemBytes();
int rasterThreads();

} // namespace lucid
