// The DXT1 / DXT5 kernels as other parts of the library (the request
// server) use them; defined in dxt.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "bc7_kernels.cuh"

namespace fastc {

// One-time per-device set-up of the DXT tables (outside any stream capture).
cudaError_t dxt_prepare(int dev);

// Encodes n jobs of one format on stream st, up to 32 per launch. Each job's
// in/out, first, nblocks, row0, out_first and flags are set by the caller;
// the block offsets within a launch are assigned here.
cudaError_t dxt_encode_jobs(JobDev *jobs, uint32_t n, bool alpha, cudaStream_t st);

// FasTC's PSNR error of count consecutive blocks (raster block first on,
// image width `width`) against the texel rows from row0 on: per block into
// block_sse, the sum into *total.
cudaError_t dxt_range_error(const uint8_t *blocks, const uint8_t *rows, uint32_t width, uint32_t row0,
                            uint32_t first, uint32_t count, bool alpha, double *block_sse,
                            double *total, cudaStream_t st);

}  // namespace fastc
