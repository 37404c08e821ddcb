// Kernel-side declarations shared by the encoder/decoder kernels and the
// C-ABI host code.
#pragma once

#include <cstdint>

namespace fastc {

// One compression job as the kernels see it: a raster range of 4x4 blocks
// of one texture (FasTC's CompressionJob, Base/include/FasTC/
// CompressionJob.h:40-140), all pointers on the device.
struct JobDev {
  const uint8_t *in;   // RGBA8 texels; texel (x, y) at in + ((y - row0) * width + x) * 4
  uint8_t *out;        // BC7 blocks; raster block b at out + (b - out_first) * 16
  uint32_t width, height;
  uint32_t row0;       // first texel row present in `in`
  uint32_t out_first;  // raster block index stored at out[0]
  uint32_t first;      // raster block index of the job's first block
  uint32_t nblocks;    // blocks in the job
  uint32_t steps, modes, metric, seed, wm_start;
  uint32_t flags;      // kJobIn16 | kJobOut16
  uint64_t begin;      // global index of the job's first block across all jobs
};

constexpr uint32_t kJobIn16 = 1u;   // 16-byte texel-row loads are legal
constexpr uint32_t kJobOut16 = 2u;  // 16-byte block stores are legal
// Watermark index = wm_start + the block's single-colour rank over every job
// of the launch (FasTC's process-global counter), instead of within its job.
constexpr uint32_t kJobWmGlobal = 4u;

constexpr int kRankChunk = 1024;    // blocks per watermark-rank chunk

// Scratch the encoder needs beyond its inputs and outputs.
struct EncodeScratch {
  uint16_t *rank_local;    // [total] single-colour rank within its chunk
  uint32_t *chunk_prefix;  // [nchunks] exclusive prefix of single-colour counts
  unsigned long long *counter;  // work counter of the persistent kernel
  uint32_t *status;        // device-side status bits
  uint32_t *singles;       // single-colour blocks in the launch (written by the scan)
  uint32_t *carry;         // running single-colour count of the ranged pre-pass
};

struct LaunchShape {
  int warps_per_cta;  // 1..8
  int ctas;           // persistent grid size
};

// Host-side launchers (bc7_kernels.cu). All are asynchronous on `stream`.
void upload_tables(int device);
int launch_encode(const JobDev *jobs_dev, int njobs, uint64_t total_blocks,
                  const EncodeScratch &scratch, LaunchShape shape, void *stream);
int launch_decode(const uint8_t *blocks, uint8_t *rgba, uint32_t width, uint32_t height,
                  int spec_semantics, void *stream);
int device_sm_count(int device);
// Per-block squared error of decoded `blocks` against the original `rgba`
// (FasTC's PSNR metric) into block_sse, and their sum into *total when
// total is not null.
int launch_block_error(const uint8_t *blocks, const uint8_t *rgba, uint32_t width,
                       uint32_t height, double *block_sse, double *total, void *stream);
// Sum of n doubles in a fixed order (one CTA), into *out.
int launch_sum(const double *v, uint64_t n, double *out, void *stream);
// The same for the blocks [first, first + count) of a texture `width`
// texels wide, `blocks` holding them from `first` on and `rows` its texels
// from row `row0` on.
int launch_range_error(const uint8_t *blocks, const uint8_t *rows, uint32_t width, uint32_t row0,
                       uint32_t first, uint32_t count, double *block_sse, double *total,
                       void *stream);
// The single-colour rank pre-pass (classify + scan); also resets the work
// counter and status of `scratch`.
int launch_rank_prepass(const JobDev *jobs_dev, int njobs, uint64_t total_blocks,
                        const EncodeScratch &scratch, void *stream);
// The same for the blocks [g0, g1) of the launch only, continuing the
// ranks of the blocks before g0 (ranked by earlier calls in order on the
// same stream); g0 a multiple of kRankChunk, and the call with g0 == 0
// resets the counter and status. Lets a caller rank each piece of a launch
// once its texels have arrived.
int launch_rank_prepass_range(const JobDev *jobs_dev, int njobs, uint64_t total_blocks,
                              uint64_t g0, uint64_t g1, const EncodeScratch &scratch, void *stream);
// Resident CTAs per SM of the encoder with this many warps per CTA.
int encode_ctas_per_sm(int warps_per_cta);

}  // namespace fastc
