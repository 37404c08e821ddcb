// fastc_bc7_compress_device_noalloc: the device-memory encode with no
// allocation of any kind inside the call.
//
// Who needs it: callers that cannot let a library allocate device memory
// while they encode. A texture streamer or renderer that has carved the
// whole device into its own pools up front has no headroom for a stray
// cudaMalloc, and a failed allocation in the middle of a frame is worse
// than a size limit known in advance. cudaMalloc can also synchronise the
// device, which a latency-bound thread cannot afford, and the stream-ordered
// allocator used by fastc_bc7_compress_device draws on the stream's memory
// pool, which some hosts reserve for themselves. Such callers get a fixed
// array in the library's own device image instead: the CUDA driver reserves
// it when it loads the module, once, and every call reuses it.
//
// It encodes with the warp-per-block engine, whose scratch is two bytes per
// block plus four per 1024 blocks, so a modest array covers a 4096 x 4096
// texture. The bytes it writes are those of fastc_bc7_compress_device.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "bc7_host.h"
#include "bc7_kernels.cuh"
#include "fastc_bc7.h"

namespace {

using fastc::JobDev;

constexpr uint64_t kMaxBlocks = FASTC_BC7_NOALLOC_MAX_BLOCKS;
constexpr uint32_t kMaxJobs = FASTC_BC7_NOALLOC_MAX_JOBS;
constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
// Layout: the job table, then the rank scratch the way carve_scratch cuts
// it (counter and status, chunk counts, per-block ranks).
constexpr size_t kJobBytes = align256((size_t)kMaxJobs * sizeof(JobDev));
constexpr size_t kRankBytes =
    align256(256 + align256(((kMaxBlocks + fastc::kRankChunk - 1) / fastc::kRankChunk) * 4) +
             kMaxBlocks * 2 + 256);

// Nothing here has to start at zero: the rank pre-pass writes every chunk
// count and block rank and resets the work counter and status before the
// encoder reads them, and the job table is written by each call.
__device__ __align__(256) uint8_t g_noalloc_scratch[kJobBytes + kRankBytes];

// The job table travels to the device inside kernel parameters, in pieces of
// kJobsPerCopy entries (2,304 bytes of parameters each): the launch keeps
// its own copy of the entries, so nothing refers to the caller's host stack
// once the call has returned.
constexpr uint32_t kJobsPerCopy = 32;
struct JobPiece {
  JobDev j[kJobsPerCopy];
};

__global__ void put_jobs_kernel(JobPiece piece, uint32_t count, JobDev *dst) {
  if (threadIdx.x < count) dst[threadIdx.x] = piece.j[threadIdx.x];
}

constexpr int kMaxDevices = 64;
void *g_base[kMaxDevices];  // address of the array on each device (guarded by g_mu)

// One-time set-up per device, with that device current: the array's address
// and the encoder's constant tables (this synchronises the device once).
// The address is the one in the runtime's primary context of the device,
// the context every runtime-API caller shares.
fastc_bc7_status device_base(int dev, void **out) {
  std::lock_guard<std::mutex> lk(fastc::host::g_mu);
  if (dev < 0 || dev >= kMaxDevices) return FASTC_BC7_ERR_NO_DEVICE;
  if (!g_base[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fastc::host::fail_cuda(e);
    fastc::upload_tables(dev);
    g_base[dev] = p;
  }
  *out = g_base[dev];
  return FASTC_BC7_OK;
}

}  // namespace

extern "C" {

fastc_bc7_status fastc_bc7_compress_device_noalloc(const fastc_bc7_job *jobs, uint32_t n,
                                                   const fastc_bc7_settings *settings,
                                                   int per_job_settings, void *stream) {
  using namespace fastc::host;
  if (!jobs && n) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  if (n == 0) return FASTC_BC7_OK;
  if (n > kMaxJobs) {
    t_last_error = "fastc_bc7_compress_device_noalloc: " + std::to_string(n) +
                   " jobs exceed the fixed job table of " + std::to_string(kMaxJobs);
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  }
  fastc_bc7_settings dflt;
  fastc_bc7_settings_default(&dflt);
  JobDev tab[kMaxJobs];  // on the stack: the host side allocates nothing either
  static_assert(kMaxJobs % kJobsPerCopy == 0, "job table pieces");
  uint64_t total = 0;
  for (uint32_t i = 0; i < n; i++) {
    const fastc_bc7_settings &st = settings ? (per_job_settings ? settings[i] : settings[0]) : dflt;
    fastc_bc7_status why;
    if (!settings_ok(st, &why)) return why;
    if (st.watermark_start == FASTC_BC7_WATERMARK_CONTINUE) return FASTC_BC7_ERR_INVALID_ARGUMENT;
    uint32_t first, count;
    if (!jobs[i].in || !jobs[i].out || !job_range(jobs[i], &first, &count) ||
        (reinterpret_cast<uintptr_t>(jobs[i].in) & 3) || (reinterpret_cast<uintptr_t>(jobs[i].out) & 3))
      return FASTC_BC7_ERR_INVALID_ARGUMENT;
    tab[i] = make_job(jobs[i], st, first, count, total);
    tab[i].flags = align_flags(jobs[i].in, jobs[i].out);
    total += count;
  }
  if (total > kMaxBlocks || rank_scratch_bytes(total) > kRankBytes) {
    t_last_error = "fastc_bc7_compress_device_noalloc: " + std::to_string(total) +
                   " blocks exceed the fixed scratch of " + std::to_string(kMaxBlocks) + " blocks";
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  }
  if (total == 0) return FASTC_BC7_OK;
  const int dev = current_device();
  if (dev < 0) return FASTC_BC7_ERR_NO_DEVICE;
  void *base = nullptr;
  {
    const fastc_bc7_status st = device_base(dev, &base);
    if (st != FASTC_BC7_OK) return st;
  }
  fastc::LaunchShape shape;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    shape = pick_shape(total);
  }
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  uint8_t *p = static_cast<uint8_t *>(base);
  for (uint32_t k = 0; k < n; k += kJobsPerCopy) {
    JobPiece piece{};
    const uint32_t cnt = n - k < kJobsPerCopy ? n - k : kJobsPerCopy;
    for (uint32_t i = 0; i < cnt; i++) piece.j[i] = tab[k + i];
    put_jobs_kernel<<<1, kJobsPerCopy, 0, cs>>>(piece, cnt, reinterpret_cast<JobDev *>(p) + k);
    CK(cudaPeekAtLastError());
  }
  const fastc::EncodeScratch sc = carve_scratch(p + kJobBytes, total);
  const int le = fastc::launch_encode(reinterpret_cast<const JobDev *>(p), (int)n, total, sc,
                                      shape, cs);
  if (le) return fail_cuda((cudaError_t)le);
  return FASTC_BC7_OK;
}

}  // extern "C"
