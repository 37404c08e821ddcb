// Host-side helpers shared by the C-ABI entry points (bc7_api.cu) and the
// request server (bc7_server.cu). Internal to the library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "bc7_kernels.cuh"
#include "bc7_pipeline.cuh"
#include "fastc_bc7.h"

namespace fastc {
namespace host {

extern thread_local std::string t_last_error;
extern std::mutex g_mu;  // guards the globals below and the host context
extern int g_warps;
extern uint32_t g_wm_next;
extern int g_ctas_per_sm;
extern int g_engine;

// Records the CUDA error text and maps it to a status.
fastc_bc7_status fail_cuda(cudaError_t e);

#define CK(expr)                                               \
  do {                                                         \
    cudaError_t e_ = (expr);                                   \
    if (e_ != cudaSuccess) return ::fastc::host::fail_cuda(e_); \
  } while (0)

// The same inside a helper that returns the cudaError_t itself (a sequence
// of enqueues whose caller drains the streams before it reports).
#define CK_RT(expr)                          \
  do {                                       \
    const cudaError_t e_ = (expr);           \
    if (e_ != cudaSuccess) return e_;        \
  } while (0)

bool settings_ok(const fastc_bc7_settings &s, fastc_bc7_status *why);
// Raster block range of a job (FasTC's BPTCC::Compress walk), or false.
bool job_range(const fastc_bc7_job &j, uint32_t *first, uint32_t *count);
int current_device();
LaunchShape pick_shape(uint64_t total);
size_t rank_scratch_bytes(uint64_t total);
// Scratch of a launch; task_bound: most cluster fits per block of its jobs.
size_t scratch_bytes(uint64_t total, int engine, int task_bound);
// Most block_task_bound() over the jobs' settings.
int task_bound_of(const fastc_bc7_settings *s, int per_job, uint32_t n);
EncodeScratch carve_scratch(void *base, uint64_t total);
JobDev make_job(const fastc_bc7_job &j, const fastc_bc7_settings &s, uint32_t first,
                uint32_t count, uint64_t begin);
uint32_t align_flags(const void *in, const void *out);
// `cls`: side streams for the pipeline engine's classes (null: one stream).
int launch_engine(const JobDev *jobs, int njobs, uint64_t total, void *scratch, int engine,
                  LaunchShape shape, int task_bound, const ClassStreams *cls, cudaStream_t st);
// `stats` not null: the logging encoder of CompressWithStats (pipeline
// engine only).
int launch_engine(const JobDev *jobs, int njobs, uint64_t total, void *scratch, int engine,
                  LaunchShape shape, int task_bound, const ClassStreams *cls,
                  const PipelineTuning &tune, cudaStream_t st,
                  fastc_bc7_block_stats *stats = nullptr, const ChunkEvents *events = nullptr);
// Side-stream sets for callers without their own: taken for one enqueue
// and given back (per device; created on first need).
ClassStreams *acquire_class_streams(int device);
void release_class_streams(int device, ClassStreams *cls);

}  // namespace host
}  // namespace fastc
