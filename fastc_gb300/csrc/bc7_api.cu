// C-ABI implementation of the GB300 BC7 encoder (include/fastc_bc7.h).
//
// Host-memory calls stage the job's texel rows into a grow-only device
// buffer, launch the encoder on a private stream and copy the blocks back.
// Device-memory calls are asynchronous and take their scratch from the
// stream-ordered allocator of the caller's stream. Plans capture the whole
// encode pipeline of a fixed job set into one CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <utility>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "bc7_format.cuh"
#include "bc7_kernels.cuh"
#include "bc7_pipeline.cuh"
#include "fastc_bc7.h"
#include "bc7_host.h"

using fastc::ClassStreams;
using fastc::EncodeScratch;
using fastc::JobDev;
using fastc::LaunchShape;

namespace fastc {
namespace host {

thread_local std::string t_last_error;
std::mutex g_mu;
int g_warps = 4;
uint32_t g_wm_next = 0;  // FASTC_BC7_WATERMARK_CONTINUE counter (guarded by g_mu)
int g_ctas_per_sm = 0;  // 0: as many as fit
int g_engine = FASTC_BC7_ENGINE_PIPELINE;

fastc_bc7_status fail_cuda(cudaError_t e) {
  t_last_error = cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return FASTC_BC7_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return FASTC_BC7_ERR_NO_DEVICE;
  return FASTC_BC7_ERR_CUDA;
}


bool settings_ok(const fastc_bc7_settings &s, fastc_bc7_status *why) {
  if (s.shape_selection_fn != nullptr) {
    *why = FASTC_BC7_ERR_UNSUPPORTED;
    return false;
  }
  if ((s.block_modes & 0xFFu) == 0 || s.error_metric > 1 || s.steps > 256) {
    *why = FASTC_BC7_ERR_INVALID_ARGUMENT;
    return false;
  }
  return true;
}

// Raster block range of a job (CP:1473-1520 semantics), or false.
bool job_range(const fastc_bc7_job &j, uint32_t *first, uint32_t *count) {
  if (j.width == 0 || j.height == 0 || (j.width | j.height) & 3) return false;
  if ((j.x_start | j.y_start | j.x_end | j.y_end) & 3) return false;
  if (j.x_start >= j.width || j.y_start >= j.height || j.x_end > j.width) return false;
  const uint64_t bw = j.width / 4, bh = j.height / 4;
  if (bw * bh > 0xFFFFFFFFull) return false;
  const uint64_t start = (uint64_t)(j.y_start / 4) * bw + j.x_start / 4;
  const uint64_t end = j.y_end > j.height - 4 ? bw * bh : (uint64_t)(j.y_end / 4) * bw + j.x_end / 4;
  *first = (uint32_t)start;
  *count = end > start ? (uint32_t)(end - start) : 0u;
  return true;
}

int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) return -1;
  return d;
}

LaunchShape pick_shape(uint64_t total) {
  const int dev = current_device();
  const int sms = fastc::device_sm_count(dev);
  int warps = g_warps;
  int per_sm = g_ctas_per_sm > 0 ? g_ctas_per_sm : fastc::encode_ctas_per_sm(warps);
  if (per_sm < 1) per_sm = 1;
  uint64_t ctas = (uint64_t)sms * (uint64_t)per_sm;
  const uint64_t need = (total + (uint64_t)warps - 1) / (uint64_t)warps;
  if (ctas > need) ctas = need;
  if (ctas < 1) ctas = 1;
  return LaunchShape{warps, (int)ctas};
}

size_t rank_scratch_bytes(uint64_t total) {
  const uint64_t nchunks = (total + fastc::kRankChunk - 1) / fastc::kRankChunk;
  return (256 + ((nchunks * 4 + 255) & ~255ull) + total * 2 + 256 + 255) & ~255ull;
}

size_t scratch_bytes(uint64_t total, int engine, int task_bound) {
  size_t b = rank_scratch_bytes(total);
  if (engine == FASTC_BC7_ENGINE_PIPELINE)
    b += fastc::pipeline_scratch_bytes(total, task_bound, fastc::device_sm_count(current_device()));
  return b;
}

int task_bound_of(const fastc_bc7_settings *s, int per_job, uint32_t n) {
  if (!s) return fastc::block_task_bound(FASTC_BC7_ALL_MODES);
  int tb = 0;
  const uint32_t m = per_job ? n : 1;
  for (uint32_t i = 0; i < m; i++) tb = std::max(tb, fastc::block_task_bound(s[i].block_modes));
  return tb;
}

EncodeScratch carve_scratch(void *base, uint64_t total) {
  uint8_t *p = static_cast<uint8_t *>(base);
  const uint64_t nchunks = (total + fastc::kRankChunk - 1) / fastc::kRankChunk;
  EncodeScratch s;
  s.counter = reinterpret_cast<unsigned long long *>(p);
  s.status = reinterpret_cast<uint32_t *>(p + 8);
  s.singles = reinterpret_cast<uint32_t *>(p + 12);
  s.carry = reinterpret_cast<uint32_t *>(p + 16);
  s.chunk_prefix = reinterpret_cast<uint32_t *>(p + 256);
  s.rank_local = reinterpret_cast<uint16_t *>(p + 256 + ((nchunks * 4 + 255) & ~255ull));
  return s;
}

JobDev make_job(const fastc_bc7_job &j, const fastc_bc7_settings &s, uint32_t first,
                uint32_t count, uint64_t begin) {
  JobDev d;
  d.in = j.in;
  d.out = j.out;
  d.width = j.width;
  d.height = j.height;
  d.row0 = 0;
  d.out_first = 0;
  d.first = first;
  d.nblocks = count;
  d.steps = s.steps;
  d.modes = s.block_modes & 0xFFu;
  d.metric = s.error_metric;
  d.seed = s.seed;
  d.wm_start = s.watermark_start;
  d.flags = 0;
  d.begin = begin;
  return d;
}

uint32_t align_flags(const void *in, const void *out) {
  uint32_t f = 0;
  if ((reinterpret_cast<uintptr_t>(in) & 15) == 0) f |= fastc::kJobIn16;
  if ((reinterpret_cast<uintptr_t>(out) & 15) == 0) f |= fastc::kJobOut16;
  return f;
}

// Encode `total` blocks of the device job table with the selected engine,
// carving the rank and pipeline scratch out of `scratch`.
int launch_engine(const JobDev *jobs, int njobs, uint64_t total, void *scratch, int engine,
                  LaunchShape shape, int task_bound, const ClassStreams *cls,
                  const fastc::PipelineTuning &tune, cudaStream_t st,
                  fastc_bc7_block_stats *stats, const fastc::ChunkEvents *events) {
  const EncodeScratch rank = carve_scratch(scratch, total);
  if (engine == FASTC_BC7_ENGINE_PIPELINE || stats) {
    void *pipe = static_cast<uint8_t *>(scratch) + rank_scratch_bytes(total);
    return fastc::launch_pipeline(jobs, njobs, total, rank, pipe,
                                  fastc::device_sm_count(current_device()), task_bound, cls, tune,
                                  st, stats, events);
  }
  return fastc::launch_encode(jobs, njobs, total, rank, shape, st);
}

int launch_engine(const JobDev *jobs, int njobs, uint64_t total, void *scratch, int engine,
                  LaunchShape shape, int task_bound, const ClassStreams *cls, cudaStream_t st) {
  return launch_engine(jobs, njobs, total, scratch, engine, shape, task_bound, cls,
                       fastc::PipelineTuning{}, st);
}

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_cls_mu;
std::vector<ClassStreams *> g_cls_free[kMaxDevices];
}  // namespace

ClassStreams *acquire_class_streams(int device) {
  if (device < 0 || device >= kMaxDevices) return nullptr;
  {
    std::lock_guard<std::mutex> lk(g_cls_mu);
    if (!g_cls_free[device].empty()) {
      ClassStreams *c = g_cls_free[device].back();
      g_cls_free[device].pop_back();
      return c;
    }
  }
  ClassStreams *c = new ClassStreams();
  if (fastc::class_streams_create(c) != cudaSuccess) {
    delete c;
    return nullptr;  // the pipeline then runs on the caller's stream alone
  }
  return c;
}

void release_class_streams(int device, ClassStreams *cls) {
  if (!cls) return;
  std::lock_guard<std::mutex> lk(g_cls_mu);
  g_cls_free[device].push_back(cls);
}

}  // namespace host
}  // namespace fastc

using namespace fastc::host;

namespace {

// Grow-only device buffer.
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t n) {
    if (n <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) cap = n;
    return e;
  }
};

// State of the host-memory entry points (guarded by g_mu).
struct HostCtx {
  int device = -1;
  cudaStream_t stream = nullptr;
  DevBuf in, out, jobs, scratch, stats;
  ClassStreams *cls = nullptr;
  cudaStream_t copy = nullptr;      // host copies that overlap the encode
  std::vector<cudaEvent_t> in_ev;   // chunk k's texels are on the device
  std::vector<cudaEvent_t> out_ev;  // chunk k's blocks are written
  cudaEvent_t copied = nullptr;     // the copy stream's work is done
} g_host;

// At least n events in each list of the host context.
cudaError_t ensure_chunk_events(size_t n) {
  for (std::vector<cudaEvent_t> *v : {&g_host.in_ev, &g_host.out_ev})
    while (v->size() < n) {
      cudaEvent_t e;
      const cudaError_t ce = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
      if (ce != cudaSuccess) return ce;
      v->push_back(e);
    }
  return cudaSuccess;
}

fastc_bc7_status host_ctx_init() {
  const int dev = current_device();
  if (dev < 0) return FASTC_BC7_ERR_NO_DEVICE;
  if (g_host.device != dev) {
    if (g_host.stream) cudaStreamDestroy(g_host.stream);
    if (g_host.copy) cudaStreamDestroy(g_host.copy);
    for (cudaEvent_t e : g_host.in_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : g_host.out_ev) cudaEventDestroy(e);
    if (g_host.copied) cudaEventDestroy(g_host.copied);
    if (g_host.cls) release_class_streams(g_host.device, g_host.cls);
    g_host = HostCtx();
    CK(cudaStreamCreateWithFlags(&g_host.stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&g_host.copy, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&g_host.copied, cudaEventDisableTiming));
    g_host.device = dev;
    g_host.cls = acquire_class_streams(dev);
  }
  fastc::upload_tables(dev);
  return FASTC_BC7_OK;
}

const fastc_bc7_settings &settings_for(const fastc_bc7_settings *s, int per_job, uint32_t i,
                                       const fastc_bc7_settings &dflt) {
  if (!s) return dflt;
  return per_job ? s[i] : s[0];
}

// Host-memory batch: stage rows, launch, copy back. Caller holds g_mu.
// `stats` (one job only): the logging encoder, its statistics copied there.
fastc_bc7_status run_host(const fastc_bc7_job *jobs, uint32_t n, const fastc_bc7_settings *s,
                          int per_job, fastc_bc7_block_stats *stats = nullptr) {
  fastc_bc7_settings dflt;
  fastc_bc7_settings_default(&dflt);
  std::vector<JobDev> dj(n);
  std::vector<size_t> in_off(n), out_off(n), in_bytes(n);
  size_t in_total = 0, out_total = 0;
  uint64_t total = 0;
  bool any_continue = false;
  for (uint32_t i = 0; i < n; i++) {
    const fastc_bc7_settings &st = settings_for(s, per_job, i, dflt);
    fastc_bc7_status why;
    if (!settings_ok(st, &why)) return why;
    uint32_t first, count;
    if (!jobs[i].in || !jobs[i].out || !job_range(jobs[i], &first, &count))
      return FASTC_BC7_ERR_INVALID_ARGUMENT;
    dj[i] = make_job(jobs[i], st, first, count, total);
    if (st.watermark_start == FASTC_BC7_WATERMARK_CONTINUE) {
      dj[i].wm_start = g_wm_next;
      dj[i].flags |= fastc::kJobWmGlobal;
      any_continue = true;
    }
    const uint32_t bw = jobs[i].width / 4;
    const uint32_t r0 = count ? first / bw : 0, r1 = count ? (first + count - 1) / bw : 0;
    in_bytes[i] = count ? (size_t)(r1 - r0 + 1) * 4 * jobs[i].width * 4 : 0;
    dj[i].row0 = r0 * 4;
    dj[i].out_first = first;
    in_off[i] = in_total;
    out_off[i] = out_total;
    in_total += (in_bytes[i] + 255) & ~(size_t)255;
    out_total += ((size_t)count * 16 + 255) & ~(size_t)255;
    total += count;
  }
  if (total == 0) return FASTC_BC7_OK;
  fastc_bc7_status st = host_ctx_init();
  if (st != FASTC_BC7_OK) return st;
  CK(g_host.in.ensure(in_total));
  CK(g_host.out.ensure(out_total));
  CK(g_host.jobs.ensure(n * sizeof(JobDev)));
  const int engine = stats ? FASTC_BC7_ENGINE_PIPELINE : g_engine;
  const int tb = stats ? fastc::block_task_bound(settings_for(s, per_job, 0, dflt).block_modes, true)
                       : task_bound_of(s, per_job, n);
  CK(g_host.scratch.ensure(scratch_bytes(total, engine, tb)));
  if (stats) CK(g_host.stats.ensure(total * sizeof(fastc_bc7_block_stats)));
  cudaStream_t cs = g_host.stream;
  uint8_t *din = static_cast<uint8_t *>(g_host.in.p);
  uint8_t *dout = static_cast<uint8_t *>(g_host.out.p);
  for (uint32_t i = 0; i < n; i++) {
    if (!dj[i].nblocks) continue;
    dj[i].in = din + in_off[i];
    dj[i].out = dout + out_off[i];
    dj[i].flags |= fastc::kJobIn16 | fastc::kJobOut16;
  }
  // Texels go up on the copy stream in job order, chunk by chunk of the
  // pipeline, so that chunk k starts once its own jobs are in while later
  // ones are still copying; blocks come back the same way as each chunk is
  // packed. (The warp-per-block engine encodes all blocks in one pass, so
  // it takes everything first.) Overlap needs page-locked host buffers;
  // with pageable ones each copy returns once staged, in the same order.
  const bool chunked = engine == FASTC_BC7_ENGINE_PIPELINE;
  const uint64_t cap = chunked ? fastc::pipeline_chunk(std::min(
                                     tb, stats ? fastc::kMaxStatsBlockTasks : fastc::kMaxBlockTasks))
                               : total;
  const size_t nchunk = (size_t)((total + cap - 1) / cap);
  CK(ensure_chunk_events(nchunk));
  uint32_t singles = 0, status = 0;
  // Everything the call enqueues on its two streams. Both are drained
  // afterwards, also after an error, so that no copy of the call still
  // touches the caller's buffers once it has returned.
  auto enqueue = [&]() -> cudaError_t {
    CK_RT(cudaMemcpyAsync(g_host.jobs.p, dj.data(), n * sizeof(JobDev), cudaMemcpyHostToDevice, cs));
    auto copy_in = [&](uint32_t i) -> cudaError_t {
      if (!dj[i].nblocks) return cudaSuccess;
      const uint8_t *src = jobs[i].in + (size_t)dj[i].row0 * jobs[i].width * 4;
      return cudaMemcpyAsync(din + in_off[i], src, in_bytes[i], cudaMemcpyHostToDevice, g_host.copy);
    };
    auto copy_out = [&](uint32_t i) -> cudaError_t {
      if (!dj[i].nblocks) return cudaSuccess;
      return cudaMemcpyAsync(jobs[i].out + (size_t)dj[i].first * 16, dout + out_off[i],
                             (size_t)dj[i].nblocks * 16, cudaMemcpyDeviceToHost, g_host.copy);
    };
    {
      uint32_t next = 0;
      for (size_t k = 0; k < nchunk; k++) {
        const uint64_t end = (k + 1) * cap;
        while (next < n && dj[next].begin < end) CK_RT(copy_in(next++));
        CK_RT(cudaEventRecord(g_host.in_ev[k], g_host.copy));
      }
    }
    if (!chunked) CK_RT(cudaStreamWaitEvent(cs, g_host.in_ev[nchunk - 1], 0));
    const EncodeScratch sc = carve_scratch(g_host.scratch.p, total);
    fastc_bc7_block_stats *dstats =
        static_cast<fastc_bc7_block_stats *>(stats ? g_host.stats.p : nullptr);
    fastc::ChunkEvents ev;
    ev.in_ready = g_host.in_ev.data();
    ev.packed = g_host.out_ev.data();
    ev.count = (int)nchunk;
    const int le = launch_engine(static_cast<const JobDev *>(g_host.jobs.p), (int)n, total,
                                 g_host.scratch.p, engine, pick_shape(total), tb, g_host.cls,
                                 fastc::PipelineTuning{}, cs, dstats, chunked ? &ev : nullptr);
    CK_RT((cudaError_t)le);
    if (chunked) {
      uint32_t next = 0;
      for (size_t k = 0; k < nchunk; k++) {
        const uint64_t end = k + 1 == nchunk ? total : (k + 1) * cap;
        CK_RT(cudaStreamWaitEvent(g_host.copy, g_host.out_ev[k], 0));
        while (next < n && dj[next].begin + dj[next].nblocks <= end) CK_RT(copy_out(next++));
      }
    } else {
      CK_RT(cudaEventRecord(g_host.out_ev[0], cs));
      CK_RT(cudaStreamWaitEvent(g_host.copy, g_host.out_ev[0], 0));
      for (uint32_t i = 0; i < n; i++) CK_RT(copy_out(i));
    }
    CK_RT(cudaEventRecord(g_host.copied, g_host.copy));
    CK_RT(cudaStreamWaitEvent(cs, g_host.copied, 0));
    if (stats)
      CK_RT(cudaMemcpyAsync(stats, dstats, total * sizeof(fastc_bc7_block_stats),
                            cudaMemcpyDeviceToHost, cs));
    if (any_continue)
      CK_RT(cudaMemcpyAsync(&singles, sc.singles, sizeof(singles), cudaMemcpyDeviceToHost, cs));
    CK_RT(cudaMemcpyAsync(&status, sc.status, sizeof(status), cudaMemcpyDeviceToHost, cs));
    return cudaSuccess;
  };
  cudaError_t e = enqueue();
  const cudaError_t se_copy = cudaStreamSynchronize(g_host.copy);
  const cudaError_t se_comp = cudaStreamSynchronize(cs);
  if (e == cudaSuccess) e = se_copy != cudaSuccess ? se_copy : se_comp;
  if (e != cudaSuccess) return fail_cuda(e);
  if (status & 2u) {  // the task-overflow status bit (bc7_block.cuh)
    // a block needed more cluster fits than the scratch was sized for; its
    // bytes are not FasTC's (never expected: the bound is computed above)
    t_last_error = "a block needed more cluster fits than the launch's task bound";
    return FASTC_BC7_ERR_INTERNAL;
  }
  if (any_continue) g_wm_next = (uint32_t)((g_wm_next + (uint64_t)singles) % 9u);
  if (stats) {
    // the mode written: the unary mode prefix of the block (CP:1096-1298)
    const uint8_t *blk = jobs[0].out + (size_t)dj[0].first * 16;
    for (uint64_t b = 0; b < total; b++) {
      const uint8_t m0 = blk[16 * b];
      stats[b].mode = m0 ? __builtin_ctz(m0) : 8;
    }
  }
  return FASTC_BC7_OK;
}

}  // namespace

struct fastc_bc7_plan_s {
  int device = -1;
  JobDev *d_jobs = nullptr;
  void *d_scratch = nullptr;
  uint64_t total = 0;
  int njobs = 0;
  EncodeScratch sc{};
  int engine = FASTC_BC7_ENGINE_PIPELINE;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t kernels = 0;  // kernel nodes of the graph
  int task_bound = 0;
  size_t scratch_size = 0;  // bytes at d_scratch
  int warps = 4;            // warps per CTA when the engine is warp-per-block
  fastc::PipelineTuning tune;
};

namespace {

// The warp-per-block engine's launch shape with `warps` warps per CTA.
LaunchShape shape_with(uint64_t total, int warps) {
  const int sms = fastc::device_sm_count(current_device());
  const int per_sm = std::max(1, fastc::encode_ctas_per_sm(warps));
  uint64_t ctas = (uint64_t)sms * (uint64_t)per_sm;
  const uint64_t need = (total + (uint64_t)warps - 1) / (uint64_t)warps;
  ctas = std::max<uint64_t>(1, std::min(ctas, need));
  return LaunchShape{warps, (int)ctas};
}

// Captures the plan's whole launch with `engine` (`warps` warps per CTA for
// the warp-per-block engine) and `tune` into a graph (private stream and
// side streams, released after the capture) and instantiates it.
cudaError_t capture_plan(const fastc_bc7_plan_s *p, int engine, int warps,
                         const fastc::PipelineTuning &tune, cudaGraph_t *graph,
                         cudaGraphExec_t *exec, uint64_t *kernels) {
  *graph = nullptr;
  *exec = nullptr;
  cudaStream_t cs = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  ClassStreams cls{};
  const bool use_cls = engine == FASTC_BC7_ENGINE_PIPELINE;
  if (e == cudaSuccess && use_cls) e = fastc::class_streams_create(&cls);
  if (e == cudaSuccess) {
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      const LaunchShape shape =
          engine == FASTC_BC7_ENGINE_PIPELINE ? pick_shape(p->total) : shape_with(p->total, warps);
      const int le = launch_engine(p->d_jobs, p->njobs, p->total, p->d_scratch, engine, shape,
                                   p->task_bound, use_cls ? &cls : nullptr, tune, cs);
      cudaError_t ee = cudaStreamEndCapture(cs, graph);
      e = le ? (cudaError_t)le : ee;
    }
  }
  if (e == cudaSuccess && !*graph) e = cudaErrorStreamCaptureInvalidated;
  if (e == cudaSuccess && kernels) {
    size_t nn = 0;
    e = cudaGraphGetNodes(*graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (e == cudaSuccess && nn) e = cudaGraphGetNodes(*graph, nodes.data(), &nn);
    *kernels = 0;
    for (size_t k = 0; k < nn && e == cudaSuccess; k++) {
      cudaGraphNodeType t;
      e = cudaGraphNodeGetType(nodes[k], &t);
      if (t == cudaGraphNodeTypeKernel) (*kernels)++;
    }
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(exec, *graph, 0);
  fastc::class_streams_destroy(&cls);
  if (cs) cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    if (*exec) cudaGraphExecDestroy(*exec);
    if (*graph) cudaGraphDestroy(*graph);
    *exec = nullptr;
    *graph = nullptr;
  }
  return e;
}

}  // namespace

extern "C" {

void fastc_bc7_settings_default(fastc_bc7_settings *s) {
  if (!s) return;
  std::memset(s, 0, sizeof(*s));
  s->block_modes = FASTC_BC7_ALL_MODES;
  s->error_metric = 0;
  s->steps = 50;
}

const char *fastc_bc7_status_string(fastc_bc7_status st) {
  switch (st) {
    case FASTC_BC7_OK: return "ok";
    case FASTC_BC7_ERR_INVALID_ARGUMENT: return "invalid argument";
    case FASTC_BC7_ERR_UNSUPPORTED: return "unsupported";
    case FASTC_BC7_ERR_OUT_OF_MEMORY: return "out of device memory";
    case FASTC_BC7_ERR_CUDA: return "CUDA error";
    case FASTC_BC7_ERR_BUDGET: return "over memory budget";
    case FASTC_BC7_ERR_TIMEOUT: return "timed out";
    case FASTC_BC7_ERR_NOT_FOUND: return "not found";
    case FASTC_BC7_ERR_CANCELLED: return "cancelled";
    case FASTC_BC7_ERR_NO_DEVICE: return "no CUDA device";
    default: return "internal error";
  }
}

const char *fastc_bc7_last_error(void) { return t_last_error.c_str(); }
uint32_t fastc_bc7_abi_version(void) { return FASTC_BC7_ABI_VERSION; }

uint64_t fastc_bc7_job_blocks(const fastc_bc7_job *job) {
  uint32_t first, count;
  if (!job || !job_range(*job, &first, &count)) return 0;
  return count;
}

fastc_bc7_status fastc_bc7_compress(const fastc_bc7_job *job, const fastc_bc7_settings *s) {
  if (!job) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_mu);
  return run_host(job, 1, s, 0);
}

fastc_bc7_status fastc_bc7_compress_stats(const fastc_bc7_job *job, const fastc_bc7_settings *s,
                                          fastc_bc7_block_stats *stats) {
  if (!job || !stats) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_mu);
  return run_host(job, 1, s, 0, stats);
}

fastc_bc7_status fastc_bc7_stats_log(const fastc_bc7_job *job, const fastc_bc7_block_stats *stats,
                                     char *buf, size_t cap, size_t *len) {
  if (!job || !len || (cap && !buf)) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  uint32_t first, count;
  if (!job_range(*job, &first, &count)) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  if (count && !stats) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  static const char *const kNames[8] = {"Zero", "One", "Two", "Three",
                                        "Four", "Five", "Six", "Seven"};
  std::string out;
  char line[128];
  auto put_d = [&](uint64_t idx, const char *name, double v) {
    const int k = std::snprintf(line, sizeof(line), "%llu: BlockStat_%s -- %g\n",
                                (unsigned long long)idx, name, v);
    out.append(line, (size_t)k);
  };
  auto put_i = [&](uint64_t idx, const char *name, int v) {
    const int k = std::snprintf(line, sizeof(line), "%llu: BlockStat_%s -- %d\n",
                                (unsigned long long)idx, name, v);
    out.append(line, (size_t)k);
  };
  char nm[64];
  for (uint32_t b = 0; b < count; b++) {
    const fastc_bc7_block_stats &st = stats[b];
    const uint64_t idx = (uint64_t)first + b;
    for (int k = 0; k < st.n_two && k < 64; k++) put_d(idx, "TwoShapeEstimate", st.two_shape[k]);
    for (int k = 0; k < st.n_three && k < 64; k++)
      put_d(idx, "ThreeShapeEstimate", st.three_shape[k]);
    put_i(idx, "Path", st.path);
    put_i(idx, "Mode", st.mode);
    for (int m = 0; m < 8; m++) {
      std::snprintf(nm, sizeof(nm), "Mode%sEstimate", kNames[m]);
      put_d(idx, nm, st.estimate[m]);
      std::snprintf(nm, sizeof(nm), "Mode%sError", kNames[m]);
      put_d(idx, nm, st.error[m]);
    }
  }
  *len = out.size();
  if (cap) std::memcpy(buf, out.data(), out.size() < cap ? out.size() : cap);
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_compress_batch(const fastc_bc7_job *jobs, uint32_t n,
                                          const fastc_bc7_settings *settings,
                                          int per_job_settings) {
  if (!jobs && n) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  if (n == 0) return FASTC_BC7_OK;
  std::lock_guard<std::mutex> lk(g_mu);
  return run_host(jobs, n, settings, per_job_settings);
}

fastc_bc7_status fastc_bc7_compress_image(const uint8_t *rgba, uint32_t width, uint32_t height,
                                          uint8_t *cmp, size_t cmp_size,
                                          const fastc_bc7_settings *s) {
  if (!rgba || !cmp || (size_t)width * height > cmp_size) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  fastc_bc7_job j{rgba, cmp, width, height, 0, 0, width, height};
  return fastc_bc7_compress(&j, s);
}

fastc_bc7_status fastc_bc7_decompress(const uint8_t *blocks, uint8_t *rgba, uint32_t width,
                                      uint32_t height, int spec) {
  if (!blocks || !rgba || width == 0 || height == 0) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_mu);
  fastc_bc7_status st = host_ctx_init();
  if (st != FASTC_BC7_OK) return st;
  const size_t nb = (size_t)((width + 3) / 4) * ((height + 3) / 4);
  const size_t img = (size_t)width * height * 4;
  CK(g_host.in.ensure(nb * 16));
  CK(g_host.out.ensure(img));
  cudaStream_t cs = g_host.stream;
  cudaError_t e = cudaMemcpyAsync(g_host.in.p, blocks, nb * 16, cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess)
    e = (cudaError_t)fastc::launch_decode(static_cast<const uint8_t *>(g_host.in.p),
                                          static_cast<uint8_t *>(g_host.out.p), width, height, spec, cs);
  if (e == cudaSuccess) e = cudaMemcpyAsync(rgba, g_host.out.p, img, cudaMemcpyDeviceToHost, cs);
  // drained also after an error: no copy of the call outlives it
  const cudaError_t se = cudaStreamSynchronize(cs);
  if (e == cudaSuccess) e = se;
  return e == cudaSuccess ? FASTC_BC7_OK : fail_cuda(e);
}

fastc_bc7_status fastc_bc7_block_error_device(const uint8_t *blocks, const uint8_t *rgba,
                                              uint32_t width, uint32_t height, double *block_sse,
                                              double *sse_total, void *stream) {
  if (!blocks || !rgba || !block_sse || width == 0 || height == 0)
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  const int le = fastc::launch_block_error(blocks, rgba, width, height, block_sse, sse_total, stream);
  if (le) return fail_cuda((cudaError_t)le);
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_psnr(const uint8_t *blocks, const uint8_t *rgba, uint32_t width,
                                uint32_t height, double *psnr, double *block_sse) {
  if (!blocks || !rgba || width == 0 || height == 0) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_mu);
  fastc_bc7_status st = host_ctx_init();
  if (st != FASTC_BC7_OK) return st;
  const size_t nb = (size_t)((width + 3) / 4) * ((height + 3) / 4);
  const size_t img = (size_t)width * height * 4;
  CK(g_host.in.ensure(img + nb * 16));
  CK(g_host.out.ensure((nb + 1) * sizeof(double)));
  cudaStream_t cs = g_host.stream;
  uint8_t *dimg = static_cast<uint8_t *>(g_host.in.p);
  uint8_t *dblk = dimg + img;  // byte loads only, so no alignment is needed
  double *dsse = static_cast<double *>(g_host.out.p);
  double total = 0.0;
  cudaError_t e = cudaMemcpyAsync(dimg, rgba, img, cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dblk, blocks, nb * 16, cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess)
    e = (cudaError_t)fastc::launch_block_error(dblk, dimg, width, height, dsse + 1, dsse, cs);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, dsse, sizeof(double), cudaMemcpyDeviceToHost, cs);
  if (e == cudaSuccess && block_sse)
    e = cudaMemcpyAsync(block_sse, dsse + 1, nb * sizeof(double), cudaMemcpyDeviceToHost, cs);
  // drained also after an error: no copy of the call outlives it
  const cudaError_t se = cudaStreamSynchronize(cs);
  if (e == cudaSuccess) e = se;
  if (e != cudaSuccess) return fail_cuda(e);
  if (psnr) *psnr = 10.0 * std::log10((3.0 * 255.0 * 255.0) / (total / ((double)width * height)));
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_decode_logical(const uint8_t *blocks, size_t n,
                                          fastc_bc7_logical_block *out) {
  if ((!blocks || !out) && n) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  static const uint32_t part2[64] = {FASTC_PART2_WORDS};
  static const uint32_t part3[64] = {FASTC_PART3_WORDS};
  static const uint8_t anc2[64] = {FASTC_ANCHOR2_BYTES};
  static const uint8_t anc3[64] = {FASTC_ANCHOR3_BYTES};
  for (size_t b = 0; b < n; b++) {
    const uint8_t *blk = blocks + 16 * b;
    fastc_bc7_logical_block &o = out[b];
    std::memset(&o, 0, sizeof(o));
    int pos = 0;
    auto bits = [&](int k) {
      uint32_t v = 0;
      for (int i = 0; i < k; i++, pos++) v |= (uint32_t)((blk[pos >> 3] >> (pos & 7)) & 1) << i;
      return v;
    };
    int mode = 0;
    while (mode < 8 && !bits(1)) mode++;
    o.mode = (uint32_t)mode;
    if (mode >= 8) continue;
    const fastc::ModeAttr a = fastc::mode_attr(mode);
    o.subsets = (uint32_t)a.subsets;
    if (a.subsets > 1) o.shape = bits(a.part_bits);
    if (a.has_rotation) o.rotation = bits(2);
    if (a.has_idx_mode) o.index_mode = bits(1);
    for (int ch = 0; ch < 4; ch++) {
      const int nb = ch == 3 ? a.alpha_bits : a.color_bits;
      for (int s = 0; s < a.subsets; s++)
        for (int e = 0; e < 2; e++) o.endpoints[s][e][ch] = nb ? (uint8_t)bits(nb) : 0xFF;
      o.depth[ch] = (uint8_t)nb;
    }
    if (a.pbit != fastc::kPBitNone) {
      for (int s = 0; s < a.subsets; s++) {
        const uint32_t shared = a.pbit == fastc::kPBitShared ? bits(1) : 0;
        for (int e = 0; e < 2; e++) {
          const uint32_t pb = a.pbit == fastc::kPBitShared ? shared : bits(1);
          for (int ch = 0; ch < 4; ch++)
            if (o.depth[ch]) o.endpoints[s][e][ch] = (uint8_t)((o.endpoints[s][e][ch] << 1) | pb);
        }
      }
      for (int ch = 0; ch < 4; ch++)
        if (o.depth[ch]) o.depth[ch]++;
    }
    const uint32_t part = a.subsets == 2 ? part2[o.shape] : (a.subsets == 3 ? part3[o.shape] : 0u);
    auto anchor = [&](int s) {
      if (s == 0) return 0;
      if (a.subsets == 2) return (int)anc2[o.shape];
      return s == 1 ? (int)(anc3[o.shape] & 15) : (int)(anc3[o.shape] >> 4);
    };
    uint8_t first[16], second[16];
    for (int i = 0; i < 16; i++) {
      const int s = (int)((part >> (2 * i)) & 3);
      first[i] = (uint8_t)bits(anchor(s) == i ? a.idx_bits - 1 : a.idx_bits);
    }
    for (int i = 0; i < 16; i++)
      second[i] = a.alpha_idx_bits ? (uint8_t)bits(i == 0 ? a.alpha_idx_bits - 1 : a.alpha_idx_bits)
                                   : first[i];
    for (int i = 0; i < 16; i++) {
      o.indices[i] = o.index_mode ? second[i] : first[i];
      o.alpha_indices[i] = o.index_mode ? first[i] : second[i];
    }
  }
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_compress_device(const fastc_bc7_job *jobs, uint32_t n,
                                           const fastc_bc7_settings *settings,
                                           int per_job_settings, void *stream) {
  if (!jobs && n) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  if (n == 0) return FASTC_BC7_OK;
  fastc_bc7_settings dflt;
  fastc_bc7_settings_default(&dflt);
  std::vector<JobDev> dj(n);
  uint64_t total = 0;
  for (uint32_t i = 0; i < n; i++) {
    const fastc_bc7_settings &st = settings_for(settings, per_job_settings, i, dflt);
    fastc_bc7_status why;
    if (!settings_ok(st, &why)) return why;
    if (st.watermark_start == FASTC_BC7_WATERMARK_CONTINUE) return FASTC_BC7_ERR_INVALID_ARGUMENT;
    uint32_t first, count;
    if (!jobs[i].in || !jobs[i].out || !job_range(jobs[i], &first, &count) ||
        (reinterpret_cast<uintptr_t>(jobs[i].in) & 3) || (reinterpret_cast<uintptr_t>(jobs[i].out) & 3))
      return FASTC_BC7_ERR_INVALID_ARGUMENT;
    dj[i] = make_job(jobs[i], st, first, count, total);
    dj[i].flags = align_flags(jobs[i].in, jobs[i].out);
    total += count;
  }
  if (total == 0) return FASTC_BC7_OK;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    const int dev = current_device();
    if (dev < 0) return FASTC_BC7_ERR_NO_DEVICE;
    fastc::upload_tables(dev);
  }
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  LaunchShape shape;
  int engine;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    shape = pick_shape(total);
    engine = g_engine;
  }
  void *buf = nullptr;
  const size_t jb = (n * sizeof(JobDev) + 255) & ~(size_t)255;
  const int tb = task_bound_of(settings, per_job_settings, n);
  CK(cudaMallocAsync(&buf, jb + scratch_bytes(total, engine, tb), cs));
  cudaError_t e = cudaMemcpyAsync(buf, dj.data(), n * sizeof(JobDev), cudaMemcpyHostToDevice, cs);
  const int dev = current_device();
  ClassStreams *cls = engine == FASTC_BC7_ENGINE_PIPELINE ? acquire_class_streams(dev) : nullptr;
  if (e == cudaSuccess)
    e = (cudaError_t)launch_engine(static_cast<const JobDev *>(buf), (int)n, total,
                                   static_cast<uint8_t *>(buf) + jb, engine, shape, tb, cls, cs);
  release_class_streams(dev, cls);
  cudaError_t ef = cudaFreeAsync(buf, cs);
  if (e != cudaSuccess) return fail_cuda(e);
  if (ef != cudaSuccess) return fail_cuda(ef);
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_decompress_device(const uint8_t *blocks, uint8_t *rgba, uint32_t width,
                                             uint32_t height, int spec, void *stream) {
  if (!blocks || !rgba || width == 0 || height == 0) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  if (reinterpret_cast<uintptr_t>(rgba) & 3) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  const int le = fastc::launch_decode(blocks, rgba, width, height, spec, stream);
  if (le) return fail_cuda((cudaError_t)le);
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_plan_create(const fastc_bc7_job *jobs, uint32_t n,
                                       const fastc_bc7_settings *settings, int per_job_settings,
                                       fastc_bc7_plan *out) {
  if (!out || (!jobs && n) || n == 0) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  fastc_bc7_settings dflt;
  fastc_bc7_settings_default(&dflt);
  std::vector<JobDev> dj(n);
  uint64_t total = 0;
  for (uint32_t i = 0; i < n; i++) {
    const fastc_bc7_settings &st = settings_for(settings, per_job_settings, i, dflt);
    fastc_bc7_status why;
    if (!settings_ok(st, &why)) return why;
    if (st.watermark_start == FASTC_BC7_WATERMARK_CONTINUE) return FASTC_BC7_ERR_INVALID_ARGUMENT;
    uint32_t first, count;
    if (!jobs[i].in || !jobs[i].out || !job_range(jobs[i], &first, &count) ||
        (reinterpret_cast<uintptr_t>(jobs[i].in) & 3) || (reinterpret_cast<uintptr_t>(jobs[i].out) & 3))
      return FASTC_BC7_ERR_INVALID_ARGUMENT;
    dj[i] = make_job(jobs[i], st, first, count, total);
    dj[i].flags = align_flags(jobs[i].in, jobs[i].out);
    total += count;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  const int dev = current_device();
  if (dev < 0) return FASTC_BC7_ERR_NO_DEVICE;
  fastc::upload_tables(dev);
  fastc_bc7_plan p = new fastc_bc7_plan_s();
  p->device = dev;
  p->total = total;
  p->njobs = (int)n;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&p->d_jobs), n * sizeof(JobDev));
  p->engine = g_engine;
  p->warps = g_warps;
  p->task_bound = task_bound_of(settings, per_job_settings, n);
  p->scratch_size = scratch_bytes(total > 0 ? total : 1, p->engine, p->task_bound);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_scratch, p->scratch_size);
  if (e == cudaSuccess)
    e = cudaMemcpy(p->d_jobs, dj.data(), n * sizeof(JobDev), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    p->sc = carve_scratch(p->d_scratch, total);
    e = capture_plan(p, p->engine, p->warps, p->tune, &p->graph, &p->exec, &p->kernels);
  }
  if (e != cudaSuccess) {
    fastc_bc7_plan_destroy(p);
    return fail_cuda(e);
  }
  *out = p;
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_plan_launch(fastc_bc7_plan p, void *stream) {
  if (!p || !p->exec) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  CK(cudaGraphLaunch(p->exec, static_cast<cudaStream_t>(stream)));
  return FASTC_BC7_OK;
}

// Sets of at most this many blocks also try the warp-per-block engine.
constexpr uint64_t kSmallSetBlocks = 1ull << 16;

fastc_bc7_status fastc_bc7_plan_autotune(fastc_bc7_plan p, void *stream, uint32_t launches) {
  if (!p || !p->exec || launches == 0) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  if (p->engine != FASTC_BC7_ENGINE_PIPELINE) return FASTC_BC7_OK;  // nothing to tune
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0));
  cudaError_t e = cudaEventCreate(&e1);
  // times `launches` launches of an instantiated graph after one warm launch
  auto time_exec = [&](cudaGraphExec_t ex, float *ms) -> cudaError_t {
    cudaError_t r = cudaGraphLaunch(ex, st);
    if (r == cudaSuccess) r = cudaEventRecord(e0, st);
    for (uint32_t k = 0; k < launches && r == cudaSuccess; k++) r = cudaGraphLaunch(ex, st);
    if (r == cudaSuccess) r = cudaEventRecord(e1, st);
    if (r == cudaSuccess) r = cudaEventSynchronize(e1);
    if (r == cudaSuccess) r = cudaEventElapsedTime(ms, e0, e1);
    return r;
  };
  float best_ms = 0.0f;
  if (e == cudaSuccess) e = time_exec(p->exec, &best_ms);
  // tries one candidate and keeps its graph when it is faster
  auto trial = [&](int engine, int warps, const fastc::PipelineTuning &t) -> cudaError_t {
    if (engine == FASTC_BC7_ENGINE_PIPELINE &&
        rank_scratch_bytes(p->total) +
                fastc::pipeline_scratch_bytes(p->total, p->task_bound,
                                              fastc::device_sm_count(current_device()),
                                              t.chunk_blocks) >
            p->scratch_size)
      return cudaSuccess;  // needs more scratch than the plan holds
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ex = nullptr;
    uint64_t kern = 0;
    cudaError_t r = capture_plan(p, engine, warps, t, &g, &ex, &kern);
    float ms = 0.0f;
    if (r == cudaSuccess) r = time_exec(ex, &ms);
    if (r == cudaSuccess && ms < best_ms) {
      std::swap(g, p->graph);
      std::swap(ex, p->exec);
      p->kernels = kern;
      p->engine = engine;
      p->warps = warps;
      p->tune = t;
      best_ms = ms;
    }
    if (ex) cudaGraphExecDestroy(ex);
    if (g) cudaGraphDestroy(g);
    return r;
  };
  // coordinate search over the pipeline's launch parameters, each at the
  // best of the ones before: CTAs per SM of the annealing kernels, the
  // hand-on threshold, the chunk size, the select grid, the setup grid
  const int ctas[] = {3, 4, 5, 6, 7};
  const int yields[] = {8, 12, 16};
  const uint64_t dflt_chunk = fastc::pipeline_chunk(p->task_bound);
  const uint64_t chunks[] = {dflt_chunk, dflt_chunk / 2, dflt_chunk / 4};
  const int sel[] = {8, 16, 32};
  const int setup[] = {6, 12, 24, 128};
  const fastc::PipelineTuning base = p->tune;
  for (int phase = 0; phase < 5 && e == cudaSuccess && p->engine == FASTC_BC7_ENGINE_PIPELINE;
       phase++) {
    const int ncand = phase == 0 ? 5 : phase == 1 ? 3 : phase == 2 ? 3 : phase == 3 ? 3 : 4;
    for (int i = 0; i < ncand && e == cudaSuccess; i++) {
      fastc::PipelineTuning t = p->tune;
      if (phase == 0) t.anneal_ctas_per_sm = ctas[i];
      else if (phase == 1) t.yield_lanes = yields[i];
      else if (phase == 2) t.chunk_blocks = chunks[i] == dflt_chunk ? 0 : chunks[i];
      else if (phase == 3) t.select_ctas_per_sm = sel[i];
      else t.setup_ctas_per_sm = setup[i];
      if (t.anneal_ctas_per_sm == p->tune.anneal_ctas_per_sm && t.yield_lanes == p->tune.yield_lanes &&
          t.chunk_blocks == p->tune.chunk_blocks && t.select_ctas_per_sm == p->tune.select_ctas_per_sm &&
          t.setup_ctas_per_sm == p->tune.setup_ctas_per_sm)
        continue;
      e = trial(FASTC_BC7_ENGINE_PIPELINE, p->warps, t);
    }
  }
  // small sets: the warp-per-block engine (one persistent kernel instead of
  // the pipeline's stages) at 2, 4 or 8 warps per CTA
  if (p->total <= kSmallSetBlocks)
    for (int w : {2, 4, 8})
      if (e == cudaSuccess) e = trial(FASTC_BC7_ENGINE_WARP_PER_BLOCK, w, base);
  cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return fail_cuda(e);
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_plan_get_tuning(fastc_bc7_plan p, fastc_bc7_plan_tuning_info *out) {
  if (!p || !out) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::memset(out, 0, sizeof(*out));
  out->engine = p->engine;
  out->warps_per_cta = p->warps;
  out->anneal_ctas_per_sm = p->tune.anneal_ctas_per_sm;
  out->yield_lanes = p->tune.yield_lanes;
  out->select_ctas_per_sm = p->tune.select_ctas_per_sm;
  out->setup_ctas_per_sm = p->tune.setup_ctas_per_sm;
  out->chunk_blocks = fastc::pipeline_chunk_blocks(p->task_bound, p->tune);
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_plan_tuning(fastc_bc7_plan p, int *anneal_ctas_per_sm, int *yield_lanes) {
  if (!p || !anneal_ctas_per_sm || !yield_lanes) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  *anneal_ctas_per_sm = p->tune.anneal_ctas_per_sm;
  *yield_lanes = p->tune.yield_lanes;
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_plan_flags(fastc_bc7_plan p, uint32_t *flags) {
  if (!p || !flags) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(flags, p->sc.status, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  return FASTC_BC7_OK;
}

uint64_t fastc_bc7_plan_blocks(fastc_bc7_plan p) { return p ? p->total : 0; }

uint64_t fastc_bc7_plan_kernels(fastc_bc7_plan p) { return p ? p->kernels : 0; }

fastc_bc7_status fastc_bc7_plan_destroy(fastc_bc7_plan p) {
  if (!p) return FASTC_BC7_OK;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->d_jobs) cudaFree(p->d_jobs);
  if (p->d_scratch) cudaFree(p->d_scratch);
  delete p;
  return FASTC_BC7_OK;
}

void fastc_bc7_set_watermark_counter(uint32_t next_entry) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_wm_next = next_entry % 9u;
}

uint32_t fastc_bc7_get_watermark_counter(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_wm_next;
}

fastc_bc7_status fastc_bc7_set_launch_shape(int warps_per_cta, int ctas_per_sm) {
  if (warps_per_cta != 0 && warps_per_cta != 1 && warps_per_cta != 2 && warps_per_cta != 4 &&
      warps_per_cta != 8)
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  if (ctas_per_sm < 0 || ctas_per_sm > 64) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_mu);
  if (warps_per_cta) g_warps = warps_per_cta;
  if (ctas_per_sm) g_ctas_per_sm = ctas_per_sm;
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_set_engine(int engine) {
  if (engine != FASTC_BC7_ENGINE_PIPELINE && engine != FASTC_BC7_ENGINE_WARP_PER_BLOCK)
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_mu);
  g_engine = engine;
  return FASTC_BC7_OK;
}

int fastc_bc7_get_engine(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_engine;
}

fastc_bc7_status fastc_bc7_get_launch_shape(int *warps_per_cta, int *ctas_per_sm) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (warps_per_cta) *warps_per_cta = g_warps;
  if (ctas_per_sm) *ctas_per_sm = g_ctas_per_sm;
  return FASTC_BC7_OK;
}

}  // extern "C"
