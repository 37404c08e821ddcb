// Continuous-batching BC7 request server (fastc_bc7_server_* in
// include/fastc_bc7.h).
//
// A worker thread owns the GPU side. Requests queue in FIFO order; whenever
// one of `max_inflight` batch slots is free, the worker admits the pending
// requests that fit the device-memory budget (texels, blocks, job table and
// encoder scratch of the batch), uploads their texel rows, launches the
// encoder on the slot's stream and queues the copy of the blocks into
// pinned staging. A host callback on the stream wakes the worker when the
// batch is done; it copies the blocks to the callers' buffers and returns
// the memory to the budget. While one batch runs, the next is admitted,
// uploaded and launched on another stream, so requests that arrive during a
// batch overlap with it on the device. Each block's result depends only on
// its texture, position and settings, so a request gives the same bytes
// alone or in any mix. After the encode each request's blocks are decoded
// and compared with its texels on the device (FasTC's PSNR metric), so the
// server reports every request's quality beside its latency. DXT1 / DXT5
// requests (fastc_dxt_server_submit) share the queue, the budget and the
// batches: a batch's BC7 requests go through the BC7 encoder, its DXT ones
// through the DXT kernel, on the same stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bc7_host.h"
#include "bc7_kernels.cuh"
#include "dxt.cuh"
#include "fastc_bc7.h"

using fastc::JobDev;
using namespace fastc::host;

namespace {

using Clock = std::chrono::steady_clock;

enum ReqState { kPending = 0, kRunning = 1, kDone = 2, kFailed = 3, kCancelled = 4 };

struct Request {
  uint64_t id = 0;
  fastc_bc7_job job{};
  fastc_bc7_settings settings{};
  int format = 0;                 // 0: BC7, FASTC_DXT1, FASTC_DXT5
  uint32_t first = 0, count = 0;  // raster block range
  uint32_t row0 = 0;              // first texel row uploaded
  size_t in_bytes = 0, out_bytes = 0;
  ReqState state = kPending;
  fastc_bc7_status status = FASTC_BC7_OK;
  double sse = 0.0;               // FasTC's PSNR metric summed over the blocks
  Clock::time_point t_submit, t_done;
};

struct Slot {
  cudaStream_t stream = nullptr;
  fastc::ClassStreams *cls = nullptr;  // the pipeline's side streams
  void *dev = nullptr;
  uint8_t *pinned = nullptr;
  size_t pinned_cap = 0;
  size_t bytes = 0;  // budget held by the batch
  std::vector<Request *> reqs;
  std::vector<size_t> out_off;
  bool busy = false;
  bool finished = false;
  cudaError_t error = cudaSuccess;
};

size_t round_up(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

struct fastc_bc7_server_s {
  fastc_bc7_server_config cfg{};
  int device = 0;
  int engine = FASTC_BC7_ENGINE_PIPELINE;
  std::mutex mu;
  std::condition_variable cv_work;  // wakes the worker
  std::condition_variable cv_done;  // wakes waiters
  std::deque<Request *> pending;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  std::vector<Slot> slots;
  uint64_t next_id = 1;
  size_t in_use = 0, peak = 0;
  bool stop = false;
  std::thread worker;
  // statistics
  std::vector<double> latencies_ms;
  uint64_t submitted = 0, completed = 0, failed = 0, cancelled = 0, rejected = 0, batches = 0;
  uint64_t pixels = 0;
  double sse = 0.0;  // of the completed requests
  bool started = false;
  Clock::time_point t_first;
  Clock::time_point t_last;

  // device bytes a batch needs, beyond the per-request texels and blocks
  // (job table, the quality sums, BC7 encoder scratch for the most cluster
  // fits per block that the batch's mode masks allow; DXT needs none)
  size_t batch_overhead(uint64_t bc7_blocks, uint64_t blocks, size_t njobs, int task_bound) const {
    return round_up(njobs * sizeof(JobDev)) + round_up(njobs * sizeof(double)) +
           round_up(blocks * sizeof(double)) +
           (bc7_blocks ? scratch_bytes(bc7_blocks, engine, task_bound) : 0);
  }

  void loop();
  void launch(Slot &s);
  void retire(Slot &s);
};

namespace {

void CUDART_CB on_batch_done(void *arg) {
  auto *pair = static_cast<std::pair<fastc_bc7_server_s *, Slot *> *>(arg);
  fastc_bc7_server_s *srv = pair->first;
  Slot *s = pair->second;
  delete pair;
  std::lock_guard<std::mutex> lk(srv->mu);
  s->finished = true;
  srv->cv_work.notify_all();
}

}  // namespace

void fastc_bc7_server_s::launch(Slot &s) {
  // Called by the worker without the lock; s.reqs/out_off/bytes are set.
  cudaError_t e = cudaSuccess;
  uint64_t total = 0, bc7_total = 0;
  size_t in_total = 0, out_total = 0;
  std::vector<size_t> in_off(s.reqs.size());
  s.out_off.assign(s.reqs.size(), 0);
  int tb = 0;
  for (size_t i = 0; i < s.reqs.size(); i++) {
    const Request &r = *s.reqs[i];
    in_off[i] = in_total;
    s.out_off[i] = out_total;
    in_total += round_up(r.in_bytes);
    out_total += round_up(r.out_bytes);
    total += r.count;
    if (r.format == 0) {
      bc7_total += r.count;
      tb = std::max(tb, fastc::block_task_bound(r.settings.block_modes));
    }
  }
  const size_t table = round_up(s.reqs.size() * sizeof(JobDev));
  const size_t sums = round_up(s.reqs.size() * sizeof(double));  // per-request error
  const size_t errs = round_up(total * sizeof(double));          // per-block error
  const size_t need = in_total + out_total + table + sums + errs +
                      (bc7_total ? scratch_bytes(bc7_total, engine, tb) : 0);
  if (s.pinned_cap < out_total + sums) {
    if (s.pinned) cudaFreeHost(s.pinned);
    s.pinned = nullptr;
    s.pinned_cap = 0;
    e = cudaMallocHost(reinterpret_cast<void **>(&s.pinned), out_total + sums);
    if (e == cudaSuccess) s.pinned_cap = out_total + sums;
  }
  if (e == cudaSuccess) e = cudaMallocAsync(&s.dev, need, s.stream);
  if (e == cudaSuccess) {
    uint8_t *din = static_cast<uint8_t *>(s.dev);
    uint8_t *dout = din + in_total;
    JobDev *dtab = reinterpret_cast<JobDev *>(dout + out_total);
    double *dsum = reinterpret_cast<double *>(reinterpret_cast<uint8_t *>(dtab) + table);
    double *derr = reinterpret_cast<double *>(reinterpret_cast<uint8_t *>(dsum) + sums);
    void *scratch = reinterpret_cast<uint8_t *>(derr) + errs;
    // BC7 requests: the encoder's job table; DXT1 / DXT5 requests: the DXT
    // kernel's launch parameters
    std::vector<JobDev> dj, dxt[2];
    uint64_t begin = 0;
    for (size_t i = 0; i < s.reqs.size() && e == cudaSuccess; i++) {
      Request &r = *s.reqs[i];
      JobDev d = make_job(r.job, r.settings, r.first, r.count, r.format == 0 ? begin : 0);
      d.in = din + in_off[i];
      d.out = dout + s.out_off[i];
      d.row0 = r.row0;
      d.out_first = r.first;
      if (r.format == 0) {
        d.flags = fastc::kJobIn16 | fastc::kJobOut16;
        dj.push_back(d);
        begin += r.count;
      } else {
        d.flags = fastc::kJobIn16 | (r.format == FASTC_DXT5 ? fastc::kJobOut16 : 0u);
        dxt[r.format == FASTC_DXT5].push_back(d);
      }
      const uint8_t *src = r.job.in + (size_t)r.row0 * r.job.width * 4;
      e = cudaMemcpyAsync(din + in_off[i], src, r.in_bytes, cudaMemcpyHostToDevice, s.stream);
    }
    if (e == cudaSuccess && !dj.empty())
      e = cudaMemcpyAsync(dtab, dj.data(), dj.size() * sizeof(JobDev), cudaMemcpyHostToDevice,
                          s.stream);
    if (e == cudaSuccess && !dj.empty()) {
      fastc::LaunchShape shape;
      {
        std::lock_guard<std::mutex> lk(g_mu);
        shape = pick_shape(bc7_total);
      }
      // batches share the GPU with other batches' stages, which fill the
      // tails of concurrent setups: never the one-stream setup
      fastc::PipelineTuning tune;
      tune.serial_setup = 0;
      e = (cudaError_t)launch_engine(dtab, (int)dj.size(), bc7_total, scratch, engine, shape, tb,
                                     s.cls, tune, s.stream, nullptr, nullptr);
    }
    for (int a = 0; a < 2 && e == cudaSuccess; a++)
      if (!dxt[a].empty())
        e = fastc::dxt_encode_jobs(dxt[a].data(), (uint32_t)dxt[a].size(), a == 1, s.stream);
    uint64_t at = 0;  // each request's quality, from its uploaded texels and its blocks
    for (size_t i = 0; i < s.reqs.size() && e == cudaSuccess; i++) {
      const Request &r = *s.reqs[i];
      if (r.format == 0)
        e = (cudaError_t)fastc::launch_range_error(dout + s.out_off[i], din + in_off[i], r.job.width,
                                                   r.row0, r.first, r.count, derr + at, dsum + i,
                                                   s.stream);
      else
        e = fastc::dxt_range_error(dout + s.out_off[i], din + in_off[i], r.job.width, r.row0, r.first,
                                   r.count, r.format == FASTC_DXT5, derr + at, dsum + i, s.stream);
      at += r.count;
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s.pinned, dout, out_total, cudaMemcpyDeviceToHost, s.stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s.pinned + out_total, dsum, s.reqs.size() * sizeof(double),
                          cudaMemcpyDeviceToHost, s.stream);
    cudaFreeAsync(s.dev, s.stream);
    s.dev = nullptr;
  }
  if (e == cudaSuccess) {
    auto *arg = new std::pair<fastc_bc7_server_s *, Slot *>(this, &s);
    e = cudaLaunchHostFunc(s.stream, on_batch_done, arg);
    if (e != cudaSuccess) delete arg;
  }
  if (e != cudaSuccess) {
    // drain what was enqueued before the error: no upload may still read a
    // request's texels once the request is reported failed
    cudaStreamSynchronize(s.stream);
    std::lock_guard<std::mutex> lk(mu);
    s.error = e;
    s.finished = true;
  }
}

void fastc_bc7_server_s::retire(Slot &s) {
  // Called by the worker without the lock, after the batch finished.
  if (s.error == cudaSuccess) {
    size_t out_total = 0;
    for (size_t i = 0; i < s.reqs.size(); i++) out_total += round_up(s.reqs[i]->out_bytes);
    for (size_t i = 0; i < s.reqs.size(); i++) {
      Request &r = *s.reqs[i];
      std::memcpy(r.job.out + (size_t)r.first * (r.out_bytes / std::max<uint32_t>(r.count, 1)),
                s.pinned + s.out_off[i], r.out_bytes);
      std::memcpy(&r.sse, s.pinned + out_total + i * sizeof(double), sizeof(double));
    }
  }
  const Clock::time_point now = Clock::now();
  std::lock_guard<std::mutex> lk(mu);
  for (Request *r : s.reqs) {
    r->t_done = now;
    if (s.error == cudaSuccess) {
      r->state = kDone;
      completed++;
      pixels += (uint64_t)r->count * 16;
      sse += r->sse;
      latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - r->t_submit).count());
    } else {
      r->state = kFailed;
      r->status = fail_cuda(s.error);
      failed++;
    }
  }
  t_last = now;
  in_use -= s.bytes;
  s.bytes = 0;
  s.reqs.clear();
  s.busy = false;
  s.finished = false;
  s.error = cudaSuccess;
  cv_done.notify_all();
}

void fastc_bc7_server_s::loop() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    // retire finished batches
    for (Slot &s : slots) {
      if (s.busy && s.finished) {
        lk.unlock();
        retire(s);
        lk.lock();
      }
    }
    // admit pending requests into a free slot
    Slot *free_slot = nullptr;
    for (Slot &s : slots)
      if (!s.busy) {
        free_slot = &s;
        break;
      }
    if (free_slot && !pending.empty()) {
      std::vector<Request *> batch;
      uint64_t blocks = 0, bc7_blocks = 0;
      size_t data = 0;
      int tb = 0;
      // A batch takes at most its share of the budget (budget / slots), so
      // that when the queue is long, batches stay small enough for every
      // slot to be in flight (a larger batch also needs the pipeline's
      // second chunk buffer); a single request may use the whole budget.
      const size_t share = cfg.memory_budget / cfg.max_inflight;
      while (!pending.empty() && batch.size() < cfg.max_batch_jobs) {
        Request *r = pending.front();
        const uint64_t nb = blocks + r->count;
        const uint64_t nb7 = bc7_blocks + (r->format == 0 ? r->count : 0);
        const size_t nd = data + round_up(r->in_bytes) + round_up(r->out_bytes);
        const int ntb =
            r->format == 0 ? std::max(tb, fastc::block_task_bound(r->settings.block_modes)) : tb;
        const size_t need = nd + batch_overhead(nb7, nb, batch.size() + 1, ntb);
        if (!batch.empty() && (nb > cfg.max_batch_blocks || need > share)) break;
        if (in_use + need > cfg.memory_budget) break;
        pending.pop_front();
        r->state = kRunning;
        batch.push_back(r);
        blocks = nb;
        bc7_blocks = nb7;
        data = nd;
        tb = ntb;
      }
      if (!batch.empty()) {
        free_slot->busy = true;
        free_slot->finished = false;
        free_slot->reqs = batch;
        free_slot->bytes = data + batch_overhead(bc7_blocks, blocks, batch.size(), tb);
        in_use += free_slot->bytes;
        peak = std::max(peak, in_use);
        batches++;
        lk.unlock();
        launch(*free_slot);
        lk.lock();
        continue;
      }
    }
    bool busy = false;
    for (Slot &s : slots) busy = busy || s.busy;
    if (stop && pending.empty() && !busy) break;
    cv_work.wait(lk);
  }
}

extern "C" {

void fastc_bc7_server_config_default(fastc_bc7_server_config *c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->memory_budget = (size_t)8 << 30;
  c->max_inflight = 3;
  c->max_batch_blocks = 1u << 22;
  c->max_batch_jobs = 4096;
}

fastc_bc7_status fastc_bc7_server_create(const fastc_bc7_server_config *cfg,
                                         fastc_bc7_server *out) {
  if (!out) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  fastc_bc7_server_config c;
  fastc_bc7_server_config_default(&c);
  if (cfg) c = *cfg;
  if (c.max_inflight == 0 || c.max_inflight > 16 || c.max_batch_jobs == 0 || c.memory_budget == 0)
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  const int dev = current_device();
  if (dev < 0) return FASTC_BC7_ERR_NO_DEVICE;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    fastc::upload_tables(dev);
  }
  {
    const cudaError_t e = fastc::dxt_prepare(dev);
    if (e != cudaSuccess) return fail_cuda(e);
  }
  auto *s = new fastc_bc7_server_s();
  s->cfg = c;
  s->device = dev;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    s->engine = g_engine;
  }
  s->slots.resize(c.max_inflight);
  for (Slot &sl : s->slots) {
    const cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) sl.cls = acquire_class_streams(dev);
    if (e != cudaSuccess) {
      for (Slot &x : s->slots)
        if (x.stream) cudaStreamDestroy(x.stream);
      delete s;
      return fail_cuda(e);
    }
  }
  s->worker = std::thread([s] { s->loop(); });
  *out = s;
  return FASTC_BC7_OK;
}

// Queues a request of format 0 (BC7, with settings st) or FASTC_DXT1 / DXT5.
static fastc_bc7_status submit_request(fastc_bc7_server s, const fastc_bc7_job *job,
                                       const fastc_bc7_settings &st, int format, uint64_t *id) {
  uint32_t first, count;
  if (!job->in || !job->out || !job_range(*job, &first, &count)) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  auto r = std::make_unique<Request>();
  r->job = *job;
  r->settings = st;
  r->format = format;
  r->first = first;
  r->count = count;
  const uint32_t bw = job->width / 4;
  const uint32_t r0 = count ? first / bw : 0, r1 = count ? (first + count - 1) / bw : 0;
  r->row0 = r0 * 4;
  r->in_bytes = count ? (size_t)(r1 - r0 + 1) * 4 * job->width * 4 : 0;
  r->out_bytes = (size_t)count * (format == FASTC_DXT1 ? 8 : 16);
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  const size_t alone =
      round_up(r->in_bytes) + round_up(r->out_bytes) +
      s->batch_overhead(format == 0 ? count : 0, count, 1,
                        format == 0 ? fastc::block_task_bound(r->settings.block_modes) : 0);
  s->submitted++;
  if (!s->started) {
    s->started = true;
    s->t_first = r->t_submit;
  }
  r->id = s->next_id++;
  *id = r->id;
  if (alone > s->cfg.memory_budget) {
    r->state = kFailed;
    r->status = FASTC_BC7_ERR_BUDGET;
    s->rejected++;
    s->reqs.emplace(r->id, std::move(r));
    return FASTC_BC7_ERR_BUDGET;
  }
  if (count == 0) {
    r->state = kDone;
    r->t_done = r->t_submit;
    s->completed++;
    s->reqs.emplace(r->id, std::move(r));
    s->cv_done.notify_all();
    return FASTC_BC7_OK;
  }
  s->pending.push_back(r.get());
  s->reqs.emplace(r->id, std::move(r));
  s->cv_work.notify_all();
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_server_submit(fastc_bc7_server s, const fastc_bc7_job *job,
                                         const fastc_bc7_settings *settings, uint64_t *id) {
  if (!s || !job || !id) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  fastc_bc7_settings st;
  fastc_bc7_settings_default(&st);
  if (settings) st = *settings;
  fastc_bc7_status why;
  if (!settings_ok(st, &why)) return why;
  if (st.watermark_start == FASTC_BC7_WATERMARK_CONTINUE) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  return submit_request(s, job, st, 0, id);
}

fastc_bc7_status fastc_dxt_server_submit(fastc_bc7_server s, const fastc_bc7_job *job, int format,
                                         uint64_t *id) {
  if (!s || !job || !id || (format != FASTC_DXT1 && format != FASTC_DXT5))
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  fastc_bc7_settings st;
  fastc_bc7_settings_default(&st);
  return submit_request(s, job, st, format, id);
}

// FasTC's Image::ComputePSNR from a summed error (Base/src/Image.cpp:206-255):
// peak 3 * 255^2 over the mean per texel; 0 texels give 0.
static double psnr_of(double sse, uint64_t texels) {
  if (texels == 0) return 0.0;
  return 10.0 * std::log10((3.0 * 255.0 * 255.0) / (sse / (double)texels));
}

static fastc_bc7_status state_status(const Request &r) {
  switch (r.state) {
    case kDone: return FASTC_BC7_OK;
    case kFailed: return r.status;
    case kCancelled: return FASTC_BC7_ERR_CANCELLED;
    default: return FASTC_BC7_ERR_TIMEOUT;
  }
}

fastc_bc7_status fastc_bc7_server_poll(fastc_bc7_server s, uint64_t id) {
  if (!s) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return FASTC_BC7_ERR_NOT_FOUND;
  return state_status(*it->second);
}

fastc_bc7_status fastc_bc7_server_wait(fastc_bc7_server s, uint64_t id, int64_t timeout_ms) {
  if (!s) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return FASTC_BC7_ERR_NOT_FOUND;
  Request *r = it->second.get();
  auto finished = [r] { return r->state == kDone || r->state == kFailed || r->state == kCancelled; };
  if (timeout_ms < 0) {
    s->cv_done.wait(lk, finished);
  } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), finished)) {
    return FASTC_BC7_ERR_TIMEOUT;
  }
  return state_status(*r);
}

fastc_bc7_status fastc_bc7_server_cancel(fastc_bc7_server s, uint64_t id) {
  if (!s) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return FASTC_BC7_ERR_NOT_FOUND;
  Request *r = it->second.get();
  if (r->state == kRunning) return FASTC_BC7_ERR_INVALID_ARGUMENT;  // already on the GPU
  if (r->state != kPending) return state_status(*r);
  s->pending.erase(std::find(s->pending.begin(), s->pending.end(), r));
  r->state = kCancelled;
  r->t_done = Clock::now();
  s->cancelled++;
  s->cv_done.notify_all();
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_server_release(fastc_bc7_server s, uint64_t id) {
  if (!s) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return FASTC_BC7_ERR_NOT_FOUND;
  const ReqState st = it->second->state;
  if (st == kPending || st == kRunning) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  s->reqs.erase(it);
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_server_get_stats(fastc_bc7_server s, fastc_bc7_server_stats *out) {
  if (!s || !out) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->cancelled = s->cancelled;
  out->rejected = s->rejected;
  out->batches = s->batches;
  out->pixels_completed = s->pixels;
  out->bytes_in_use = s->in_use;
  out->peak_bytes = s->peak;
  std::vector<double> l = s->latencies_ms;
  if (!l.empty()) {
    std::sort(l.begin(), l.end());
    auto pct = [&l](double q) {
      const size_t i = (size_t)std::min<double>((double)(l.size() - 1), q * (double)(l.size() - 1) + 0.5);
      return l[i];
    };
    out->p50_latency_ms = pct(0.50);
    out->p99_latency_ms = pct(0.99);
    out->max_latency_ms = l.back();
    double sum = 0;
    for (double v : l) sum += v;
    out->mean_latency_ms = sum / (double)l.size();
  }
  if (s->started && s->completed) {
    const double secs = std::chrono::duration<double>(s->t_last - s->t_first).count();
    out->mpix_per_s = secs > 0 ? (double)s->pixels / secs / 1e6 : 0.0;
  }
  out->psnr_db = psnr_of(s->sse, s->pixels);
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_server_request_psnr(fastc_bc7_server s, uint64_t id, double *psnr) {
  if (!s || !psnr) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return FASTC_BC7_ERR_NOT_FOUND;
  const Request &r = *it->second;
  const fastc_bc7_status st = state_status(r);
  if (st != FASTC_BC7_OK) return st;
  *psnr = psnr_of(r.sse, (uint64_t)r.count * 16);
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_bc7_server_destroy(fastc_bc7_server s) {
  if (!s) return FASTC_BC7_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  for (Slot &sl : s->slots) {
    if (sl.stream) {
      cudaStreamSynchronize(sl.stream);
      cudaStreamDestroy(sl.stream);
    }
    release_class_streams(s->device, sl.cls);
    if (sl.pinned) cudaFreeHost(sl.pinned);
  }
  delete s;
  return FASTC_BC7_OK;
}

}  // extern "C"
