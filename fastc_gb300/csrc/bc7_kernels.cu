// BC7 (BPTC) encode/decode kernels for sm_103a.
//
// Encode pipeline, all on one stream:
//   1. classify_kernel  one thread per block: single-colour flag and its
//                        rank inside a 1024-block chunk (CTA-wide scan).
//   2. scan_kernel      one CTA: exclusive prefix of the chunk counts, so a
//                        block's single-colour rank is global; resets the
//                        work counter.
//   3. encode_kernel    persistent; one warp owns one 4x4 block at a time,
//                        pulling block indices from an atomic counter (this
//                        replaces FasTC's ThreadGroup / WorkerQueue /
//                        CompressAtomic host scheduling). The warp stages the
//                        16 texels in shared memory with 128-bit loads,
//                        estimates the 64 two-subset and 64 three-subset
//                        shapes two per lane, runs one cluster fit
//                        (mode x subset x rotation x index mode) per lane,
//                        then lane 0 picks the winner and packs 128 bits.
//
// The file is compiled once per warp count of the encoder
// (FASTC_WPB_WARPS = 1, 2, 4 or 8), each object holding one instantiation
// of encode_kernel so that the four compile in parallel; the object built
// with FASTC_WPB_WARPS == 4 (the default) also holds the rest of the file.
// The tables below have internal linkage, one copy per object.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <cstdio>

#include "bc7_encode.cuh"
#include "bc7_format.cuh"
#include "bc7_kernels.cuh"
#include "bc7_block.cuh"
#include "bc7_pipeline.cuh"

#ifndef FASTC_WPB_WARPS
#define FASTC_WPB_WARPS 4
#endif
#define FASTC_WPB_MAIN (FASTC_WPB_WARPS == 4)
#define FASTC_CAT2(a, b) a##b
#define FASTC_CAT(a, b) FASTC_CAT2(a, b)

namespace fastc {

static __constant__ uint32_t c_part2[64] = {FASTC_PART2_WORDS};
static __constant__ uint32_t c_part3[64] = {FASTC_PART3_WORDS};
static __constant__ uint8_t c_anchor2[64] = {FASTC_ANCHOR2_BYTES};
static __constant__ uint8_t c_anchor3[64] = {FASTC_ANCHOR3_BYTES};
static __constant__ uint32_t c_watermark[9] = {FASTC_WATERMARK_WORDS};
// Single-colour mode-5 endpoints: byte 0 = 7-bit first, byte 1 = 7-bit second.
static __constant__ uint32_t c_opt7[256];
// Mode-4 constant-alpha endpoints: byte 0 = a1, byte 1 = a2.
static __constant__ uint32_t c_opt6[256];

// The per-warp-count objects: launch, occupancy and table upload of their
// encode_kernel instantiation.
int wpb_launch_w1(const JobDev *, int, uint64_t, const EncodeScratch &, int, cudaStream_t);
int wpb_launch_w2(const JobDev *, int, uint64_t, const EncodeScratch &, int, cudaStream_t);
int wpb_launch_w4(const JobDev *, int, uint64_t, const EncodeScratch &, int, cudaStream_t);
int wpb_launch_w8(const JobDev *, int, uint64_t, const EncodeScratch &, int, cudaStream_t);
int wpb_occupancy_w1();
int wpb_occupancy_w2();
int wpb_occupancy_w4();
int wpb_occupancy_w8();
void wpb_upload_w1(const uint32_t *opt7, const uint32_t *opt6);
void wpb_upload_w2(const uint32_t *opt7, const uint32_t *opt6);
void wpb_upload_w4(const uint32_t *opt7, const uint32_t *opt6);
void wpb_upload_w8(const uint32_t *opt7, const uint32_t *opt6);

#if FASTC_WPB_MAIN


// ---------------------------------------------------------------------------
// Host-side generation of the two endpoint lookup tables, from the generator
// FasTC documents beside them (BPTCEncoder/src/BCLookupTables.h:44-95 and
// :355-449): for every 8-bit value, the endpoint pair whose interpolant lands
// closest to it.
// ---------------------------------------------------------------------------

static void build_endpoint_tables(uint32_t opt7[256], uint32_t opt6[256]) {
  uint32_t vals[256];
  uint32_t n = 0, last = 0xFFFFFFFFu;
  for (uint32_t i = 0; i < 256; i++) {
    const uint32_t num = ((i >> 1) << 1) | (i >> 7);
    if (num != last) vals[n++] = last = num;
  }
  for (uint32_t i = 0; i < 256; i++) {
    uint32_t best = 0xFFFFFFFFu, bj = 0, bk = 0;
    for (uint32_t j = 0; j < n; j++)
      for (uint32_t k = 0; k < n; k++) {
        const uint32_t c = (43 * vals[j] + 21 * vals[k] + 32) >> 6;
        const uint32_t d = i > c ? i - c : c - i;
        if (d < best) {
          best = d;
          bj = j;
          bk = k;
        }
      }
    opt7[i] = (vals[bj] >> 1) | ((vals[bk] >> 1) << 8);
  }
  // 6-bit table: entry[s] = {kind flag, lo, hi} with the better of the
  // midpoint and one-third fits first.
  n = 0;
  last = 0xFFFFFFFFu;
  for (uint32_t i = 0; i < 256; i++) {
    const uint32_t num = ((i >> 2) << 2) | (i >> 6);
    if (num != last) vals[n++] = last = num;
  }
  for (uint32_t i = 0; i < 256; i++) {
    uint32_t e[2][4] = {{1, 0, 0, 0xFFFFFFFFu}, {0, 0, 0, 0xFFFFFFFFu}};
    for (int kind = 0; kind < 2; kind++) {
      uint32_t best = 0xFFFFFFFFu, bj = 0, bk = 0;
      for (uint32_t j = 0; j < n; j++)
        for (uint32_t k = j; k < n; k++) {
          const uint32_t c = kind == 0 ? (vals[j] + vals[k]) / 2 : (2 * vals[j] + vals[k]) / 3;
          const uint32_t d = i > c ? i - c : c - i;
          if (d < best) {
            best = d;
            bj = j;
            bk = k;
          }
        }
      e[kind][1] = vals[bj] >> 2;
      e[kind][2] = vals[bk] >> 2;
      e[kind][3] = best;
    }
    const int first = e[1][3] > e[0][3] ? 0 : 1;
    const uint32_t *t0 = e[first], *t1 = e[1 - first];
    // FasTC's mode-4 constant-alpha rule (Compressor.cpp:731-747), with
    // both lookups at the same alpha value.
    uint32_t a1, a2;
    if (t0[0]) {
      a1 = (t1[1] << 2) | (t0[1] >> 4);
      a2 = (t1[2] << 2) | (t0[1] >> 4);
    } else {
      a1 = (t0[1] << 2) | (t0[1] >> 4);
      a2 = (t0[2] << 2) | (t0[1] >> 4);
    }
    opt6[i] = (a1 & 0xFF) | ((a2 & 0xFF) << 8);
  }
}

void upload_tables(int device) {
  static bool done[64] = {false};
  if (device < 0 || device >= 64 || done[device]) return;
  uint32_t opt7[256], opt6[256];
  build_endpoint_tables(opt7, opt6);
  wpb_upload_w1(opt7, opt6);
  wpb_upload_w2(opt7, opt6);
  wpb_upload_w4(opt7, opt6);
  wpb_upload_w8(opt7, opt6);
  upload_pipeline_tables(device, opt7, opt6);
  done[device] = true;
}

int device_sm_count(int device) {
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
  return n > 0 ? n : 1;
}
#endif  // FASTC_WPB_MAIN

// ---------------------------------------------------------------------------
// Job lookup and block loads
// ---------------------------------------------------------------------------

__device__ __forceinline__ int find_job(const JobDev *jobs, int njobs, uint64_t g) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].begin <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Row r (0..3) of raster block `lin` of job `jb`: four texels.
__device__ __forceinline__ uint4 load_row(const JobDev &jb, uint32_t lin, int r) {
  const uint32_t bw = jb.width >> 2;
  const uint32_t bx = lin % bw, by = lin / bw;
  const size_t off =
      ((size_t)(by * 4 + r - jb.row0) * jb.width + (size_t)bx * 4) * 4;
  const uint8_t *p = jb.in + off;
  if (jb.flags & kJobIn16) return __ldg(reinterpret_cast<const uint4 *>(p));
  const uint32_t *q = reinterpret_cast<const uint32_t *>(p);
  return make_uint4(__ldg(q), __ldg(q + 1), __ldg(q + 2), __ldg(q + 3));
}

__device__ __forceinline__ void store_block(const JobDev &jb, uint32_t lin, const uint32_t w[4]) {
  uint8_t *dst = jb.out + (size_t)(lin - jb.out_first) * 16;
  if (jb.flags & kJobOut16) {
    *reinterpret_cast<uint4 *>(dst) = make_uint4(w[0], w[1], w[2], w[3]);
  } else {
    uint32_t *d = reinterpret_cast<uint32_t *>(dst);
    d[0] = w[0];
    d[1] = w[1];
    d[2] = w[2];
    d[3] = w[3];
  }
}

#if FASTC_WPB_MAIN
// ---------------------------------------------------------------------------
// 1+2. Single-colour watermark ranks
// ---------------------------------------------------------------------------

// CTA b ranks the blocks of rank chunk r0 + b.
__global__ void __launch_bounds__(kRankChunk) classify_kernel(const JobDev *jobs, int njobs,
                                                              uint64_t total,
                                                              uint16_t *rank_local,
                                                              uint32_t *chunk_total, uint32_t r0) {
  __shared__ uint32_t s_warp[32];
  const uint32_t rc = r0 + blockIdx.x;
  const uint64_t g = (uint64_t)rc * kRankChunk + threadIdx.x;
  bool same = false;
  if (g < total) {
    const JobDev &jb = jobs[find_job(jobs, njobs, g)];
    const uint32_t lin = jb.first + (uint32_t)(g - jb.begin);
    const uint4 r0 = load_row(jb, lin, 0);
    same = r0.y == r0.x && r0.z == r0.x && r0.w == r0.x;
#pragma unroll
    for (int r = 1; r < 4; r++) {
      const uint4 v = load_row(jb, lin, r);
      same = same && v.x == r0.x && v.y == r0.x && v.z == r0.x && v.w == r0.x;
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t bal = __ballot_sync(0xFFFFFFFFu, same);
  if (lane == 0) s_warp[wid] = __popc(bal);
  __syncthreads();
  if (wid == 0) {
    const uint32_t v = s_warp[lane];
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += t;
    }
    s_warp[lane] = incl - v;
    if (lane == 31) chunk_total[rc] = incl;
  }
  __syncthreads();
  if (g < total)
    rank_local[g] = (uint16_t)(s_warp[wid] + __popc(bal & ((1u << lane) - 1u)));
}

// Exclusive scan of the chunk counts [r0, r1) in place, continuing from
// *carry (the single-colour blocks before chunk r0; r0 == 0 starts from 0
// and resets the work counter and status); leaves the running total in
// *carry and in *singles. One CTA.
__global__ void __launch_bounds__(1024) scan_range_kernel(uint32_t *chunk, uint32_t r0, uint32_t r1,
                                                          uint32_t *carry, unsigned long long *counter,
                                                          uint32_t *status, uint32_t *singles) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    s_carry = r0 == 0 ? 0u : *carry;
    if (r0 == 0) {
      *counter = 0ull;
      *status = 0u;
    }
  }
  __syncthreads();
  for (uint32_t base = r0; base < r1; base += 1024) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < r1 ? chunk[i] : 0u;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      const uint32_t w = s_warp[lane];
      uint32_t wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
        if (lane >= o) wi += t;
      }
      s_warp[lane] = wi - w;
    }
    __syncthreads();
    const uint32_t c = s_carry;
    if (i < r1) chunk[i] = c + s_warp[wid] + incl - v;
    __syncthreads();
    if (threadIdx.x == 1023) s_carry = c + s_warp[wid] + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *carry = s_carry;
    *singles = s_carry;
  }
}

// Exclusive scan of the chunk counts, in place; also resets the counter.
__global__ void __launch_bounds__(1024) scan_kernel(uint32_t *chunk, uint32_t nchunks,
                                                     unsigned long long *counter,
                                                     uint32_t *status, uint32_t *singles) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    s_carry = 0;
    *counter = 0ull;
    *status = 0u;
  }
  __syncthreads();
  for (uint32_t base = 0; base < nchunks; base += 1024) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < nchunks ? chunk[i] : 0u;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      const uint32_t w = s_warp[lane];
      uint32_t wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
        if (lane >= o) wi += t;
      }
      s_warp[lane] = wi - w;
    }
    __syncthreads();
    const uint32_t carry = s_carry;
    if (i < nchunks) chunk[i] = carry + s_warp[wid] + incl - v;
    __syncthreads();
    if (threadIdx.x == 1023) s_carry = carry + s_warp[wid] + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *singles = s_carry;
}

#endif  // FASTC_WPB_MAIN

// ---------------------------------------------------------------------------
// 3. Encoder
// ---------------------------------------------------------------------------

template <int kWarps>
__global__ void __launch_bounds__(kWarps * 32) encode_kernel(
    const JobDev *__restrict__ jobs, int njobs, uint64_t total,
    const uint16_t *__restrict__ rank_local, const uint32_t *__restrict__ chunk_prefix,
    unsigned long long *counter, uint32_t *status) {
  __shared__ uint32_t s_part2[64], s_part3[64];
  __shared__ uint8_t s_anc2[64], s_anc3[64];
  __shared__ uint32_t s_px[kWarps][16];
  __shared__ FitOut s_fit[kWarps][kMaxTasks];
  for (int i = threadIdx.x; i < 64; i += blockDim.x) {
    s_part2[i] = c_part2[i];
    s_part3[i] = c_part3[i];
    s_anc2[i] = c_anchor2[i];
    s_anc3[i] = c_anchor3[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t *px = s_px[wid];
  FitOut *fit = s_fit[wid];
  for (;;) {
    unsigned long long g = 0;
    if (lane == 0) g = atomicAdd(counter, 1ull);
    g = __shfl_sync(0xFFFFFFFFu, g, 0);
    if (g >= total) break;
    const JobDev &jb = jobs[find_job(jobs, njobs, g)];
    const uint32_t lin = jb.first + (uint32_t)(g - jb.begin);
    const uint32_t bwid = jb.width >> 2;
    const uint32_t bx = lin % bwid, by = lin / bwid;
    if (lane < 4) {
      const uint4 v = load_row(jb, lin, lane);
      px[lane * 4 + 0] = v.x;
      px[lane * 4 + 1] = v.y;
      px[lane * 4 + 2] = v.z;
      px[lane * 4 + 3] = v.w;
    }
    __syncwarp();
    bool same = true, transparent = true;
    for (int i = 0; i < 16; i++) {
      same = same && px[i] == px[0];
      transparent = transparent && (px[i] >> 24) == 0;
    }
    uint32_t out[4];
    if (same) {
      if (lane == 0) {
        const uint64_t gb = jb.begin;
        const uint32_t rg = chunk_prefix[g / kRankChunk] + rank_local[g];
        const uint32_t rb = (jb.flags & kJobWmGlobal)
                                ? 0u
                                : chunk_prefix[gb / kRankChunk] + rank_local[gb];
        single_color_block(px[0], jb.wm_start + (rg - rb), c_opt7, c_watermark, out);
        store_block(jb, lin, out);
      }
      __syncwarp();
      continue;
    }
    if (transparent) {
      if (lane == 0) {
        out[0] = 1u << 6;
        out[1] = out[2] = out[3] = 0;
        store_block(jb, lin, out);
      }
      __syncwarp();
      continue;
    }
    const Selection sel = box_selection_warp(px, s_part2, s_part3, (int)jb.metric, lane);
    uint32_t modes = sel.modes & jb.modes;
    if (modes == 0) modes = jb.modes & 0xFF;  // FasTC: undefined behaviour
    Task tk{0, 0, 0, 0, 0};
    int ntasks = enumerate_tasks(sel, modes, -1, tk);
    if (ntasks > kMaxTasks) {  // not reachable with BC7's mode table
      if (lane == 0) atomicOr(status, kStatusTaskOverflow);
      modes = 0u;  // the combine step below then finds no mode
      ntasks = 0;
    }
    for (int t = lane; t < ntasks && t < kMaxTasks; t += 32) {
      enumerate_tasks(sel, modes, t, tk);
      run_task(tk, sel, px, s_part2, s_part3, c_opt6, jb, bx, by, status, fit[t]);
    }
    __syncwarp();
    if (lane == 0) {
      // CompressClusters' arg-min: strict <, in mode order (CP:1752-1817)
      double best = DBL_MAX;
      int best_mode = 8, best_slot = 0, best_first = 0, best_rot = 0, best_im = 0;
      int t = 0;
      const uint32_t nshapes = sel.nshapes < 5 ? sel.nshapes : 5;
      for (int oi = 0; oi < 8; oi++) {
        const int mode = mode_order(oi);
        if (!(modes & (1u << mode))) continue;
        const ModeAttr a = mode_attr(mode);
        for (uint32_t s = 0; s < nshapes; s++) {
          if (a.subsets != 1 && (uint32_t)a.subsets != sel.nparts[s]) continue;
          if (sel.shape[s] >= 16 && mode == 0) continue;
          double total_err = 0.0;
          int first = t, rot = 0, im = 0;
          if (a.has_rotation) {
            const int nim = mode == 4 ? 2 : 1;
            double b = DBL_MAX;
            for (int r = 0; r < 4; r++)
              for (int k = 0; k < nim; k++, t++)
                if (fit[t].err < b) {
                  b = fit[t].err;
                  first = t;
                  rot = r;
                  im = k;
                }
            total_err = total_err + b;
          } else {
            for (int ci = 0; ci < a.subsets; ci++, t++) total_err = total_err + fit[t].err;
          }
          if (total_err < best) {
            best = total_err;
            best_mode = mode;
            best_slot = (int)s;
            best_first = first;
            best_rot = rot;
            best_im = im;
          }
        }
      }
      if (best_mode == 8) {
        out[0] = 1u << 6;
        out[1] = out[2] = out[3] = 0;
      } else {
        pack_block(best_mode, sel, best_slot, fit + best_first, s_anc2, s_anc3, s_part2,
                   s_part3, best_rot, best_im, out);
      }
      store_block(jb, lin, out);
    }
    __syncwarp();
  }
}

int FASTC_CAT(wpb_launch_w, FASTC_WPB_WARPS)(const JobDev *jobs_dev, int njobs, uint64_t total,
                                              const EncodeScratch &sc, int ctas, cudaStream_t st) {
  encode_kernel<FASTC_WPB_WARPS><<<ctas, FASTC_WPB_WARPS * 32, 0, st>>>(
      jobs_dev, njobs, total, sc.rank_local, sc.chunk_prefix, sc.counter, sc.status);
  return (int)cudaPeekAtLastError();
}

int FASTC_CAT(wpb_occupancy_w, FASTC_WPB_WARPS)() {
  int n = 0;
  const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &n, encode_kernel<FASTC_WPB_WARPS>, FASTC_WPB_WARPS * 32, 0);
  return (e == cudaSuccess && n > 0) ? n : 1;
}

void FASTC_CAT(wpb_upload_w, FASTC_WPB_WARPS)(const uint32_t *opt7, const uint32_t *opt6) {
  cudaMemcpyToSymbol(c_opt7, opt7, 256 * sizeof(uint32_t));
  cudaMemcpyToSymbol(c_opt6, opt6, 256 * sizeof(uint32_t));
}

#if FASTC_WPB_MAIN
int encode_ctas_per_sm(int warps) {
  switch (warps) {
    case 1: return wpb_occupancy_w1();
    case 2: return wpb_occupancy_w2();
    case 8: return wpb_occupancy_w8();
    default: return wpb_occupancy_w4();
  }
}

int launch_rank_prepass(const JobDev *jobs_dev, int njobs, uint64_t total,
                        const EncodeScratch &sc, void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (total == 0) return 0;
  const uint32_t nchunks = (uint32_t)((total + kRankChunk - 1) / kRankChunk);
  classify_kernel<<<nchunks, kRankChunk, 0, st>>>(jobs_dev, njobs, total, sc.rank_local,
                                                  sc.chunk_prefix, 0u);
  scan_kernel<<<1, 1024, 0, st>>>(sc.chunk_prefix, nchunks, sc.counter, sc.status,
                                  sc.singles);
  return (int)cudaPeekAtLastError();
}

int launch_rank_prepass_range(const JobDev *jobs_dev, int njobs, uint64_t total, uint64_t g0,
                              uint64_t g1, const EncodeScratch &sc, void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (g1 <= g0) return 0;
  const uint32_t r0 = (uint32_t)(g0 / kRankChunk);
  const uint32_t r1 = (uint32_t)((g1 + kRankChunk - 1) / kRankChunk);
  classify_kernel<<<r1 - r0, kRankChunk, 0, st>>>(jobs_dev, njobs, total, sc.rank_local,
                                                  sc.chunk_prefix, r0);
  scan_range_kernel<<<1, 1024, 0, st>>>(sc.chunk_prefix, r0, r1, sc.carry, sc.counter, sc.status,
                                        sc.singles);
  return (int)cudaPeekAtLastError();
}

int launch_encode(const JobDev *jobs_dev, int njobs, uint64_t total, const EncodeScratch &sc,
                  LaunchShape shape, void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (total == 0) return 0;
  {
    const int e = launch_rank_prepass(jobs_dev, njobs, total, sc, stream);
    if (e) return e;
  }
  const int ctas = shape.ctas > 0 ? shape.ctas : 1;
  switch (shape.warps_per_cta) {
    case 1: return wpb_launch_w1(jobs_dev, njobs, total, sc, ctas, st);
    case 2: return wpb_launch_w2(jobs_dev, njobs, total, sc, ctas, st);
    case 8: return wpb_launch_w8(jobs_dev, njobs, total, sc, ctas, st);
    default: return wpb_launch_w4(jobs_dev, njobs, total, sc, ctas, st);
  }
}

// ---------------------------------------------------------------------------
// Decoder (FasTC BPTCEncoder/src/Decompressor.cpp:32-367), one thread per
// block. `spec` selects BC7 interpolation for mode-4 blocks with index mode
// 1; otherwise the block decodes exactly as FasTC's decoder does, which
// looks the swapped index sets up in the unswapped weight rows.
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t get_bits(const uint32_t w[4], int &pos, int n) {
  uint32_t v = 0;
  for (int i = 0; i < n; i++, pos++) v |= ((w[pos >> 5] >> (pos & 31)) & 1u) << i;
  return v;
}

__device__ __forceinline__ void weights_padded(int bits, uint32_t j, uint32_t &w0, uint32_t &w1) {
  if (j >= (1u << bits)) {
    w0 = w1 = 0;
    return;
  }
  w1 = weight1(bits, j);
  w0 = 64u - w1;
}

// The 16 texels (RGBA8, R in the low byte) of one 128-bit block.
__device__ void decode_block(const uint32_t w[4], int spec, uint32_t outpx[16]) {
  int pos = 0, mode = 0;
  while (mode < 8 && !get_bits(w, pos, 1)) mode++;
  if (mode >= 8) {
    for (int i = 0; i < 16; i++) outpx[i] = 0;
  } else {
    const ModeAttr a = mode_attr(mode);
    const int nsub = a.subsets;
    int im = 0, rot = 0, shape = 0;
    if (nsub > 1) shape = (int)get_bits(w, pos, mode == 0 ? 4 : 6);
    else if (a.has_rotation) {
      rot = (int)get_bits(w, pos, 2);
      if (a.has_idx_mode) im = (int)get_bits(w, pos, 1);
    }
    uint32_t cp = (uint32_t)a.color_bits, ap = (uint32_t)a.alpha_bits;
    uint32_t eps[3][2][4];
    for (int ch = 0; ch < 3; ch++)
      for (int i = 0; i < nsub; i++)
        for (int e = 0; e < 2; e++) eps[i][e][ch] = (get_bits(w, pos, (int)cp) << (8 - cp)) & 0xFF;
    for (int i = 0; i < nsub; i++)
      for (int e = 0; e < 2; e++)
        eps[i][e][3] = ap == 0 ? 0xFFu : ((get_bits(w, pos, (int)ap) << (8 - ap)) & 0xFF);
    if (a.pbit != kPBitNone) {
      cp++;
      ap++;
      for (int i = 0; i < nsub; i++) {
        if (a.pbit == kPBitShared) {
          const uint32_t pb = get_bits(w, pos, 1);
          for (int e = 0; e < 2; e++)
            for (int ch = 0; ch < 4; ch++) eps[i][e][ch] |= pb << (8 - (ch == 3 ? ap : cp));
        } else {
          for (int e = 0; e < 2; e++) {
            const uint32_t pb = get_bits(w, pos, 1);
            for (int ch = 0; ch < 4; ch++) eps[i][e][ch] |= pb << (8 - (ch == 3 ? ap : cp));
          }
        }
      }
    }
    for (int i = 0; i < nsub; i++)
      for (int e = 0; e < 2; e++)
        for (int ch = 0; ch < 4; ch++) {
          const uint32_t prec = ch == 3 ? ap : cp;
          eps[i][e][ch] = (eps[i][e][ch] | (eps[i][e][ch] >> prec)) & 0xFF;
        }
    const uint32_t part = nsub == 2 ? c_part2[shape] : (nsub == 3 ? c_part3[shape] : 0u);
    uint32_t cidx[16], aidx[16];
    const int cb = a.idx_bits, ab = a.alpha_idx_bits;
    for (int i = 0; i < 16; i++) {
      const int s = (int)((part >> (2 * i)) & 3);
      const int anchor = s == 0 ? 0 : (nsub == 2 ? c_anchor2[shape] : (s == 1 ? (c_anchor3[shape] & 15) : (c_anchor3[shape] >> 4)));
      cidx[i] = get_bits(w, pos, anchor == i ? cb - 1 : cb);
    }
    int ncb = cb, nab = ab;
    if (ab == 0) {
      for (int i = 0; i < 16; i++) aidx[i] = cidx[i];
    } else {
      for (int i = 0; i < 16; i++) aidx[i] = get_bits(w, pos, i == 0 ? ab - 1 : ab);
      if (im) {
        for (int i = 0; i < 16; i++) {
          const uint32_t t = aidx[i];
          aidx[i] = cidx[i];
          cidx[i] = t;
        }
        if (spec) {
          ncb = ab;
          nab = cb;
        }
      }
    }
    for (int i = 0; i < 16; i++) {
      const int s = (int)((part >> (2 * i)) & 3);
      uint32_t p = 0;
      for (int ch = 0; ch < 4; ch++) {
        uint32_t w0, w1, ip;
        if (ch == 3 && nab > 0) {
          weights_padded(nab, aidx[i], w0, w1);
          ip = (eps[s][0][3] * w0 + eps[s][1][3] * w1 + 32u) >> 6;
        } else {
          weights_padded(ncb, cidx[i], w0, w1);
          ip = (eps[s][0][ch] * w0 + eps[s][1][ch] * w1 + 32u) >> 6;
        }
        p |= (ip & 0xFF) << (8 * ch);
      }
      if (rot >= 1 && rot <= 3) {
        const int c = rot - 1;
        const uint32_t x = (p >> (8 * c)) & 0xFF, y = p >> 24;
        p = (p & ~(0xFFu << (8 * c)) & 0x00FFFFFFu) | (y << (8 * c)) | (x << 24);
      }
      outpx[i] = p;
    }
  }
}

__device__ __forceinline__ void load_block_words(const uint8_t *src, uint32_t w[4]) {
  for (int i = 0; i < 4; i++)
    w[i] = (uint32_t)src[4 * i] | ((uint32_t)src[4 * i + 1] << 8) |
           ((uint32_t)src[4 * i + 2] << 16) | ((uint32_t)src[4 * i + 3] << 24);
}

__global__ void decode_kernel(const uint8_t *__restrict__ blocks, uint8_t *__restrict__ rgba,
                              uint32_t width, uint32_t height, int spec) {
  const uint32_t bw = (width + 3) / 4, bh = (height + 3) / 4;
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= (uint64_t)bw * bh) return;
  const uint32_t bx = (uint32_t)(b % bw), by = (uint32_t)(b / bw);
  uint32_t w[4];
  load_block_words(blocks + b * 16, w);
  uint32_t outpx[16];
  decode_block(w, spec, outpx);
  for (int r = 0; r < 4; r++) {
    const uint32_t y = by * 4 + r;
    if (y >= height) break;
    for (int c = 0; c < 4; c++) {
      const uint32_t x = bx * 4 + c;
      if (x >= width) break;
      *reinterpret_cast<uint32_t *>(rgba + ((size_t)y * width + x) * 4) = outpx[4 * r + c];
    }
  }
}

// ---------------------------------------------------------------------------
// Quality: FasTC's Image::ComputePSNR metric (Base/src/Image.cpp:206-255),
// per 4x4 block. Per texel, RGB premultiplied by alpha / 255 in double,
// the three squared differences summed in channel order; per block, the
// texels in row order (texels outside the image are skipped). One thread
// decodes its block (FasTC's decoder semantics) and compares it with the
// original texels, so no decoded image is written.
// ---------------------------------------------------------------------------

__device__ __forceinline__ double texel_sse(uint32_t a, uint32_t b) {
  const double ra = (double)(a >> 24) / 255.0, ua = (double)(b >> 24) / 255.0;
  double s = 0.0;
  for (int c = 0; c < 3; c++) {
    const double d = ra * (double)((a >> (8 * c)) & 0xFF) - ua * (double)((b >> (8 * c)) & 0xFF);
    s += d * d;
  }
  return s;
}

__global__ void block_error_kernel(const uint8_t *__restrict__ blocks,
                                   const uint8_t *__restrict__ rgba, uint32_t width,
                                   uint32_t height, double *__restrict__ sse) {
  const uint32_t bw = (width + 3) / 4, bh = (height + 3) / 4;
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= (uint64_t)bw * bh) return;
  const uint32_t bx = (uint32_t)(b % bw), by = (uint32_t)(b / bw);
  uint32_t w[4];
  load_block_words(blocks + b * 16, w);
  uint32_t dec[16];
  decode_block(w, 0, dec);
  double s = 0.0;
  for (int r = 0; r < 4; r++) {
    const uint32_t y = by * 4 + r;
    if (y >= height) break;
    for (int c = 0; c < 4; c++) {
      const uint32_t x = bx * 4 + c;
      if (x >= width) break;
      const uint8_t *p = rgba + ((size_t)y * width + x) * 4;
      const uint32_t orig = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) |
                            ((uint32_t)p[3] << 24);
      s += texel_sse(orig, dec[4 * r + c]);
    }
  }
  sse[b] = s;
}

// Sum of n doubles in a fixed order (one CTA): thread t adds entries t,
// t + 1024, ... in sequence, then a pairwise tree over the threads. The
// result does not depend on scheduling, so it repeats bit for bit.
__global__ void __launch_bounds__(1024) sum_kernel(const double *__restrict__ v, uint64_t n,
                                                   double *__restrict__ out) {
  __shared__ double s[1024];
  double acc = 0.0;
  for (uint64_t i = threadIdx.x; i < n; i += 1024) acc += v[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int h = 512; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

// The same over a raster range of blocks [first, first + count) of a
// texture of `width` texels, blocks[k] holding block first + k and `rows`
// the texels from row row0 on (as a job uploads them).
__global__ void range_error_kernel(const uint8_t *__restrict__ blocks,
                                   const uint8_t *__restrict__ rows, uint32_t width, uint32_t row0,
                                   uint32_t first, uint32_t count, double *__restrict__ sse) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint32_t bw = width / 4, b = first + k;
  const uint32_t bx = b % bw, by = b / bw;
  uint32_t w[4];
  load_block_words(blocks + (size_t)k * 16, w);
  uint32_t dec[16];
  decode_block(w, 0, dec);
  double s = 0.0;
  for (int r = 0; r < 4; r++)
    for (int c = 0; c < 4; c++) {
      const uint8_t *p = rows + ((size_t)(by * 4 + r - row0) * width + bx * 4 + c) * 4;
      const uint32_t orig = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) |
                            ((uint32_t)p[3] << 24);
      s += texel_sse(orig, dec[4 * r + c]);
    }
  sse[k] = s;
}

int launch_range_error(const uint8_t *blocks, const uint8_t *rows, uint32_t width, uint32_t row0,
                       uint32_t first, uint32_t count, double *block_sse, double *total,
                       void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (count == 0) return 0;
  range_error_kernel<<<(count + 127) / 128, 128, 0, st>>>(blocks, rows, width, row0, first, count,
                                                           block_sse);
  sum_kernel<<<1, 1024, 0, st>>>(block_sse, count, total);
  return (int)cudaPeekAtLastError();
}

int launch_sum(const double *v, uint64_t n, double *out, void *stream) {
  sum_kernel<<<1, 1024, 0, static_cast<cudaStream_t>(stream)>>>(v, n, out);
  return (int)cudaPeekAtLastError();
}

int launch_block_error(const uint8_t *blocks, const uint8_t *rgba, uint32_t width,
                       uint32_t height, double *block_sse, double *total, void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint64_t nb = (uint64_t)((width + 3) / 4) * ((height + 3) / 4);
  if (nb == 0) return 0;
  const int threads = 128;
  block_error_kernel<<<(unsigned)((nb + threads - 1) / threads), threads, 0, st>>>(
      blocks, rgba, width, height, block_sse);
  if (total) sum_kernel<<<1, 1024, 0, st>>>(block_sse, nb, total);
  return (int)cudaPeekAtLastError();
}

int launch_decode(const uint8_t *blocks, uint8_t *rgba, uint32_t width, uint32_t height,
                  int spec, void *stream) {
  const uint64_t nb = (uint64_t)((width + 3) / 4) * ((height + 3) / 4);
  if (nb == 0) return 0;
  const int threads = 256;
  const uint64_t grid = (nb + threads - 1) / threads;
  decode_kernel<<<(unsigned)grid, threads, 0, static_cast<cudaStream_t>(stream)>>>(
      blocks, rgba, width, height, spec);
  return (int)cudaPeekAtLastError();
}
#endif  // FASTC_WPB_MAIN

}  // namespace fastc
