// Task-parallel BC7 encoder for sm_103a.
//
// The block search of FasTC's CompressBC7Block (BPTCEncoder/src/
// Compressor.cpp:1819-1860) is split into stages so that every warp runs 32
// pieces of identical work:
//
//   select_kernel   one warp per 4x4 block (texels staged in shared memory
//                   from 128-bit loads): trivial blocks, the 64+64 shape
//                   estimate of BoxSelection, and the number of cluster fits
//                   each BC7 mode needs.
//   count scan      exclusive scan of those counts, class-major (a class is
//                   a mode and colour index width), so all fits of one class
//                   are contiguous in the task arrays.
//   emit_kernel     one thread per block writes its task descriptors.
//   setup_kernel    one thread per cluster fit (per block for mode 6, whose
//                   two shape slots share the cluster): PCA, k-means, least
//                   squares, grid clamp, first QuantizedError (CP:921-1094,
//                   632-919), and an exact lower bound of the fit's error;
//                   fits with annealing work go to their class's list.
//   bound_kernel    one thread per block, after every class's setup: fits
//                   of candidates whose lower bound exceeds the block's
//                   least setup total cannot win and skip the annealing.
//   order_kernel    the remaining fits of a class in point-count order.
//   anneal_kernel   one persistent launch per class; one thread per fit,
//                   refilled from the class list: the simulated annealing
//                   (CP:538-630) on integer endpoints with an exact integer
//                   QuantizedError (dp2a projection, paired palette, dp4a);
//                   the rotation classes hand sparse warps' fits on to two
//                   generations of continuation launches.
//   choose_kernel   one thread per block: FasTC's arg-min over modes
//                   (CP:1752-1817); reindex_kernel: indices of the winning
//                   annealed fits; pack_kernel: the 128-bit packing
//                   (CP:1096-1298).
//
// Blocks are processed in chunks so that the task arrays fit a fixed
// scratch size; every stage is asynchronous and graph-capturable.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "bc7_block.cuh"
#include "bc7_encode.cuh"
#include "bc7_format.cuh"
#include "bc7_intqe.cuh"
#include "bc7_kernels.cuh"
#include "bc7_pipeline.cuh"

namespace fastc {

__constant__ uint32_t q_part2[64] = {FASTC_PART2_WORDS};
__constant__ uint32_t q_part3[64] = {FASTC_PART3_WORDS};
__constant__ uint8_t q_anchor2[64] = {FASTC_ANCHOR2_BYTES};
__constant__ uint8_t q_anchor3[64] = {FASTC_ANCHOR3_BYTES};
__constant__ uint32_t q_watermark[9] = {FASTC_WATERMARK_WORDS};
__constant__ uint32_t q_opt7[256];
__constant__ uint32_t q_opt6[256];
// QuantizeChannel (RGBAEndpoints.cpp:126-165) tabulated for masks of the top
// `prec` bits, prec = 1..8, and p-bit -1/0/1: [prec-1][pbit+1][value].
__constant__ uint8_t q_qlut[8][3][256];
// single_channel_search() for every row and value, built once per device.
__device__ uint32_t g_sct[kSctRows * 256];
// The shape estimate's subsets as tasks (select stage): the member masks of
// the 128 subsets of the two-subset shapes and of the 140 distinct subsets
// of the three-subset shapes (192 less the repeats), each list sorted by
// member count, most first, so that the 32 lanes of a round loop over the
// same number of texels; and for subset k of shape s, the position of its
// mask in the list ([s * 2 + k], [s * 3 + k]).
constexpr int kSub2 = 128, kSub3 = 160;  // list lengths (the second padded to 5 rounds)
__constant__ uint16_t q_sub2_mask[kSub2];
__constant__ uint8_t q_sub2_pos[64 * 2];
__constant__ uint16_t q_sub3_mask[kSub3];
__constant__ uint8_t q_sub3_pos[64 * 3];

__global__ void build_sct_kernel() {
  const int row = blockIdx.x, val = threadIdx.x;
  const int ib = row % 3 + 2, pvar = (row / 3) % 5, nbits = row / 15 + 1;
  const int havepbit = pvar != 0;
  const int pl = havepbit ? (pvar - 1) & 1 : 0, ph = havepbit ? (pvar - 1) >> 1 : 0;
  g_sct[row * 256 + val] = single_channel_search((uint32_t)val, nbits, havepbit, pl, ph, ib);
}

// ---------------------------------------------------------------------------
// Host-side table construction
// ---------------------------------------------------------------------------

static uint8_t host_quantize(uint32_t val, uint32_t mask, int pbit) {
  if (mask == 0xFF) return (uint8_t)val;
  if (mask == 0) return 0xFF;
  uint32_t prec = 0;
  for (uint32_t m = mask; m; m &= m - 1) prec++;
  const uint32_t step = 1u << (8 - prec);
  uint32_t lval = val & mask, hval = lval + step;
  if (pbit >= 0) {
    prec++;
    lval |= (uint32_t)(pbit != 0) << (8 - prec);
    hval |= (uint32_t)(pbit != 0) << (8 - prec);
  }
  if (lval > val) {
    lval -= step;
    hval -= step;
  }
  lval |= lval >> prec;
  hval |= hval >> prec;
  const uint32_t l8 = lval & 0xFF, h8 = hval & 0xFF;
  const uint32_t dl = val > l8 ? val - l8 : l8 - val, dh = val > h8 ? val - h8 : h8 - val;
  return (uint8_t)(dl < dh ? l8 : h8);
}

// Member masks of (shape, subset), distinct ones once, sorted by member
// count (most first; ties in shape and subset order); pos[s * nsub + k] =
// position of the mask of subset k of shape s. Returns the list length.
static int build_subset_list(const uint32_t part[64], int nsub, uint16_t *list, uint8_t *pos) {
  uint16_t masks[64 * 3];
  int n = 0;
  for (int sh = 0; sh < 64; sh++)
    for (int k = 0; k < nsub; k++) {
      uint16_t m = 0;
      for (int i = 0; i < 16; i++)
        if ((int)((part[sh] >> (2 * i)) & 3u) == k) m |= (uint16_t)(1u << i);
      bool seen = false;
      for (int j = 0; j < n; j++) seen = seen || masks[j] == m;
      if (!seen) masks[n++] = m;
    }
  int len = 0;
  for (int cnt = 16; cnt >= 1; cnt--)
    for (int j = 0; j < n; j++)
      if (__builtin_popcount(masks[j]) == cnt) list[len++] = masks[j];
  for (int sh = 0; sh < 64; sh++)
    for (int k = 0; k < nsub; k++) {
      uint16_t m = 0;
      for (int i = 0; i < 16; i++)
        if ((int)((part[sh] >> (2 * i)) & 3u) == k) m |= (uint16_t)(1u << i);
      for (int j = 0; j < len; j++)
        if (list[j] == m) pos[sh * nsub + k] = (uint8_t)j;
    }
  return len;
}

void upload_pipeline_tables(int device, const uint32_t opt7[256], const uint32_t opt6[256]) {
  static bool done[64] = {false};
  if (device < 0 || device >= 64 || done[device]) return;
  {
    static const uint32_t part2[64] = {FASTC_PART2_WORDS};
    static const uint32_t part3[64] = {FASTC_PART3_WORDS};
    uint16_t l2[kSub2] = {0}, l3[kSub3] = {0};
    uint8_t p2[128] = {0}, p3[192] = {0};
    const int n2 = build_subset_list(part2, 2, l2, p2);
    const int n3 = build_subset_list(part3, 3, l3, p3);
    if (n2 != kSub2 || n3 > kSub3) {  // fixed by the BC7 partition tables
      fprintf(stderr, "fastc_bc7: unexpected partition subset counts %d, %d\n", n2, n3);
      abort();
    }
    cudaMemcpyToSymbol(q_sub2_mask, l2, sizeof(l2));
    cudaMemcpyToSymbol(q_sub2_pos, p2, sizeof(p2));
    cudaMemcpyToSymbol(q_sub3_mask, l3, sizeof(l3));
    cudaMemcpyToSymbol(q_sub3_pos, p3, sizeof(p3));
  }
  static uint8_t lut[8][3][256];
  for (int p = 1; p <= 8; p++)
    for (int b = -1; b <= 1; b++)
      for (int v = 0; v < 256; v++)
        lut[p - 1][b + 1][v] = host_quantize((uint32_t)v, (0xFFu << (8 - p)) & 0xFFu, b);
  cudaMemcpyToSymbol(q_qlut, lut, sizeof(lut));
  cudaMemcpyToSymbol(q_opt7, opt7, 256 * sizeof(uint32_t));
  cudaMemcpyToSymbol(q_opt6, opt6, 256 * sizeof(uint32_t));
  build_sct_kernel<<<kSctRows, 256>>>();
  cudaDeviceSynchronize();
  done[device] = true;
}

// ---------------------------------------------------------------------------
// Shared helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ int find_job_p(const JobDev *jobs, int njobs, uint64_t g) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].begin <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ uint4 load_row_p(const JobDev &jb, uint32_t lin, int r) {
  const uint32_t bw = jb.width >> 2;
  const uint32_t bx = lin % bw, by = lin / bw;
  const size_t off = ((size_t)(by * 4 + r - jb.row0) * jb.width + (size_t)bx * 4) * 4;
  const uint8_t *p = jb.in + off;
  if (jb.flags & kJobIn16) return __ldg(reinterpret_cast<const uint4 *>(p));
  const uint32_t *q = reinterpret_cast<const uint32_t *>(p);
  return make_uint4(__ldg(q), __ldg(q + 1), __ldg(q + 2), __ldg(q + 3));
}

__device__ __forceinline__ void store_block_p(const JobDev &jb, uint32_t lin, const uint32_t w[4]) {
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

__device__ __forceinline__ Selection sel_of(const BlockSel &b) {
  Selection s;
  s.nshapes = b.nshapes;
  s.shape[0] = b.shape0;
  s.shape[1] = b.shape1;
  s.nparts[0] = 2;
  s.nparts[1] = b.nshapes > 1 ? 3 : 0;
  s.modes = b.modes;
  return s;
}

// Number of cluster fits CompressClusters (CP:1752-1817) runs for class c.
__device__ __forceinline__ int class_task_count(const Selection &sel, uint32_t modes, int c) {
  const int mode = class_mode(c);
  if (!(modes & (1u << mode))) return 0;
  const ModeAttr a = mode_attr(mode);
  const uint32_t nshapes = sel.nshapes < 5 ? sel.nshapes : 5;
  int n = 0;
  for (uint32_t s = 0; s < nshapes; s++) {
    if (a.subsets != 1 && (uint32_t)a.subsets != sel.nparts[s]) continue;
    if (sel.shape[s] >= 16 && mode == 0) continue;
    n += a.has_rotation ? 4 : a.subsets;
  }
  return n;
}

// The i-th fit of class c: shape slot, then subset (or rotation), in
// CompressClusters' order.
__device__ __forceinline__ Task class_task(const Selection &sel, int c, int i) {
  const int mode = class_mode(c);
  const ModeAttr a = mode_attr(mode);
  const uint32_t nshapes = sel.nshapes < 5 ? sel.nshapes : 5;
  Task t{mode, 0, 0, 0, class_im(c)};
  for (uint32_t s = 0; s < nshapes; s++) {
    if (a.subsets != 1 && (uint32_t)a.subsets != sel.nparts[s]) continue;
    if (sel.shape[s] >= 16 && mode == 0) continue;
    const int per = a.has_rotation ? 4 : a.subsets;
    if (i < per) {
      t.slot = (int)s;
      if (a.has_rotation) t.rot = i;
      else t.subset = i;
      return t;
    }
    i -= per;
  }
  return t;
}

__device__ __forceinline__ uint32_t part_word_of(const Selection &sel, int mode, int slot) {
  const int ns = mode_attr(mode).subsets;
  const uint32_t shape = sel.shape[slot];
  return ns == 2 ? q_part2[shape] : (ns == 3 ? q_part3[shape] : 0u);
}

// offset of entry i of a chunk-scanned array
__device__ __forceinline__ uint32_t scanned(const uint16_t *local, const uint32_t *chunk, uint64_t i) {
  return chunk[i / kRankChunk] + local[i];
}

// ---------------------------------------------------------------------------
// select
// ---------------------------------------------------------------------------

// One subset of the shape estimate as a task: the subset's members (mask of
// texel positions) of the block's texels `px`, their bounding-box corners
// as the endpoints of an unquantized QuantizedError (CP:1626-1655). A shape
// adds for this subset 0 for a one-point box, else 0.0001 + the error; the
// error is an integer below 2^23, returned with bit 31 set when the box has
// more than one point.
template <int kBits>
__device__ __forceinline__ uint32_t estimate_subset_int(const uint32_t *px, uint32_t mask,
                                                        uint4 *pal) {
  uint32_t mn = 0xFFFFFFFFu, mx = 0u;
  int se = 0;
#pragma unroll 1
  for (uint32_t m = mask; m; m &= m - 1) {
    const uint32_t e = px[__ffs(m) - 1];
    mn = __vminu4(mn, e);
    mx = __vmaxu4(mx, e);
    se += (int)__dp4a(e, e, 0u);
  }
  if (mn == mx) return 0u;
  const Proj pj = make_proj(mn, mx);
  palette_sq<kBits>(mn, mx, pal);
  int acc = 0;
#pragma unroll 1
  for (uint32_t m = mask; m; m &= m - 1) {
    const uint32_t e = px[__ffs(m) - 1];
    bool two;
    const int j1 = nearest_pair<kBits>(pj, e, two);
    int bj;
    acc += pair_term(e, pal, j1, two, bj);
  }
  return 0x80000000u | (uint32_t)(se + acc);
}

// A shape's estimate as FasTC sums it in double: per subset, in order, 0
// or 0.0001 + the error.
template <int kNSub>
__device__ __forceinline__ double shape_estimate_double(const uint32_t *est, const uint8_t *pos,
                                                        int sh) {
  double err = 0.0;
#pragma unroll
  for (int k = 0; k < kNSub; k++) {
    const uint32_t v = est[pos[sh * kNSub + k]];
    double e = 0.0;
    if (v) {
      e = 0.0001;
      e = e + (double)(float)(int)(v & 0x7FFFFFFFu);
    }
    err = err + e;
  }
  return err;
}

// One pass of BoxSelection (CP:1670-1750) for the uniform metric: every
// distinct subset estimated once, in rounds of 32 lanes over the
// member-count-sorted list, into the warp's `est`; each lane then sums the
// subsets of shapes `lane` and `lane + 32`. The choice is made on integers:
// a shape's double estimate is its integer total plus at most three times
// 0.0001 (and rounding far below that), so the first shape with estimate 0
// is the first with no multi-point box, and the least estimate is among the
// shapes of least integer total; only when several shapes share that total
// are their double estimates formed and compared (strict <, first index
// wins, as FasTC's loop). Returns the chosen shape; `zero` is set when it
// is FasTC's early exit (estimate below 1e-9).
template <int kNSub>
__device__ __forceinline__ int select_shape_int(const uint32_t *px, int lane, uint32_t *est,
                                                uint4 *pal, bool &zero) {
  constexpr int kBits = kNSub == 2 ? 3 : 2;
  constexpr int kLen = kNSub == 2 ? kSub2 : kSub3;
  const uint16_t *list = kNSub == 2 ? q_sub2_mask : q_sub3_mask;
  const uint8_t *pos = kNSub == 2 ? q_sub2_pos : q_sub3_pos;
#pragma unroll 1
  for (int r = lane; r < kLen; r += 32) {
    const uint32_t m = list[r];
    est[r] = m ? estimate_subset_int<kBits>(px, m, pal) : 0u;
  }
  __syncwarp();
  uint32_t tot[2];
  bool any[2];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int sh = lane + 32 * h;
    uint32_t t = 0, f = 0;
#pragma unroll
    for (int k = 0; k < kNSub; k++) {
      const uint32_t v = est[pos[sh * kNSub + k]];
      t += v & 0x7FFFFFFFu;
      f |= v;
    }
    tot[h] = t;
    any[h] = (f >> 31) != 0;
  }
  const uint64_t z = (uint64_t)__ballot_sync(0xFFFFFFFFu, !any[0]) |
                     ((uint64_t)__ballot_sync(0xFFFFFFFFu, !any[1]) << 32);
  int chosen;
  if (z) {
    zero = true;
    chosen = __ffsll((long long)z) - 1;
  } else {
    zero = false;
    uint32_t mt = min(tot[0], tot[1]);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) mt = min(mt, __shfl_xor_sync(0xFFFFFFFFu, mt, o));
    const uint64_t cand = (uint64_t)__ballot_sync(0xFFFFFFFFu, tot[0] == mt) |
                          ((uint64_t)__ballot_sync(0xFFFFFFFFu, tot[1] == mt) << 32);
    if (__popcll(cand) == 1) {
      chosen = __ffsll((long long)cand) - 1;
    } else {
      double be = tot[0] == mt ? shape_estimate_double<kNSub>(est, pos, lane) : DBL_MAX;
      const double e1 = tot[1] == mt ? shape_estimate_double<kNSub>(est, pos, lane + 32) : DBL_MAX;
      int bi = lane;
      argmin_pair(be, bi, e1, lane + 32);
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        const double oe = __shfl_xor_sync(0xFFFFFFFFu, be, o);
        const int oi = __shfl_xor_sync(0xFFFFFFFFu, bi, o);
        argmin_pair(be, bi, oe, oi);
      }
      chosen = bi;
    }
  }
  __syncwarp();
  return chosen;
}

// The float-metric estimate, kept out of line.
__device__ __noinline__ double estimate_shape_float(const uint32_t *px, uint32_t part, int nsub,
                                                    int bits, int metric) {
  float w[4];
#pragma unroll
  for (int c = 0; c < 4; c++) w[c] = base_weight(metric, c);
  return estimate_shape(px, part, nsub, bits, w);
}

// One pass of BoxSelection (CP:1670-1750) for the nonuniform metric over
// the 64 shapes with kNSub subsets, two shapes per lane: the estimates of
// this lane's shapes.
template <int kNSub>
__device__ __forceinline__ void estimate_pair(const uint32_t *px, const uint32_t *part, int metric,
                                              int lane, double &e0, double &e1) {
  constexpr int kBits = kNSub == 2 ? 3 : 2;
#pragma unroll 1
  for (int h = 0; h < 2; h++) {
    const uint32_t pw = part[lane + 32 * h];
    const double v = estimate_shape_float(px, pw, kNSub, kBits, metric);
    if (h == 0) e0 = v;
    else e1 = v;
  }
}

// BoxSelection with the integer estimate (same result as box_selection_warp).
__device__ __forceinline__ Selection box_selection_pipe(const uint32_t *px,
                                                        const uint32_t *part2,
                                                        const uint32_t *part3, int metric,
                                                        int lane, uint4 *pal, uint32_t *est) {
  Selection r;
  r.nshapes = 1;
  r.shape[0] = r.shape[1] = 0;
  r.nparts[0] = 2;
  r.nparts[1] = 0;
  r.modes = 0xFF;
  bool opaque = true;
  for (int i = 0; i < 16; i++) opaque = opaque && ((px[i] >> 24) >= 250);
#pragma unroll
  for (int pass = 0; pass < 2; pass++) {
    const int nsub = pass ? 3 : 2;
    if (metric == 0) {
      bool zero;
      const int sh = pass ? select_shape_int<3>(px, lane, est, pal, zero)
                          : select_shape_int<2>(px, lane, est, pal, zero);
      r.shape[pass] = (uint32_t)sh;
      r.nparts[pass] = (uint32_t)nsub;
      if (zero) {
        r.modes = pass ? kModesThree : kModesTwo;
        return r;
      }
      if (pass == 0) {
        if (!opaque) {
          r.modes &= kModesAlpha;
          return r;
        }
        r.modes &= ~((1u << 4) | (1u << 5));
        r.nshapes = 2;
      }
      continue;
    }
    double e0, e1;
    if (pass) estimate_pair<3>(px, part3, metric, lane, e0, e1);
    else estimate_pair<2>(px, part2, metric, lane, e0, e1);
    const uint64_t zero = (uint64_t)__ballot_sync(0xFFFFFFFFu, e0 < 1e-9) |
                          ((uint64_t)__ballot_sync(0xFFFFFFFFu, e1 < 1e-9) << 32);
    if (zero) {
      r.shape[pass] = (uint32_t)(__ffsll((long long)zero) - 1);
      r.nparts[pass] = (uint32_t)nsub;
      r.modes = pass ? kModesThree : kModesTwo;
      return r;
    }
    double be = e0;
    int bi = lane;
    argmin_pair(be, bi, e1, lane + 32);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      const double oe = __shfl_xor_sync(0xFFFFFFFFu, be, o);
      const int oi = __shfl_xor_sync(0xFFFFFFFFu, bi, o);
      argmin_pair(be, bi, oe, oi);
    }
    r.shape[pass] = (uint32_t)bi;
    r.nparts[pass] = (uint32_t)nsub;
    if (pass == 0) {
      if (!opaque) {
        r.modes &= kModesAlpha;
        return r;
      }
      r.modes &= ~((1u << 4) | (1u << 5));
      r.nshapes = 2;
    }
  }
  return r;
}

// ---------------------------------------------------------------------------
// The logging encoder's shape search (CompressWithStats with a log stream,
// CP:1862-1936, 2046-2166), with the statistics it logs
// ---------------------------------------------------------------------------

// EstimateTwoClusterErrorStats / EstimateThreeClusterErrorStats
// (CP:1862-1928) for subset ci of a shape: the subset's bounding box
// quantised with the colour grids of two modes (1 and 3, or 0 and 2), each
// error the estimate of its mode; the subset adds 0.0001 + the smaller.
__device__ __noinline__ double stats_subset(const uint32_t *px, uint32_t part, int ci, bool three,
                                            int metric, double &e0, double &e1) {
  Cluster c;
  uint32_t buf[16];
  make_cluster(px, part, ci, buf, 1, c);
  float v[4];
#pragma unroll
  for (int k = 0; k < 4; k++) v[k] = __fsub_rn(c.mx[k], c.mn[k]);
  if (sqlen4(v) == 0.0f) {
    e0 = e1 = 0.0;
    return 0.0;
  }
  float w[4];
#pragma unroll
  for (int k = 0; k < 4; k++) w[k] = base_weight(metric, k);
  const int bits = three ? 2 : 3;
  const uint32_t m0 = three ? 0xFFF0F0F0u : 0xFFFCFCFCu;
  const uint32_t m1 = three ? 0xFFF8F8F8u : 0xFFFEFEFEu;
  const double bias = three ? 0.0001 : 0.0;
  e0 = bias + (double)quantized_error(c, c.mn, c.mx, bits, m0, w, -1, nullptr);
  e1 = bias + (double)quantized_error(c, c.mn, c.mx, bits, m1, w, -1, nullptr);
  double err = 0.0001;
  err += e0 < e1 ? e0 : e1;
  return err;
}

__device__ __forceinline__ double warp_min_double(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v = fmin(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  return v;
}

// One shape loop of the logging encoder (CP:2066-2114 with nsub 2,
// 2118-2166 with nsub 3), shapes `lane` and `lane + 32` on this lane. The
// loop stops after the first shape whose estimate is below 1e-9; over the
// shapes up to there it records each estimate below all before it (the
// last of them is the shape chosen) and keeps the least of each mode's
// summed estimates. Returns the chosen shape; `exact` is set on the stop.
template <int kNSub>
__device__ int stats_shapes(const uint32_t *px, const uint32_t *part, int metric, int lane,
                            fastc_bc7_block_stats *st, double &est_a, double &est_b, bool &exact) {
  constexpr bool kThree = kNSub == 3;
  double err[2], acc[2][2];
#pragma unroll 1
  for (int h = 0; h < 2; h++) {
    const uint32_t pw = part[lane + 32 * h];
    double e = 0.0, a0 = 0.0, a1 = 0.0;
#pragma unroll 1
    for (int ci = 0; ci < kNSub; ci++) {
      double e0, e1;
      e += stats_subset(px, pw, ci, kThree, metric, e0, e1);
      a0 = ci == 0 ? e0 : a0 + e0;
      a1 = ci == 0 ? e1 : a1 + e1;
    }
    err[h] = e;
    acc[h][0] = a0;
    acc[h][1] = a1;
  }
  const uint64_t z = (uint64_t)__ballot_sync(0xFFFFFFFFu, err[0] < 1e-9) |
                     ((uint64_t)__ballot_sync(0xFFFFFFFFu, err[1] < 1e-9) << 32);
  const int last = z ? __ffsll((long long)z) - 1 : 63;  // last shape the loop visits
  exact = z != 0;
  // exclusive prefix minimum of the estimates in shape order
  double incl[2];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    double v = err[h];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(0xFFFFFFFFu, v, o);
      if (lane >= o) v = fmin(v, t);
    }
    incl[h] = v;
  }
  const double min0 = __shfl_sync(0xFFFFFFFFu, incl[0], 31);
  incl[1] = fmin(incl[1], min0);
  double excl[2];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const double t = __shfl_up_sync(0xFFFFFFFFu, incl[h], 1);
    excl[h] = lane > 0 ? t : (h == 0 ? DBL_MAX : min0);
  }
  bool rec[2];
  double ea = DBL_MAX, eb = DBL_MAX;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int sh = lane + 32 * h;
    const bool in = sh <= last;
    rec[h] = in && err[h] < excl[h];
    if (in) {
      ea = fmin(ea, acc[h][0]);
      eb = fmin(eb, acc[h][1]);
    }
  }
  est_a = warp_min_double(ea);
  est_b = warp_min_double(eb);
  const uint32_t r0 = __ballot_sync(0xFFFFFFFFu, rec[0]), r1 = __ballot_sync(0xFFFFFFFFu, rec[1]);
  const uint32_t below = (1u << lane) - 1u;
  double *list = kThree ? st->three_shape : st->two_shape;
  if (rec[0]) list[__popc(r0 & below)] = err[0];
  if (rec[1]) list[__popc(r0) + __popc(r1 & below)] = err[1];
  if (lane == 0) {
    if (kThree) st->n_three = __popc(r0) + __popc(r1);
    else st->n_two = __popc(r0) + __popc(r1);
  }
  return r1 ? 32 + 31 - __clz((int)r1) : 31 - __clz((int)r0);
}

// CompressBC7Block with a BlockLogger (CP:1938-2183) up to the cluster
// fits, for a block that is neither one colour nor fully transparent: the
// selection and the statistics (path, per-mode estimates, improving shape
// estimates; the errors stay -1).
__device__ Selection box_selection_stats(const uint32_t *px, const uint32_t *part2,
                                         const uint32_t *part3, int metric, int lane,
                                         fastc_bc7_block_stats *st) {
  bool opaque = true;
  for (int i = 0; i < 16; i++) opaque = opaque && (px[i] >> 24) == 255u;
  // mode 6's estimate: the whole block's box, 4 buckets (CP:2046-2058)
  double est6;
  {
    Cluster c;
    uint32_t buf[16];
    make_cluster(px, 0u, 0, buf, 1, c);
    float v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = __fsub_rn(c.mx[k], c.mn[k]);
    if (sqlen4(v) == 0.0f) {
      est6 = 0.0;
    } else {
      float w[4];
#pragma unroll
      for (int k = 0; k < 4; k++) w[k] = base_weight(metric, k);
      est6 = 0.0001 + (double)quantized_error(c, c.mn, c.mx, 2, 0xFEFEFEFEu, w, -1, nullptr);
    }
  }
  Selection r;
  r.nshapes = opaque ? 2 : 1;
  r.nparts[0] = 2;
  r.nparts[1] = opaque ? 3 : 0;
  r.shape[1] = 0;
  r.modes = 0xFF;
  double e1, e3, e0 = -1.0, e2 = -1.0;
  bool exact;
  r.shape[0] = (uint32_t)stats_shapes<2>(px, part2, metric, lane, st, e1, e3, exact);
  int path = 3;
  if (exact) {
    r.modes = kModesTwo;
    path = 2;
  }
  if (opaque) {
    r.shape[1] = (uint32_t)stats_shapes<3>(px, part3, metric, lane, st, e0, e2, exact);
    if (exact) {
      r.modes = kModesThree;
      path = 2;
    }
  } else if (lane == 0) {
    st->n_three = 0;
  }
  if (lane < 8) {
    const double v = lane == 0 ? e0 : lane == 1 ? e1 : lane == 2 ? e2 : lane == 3 ? e3
                     : lane == 6 ? est6 : -1.0;
    st->estimate[lane] = v;
    st->error[lane] = -1.0;
  }
  if (lane == 0) {
    st->path = path;
    st->mode = -1;
  }
  return r;
}

// A one-colour or transparent block's statistics (CP:1938-1960).
__device__ __forceinline__ void trivial_stats(fastc_bc7_block_stats *st, int lane, int path) {
  if (lane < 8) {
    st->estimate[lane] = -1.0;
    st->error[lane] = -1.0;
  }
  if (lane == 0) {
    st->path = path;
    st->mode = path == 0 ? 5 : 6;
    st->n_two = st->n_three = 0;
  }
}

// kStats: the logging encoder's selection, with its statistics written to
// stats[global block index].
template <int kWarps, bool kStats>
__global__ void __launch_bounds__(kWarps * 32) select_kernel(
    const JobDev *__restrict__ jobs, int njobs, uint64_t c0, uint32_t nb,
    const uint16_t *__restrict__ rank_local, const uint32_t *__restrict__ rank_chunk,
    BlockSel *__restrict__ sel, uint8_t *__restrict__ counts, int task_bound, uint32_t *status,
    fastc_bc7_block_stats *__restrict__ stats) {
  static_assert(kWarps * 32 == kLaneStride, "shared arrays use the lane stride");
  __shared__ uint32_t s_part2[64], s_part3[64];
  __shared__ uint32_t s_px[kWarps][16];
  __shared__ uint4 s_pal[8 * kLaneStride];
  __shared__ uint32_t s_est[kWarps][kSub3];
  for (int i = threadIdx.x; i < 64; i += blockDim.x) {
    s_part2[i] = q_part2[i];
    s_part3[i] = q_part3[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t *px = s_px[wid];
  for (uint32_t gl = blockIdx.x * kWarps + wid; gl < nb; gl += gridDim.x * kWarps) {
    const uint64_t g = c0 + gl;
    const int j = find_job_p(jobs, njobs, g);
    const JobDev &jb = jobs[j];
    const uint32_t lin = jb.first + (uint32_t)(g - jb.begin);
    if (lane < 4) {
      const uint4 v = load_row_p(jb, lin, lane);
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
    BlockSel bs;
    bs.job = (uint32_t)j;
    bs.lin = lin;
    bs.shape0 = bs.shape1 = bs.nshapes = 0;
    bs.modes = 0;
    bs.done = 1;
    bs.pad[0] = bs.pad[1] = bs.pad[2] = 0;
    if (same || transparent) {
      if (kStats) trivial_stats(stats + g, lane, same ? 0 : 1);
      if (lane < kClasses) counts[(uint64_t)lane * nb + gl] = 0;
      if (lane == 0) {
        uint32_t out[4];
        if (same) {
          const uint64_t gb = jb.begin;
          const uint32_t rg = rank_chunk[g / kRankChunk] + rank_local[g];
          const uint32_t rb = (jb.flags & kJobWmGlobal)
                                  ? 0u
                                  : rank_chunk[gb / kRankChunk] + rank_local[gb];
          single_color_block(px[0], jb.wm_start + (rg - rb), q_opt7, q_watermark, out);
        } else {
          out[0] = 1u << 6;
          out[1] = out[2] = out[3] = 0;
        }
        store_block_p(jb, lin, out);
        sel[gl] = bs;
      }
      __syncwarp();
      continue;
    }
    const Selection s =
        kStats ? box_selection_stats(px, s_part2, s_part3, (int)jb.metric, lane, stats + g)
               : box_selection_pipe(px, s_part2, s_part3, (int)jb.metric, lane,
                                    s_pal + threadIdx.x, s_est[wid]);
    uint32_t modes = s.modes & jb.modes;
    if (modes == 0) modes = jb.modes & 0xFF;  // FasTC: undefined behaviour
    const int c = lane < kClasses ? class_task_count(s, modes, lane) : 0;
    int total = c;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) total += __shfl_xor_sync(0xFFFFFFFFu, total, o);
    const bool overflow = total > task_bound;  // not reachable: the host computed the bound
    if (lane < kClasses) counts[(uint64_t)lane * nb + gl] = overflow ? 0 : (uint8_t)c;
    if (lane == 0) {
      bs.shape0 = (uint8_t)s.shape[0];
      bs.shape1 = (uint8_t)s.shape[1];
      bs.nshapes = (uint8_t)s.nshapes;
      bs.modes = overflow ? 0 : (uint8_t)modes;
      bs.done = 0;
      if (overflow) atomicOr(status, 2u);
      sel[gl] = bs;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// counts -> offsets (two-level exclusive scan)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kRankChunk) scan_local_u8_kernel(const uint8_t *in, uint64_t n,
                                                                   uint16_t *local,
                                                                   uint32_t *chunk_total) {
  __shared__ uint32_t s_warp[32];
  const uint64_t i = (uint64_t)blockIdx.x * kRankChunk + threadIdx.x;
  const uint32_t v = i < n ? in[i] : 0u;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
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
    if (lane == 31) chunk_total[blockIdx.x] = wi;
  }
  __syncthreads();
  if (i < n) local[i] = (uint16_t)(s_warp[wid] + incl - v);
}

// In-place exclusive scan of the chunk totals; writes the grand total and
// resets the annealing queue.
__global__ void __launch_bounds__(1024) scan_chunks_kernel(uint32_t *chunk, uint32_t nchunks,
                                                           PipelineCounters *ctr) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_carry = 0;
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
  if (threadIdx.x < kClasses) {
    ctr->anneal_next[threadIdx.x] = 0ull;
    ctr->anneal_count[threadIdx.x] = 0u;
    ctr->cont_next[threadIdx.x] = 0ull;
    ctr->cont_count[threadIdx.x] = 0u;
    ctr->reindex_count[threadIdx.x] = 0u;
  }
  if (threadIdx.x < kClasses * 17) (&ctr->nhist[0][0])[threadIdx.x] = 0u;
  if (threadIdx.x == 0) ctr->tasks = s_carry;
}

// ---------------------------------------------------------------------------
// emit
// ---------------------------------------------------------------------------

__global__ void emit_kernel(uint32_t nb, const uint8_t *__restrict__ counts,
                            const uint16_t *__restrict__ local, const uint32_t *__restrict__ chunk,
                            uint2 *__restrict__ desc) {
  const uint32_t gl = blockIdx.x * blockDim.x + threadIdx.x;
  if (gl >= nb) return;
  for (int cl = 0; cl < kClasses; cl++) {
    const uint64_t i = (uint64_t)cl * nb + gl;
    const uint32_t c = counts[i];
    if (!c) continue;
    const uint32_t base = scanned(local, chunk, i);
    for (uint32_t k = 0; k < c; k++) desc[base + k] = make_uint2(gl, (uint32_t)cl | (k << 8));
  }
}

// ---------------------------------------------------------------------------
// setup: one thread per cluster fit
// ---------------------------------------------------------------------------

constexpr int kSetupThreads = 128;
static_assert(kSetupThreads == kLaneStride, "setup arrays use the lane stride");

// First task of class C in the chunk's class-major task arrays.
__device__ __forceinline__ uint32_t class_begin(const uint16_t *local, const uint32_t *chunk,
                                                const PipelineCounters *ctr, uint32_t nb, int c) {
  return c < kClasses ? scanned(local, chunk, (uint64_t)c * nb) : ctr->tasks;
}

// One launch per class (the mode is a compile-time constant, so each
// kernel holds only its own mode's path).
template <int C>
__global__ void __launch_bounds__(kSetupThreads, (class_mode(C) == 6 ? 3 : 6)) setup_kernel(
    const JobDev *__restrict__ jobs, uint32_t nb, const BlockSel *__restrict__ sel,
    const uint2 *__restrict__ desc, const uint16_t *__restrict__ local,
    const uint32_t *__restrict__ chunk, const uint8_t *__restrict__ counts,
    PipelineCounters *__restrict__ ctr, TaskState *__restrict__ state, AnnealRec *__restrict__ arec,
    uint32_t *status) {
  constexpr int kMode = class_mode(C);
  constexpr ModeAttr kA = mode_attr(kMode);
  // Mode 6 runs once per shape slot (CompressClusters searches the
  // one-subset modes with every slot), on the same cluster: the setup is
  // the same and only the annealing stream differs, so one thread per block
  // sets it up and writes the fit of each slot.
  constexpr bool kPerBlock = kMode == 6;
  __shared__ uint32_t s_px[kSetupThreads * 17];
  __shared__ uint32_t s_pts[16 * kSetupThreads];
  // palette of the integer QuantizedError (up to 8 entries; the 16-entry
  // class uses the float restatement)
  __shared__ uint4 s_pal[8 * kSetupThreads];
  uint32_t *px = s_px + threadIdx.x * 17;
  uint32_t *pts = s_pts + threadIdx.x;
  const uint32_t begin = class_begin(local, chunk, ctr, nb, C);
  const uint32_t end = class_begin(local, chunk, ctr, nb, C + 1);
  const int lane = threadIdx.x & 31;
  const uint32_t items = kPerBlock ? nb : end - begin;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < items; k += gridDim.x * blockDim.x) {
    uint32_t t, gl;
    int i = 0, ndup = 1;
    if (kPerBlock) {
      gl = k;
      ndup = (int)counts[(uint64_t)C * nb + gl];
      if (ndup == 0) continue;
      t = scanned(local, chunk, (uint64_t)C * nb + gl);
    } else {
      t = begin + k;
      const uint2 d = desc[t];
      gl = d.x;
      i = (int)(d.y >> 8);
    }
    const BlockSel bs = sel[gl];
    const JobDev &jb = jobs[bs.job];
    const Selection s = sel_of(bs);
    const Task tk = class_task(s, C, i);
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const uint4 v = load_row_p(jb, bs.lin, r);
      px[r * 4 + 0] = v.x;
      px[r * 4 + 1] = v.y;
      px[r * 4 + 2] = v.z;
      px[r * 4 + 3] = v.w;
    }
    const uint32_t bw = jb.width >> 2;
    const uint32_t bx = bs.lin % bw, by = bs.lin / bw;
    ModeCtx m;
    m.mode = kMode;
    m.a = kA;
    m.steps = (int)jb.steps;
    m.metric = (int)jb.metric;
    m.rot = tk.rot;
    m.idx_mode = tk.im;
    m.status = status;
    m.lcg = 0;
    m.sct = g_sct;
    m.pal = s_pal + threadIdx.x;
    Cluster c;
    make_cluster(px, part_word_of(s, kMode, tk.slot), tk.subset, pts, kSetupThreads, c);
    c.aux = px;  // the block's texels are not read again
    c.aux_stride = 1;
    FitSetup st;
    st.idx = 0;
    st.pbit = 0;
    TaskState o;
    o.aerr = 0.0;
    o.aidx = 0;
    o.a1 = o.a2 = 0.0f;
    constexpr int kNB = 1 << (class_im(C) ? kA.alpha_idx_bits : kA.idx_bits);
    constexpr int kANB = 1 << (class_im(C) ? kA.idx_bits : kA.alpha_idx_bits);
    if constexpr (kA.has_rotation != 0) {
      fit_alpha_setup<kNB, kANB, (kNB >= 8)>(m, c, q_opt6, st, o.a1, o.a2, o.aidx, o.aerr);
    } else {
      fit_rgb_setup_t<kNB, (kNB >= 8)>(m, c, st);
    }
    o.err = st.err;
    o.idx = st.idx;
    o.p1 = to_pixel(st.p1, 0xFFFFFFFFu, -1);
    o.p2 = to_pixel(st.p2, 0xFFFFFFFFu, -1);
    o.gl = gl;
    o.mode = (uint8_t)kMode;
    o.subset = (uint8_t)tk.subset;
    o.rotim = (uint8_t)((tk.rot << 1) | tk.im);
    o.steps = (uint16_t)jb.steps;
    o.pbit = (uint8_t)st.pbit;
    o.flags = (uint8_t)((st.anneal ? kTaskAnneal : 0u) | (jb.metric ? kTaskNonuniform : 0u));
    const float lb = st.anneal && !jb.metric ? qe_lower_bound<kNB>(pts, kSetupThreads, c.n) : 0.0f;
    const uint64_t idx0 = o.idx;
#pragma unroll 1
    for (int dup = 0; dup < (kPerBlock ? 2 : 1); dup++) {
      const bool here = dup < ndup;
      const int slot = kPerBlock ? class_task(s, C, dup).slot : tk.slot;
      o.slot = (uint8_t)slot;
      o.lcg = fit_seed(jb.seed, bx, by,
                       (uint32_t)((kMode << 8) | (slot << 7) | (tk.subset << 4) | (tk.rot << 1) | tk.im));
      o.idx = idx0;
      // append to the class's annealing list (warp-aggregated)
      const bool add = here && st.anneal;
      const uint32_t peers = __ballot_sync(__activemask(), add);
      if (add) {
        const int leader = __ffs(peers) - 1;
        uint32_t pos = 0;
        if (lane == leader) pos = atomicAdd(&ctr->anneal_count[C], (uint32_t)__popc(peers));
        pos = __shfl_sync(peers, pos, leader) + __popc(peers & ((1u << lane) - 1u));
        // the bound stage reads the fit's error bound, list position and
        // point count from idx (the re-index stage rewrites it)
        o.idx = (uint64_t)__float_as_uint(lb) | ((uint64_t)pos << 32) | ((uint64_t)c.n << 56);
        uint4 *r = reinterpret_cast<uint4 *>(arec + begin + pos);
#pragma unroll
        for (int q = 0; q < 4; q++)
          r[q] = make_uint4(pts[(4 * q + 0) * kSetupThreads], pts[(4 * q + 1) * kSetupThreads],
                            pts[(4 * q + 2) * kSetupThreads], pts[(4 * q + 3) * kSetupThreads]);
        const uint32_t ef = __float_as_uint((float)o.err);
        r[4] = make_uint4((uint32_t)c.tex, (uint32_t)(c.tex >> 32), o.p1, o.p2);
        r[5] = make_uint4(ef, o.lcg, t + (uint32_t)dup,
                          (uint32_t)o.steps | ((uint32_t)c.n << 16) | ((uint32_t)o.pbit << 24));
        r[6] = make_uint4((uint32_t)tk.rot | ((uint32_t)o.flags << 8), o.p1, o.p2, ef);
        r[7] = make_uint4((uint32_t)o.pbit, 0u, 0u, 0u);
      }
      if (here) state[t + (uint32_t)dup] = o;
    }
  }
}

// Per block, after every class's setup: FasTC keeps the candidate (mode and
// shape slot) with the least total error, and annealing only lowers a fit's
// error, so the winner's final total is at most U, the least total at the
// setup errors. A candidate whose error lower bound exceeds U cannot win:
// its fits skip the annealing and keep their setup errors, which are at
// least the bound, so the arg-min of the choose stage is unchanged. The
// bound of a multi-subset candidate is the sum over its subsets (a fit
// that does not anneal counts with its error); a rotation fit competes on
// its own (the mode keeps its best rotation), with its exact alpha error
// added. The fits left to anneal get their rank among the class's fits
// with as many points (point-count order for the annealing lanes), the
// others a dead key.
constexpr uint32_t kDeadKey = 0xFFFFFFFFu;

__device__ __forceinline__ void keep_fit(PipelineCounters *ctr, uint32_t *keys, uint32_t base,
                                         uint64_t info, bool alive, int c) {
  const uint32_t pos = (uint32_t)(info >> 32) & 0xFFFFFFu;
  const int n = (int)(info >> 56);
  const int lane = threadIdx.x & 31;
  const unsigned act = __activemask();
  const unsigned grp = __match_any_sync(act, alive ? (unsigned)(c * 32 + n) : 0xFFFFFFFFu);
  const int leader = __ffs(grp) - 1;
  uint32_t r0 = 0;
  if (alive && lane == leader) r0 = atomicAdd(&ctr->nhist[c][n], (uint32_t)__popc(grp));
  r0 = __shfl_sync(act, r0, leader);
  keys[base + pos] = alive ? ((uint32_t)n << 24) | (r0 + __popc(grp & ((1u << lane) - 1u))) : kDeadKey;
}

__device__ __forceinline__ float fit_bound(const TaskState &o) {
  return (o.flags & kTaskAnneal) ? __uint_as_float((uint32_t)o.idx) : (float)o.err;
}

__global__ void __launch_bounds__(128) bound_kernel(uint32_t nb, const BlockSel *__restrict__ sel,
                                                    const uint16_t *__restrict__ local,
                                                    const uint32_t *__restrict__ chunk,
                                                    const TaskState *__restrict__ state,
                                                    PipelineCounters *__restrict__ ctr,
                                                    uint32_t *__restrict__ keys) {
  const uint32_t gl = blockIdx.x * blockDim.x + threadIdx.x;
  if (gl >= nb) return;
  const BlockSel bs = sel[gl];
  if (bs.done) return;
  const Selection s = sel_of(bs);
  const uint32_t modes = bs.modes;
  const uint32_t nshapes = s.nshapes < 5 ? s.nshapes : 5;
  double U = DBL_MAX;
  for (int pass = 0; pass < 2; pass++) {
    for (int oi = 0; oi < 8; oi++) {
      const int mode = mode_order(oi);
      if (!(modes & (1u << mode))) continue;
      const ModeAttr a = mode_attr(mode);
      const int nim = mode == 4 ? 2 : 1;
      uint32_t cbase[2];
      for (int k = 0; k < nim; k++)
        cbase[k] = scanned(local, chunk, (uint64_t)class_of(mode, k) * nb + gl);
      uint32_t t = cbase[0];
      int slot_rank = 0;
      for (uint32_t sl = 0; sl < nshapes; sl++) {
        if (a.subsets != 1 && (uint32_t)a.subsets != s.nparts[sl]) continue;
        if (s.shape[sl] >= 16 && mode == 0) continue;
        if (a.has_rotation) {
          for (int r = 0; r < 4; r++)
            for (int k = 0; k < nim; k++) {
              const uint32_t tt = cbase[k] + (uint32_t)(slot_rank * 4 + r);
              const TaskState &o = state[tt];
              if (pass == 0) {
                U = fmin(U, o.err + o.aerr);
              } else if (o.flags & kTaskAnneal) {
                const int c = class_of(mode, k);
                const bool alive = !((double)fit_bound(o) + o.aerr > U + 1.0);
                keep_fit(ctr, keys, scanned(local, chunk, (uint64_t)c * nb), o.idx, alive, c);
              }
            }
        } else if (pass == 0) {
          double total = 0.0;
          for (int ci = 0; ci < a.subsets; ci++) total = total + state[t + ci].err;
          U = fmin(U, total);
        } else {
          double lb = 0.0;
          for (int ci = 0; ci < a.subsets; ci++) lb += (double)fit_bound(state[t + ci]);
          const bool alive = !(lb > U + 1.0);
          const int c = class_of(mode, 0);
          const uint32_t base = scanned(local, chunk, (uint64_t)c * nb);
          for (int ci = 0; ci < a.subsets; ci++) {
            const TaskState &o = state[t + ci];
            if (o.flags & kTaskAnneal) keep_fit(ctr, keys, base, o.idx, alive, c);
          }
        }
        if (!a.has_rotation) t += (uint32_t)a.subsets;
        slot_rank++;
      }
    }
  }
}

// The order in which the annealing lanes take the class's fits that are
// left after the bound stage, by point count (most points first), so that
// the lanes of a warp loop over the same number of texels. perm[k] = list
// index of the k-th fit to take.
template <int C>
__global__ void __launch_bounds__(128) order_kernel(uint32_t nb, const uint16_t *__restrict__ local,
                                                    const uint32_t *__restrict__ chunk,
                                                    const PipelineCounters *__restrict__ ctr,
                                                    const uint32_t *__restrict__ keys,
                                                    uint32_t *__restrict__ perm) {
  __shared__ uint32_t s_off[17];
  const uint32_t count = ctr->anneal_count[C];
  if (blockIdx.x * blockDim.x >= count) return;
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (int n = 16; n >= 0; n--) {
      s_off[n] = acc;
      acc += ctr->nhist[C][n];
    }
  }
  __syncthreads();
  const uint32_t base = scanned(local, chunk, (uint64_t)C * nb);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const uint32_t key = keys[base + i];
    if (key != kDeadKey) perm[base + s_off[key >> 24] + (key & 0xFFFFFFu)] = i;
  }
}

// ---------------------------------------------------------------------------
// anneal: one launch per class, persistent, one thread per fit, refilled
// from the class's list
// ---------------------------------------------------------------------------

constexpr int kAnnealThreads = kLaneStride;

// ToPixel (RGBAEndpoints.cpp:167-177) of integer endpoints through the table.
template <int kColorBits, int kAlphaBits>
__device__ __forceinline__ uint32_t qpix(const uint8_t *lut, uint32_t v, int pbit) {
  const uint8_t *lc = lut + ((kColorBits - 1) * 3 + (pbit + 1)) * 256;
  uint32_t r = (uint32_t)lc[v & 0xFF] | ((uint32_t)lc[(v >> 8) & 0xFF] << 8) |
               ((uint32_t)lc[(v >> 16) & 0xFF] << 16);
  if (kAlphaBits == 0) return r | 0xFF000000u;
  const uint8_t *la = lut + ((kAlphaBits - 1) * 3 + (pbit + 1)) * 256;
  return r | ((uint32_t)la[v >> 24] << 24);
}

// Squared error of a texel against a palette colour, per FasTC's metric.
template <bool kUniform>
__device__ __forceinline__ float texel_err(uint32_t e, uint32_t pal, const float *w) {
  const uint32_t ad = __vabsdiffu4(e, pal);
  if constexpr (kUniform) {
    return (float)__dp4a(ad, ad, 0u);
  } else {
    float ev[4];
#pragma unroll
    for (int c = 0; c < 4; c++) ev[c] = __fmul_rn((float)((ad >> (8 * c)) & 0xFF), w[c]);
    return sqlen4(ev);
  }
}

// QuantizedError (RGBAEndpoints.cpp:190-310) for integer endpoints q1/q2 and
// the fit's texels. The projection floor(D k / L) is exact integer
// arithmetic; FasTC's float rounding only matters when D k is a multiple of
// L, and that case repeats its float division and product.
template <int kBits, bool kRot, bool kUniform, bool kIdx>
__device__ __forceinline__ float qe_simd(const uint32_t *pts, const uint32_t *proj, uint32_t *pal,
                                         int n, uint32_t q1, uint32_t q2, const float *w,
                                         uint64_t tex, uint64_t &idx) {
  constexpr int kNB = 1 << kBits;
  constexpr uint32_t km = kNB - 1;
  constexpr int T = kAnnealThreads;
  int u1[4], dir[4];
#pragma unroll
  for (int c = 0; c < 4; c++) {
    u1[c] = (int)((q1 >> (8 * c)) & 0xFF);
    dir[c] = (int)((q2 >> (8 * c)) & 0xFF) - u1[c];
  }
  const int L = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2] + dir[3] * dir[3];
  uint32_t itotal = 0;
  float ftotal = 0.0f;
  if (L == 0) {
    for (int k = 0; k < n; k++) {
      const uint32_t e = pts[k * T];
      if (kUniform) {
        const uint32_t ad = __vabsdiffu4(e, q1);
        itotal += __dp4a(ad, ad, 0u);
      } else {
        ftotal = __fadd_rn(ftotal, texel_err<false>(e, q1, w));
      }
      if (kIdx) set_nib(idx, (int)((tex >> (4 * k)) & 15), 0);
    }
    return kUniform ? (float)itotal : ftotal;
  }
  // palette of the interpolated colours, two 16-bit lanes at a time
  {
    const uint32_t rb1 = q1 & 0x00FF00FFu, ga1 = (q1 >> 8) & 0x00FF00FFu;
    const uint32_t rb2 = q2 & 0x00FF00FFu, ga2 = (q2 >> 8) & 0x00FF00FFu;
#pragma unroll
    for (int j = 0; j < kNB; j++) {
      const uint32_t w1 = wt<kBits>(j), w0 = 64u - w1;
      const uint32_t vrb = rb1 * w0 + rb2 * w1 + 0x00200020u;
      const uint32_t vga = ga1 * w0 + ga2 * w1 + 0x00200020u;
      pal[j * T] = ((vrb >> 6) & 0x00FF00FFu) | (((vga >> 6) & 0x00FF00FFu) << 8);
    }
  }
  const uint32_t dlo = ((uint32_t)dir[0] & 0xFFFFu) | ((uint32_t)dir[1] << 16);
  const uint32_t dhi = ((uint32_t)dir[2] & 0xFFFFu) | ((uint32_t)dir[3] << 16);
  const int negk = -(dir[0] * u1[0] + dir[1] * u1[1] + dir[2] * u1[2] + dir[3] * u1[3]);
  const uint32_t R = L > 1 ? 0xFFFFFFFFu / (uint32_t)L + 1u : 0u;
  for (int k = 0; k < n; k++) {
    const uint32_t e = pts[k * T];
    const uint32_t p = kRot ? proj[k * T] : e;
    const int D = dp2a_hi(dhi, p, dp2a_lo(dlo, p, negk));
    int j1, j2;
    if (D <= 0) {
      j1 = j2 = 0;
    } else if (D >= L) {
      j1 = j2 = (int)km;
    } else {
      const uint32_t num = (uint32_t)D * km;
      uint32_t q = __umulhi(num, R);
      int r = (int)(num - q * (uint32_t)L);
      if (r < 0) {
        q--;
        r += L;
      }
      j1 = (int)q;
      j2 = (int)q + 1;
      if (r == 0) {
        const float sc = __fmul_rn(__fdiv_rn((float)D, (float)L), (float)km);
        j1 = min(max(0, __float2int_rz(floorf(sc))), (int)km);
        j2 = min(__float2int_rz(ceilf(sc)), (int)km);
      }
    }
    const float e1 = texel_err<kUniform>(e, pal[j1 * T], w);
    float best = e1;
    int bj = j1;
    if (j2 > j1) {
      const float e2 = texel_err<kUniform>(e, pal[(j1 + 1) * T], w);
      if (e2 < e1) {
        best = e2;
        bj = j1 + 1;
      }
    }
    if (kUniform) itotal += (uint32_t)best;
    else ftotal = __fadd_rn(ftotal, best);
    if (kIdx) set_nib(idx, (int)((tex >> (4 * k)) & 15), (uint32_t)bj);
  }
  return kUniform ? (float)itotal : ftotal;
}

struct Lane {
  uint32_t t;
  uint32_t p1, p2, b1, b2, lcg;
  int cur_pbit, best_pbit, energy, steps, n;
  float cur_err, best_err;
  uint64_t tex;
  float w[4];
  int se;         // sum of |e|^2 over the fit's texels
  uint32_t psel;  // byte selector of the projected point (rotation modes)
  int rot;
  bool uniform;
};

// Quantized error of endpoints q1, q2 for class C: integer path for the
// uniform metric, the float path otherwise.
template <int C, bool kIdx>
__device__ __forceinline__ float class_qe(const Lane &s, const uint32_t (&ereg)[16],
                                          const uint32_t (&preg)[16],
                                          const uint32_t *pts, const uint32_t *proj, uint4 *pal,
                                          uint32_t *palf, uint32_t q1, uint32_t q2, uint64_t &idx) {
  constexpr int kMode = class_mode(C);
  constexpr ModeAttr a = mode_attr(kMode);
  constexpr int kBits = class_im(C) ? a.alpha_idx_bits : a.idx_bits;
  constexpr bool kRot = a.has_rotation != 0;
  constexpr bool kN16 = a.subsets == 1;
  if (s.uniform) {
    if constexpr (kN16) return qe_reg<kBits, kRot, kIdx>(ereg, preg, s.se, pal, q1, q2, idx);
    else return qe_smem<kBits, kIdx>(pts, s.n, s.tex, s.se, pal, q1, q2, idx);
  }
  // float metric: palette as plain colours in the same buffer
  return qe_simd<kBits, kRot, false, kIdx>(pts, proj, palf, s.n, q1, q2, s.w, s.tex, idx);
}

// One iteration of OptimizeEndpointsForCluster's loop (CP:583-624) for
// class C; returns true when the fit is finished.
template <int C>
__device__ __forceinline__ bool anneal_step(Lane &s, const uint32_t (&ereg)[16],
                                            const uint32_t (&preg)[16], const uint32_t *pts,
                                            const uint32_t *proj, uint4 *pal, uint32_t *palf,
                                            const uint8_t *lut) {
  constexpr int kMode = class_mode(C);
  constexpr ModeAttr a = mode_attr(kMode);
  constexpr bool kHasPbits = a.pbit != kPBitNone;
  if (!(s.best_err > 0.0f && s.energy < s.steps)) return true;
  // PickBestNeighboringEndpoints (CP:426-498) on integer endpoints
  constexpr int sc = 1 << (8 - a.color_bits);
  constexpr int sa = kMode < 4 ? 0 : (1 << (8 - a.alpha_bits));
  int npbit = 0;
  if (kHasPbits) npbit = a.pbit == kPBitShared ? (s.cur_pbit + 1) % 2 : 3 - s.cur_pbit;
  const int cur_combo = pbit_combo(a, s.cur_pbit);
  uint32_t np1 = s.p1, np2 = s.p2;
  bool visited = true;
  int guard = -1;
  while (visited && ++guard < 16) {
#pragma unroll
    for (int pt = 0; pt < 2; pt++) {
      const uint32_t p = pt ? s.p1 : s.p2;
      const uint32_t dir = lcg_next(s.lcg) % 16;
      const int old = pt ? pb_second(cur_combo) : pb_first(cur_combo);
      uint32_t np = 0;
#pragma unroll
      for (int c = 0; c < 4; c++) {
        int v = (int)((p >> (8 * c)) & 0xFF);
        const int st = c == 3 ? sa : sc;
        const bool down = (dir >> c) & 1;
        if (kHasPbits) {
          if (down && old == 0) v -= st;
          else if (!down && old == 1) v += st;
        } else {
          v = down ? v - st : v + st;
        }
        v = min(max(v, 0), 255);
        np |= (uint32_t)v << (8 * c);
      }
      if (pt) np1 = np;
      else np2 = np;
    }
    visited = np1 == s.b1 && np2 == s.b2 && npbit == s.best_pbit;
  }
  // QuantizedError with the new p-bit combo (kPBits[0] for modes without
  // p-bits, as FasTC passes it)
  const int pc = pbit_combo(a, npbit);
  const uint32_t q1 = qpix<a.color_bits, a.alpha_bits>(lut, np1, pb_first(pc));
  const uint32_t q2 = qpix<a.color_bits, a.alpha_bits>(lut, np2, pb_second(pc));
  uint64_t unused = 0;
  const float err = class_qe<C, false>(s, ereg, preg, pts, proj, pal, palf, q1, q2, unused);
  // AcceptNewEndpointError (CP:524-536)
  bool accept = err < s.cur_err;
  if (!accept) {
    const uint32_t r16 = lcg_next(s.lcg) & 0xFFFF;
    const uint32_t mant = (r16 << 8) | (r16 >> 7);
    const float r = __fsub_rn(__uint_as_float((127u << 23) | mant), 1.0f);
    // A nonzero draw is at least 2^-15 and exp(x) < 2^-15 for x < -10.5, so
    // when 0.1 (err - cur) (steps - 1) > 12 energy (x < -12 with room for
    // rounding) the move is rejected without FasTC's divisions and exp.
    const bool hopeless = mant != 0 && s.energy > 0 &&
                          __fmul_rn(__fmul_rn(__fsub_rn(err, s.cur_err), 0.1f), (float)(s.steps - 1)) >
                              12.0f * (float)s.energy;
    if (r < 1.0f && !hopeless) {
      const float temp = __fdiv_rn((float)s.energy, (float)(s.steps - 1));
      const float x = __fdiv_rn(__fmul_rn(0.1f, __fsub_rn(s.cur_err, err)), temp);
      accept = mant == 0 ? (x > -745.0f) : (r < portable_expf(x));
    }
  }
  if (accept) {
    s.cur_err = err;
    s.p1 = np1;
    s.p2 = np2;
    s.cur_pbit = npbit;
  }
  if (err < s.best_err) {
    s.b1 = np1;
    s.b2 = np2;
    s.best_pbit = npbit;
    s.best_err = err;
    s.energy = 0;
  }
  s.energy++;
  return false;
}

// Continuation lists: two generations for each rotation class (modes 4
// and 5, classes 4-6), list (generation - 1) * 3 + class - 4.
constexpr int kContLists = 6;
__host__ __device__ constexpr int cont_list(int c, int gen) { return (gen - 1) * 3 + (c - 4); }

// kPhase 0: the class's list of fits from the setup stage. When that list
// is empty, a warp with at most yield_lanes lanes still annealing writes
// their fits, mid-flight, to the class's first continuation list and
// exits, instead of running on with most lanes idle (fit lengths vary
// more than tenfold). kPhase 1: that list, handing on to the second list
// the same way; kPhase 2: the second list, run to completion. Only the
// rotation classes, whose fits are long, hand fits on.
template <int C, int kPhase>
__global__ void __launch_bounds__(kAnnealThreads) anneal_kernel(
    uint32_t nb, const uint16_t *__restrict__ local, const uint32_t *__restrict__ chunk,
    PipelineCounters *__restrict__ ctr, const AnnealRec *__restrict__ arec,
    const uint32_t *__restrict__ perm, AnnealRec *__restrict__ cont, uint32_t cont_cap,
    int yield_lanes, TaskState *__restrict__ state) {
  constexpr int kMode = class_mode(C);
  constexpr ModeAttr a = mode_attr(kMode);
  constexpr int kBits = class_im(C) ? a.alpha_idx_bits : a.idx_bits;
  constexpr bool kRot = a.has_rotation != 0;
  constexpr int T = kAnnealThreads;
  constexpr bool kCont = kPhase > 0;
  constexpr bool kYields = kRot && kPhase < 2;
  constexpr int kRefillBatch = kRot || kCont ? 1 : 4;
  constexpr int kIn = kCont ? cont_list(C, kPhase) : 0;        // list read by a continuation phase
  constexpr int kOut = kYields ? cont_list(C, kPhase + 1) : 0;  // list fits are handed on to
  AnnealRec *clist = cont + (size_t)kIn * cont_cap;
  AnnealRec *olist = cont + (size_t)kOut * cont_cap;
  if (kCont && blockIdx.x * (uint32_t)T >= ctr->cont_count[kIn]) return;
  __shared__ uint8_t s_lut[8 * 3 * 256];
  __shared__ uint32_t s_pts[16 * T];
  __shared__ uint32_t s_proj[kRot ? 16 * T : 1];
  __shared__ uint4 s_pal[(1 << kBits) * T];
  for (int i = threadIdx.x; i < 8 * 3 * 256; i += blockDim.x) s_lut[i] = (&q_qlut[0][0][0])[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  uint32_t *pts = s_pts + threadIdx.x;
  uint32_t *proj = kRot ? s_proj + threadIdx.x : pts;
  uint4 *pal = s_pal + threadIdx.x;
  uint32_t *palf = reinterpret_cast<uint32_t *>(s_pal) + threadIdx.x;  // float-metric palette
  // the fits left after the bound stage, in the order of perm
  uint32_t count = 0;
  if (kCont) {
    count = ctr->cont_count[kIn];
  } else {
#pragma unroll
    for (int n = 0; n <= 16; n++) count += ctr->nhist[C][n];
  }
  const uint32_t lbase = scanned(local, chunk, (uint64_t)C * nb);
  const AnnealRec *list = kCont ? clist : arec + lbase;
  constexpr bool kOrdered = !kCont;
  unsigned long long *cursor = kCont ? &ctr->cont_next[kIn] : &ctr->anneal_next[C];
  Lane s;
  uint32_t ereg[16], preg[16];
  bool active = false, exhausted = false;
  for (;;) {
    const bool need = !active && !exhausted;
    uint32_t nmask = __ballot_sync(0xFFFFFFFFu, need);
    // Short fits finish every few steps somewhere in the warp; refilling in
    // batches of kRefillBatch lanes (or when no lane is left running) keeps
    // the divergent refill and its two memory round trips rare.
    if (__popc(nmask) < kRefillBatch && __ballot_sync(0xFFFFFFFFu, active) != 0) nmask = 0;
    if (nmask) {
      unsigned long long b0 = 0;
      const int leader = __ffs(nmask) - 1;
      if (lane == leader) b0 = atomicAdd(cursor, (unsigned long long)__popc(nmask));
      b0 = __shfl_sync(0xFFFFFFFFu, b0, leader);
      if (need) {
        const unsigned long long k = b0 + __popc(nmask & ((1u << lane) - 1u));
        if (k >= count) {
          exhausted = true;
        } else {
          const uint32_t li = kOrdered ? __ldg(perm + lbase + (uint32_t)k) : (uint32_t)k;
          const uint4 *r = reinterpret_cast<const uint4 *>(list + li);
          uint4 v[8];
#pragma unroll
          for (int q = 0; q < 8; q++) v[q] = kCont ? r[q] : __ldg(r + q);
          const int rot = (int)(v[6].x & 0xFF);
          const uint32_t flags = (v[6].x >> 8) & 0xFF;
          s.t = v[5].z;
          s.p1 = v[4].z;
          s.p2 = v[4].w;
          s.b1 = v[6].y;
          s.b2 = v[6].z;
          s.cur_pbit = (int)(v[5].w >> 24);
          s.best_pbit = (int)(v[7].x & 0xFF);
          s.cur_err = __uint_as_float(v[5].x);
          s.best_err = __uint_as_float(v[6].w);
          s.lcg = v[5].y;
          s.energy = (int)(v[6].x >> 16);
          s.steps = (int)(v[5].w & 0xFFFF);
          s.n = (int)((v[5].w >> 16) & 0xFF);
          s.tex = (uint64_t)v[4].x | ((uint64_t)v[4].y << 32);
          s.uniform = !(flags & kTaskNonuniform);
          // projected point: channel rot-1 takes the texel's alpha, alpha is 255
          s.psel = rot ? (0x4210u & ~(0xFu << (4 * (rot - 1)))) | (3u << (4 * (rot - 1))) : 0x4210u;
          s.rot = rot;
          ModeCtx m;
          m.a = a;
          m.rot = rot;
          m.metric = s.uniform ? 0 : 1;
          metric_of(m, s.w);
          int se = 0;
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const uint32_t vv[4] = {v[q].x, v[q].y, v[q].z, v[q].w};
#pragma unroll
            for (int c = 0; c < 4; c++) {
              const uint32_t e = vv[c];
              ereg[4 * q + c] = e;
              if (4 * q + c < s.n) se += (int)__dp4a(e, e, 0u);
              pts[(4 * q + c) * T] = e;
              if (kRot) {
                preg[4 * q + c] = __byte_perm(e, 0xFFFFFFFFu, s.psel);
                proj[(4 * q + c) * T] = preg[4 * q + c];
              }
            }
          }
          s.se = se;
          active = true;
        }
      }
    }
    if (__all_sync(0xFFFFFFFFu, exhausted && !active)) break;
    // a lane finished (nmask != 0): with the list empty, maybe retire
    if (kYields && nmask) {
      const uint32_t act = __ballot_sync(0xFFFFFFFFu, active);
      if (__any_sync(0xFFFFFFFFu, exhausted) && __popc(act) <= yield_lanes) {
        // hand the unfinished fits on and retire the warp
        const int leader = __ffs(act) - 1;
        uint32_t pos = 0;
        if (lane == leader) pos = atomicAdd(&ctr->cont_count[kOut], (uint32_t)__popc(act));
        pos = __shfl_sync(0xFFFFFFFFu, pos, leader) + __popc(act & ((1u << lane) - 1u));
        if (active) {
          // the list holds one record per lane of the grid, so pos < cont_cap
          uint4 *w = reinterpret_cast<uint4 *>(olist + pos);
#pragma unroll
          for (int q = 0; q < 4; q++)
            w[q] = make_uint4(pts[(4 * q + 0) * T], pts[(4 * q + 1) * T], pts[(4 * q + 2) * T],
                              pts[(4 * q + 3) * T]);
          w[4] = make_uint4((uint32_t)s.tex, (uint32_t)(s.tex >> 32), s.p1, s.p2);
          w[5] = make_uint4(__float_as_uint(s.cur_err), s.lcg, s.t,
                            (uint32_t)s.steps | ((uint32_t)s.n << 16) | ((uint32_t)s.cur_pbit << 24));
          w[6] = make_uint4((uint32_t)s.rot | ((s.uniform ? 0u : (uint32_t)kTaskNonuniform) << 8) |
                                ((uint32_t)s.energy << 16),
                            s.b1, s.b2, __float_as_uint(s.best_err));
          w[7] = make_uint4((uint32_t)s.best_pbit, 0u, 0u, 0u);
        }
        break;
      }
    }
    if (active) {
      if (anneal_step<C>(s, ereg, preg, pts, proj, pal, palf, s_lut)) {
        // the indices of the best endpoints are recomputed by the pack
        // stage for the fits that win their block
        TaskState &o = state[s.t];
        o.p1 = s.b1;
        o.p2 = s.b2;
        o.pbit = (uint8_t)s.best_pbit;
        o.err = (double)s.best_err;
        active = false;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// pack: one thread per block
// ---------------------------------------------------------------------------

__device__ __forceinline__ void fit_out_of(const TaskState &o, FitOut &f) {
  const bool rotation = mode_attr(o.mode).has_rotation != 0;
  unpack4(o.p1, f.p1);
  unpack4(o.p2, f.p2);
  if (rotation) {
    f.p1[3] = o.a1;
    f.p2[3] = o.a2;
  }
  f.err = o.err;
  f.idx = o.idx;
  f.aidx = o.aidx;
  f.pbit = o.pbit;
}

// Colour indices of an annealed fit at its best endpoints: the
// QuantizedError call that ends OptimizeEndpointsForCluster (CP:626-629),
// run by the pack stage for winning fits only. px: the block's 16 texels,
// thread-private, stride kLaneStride.
template <int C>
__device__ __noinline__ uint64_t fit_indices(const TaskState &o, const uint32_t *px, uint32_t part,
                                             const uint8_t *lut, uint32_t *pts, uint32_t *proj,
                                             uint4 *pal, uint32_t *palf) {
  constexpr int kMode = class_mode(C);
  constexpr ModeAttr a = mode_attr(kMode);
  constexpr bool kRot = a.has_rotation != 0;
  constexpr int T = kLaneStride;
  Lane s;
  const int rot = o.rotim >> 1;
  s.uniform = !(o.flags & kTaskNonuniform);
  s.psel = rot ? (0x4210u & ~(0xFu << (4 * (rot - 1)))) | (3u << (4 * (rot - 1))) : 0x4210u;
  ModeCtx m;
  m.a = a;
  m.rot = rot;
  m.metric = s.uniform ? 0 : 1;
  metric_of(m, s.w);
  uint32_t ereg[16], preg[16];
#pragma unroll
  for (int k = 0; k < 16; k++) {
    ereg[k] = px[k * T];
    preg[k] = __byte_perm(ereg[k], 0xFFFFFFFFu, s.psel);
  }
  int n = 0, se = 0;
  uint64_t tex = 0;
  for (int i = 0; i < 16; i++) {
    if ((int)((part >> (2 * i)) & 3u) != o.subset) continue;
    const uint32_t e = px[i * T];
    pts[n * T] = e;
    if (kRot) proj[n * T] = __byte_perm(e, 0xFFFFFFFFu, s.psel);
    tex |= (uint64_t)i << (4 * n);
    se += (int)__dp4a(e, e, 0u);
    n++;
  }
  s.n = n;
  s.tex = tex;
  s.se = se;
  const int pc = pbit_combo(a, o.pbit);
  const uint32_t q1 = qpix<a.color_bits, a.alpha_bits>(lut, o.p1, pb_first(pc));
  const uint32_t q2 = qpix<a.color_bits, a.alpha_bits>(lut, o.p2, pb_second(pc));
  uint64_t idx = 0;
  class_qe<C, true>(s, ereg, preg, pts, proj, pal, palf, q1, q2, idx);
  return idx;
}

constexpr int kPackThreads = kLaneStride;

// The winning fit of a block: mode | slot << 4 | rotation << 8 | index mode
// << 12 (mode 8: no fit, 9: block already written), first task index.
__device__ __forceinline__ uint2 make_winner(int mode, int slot, int rot, int im, uint32_t first) {
  return make_uint2((uint32_t)mode | ((uint32_t)slot << 4) | ((uint32_t)rot << 8) | ((uint32_t)im << 12),
                    first);
}

// Per block: FasTC's arg-min over modes and shape slots (CompressClusters,
// CP:1752-1817, strict <, mode order {0,2,1,3,7,4,5,6}); the winner's
// annealed fits go to their class's re-index list.
__global__ void __launch_bounds__(kPackThreads) choose_kernel(
    uint32_t nb, const BlockSel *__restrict__ sel, const uint16_t *__restrict__ local,
    const uint32_t *__restrict__ chunk, const TaskState *__restrict__ state,
    PipelineCounters *__restrict__ ctr, uint2 *__restrict__ win, uint32_t *__restrict__ rlist,
    uint32_t rcap) {
  const uint32_t gl = blockIdx.x * blockDim.x + threadIdx.x;
  if (gl >= nb) return;
  const BlockSel bs = sel[gl];
  if (bs.done) {
    win[gl] = make_winner(9, 0, 0, 0, 0);
    return;
  }
  const Selection s = sel_of(bs);
  const uint32_t modes = bs.modes;
  double best = DBL_MAX;
  int best_mode = 8, best_slot = 0, best_rot = 0, best_im = 0;
  uint32_t best_first = 0;
  const uint32_t nshapes = s.nshapes < 5 ? s.nshapes : 5;
  for (int oi = 0; oi < 8; oi++) {
    const int mode = mode_order(oi);
    if (!(modes & (1u << mode))) continue;
    const ModeAttr a = mode_attr(mode);
    const int nim = mode == 4 ? 2 : 1;
    uint32_t cbase[2];
    for (int k = 0; k < nim; k++)
      cbase[k] = scanned(local, chunk, (uint64_t)class_of(mode, k) * nb + gl);
    uint32_t t = cbase[0];
    int slot_rank = 0;
    for (uint32_t sl = 0; sl < nshapes; sl++) {
      if (a.subsets != 1 && (uint32_t)a.subsets != s.nparts[sl]) continue;
      if (s.shape[sl] >= 16 && mode == 0) continue;
      double total = 0.0;
      uint32_t first = t;
      int rot = 0, im = 0;
      if (a.has_rotation) {
        // rotation-major, index-mode-minor, like CompressionMode::Compress
        double b = DBL_MAX;
        for (int r = 0; r < 4; r++)
          for (int k = 0; k < nim; k++) {
            const uint32_t tt = cbase[k] + (uint32_t)(slot_rank * 4 + r);
            const double e = state[tt].err + state[tt].aerr;
            if (e < b) {
              b = e;
              first = tt;
              rot = r;
              im = k;
            }
          }
        total = total + b;
      } else {
        for (int ci = 0; ci < a.subsets; ci++, t++) total = total + state[t].err;
      }
      slot_rank++;
      if (total < best) {
        best = total;
        best_mode = mode;
        best_slot = (int)sl;
        best_first = first;
        best_rot = rot;
        best_im = im;
      }
    }
  }
  win[gl] = make_winner(best_mode, best_slot, best_rot, best_im, best_first);
  if (best_mode == 8) return;
  const int ns = mode_attr(best_mode).subsets;
  for (int k = 0; k < ns; k++) {
    const uint32_t tt = best_first + (uint32_t)k;
    if (!(state[tt].flags & kTaskAnneal)) continue;
    const int c = class_of(best_mode, best_im);
    const uint32_t pos = atomicAdd(&ctr->reindex_count[c], 1u);
    rlist[(size_t)c * rcap + pos] = tt;  // at most one winner per block and 3 subsets: pos < rcap
  }
}

// One thread per annealed winning fit of class C: its indices at the best
// endpoints (the QuantizedError call that ends the annealing, CP:626-629).
template <int C>
__global__ void __launch_bounds__(kPackThreads) reindex_kernel(
    const JobDev *__restrict__ jobs, const BlockSel *__restrict__ sel,
    const PipelineCounters *__restrict__ ctr, const uint32_t *__restrict__ rlist, uint32_t rcap,
    TaskState *__restrict__ state) {
  constexpr int T = kPackThreads;
  constexpr ModeAttr kA = mode_attr(class_mode(C));
  constexpr bool kN16 = kA.subsets == 1;  // the points are the block's texels, in order
  constexpr bool kRot = kA.has_rotation != 0;
  const uint32_t count = ctr->reindex_count[C];
  if (blockIdx.x * (uint32_t)T >= count) return;
  __shared__ uint8_t s_lut[8 * 3 * 256];
  __shared__ uint32_t s_px[16 * T], s_pts[kN16 ? 1 : 16 * T], s_proj[kRot ? 16 * T : 1];
  __shared__ uint4 s_pal[(1 << (class_im(C) ? mode_attr(class_mode(C)).alpha_idx_bits
                                            : mode_attr(class_mode(C)).idx_bits)) * T];
  for (int i = threadIdx.x; i < 8 * 3 * 256; i += blockDim.x) s_lut[i] = (&q_qlut[0][0][0])[i];
  __syncthreads();
  for (uint32_t i = blockIdx.x * T + threadIdx.x; i < count; i += gridDim.x * T) {
    const uint32_t tt = rlist[(size_t)C * rcap + i];
    TaskState &o = state[tt];
    const BlockSel bs = sel[o.gl];
    const JobDev &jb = jobs[bs.job];
    uint32_t *px = s_px + threadIdx.x;
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const uint4 v = load_row_p(jb, bs.lin, r);
      px[(4 * r + 0) * T] = v.x;
      px[(4 * r + 1) * T] = v.y;
      px[(4 * r + 2) * T] = v.z;
      px[(4 * r + 3) * T] = v.w;
    }
    const uint32_t part = part_word_of(sel_of(bs), class_mode(C), o.slot);
    const TaskState oc = o;
    uint32_t *pts = kN16 ? px : s_pts + threadIdx.x;
    uint32_t *proj = kRot ? s_proj + threadIdx.x : pts;
    o.idx = fit_indices<C>(oc, px, part, s_lut, pts, proj, s_pal + threadIdx.x,
                           reinterpret_cast<uint32_t *>(s_pal) + threadIdx.x);
  }
}

// Per block: the 128-bit packing of the winner (CompressionMode::Pack,
// CP:1096-1298).
__global__ void __launch_bounds__(kPackThreads) pack_kernel(const JobDev *__restrict__ jobs, uint32_t nb,
                            const BlockSel *__restrict__ sel, const uint2 *__restrict__ win,
                            const TaskState *__restrict__ state) {
  __shared__ uint32_t s_part2[64], s_part3[64];
  __shared__ uint8_t s_anc2[64], s_anc3[64];
  for (int i = threadIdx.x; i < 64; i += blockDim.x) {
    s_part2[i] = q_part2[i];
    s_part3[i] = q_part3[i];
    s_anc2[i] = q_anchor2[i];
    s_anc3[i] = q_anchor3[i];
  }
  __syncthreads();
  const uint32_t gl = blockIdx.x * blockDim.x + threadIdx.x;
  if (gl >= nb) return;
  const uint2 w = win[gl];
  const int best_mode = (int)(w.x & 15);
  if (best_mode == 9) return;
  const BlockSel bs = sel[gl];
  const JobDev &jb = jobs[bs.job];
  uint32_t out[4];
  if (best_mode == 8) {
    out[0] = 1u << 6;
    out[1] = out[2] = out[3] = 0;
  } else {
    const Selection s = sel_of(bs);
    FitOut f[3];
    const int ns = mode_attr(best_mode).subsets;
    for (int k = 0; k < ns; k++) fit_out_of(state[w.y + k], f[k]);
    pack_block(best_mode, s, (int)((w.x >> 4) & 15), f, s_anc2, s_anc3, s_part2, s_part3,
               (int)((w.x >> 8) & 15), (int)((w.x >> 12) & 15), out);
  }
  store_block_p(jb, bs.lin, out);
}

// ---------------------------------------------------------------------------
// launcher
// ---------------------------------------------------------------------------

namespace {

// Continuation records per class: one per lane of an annealing grid at
// most (a lane hands on at most one fit), and never more than the tasks.
uint64_t cont_capacity(uint64_t nb, int tb, int sm_count) {
  const uint64_t lanes = (uint64_t)sm_count * 2048u;  // resident threads per SM
  const uint64_t tasks = (uint64_t)tb * nb;
  return lanes < tasks ? lanes : tasks;
}

// Bytes of one chunk buffer for chunks of at most nb blocks.
size_t chunk_buffer_bytes(uint64_t nb, int tb, int sm_count) {
  const uint64_t n8 = (uint64_t)kClasses * nb;
  const uint64_t tmax = (uint64_t)tb * nb;
  size_t b = kCountersSlot;  // PipelineCounters
  b += (nb * sizeof(BlockSel) + 255) & ~255ull;
  b += (n8 + 255) & ~255ull;
  b += (n8 * 2 + 255) & ~255ull;
  b += (((n8 + kRankChunk - 1) / kRankChunk) * 4 + 255) & ~255ull;
  b += (tmax * sizeof(uint2) + 255) & ~255ull;
  b += (tmax * sizeof(TaskState) + 255) & ~255ull;
  b += (tmax * sizeof(AnnealRec) + 255) & ~255ull;
  b += (kContLists * cont_capacity(nb, tb, sm_count) * sizeof(AnnealRec) + 255) & ~255ull;
  b += (nb * sizeof(uint2) + 255) & ~255ull;                      // winners
  b += ((uint64_t)kClasses * 3 * nb * sizeof(uint32_t) + 255) & ~255ull;  // re-index lists
  b += 2 * ((tmax * sizeof(uint32_t) + 255) & ~255ull);           // point-count keys, order
  return b;
}

struct ChunkBuf {
  PipelineCounters *ctr;
  BlockSel *sel;
  uint8_t *counts;
  uint16_t *local;
  uint32_t *chunk;
  uint2 *desc;
  TaskState *state;
  AnnealRec *arec;
  AnnealRec *cont;
  uint32_t cont_cap;
  uint2 *win;
  uint32_t *rlist;
  uint32_t rcap;
  uint32_t *keys, *perm;
};

ChunkBuf carve_chunk(uint8_t *p, uint64_t nb, int tb, int sm_count) {
  ChunkBuf c;
  c.ctr = reinterpret_cast<PipelineCounters *>(p);
  p += kCountersSlot;
  c.sel = reinterpret_cast<BlockSel *>(p);
  p += (nb * sizeof(BlockSel) + 255) & ~255ull;
  c.counts = p;
  p += ((uint64_t)kClasses * nb + 255) & ~255ull;
  c.local = reinterpret_cast<uint16_t *>(p);
  p += ((uint64_t)kClasses * 2 * nb + 255) & ~255ull;
  c.chunk = reinterpret_cast<uint32_t *>(p);
  p += ((((uint64_t)kClasses * nb + kRankChunk - 1) / kRankChunk) * 4 + 255) & ~255ull;
  c.desc = reinterpret_cast<uint2 *>(p);
  p += ((uint64_t)tb * nb * sizeof(uint2) + 255) & ~255ull;
  c.state = reinterpret_cast<TaskState *>(p);
  p += ((uint64_t)tb * nb * sizeof(TaskState) + 255) & ~255ull;
  c.arec = reinterpret_cast<AnnealRec *>(p);
  p += ((uint64_t)tb * nb * sizeof(AnnealRec) + 255) & ~255ull;
  c.cont = reinterpret_cast<AnnealRec *>(p);
  c.cont_cap = (uint32_t)cont_capacity(nb, tb, sm_count);
  p += ((uint64_t)kContLists * c.cont_cap * sizeof(AnnealRec) + 255) & ~255ull;
  c.win = reinterpret_cast<uint2 *>(p);
  p += (nb * sizeof(uint2) + 255) & ~255ull;
  c.rlist = reinterpret_cast<uint32_t *>(p);
  c.rcap = (uint32_t)(3 * nb);
  p += ((uint64_t)kClasses * 3 * nb * sizeof(uint32_t) + 255) & ~255ull;
  c.keys = reinterpret_cast<uint32_t *>(p);
  p += ((uint64_t)tb * nb * sizeof(uint32_t) + 255) & ~255ull;
  c.perm = reinterpret_cast<uint32_t *>(p);
  return c;
}

}  // namespace

int block_task_bound(uint32_t modes, bool stats) {
  modes &= 0xFFu;
  // BoxSelection's outcomes (CP:1670-1750): opaque blocks search two shape
  // slots (2 and 3 subsets) with modes 4 and 5 removed, or one slot's modes
  // after an exact fit; other blocks one 2-subset slot with the alpha modes.
  // The logging encoder's (CP:2046-2166): every mode, on two slots for
  // opaque blocks and one for the others, or the exact fit's modes.
  struct Outcome { uint32_t modes; int nshapes; };
  const Outcome plain[4] = {{0xFFu & ~((1u << 4) | (1u << 5)), 2}, {kModesTwo, 1},
                            {kModesThree, 2}, {kModesAlpha, 1}};
  const Outcome logged[4] = {{0xFFu, 2}, {kModesTwo, 2}, {kModesThree, 2}, {0xFFu, 1}};
  const Outcome *outs = stats ? logged : plain;
  int worst = 0;
  for (int oi = 0; oi < 4; oi++) {
    const Outcome &o = outs[oi];
    uint32_t m = o.modes & modes;
    if (m == 0) m = modes;  // the fallback to the caller's mask
    int n = 0;
    for (int mode = 0; mode < 8; mode++) {
      if (!(m & (1u << mode))) continue;
      const ModeAttr a = mode_attr(mode);
      for (int sl = 0; sl < o.nshapes; sl++) {
        const int nparts = sl == 0 ? 2 : 3;
        if (a.subsets != 1 && a.subsets != nparts) continue;
        n += a.has_rotation ? 4 * (mode == 4 ? 2 : 1) : a.subsets;
      }
    }
    worst = n > worst ? n : worst;
  }
  return worst;
}

uint64_t pipeline_chunk_blocks(int task_bound, const PipelineTuning &tune) {
  const uint64_t dflt = pipeline_chunk(task_bound);
  if (tune.chunk_blocks == 0 || tune.chunk_blocks >= dflt) return dflt;
  const uint64_t c = tune.chunk_blocks / kRankChunk * kRankChunk;
  return c < kRankChunk ? kRankChunk : c;
}

size_t pipeline_scratch_bytes(uint64_t total_blocks, int task_bound, int sm_count,
                              uint64_t chunk_blocks) {
  PipelineTuning t;
  t.chunk_blocks = chunk_blocks;
  const uint64_t cap = pipeline_chunk_blocks(task_bound, t);
  const uint64_t nb = total_blocks < cap ? total_blocks : cap;
  const int nbuf = total_blocks > cap ? 2 : 1;
  return (size_t)nbuf * chunk_buffer_bytes(nb, task_bound, sm_count);
}

size_t pipeline_scratch_bytes(uint64_t total_blocks, int task_bound, int sm_count) {
  const uint64_t cap = pipeline_chunk(task_bound);
  const uint64_t nb = total_blocks < cap ? total_blocks : cap;
  const int nbuf = total_blocks > cap ? 2 : 1;
  return (size_t)nbuf * chunk_buffer_bytes(nb, task_bound, sm_count);
}

cudaError_t class_streams_create(ClassStreams *cs) {
  *cs = ClassStreams{};
  cudaError_t e = cudaSuccess;
  for (int b = 0; b < 2 && e == cudaSuccess; b++) {
    e = cudaEventCreateWithFlags(&cs->fork[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&cs->bound[b], cudaEventDisableTiming);
    for (int c = 0; c < kClasses && e == cudaSuccess; c++)
      e = cudaEventCreateWithFlags(&cs->join[b][c], cudaEventDisableTiming);
    for (int c = 0; c < kClasses && e == cudaSuccess; c++)
      e = cudaEventCreateWithFlags(&cs->setup[b][c], cudaEventDisableTiming);
  }
  for (int b = 0; b < 2 && e == cudaSuccess; b++)
    for (int c = 0; c < kClasses && e == cudaSuccess; c++)
      e = cudaStreamCreateWithFlags(&cs->side[b][c], cudaStreamNonBlocking);
  if (e != cudaSuccess) class_streams_destroy(cs);
  return e;
}

void class_streams_destroy(ClassStreams *cs) {
  for (int b = 0; b < 2; b++)
    for (int c = 0; c < kClasses; c++)
      if (cs->side[b][c]) cudaStreamDestroy(cs->side[b][c]);
  for (int b = 0; b < 2; b++) {
    if (cs->fork[b]) cudaEventDestroy(cs->fork[b]);
    if (cs->bound[b]) cudaEventDestroy(cs->bound[b]);
    for (int c = 0; c < kClasses; c++) {
      if (cs->join[b][c]) cudaEventDestroy(cs->join[b][c]);
      if (cs->setup[b][c]) cudaEventDestroy(cs->setup[b][c]);
    }
  }
  *cs = ClassStreams{};
}

namespace {

struct ChunkArgs {
  const JobDev *jobs;
  uint32_t nb;
  const BlockSel *sel;
  const uint2 *desc;
  const uint16_t *local;
  const uint32_t *chunk;
  const uint8_t *counts;
  PipelineCounters *ctr;
  TaskState *state;
  AnnealRec *arec;
  AnnealRec *cont;
  uint32_t cont_cap;
  uint32_t *keys, *perm;
  uint32_t *status;
  int sm_count;
  int anneal_ctas, yield_lanes;
  int setup_ctas;  // per SM, cap of the setup grid
};

// Resident CTAs per SM of a kernel (queried once per process; the kernels
// are the same on every device of one architecture).
template <typename K>
int resident_ctas(K kernel, int threads) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, 0) != cudaSuccess || n < 1)
    n = 1;
  return n;
}

// Most fits of class C one block can have: four rotations per shape slot
// for the rotation modes, one fit per subset otherwise; one-subset modes
// repeat for both shape slots.
constexpr int class_block_fits(int c) {
  return mode_attr(class_mode(c)).has_rotation ? 8
         : mode_attr(class_mode(c)).subsets == 1 ? 2
                                                  : mode_attr(class_mode(c)).subsets;
}

template <int C>
void launch_setup(const ChunkArgs &a, cudaStream_t s) {
  // one thread per fit (per block for mode 6; latency-bound; threads past
  // the class's fits return at once)
  const uint64_t fits = (uint64_t)a.nb * (class_mode(C) == 6 ? 1 : class_block_fits(C));
  const uint64_t setup_ctas_max = (uint64_t)a.sm_count * (uint64_t)a.setup_ctas;
  uint64_t setup_ctas = (fits + kSetupThreads - 1) / kSetupThreads;
  if (setup_ctas > setup_ctas_max) setup_ctas = setup_ctas_max;
  setup_kernel<C><<<(unsigned)setup_ctas, kSetupThreads, 0, s>>>(a.jobs, a.nb, a.sel, a.desc, a.local,
                                                           a.chunk, a.counts, a.ctr, a.state,
                                                           a.arec, a.status);
}

template <int C>
void launch_anneal(const ChunkArgs &a, cudaStream_t s) {
  // the annealing kernel is persistent: no more CTAs than can be resident
  static const int anneal_res = resident_ctas(anneal_kernel<C, 0>, kAnnealThreads);
  // below the resident limit, so that setup and select CTAs of other
  // chunks and classes share the SMs
  const int anneal_per_sm = anneal_res < a.anneal_ctas ? anneal_res : a.anneal_ctas;
  const uint64_t fits = (uint64_t)a.nb * class_block_fits(C);
  const uint64_t order_ctas_max = (uint64_t)a.sm_count * 16;
  uint64_t order_ctas = (fits + 127) / 128;
  if (order_ctas > order_ctas_max) order_ctas = order_ctas_max;
  order_kernel<C><<<(unsigned)order_ctas, 128, 0, s>>>(a.nb, a.local, a.chunk, a.ctr, a.keys, a.perm);
  anneal_kernel<C, 0><<<a.sm_count * anneal_per_sm, kAnnealThreads, 0, s>>>(
      a.nb, a.local, a.chunk, a.ctr, a.arec, a.perm, a.cont, a.cont_cap, a.yield_lanes, a.state);
  if (mode_attr(class_mode(C)).has_rotation) {
    anneal_kernel<C, 1><<<a.sm_count * anneal_per_sm, kAnnealThreads, 0, s>>>(
        a.nb, a.local, a.chunk, a.ctr, a.arec, a.perm, a.cont, a.cont_cap, a.yield_lanes, a.state);
    anneal_kernel<C, 2><<<a.sm_count * anneal_per_sm, kAnnealThreads, 0, s>>>(
        a.nb, a.local, a.chunk, a.ctr, a.arec, a.perm, a.cont, a.cont_cap, a.yield_lanes, a.state);
  }
}

void launch_class_any(int c, bool anneal, const ChunkArgs &a, cudaStream_t s) {
  switch (c) {
#define FASTC_CLASS_CASE(k) \
    case k: anneal ? launch_anneal<k>(a, s) : launch_setup<k>(a, s); break;
    FASTC_CLASS_CASE(0)
    FASTC_CLASS_CASE(1)
    FASTC_CLASS_CASE(2)
    FASTC_CLASS_CASE(3)
    FASTC_CLASS_CASE(4)
    FASTC_CLASS_CASE(5)
    FASTC_CLASS_CASE(6)
    FASTC_CLASS_CASE(7)
    default: anneal ? launch_anneal<8>(a, s) : launch_setup<8>(a, s); break;
#undef FASTC_CLASS_CASE
  }
}

void launch_bound(const ChunkArgs &a, cudaStream_t s) {
  bound_kernel<<<(a.nb + 127) / 128, 128, 0, s>>>(a.nb, a.sel, a.local, a.chunk, a.state, a.ctr,
                                                  a.keys);
}

// Classes in the order their work is enqueued: the longest first, so that
// the short ones fill the tail.
constexpr int kClassOrder[kClasses] = {6, 7, 5, 4, 3, 1, 8, 2, 0};

template <int C>
void reindex_class(const JobDev *jobs, const ChunkBuf &b, int sm_count, cudaStream_t st) {
  reindex_kernel<C><<<sm_count * 4, kPackThreads, 0, st>>>(jobs, b.sel, b.ctr, b.rlist, b.rcap,
                                                           b.state);
}

void reindex_all(const JobDev *jobs, const ChunkBuf &b, int sm_count, cudaStream_t st) {
  reindex_class<0>(jobs, b, sm_count, st);
  reindex_class<1>(jobs, b, sm_count, st);
  reindex_class<2>(jobs, b, sm_count, st);
  reindex_class<3>(jobs, b, sm_count, st);
  reindex_class<4>(jobs, b, sm_count, st);
  reindex_class<5>(jobs, b, sm_count, st);
  reindex_class<6>(jobs, b, sm_count, st);
  reindex_class<7>(jobs, b, sm_count, st);
  reindex_class<8>(jobs, b, sm_count, st);
}

}  // namespace

// Stage order on the caller's stream `st` for chunks 0, 1, 2, ...:
//   select(0) fork(0) | select(1) fork(1) join(0) pack(0) | select(2) ...
// fork(i) starts chunk i's classes on the side streams, join(i) waits for
// them; chunk i uses buffer i % 2, which select(i) may only overwrite after
// pack(i - 2), earlier on `st`.
int launch_pipeline(const JobDev *jobs, int njobs, uint64_t total, const EncodeScratch &rank,
                    void *scratch, int sm_count, int task_bound, const ClassStreams *cls,
                    const PipelineTuning &tune, void *stream, fastc_bc7_block_stats *stats,
                    const ChunkEvents *events) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (total == 0) return 0;
  const int tmax = stats ? kMaxStatsBlockTasks : kMaxBlockTasks;
  const int tb = task_bound < 1 ? 1 : (task_bound > tmax ? tmax : task_bound);
  int e = 0;
  const uint64_t cap = pipeline_chunk_blocks(tb, tune);
  const uint64_t nbmax = total < cap ? total : cap;
  ChunkBuf bufs[2];
  bufs[0] = carve_chunk(static_cast<uint8_t *>(scratch), nbmax, tb, sm_count);
  bufs[1] = total > cap ? carve_chunk(static_cast<uint8_t *>(scratch) +
                                          chunk_buffer_bytes(nbmax, tb, sm_count),
                                      nbmax, tb, sm_count)
                        : bufs[0];
  auto pack = [&](const ChunkBuf &b, uint32_t nb, int parity, int chunk) -> int {
    if (cls) {
      for (int c = 0; c < kClasses; c++) {
        const cudaError_t ce = cudaStreamWaitEvent(st, cls->join[parity][c], 0);
        if (ce != cudaSuccess) return (int)ce;
      }
    }
    const unsigned ctas = (nb + kPackThreads - 1) / kPackThreads;
    choose_kernel<<<ctas, kPackThreads, 0, st>>>(nb, b.sel, b.local, b.chunk, b.state, b.ctr, b.win,
                                                 b.rlist, b.rcap);
    reindex_all(jobs, b, sm_count, st);
    pack_kernel<<<ctas, kPackThreads, 0, st>>>(jobs, nb, b.sel, b.win, b.state);
    if (events && events->packed && chunk < events->count) {
      const cudaError_t ce = cudaEventRecord(events->packed[chunk], st);
      if (ce != cudaSuccess) return (int)ce;
    }
    return (int)cudaPeekAtLastError();
  };
  // One launch of a single large chunk runs its classes' setup kernels one
  // after another: setups of different classes running at once compete for
  // the SMs' instruction cache (their code is large). With several chunks,
  // or a small one, the concurrent setups fill each other's tails instead.
  const bool serial_setup =
      tune.serial_setup > 0 || (tune.serial_setup < 0 && total <= cap && total >= kSerialSetupBlocks);
  uint32_t prev_nb = 0;
  int i = 0;
  for (uint64_t c0 = 0; c0 < total; c0 += cap, i++) {
    const ChunkBuf &b = bufs[i & 1];
    const uint32_t nb = (uint32_t)(total - c0 < cap ? total - c0 : cap);
    const uint64_t n8 = (uint64_t)kClasses * nb;
    const uint32_t nchunks = (uint32_t)((n8 + kRankChunk - 1) / kRankChunk);
    const uint64_t sel_max = (uint64_t)sm_count * (uint64_t)(tune.select_ctas_per_sm > 0 ? tune.select_ctas_per_sm : 16);
    const int sel_ctas = (int)((nb + 3) / 4 < sel_max ? (nb + 3) / 4 : sel_max);
    // the chunk's texels, then its single-colour ranks (continuing the
    // earlier chunks'), before anything reads them
    if (events && events->in_ready && i < events->count) {
      const cudaError_t ce = cudaStreamWaitEvent(st, events->in_ready[i], 0);
      if (ce != cudaSuccess) return (int)ce;
    }
    e = launch_rank_prepass_range(jobs, njobs, total, c0, c0 + nb, rank, stream);
    if (e) return e;
    if (stats)
      select_kernel<4, true><<<sel_ctas, 128, 0, st>>>(jobs, njobs, c0, nb, rank.rank_local,
                                                       rank.chunk_prefix, b.sel, b.counts, tb,
                                                       rank.status, stats);
    else
      select_kernel<4, false><<<sel_ctas, 128, 0, st>>>(jobs, njobs, c0, nb, rank.rank_local,
                                                        rank.chunk_prefix, b.sel, b.counts, tb,
                                                        rank.status, nullptr);
    scan_local_u8_kernel<<<nchunks, kRankChunk, 0, st>>>(b.counts, n8, b.local, b.chunk);
    scan_chunks_kernel<<<1, 1024, 0, st>>>(b.chunk, nchunks, b.ctr);
    emit_kernel<<<(nb + 255) / 256, 256, 0, st>>>(nb, b.counts, b.local, b.chunk, b.desc);
    const ChunkArgs args{jobs,   nb,     b.sel,  b.desc,     b.local, b.chunk, b.counts, b.ctr, b.state,
                         b.arec, b.cont, b.cont_cap, b.keys, b.perm, rank.status, sm_count,
                         tune.anneal_ctas_per_sm < 1 ? 1 : tune.anneal_ctas_per_sm, tune.yield_lanes,
                         tune.setup_ctas_per_sm < 1 ? 128 : tune.setup_ctas_per_sm};
    if (cls) {
      const int par = i & 1;
      cudaError_t ce = cudaEventRecord(cls->fork[par], st);
      const cudaStream_t *side = cls->side[par];
      for (int c = 0; c < kClasses && ce == cudaSuccess; c++)
        ce = cudaStreamWaitEvent(side[c], cls->fork[par], 0);
      if (ce != cudaSuccess) return (int)ce;
      // the bound stage runs on the first class's stream once every
      // class's setup is done (there, or on their own streams); every
      // class's annealing waits for it
      const int lead = kClassOrder[0];
      for (int k = 0; k < kClasses; k++)
        launch_class_any(kClassOrder[k], false, args, side[serial_setup ? lead : kClassOrder[k]]);
      for (int c = 0; c < kClasses && ce == cudaSuccess && !serial_setup; c++) {
        if (c == lead) continue;
        ce = cudaEventRecord(cls->setup[par][c], side[c]);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(side[lead], cls->setup[par][c], 0);
      }
      if (ce != cudaSuccess) return (int)ce;
      launch_bound(args, side[lead]);
      ce = cudaEventRecord(cls->bound[par], side[lead]);
      for (int c = 0; c < kClasses && ce == cudaSuccess; c++)
        if (c != lead) ce = cudaStreamWaitEvent(side[c], cls->bound[par], 0);
      if (ce != cudaSuccess) return (int)ce;
      for (int k = 0; k < kClasses; k++) launch_class_any(kClassOrder[k], true, args, side[kClassOrder[k]]);
      for (int c = 0; c < kClasses && ce == cudaSuccess; c++)
        ce = cudaEventRecord(cls->join[par][c], side[c]);
      if (ce != cudaSuccess) return (int)ce;
      if (i > 0) {
        e = pack(bufs[(i - 1) & 1], prev_nb, (i - 1) & 1, i - 1);
        if (e) return e;
      }
    } else {
      for (int k = 0; k < kClasses; k++) launch_class_any(kClassOrder[k], false, args, st);
      launch_bound(args, st);
      for (int k = 0; k < kClasses; k++) launch_class_any(kClassOrder[k], true, args, st);
      e = pack(b, nb, 0, i);
      if (e) return e;
    }
    e = (int)cudaPeekAtLastError();
    if (e) return e;
    prev_nb = nb;
  }
  if (cls) return pack(bufs[(i - 1) & 1], prev_nb, (i - 1) & 1, i - 1);
  return 0;
}

}  // namespace fastc
