// BC7 (BPTC) encoder device functions.
//
// Each function restates one step of FasTC's per-block search and keeps its
// floating-point operand order exactly; the translation unit is compiled
// with -fmad=false and IEEE division/sqrt, so every float operation rounds
// like FasTC's x86-64 build (SSE2, no FMA). File:line citations are into
// the FasTC project: Compressor.cpp (CP) and RGBAEndpoints.{h,cpp} (RE)
// under BPTCEncoder/src, MatrixSquare.h / VectorBase.h under
// Base/include/FasTC.
//
// Differences from FasTC, all deliberate:
//   * Randomness: every cluster fit owns an LCG stream seeded from
//     (seed, block x, block y, fit id) instead of one process-global stream,
//     so a block's result does not depend on scheduling or batching. The
//     generator and how draws are consumed are FasTC's (CP:358-362,
//     426-536), including glibc's 16-bit fastrand().
//   * The annealing acceptance test evaluates exp in float (Cephes expf,
//     restated below) instead of double.
//   * k-means loops that FasTC runs until a fixed point are bounded at
//     kMaxKMeansIters iterations; hitting the bound sets a status bit.
#pragma once

#include <cfloat>
#include <cstdint>

#include "bc7_format.cuh"
#include "bc7_intqe.cuh"

namespace fastc {

constexpr int kMaxKMeansIters = 256;
constexpr uint32_t kStatusKMeansCap = 1u;

// --------------------------------------------------------------------------
// Small helpers
// --------------------------------------------------------------------------

__device__ __forceinline__ float dot4(const float *a, const float *b) {
  float s = 0.0f;
#pragma unroll
  for (int i = 0; i < 4; i++) s = __fadd_rn(s, __fmul_rn(a[i], b[i]));
  return s;
}

// dot4(a, a) without its leading 0 + a0 * a0: a square is never -0, so
// adding it to +0 gives it back exactly and the sum is the same float.
__device__ __forceinline__ float sqlen4(const float *a) {
  float s = __fmul_rn(a[0], a[0]);
#pragma unroll
  for (int i = 1; i < 4; i++) s = __fadd_rn(s, __fmul_rn(a[i], a[i]));
  return s;
}

__device__ __forceinline__ float length4(const float *a) {
  return __fsqrt_rn(sqlen4(a));
}

__device__ __forceinline__ void normalize4(float *a) {
  const float len = length4(a);
#pragma unroll
  for (int i = 0; i < 4; i++) a[i] = __fdiv_rn(a[i], len);
}

__device__ __forceinline__ bool eq4(const float *a, const float *b) {
  return a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3];
}

// std::min / std::max argument semantics (NaN handling included)
__device__ __forceinline__ float min_std(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float max_std(float a, float b) { return (a < b) ? b : a; }

__device__ __forceinline__ uint32_t sad8(uint32_t a, uint32_t b) {
  a &= 0xFF;
  b &= 0xFF;
  return a > b ? a - b : b - a;
}

__device__ __forceinline__ void unpack4(uint32_t px, float *v) {
  v[0] = (float)(px & 0xFF);
  v[1] = (float)((px >> 8) & 0xFF);
  v[2] = (float)((px >> 16) & 0xFF);
  v[3] = (float)(px >> 24);
}

// QuantizeChannel (RE:126-165).
__device__ __forceinline__ uint32_t quantize_channel(uint32_t val, uint32_t mask,
                                                     int pbit) {
  if (mask == 0xFF) return val;
  if (mask == 0) return 0xFF;
  uint32_t prec = __popc(mask);
  const uint32_t step = 1u << (8 - prec);
  uint32_t lval = val & mask;
  uint32_t hval = lval + step;
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
  return sad8(val, lval) < sad8(val, hval) ? (lval & 0xFF) : (hval & 0xFF);
}

// uint32(x + 0.5) with x widened to double (RE:169-172): rounding the float
// sum toward -inf and truncating gives the same integer for |x| < 2^23.
__device__ __forceinline__ uint32_t round_half_up(float x) {
  return (uint32_t)__float2int_rz(__fadd_rd(x, 0.5f));
}

// RGBAVector::ToPixel (RE:167-177).
__device__ __forceinline__ uint32_t to_pixel(const float *v, uint32_t mask, int pbit) {
  uint32_t r = 0;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const uint32_t q =
        quantize_channel(round_half_up(v[c]) & 0xFF, (mask >> (8 * c)) & 0xFF, pbit);
    r |= q << (8 * c);
  }
  return r;
}

// --------------------------------------------------------------------------
// Mode context: the state of one FasTC CompressionMode object
// --------------------------------------------------------------------------

struct ModeCtx {
  int mode;
  ModeAttr a;
  int steps;
  int metric;
  int rot;       // m_RotateMode
  int idx_mode;  // m_IndexMode
  uint32_t lcg;  // this fit's annealing stream
  uint32_t *status;
  const uint32_t *sct;  // single_color_table() results, or nullptr to search
  // Palette scratch (stride kLaneStride) for the exact integer
  // QuantizedError of the uniform metric; nullptr: the float restatement.
  uint4 *pal;
};

// kErrorMetrics (CP:205-208)
__device__ __forceinline__ float base_weight(int metric, int c) {
  if (metric == 0 || c == 3) return 1.0f;
  return c == 0 ? __fsqrt_rn(0.3f) : (c == 1 ? __fsqrt_rn(0.56f) : __fsqrt_rn(0.11f));
}

__device__ __forceinline__ int rotation_of(const ModeCtx &m) {
  return m.a.has_rotation ? m.rot : 0;
}

// GetNumberOfBitsPerIndex / GetNumberOfBitsPerAlpha (CompressionMode.h:151-165)
__device__ __forceinline__ int bits_index(const ModeCtx &m, int im) {
  if (im < 0) im = m.idx_mode;
  return im == 0 ? m.a.idx_bits : m.a.alpha_idx_bits;
}
__device__ __forceinline__ int bits_alpha(const ModeCtx &m, int im) {
  if (im < 0) im = m.idx_mode;
  return im == 0 ? m.a.alpha_idx_bits : m.a.idx_bits;
}

// GetErrorMetric with the rotation permutation (CompressionMode.h:196-205)
__device__ __forceinline__ void metric_of(const ModeCtx &m, float *w) {
#pragma unroll
  for (int c = 0; c < 4; c++) w[c] = base_weight(m.metric, c);
  const int r = rotation_of(m);
  if (r >= 1) {
    const float t = w[r - 1];
    w[r - 1] = w[3];
    w[3] = t;
  }
}

// GetQuantizationMask (CompressionMode.h:212-232)
__device__ __forceinline__ uint32_t qmask_of(const ModeAttr &a) {
  const uint32_t cm = (0xFFu << (8 - a.color_bits)) & 0xFFu;
  const uint32_t am = a.alpha_bits ? (0xFFu << (8 - a.alpha_bits)) & 0xFFu : 0u;
  return cm | (cm << 8) | (cm << 16) | (am << 24);
}

__device__ __forceinline__ int num_pbit_combos(const ModeAttr &a) {
  return a.pbit == kPBitShared ? 2 : (a.pbit == kPBitUnique ? 4 : 1);
}

// GetPBitCombo (CompressionMode.h:243-250); returns bit0 = first endpoint's
// p-bit, bit1 = second's.
__device__ __forceinline__ int pbit_combo(const ModeAttr &a, int idx) {
  if (a.pbit == kPBitShared) return idx ? 3 : 0;
  if (a.pbit == kPBitUnique) {
    // kPBits = {0,0},{0,1},{1,0},{1,1}
    const int i = idx & 3;
    return ((i >> 1) & 1) | ((i & 1) << 1);
  }
  return 0;
}
__device__ __forceinline__ int pb_first(int combo) { return combo & 1; }
__device__ __forceinline__ int pb_second(int combo) { return (combo >> 1) & 1; }

// --------------------------------------------------------------------------
// Clusters (RE:104-227). A cluster holds its member texels compacted in
// texel order (FasTC's m_PointMap order): point k is px[k * stride], its
// texel index is nibble k of `tex`.
// --------------------------------------------------------------------------

struct Cluster {
  const uint32_t *px;  // member texels, compacted
  int stride;
  uint64_t tex;        // texel index of each point, 4 bits per point
  int n;
  int rot;    // alpha path: channel (1..3) swapped into alpha, 0 = none
  bool a255;  // alpha path: alpha of every point forced to 255
  float avg[4], mn[4], mx[4];
  uint32_t *aux;  // 16 words of scratch (principal_axis), element k at aux[k * aux_stride]
  int aux_stride;
};

__device__ __forceinline__ uint32_t cl_pixel(const Cluster &c, int k) { return c.px[k * c.stride]; }
__device__ __forceinline__ int cl_texel(const Cluster &c, int k) { return (int)((c.tex >> (4 * k)) & 15); }

__device__ __forceinline__ void cl_point(const Cluster &c, int k, float *p) {
  unpack4(cl_pixel(c, k), p);
  if (c.a255) {
    if (c.rot) p[c.rot - 1] = p[3];
    p[3] = 255.0f;
  }
}

// RGBACluster ctor + SetPartition/Recalculate (RE:108-127, 205-226). The
// members of `subset` among the 16 texels `px` are written to `buf` (stride
// `bstride`) in texel order.
__device__ __forceinline__ void make_cluster(const uint32_t *px, uint32_t part_word,
                                             int subset, uint32_t *buf, int bstride, Cluster &c) {
  c.px = buf;
  c.stride = bstride;
  c.aux = nullptr;
  c.aux_stride = 0;
  c.tex = 0;
  c.n = 0;
  c.rot = 0;
  c.a255 = false;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    c.avg[k] = 0.0f;
    c.mn[k] = FLT_MAX;
    c.mx[k] = -FLT_MAX;
  }
  for (int i = 0; i < 16; i++) {
    if ((int)((part_word >> (2 * i)) & 3) != subset) continue;
    float p[4];
    unpack4(px[i], p);
    buf[c.n * bstride] = px[i];
    c.tex |= (uint64_t)i << (4 * c.n);
    c.n++;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      c.avg[k] = __fadd_rn(c.avg[k], p[k]);
      c.mn[k] = min_std(p[k], c.mn[k]);
      c.mx[k] = max_std(p[k], c.mx[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < 4; k++) c.avg[k] = __fdiv_rn(c.avg[k], (float)c.n);
}

__device__ __forceinline__ bool all_same_point(const Cluster &c) { return eq4(c.mx, c.mn); }

__device__ __forceinline__ void set_nib(uint64_t &v, int t, uint32_t x) {
  v = (v & ~(0xFull << (4 * t))) | ((uint64_t)(x & 0xF) << (4 * t));
}
__device__ __forceinline__ uint32_t get_nib(uint64_t v, int t) {
  return (uint32_t)(v >> (4 * t)) & 0xF;
}

// RGBACluster::QuantizedError<nBuckets> (RE:190-310). pb = -1 means the
// caller passed no p-bits; otherwise bit0/bit1 are the endpoints' p-bits.
__device__ inline float quantized_error(const Cluster &c, const float *p1, const float *p2,
                                 int bits, uint32_t qmask, const float *w, int pb,
                                 uint64_t *idx) {
  const int nb = 1 << bits;
  const uint32_t q1 = to_pixel(p1, qmask, pb < 0 ? -1 : pb_first(pb));
  const uint32_t q2 = to_pixel(p2, qmask, pb < 0 ? -1 : pb_second(pb));
  float u1[4], u2[4], d[4], dir[4];
  unpack4(q1, u1);
  unpack4(q2, u2);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    d[k] = __fsub_rn(u1[k], u2[k]);
    dir[k] = __fsub_rn(u2[k], u1[k]);
  }
  const float lsq = sqlen4(d);
  float total = 0.0f;
  if (lsq == 0.0f) {
    for (int i = 0; i < c.n; i++) {
      const uint32_t e = cl_pixel(c, i);
      float ev[4];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const uint32_t ip = (q1 >> (8 * k)) & 0xFF;
        ev[k] = __fmul_rn((float)sad8(e >> (8 * k), ip), w[k]);
      }
      total = __fadd_rn(total, sqlen4(ev));
      if (idx) set_nib(*idx, cl_texel(c, i), 0);
    }
    return total;
  }
  for (int i = 0; i < c.n; i++) {
    const uint32_t epx = cl_pixel(c, i);
    float pt[4], t[4];
    cl_point(c, i, pt);
#pragma unroll
    for (int k = 0; k < 4; k++) t[k] = __fsub_rn(pt[k], u1[k]);
    const float pct = __fdiv_rn(dot4(t, dir), lsq);
    const float scaled = __fmul_rn(pct, (float)(nb - 1));
    int j1 = __float2int_rz(floorf(scaled));
    int j2 = __float2int_rz(ceilf(scaled));
    j1 = min(max(0, j1), nb - 1);
    j2 = min(j2, nb - 1);
    float min_err = FLT_MAX;
    uint32_t best = 0;
    int j = j1;
    do {
      const uint32_t w1 = weight1(bits, (uint32_t)j), w0 = 64u - w1;
      float ev[4];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const uint32_t a = (q1 >> (8 * k)) & 0xFF, b = (q2 >> (8 * k)) & 0xFF;
        const uint32_t ip = ((a * w0 + b * w1 + 32u) >> 6) & 0xFF;
        ev[k] = __fmul_rn((float)sad8(epx >> (8 * k), ip), w[k]);
      }
      const float err = sqlen4(ev);
      if (err < min_err) {
        min_err = err;
        best = (uint32_t)j;
      } else if (err > min_err) {
        break;
      }
    } while (++j <= j2);
    total = __fadd_rn(total, min_err);
    if (idx) set_nib(*idx, cl_texel(c, i), best);
  }
  return total;
}

// --------------------------------------------------------------------------
// Principal axis (RE:327-428) and power iteration (MatrixSquare.h:44-105)
// --------------------------------------------------------------------------

__device__ inline void power_method(const float m[4][4], float *out) {
  float b[4] = {0.5f, 0.5f, 0.5f, 0.5f};
  bool bad = false, fixed = false;
  int iters = 0;
  while (!fixed && ++iters < 5) {
    float nb[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      float s = 0.0f;
#pragma unroll
      for (int i = 0; i < 4; i++) s = __fadd_rn(s, __fmul_rn(m[j][i], b[i]));
      nb[j] = s;
    }
    const float len = length4(nb);
    // (double)len < 1e-10: 1e-10f is the least float above 1e-10, so for a
    // float the test is the same in single precision
    if (len < 1e-10f) {
      if (bad) break;
      b[0] = b[1] = 1.0f;
      normalize4(b);
      bad = true;
      continue;
    }
    normalize4(nb);
    // fabs((double)x) < 1e-8 for a float x: 1e-8f is the greatest float
    // below 1e-8, so the test is |x| <= 1e-8f
    if (fabsf(__fsub_rn(1.0f, dot4(b, nb))) <= 1e-8f) fixed = true;
#pragma unroll
    for (int k = 0; k < 4; k++) b[k] = nb[k];
  }
#pragma unroll
  for (int k = 0; k < 4; k++) out[k] = b[k];
}

__device__ __forceinline__ uint32_t cl_packed(const Cluster &c, int k);

// The unique points are kept packed (they are bytes) in the cluster's
// scratch words instead of a float array, and found only as far as the
// tests below read them: the collinearity test usually stops at the third
// unique point, so the whole list is rarely needed. The list, where read,
// is FasTC's (points in cluster order, first occurrences).
__device__ inline void principal_axis(const Cluster &c, float *axis) {
  uint32_t *up = c.aux;
  const int us = c.aux_stride;
  int nu = 0, scan = 0;  // unique points found, next point to look at
  auto find_unique = [&](int want) {
    while (nu < want && scan < c.n) {
      const uint32_t q = cl_packed(c, scan++);
      bool has = false;
      for (int j = 0; j < nu; j++) has = has || up[j * us] == q;
      if (!has) {
        up[nu * us] = q;
        nu++;
      }
    }
  };
  find_unique(2);
  if (nu == 1) {
    axis[0] = axis[1] = axis[2] = axis[3] = 0.0f;
    return;
  }
  float u0[4], u1[4], dir[4];
  unpack4(up[0], u0);
  unpack4(up[us], u1);
#pragma unroll
  for (int k = 0; k < 4; k++) dir[k] = __fsub_rn(u1[k], u0[k]);
  normalize4(dir);
  bool collinear = true;
  for (int i = 2; i < c.n; i++) {  // bounded by the point count; slots past the
                                   // unique count read (-1,-1,-1,-1)
    find_unique(i + 1);
    float ui[4] = {-1.0f, -1.0f, -1.0f, -1.0f};
    if (i < nu) unpack4(up[i * us], ui);
    float v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = __fsub_rn(ui[k], u0[k]);
    // fabs(fabs((double)a) - (double)b) > 1e-7 in single precision: b is 0
    // (then a is 0 too) or the root of an integer >= 1; where |a - b| is
    // below b / 2 the float difference is exact (Sterbenz), elsewhere it is
    // at least 0.5 either way. 1e-7f is the least float above 1e-7.
    if (fabsf(__fsub_rn(fabsf(dot4(v, dir)), length4(v))) >= 1e-7f) {
      collinear = false;
      break;
    }
  }
  if (collinear) {
#pragma unroll
    for (int k = 0; k < 4; k++) axis[k] = dir[k];
    return;
  }
  // The ten sums of the covariance in one pass over the points; each sum
  // adds the same products in the same order as one pass per entry.
  float cs[10];
#pragma unroll
  for (int m = 0; m < 10; m++) cs[m] = 0.0f;
  for (int t = 0; t < c.n; t++) {
    float p[4], d[4];
    cl_point(c, t, p);
#pragma unroll
    for (int k = 0; k < 4; k++) d[k] = __fsub_rn(p[k], c.avg[k]);
    int m = 0;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j <= i; j++, m++) cs[m] = __fadd_rn(cs[m], __fmul_rn(d[i], d[j]));
  }
  float cov[4][4];
  int m = 0;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j <= i; j++, m++) {
      cov[i][j] = __fdiv_rn(cs[m], 3.0f);
      cov[j][i] = cov[i][j];
    }
  power_method(cov, axis);
}

// --------------------------------------------------------------------------
// Random numbers and the annealing acceptance test
// --------------------------------------------------------------------------

// fastrand (CP:358-362) with glibc's RAND_MAX: the top 16 bits of the state.
__device__ __forceinline__ uint32_t lcg_next(uint32_t &s) {
  s = 214013u * s + 2531011u;
  return s >> 16;
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {  // splitmix64 finaliser
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Per-fit stream seed: a pure function of (seed, block x, block y, fit id).
__device__ __forceinline__ uint32_t fit_seed(uint32_t seed, uint32_t bx, uint32_t by,
                                             uint32_t fit) {
  uint64_t k = mix64(((uint64_t)bx << 32) | by);
  k = mix64(k + (uint64_t)seed * 0x9E3779B97F4A7C15ull + fit);
  return (uint32_t)(k >> 32);
}

// exp(x) for x <= 0 after Cephes expf (S. L. Moshier): Cody-Waite reduction
// by ln 2 split in two, a degree-5 polynomial, exact scaling by 2^n. Only
// rounded +, *, floor and bit construction, so host and device agree.
__device__ __forceinline__ float portable_expf(float x) {
  if (x != x) return x;
  if (x > 0.0f) x = 0.0f;
  if (x < -103.0f) return 0.0f;
  const float fn = floorf(__fadd_rn(__fmul_rn(x, 1.44269504088896341f), 0.5f));
  float r = __fsub_rn(x, __fmul_rn(fn, 0.693359375f));
  r = __fsub_rn(r, __fmul_rn(fn, -2.12194440e-4f));
  const float z = __fmul_rn(r, r);
  float p = 1.9875691500e-4f;
  p = __fadd_rn(__fmul_rn(p, r), 1.3981999507e-3f);
  p = __fadd_rn(__fmul_rn(p, r), 8.3334519073e-3f);
  p = __fadd_rn(__fmul_rn(p, r), 4.1665795894e-2f);
  p = __fadd_rn(__fmul_rn(p, r), 1.6666665459e-1f);
  p = __fadd_rn(__fmul_rn(p, r), 5.0000001201e-1f);
  p = __fadd_rn(__fadd_rn(__fmul_rn(p, z), r), 1.0f);
  int n = __float2int_rz(fn);
  if (n < -125) {
    p = __fmul_rn(p, __int_as_float((127 - 64) << 23));
    n += 64;
  }
  return __fmul_rn(p, __int_as_float((n + 127) << 23));
}

// AcceptNewEndpointError (CP:524-536): accept better errors outright, else
// draw r = frand() (CP:506-519) and accept when r < exp(0.1 (old-new)/temp).
__device__ __forceinline__ bool accept_error(ModeCtx &m, float new_err, float old_err,
                                             float temp) {
  if (new_err < old_err) return true;
  const uint32_t r16 = lcg_next(m.lcg) & 0xFFFF;
  const uint32_t mant = (r16 << 8) | (r16 >> 7);
  const float r = __fsub_rn(__uint_as_float((127u << 23) | mant), 1.0f);
  if (r >= 1.0f) return false;  // bit 15 of the draw reached the exponent
  const float x = __fdiv_rn(__fmul_rn(0.1f, __fsub_rn(old_err, new_err)), temp);
  if (mant == 0) return x > -745.0f;  // r == 0 accepts any p > 0
  return r < portable_expf(x);
}

// --------------------------------------------------------------------------
// Endpoint fitting
// --------------------------------------------------------------------------

__device__ __forceinline__ void clamp_endpoints(float *p1, float *p2) {  // RE:436-441
#pragma unroll
  for (int k = 0; k < 4; k++) {
    p1[k] = p1[k] < 0.0f ? 0.0f : (p1[k] > 255.0f ? 255.0f : p1[k]);
    p2[k] = p2[k] < 0.0f ? 0.0f : (p2[k] > 255.0f ? 255.0f : p2[k]);
  }
}

// ClampEndpointsToGrid (CP:212-250)
__device__ inline void clamp_to_grid(const ModeCtx &m, float *p1, float *p2, uint32_t &best_pbit) {
  const int nc = num_pbit_combos(m.a);
  const uint32_t qm = qmask_of(m.a);
  clamp_endpoints(p1, p2);
  float min_dist = FLT_MAX;
  float b1[4] = {-1.0f, -1.0f, -1.0f, -1.0f}, b2[4] = {-1.0f, -1.0f, -1.0f, -1.0f};
  for (int i = 0; i < nc; i++) {
    const int pc = pbit_combo(m.a, i);
    const uint32_t q1 = to_pixel(p1, qm, nc > 1 ? pb_first(pc) : -1);
    const uint32_t q2 = to_pixel(p2, qm, nc > 1 ? pb_second(pc) : -1);
    float n1[4], n2[4], d1[4], d2[4];
    unpack4(q1, n1);
    unpack4(q2, n2);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      d1[k] = __fsub_rn(n1[k], p1[k]);
      d2[k] = __fsub_rn(n2[k], p2[k]);
    }
    const float dist = __fadd_rn(dot4(d1, d1), dot4(d2, d2));
    if (dist < min_dist) {
      min_dist = dist;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        b1[k] = n1[k];
        b2[k] = n2[k];
      }
      best_pbit = (uint32_t)i;
    }
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    p1[k] = b1[k];
    p2[k] = b2[k];
  }
}

// The per-channel search of CompressSingleColor (CP:262-336): the first
// (i, j) pair, in row-major order, whose interpolant at index 1 lands
// closest to `val`, with FasTC's early exit on an exact hit. The result
// depends only on (val, channel bits, p-bits of the two endpoints, index
// bits): byte 0 = low endpoint, byte 1 = high endpoint, bits 16+ = distance.
__host__ __device__ inline uint32_t single_channel_search(uint32_t val, int nbits, int havepbit,
                                                          int pl, int ph, int ib) {
  const int nposs = 1 << nbits;
  const int eb = havepbit ? nbits + 1 : nbits;
  const uint32_t w1 = weight1(ib, 1), w0 = 64u - w1;
  uint32_t bestd = 0xFF, bi = 0xFFFFFFFFu, bj = 0xFFFFFFFFu;
  for (int i = 0; bestd > 0 && i < nposs; i++) {
    int vl = i;
    if (havepbit) vl = (vl << 1) | pl;
    uint32_t v1 = (uint32_t)(vl << (8 - eb));
    v1 |= v1 >> eb;
    for (int j = 0; bestd > 0 && j < nposs; j++) {
      int vh = j;
      if (havepbit) vh = (vh << 1) | ph;
      uint32_t v2 = (uint32_t)(vh << (8 - eb));
      v2 |= v2 >> eb;
      const uint32_t cmb = (w0 * v1 + w1 * v2 + 32u) >> 6;
      const uint32_t d = cmb > val ? cmb - val : val - cmb;
      if (d < bestd) {
        bestd = d;
        bi = v1;
        bj = v2;
      }
    }
  }
  return (bi & 0xFF) | ((bj & 0xFF) << 8) | (bestd << 16);
}

// Index of a single-colour table row: channel bits 1..8, p-bit variant
// (0: none, 1 + pl + 2 ph), index bits 2..4.
__host__ __device__ constexpr int sct_row(int nbits, int pvar, int ib) {
  return ((nbits - 1) * 5 + pvar) * 3 + (ib - 2);
}
constexpr int kSctRows = 8 * 5 * 3;

// CompressSingleColor (CP:252-353)
__device__ inline float single_color(const ModeCtx &m, const float *p, float *p1, float *p2,
                                     uint32_t &best_pbit) {
  const uint32_t pixel = to_pixel(p, 0xFFFFFFFFu, -1);
  float best_err = FLT_MAX;
  const int nc = num_pbit_combos(m.a);
  const bool havepbit = m.a.pbit != kPBitNone;
  const int ib = bits_index(m, -1);
  for (int pbi = 0; pbi < nc; pbi++) {
    const int combo = pbit_combo(m.a, pbi);
    uint32_t dist[4] = {0, 0, 0, 0};
    uint32_t bi[4], bj[4];
    for (int ci = 0; ci < 4; ci++) {
      const uint32_t val = (pixel >> (ci * 8)) & 0xFF;
      const int nbits = ci == 3 ? m.a.alpha_bits : m.a.color_bits;
      if (nbits == 0) {
        bi[ci] = bj[ci] = 0xFF;
        dist[ci] = max(dist[ci], 0xFFu - val);
        continue;
      }
      const int pl = pb_first(combo), ph = pb_second(combo);
      const uint32_t r = m.sct ? m.sct[sct_row(nbits, havepbit ? 1 + pl + 2 * ph : 0, ib) * 256 + val]
                               : single_channel_search(val, nbits, havepbit, pl, ph, ib);
      bi[ci] = r & 0xFF;
      bj[ci] = (r >> 8) & 0xFF;
      dist[ci] = max(r >> 16, dist[ci]);
    }
    float err = 0.0f;
    for (int i = 0; i < 4; i++) {
      const float e = __fmul_rn((float)dist[i], base_weight(m.metric, i));
      err = __fadd_rn(err, __fmul_rn(e, e));
    }
    if (err < best_err) {
      best_err = err;
      best_pbit = (uint32_t)pbi;
#pragma unroll
      for (int ci = 0; ci < 4; ci++) {
        p1[ci] = (float)bi[ci];
        p2[ci] = (float)bj[ci];
      }
    }
  }
  return best_err;
}

// PickBestNeighboringEndpoints (CP:426-498); the visited list only ever
// holds the best state found so far.
__device__ inline void pick_neighbor(ModeCtx &m, const float *p1, const float *p2, int cur_pbit,
                              float *np1, float *np2, int &npbit, const float *vis1,
                              const float *vis2, int vis_pbit) {
  float step[4];
  const float cs = (float)(1 << (8 - m.a.color_bits));
  step[0] = step[1] = step[2] = cs;
  step[3] = (float)(1 << (8 - m.a.alpha_bits));
  if (m.mode < 4) step[(rotation_of(m) + 3) % 4] = 0.0f;
  const bool has_pbits = m.a.pbit != kPBitNone;
  if (has_pbits) npbit = m.a.pbit == kPBitShared ? (cur_pbit + 1) % 2 : 3 - cur_pbit;
  const int cur_combo = pbit_combo(m.a, cur_pbit);
  bool visited = true;
  int guard = -1;
  while (visited && ++guard < 16) {
#pragma unroll
    for (int pt = 0; pt < 2; pt++) {
      const float *p = pt ? p1 : p2;
      float *np = pt ? np1 : np2;
      const uint32_t dir = lcg_next(m.lcg) % 16;
      // pt indexes the combo although pt == 0 moves the second endpoint
      const int old = pt ? pb_second(cur_combo) : pb_first(cur_combo);
#pragma unroll
      for (int k = 0; k < 4; k++) {
        float v = p[k];
        const bool down = (dir >> k) & 1;
        if (has_pbits) {
          if (down && old == 0) v = __fsub_rn(v, step[k]);
          else if (!down && old == 1) v = __fadd_rn(v, step[k]);
        } else {
          v = down ? __fsub_rn(v, step[k]) : __fadd_rn(v, step[k]);
        }
        np[k] = min_std(max_std(v, 0.0f), 255.0f);
      }
    }
    visited = eq4(vis1, np1) && eq4(vis2, np2) && vis_pbit == npbit;
  }
}

// OptimizeEndpointsForCluster (CP:538-630), from the point after its first
// QuantizedError and the snap of p1/p2 onto the grid: p1/p2 hold grid
// values, cur_err/best_idx/best_pbit the starting error, indices and p-bits.
__device__ inline float anneal_from(ModeCtx &m, const Cluster &c, float *p1, float *p2,
                             float cur_err, uint64_t &best_idx, uint32_t &best_pbit) {
  const int ib = bits_index(m, -1);
  const uint32_t qm = qmask_of(m.a);
  float w[4];
  metric_of(m, w);
  int cur_pbit = (int)best_pbit;
  float best_err = cur_err;
  float bp1[4], bp2[4], vis1[4], vis2[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    bp1[k] = vis1[k] = p1[k];
    bp2[k] = vis2[k] = p2[k];
  }
  int vis_pbit = cur_pbit;
  const int max_energy = m.steps;
  for (int energy = 0; best_err > 0.0f && energy < max_energy; energy++) {
    const float temp = __fdiv_rn((float)energy, (float)(max_energy - 1));
    float np1[4], np2[4];
    int npbit = 0;
    pick_neighbor(m, p1, p2, cur_pbit, np1, np2, npbit, vis1, vis2, vis_pbit);
    uint64_t idx = 0;
    const float err = quantized_error(c, np1, np2, ib, qm, w, pbit_combo(m.a, npbit), &idx);
    if (accept_error(m, err, cur_err, temp)) {
      cur_err = err;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        p1[k] = np1[k];
        p2[k] = np2[k];
      }
      cur_pbit = npbit;
    }
    if (err < best_err) {
      best_idx = idx;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        bp1[k] = vis1[k] = np1[k];
        bp2[k] = vis2[k] = np2[k];
      }
      best_pbit = (uint32_t)npbit;
      vis_pbit = npbit;
      best_err = err;
      energy = 0;
    }
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    p1[k] = bp1[k];
    p2[k] = bp2[k];
  }
  return best_err;
}

// A cluster fit up to the point where FasTC starts annealing.
struct FitSetup {
  double err;       // final error when !anneal (CompressCluster's return value)
  float errf;       // starting error of the annealing
  float p1[4], p2[4];
  uint64_t idx;     // 4 bits per texel
  uint32_t pbit;
  bool anneal;      // the annealing loop has work (steps > 0, error > 0)
};

// Point k of the cluster as packed bytes: cl_point() without the float
// conversion (the rotation swap and forced alpha of the alpha path applied).
__device__ __forceinline__ uint32_t cl_packed(const Cluster &c, int k) {
  const uint32_t px = cl_pixel(c, k);
  if (!c.a255) return px;
  uint32_t sel = 0x4210u;  // bytes 0-2 from the pixel, byte 3 = 0xFF
  if (c.rot) sel = (sel & ~(0xFu << (4 * (c.rot - 1)))) | (3u << (4 * (c.rot - 1)));
  return __byte_perm(px, 0xFFFFFFFFu, sel);
}

// CompressionMode::CompressCluster (CP:921-1094) up to the annealing, for
// kNB = 2^index-bits palette entries: single colour, PCA endpoints, the
// k-means refinement, least squares, grid clamp and the first
// QuantizedError. With kNB a constant the level loops unroll and the k-means
// levels stay in registers; the members' per-level sums are exact integers
// (sums of at most 16 bytes), so they are accumulated as integers, which
// equals FasTC's float sums. kSmemAcc: the per-level sums live in the
// thread's palette scratch (ka_level) instead of registers, one
// read-modify-write per point instead of a predicated add per level.
// Level j's sum in the thread's own palette slots (the 8 uint4 words
// m.pal[k * kLaneStride], two 64-bit halves each), which no other thread
// touches.
__device__ __forceinline__ uint64_t &ka_level(const ModeCtx &m, int j) {
  return reinterpret_cast<uint64_t *>(m.pal + (j >> 1) * kLaneStride)[j & 1];
}

template <int kNB, bool kSmemAcc = false>
__device__ inline void fit_rgb_setup_t(ModeCtx &m, const Cluster &c, FitSetup &st) {
  float *p1 = st.p1, *p2 = st.p2;
  uint64_t &idx = st.idx;
  uint32_t &pbit = st.pbit;
  st.anneal = false;
  st.errf = 0.0f;
  if (all_same_point(c)) {
    float p0[4];
    cl_point(c, 0, p0);
    const double e = single_color(m, p0, p1, p2, pbit);
    for (int i = 0; i < c.n; i++) set_nib(idx, cl_texel(c, i), 1);
    st.err = (double)c.n * e;
    return;
  }
  constexpr int nb = kNB;
  constexpr int kUnroll = kNB;
  float axis[4];
  principal_axis(c, axis);
  float mindp = FLT_MAX, maxdp = -FLT_MAX;
  for (int i = 0; i < c.n; i++) {
    float p[4], t[4];
    cl_point(c, i, p);
#pragma unroll
    for (int k = 0; k < 4; k++) t[k] = __fsub_rn(p[k], c.avg[k]);
    const float dp = dot4(t, axis);
    if (dp < mindp) mindp = dp;
    if (dp > maxdp) maxdp = dp;
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    p1[k] = __fadd_rn(c.avg[k], __fmul_rn(axis[k], mindp));
    p2[k] = __fadd_rn(c.avg[k], __fmul_rn(axis[k], maxdp));
  }
  clamp_endpoints(p1, p2);

  float pts[kNB][4];
  uint32_t npts[kNB];
#pragma unroll kUnroll
  for (int i = 0; i < nb; i++) {
    const float s = __fdiv_rn((float)i, (float)(nb - 1));
#pragma unroll
    for (int k = 0; k < 4; k++)
      pts[i][k] = __fadd_rn(__fmul_rn(p1[k], __fsub_rn(1.0f, s)), __fmul_rn(p2[k], s));
  }
  bool fixed = false;
  int iters = 0;
  while (!fixed) {
    if (++iters > kMaxKMeansIters) {
      atomicOr(m.status, kStatusKMeansCap);
      break;
    }
    // per level: channel sums in 13-bit fields, member count from bit 52
    uint64_t acc[kSmemAcc ? 1 : kNB];
    if constexpr (kSmemAcc) {
#pragma unroll
      for (int j = 0; j < nb; j++) ka_level(m, j) = 0;
    } else {
#pragma unroll kUnroll
      for (int j = 0; j < nb; j++) acc[j] = 0;
    }
    for (int i = 0; i < c.n; i++) {
      float p[4];
      cl_point(c, i, p);
      int minb = 0;
      float mind = FLT_MAX;
#pragma unroll kUnroll
      for (int j = 0; j < nb; j++) {
        float v[4];
#pragma unroll
        for (int k = 0; k < 4; k++) v[k] = __fsub_rn(p[k], pts[j][k]);
        const float d = sqlen4(v);
        if (d < mind) {
          mind = d;
          minb = j;
        }
      }
      const uint32_t q = cl_packed(c, i);
      const uint64_t add = (uint64_t)(q & 0xFF) | ((uint64_t)((q >> 8) & 0xFF) << 13) |
                           ((uint64_t)((q >> 16) & 0xFF) << 26) | ((uint64_t)(q >> 24) << 39) |
                           (1ull << 52);
      if constexpr (kSmemAcc) {
        ka_level(m, minb) += add;
      } else {
#pragma unroll
        for (int j = 0; j < nb; j++) acc[j] += j == minb ? add : 0ull;
      }
    }
    fixed = true;
#pragma unroll kUnroll
    for (int j = 0; j < nb; j++) {
      const uint64_t aj = kSmemAcc ? ka_level(m, j) : acc[j];
      const uint32_t cnt = (uint32_t)(aj >> 52);
      float np[4];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        np[k] = (float)(uint32_t)((aj >> (13 * k)) & 0x1FFFu);
        if (cnt) np[k] = __fdiv_rn(np[k], (float)cnt);
      }
      npts[j] = cnt;
      if (!eq4(pts[j], np)) fixed = false;
#pragma unroll
      for (int k = 0; k < 4; k++) pts[j][k] = np[k];
    }
  }
  int filled = 0, last = -1;
#pragma unroll kUnroll
  for (int j = 0; j < nb; j++)
    if (npts[j] > 0) {
      filled++;
      last = j;
    }
  if (filled == 1) {
    float pl[4];
#pragma unroll kUnroll
    for (int j = 0; j < nb; j++)
      if (j == last)
#pragma unroll
        for (int k = 0; k < 4; k++) pl[k] = pts[j][k];
    const double e = single_color(m, pl, p1, p2, pbit);
    for (int i = 0; i < c.n; i++) set_nib(idx, cl_texel(c, i), 1);
    st.err = (double)c.n * e;
    return;
  }
  float asq = 0.0f, bsq = 0.0f, ab = 0.0f;
  float ax[4] = {0.0f, 0.0f, 0.0f, 0.0f}, bx[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll kUnroll
  for (int j = 0; j < nb; j++) {
    const float fb = (float)(nb - 1);
    const float a = __fdiv_rn((float)(nb - 1 - j), fb), b = __fdiv_rn((float)j, fb);
    const float fn = (float)npts[j];
    asq = __fadd_rn(asq, __fmul_rn(__fmul_rn(fn, a), a));
    bsq = __fadd_rn(bsq, __fmul_rn(__fmul_rn(fn, b), b));
    ab = __fadd_rn(ab, __fmul_rn(__fmul_rn(fn, a), b));
#pragma unroll
    for (int k = 0; k < 4; k++) {
      ax[k] = __fadd_rn(ax[k], __fmul_rn(__fmul_rn(pts[j][k], a), fn));
      bx[k] = __fadd_rn(bx[k], __fmul_rn(__fmul_rn(pts[j][k], b), fn));
    }
  }
  const float f = __fdiv_rn(1.0f, __fsub_rn(__fmul_rn(asq, bsq), __fmul_rn(ab, ab)));
#pragma unroll
  for (int k = 0; k < 4; k++) {
    p1[k] = __fmul_rn(__fsub_rn(__fmul_rn(ax[k], bsq), __fmul_rn(bx[k], ab)), f);
    p2[k] = __fmul_rn(__fsub_rn(__fmul_rn(bx[k], asq), __fmul_rn(ax[k], ab)), f);
  }
  clamp_to_grid(m, p1, p2, pbit);
  const uint32_t qm = qmask_of(m.a);
  const int pc = pbit_combo(m.a, (int)pbit);
  const bool hp = m.a.pbit != kPBitNone;
  const uint32_t q1 = to_pixel(p1, qm, hp ? pb_first(pc) : -1);
  const uint32_t q2 = to_pixel(p2, qm, hp ? pb_second(pc) : -1);
  if (kNB <= 8 && m.pal && m.metric == 0 && c.stride == kLaneStride) {
    // The same QuantizedError in exact integers (bc7_intqe.cuh); the
    // points are the cluster's (rotated) points, the error pixels its
    // texels, as in the float restatement, and the endpoints are quantized
    // the way it quantizes them: with the combination's p-bits even for
    // modes without p-bits (FasTC passes kPBits[0] there).
    constexpr int kBits = kNB == 4 ? 2 : 3;
    const uint32_t e1 = to_pixel(p1, qm, pb_first(pc));
    const uint32_t e2 = to_pixel(p2, qm, pb_second(pc));
    int se = 0;
    for (int i = 0; i < c.n; i++) {
      const uint32_t e = cl_pixel(c, i);
      se += (int)__dp4a(e, e, 0u);
    }
    uint64_t ix = 0;
    if (c.a255) {
      uint32_t e[16];
#pragma unroll
      for (int k = 0; k < 16; k++) e[k] = cl_pixel(c, k);
      uint32_t pr[16];
#pragma unroll
      for (int k = 0; k < 16; k++) pr[k] = cl_packed(c, k);
      st.errf = qe_reg<kBits, true, true>(e, pr, se, m.pal, e1, e2, ix);
    } else {
      st.errf = qe_smem<kBits, true>(c.px, c.n, c.tex, se, m.pal, e1, e2, ix);
    }
    idx = ix;
  } else {
    float w[4];
    metric_of(m, w);
    st.errf = quantized_error(c, p1, p2, bits_index(m, -1), qm, w, pc, &idx);
  }
  unpack4(q1, p1);
  unpack4(q2, p2);
  st.err = (double)st.errf;
  st.anneal = m.steps > 0 && st.errf > 0.0f;
}

__device__ inline void fit_rgb_setup(ModeCtx &m, const Cluster &c, FitSetup &st) {
  switch (bits_index(m, -1)) {
    case 2: fit_rgb_setup_t<4>(m, c, st); break;
    case 3: fit_rgb_setup_t<8>(m, c, st); break;
    default: fit_rgb_setup_t<16>(m, c, st); break;
  }
}

__device__ inline double fit_rgb(ModeCtx &m, const Cluster &c, float *p1, float *p2,
                          uint64_t &idx, uint32_t &pbit) {
  FitSetup st;
  st.idx = idx;
  st.pbit = pbit;
  fit_rgb_setup(m, c, st);
  if (st.anneal) st.err = (double)anneal_from(m, c, st.p1, st.p2, st.errf, st.idx, st.pbit);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    p1[k] = st.p1[k];
    p2[k] = st.p2[k];
  }
  idx = st.idx;
  pbit = st.pbit;
  return st.err;
}

template <int kANB>
__device__ inline void alpha_fit_t(const ModeCtx &m, const Cluster &c, uint32_t ch, float amin,
                                   float amax, const uint32_t *opt6, float &a1_out, float &a2_out,
                                   uint64_t &aidx, double &aerr_out);

// The alpha channel (channel `ch` of the texels) of the block, and its range.
__device__ __forceinline__ float cl_alpha(const Cluster &c, int i, uint32_t ch) {
  return (float)((cl_pixel(c, i) >> (8 * ch)) & 0xFF);
}

__device__ inline void alpha_fit_any(const ModeCtx &m, const Cluster &c, uint32_t ch, float amin,
                                     float amax, const uint32_t *opt6, float &a1, float &a2,
                                     uint64_t &aidx, double &aerr) {
  if (bits_alpha(m, -1) == 2) alpha_fit_t<4>(m, c, ch, amin, amax, opt6, a1, a2, aidx, aerr);
  else alpha_fit_t<8>(m, c, ch, amin, amax, opt6, a1, a2, aidx, aerr);
}

// CompressionMode::CompressCluster, separate-alpha version (CP:632-919).
// `c` is the whole block; the colour fit runs on a rotated copy whose
// statistics and error pixels stay those of the unrotated block.
__device__ inline double fit_alpha(ModeCtx &m, const Cluster &c, const uint32_t *opt6,
                            float *p1, float *p2, uint64_t &idx, uint64_t &aidx) {
  Cluster rgb = c;
  rgb.rot = rotation_of(m);
  rgb.a255 = true;
  const int r = rgb.rot;
  const uint32_t ch = r ? r - 1 : 3;
  float amin = FLT_MAX, amax = -FLT_MAX;
  for (int i = 0; i < 16; i++) {
    const float av = cl_alpha(c, i, ch);
    amin = min_std(av, amin);
    amax = max_std(av, amax);
  }
  uint32_t dummy = 0;
  float rp1[4], rp2[4];
  const double rgb_err = fit_rgb(m, rgb, rp1, rp2, idx, dummy);
  double aerr;
  float a1, a2;
  alpha_fit_any(m, c, ch, amin, amax, opt6, a1, a2, aidx, aerr);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    p1[k] = rp1[k];
    p2[k] = rp2[k];
  }
  p1[3] = a1;
  p2[3] = a2;
  return rgb_err + aerr;
}

// The separate-alpha fit up to the colour fit's annealing: the colour part
// in `st` (rotated cluster, CP:664-701), the alpha part complete. kNB: the
// colour and alpha palette sizes (0: from the mode context).
template <int kNB = 0, int kANB = 0, bool kSmemAcc = false>
__device__ inline void fit_alpha_setup(ModeCtx &m, const Cluster &c, const uint32_t *opt6,
                                FitSetup &st, float &a1, float &a2, uint64_t &aidx,
                                double &aerr) {
  Cluster rgb = c;
  rgb.rot = rotation_of(m);
  rgb.a255 = true;
  const int r = rgb.rot;
  const uint32_t ch = r ? r - 1 : 3;
  float amin = FLT_MAX, amax = -FLT_MAX;
  for (int i = 0; i < 16; i++) {
    const float av = cl_alpha(c, i, ch);
    amin = min_std(av, amin);
    amax = max_std(av, amax);
  }
  st.idx = 0;
  st.pbit = 0;
  if constexpr (kNB > 0) {
    fit_rgb_setup_t<kNB, kSmemAcc>(m, rgb, st);
    alpha_fit_t<kANB>(m, c, ch, amin, amax, opt6, a1, a2, aidx, aerr);
  } else {
    fit_rgb_setup(m, rgb, st);
    alpha_fit_any(m, c, ch, amin, amax, opt6, a1, a2, aidx, aerr);
  }
}

// The alpha half of CompressCluster's separate-alpha version (CP:703-911):
// 1-D k-means on the rotated channel, least squares, quantisation and the
// per-texel bucket search, for kANB = 2^alpha-index-bits levels.
// Independent of the colour fit's annealing. Bucket sums are sums of at
// most 16 bytes, exact in float, so they are accumulated as integers.
template <int kANB>
__device__ inline void alpha_fit_t(const ModeCtx &m, const Cluster &c, uint32_t ch, float amin,
                                   float amax, const uint32_t *opt6, float &a1_out, float &a2_out,
                                   uint64_t &aidx, double &aerr_out) {
  float a1 = amin, a2 = amax;
  double aerr;
  const int abits = bits_alpha(m, -1);
  float w[4];
  metric_of(m, w);
  const float wa = w[3];
  constexpr int nb = kANB;
  if (a1 == a2) {
    const uint32_t abe = (uint32_t)a1;
    if (m.mode == 5) {
      aidx = 0;
      aerr = 0.0;
    } else {
      const uint32_t e = opt6[abe];
      a1 = (float)(e & 0xFF);
      a2 = (float)((e >> 8) & 0xFF);
      const uint32_t ai = m.idx_mode == 1 ? 1u : 2u;
      aidx = 0x1111111111111111ull * ai;
      const uint32_t w1 = weight1(abits, ai), w0 = 64u - w1;
      const uint32_t ip = ((((uint32_t)a1) * w0 + ((uint32_t)a2) * w1 + 32u) >> 6) & 0xFF;
      float pe = __fmul_rn(wa, (float)(abe > ip ? abe - ip : ip - abe));
      pe = __fmul_rn(pe, pe);
      aerr = (double)__fmul_rn(16.0f, pe);
    }
  } else {
    float vals[nb];
#pragma unroll
    for (int j = 0; j < nb; j++) {
      const float fb = (float)(nb - 1);
      vals[j] = __fadd_rn(amin, __fmul_rn(__fdiv_rn((float)j, fb), __fsub_rn(amax, amin)));
    }
    uint64_t bk = 0;  // bucket of texel i in nibble i
    for (int i = 0; i < 16; i++) {
      const float av = cl_alpha(c, i, ch);
      float md = 255.0f;
      uint32_t b = 0;
#pragma unroll
      for (int j = 0; j < nb; j++) {
        const float d = fabsf(__fsub_rn(av, vals[j]));
        if (d < md) {
          md = d;
          b = (uint32_t)j;
        }
      }
      bk |= (uint64_t)b << (4 * i);
    }
    float npts[nb];
    bool fixed = false;
    int iters = 0;
    while (!fixed) {
      if (++iters > kMaxKMeansIters) {
        atomicOr(m.status, kStatusKMeansCap);
        break;
      }
      uint32_t sum[nb], cnt[nb];
#pragma unroll
      for (int j = 0; j < nb; j++) sum[j] = cnt[j] = 0;
      for (int i = 0; i < 16; i++) {
        const uint32_t av = (cl_pixel(c, i) >> (8 * ch)) & 0xFF;
        const uint32_t b = (uint32_t)((bk >> (4 * i)) & 15);
#pragma unroll
        for (int j = 0; j < nb; j++) {
          sum[j] += b == (uint32_t)j ? av : 0u;
          cnt[j] += b == (uint32_t)j ? 1u : 0u;
        }
      }
      float avg[nb];
      fixed = true;
#pragma unroll
      for (int j = 0; j < nb; j++) {
        npts[j] = (float)cnt[j];
        avg[j] = (float)sum[j];
        if (npts[j] > 0.0f) avg[j] = __fdiv_rn(avg[j], npts[j]);
        fixed = fixed && (avg[j] == vals[j]);
        vals[j] = avg[j];
      }
      bk = 0;
      for (int i = 0; i < 16; i++) {
        const float av = cl_alpha(c, i, ch);
        float md = 255.0f;
        uint32_t b = 0;
#pragma unroll
        for (int j = 0; j < nb; j++) {
          const float d = fabsf(__fsub_rn(av, vals[j]));
          if (d < md) {
            md = d;
            b = (uint32_t)j;
          }
        }
        bk |= (uint64_t)b << (4 * i);
      }
    }
    float asq = 0.0f, bsq = 0.0f, ab = 0.0f, ax = 0.0f, bx = 0.0f;
#pragma unroll
    for (int j = 0; j < nb; j++) {
      const float fb = (float)(nb - 1);
      const float a = __fdiv_rn((float)(nb - 1 - j), fb), b = __fdiv_rn((float)j, fb);
      const float n = npts[j], x = vals[j];
      asq = __fadd_rn(asq, __fmul_rn(__fmul_rn(n, a), a));
      bsq = __fadd_rn(bsq, __fmul_rn(__fmul_rn(n, b), b));
      ab = __fadd_rn(ab, __fmul_rn(__fmul_rn(n, a), b));
      ax = __fadd_rn(ax, __fmul_rn(__fmul_rn(x, a), n));
      bx = __fadd_rn(bx, __fmul_rn(__fmul_rn(x, b), n));
    }
    const float f = __fdiv_rn(1.0f, __fsub_rn(__fmul_rn(asq, bsq), __fmul_rn(ab, ab)));
    a1 = __fmul_rn(f, __fsub_rn(__fmul_rn(ax, bsq), __fmul_rn(bx, ab)));
    a2 = __fmul_rn(f, __fsub_rn(__fmul_rn(bx, asq), __fmul_rn(ax, ab)));
    a1 = min_std(255.0f, max_std(0.0f, a1));
    a2 = min_std(255.0f, max_std(0.0f, a2));
    const uint32_t amask = (uint32_t)(((int)(int8_t)-0x7F) >> (m.a.alpha_bits - 1)) & 0xFF;
    const uint32_t a1b = quantize_channel((uint32_t)a1 & 0xFF, amask, -1);
    const uint32_t a2b = quantize_channel((uint32_t)a2 & 0xFF, amask, -1);
    aerr = 0.0;
    if (wa == 1.0f) {
      // Uniform weight: each texel's error is the square of an integer below
      // 256, exact in float, and sixteen of them sum exactly in double, so
      // the integer sum is the same number without double arithmetic.
      uint32_t ie = 0;
      for (int i = 0; i < 16; i++) {
        const uint32_t val = (cl_pixel(c, i) >> (8 * ch)) & 0xFF;
        uint32_t me = 0xFFFFFFFFu, bb = 0;
#pragma unroll
        for (int j = 0; j < nb; j++) {
          const uint32_t w1 = weight1(abits, (uint32_t)j), w0 = 64u - w1;
          const uint32_t ip = ((a1b * w0 + a2b * w1 + 32u) >> 6) & 0xFF;
          const uint32_t d = val > ip ? val - ip : ip - val;
          if (d * d < me) {
            me = d * d;
            bb = (uint32_t)j;
          }
        }
        ie += me;
        set_nib(aidx, i, bb);
      }
      aerr = (double)ie;
    } else {
      for (int i = 0; i < 16; i++) {
        const uint32_t val = (cl_pixel(c, i) >> (8 * ch)) & 0xFF;
        float me = FLT_MAX;
        uint32_t bb = 0;
#pragma unroll
        for (int j = 0; j < nb; j++) {
          const uint32_t w1 = weight1(abits, (uint32_t)j), w0 = 64u - w1;
          const uint32_t ip = ((a1b * w0 + a2b * w1 + 32u) >> 6) & 0xFF;
          float pe = __fmul_rn(wa, (float)(val > ip ? val - ip : ip - val));
          pe = __fmul_rn(pe, pe);
          if (pe < me) {
            me = pe;
            bb = (uint32_t)j;
          }
        }
        aerr = aerr + (double)me;
        set_nib(aidx, i, bb);
      }
    }
  }
  a1_out = a1;
  a2_out = a2;
  aerr_out = aerr;
}

}  // namespace fastc
