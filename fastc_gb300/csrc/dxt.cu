// DXT1 / DXT5 (BC1 / BC3) encoder and decoder for sm_103a, FasTC's second
// compression path (DXTEncoder/src/Compressor.cpp:47-93): every 4x4 block
// of a job through the stb_dxt v1.06 block encoder that FasTC vendors
// (DXTEncoder/src/stb_dxt.h, stb_compress_dxt_block :623), with dithering
// and one refinement pass; DXT5 adds the alpha block. The method, restated
// per step below from its published description (the stb_dxt.h lines each
// step corresponds to are given with it), keeps every integer step and the
// float and double operation order (the file is compiled without
// contraction), so the blocks are FasTC's bit for bit. One thread per
// block: about 3,400 instructions per block, all in registers.
//
// Jobs travel to the device inside kernel parameters (up to 32 per launch),
// so the device entry point allocates nothing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "bc7_host.h"
#include "bc7_kernels.cuh"
#include "dxt.cuh"
#include "fastc_bc7.h"

namespace fastc {
namespace {

__host__ __device__ inline int mul8bit(int a, int b) {
  const int t = a * b + 128;
  return (t + (t >> 8)) >> 8;
}
__host__ __device__ inline int lerp13(int a, int b) { return (2 * a + b) / 3; }
// 565 expansion by bit replication
__host__ __device__ inline int exp5(int q) { return (q << 3) | (q >> 2); }
__host__ __device__ inline int exp6(int q) { return (q << 2) | (q >> 4); }

// Per 8-bit value, the best endpoint pair (high, low) of the single-colour
// encoding (stb_dxt.h :121-147, built at :603-621): the pair whose 1/3
// interpolant reproduces the value, with 3 % of the endpoints' distance as
// a penalty; packed high | low << 8. In global memory (read through the
// read-only cache: lanes index it divergently).
__device__ uint16_t g_dxt_match[2][256];  // [0]: 5-bit channels, [1]: 6-bit

void build_match_tables(uint16_t (*tab)[256]) {
  for (int pass = 0; pass < 2; pass++) {
    const int size = pass ? 64 : 32;
    for (int v = 0; v < 256; v++) {
      int best = 256;
      for (int lo = 0; lo < size; lo++)
        for (int hi = 0; hi < size; hi++) {
          const int eh = pass ? exp6(hi) : exp5(hi), el = pass ? exp6(lo) : exp5(lo);
          const int err = std::abs(lerp13(eh, el) - v) + std::abs(eh - el) * 3 / 100;
          if (err < best) {
            tab[pass][v] = (uint16_t)(hi | (lo << 8));
            best = err;
          }
        }
    }
  }
}

// The dither's 565 quantisers (the tables of stb_dxt.h :603-621): the
// channel value (clamped to 0..255, as the table indexed from -8 to 263 is)
// to its nearest 5- or 6-bit level, expanded back to 8 bits. Arithmetic rather than a table, so
// that divergent lanes do not serialise on a lookup.
__device__ __forceinline__ int quant5(int v) { return exp5(mul8bit(min(max(v, 0), 255), 31)); }
__device__ __forceinline__ int quant6(int v) { return exp6(mul8bit(min(max(v, 0), 255), 63)); }

__device__ __forceinline__ int ch8(uint32_t p, int c) { return (int)((p >> (8 * c)) & 0xFF); }

__device__ __forceinline__ uint16_t as565(int r, int g, int b) {
  return (uint16_t)((mul8bit(r, 31) << 11) + (mul8bit(g, 63) << 5) + mul8bit(b, 31));
}

// The palette of endpoints c0, c1 as packed RGB (4-colour interpolation;
// stb_dxt.h :149-157).
__device__ __forceinline__ void dxt_palette(uint16_t c0, uint16_t c1, int col[4][3]) {
  col[0][0] = exp5((c0 >> 11) & 31);
  col[0][1] = exp6((c0 >> 5) & 63);
  col[0][2] = exp5(c0 & 31);
  col[1][0] = exp5((c1 >> 11) & 31);
  col[1][1] = exp6((c1 >> 5) & 63);
  col[1][2] = exp5(c1 & 31);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    col[2][k] = lerp13(col[0][k], col[1][k]);
    col[3][k] = lerp13(col[1][k], col[0][k]);
  }
}

// Floyd-Steinberg dither of each RGB channel to its 565 grid, row by row
// (stb_dxt.h :159-184).
__device__ __forceinline__ void dxt_dither(const uint32_t (&px)[16], uint32_t (&out)[16]) {
#pragma unroll
  for (int i = 0; i < 16; i++) out[i] = 0;
#pragma unroll
  for (int ch = 0; ch < 3; ch++) {
    auto q = [ch](int v) { return ch == 1 ? quant6(v) : quant5(v); };
    int p0 = 0, p1 = 0, p2 = 0, p3 = 0;  // the row above's errors
#pragma unroll
    for (int y = 0; y < 4; y++) {
      const int s0 = ch8(px[4 * y], ch), s1 = ch8(px[4 * y + 1], ch);
      const int s2 = ch8(px[4 * y + 2], ch), s3 = ch8(px[4 * y + 3], ch);
      const int d0 = q(s0 + ((3 * p1 + 5 * p0) >> 4));
      const int e0 = s0 - d0;
      const int d1 = q(s1 + ((7 * e0 + 3 * p2 + 5 * p1 + p0) >> 4));
      const int e1 = s1 - d1;
      const int d2 = q(s2 + ((7 * e1 + 3 * p3 + 5 * p2 + p1) >> 4));
      const int e2 = s2 - d2;
      const int d3 = q(s3 + ((7 * e2 + 5 * p3 + p2) >> 4));
      const int e3 = s3 - d3;
      out[4 * y] |= (uint32_t)d0 << (8 * ch);
      out[4 * y + 1] |= (uint32_t)d1 << (8 * ch);
      out[4 * y + 2] |= (uint32_t)d2 << (8 * ch);
      out[4 * y + 3] |= (uint32_t)d3 << (8 * ch);
      p0 = e0;
      p1 = e1;
      p2 = e2;
      p3 = e3;
    }
  }
}

// Indices: each texel's projection on the endpoint direction against the
// midpoints of the palette's projections, with the projection error diffused
// Floyd-Steinberg style (stb_dxt.h :186-281, dithered branch).
__device__ __forceinline__ uint32_t dxt_match(const uint32_t (&px)[16], const int (&col)[4][3]) {
  const int dr = col[0][0] - col[1][0], dg = col[0][1] - col[1][1], db = col[0][2] - col[1][2];
  int stops[4];
#pragma unroll
  for (int i = 0; i < 4; i++) stops[i] = col[i][0] * dr + col[i][1] * dg + col[i][2] * db;
  const int c0p = ((stops[1] + stops[3]) >> 1) << 4;
  const int half = ((stops[3] + stops[2]) >> 1) << 4;
  const int c3p = ((stops[2] + stops[0]) >> 1) << 4;
  int p0 = 0, p1 = 0, p2 = 0, p3 = 0;
  uint32_t mask = 0;
#pragma unroll
  for (int y = 0; y < 4; y++) {
    int e[4];
#pragma unroll
    for (int x = 0; x < 4; x++) {
      const uint32_t t = px[4 * y + x];
      const int dot = ch8(t, 0) * dr + ch8(t, 1) * dg + ch8(t, 2) * db;
      const int diff = x == 0 ? 3 * p1 + 5 * p0
                       : x == 1 ? 7 * e[0] + 3 * p2 + 5 * p1 + p0
                       : x == 2 ? 7 * e[1] + 3 * p3 + 5 * p2 + p1
                                : 7 * e[2] + 5 * p3 + p2;
      const int v = (dot << 4) + diff;
      const int step = v < half ? (v < c0p ? 1 : 3) : (v < c3p ? 2 : 0);
      e[x] = dot - stops[step];
      mask |= (uint32_t)step << (8 * y + 2 * x);
    }
    p0 = e[0];
    p1 = e[1];
    p2 = e[2];
    p3 = e[3];
  }
  return mask;
}

// Endpoints from the principal axis of the (dithered) texels: four power
// iterations on the RGB covariance from the bounding box's extent, the
// axis scaled to 512 (or the luma weights when it is short), the texels
// with the least and greatest projection (stb_dxt.h :283-385).
__device__ __forceinline__ void dxt_axis(const uint32_t (&px)[16], uint16_t &max16, uint16_t &min16) {
  int mu[3], mn[3], mx[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    int s = ch8(px[0], c), lo = s, hi = s;
#pragma unroll
    for (int i = 1; i < 16; i++) {
      const int v = ch8(px[i], c);
      s += v;
      if (v < lo) lo = v;
      else if (v > hi) hi = v;
    }
    mu[c] = (s + 8) >> 4;
    mn[c] = lo;
    mx[c] = hi;
  }
  int cov[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < 16; i++) {
    const int r = ch8(px[i], 0) - mu[0], g = ch8(px[i], 1) - mu[1], b = ch8(px[i], 2) - mu[2];
    cov[0] += r * r;
    cov[1] += r * g;
    cov[2] += r * b;
    cov[3] += g * g;
    cov[4] += g * b;
    cov[5] += b * b;
  }
  float cf[6];
#pragma unroll
  for (int i = 0; i < 6; i++) cf[i] = __fdiv_rn((float)cov[i], 255.0f);
  float vr = (float)(mx[0] - mn[0]), vg = (float)(mx[1] - mn[1]), vb = (float)(mx[2] - mn[2]);
#pragma unroll
  for (int it = 0; it < 4; it++) {
    const float r = __fadd_rn(__fadd_rn(__fmul_rn(vr, cf[0]), __fmul_rn(vg, cf[1])), __fmul_rn(vb, cf[2]));
    const float g = __fadd_rn(__fadd_rn(__fmul_rn(vr, cf[1]), __fmul_rn(vg, cf[3])), __fmul_rn(vb, cf[4]));
    const float b = __fadd_rn(__fadd_rn(__fmul_rn(vr, cf[2]), __fmul_rn(vg, cf[4])), __fmul_rn(vb, cf[5]));
    vr = r;
    vg = g;
    vb = b;
  }
  double magn = fabs((double)vr);
  if (fabs((double)vg) > magn) magn = fabs((double)vg);
  if (fabs((double)vb) > magn) magn = fabs((double)vb);
  int ar, ag, ab;
  if (magn < 4.0) {
    ar = 299;
    ag = 587;
    ab = 114;
  } else {
    magn = __ddiv_rn(512.0, magn);
    ar = (int)__dmul_rn((double)vr, magn);
    ag = (int)__dmul_rn((double)vg, magn);
    ab = (int)__dmul_rn((double)vb, magn);
  }
  int dmin = 0x7fffffff, dmax = -0x7fffffff;
  uint32_t pmin = px[0], pmax = px[0];
#pragma unroll
  for (int i = 0; i < 16; i++) {
    const int d = ch8(px[i], 0) * ar + ch8(px[i], 1) * ag + ch8(px[i], 2) * ab;
    if (d < dmin) {
      dmin = d;
      pmin = px[i];
    }
    if (d > dmax) {
      dmax = d;
      pmax = px[i];
    }
  }
  max16 = as565(ch8(pmax, 0), ch8(pmax, 1), ch8(pmax, 2));
  min16 = as565(ch8(pmin, 0), ch8(pmin, 1), ch8(pmin, 2));
}

__device__ __forceinline__ int clamp_trunc(float y, int hi) {
  const int x = (int)y;  // toward zero; y is finite and small here
  return x < 0 ? 0 : (x > hi ? hi : x);
}

__device__ __forceinline__ void single_colour_pair(int r, int g, int b, uint16_t &max16,
                                                   uint16_t &min16) {
  const uint32_t mr = __ldg(&g_dxt_match[0][r]), mg = __ldg(&g_dxt_match[1][g]),
                 mb = __ldg(&g_dxt_match[0][b]);
  max16 = (uint16_t)(((mr & 0xFF) << 11) | ((mg & 0xFF) << 5) | (mb & 0xFF));
  min16 = (uint16_t)(((mr >> 8) << 11) | ((mg >> 8) << 5) | (mb >> 8));
}

// Least-squares endpoints for the indices in `mask` (normal equations,
// Cramer's rule), or the mean's single-colour pair when every texel has the
// same index; true when the endpoints changed (stb_dxt.h :387-475).
__device__ __forceinline__ bool dxt_refine(const uint32_t (&px)[16], uint16_t &max16, uint16_t &min16,
                                           uint32_t mask) {
  const uint16_t old_min = min16, old_max = max16;
  uint16_t mx16, mn16;
  if ((mask ^ (mask << 2)) < 4) {
    int r = 8, g = 8, b = 8;
#pragma unroll
    for (int i = 0; i < 16; i++) {
      r += ch8(px[i], 0);
      g += ch8(px[i], 1);
      b += ch8(px[i], 2);
    }
    single_colour_pair(r >> 4, g >> 4, b >> 4, mx16, mn16);
  } else {
    // per index: the high endpoint's weight in thirds, and the products of
    // the weights packed as xx << 16 | yy << 8 | xy
    int acc = 0, a1[3] = {0, 0, 0}, a2[3] = {0, 0, 0};
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const int step = (int)((mask >> (2 * i)) & 3);
      const int w1 = step == 0 ? 3 : step == 1 ? 0 : step == 2 ? 2 : 1;
      acc += step == 0 ? 0x090000 : step == 1 ? 0x000900 : step == 2 ? 0x040102 : 0x010402;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        a1[c] += w1 * ch8(px[i], c);
        a2[c] += ch8(px[i], c);
      }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) a2[c] = 3 * a2[c] - a1[c];
    const int xx = acc >> 16, yy = (acc >> 8) & 0xff, xy = acc & 0xff;
    const float frb = __fdiv_rn(__fdiv_rn(93.0f, 255.0f), (float)(xx * yy - xy * xy));
    const float fg = __fdiv_rn(__fmul_rn(frb, 63.0f), 31.0f);
    auto q = [&](int v, float f, int hi) {
      return clamp_trunc(__fadd_rn(__fmul_rn((float)v, f), 0.5f), hi);
    };
    mx16 = (uint16_t)((q(a1[0] * yy - a2[0] * xy, frb, 31) << 11) |
                      (q(a1[1] * yy - a2[1] * xy, fg, 63) << 5) | q(a1[2] * yy - a2[2] * xy, frb, 31));
    mn16 = (uint16_t)((q(a2[0] * xx - a1[0] * xy, frb, 31) << 11) |
                      (q(a2[1] * xx - a1[1] * xy, fg, 63) << 5) | q(a2[2] * xx - a1[2] * xy, frb, 31));
  }
  min16 = mn16;
  max16 = mx16;
  return old_min != mn16 || old_max != mx16;
}

// The 8-byte colour block: max16, min16, 32 index bits (stb_dxt.h
// :477-549: the constant-block shortcut, dither, fit, match, one refinement,
// the endpoint order swap).
__device__ __forceinline__ uint2 dxt_color_block(const uint32_t (&px)[16]) {
  uint32_t mask;
  uint16_t mx16, mn16;
  bool same = true;
#pragma unroll
  for (int i = 1; i < 16; i++) same = same && px[i] == px[0];
  if (same) {
    mask = 0xaaaaaaaau;
    single_colour_pair(ch8(px[0], 0), ch8(px[0], 1), ch8(px[0], 2), mx16, mn16);
  } else {
    uint32_t d[16];
    dxt_dither(px, d);
    dxt_axis(d, mx16, mn16);
    // match, refine, and match again when the refinement moved the
    // endpoints (one copy of the match code: the kernel is instruction-
    // cache bound when it is inlined twice)
#pragma unroll 1
    for (int pass = 0;; pass++) {
      mask = 0;
      if (mx16 != mn16) {
        int col[4][3];
        dxt_palette(mx16, mn16, col);
        mask = dxt_match(px, col);
      }
      if (pass == 1 || !dxt_refine(d, mx16, mn16, mask)) break;
    }
  }
  if (mx16 < mn16) {
    const uint16_t t = mn16;
    mn16 = mx16;
    mx16 = t;
    mask ^= 0x55555555u;
  }
  return make_uint2((uint32_t)mx16 | ((uint32_t)mn16 << 16), mask);
}

// The 8-byte alpha block: max, min, 16 3-bit indices by the bias rule
// (stb_dxt.h :551-601).
__device__ __forceinline__ uint2 dxt_alpha_block(const uint32_t (&px)[16]) {
  int mn = (int)(px[0] >> 24), mx = mn;
#pragma unroll
  for (int i = 1; i < 16; i++) {
    const int a = (int)(px[i] >> 24);
    if (a < mn) mn = a;
    else if (a > mx) mx = a;
  }
  const int dist = mx - mn, dist4 = dist * 4, dist2 = dist * 2;
  const int bias = (dist < 8 ? dist - 1 : dist / 2 + 2) - mn * 7;
  uint64_t bits = 0;
#pragma unroll
  for (int i = 0; i < 16; i++) {
    int a = (int)(px[i] >> 24) * 7 + bias, ind = 0;
    if (a >= dist4) {
      ind = 4;
      a -= dist4;
    }
    if (a >= dist2) {
      ind += 2;
      a -= dist2;
    }
    ind += a >= dist;
    ind = -ind & 7;  // the linear scale to DXT5 order: 0 and 1 are the ends
    ind ^= 2 > ind;
    bits |= (uint64_t)ind << (3 * i);
  }
  const uint64_t w = (uint64_t)mx | ((uint64_t)mn << 8) | (bits << 16);
  return make_uint2((uint32_t)w, (uint32_t)(w >> 32));
}

constexpr int kDxtJobsPerLaunch = 32;
struct DxtLaunch {
  JobDev job[kDxtJobsPerLaunch];
  uint32_t njobs;
};

// One thread per block of up to 32 jobs (their blocks in one index space).
#ifndef FASTC_DXT_MIN_BLOCKS
#define FASTC_DXT_MIN_BLOCKS 4  // 128 registers: four CTAs of 128 threads per SM
#endif
template <bool kAlpha>
__global__ void __launch_bounds__(128, FASTC_DXT_MIN_BLOCKS) dxt_encode_kernel(const DxtLaunch L, uint64_t total) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  int j = 0;
  while (j + 1 < (int)L.njobs && L.job[j + 1].begin <= g) j++;
  const JobDev &jb = L.job[j];
  const uint32_t lin = jb.first + (uint32_t)(g - jb.begin);
  const uint32_t bw = jb.width >> 2, bx = lin % bw, by = lin / bw;
  uint32_t px[16];
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const uint8_t *p = jb.in + ((size_t)(by * 4 + r - jb.row0) * jb.width + (size_t)bx * 4) * 4;
    uint4 v;
    if (jb.flags & kJobIn16) {
      v = __ldg(reinterpret_cast<const uint4 *>(p));
    } else {
      const uint32_t *q = reinterpret_cast<const uint32_t *>(p);
      v = make_uint4(__ldg(q), __ldg(q + 1), __ldg(q + 2), __ldg(q + 3));
    }
    px[4 * r] = v.x;
    px[4 * r + 1] = v.y;
    px[4 * r + 2] = v.z;
    px[4 * r + 3] = v.w;
  }
  const uint2 c = dxt_color_block(px);
  uint8_t *dst = jb.out + (size_t)(lin - jb.out_first) * (kAlpha ? 16 : 8);
  if (kAlpha) {
    const uint2 a = dxt_alpha_block(px);
    if (jb.flags & kJobOut16) {
      *reinterpret_cast<uint4 *>(dst) = make_uint4(a.x, a.y, c.x, c.y);
    } else {
      uint32_t *d = reinterpret_cast<uint32_t *>(dst);
      d[0] = a.x;
      d[1] = a.y;
      d[2] = c.x;
      d[3] = c.y;
    }
  } else if ((reinterpret_cast<uintptr_t>(dst) & 7) == 0) {
    *reinterpret_cast<uint2 *>(dst) = c;
  } else {
    uint32_t *d = reinterpret_cast<uint32_t *>(dst);
    d[0] = c.x;
    d[1] = c.y;
  }
}

// FasTC's decoder (DXTEncoder/src/Decompressor.cpp:26-95) for one block:
// 565 expanded by bit replication; 4 colours when the first endpoint word
// is larger (always for DXT5's colour half), else 3 colours and black; DXT1
// alpha 255; DXT5's 8-entry alpha palette (6 interpolants, or 4 with 0 and
// 255 when the first alpha is not larger). out[i] = texel i, RGBA in bytes
// 0..3.
template <bool kAlpha>
__device__ __forceinline__ void dxt_decode_block(const uint8_t *__restrict__ src, uint32_t (&out)[16]) {
  uint32_t alpha[16];
  if (kAlpha) {
    const int a0 = src[0], a1 = src[1];
    uint64_t m = 0;
    for (int k = 0; k < 6; k++) m |= (uint64_t)src[2 + k] << (8 * k);
    for (int i = 0; i < 16; i++) {
      const int idx = (int)((m >> (3 * i)) & 7);
      int v;
      if (idx < 2) v = idx ? a1 : a0;
      else if (a0 > a1) v = ((8 - idx) * a0 + (idx - 1) * a1) / 7;
      else v = idx < 6 ? ((6 - idx) * a0 + (idx - 1) * a1) / 5 : (idx == 6 ? 0 : 255);
      alpha[i] = (uint32_t)v << 24;
    }
    src += 8;
  } else {
    for (int i = 0; i < 16; i++) alpha[i] = 0xFF000000u;
  }
  const uint16_t c0 = (uint16_t)(src[0] | (src[1] << 8)), c1 = (uint16_t)(src[2] | (src[3] << 8));
  int col[4][3];
  dxt_palette(c0, c1, col);  // (2a + b) / 3 and (a + 2b) / 3, as FasTC's decoder
  if (!kAlpha && !(c0 > c1)) {
    for (int k = 0; k < 3; k++) {
      col[2][k] = (col[0][k] + col[1][k]) / 2;
      col[3][k] = 0;
    }
  }
  const uint32_t m = (uint32_t)src[4] | ((uint32_t)src[5] << 8) | ((uint32_t)src[6] << 16) |
                     ((uint32_t)src[7] << 24);
  for (int i = 0; i < 16; i++) {
    const int *c = col[(m >> (2 * i)) & 3];
    out[i] = alpha[i] | (uint32_t)c[0] | ((uint32_t)c[1] << 8) | ((uint32_t)c[2] << 16);
  }
}

// FasTC's DecompressDXT1 / DXT5 (Decompressor.cpp:98-155): one thread per
// block, texels outside the image skipped.
template <bool kAlpha>
__global__ void dxt_decode_kernel(const uint8_t *__restrict__ blocks, uint8_t *__restrict__ rgba,
                                  uint32_t width, uint32_t height) {
  const uint32_t bw = (width + 3) / 4, bh = (height + 3) / 4;
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= (uint64_t)bw * bh) return;
  const uint32_t bx = (uint32_t)(b % bw), by = (uint32_t)(b / bw);
  uint32_t px[16];
  dxt_decode_block<kAlpha>(blocks + b * (kAlpha ? 16 : 8), px);
  for (int y = 0; y < 4; y++) {
    if (by * 4 + y >= height) break;
    for (int x = 0; x < 4; x++) {
      if (bx * 4 + x >= width) break;
      *reinterpret_cast<uint32_t *>(rgba + ((size_t)(by * 4 + y) * width + bx * 4 + x) * 4) = px[4 * y + x];
    }
  }
}

// FasTC's Image::ComputePSNR metric (Base/src/Image.cpp:206-255) per 4x4
// block of decoded DXT blocks against the original texels: per texel, RGB
// premultiplied by alpha / 255 in double, the three squared differences
// summed in channel order; per block, the texels in row order (texels
// outside the image skipped).
template <bool kAlpha>
__global__ void dxt_error_kernel(const uint8_t *__restrict__ blocks, const uint8_t *__restrict__ rgba,
                                 uint32_t width, uint32_t height, double *__restrict__ sse) {
  const uint32_t bw = (width + 3) / 4, bh = (height + 3) / 4;
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= (uint64_t)bw * bh) return;
  const uint32_t bx = (uint32_t)(b % bw), by = (uint32_t)(b / bw);
  uint32_t dec[16];
  dxt_decode_block<kAlpha>(blocks + b * (kAlpha ? 16 : 8), dec);
  double s = 0.0;
  for (int y = 0; y < 4; y++) {
    if (by * 4 + y >= height) break;
    for (int x = 0; x < 4; x++) {
      if (bx * 4 + x >= width) break;
      const uint8_t *p = rgba + ((size_t)(by * 4 + y) * width + bx * 4 + x) * 4;
      const uint32_t d = dec[4 * y + x];
      const double ra = (double)p[3] / 255.0, ua = (double)(d >> 24) / 255.0;
      double t = 0.0;  // the texel's three terms first, then the block's running sum
      for (int c = 0; c < 3; c++) {
        const double e = ra * (double)p[c] - ua * (double)((d >> (8 * c)) & 0xFF);
        t += e * e;
      }
      s += t;
    }
  }
  sse[b] = s;
}

// The same error for count consecutive blocks of an image (raster block
// first on), the texels given from row row0 on.
template <bool kAlpha>
__global__ void dxt_range_error_kernel(const uint8_t *__restrict__ blocks,
                                       const uint8_t *__restrict__ rows, uint32_t width, uint32_t row0,
                                       uint32_t first, uint32_t count, double *__restrict__ sse) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint32_t bw = width / 4, b = first + k;
  const uint32_t bx = b % bw, by = b / bw;
  uint32_t dec[16];
  dxt_decode_block<kAlpha>(blocks + (size_t)k * (kAlpha ? 16 : 8), dec);
  double s = 0.0;
  for (int y = 0; y < 4; y++)
    for (int x = 0; x < 4; x++) {
      const uint8_t *p = rows + ((size_t)(by * 4 + y - row0) * width + bx * 4 + x) * 4;
      const uint32_t d = dec[4 * y + x];
      const double ra = (double)p[3] / 255.0, ua = (double)(d >> 24) / 255.0;
      double t = 0.0;
      for (int c = 0; c < 3; c++) {
        const double e = ra * (double)p[c] - ua * (double)((d >> (8 * c)) & 0xFF);
        t += e * e;
      }
      s += t;
    }
  sse[k] = s;
}

cudaError_t launch_dxt_error(const uint8_t *blocks, const uint8_t *rgba, uint32_t width, uint32_t height,
                             bool alpha, double *block_sse, double *total, cudaStream_t st) {
  const uint64_t nb = (uint64_t)((width + 3) / 4) * ((height + 3) / 4);
  const unsigned grid = (unsigned)((nb + 127) / 128);
  if (alpha) dxt_error_kernel<true><<<grid, 128, 0, st>>>(blocks, rgba, width, height, block_sse);
  else dxt_error_kernel<false><<<grid, 128, 0, st>>>(blocks, rgba, width, height, block_sse);
  if (total) {
    const int e = launch_sum(block_sse, nb, total, st);
    if (e) return (cudaError_t)e;
  }
  return cudaPeekAtLastError();
}

std::mutex g_dxt_mu;
bool g_dxt_ready[64];

cudaError_t dxt_setup(int dev) {
  std::lock_guard<std::mutex> lk(g_dxt_mu);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (g_dxt_ready[dev]) return cudaSuccess;
  static uint16_t t[2][256];
  build_match_tables(t);
  const cudaError_t e = cudaMemcpyToSymbol(g_dxt_match, t, sizeof(t));
  if (e == cudaSuccess) g_dxt_ready[dev] = true;
  return e;
}

// Encodes up to kDxtJobsPerLaunch device jobs (dj[k].begin their block
// offsets) in one launch.
cudaError_t dxt_launch(const JobDev *dj, uint32_t n, uint64_t total, bool alpha, cudaStream_t st) {
  if (total == 0) return cudaSuccess;
  DxtLaunch L{};
  for (uint32_t k = 0; k < n; k++) L.job[k] = dj[k];
  L.njobs = n;
  const unsigned grid = (unsigned)((total + 127) / 128);
  if (alpha) dxt_encode_kernel<true><<<grid, 128, 0, st>>>(L, total);
  else dxt_encode_kernel<false><<<grid, 128, 0, st>>>(L, total);
  return cudaPeekAtLastError();
}

// Validates the jobs and fills their device-side descriptions (pointers
// set by the caller); returns false on a bad job.
bool dxt_jobs(const fastc_bc7_job *jobs, uint32_t n, std::vector<JobDev> *out) {
  fastc_bc7_settings dflt;
  fastc_bc7_settings_default(&dflt);
  out->resize(n);
  for (uint32_t i = 0; i < n; i++) {
    uint32_t first, count;
    if (!jobs[i].in || !jobs[i].out || !host::job_range(jobs[i], &first, &count) ||
        (reinterpret_cast<uintptr_t>(jobs[i].in) & 3) || (reinterpret_cast<uintptr_t>(jobs[i].out) & 3))
      return false;
    (*out)[i] = host::make_job(jobs[i], dflt, first, count, 0);
  }
  return true;
}

// Host-memory calls: staging buffers, and three streams so that a group's
// texel upload, the previous group's encode and the group before's block
// download overlap (the copies, not the encode, bound these calls).
struct DxtHostContext {
  void *in = nullptr, *out = nullptr;
  size_t in_cap = 0, out_cap = 0;
  cudaStream_t h2d = nullptr, comp = nullptr, d2h = nullptr;
  std::vector<cudaEvent_t> ev;
  int device = -1;
} g_dxt_host;

cudaError_t ensure(void **p, size_t *cap, size_t n) {
  if (n <= *cap) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const cudaError_t e = cudaMalloc(p, n);
  if (e == cudaSuccess) *cap = n;
  return e;
}

// The context of device `dev` (the current one); a previous device's
// objects are released on that device.
cudaError_t host_context(int dev, size_t events) {
  DxtHostContext &h = g_dxt_host;
  if (h.device != dev) {
    if (h.device >= 0 && cudaSetDevice(h.device) == cudaSuccess) {
      cudaFree(h.in);
      cudaFree(h.out);
      for (cudaEvent_t e : h.ev) cudaEventDestroy(e);
      cudaStreamDestroy(h.h2d);
      cudaStreamDestroy(h.comp);
      cudaStreamDestroy(h.d2h);
    }
    h = DxtHostContext();
    cudaError_t e = cudaSetDevice(dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h.h2d, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h.comp, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h.d2h, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    h.device = dev;
  }
  while (h.ev.size() < events) {
    cudaEvent_t e;
    const cudaError_t st = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (st != cudaSuccess) return st;
    h.ev.push_back(e);
  }
  return cudaSuccess;
}

}  // namespace

cudaError_t dxt_prepare(int dev) { return dxt_setup(dev); }

cudaError_t dxt_encode_jobs(JobDev *jobs, uint32_t n, bool alpha, cudaStream_t st) {
  for (uint32_t k0 = 0; k0 < n; k0 += kDxtJobsPerLaunch) {
    const uint32_t m = std::min<uint32_t>(kDxtJobsPerLaunch, n - k0);
    uint64_t begin = 0;
    for (uint32_t k = k0; k < k0 + m; k++) {
      jobs[k].begin = begin;
      begin += jobs[k].nblocks;
    }
    const cudaError_t e = dxt_launch(jobs + k0, m, begin, alpha, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t dxt_range_error(const uint8_t *blocks, const uint8_t *rows, uint32_t width, uint32_t row0,
                            uint32_t first, uint32_t count, bool alpha, double *block_sse,
                            double *total, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  const unsigned grid = (count + 127) / 128;
  if (alpha) dxt_range_error_kernel<true><<<grid, 128, 0, st>>>(blocks, rows, width, row0, first, count, block_sse);
  else dxt_range_error_kernel<false><<<grid, 128, 0, st>>>(blocks, rows, width, row0, first, count, block_sse);
  const int e = launch_sum(block_sse, count, total, st);
  if (e) return (cudaError_t)e;
  return cudaPeekAtLastError();
}

}  // namespace fastc

using fastc::JobDev;
using namespace fastc::host;

extern "C" {

fastc_bc7_status fastc_dxt_compress_device(const fastc_bc7_job *jobs, uint32_t n, int format,
                                           void *stream) {
  if ((!jobs && n) || (format != FASTC_DXT1 && format != FASTC_DXT5))
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::vector<JobDev> dj;
  if (!fastc::dxt_jobs(jobs, n, &dj)) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  const int dev = current_device();
  if (dev < 0) return FASTC_BC7_ERR_NO_DEVICE;
  CK(fastc::dxt_setup(dev));
  const bool alpha = format == FASTC_DXT5;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  for (uint32_t k0 = 0; k0 < n; k0 += fastc::kDxtJobsPerLaunch) {
    const uint32_t m = std::min<uint32_t>(fastc::kDxtJobsPerLaunch, n - k0);
    uint64_t begin = 0;
    for (uint32_t k = 0; k < m; k++) {
      JobDev &d = dj[k0 + k];
      d.flags = fastc::host::align_flags(jobs[k0 + k].in, jobs[k0 + k].out);
      if (!alpha) d.flags &= ~fastc::kJobOut16;
      d.begin = begin;
      begin += d.nblocks;
    }
    CK(fastc::dxt_launch(dj.data() + k0, m, begin, alpha, st));
  }
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_dxt_compress_batch(const fastc_bc7_job *jobs, uint32_t n, int format) {
  if ((!jobs && n) || (format != FASTC_DXT1 && format != FASTC_DXT5)) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  std::vector<JobDev> dj;
  if (!fastc::dxt_jobs(jobs, n, &dj)) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  const bool alpha = format == FASTC_DXT5;
  const size_t bsz = alpha ? 16 : 8;
  // per job: the texel rows its blocks cover, staged at 256-byte offsets
  std::vector<size_t> in_off(n), in_bytes(n), out_off(n);
  size_t in_total = 0, out_total = 0;
  uint64_t total = 0;
  for (uint32_t i = 0; i < n; i++) {
    JobDev &d = dj[i];
    const uint32_t bw = jobs[i].width / 4;
    const uint32_t r0 = d.nblocks ? d.first / bw : 0, r1 = d.nblocks ? (d.first + d.nblocks - 1) / bw : 0;
    in_bytes[i] = d.nblocks ? (size_t)(r1 - r0 + 1) * 4 * jobs[i].width * 4 : 0;
    d.row0 = r0 * 4;
    d.out_first = d.first;
    in_off[i] = in_total;
    out_off[i] = out_total;
    in_total += (in_bytes[i] + 255) & ~(size_t)255;
    out_total += ((size_t)d.nblocks * bsz + 255) & ~(size_t)255;
    total += d.nblocks;
  }
  if (total == 0) return FASTC_BC7_OK;
  const int dev = current_device();
  if (dev < 0) return FASTC_BC7_ERR_NO_DEVICE;
  CK(fastc::dxt_setup(dev));
  const uint32_t groups = (n + fastc::kDxtJobsPerLaunch - 1) / fastc::kDxtJobsPerLaunch;
  std::lock_guard<std::mutex> lk(fastc::g_dxt_mu);
  CK(fastc::host_context(dev, 2 * (size_t)groups));
  fastc::DxtHostContext &h = fastc::g_dxt_host;
  // Page-locked host buffers (cudaHostAlloc, cudaHostRegister) are mapped
  // into the device's address space: the kernel then reads the texels and
  // writes the blocks across the host link itself, with no staging copies
  // (on GB300 the NVLink-C2C link to the Grace CPU). Every job's buffers
  // must be page-locked for this; otherwise the rows are staged below.
  bool mapped = true;
  std::vector<JobDev> zj(dj);
  for (uint32_t i = 0; i < n && mapped; i++) {
    if (!zj[i].nblocks) continue;
    cudaPointerAttributes ai{}, ao{};
    if (cudaPointerGetAttributes(&ai, jobs[i].in) != cudaSuccess ||
        cudaPointerGetAttributes(&ao, jobs[i].out) != cudaSuccess) {
      cudaGetLastError();
      mapped = false;
      break;
    }
    mapped = ai.type == cudaMemoryTypeHost && ao.type == cudaMemoryTypeHost && ai.devicePointer &&
             ao.devicePointer;
    if (mapped) {
      zj[i].in = static_cast<const uint8_t *>(ai.devicePointer);
      zj[i].out = static_cast<uint8_t *>(ao.devicePointer);
      zj[i].row0 = 0;
      zj[i].out_first = 0;
    }
  }
  // Every stream of the call is drained before it returns, also after an
  // error, so that no copy or kernel of the call still touches the caller's
  // buffers afterwards; the first error is reported.
  const cudaStream_t ss[3] = {h.comp, h.h2d, h.d2h};
  auto drain = [&](cudaError_t e) -> fastc_bc7_status {
    for (cudaStream_t st : ss) {
      const cudaError_t se = cudaStreamSynchronize(st);
      if (e == cudaSuccess) e = se;
    }
    return e == cudaSuccess ? FASTC_BC7_OK : fail_cuda(e);
  };
  cudaError_t e = cudaSuccess;
  if (mapped) {
    // the groups' launches are independent: spread over the three streams
    // so that small groups overlap while the link is busy
    uint32_t g = 0;
    for (uint32_t k0 = 0; k0 < n && e == cudaSuccess; k0 += fastc::kDxtJobsPerLaunch, g++) {
      const uint32_t m = std::min<uint32_t>(fastc::kDxtJobsPerLaunch, n - k0);
      uint64_t begin = 0;
      for (uint32_t k = k0; k < k0 + m; k++) {
        JobDev &d = zj[k];
        d.flags = fastc::host::align_flags(d.in, d.out);
        if (!alpha) d.flags &= ~fastc::kJobOut16;
        d.begin = begin;
        begin += d.nblocks;
      }
      e = fastc::dxt_launch(zj.data() + k0, m, begin, alpha, ss[g % 3]);
    }
    return drain(e);
  }
  CK(fastc::ensure(&h.in, &h.in_cap, in_total));
  CK(fastc::ensure(&h.out, &h.out_cap, out_total));
  uint8_t *in = static_cast<uint8_t *>(h.in), *out = static_cast<uint8_t *>(h.out);
  for (uint32_t g = 0; g < groups && e == cudaSuccess; g++) {
    const uint32_t k0 = g * fastc::kDxtJobsPerLaunch;
    const uint32_t m = std::min<uint32_t>(fastc::kDxtJobsPerLaunch, n - k0);
    uint64_t begin = 0;
    for (uint32_t k = k0; k < k0 + m && e == cudaSuccess; k++) {
      JobDev &d = dj[k];
      if (d.nblocks)
        e = cudaMemcpyAsync(in + in_off[k], jobs[k].in + (size_t)d.row0 * jobs[k].width * 4, in_bytes[k],
                            cudaMemcpyHostToDevice, h.h2d);
      d.in = in + in_off[k];
      d.out = out + out_off[k];
      d.flags = fastc::kJobIn16 | (alpha ? fastc::kJobOut16 : 0u);
      d.begin = begin;
      begin += d.nblocks;
    }
    if (e == cudaSuccess) e = cudaEventRecord(h.ev[2 * g], h.h2d);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h.comp, h.ev[2 * g], 0);
    if (e == cudaSuccess) e = fastc::dxt_launch(dj.data() + k0, m, begin, alpha, h.comp);
    if (e == cudaSuccess) e = cudaEventRecord(h.ev[2 * g + 1], h.comp);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h.d2h, h.ev[2 * g + 1], 0);
    for (uint32_t k = k0; k < k0 + m && e == cudaSuccess; k++)
      if (dj[k].nblocks)
        e = cudaMemcpyAsync(jobs[k].out + (size_t)dj[k].first * bsz, out + out_off[k],
                            (size_t)dj[k].nblocks * bsz, cudaMemcpyDeviceToHost, h.d2h);
  }
  return drain(e);
}

fastc_bc7_status fastc_dxt_compress(const fastc_bc7_job *job, int format) {
  if (!job) return FASTC_BC7_ERR_INVALID_ARGUMENT;
  return fastc_dxt_compress_batch(job, 1, format);
}

fastc_bc7_status fastc_dxt_block_error_device(const uint8_t *blocks, const uint8_t *rgba, uint32_t width,
                                              uint32_t height, int format, double *block_sse, double *total,
                                              void *stream) {
  if (!blocks || !rgba || !block_sse || width == 0 || height == 0 ||
      (format != FASTC_DXT1 && format != FASTC_DXT5))
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  const int dev = current_device();
  if (dev < 0) return FASTC_BC7_ERR_NO_DEVICE;
  CK(fastc::launch_dxt_error(blocks, rgba, width, height, format == FASTC_DXT5, block_sse, total,
                             static_cast<cudaStream_t>(stream)));
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_dxt_psnr(const uint8_t *blocks, const uint8_t *rgba, uint32_t width, uint32_t height,
                                int format, double *psnr, double *block_sse) {
  if (!blocks || !rgba || width == 0 || height == 0 || (format != FASTC_DXT1 && format != FASTC_DXT5))
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  const int dev = current_device();
  if (dev < 0) return FASTC_BC7_ERR_NO_DEVICE;
  const size_t nb = (size_t)((width + 3) / 4) * ((height + 3) / 4);
  const size_t bsz = format == FASTC_DXT5 ? 16 : 8, img = (size_t)width * height * 4;
  std::lock_guard<std::mutex> lk(fastc::g_dxt_mu);
  CK(fastc::host_context(dev, 0));
  fastc::DxtHostContext &h = fastc::g_dxt_host;
  // texels, then the blocks (byte loads), in the input buffer; the per-block
  // errors after the total in the output buffer
  CK(fastc::ensure(&h.in, &h.in_cap, img + nb * bsz));
  CK(fastc::ensure(&h.out, &h.out_cap, (nb + 1) * sizeof(double)));
  uint8_t *dimg = static_cast<uint8_t *>(h.in), *dblk = dimg + img;
  double *dsse = static_cast<double *>(h.out);
  double total = 0.0;
  cudaError_t e = cudaMemcpyAsync(dimg, rgba, img, cudaMemcpyHostToDevice, h.comp);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dblk, blocks, nb * bsz, cudaMemcpyHostToDevice, h.comp);
  if (e == cudaSuccess)
    e = fastc::launch_dxt_error(dblk, dimg, width, height, format == FASTC_DXT5, dsse + 1, dsse, h.comp);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, dsse, sizeof(double), cudaMemcpyDeviceToHost, h.comp);
  if (e == cudaSuccess && block_sse)
    e = cudaMemcpyAsync(block_sse, dsse + 1, nb * sizeof(double), cudaMemcpyDeviceToHost, h.comp);
  // drained also after an error: no copy of the call outlives it
  const cudaError_t se = cudaStreamSynchronize(h.comp);
  if (e == cudaSuccess) e = se;
  if (e != cudaSuccess) return fail_cuda(e);
  if (psnr) *psnr = 10.0 * std::log10((3.0 * 255.0 * 255.0) / (total / ((double)width * height)));
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_dxt_decompress_device(const uint8_t *blocks, uint8_t *rgba, uint32_t width,
                                             uint32_t height, int format, void *stream) {
  if (!blocks || !rgba || width == 0 || height == 0 || (reinterpret_cast<uintptr_t>(rgba) & 3) ||
      (format != FASTC_DXT1 && format != FASTC_DXT5))
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  const int dev = current_device();
  if (dev < 0) return FASTC_BC7_ERR_NO_DEVICE;
  CK(fastc::dxt_setup(dev));
  const uint64_t nb = (uint64_t)((width + 3) / 4) * ((height + 3) / 4);
  const unsigned grid = (unsigned)((nb + 127) / 128);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (format == FASTC_DXT5) fastc::dxt_decode_kernel<true><<<grid, 128, 0, st>>>(blocks, rgba, width, height);
  else fastc::dxt_decode_kernel<false><<<grid, 128, 0, st>>>(blocks, rgba, width, height);
  CK(cudaPeekAtLastError());
  return FASTC_BC7_OK;
}

fastc_bc7_status fastc_dxt_decompress(const uint8_t *blocks, uint8_t *rgba, uint32_t width,
                                      uint32_t height, int format) {
  if (!blocks || !rgba || width == 0 || height == 0 || (format != FASTC_DXT1 && format != FASTC_DXT5))
    return FASTC_BC7_ERR_INVALID_ARGUMENT;
  const int dev = current_device();
  if (dev < 0) return FASTC_BC7_ERR_NO_DEVICE;
  CK(fastc::dxt_setup(dev));
  const size_t nb = (size_t)((width + 3) / 4) * ((height + 3) / 4);
  const size_t bsz = format == FASTC_DXT5 ? 16 : 8, img = (size_t)width * height * 4;
  std::lock_guard<std::mutex> lk(fastc::g_dxt_mu);
  CK(fastc::host_context(dev, 0));
  fastc::DxtHostContext &h = fastc::g_dxt_host;
  CK(fastc::ensure(&h.in, &h.in_cap, nb * bsz));
  CK(fastc::ensure(&h.out, &h.out_cap, img));
  cudaError_t e = cudaMemcpyAsync(h.in, blocks, nb * bsz, cudaMemcpyHostToDevice, h.comp);
  if (e == cudaSuccess) {
    const unsigned grid = (unsigned)((nb + 127) / 128);
    const uint8_t *din = static_cast<const uint8_t *>(h.in);
    uint8_t *dout = static_cast<uint8_t *>(h.out);
    if (format == FASTC_DXT5) fastc::dxt_decode_kernel<true><<<grid, 128, 0, h.comp>>>(din, dout, width, height);
    else fastc::dxt_decode_kernel<false><<<grid, 128, 0, h.comp>>>(din, dout, width, height);
    e = cudaPeekAtLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(rgba, h.out, img, cudaMemcpyDeviceToHost, h.comp);
  // drained also after an error: no copy of the call outlives it
  const cudaError_t se = cudaStreamSynchronize(h.comp);
  if (e == cudaSuccess) e = se;
  return e == cudaSuccess ? FASTC_BC7_OK : fail_cuda(e);
}

}  // extern "C"
