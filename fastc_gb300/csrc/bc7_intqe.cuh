// Uniform-metric QuantizedError (FasTC RGBAEndpoints.cpp:190-310) in exact
// integer arithmetic, for integer endpoints: used by the shape estimate of
// the select stage and by the annealing loop (bc7_pipeline.cu).
#pragma once

#include <climits>
#include <cstdint>

namespace fastc {

// Threads per CTA of the kernels that use these helpers: per-thread arrays
// in shared memory are interleaved with this stride (element k of thread t
// at [k * kLaneStride + t]), so a warp's accesses hit 32 distinct banks.
constexpr int kLaneStride = 128;

// Weight of a `kBits`-bit index (constant divisor).
template <int kBits>
__device__ __forceinline__ uint32_t wt(int j) {
  return (64u * (uint32_t)j + (uint32_t)(((1 << kBits) - 1) / 2)) / (uint32_t)((1 << kBits) - 1);
}

// d = c + a.h0 * b.b0 + a.h1 * b.b1 (lo) / b.b2, b.b3 (hi); a signed 16-bit
// pairs, b unsigned bytes.
__device__ __forceinline__ int dp2a_lo(uint32_t a, uint32_t b, int c) {
  int d;
  asm("dp2a.lo.s32.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}
__device__ __forceinline__ int dp2a_hi(uint32_t a, uint32_t b, int c) {
  int d;
  asm("dp2a.hi.s32.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

// Uniform-metric QuantizedError in exact integers. For a texel e and a
// palette colour c, |e - c|^2 = |e|^2 + |c|^2 - 2 e.c: |e|^2 summed over the
// fit is a constant of the fit, |c|^2 is tabulated with the palette, and
// e.c is one dp4a. The two candidates FasTC compares for each texel (the
// indices either side of its projection) share |e|^2, so comparing
// |c|^2 - 2 e.c picks the same index, and the totals are the same integers.

// Palette entry j holds colour j and colour j + 1 with their squared
// lengths, (c_j, |c_j|^2, c_j+1, |c_j+1|^2), so one 16-byte load serves both
// candidates; the last entry repeats its colour.
template <int kBits>
__device__ __forceinline__ void palette_sq(uint32_t q1, uint32_t q2, uint4 *pal) {
  constexpr int T = kLaneStride;
  constexpr int kN = 1 << kBits;
  const uint32_t rb1 = q1 & 0x00FF00FFu, ga1 = (q1 >> 8) & 0x00FF00FFu;
  const uint32_t rb2 = q2 & 0x00FF00FFu, ga2 = (q2 >> 8) & 0x00FF00FFu;
  uint32_t prev = 0, prev_sq = 0;
#pragma unroll
  for (int j = 0; j < kN; j++) {
    const uint32_t w1 = wt<kBits>(j), w0 = 64u - w1;
    const uint32_t vrb = rb1 * w0 + rb2 * w1 + 0x00200020u;
    const uint32_t vga = ga1 * w0 + ga2 * w1 + 0x00200020u;
    const uint32_t c = ((vrb >> 6) & 0x00FF00FFu) | (((vga >> 6) & 0x00FF00FFu) << 8);
    const uint32_t sq = __dp4a(c, c, 0u);
    if (j > 0) pal[(j - 1) * T] = make_uint4(prev, prev_sq, c, sq);
    if (j == kN - 1) pal[j * T] = make_uint4(c, sq, c, sq);
    prev = c;
    prev_sq = sq;
  }
}

// The projection onto q2 - q1: D = (p - q1).(q2 - q1) by two dp2a, and
// floor(D k / L) by a multiply-high with R = floor((2^32 - 1) / L) + 1,
// which never undershoots and overshoots by at most one (never when D k is
// a multiple of L).
struct Proj {
  uint32_t dlo, dhi, R;
  int negk, L;
};

__device__ __forceinline__ Proj make_proj(uint32_t q1, uint32_t q2) {
  int u1[4], dir[4];
#pragma unroll
  for (int c = 0; c < 4; c++) {
    u1[c] = (int)((q1 >> (8 * c)) & 0xFF);
    dir[c] = (int)((q2 >> (8 * c)) & 0xFF) - u1[c];
  }
  Proj pj;
  pj.L = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2] + dir[3] * dir[3];
  pj.dlo = ((uint32_t)dir[0] & 0xFFFFu) | ((uint32_t)dir[1] << 16);
  pj.dhi = ((uint32_t)dir[2] & 0xFFFFu) | ((uint32_t)dir[3] << 16);
  pj.negk = -(dir[0] * u1[0] + dir[1] * u1[1] + dir[2] * u1[2] + dir[3] * u1[3]);
  pj.R = 0xFFFFFFFFu / (uint32_t)(pj.L > 0 ? pj.L : 1) + 1u;  // 0 for L == 1 (then D >= L decides)
  return pj;
}

// The candidates FasTC compares for projected point p: j1 = floor(D k / L)
// clamped to [0, k], and j1 + 1 unless D k / L is an integer or clamped.
// FasTC computes the quotient in float, fl(fl(D / L) k); where D k is a
// multiple of L, D / L is exactly j / k, and fl(fl(j / k) k) == j for every
// j < k in {3, 7, 15} (checked exhaustively in the tests), so the integer
// quotient always reproduces FasTC's two indices.
template <int kBits>
__device__ __forceinline__ int nearest_pair(const Proj &pj, uint32_t p, bool &two) {
  constexpr int km = (1 << kBits) - 1;
  const int D = dp2a_hi(pj.dhi, p, dp2a_lo(pj.dlo, p, pj.negk));
  const uint32_t num = (uint32_t)max(D, 0) * (uint32_t)km;
  const uint32_t q = __umulhi(num, pj.R);
  const int r = (int)(num - q * (uint32_t)pj.L);
  const bool over = D >= pj.L;
  two = (r != 0) & !over;
  return over ? km : (int)q - (r < 0 ? 1 : 0);
}

// |c|^2 - 2 e.c of the better candidate, and its index.
__device__ __forceinline__ int pair_term(uint32_t e, const uint4 *pal, int j1, bool two, int &bj) {
  constexpr int T = kLaneStride;
  const uint4 a = pal[j1 * T];
  const int t1 = (int)a.y - 2 * (int)__dp4a(e, a.x, 0u);
  const int t2 = (int)a.w - 2 * (int)__dp4a(e, a.z, 0u);
  const bool second = two & (t2 < t1);
  bj = j1 + (second ? 1 : 0);
  return second ? t2 : t1;
}

// Ascending sort of 16 integers in registers (bitonic network, fixed
// indices so that the array is never addressed dynamically).
__device__ __forceinline__ void sort16(int (&v)[16]) {
#pragma unroll
  for (int k = 2; k <= 16; k <<= 1)
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int l = i ^ j;
        if (l > i) {
          const int a = v[i], b = v[l];
          const bool up = (i & k) == 0;
          v[i] = up ? min(a, b) : max(a, b);
          v[l] = up ? max(a, b) : min(a, b);
        }
      }
}

// A lower bound on the uniform-metric QuantizedError of n texels against
// ANY pair of endpoints with a kLevels-colour palette, for pruning fits
// that cannot win their block; the larger of two bounds.
//
// Line term: every palette colour is the exact interpolation rounded per
// channel (at most half a unit), so it lies within one unit of the line
// through the endpoints; a texel at distance d from that line has error at
// least max(0, d - 1)^2 >= d^2 - 2d. Summed: S - 2 sqrt(n S)
// (Cauchy-Schwarz), with S = sum d^2 >= R, the scatter left after the
// best-fitting line (trace minus largest eigenvalue of the scatter matrix);
// the bound grows with S for S >= n, so R - 2 sqrt(n R) holds whenever
// R >= n. The largest eigenvalue of the scatter A scaled to unit trace is
// at most sqrt(|A^2|_F) (the fourth root of the sum of the eigenvalues'
// fourth powers). The scatter is exact in integers; the float steps after
// it are covered by a margin of 1e-5 of the trace.
//
// Palette-size term: on any unit direction u a texel's error is at least
// (u.p - u.c)^2, so the error is at least the best kLevels-level
// quantisation of the projections u.p (1-D k-means; its groups are runs of
// the sorted projections). A run of span w costs at least w^2 / 2, and the
// runs' spans add up to at least G, the n - kLevels smallest gaps between
// sorted projections, so the error is at least G^2 / (2 kLevels). It is
// computed for 4-colour palettes (where it prunes; with 8 or 16 colours the
// clusters rarely have enough texels). u is the scatter's principal
// direction (four power iterations), rounded to an integer
// direction d with components in 1/64 of the largest, so the projections
// d.p are exact integers and the term is G^2 / (2 kLevels |d|^2).
template <int kLevels>
__device__ __forceinline__ float qe_lower_bound(const uint32_t *pts, int stride, int n) {
  int s[4] = {0, 0, 0, 0}, q[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < n; k++) {
    const uint32_t e = pts[k * stride];
    int v[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      v[c] = (int)((e >> (8 * c)) & 0xFF);
      s[c] += v[c];
    }
    int m = 0;
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = a; b < 4; b++) q[m++] += v[a] * v[b];
  }
  // n * scatter: entries below 16 * 16 * 255^2 < 2^24, exact in float
  float A[4][4];
  int tr = 0, m = 0;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = a; b < 4; b++) {
      const int v = n * q[m++] - s[a] * s[b];
      if (a == b) tr += v;
      A[a][b] = A[b][a] = (float)v;
    }
  if (tr <= 0) return 0.0f;
  const float inv = 1.0f / (float)tr;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) A[a][b] *= inv;
  float f = 0.0f;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = a; b < 4; b++) {
      const float v = A[a][0] * A[0][b] + A[a][1] * A[1][b] + A[a][2] * A[2][b] + A[a][3] * A[3][b];
      f += (a == b ? 1.0f : 2.0f) * v * v;
    }
  const float lam = sqrtf(sqrtf(f));
  const float R = fmaxf(0.0f, 1.0f - lam - 1e-5f) * ((float)tr / (float)n);
  const float fn = (float)n;
  const float line = R >= fn ? fmaxf(0.0f, R - 2.0f * sqrtf(fn * R) - 1e-3f * R) : 0.0f;
  // the palette-size term prunes in practice for 4-colour palettes only
  if (kLevels != 4 || n <= kLevels) return line;
  int d0 = 0;
#pragma unroll
  for (int c = 1; c < 4; c++)
    if (A[c][c] > A[d0][d0]) d0 = c;
  float u[4];
#pragma unroll
  for (int c = 0; c < 4; c++) u[c] = d0 == 0 ? A[c][0] : d0 == 1 ? A[c][1] : d0 == 2 ? A[c][2] : A[c][3];
#pragma unroll
  for (int it = 0; it < 4; it++) {
    float w[4], mx = 0.0f;
#pragma unroll
    for (int a = 0; a < 4; a++) {
      w[a] = A[a][0] * u[0] + A[a][1] * u[1] + A[a][2] * u[2] + A[a][3] * u[3];
      mx = fmaxf(mx, fabsf(w[a]));
    }
    if (!(mx > 0.0f)) return line;
    const float r = 1.0f / mx;
#pragma unroll
    for (int a = 0; a < 4; a++) u[a] = w[a] * r;
  }
  const float um = fmaxf(fmaxf(fabsf(u[0]), fabsf(u[1])), fmaxf(fabsf(u[2]), fabsf(u[3])));
  int d[4], dd = 0;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    d[c] = __float2int_rn(u[c] * 64.0f / um);
    dd += d[c] * d[c];
  }
  if (dd == 0) return line;
  int sp[16];
#pragma unroll
  for (int k = 0; k < 16; k++) {
    sp[k] = INT_MAX;
    if (k < n) {
      const uint32_t e = pts[k * stride];
      sp[k] = d[0] * (int)(e & 0xFF) + d[1] * (int)((e >> 8) & 0xFF) + d[2] * (int)((e >> 16) & 0xFF) +
              d[3] * (int)(e >> 24);
    }
  }
  sort16(sp);
  // G = the gaps' sum less the three largest gaps
  int sum = 0, g1 = 0, g2 = 0, g3 = 0;
#pragma unroll
  for (int k = 0; k < 15; k++) {
    const int g = k + 1 < n ? sp[k + 1] - sp[k] : 0;
    sum += g;
    const int a = max(g1, g), b = max(g2, min(g1, g)), c = max(g3, min(g2, g));
    g1 = a;
    g2 = b;
    g3 = c;
  }
  const int G = sum - g1 - g2 - g3;
  const float fg = (float)G;
  return fmaxf(line, fg * fg / (float)(2 * kLevels * dd) * (1.0f - 1e-5f));
}

// Sixteen texels in registers (one-subset modes; texel k is point k).
// pr: the projected points of the rotation modes (the texel with the
// rotated channel and alpha 255); for other modes the texels themselves.
template <int kBits, bool kRot, bool kIdx>
__device__ __forceinline__ float qe_reg(const uint32_t (&e)[16], const uint32_t (&pr)[16], int se,
                                        uint4 *pal, uint32_t q1, uint32_t q2, uint64_t &idx) {
  const Proj pj = make_proj(q1, q2);
  int acc = 0;
  if (pj.L == 0) {
    const int sq = (int)__dp4a(q1, q1, 0u);
#pragma unroll
    for (int k = 0; k < 16; k++) acc += sq - 2 * (int)__dp4a(e[k], q1, 0u);
    return (float)(se + acc);
  }
  palette_sq<kBits>(q1, q2, pal);
#pragma unroll
  for (int k = 0; k < 16; k++) {
    bool two;
    const int j1 = nearest_pair<kBits>(pj, kRot ? pr[k] : e[k], two);
    int bj;
    acc += pair_term(e[k], pal, j1, two, bj);
    if (kIdx) idx |= (uint64_t)bj << (4 * k);
  }
  return (float)(se + acc);
}

// n texels from shared memory (multi-subset modes), texel ids in `tex`.
template <int kBits, bool kIdx>
__device__ __forceinline__ float qe_smem(const uint32_t *pts, int n, uint64_t tex, int se,
                                         uint4 *pal, uint32_t q1, uint32_t q2, uint64_t &idx) {
  constexpr int T = kLaneStride;
  const Proj pj = make_proj(q1, q2);
  int acc = 0;
  if (pj.L == 0) {
    const int sq = (int)__dp4a(q1, q1, 0u);
    for (int k = 0; k < n; k++) acc += sq - 2 * (int)__dp4a(pts[k * T], q1, 0u);
    return (float)(se + acc);
  }
  palette_sq<kBits>(q1, q2, pal);
#pragma unroll 4
  for (int k = 0; k < n; k++) {
    const uint32_t e = pts[k * T];
    bool two;
    const int j1 = nearest_pair<kBits>(pj, e, two);
    int bj;
    acc += pair_term(e, pal, j1, two, bj);
    if (kIdx) idx |= (uint64_t)bj << (4 * ((tex >> (4 * k)) & 15));
  }
  return (float)(se + acc);
}

}  // namespace fastc
