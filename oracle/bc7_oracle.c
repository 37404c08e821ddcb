/*
 * bc7_oracle.c -- CPU restatement of FasTC's BC7 (BPTC) encode path.
 *
 * TEST INFRASTRUCTURE ONLY (see bc7_oracle.h). Each function names the
 * reference function it restates, by file:line within the FasTC project.
 * Floating-point expressions keep the reference's operand order and its
 * float/double mix; the Makefile disables FMA contraction so that every
 * float operation rounds exactly as in the reference's x86-64 build.
 *
 * Reference files: BPTCEncoder/src/Compressor.cpp (CP),
 * BPTCEncoder/src/RGBAEndpoints.{h,cpp} (RE), BPTCEncoder/src/
 * CompressionMode.h (CM), BPTCEncoder/src/Decompressor.cpp (DC),
 * Base/include/FasTC/{VectorBase,MatrixSquare,MatrixBase,BitStream}.h.
 */
#define _POSIX_C_SOURCE 200809L
#include "bc7_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Format constants                                                          */
/* ------------------------------------------------------------------------ */

enum { PB_SHARED = 0, PB_UNIQUE = 1, PB_NONE = 2 };

/* BC7 mode table (CP:170-203). */
typedef struct {
  int part_bits, subsets, idx_bits, alpha_idx_bits, color_bits, alpha_bits;
  int has_rotation, has_idx_mode, pbit;
} mode_attr;

static const mode_attr kMode[8] = {
    {4, 3, 3, 0, 4, 0, 0, 0, PB_UNIQUE}, {6, 2, 3, 0, 6, 0, 0, 0, PB_SHARED},
    {6, 3, 2, 0, 5, 0, 0, 0, PB_NONE},   {6, 2, 2, 0, 7, 0, 0, 0, PB_UNIQUE},
    {0, 1, 2, 3, 5, 6, 1, 1, PB_NONE},   {0, 1, 2, 2, 7, 8, 1, 0, PB_NONE},
    {0, 1, 4, 0, 7, 7, 0, 0, PB_UNIQUE}, {6, 2, 2, 0, 5, 5, 0, 0, PB_UNIQUE},
};

/* BC7 interpolation weights of the second endpoint, for 2/3/4-bit indices
 * (CP:159-168 stores the pairs {64-w, w}). */
static const uint32_t kW2[4] = {0, 21, 43, 64};
static const uint32_t kW3[8] = {0, 9, 18, 27, 37, 46, 55, 64};
static const uint32_t kW4[16] = {0,  4,  9,  13, 17, 21, 26, 30,
                                 34, 38, 43, 47, 51, 55, 60, 64};

static uint32_t weight1(int bits, int j) {
  return bits == 2 ? kW2[j] : (bits == 3 ? kW3[j] : kW4[j]);
}

/* The reference's weight table rows are 16 entries wide and zero-padded
 * past 2^bits; its decoder can index the padding (see decode_block). */
static void weights_padded(int bits, uint32_t j, uint32_t *w0, uint32_t *w1) {
  if (j >= (1u << bits)) {
    *w0 = *w1 = 0;
    return;
  }
  *w1 = weight1(bits, (int)j);
  *w0 = 64 - *w1;
}

/* BC7 partition tables, one digit per texel (Shapes.h:24-53). */
static const char *kPart2[64] = {
    "0011001100110011", "0001000100010001", "0111011101110111", "0001001100110111",
    "0000000100010011", "0011011101111111", "0001001101111111", "0000000100110111",
    "0000000000010011", "0011011111111111", "0000000101111111", "0000000000010111",
    "0001011111111111", "0000000011111111", "0000111111111111", "0000000000001111",
    "0000100011101111", "0111000100000000", "0000000010001110", "0111001100010000",
    "0011000100000000", "0000100011001110", "0000000010001100", "0111001100110001",
    "0011000100010000", "0000100010001100", "0110011001100110", "0011011001101100",
    "0001011111101000", "0000111111110000", "0111000110001110", "0011100110011100",
    "0101010101010101", "0000111100001111", "0101101001011010", "0011001111001100",
    "0011110000111100", "0101010110101010", "0110100101101001", "0101101010100101",
    "0111001111001110", "0001001111001000", "0011001001001100", "0011101111011100",
    "0110100110010110", "0011110011000011", "0110011010011001", "0000011001100000",
    "0100111001000000", "0010011100100000", "0000001001110010", "0000010011100100",
    "0110110010010011", "0011011011001001", "0110001110011100", "0011100111000110",
    "0110110011001001", "0110001100111001", "0111111010000001", "0001100011100111",
    "0000111100110011", "0011001111110000", "0010001011101110", "0100010001110111",
};

static const char *kPart3[64] = {
    "0011001102212222", "0001001122112221", "0000200122112211", "0222002200110111",
    "0000000011221122", "0011001100220022", "0022002211111111", "0011001122112211",
    "0000000011112222", "0000111111112222", "0000111122222222", "0012001200120012",
    "0112011201120112", "0122012201220122", "0011011211221222", "0011200122002220",
    "0001001101121122", "0111001120012200", "0000112211221122", "0022002200221111",
    "0111011102220222", "0001000122212221", "0000001101220122", "0000110022102210",
    "0122012200110000", "0012001211222222", "0110122112210110", "0000011012211221",
    "0022110211020022", "0110011020022222", "0011012201220011", "0000200022112221",
    "0000000211221222", "0222002200120011", "0011001200220222", "0120012001200120",
    "0000111122220000", "0120120120120120", "0120201212010120", "0011220011220011",
    "0011112222000011", "0101010122222222", "0000000021212121", "0022112200221122",
    "0022001100220011", "0220122102201221", "0101222222220101", "0000212121212121",
    "0101010101012222", "0222011102220111", "0002111200021112", "0000211221122112",
    "0222011101110222", "0002111211120002", "0110011001102222", "0000000021122112",
    "0110011022222222", "0022001100110022", "0022112211220022", "0000000000002112",
    "0002000100020001", "0222122202221222", "0101222222222222", "0111201122012220",
};

/* Anchor texels of subsets 1 and 2 (AnchorTables.h:22-51). */
static const uint8_t kAnchor2[64] = {
    15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15,
    15, 2,  8,  2,  2,  8,  8,  15, 2,  8,  2,  2,  8,  8,  2,  2,
    15, 15, 6,  8,  2,  8,  15, 15, 2,  8,  2,  2,  2,  15, 15, 6,
    6,  2,  6,  8,  15, 15, 2,  2,  15, 15, 15, 15, 15, 2,  2,  15};
static const uint8_t kAnchor3a[64] = {
    3,  3,  15, 15, 8,  3,  15, 15, 8,  8,  6,  6,  6,  5,  3,  3,
    3,  3,  8,  15, 3,  3,  6,  10, 5,  8,  8,  6,  8,  5,  15, 15,
    8,  15, 3,  5,  6,  10, 8,  15, 15, 3,  15, 5,  15, 15, 15, 15,
    3,  15, 5,  5,  5,  8,  5,  10, 5,  10, 8,  13, 15, 12, 3,  3};
static const uint8_t kAnchor3b[64] = {
    15, 8,  8,  3,  15, 15, 3,  8,  15, 15, 15, 15, 15, 15, 15, 8,
    15, 8,  15, 3,  15, 8,  15, 8,  3,  15, 6,  10, 15, 15, 10, 8,
    15, 3,  15, 10, 10, 8,  9,  10, 6,  15, 8,  15, 3,  6,  6,  8,
    15, 3,  15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 3,  15, 15, 8};

/* Single-colour watermark alpha indices (CP:135-139), used verbatim because
 * they are part of the emitted bits. */
static const uint32_t kWatermark[9] = {0x32b92180, 0x32ba3080, 0x31103200,
                                       0x28103c80, 0x32bb3080, 0x25903600,
                                       0x3530b900, 0x3b32b180, 0x34b5b98};

static const int kPBits[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};

static int subset_of(int texel, int shape, int nsub) {
  if (nsub == 2) return kPart2[shape][texel] - '0';
  if (nsub == 3) return kPart3[shape][texel] - '0';
  return 0;
}

/* GetAnchorIndexForSubset (AnchorTables.h:55-83). */
static int anchor_of(int subset, int shape, int nsub) {
  if (subset == 1) return nsub == 2 ? kAnchor2[shape] : kAnchor3a[shape];
  if (subset == 2) return kAnchor3b[shape];
  return 0;
}

/* Optimal7CompressBC7Mode5 / Optimal6CompressDXT1, regenerated at first use
 * from the generator documented in BCLookupTables.h:44-95 / :355-449. */
static uint8_t gOpt7[256][2];
static uint8_t gOpt6[256][2][3];
static pthread_once_t gTablesOnce = PTHREAD_ONCE_INIT;

static void build_tables(void) {
  uint32_t vals[256];
  /* 7-bit endpoints, target = (43*a + 21*b + 32) >> 6 */
  {
    uint32_t n = 0, last = 0xFFFFFFFFu;
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t num = ((i >> 1) << 1) | (i >> 7);
      if (num != last) vals[n++] = last = num;
    }
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t best = 0xFFFFFFFFu, bj = 0, bk = 0;
      for (uint32_t j = 0; j < n; j++)
        for (uint32_t k = 0; k < n; k++) {
          uint32_t c = (43 * vals[j] + 21 * vals[k] + 32) >> 6;
          uint32_t d = i > c ? i - c : c - i;
          if (d < best) { best = d; bj = j; bk = k; }
        }
      gOpt7[i][0] = (uint8_t)(vals[bj] >> 1);
      gOpt7[i][1] = (uint8_t)(vals[bk] >> 1);
    }
  }
  /* 6-bit endpoints: best midpoint pair and best one-third pair */
  {
    uint32_t n = 0, last = 0xFFFFFFFFu;
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t num = ((i >> 2) << 2) | (i >> 6);
      if (num != last) vals[n++] = last = num;
    }
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t e[2][4] = {{1, 0, 0, 0xFFFFFFFFu}, {0, 0, 0, 0xFFFFFFFFu}};
      for (int kind = 0; kind < 2; kind++) {
        uint32_t best = 0xFFFFFFFFu, bj = 0, bk = 0;
        for (uint32_t j = 0; j < n; j++)
          for (uint32_t k = j; k < n; k++) {
            uint32_t c = kind == 0 ? (vals[j] + vals[k]) / 2
                                   : (2 * vals[j] + vals[k]) / 3;
            uint32_t d = i > c ? i - c : c - i;
            if (d < best) { best = d; bj = j; bk = k; }
          }
        e[kind][1] = vals[bj];
        e[kind][2] = vals[bk];
        e[kind][3] = best;
      }
      int first = e[1][3] > e[0][3] ? 0 : 1;
      for (int s = 0; s < 2; s++) {
        int k = s == 0 ? first : 1 - first;
        gOpt6[i][s][0] = (uint8_t)e[k][0];
        gOpt6[i][s][1] = (uint8_t)(e[k][1] >> 2);
        gOpt6[i][s][2] = (uint8_t)(e[k][2] >> 2);
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Vector helpers (VectorBase.h:96-112: sequential Dot, Length, Normalize)    */
/* ------------------------------------------------------------------------ */

static float dot4(const float *a, const float *b) {
  float s = 0.0f;
  for (int i = 0; i < 4; i++) s += a[i] * b[i];
  return s;
}

/* sqrt of the long-double-widened value rounded back to float equals the
 * correctly rounded sqrtf. */
static float length4(const float *a) { return sqrtf(dot4(a, a)); }

static void normalize4(float *a) {
  float len = length4(a);
  for (int i = 0; i < 4; i++) a[i] /= len;
}

static int eq4(const float *a, const float *b) {
  return a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3];
}

static float fmin_std(float a, float b) { return (b < a) ? b : a; } /* std::min */
static float fmax_std(float a, float b) { return (a < b) ? b : a; } /* std::max */

/* ------------------------------------------------------------------------ */
/* Quantisation (RE:126-177, CM:212-250)                                     */
/* ------------------------------------------------------------------------ */

static uint8_t sad8(uint8_t a, uint8_t b) { return a > b ? a - b : b - a; }

static uint32_t popc8(uint32_t m) {
  uint32_t c = 0;
  for (; m; m &= m - 1) c++;
  return c;
}

/* QuantizeChannel (RE:126-165). */
static uint8_t quantize_channel(uint8_t val, uint8_t mask, int pbit) {
  if (mask == 0xFF) return val;
  if (mask == 0) return 0xFF;
  uint32_t prec = popc8(mask);
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
  return sad8(val, (uint8_t)lval) < sad8(val, (uint8_t)hval) ? (uint8_t)lval
                                                             : (uint8_t)hval;
}

/* uint32(x + 0.5) with x a float widened to double, as the x86-64 build
 * converts it (through a signed 64-bit truncation). */
static uint32_t round_half_up(float x) {
  double d = (double)x + 0.5;
  if (d != d) return 0;
  return (uint32_t)(int64_t)d;
}

/* RGBAVector::ToPixel (RE:167-177). */
static uint32_t to_pixel(const float *v, uint32_t mask, int pbit) {
  uint32_t r = 0;
  for (int c = 0; c < 4; c++) {
    uint8_t q = quantize_channel((uint8_t)(round_half_up(v[c]) & 0xFF),
                                 (uint8_t)((mask >> (8 * c)) & 0xFF), pbit);
    r |= (uint32_t)q << (8 * c);
  }
  return r;
}

static void pixel_to_vec(uint32_t px, float *v) {
  for (int c = 0; c < 4; c++) v[c] = (float)((px >> (8 * c)) & 0xFF);
}

/* ------------------------------------------------------------------------ */
/* Mode context: the state of one CompressionMode object (CM:62-101)          */
/* ------------------------------------------------------------------------ */

typedef struct {
  int mode;
  const mode_attr *a;
  int steps;
  int metric;
  int rot;      /* m_RotateMode */
  int idx_mode; /* m_IndexMode */
  int exp_mode;
  uint32_t *lcg; /* annealing RNG state */
} mode_ctx;

static const float kMetricNonuniform[4] = {0.0f, 0.0f, 0.0f, 1.0f};
static float gMetricW[2][4];
static pthread_once_t gMetricOnce = PTHREAD_ONCE_INIT;
static void build_metric(void) {
  /* kErrorMetrics (CP:205-208) */
  for (int i = 0; i < 4; i++) gMetricW[0][i] = 1.0f;
  gMetricW[1][0] = sqrtf(0.3f);
  gMetricW[1][1] = sqrtf(0.56f);
  gMetricW[1][2] = sqrtf(0.11f);
  gMetricW[1][3] = kMetricNonuniform[3];
}

static int rotation_of(const mode_ctx *m) { return m->a->has_rotation ? m->rot : 0; }

/* GetNumberOfBitsPerIndex / GetNumberOfBitsPerAlpha (CM:151-165). */
static int bits_index(const mode_ctx *m, int idx_mode) {
  if (idx_mode < 0) idx_mode = m->idx_mode;
  return idx_mode == 0 ? m->a->idx_bits : m->a->alpha_idx_bits;
}
static int bits_alpha(const mode_ctx *m, int idx_mode) {
  if (idx_mode < 0) idx_mode = m->idx_mode;
  return idx_mode == 0 ? m->a->alpha_idx_bits : m->a->idx_bits;
}

/* GetErrorMetric with the rotation permutation (CM:196-205). */
static void metric_of(const mode_ctx *m, float *w) {
  const float *b = gMetricW[m->metric];
  w[0] = b[0]; w[1] = b[1]; w[2] = b[2]; w[3] = b[3];
  switch (rotation_of(m)) {
    case 1: w[0] = b[3]; w[3] = b[0]; break;
    case 2: w[1] = b[3]; w[3] = b[1]; break;
    case 3: w[2] = b[3]; w[3] = b[2]; break;
    default: break;
  }
}

/* GetQuantizationMask (CM:212-232). */
static uint32_t qmask_of(const mode_ctx *m) {
  uint32_t cm = (0xFFu << (8 - m->a->color_bits)) & 0xFFu;
  uint32_t am = m->a->alpha_bits ? (0xFFu << (8 - m->a->alpha_bits)) & 0xFFu : 0;
  return cm | (cm << 8) | (cm << 16) | (am << 24);
}

static int num_pbit_combos(const mode_ctx *m) {
  return m->a->pbit == PB_SHARED ? 2 : (m->a->pbit == PB_UNIQUE ? 4 : 1);
}

/* GetPBitCombo (CM:243-250). */
static const int *pbit_combo(const mode_ctx *m, int idx) {
  if (m->a->pbit == PB_SHARED) return idx ? kPBits[3] : kPBits[0];
  if (m->a->pbit == PB_UNIQUE) return kPBits[idx % 4];
  return kPBits[0];
}

/* ------------------------------------------------------------------------ */
/* Clusters (RE:104-227)                                                     */
/* ------------------------------------------------------------------------ */

typedef struct {
  int n;
  float pt[16][4];  /* GetPoint order */
  uint32_t px[16];  /* GetPixel: the texel as loaded, never rotated */
  float avg[4], mn[4], mx[4];
} cluster;

/* RGBACluster ctor + SetPartition/Recalculate (RE:108-127, 205-226). */
static void make_cluster(const uint32_t block[16], int shape, int nsub,
                         int subset, cluster *c) {
  c->n = 0;
  for (int k = 0; k < 4; k++) {
    c->avg[k] = 0.0f;
    c->mn[k] = FLT_MAX;
    c->mx[k] = -FLT_MAX;
  }
  for (int i = 0; i < 16; i++) {
    if (subset_of(i, shape, nsub) != subset) continue;
    float *p = c->pt[c->n];
    pixel_to_vec(block[i], p);
    c->px[c->n] = block[i];
    for (int k = 0; k < 4; k++) c->avg[k] += p[k];
    for (int k = 0; k < 4; k++) {
      c->mn[k] = fmin_std(p[k], c->mn[k]);
      c->mx[k] = fmax_std(p[k], c->mx[k]);
    }
    c->n++;
  }
  for (int k = 0; k < 4; k++) c->avg[k] /= (float)c->n;
}

static int all_same_point(const cluster *c) { return eq4(c->mx, c->mn); }

/* Work counters (diagnostic): QuantizedError calls and texel-bucket
 * evaluations (one per palette entry tried for a texel), summed over all
 * threads. */
static uint64_t g_qe_calls, g_qe_evals;
void bc7o_qe_counters(uint64_t out[2], int reset) {
  out[0] = __atomic_load_n(&g_qe_calls, __ATOMIC_RELAXED);
  out[1] = __atomic_load_n(&g_qe_evals, __ATOMIC_RELAXED);
  if (reset) {
    __atomic_store_n(&g_qe_calls, 0, __ATOMIC_RELAXED);
    __atomic_store_n(&g_qe_evals, 0, __ATOMIC_RELAXED);
  }
}

static float quantized_error_body(const cluster *c, const float *p1, const float *p2,
                                  int nbuckets, uint32_t mask, const float *metric,
                                  const int *pbits, uint8_t *indices, uint64_t *evals);

/* RGBACluster::QuantizedError<nBuckets> (RE:190-310). */
static float quantized_error(const cluster *c, const float *p1,
                             const float *p2, int nbuckets, uint32_t mask,
                             const float *metric, const int *pbits,
                             uint8_t *indices) {
  uint64_t evals = 0;
  const float e = quantized_error_body(c, p1, p2, nbuckets, mask, metric, pbits, indices, &evals);
  __atomic_fetch_add(&g_qe_calls, 1, __ATOMIC_RELAXED);
  __atomic_fetch_add(&g_qe_evals, evals, __ATOMIC_RELAXED);
  return e;
}

static float quantized_error_body(const cluster *c, const float *p1, const float *p2,
                                  int nbuckets, uint32_t mask, const float *metric,
                                  const int *pbits, uint8_t *indices, uint64_t *evals) {
  const int prec = nbuckets == 4 ? 2 : (nbuckets == 8 ? 3 : 4);
  uint32_t qp1 = pbits ? to_pixel(p1, mask, pbits[0]) : to_pixel(p1, mask, -1);
  uint32_t qp2 = pbits ? to_pixel(p2, mask, pbits[1]) : to_pixel(p2, mask, -1);
  float u1[4], u2[4], d[4], dir[4];
  pixel_to_vec(qp1, u1);
  pixel_to_vec(qp2, u2);
  for (int k = 0; k < 4; k++) {
    d[k] = u1[k] - u2[k];
    dir[k] = u2[k] - u1[k];
  }
  const float lsq = dot4(d, d);
  float total = 0.0f;
  if (lsq == 0) {
    for (int i = 0; i < c->n; i++) {
      float ev[4];
      for (int k = 0; k < 4; k++) {
        uint32_t a = (qp1 >> (8 * k)) & 0xFF;
        uint32_t ip = ((a * 64 + 32) >> 6) & 0xFF;
        uint8_t dist = sad8((uint8_t)((c->px[i] >> (8 * k)) & 0xFF), (uint8_t)ip);
        ev[k] = (float)dist * metric[k];
      }
      total += dot4(ev, ev);
      if (indices) indices[i] = 0;
    }
    *evals += (uint64_t)c->n;
    return total;
  }
  for (int i = 0; i < c->n; i++) {
    float t[4];
    for (int k = 0; k < 4; k++) t[k] = c->pt[i][k] - u1[k];
    const float pct = dot4(t, dir) / lsq;
    const float scaled = pct * (float)(nbuckets - 1);
    int j1 = (int)floor((double)scaled);
    int j2 = (int)ceil((double)scaled);
    j1 = j1 < 0 ? 0 : j1;
    j1 = j1 > nbuckets - 1 ? nbuckets - 1 : j1;
    j2 = j2 > nbuckets - 1 ? nbuckets - 1 : j2;
    float min_err = FLT_MAX;
    uint8_t best = 0;
    int j = j1;
    do {
      ++*evals;
      const uint32_t w1 = weight1(prec, j), w0 = 64 - w1;
      float ev[4];
      for (int k = 0; k < 4; k++) {
        uint32_t a = (qp1 >> (8 * k)) & 0xFF, b = (qp2 >> (8 * k)) & 0xFF;
        uint32_t ip = ((a * w0 + b * w1 + 32) >> 6) & 0xFF;
        uint8_t dist = sad8((uint8_t)((c->px[i] >> (8 * k)) & 0xFF), (uint8_t)ip);
        ev[k] = (float)dist * metric[k];
      }
      float err = dot4(ev, ev);
      if (err < min_err) {
        min_err = err;
        best = (uint8_t)j;
      } else if (err > min_err) {
        break;
      }
    } while (++j <= j2);
    total += min_err;
    if (indices) indices[i] = best;
  }
  return total;
}

/* ------------------------------------------------------------------------ */
/* Principal axis (RE:327-428) and PowerMethod (MatrixSquare.h:44-105)        */
/* ------------------------------------------------------------------------ */

static void power_method(const float m[4][4], float *out) {
  float b[4] = {0.5f, 0.5f, 0.5f, 0.5f}; /* 1/sqrt(4) */
  int bad = 0, fixed = 0, iters = 0;
  while (!fixed && ++iters < 5) {
    float nb[4];
    for (int j = 0; j < 4; j++) {
      float s = 0.0f;
      for (int i = 0; i < 4; i++) s += m[j][i] * b[i];
      nb[j] = s;
    }
    const float len = length4(nb);
    if ((double)len < 1e-10) {
      if (bad) {
        memcpy(out, b, sizeof(b));
        return;
      }
      b[0] = b[1] = 1.0f;
      normalize4(b);
      bad = 1;
      continue;
    }
    normalize4(nb);
    if (fabs((double)(1.0f - dot4(b, nb))) < 1e-8) fixed = 1;
    memcpy(b, nb, sizeof(b));
  }
  memcpy(out, b, sizeof(b));
}

static void principal_axis(const cluster *c, float *axis) {
  float to_pts[16][4];
  for (int i = 0; i < c->n; i++)
    for (int k = 0; k < 4; k++) to_pts[i][k] = c->pt[i][k] - c->avg[k];

  /* unique points; unused slots keep RGBAVector's default (-1,-1,-1,-1) */
  float upts[16][4];
  for (int i = 0; i < 16; i++)
    for (int k = 0; k < 4; k++) upts[i][k] = -1.0f;
  int nu = 0;
  for (int i = 0; i < c->n; i++) {
    int has = 0;
    for (int j = 0; j < nu; j++)
      if (eq4(upts[j], c->pt[i])) has = 1;
    if (!has) memcpy(upts[nu++], c->pt[i], sizeof(upts[0]));
  }
  if (nu == 1) {
    axis[0] = axis[1] = axis[2] = axis[3] = 0.0f;
    return;
  }
  float dir[4];
  for (int k = 0; k < 4; k++) dir[k] = upts[1][k] - upts[0][k];
  normalize4(dir);
  int collinear = 1;
  /* the bound is the cluster's point count, not the unique count */
  for (int i = 2; i < c->n; i++) {
    float v[4];
    for (int k = 0; k < 4; k++) v[k] = upts[i][k] - upts[0][k];
    if (fabs(fabs((double)dot4(v, dir)) - (double)length4(v)) > 1e-7) {
      collinear = 0;
      break;
    }
  }
  if (collinear) {
    memcpy(axis, dir, sizeof(dir));
    return;
  }
  float cov[4][4];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j <= i; j++) {
      float s = 0.0f;
      for (int k = 0; k < c->n; k++) s += to_pts[k][i] * to_pts[k][j];
      cov[i][j] = s / 3.0f;
      cov[j][i] = cov[i][j];
    }
  power_method((const float(*)[4])cov, axis);
}

/* ------------------------------------------------------------------------ */
/* RNG and acceptance (CP:358-362, 506-536)                                  */
/* ------------------------------------------------------------------------ */

/* fastrand (CP:358-362) masks with RAND_MAX, which glibc defines as
 * 0x7FFFFFFF: the value is the full top 16 bits of the state. The
 * reference's COMPILE_ASSERT(RAND_MAX == 0x7FFF) (CP:521) declares a
 * zero-length array under gcc instead of failing. */
static uint32_t lcg_next(uint32_t *s) {
  *s = 214013u * *s + 2531011u;
  return *s >> 16;
}

static uint64_t mix64(uint64_t z) { /* splitmix64 finaliser */
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

uint32_t bc7o_fit_seed(uint32_t seed, uint32_t bx, uint32_t by, uint32_t fit) {
  uint64_t k = mix64(((uint64_t)bx << 32) | by);
  k = mix64(k + (uint64_t)seed * 0x9E3779B97F4A7C15ull + fit);
  return (uint32_t)(k >> 32);
}

/* exp for x <= 0 from Cephes expf (S. L. Moshier): Cody-Waite reduction by
 * ln 2 in two parts, degree-5 polynomial, exact scaling by 2^n. Only +, *,
 * floor and bit construction, so the GPU reproduces it bit for bit. */
float bc7o_expf(float x) {
  if (x != x) return x;
  if (x > 0.0f) x = 0.0f; /* only the non-positive branch is used */
  if (x < -103.0f) return 0.0f;
  const float fn = floorf(x * 1.44269504088896341f + 0.5f);
  float r = x - fn * 0.693359375f;
  r = r - fn * -2.12194440e-4f;
  const float z = r * r;
  float p = 1.9875691500e-4f;
  p = p * r + 1.3981999507e-3f;
  p = p * r + 8.3334519073e-3f;
  p = p * r + 4.1665795894e-2f;
  p = p * r + 1.6666665459e-1f;
  p = p * r + 5.0000001201e-1f;
  p = p * z + r + 1.0f;
  int n = (int)fn;
  union { uint32_t u; float f; } s;
  if (n < -125) {
    s.u = (uint32_t)(127 - 64) << 23;
    p *= s.f;
    n += 64;
  }
  s.u = (uint32_t)(n + 127) << 23;
  return p * s.f;
}

/* AcceptNewEndpointError (CP:524-536). The draw happens whenever the new
 * error is not strictly better, as in the reference. */
static int accept_error(const mode_ctx *m, float new_err, float old_err,
                        float temp) {
  if (new_err < old_err) return 1;
  /* frand (CP:506-519): with a 16-bit draw, bit 15 lands in the float's
   * exponent and r falls in [1, 3), which no p <= 1 accepts. */
  const uint32_t r16 = lcg_next(m->lcg) & 0xFFFF;
  const uint32_t mant = (r16 << 8) | (r16 >> 7);
  union { uint32_t u; float f; } fu;
  fu.u = (127u << 23) | mant;
  const float r = fu.f - 1.0f;
  if (m->exp_mode == BC7O_EXP_LIBM) {
    const double p =
        exp((0.1f * ((double)old_err - (double)new_err)) / (double)temp);
    return (double)r < p;
  }
  if (r >= 1.0f) return 0;
  const float x = (0.1f * (old_err - new_err)) / temp;
  if (mant == 0) return x > -745.0f; /* r == 0 accepts any p > 0 */
  return r < bc7o_expf(x);
}

/* ------------------------------------------------------------------------ */
/* Endpoint fitting                                                          */
/* ------------------------------------------------------------------------ */

static void clamp_endpoints(float *p1, float *p2) { /* RE:436-441 */
  for (int k = 0; k < 4; k++) {
    p1[k] = p1[k] < 0.0f ? 0.0f : (p1[k] > 255.0f ? 255.0f : p1[k]);
    p2[k] = p2[k] < 0.0f ? 0.0f : (p2[k] > 255.0f ? 255.0f : p2[k]);
  }
}

/* ClampEndpointsToGrid (CP:212-250). */
static void clamp_to_grid(const mode_ctx *m, float *p1, float *p2,
                          uint8_t *best_pbit) {
  const int nc = num_pbit_combos(m);
  const uint32_t qm = qmask_of(m);
  clamp_endpoints(p1, p2);
  float min_dist = FLT_MAX;
  float b1[4] = {-1, -1, -1, -1}, b2[4] = {-1, -1, -1, -1};
  for (int i = 0; i < nc; i++) {
    uint32_t q1, q2;
    if (nc > 1) {
      q1 = to_pixel(p1, qm, pbit_combo(m, i)[0]);
      q2 = to_pixel(p2, qm, pbit_combo(m, i)[1]);
    } else {
      q1 = to_pixel(p1, qm, -1);
      q2 = to_pixel(p2, qm, -1);
    }
    float n1[4], n2[4], d1[4], d2[4];
    pixel_to_vec(q1, n1);
    pixel_to_vec(q2, n2);
    for (int k = 0; k < 4; k++) {
      d1[k] = n1[k] - p1[k];
      d2[k] = n2[k] - p2[k];
    }
    const float dist = dot4(d1, d1) + dot4(d2, d2);
    if (dist < min_dist) {
      min_dist = dist;
      memcpy(b1, n1, sizeof(b1));
      memcpy(b2, n2, sizeof(b2));
      *best_pbit = (uint8_t)i;
    }
  }
  memcpy(p1, b1, sizeof(b1));
  memcpy(p2, b2, sizeof(b2));
}

/* CompressSingleColor (CP:252-353). */
static float single_color(const mode_ctx *m, const float *p, float *p1,
                          float *p2, uint8_t *best_pbit) {
  const uint32_t pixel = to_pixel(p, 0xFFFFFFFFu, -1);
  float best_err = FLT_MAX;
  for (int pbi = 0; pbi < num_pbit_combos(m); pbi++) {
    const int *combo = pbit_combo(m, pbi);
    uint32_t dist[4] = {0, 0, 0, 0};
    uint32_t bi[4], bj[4];
    memset(bi, 0xFF, sizeof(bi));
    memset(bj, 0xFF, sizeof(bj));
    for (int ci = 0; ci < 4; ci++) {
      const uint32_t val = (pixel >> (ci * 8)) & 0xFF;
      int nbits = ci == 3 ? m->a->alpha_bits : m->a->color_bits;
      if (nbits == 0) {
        bi[ci] = bj[ci] = 0xFF;
        dist[ci] = dist[ci] > 0xFF - val ? dist[ci] : 0xFF - val;
        continue;
      }
      const int nposs = 1 << nbits;
      int hv[256], lv[256];
      const int havepbit = m->a->pbit != PB_NONE;
      if (havepbit) nbits++;
      for (int i = 0; i < nposs; i++) {
        int vh = i, vl = i;
        if (havepbit) {
          vh = (vh << 1) | combo[1];
          vl = (vl << 1) | combo[0];
        }
        hv[i] = vh << (8 - nbits);
        hv[i] |= hv[i] >> nbits;
        lv[i] = vl << (8 - nbits);
        lv[i] |= lv[i] >> nbits;
      }
      const int bits = bits_index(m, -1);
      const uint32_t w1 = weight1(bits, 1), w0 = 64 - w1;
      uint32_t bestd = 0xFF;
      for (int i = 0; bestd > 0 && i < nposs; i++)
        for (int j = 0; bestd > 0 && j < nposs; j++) {
          const uint32_t v1 = (uint32_t)lv[i], v2 = (uint32_t)hv[j];
          const uint32_t cmb = (w0 * v1 + w1 * v2 + 32) >> 6;
          const uint32_t e = cmb > val ? cmb - val : val - cmb;
          if (e < bestd) {
            bestd = e;
            bi[ci] = v1;
            bj[ci] = v2;
          }
        }
      dist[ci] = bestd > dist[ci] ? bestd : dist[ci];
    }
    const float *w = gMetricW[m->metric];
    float err = 0.0f;
    for (int i = 0; i < 4; i++) {
      const float e = (float)dist[i] * w[i];
      err += e * e;
    }
    if (err < best_err) {
      best_err = err;
      *best_pbit = (uint8_t)pbi;
      for (int ci = 0; ci < 4; ci++) {
        p1[ci] = (float)bi[ci];
        p2[ci] = (float)bj[ci];
      }
    }
  }
  return best_err;
}

/* PickBestNeighboringEndpoints (CP:426-498). */
static void pick_neighbor(const mode_ctx *m, const float *p1, const float *p2,
                          int cur_pbit, float *np1, float *np2, int *npbit,
                          const float *vis1, const float *vis2, int vis_pbit) {
  float step[4];
  const float cs = 1.0f * (float)(1 << (8 - m->a->color_bits));
  step[0] = step[1] = step[2] = cs;
  step[3] = 1.0f * (float)(1 << (8 - m->a->alpha_bits));
  if (m->mode < 4) step[(rotation_of(m) + 3) % 4] = 0.0f; /* m_IsOpaque */
  const int has_pbits = m->a->pbit != PB_NONE;
  if (has_pbits) *npbit = m->a->pbit == PB_SHARED ? (cur_pbit + 1) % 2 : 3 - cur_pbit;
  int visited = 1, guard = -1;
  while (visited && ++guard < 16) {
    for (int pt = 0; pt < 2; pt++) {
      const float *p = pt ? p1 : p2;
      float *np = pt ? np1 : np2;
      memcpy(np, p, 4 * sizeof(float));
      const uint32_t dir = lcg_next(m->lcg) % 16;
      if (has_pbits) {
        const int old = pbit_combo(m, cur_pbit)[pt];
        for (int k = 0; k < 4; k++) {
          const int down = (dir >> k) & 1;
          if (down && old == 0) np[k] -= step[k];
          else if (!down && old == 1) np[k] += step[k];
        }
      } else {
        for (int k = 0; k < 4; k++) {
          if ((dir >> k) & 1) np[k] -= step[k];
          else np[k] += step[k];
        }
      }
      for (int k = 0; k < 4; k++) np[k] = fmin_std(fmax_std(np[k], 0.0f), 255.0f);
    }
    visited = eq4(vis1, np1) && eq4(vis2, np2) && vis_pbit == *npbit;
  }
}

/* OptimizeEndpointsForCluster (CP:538-630). Indices are in point order. */
/* Diagnostic trace of one block's cluster fits (bc7o_trace_block only):
 * where the fit being computed records its setup error (the QuantizedError
 * the annealing starts from) and, for the rotation modes, its alpha error.
 * Set only while bc7o_trace_block runs, on its own thread. */
typedef struct {
  double init, aerr;
  int annealed; /* reached the QuantizedError path (not a single-colour shortcut) */
} fit_note;
static __thread fit_note *g_note;
static __thread bc7o_fit_trace *g_trace;
static __thread int g_ntrace, g_trace_cap;

static float optimize_endpoints(const mode_ctx *m, const cluster *c, float *p1,
                                float *p2, uint8_t *best_idx,
                                uint8_t *best_pbit) {
  const int nb = 1 << bits_index(m, -1);
  const uint32_t qm = qmask_of(m);
  float metric[4];
  metric_of(m, metric);
  float cur_err = quantized_error(c, p1, p2, nb, qm, metric,
                                  pbit_combo(m, *best_pbit), best_idx);
  if (g_note) {
    g_note->init = cur_err;
    g_note->annealed = 1;
  }
  int cur_pbit = *best_pbit;
  float best_err = cur_err;
  uint32_t q1, q2;
  if (m->a->pbit != PB_NONE) {
    q1 = to_pixel(p1, qm, pbit_combo(m, *best_pbit)[0]);
    q2 = to_pixel(p2, qm, pbit_combo(m, *best_pbit)[1]);
  } else {
    q1 = to_pixel(p1, qm, -1);
    q2 = to_pixel(p2, qm, -1);
  }
  pixel_to_vec(q1, p1);
  pixel_to_vec(q2, p2);
  float bp1[4], bp2[4];
  memcpy(bp1, p1, sizeof(bp1));
  memcpy(bp2, p2, sizeof(bp2));
  float vis1[4], vis2[4];
  int vis_pbit = cur_pbit;
  memcpy(vis1, p1, sizeof(vis1));
  memcpy(vis2, p2, sizeof(vis2));
  const int max_energy = m->steps;
  for (int energy = 0; best_err > 0 && energy < max_energy; energy++) {
    const float temp = (float)energy / (float)(max_energy - 1);
    uint8_t idx[16];
    float np1[4], np2[4];
    int npbit = 0;
    pick_neighbor(m, p1, p2, cur_pbit, np1, np2, &npbit, vis1, vis2, vis_pbit);
    const float err = quantized_error(c, np1, np2, nb, qm, metric,
                                      pbit_combo(m, npbit), idx);
    if (accept_error(m, err, cur_err, temp)) {
      cur_err = err;
      memcpy(p1, np1, sizeof(np1));
      memcpy(p2, np2, sizeof(np2));
      cur_pbit = npbit;
    }
    if (err < best_err) {
      memcpy(best_idx, idx, sizeof(idx));
      memcpy(bp1, np1, sizeof(bp1));
      memcpy(bp2, np2, sizeof(bp2));
      *best_pbit = (uint8_t)npbit;
      best_err = err;
      memcpy(vis1, np1, sizeof(vis1));
      memcpy(vis2, np2, sizeof(vis2));
      vis_pbit = npbit;
      energy = 0;
    }
  }
  memcpy(p1, bp1, sizeof(bp1));
  memcpy(p2, bp2, sizeof(bp2));
  return best_err;
}

/* CompressionMode::CompressCluster, colour version (CP:921-1094). */
static double fit_rgb(const mode_ctx *m, const cluster *c, float *p1,
                      float *p2, uint8_t *idx, uint8_t *pbit) {
  if (all_same_point(c)) {
    const double e = single_color(m, c->pt[0], p1, p2, pbit);
    for (int i = 0; i < c->n; i++) idx[i] = 1;
    return (double)c->n * e;
  }
  const int nb = 1 << bits_index(m, -1);
  float axis[4];
  principal_axis(c, axis);
  float mindp = FLT_MAX, maxdp = -FLT_MAX;
  for (int i = 0; i < c->n; i++) {
    float t[4];
    for (int k = 0; k < 4; k++) t[k] = c->pt[i][k] - c->avg[k];
    const float dp = dot4(t, axis);
    if (dp < mindp) mindp = dp;
    if (dp > maxdp) maxdp = dp;
  }
  for (int k = 0; k < 4; k++) {
    p1[k] = c->avg[k] + axis[k] * mindp;
    p2[k] = c->avg[k] + axis[k] * maxdp;
  }
  clamp_endpoints(p1, p2);

  float pts[16][4];
  uint32_t npts[16];
  for (int i = 0; i < nb; i++) {
    const float s = (float)i / (float)(nb - 1);
    for (int k = 0; k < 4; k++) pts[i][k] = p1[k] * (1.0f - s) + p2[k] * s;
  }
  uint32_t bidx[16] = {0};
  int fixed = 0;
  while (!fixed) {
    float newp[16][4];
    for (int i = 0; i < c->n; i++) {
      int minb = -1;
      float mind = FLT_MAX;
      for (int j = 0; j < nb; j++) {
        float v[4];
        for (int k = 0; k < 4; k++) v[k] = c->pt[i][k] - pts[j][k];
        const float d = dot4(v, v);
        if (d < mind) {
          mind = d;
          minb = j;
        }
      }
      bidx[i] = (uint32_t)minb;
    }
    for (int i = 0; i < nb; i++) {
      npts[i] = 0;
      for (int k = 0; k < 4; k++) newp[i][k] = 0.0f;
      for (int j = 0; j < c->n; j++) {
        if (bidx[j] == (uint32_t)i) {
          npts[i]++;
          for (int k = 0; k < 4; k++) newp[i][k] += c->pt[j][k];
        }
      }
      if (npts[i] != 0)
        for (int k = 0; k < 4; k++) newp[i][k] /= (float)npts[i];
    }
    fixed = 1;
    for (int i = 0; i < nb; i++)
      if (!eq4(pts[i], newp[i])) fixed = 0;
    memcpy(pts, newp, (size_t)nb * sizeof(pts[0]));
  }
  int filled = 0, last = -1;
  for (int i = 0; i < nb; i++)
    if (npts[i] > 0) {
      filled++;
      last = i;
    }
  if (filled == 1) {
    const double e = single_color(m, pts[last], p1, p2, pbit);
    for (int i = 0; i < c->n; i++) idx[i] = 1;
    return (double)c->n * e;
  }
  float asq = 0.0f, bsq = 0.0f, ab = 0.0f, ax[4] = {0, 0, 0, 0},
        bx[4] = {0, 0, 0, 0};
  for (int i = 0; i < nb; i++) {
    const float fbi = (float)(nb - 1 - i), fb = (float)(nb - 1), fi = (float)i;
    const float fn = (float)(int)npts[i];
    const float a = fbi / fb, b = fi / fb;
    asq += fn * a * a;
    bsq += fn * b * b;
    ab += fn * a * b;
    for (int k = 0; k < 4; k++) {
      ax[k] += pts[i][k] * a * fn;
      bx[k] += pts[i][k] * b * fn;
    }
  }
  const float f = 1.0f / (asq * bsq - ab * ab);
  for (int k = 0; k < 4; k++) {
    p1[k] = (ax[k] * bsq - bx[k] * ab) * f;
    p2[k] = (bx[k] * asq - ax[k] * ab) * f;
  }
  clamp_to_grid(m, p1, p2, pbit);
  return optimize_endpoints(m, c, p1, p2, idx, pbit);
}

/* CompressionMode::CompressCluster, separate-alpha version (CP:632-919). */
static double fit_alpha(const mode_ctx *m, const cluster *c, float *p1,
                        float *p2, uint8_t *idx, uint8_t *aidx) {
  if (all_same_point(c)) {
    uint8_t dummy = 0;
    const double e = single_color(m, c->pt[0], p1, p2, &dummy);
    for (int i = 0; i < c->n; i++) idx[i] = aidx[i] = 1;
    return (double)c->n * e;
  }
  /* a copy whose avg/min/max and pixels stay those of the unrotated block */
  cluster rgb = *c;
  float avals[16] = {0};
  float amin = FLT_MAX, amax = -FLT_MAX;
  for (int i = 0; i < rgb.n; i++) {
    float *v = rgb.pt[i];
    const int r = rotation_of(m);
    if (r >= 1 && r <= 3) {
      const float t = v[r - 1];
      v[r - 1] = v[3];
      v[3] = t;
    }
    avals[i] = v[3];
    v[3] = 255.0f;
    amin = fmin_std(avals[i], amin);
    amax = fmax_std(avals[i], amax);
  }
  uint8_t dummy = 0;
  float rp1[4], rp2[4];
  const double rgb_err = fit_rgb(m, &rgb, rp1, rp2, idx, &dummy);

  float a1 = amin, a2 = amax;
  double aerr = DBL_MAX;
  const int abits = bits_alpha(m, -1);
  float metric[4];
  metric_of(m, metric);
  const float wa = metric[3];
  const int nb = 1 << abits;
  if (a1 == a2) {
    const uint8_t a1be = (uint8_t)a1, a2be = (uint8_t)a2;
    if (m->mode == 5) {
      for (int i = 0; i < 16; i++) aidx[i] = 0;
      aerr = 0.0;
    } else {
      if (gOpt6[a1be][0][0]) {
        a1 = (float)((gOpt6[a1be][1][1] << 2) | (gOpt6[a1be][0][1] >> 4));
        a2 = (float)((gOpt6[a2be][1][2] << 2) | (gOpt6[a2be][0][1] >> 4));
      } else {
        a1 = (float)((gOpt6[a1be][0][1] << 2) | (gOpt6[a1be][0][1] >> 4));
        a2 = (float)((gOpt6[a2be][0][2] << 2) | (gOpt6[a2be][0][1] >> 4));
      }
      const uint8_t ai = m->idx_mode == 1 ? 1 : 2;
      for (int i = 0; i < 16; i++) aidx[i] = ai;
      const uint32_t w1 = weight1(abits, ai), w0 = 64 - w1;
      const uint32_t a1i = (uint32_t)a1, a2i = (uint32_t)a2;
      const uint8_t ip = (uint8_t)(((a1i * w0) + (a2i * w1) + 32) >> 6);
      float pe = wa * (float)(a1be > ip ? a1be - ip : ip - a1be);
      pe *= pe;
      aerr = 16 * pe;
    }
  } else {
    float vals[8] = {0};
    uint32_t bk[16] = {0};
    for (int i = 0; i < nb; i++) {
      const float fi = (float)i, fb = (float)(nb - 1);
      vals[i] = amin + (fi / fb) * (amax - amin);
    }
    for (int i = 0; i < 16; i++) {
      float md = 255.0f;
      for (int j = 0; j < nb; j++) {
        const float d = (float)fabs((double)(avals[i] - vals[j]));
        if (d < md) {
          md = d;
          bk[i] = (uint32_t)j;
        }
      }
    }
    float npts[8];
    int fixed = 0;
    while (!fixed) {
      float avg[8] = {0};
      memset(npts, 0, sizeof(npts));
      for (int i = 0; i < nb; i++) {
        for (int j = 0; j < 16; j++)
          if (bk[j] == (uint32_t)i) {
            avg[i] += avals[j];
            npts[i] += 1.0f;
          }
        if (npts[i] > 0.0f) avg[i] /= npts[i];
      }
      fixed = 1;
      for (int i = 0; i < nb; i++) fixed = fixed && (avg[i] == vals[i]);
      memcpy(vals, avg, sizeof(vals));
      for (int i = 0; i < 16; i++) {
        float md = 255.0f;
        for (int j = 0; j < nb; j++) {
          const float d = (float)fabs((double)(avals[i] - vals[j]));
          if (d < md) {
            md = d;
            bk[i] = (uint32_t)j;
          }
        }
      }
    }
    float asq = 0.0f, bsq = 0.0f, ab = 0.0f, ax = 0.0f, bx = 0.0f;
    for (int i = 0; i < nb; i++) {
      const float fbi = (float)(nb - 1 - i), fb = (float)(nb - 1), fi = (float)i;
      const float a = fbi / fb, b = fi / fb;
      const float n = npts[i], x = vals[i];
      asq += n * a * a;
      bsq += n * b * b;
      ab += n * a * b;
      ax += x * a * n;
      bx += x * b * n;
    }
    const float f = 1.0f / (asq * bsq - ab * ab);
    a1 = f * (ax * bsq - bx * ab);
    a2 = f * (bx * asq - ax * ab);
    a1 = fmin_std(255.0f, fmax_std(0.0f, a1));
    a2 = fmin_std(255.0f, fmax_std(0.0f, a2));
    const uint8_t amask = (uint8_t)((int8_t)-0x7F >> (m->a->alpha_bits - 1));
    const uint8_t a1b = quantize_channel((uint8_t)a1, amask, -1);
    const uint8_t a2b = quantize_channel((uint8_t)a2, amask, -1);
    aerr = 0.0;
    for (int i = 0; i < 16; i++) {
      const uint8_t val = (uint8_t)avals[i];
      float me = FLT_MAX;
      int bb = -1;
      for (int j = 0; j < nb; j++) {
        const uint32_t w1 = weight1(abits, j), w0 = 64 - w1;
        const uint8_t ip = (uint8_t)(((a1b * w0) + (a2b * w1) + 32) >> 6);
        float pe = wa * (float)(val > ip ? val - ip : ip - val);
        pe *= pe;
        if (pe < me) {
          me = pe;
          bb = j;
        }
      }
      aerr += me;
      aidx[i] = (uint8_t)bb;
    }
  }
  for (int k = 0; k < 3; k++) {
    p1[k] = rp1[k];
    p2[k] = rp2[k];
  }
  p1[3] = a1;
  p2[3] = a2;
  if (g_note) g_note->aerr = aerr;
  return rgb_err + aerr;
}

/* ------------------------------------------------------------------------ */
/* Mode compression and packing (CP:1096-1371)                               */
/* ------------------------------------------------------------------------ */

typedef struct {
  float p1[3][4], p2[3][4];
  uint8_t idx[3][16];
  uint8_t aidx[16];
  uint8_t pbit[3];
  int8_t rot, idx_mode;
  uint16_t shape;
} params;

typedef struct {
  const bc7o_settings *s;
  uint32_t bx, by;
  uint32_t *lcg; /* single-stream state */
} block_ctx;

static void init_ctx(mode_ctx *m, int mode, const block_ctx *b) {
  m->mode = mode;
  m->a = &kMode[mode];
  m->steps = (int)b->s->steps;
  m->metric = (int)b->s->metric;
  m->rot = 0;
  m->idx_mode = 0;
  m->exp_mode = (int)b->s->exp_mode;
  m->lcg = b->lcg;
}

/* Whether the fit bound includes the palette-size term (diagnostic switch
 * for comparing the pruning with and without it; on by default). */
static int g_level_bound = 1;
void bc7o_set_level_bound(int on) { g_level_bound = on; }

static void sort_ints(int *v, int n) {
  for (int i = 1; i < n; i++)
    for (int j = i; j > 0 && v[j - 1] > v[j]; j--) {
      const int t = v[j];
      v[j] = v[j - 1];
      v[j - 1] = t;
    }
}

/* The palette-size term of the GPU pipeline's bound (qe_lower_bound in
 * fastc_gb300/csrc/bc7_intqe.cuh), in the same steps. A palette has k
 * colours, so on any unit direction u the error is at least the best
 * k-level quantisation of the texels' projections (1-D k-means, whose
 * groups are runs of the sorted projections); a run of span w costs at
 * least w^2 / 2, and the spans add up to at least the n - k smallest gaps
 * between sorted projections (G), so the error is at least G^2 / (2 k).
 * u is the scatter's principal direction (power iteration on the
 * unit-trace scatter A), rounded to an integer direction d (components in
 * 1/64 of the largest), so the projections d.p are exact integers and the
 * bound is G^2 / (2 k |d|^2). Like the GPU, it is computed for 4-colour
 * palettes only, with four power iterations. */
static float level_bound(const uint32_t *px, int n, int k, float A[4][4]) {
  if (k != 4 || n <= k) return 0.0f; /* computed for 4-colour palettes only */
  int d0 = 0;
  for (int c = 1; c < 4; c++)
    if (A[c][c] > A[d0][d0]) d0 = c;
  float v[4];
  for (int c = 0; c < 4; c++) v[c] = A[c][d0];
  for (int it = 0; it < 4; it++) {
    float w[4], m = 0.0f;
    for (int a = 0; a < 4; a++) {
      w[a] = A[a][0] * v[0] + A[a][1] * v[1] + A[a][2] * v[2] + A[a][3] * v[3];
      const float x = fabsf(w[a]);
      if (x > m) m = x;
    }
    if (!(m > 0.0f)) return 0.0f;
    const float r = 1.0f / m;
    for (int a = 0; a < 4; a++) v[a] = w[a] * r;
  }
  float m = 0.0f;
  for (int c = 0; c < 4; c++)
    if (fabsf(v[c]) > m) m = fabsf(v[c]);
  int d[4], dd = 0;
  for (int c = 0; c < 4; c++) {
    d[c] = (int)rintf(v[c] * 64.0f / m);
    dd += d[c] * d[c];
  }
  if (dd == 0) return 0.0f;
  int sp[16], g[16];
  for (int i = 0; i < n; i++) {
    sp[i] = 0;
    for (int c = 0; c < 4; c++) sp[i] += d[c] * (int)((px[i] >> (8 * c)) & 0xFF);
  }
  sort_ints(sp, n);
  for (int i = 0; i + 1 < n; i++) g[i] = sp[i + 1] - sp[i];
  sort_ints(g, n - 1);
  int G = 0;
  for (int i = 0; i < n - k; i++) G += g[i];
  const float fg = (float)G;
  return fg * fg / (float)(2 * k * dd) * (1.0f - 1e-5f);
}

/* The GPU pipeline's error lower bound for a fit of n texels and a k-colour
 * palette (qe_lower_bound in fastc_gb300/csrc/bc7_intqe.cuh), in the same
 * float steps: the larger of the scatter left after the best line (from an
 * upper bound on the largest eigenvalue, less the palette's rounding slack)
 * and the palette-size term above. */
static float fit_lower_bound(const uint32_t *px, int n, int k) {
  int sm[4] = {0, 0, 0, 0}, q[10] = {0};
  for (int k = 0; k < n; k++) {
    int v[4];
    for (int c = 0; c < 4; c++) {
      v[c] = (int)((px[k] >> (8 * c)) & 0xFF);
      sm[c] += v[c];
    }
    int j = 0;
    for (int a = 0; a < 4; a++)
      for (int b = a; b < 4; b++) q[j++] += v[a] * v[b];
  }
  float A[4][4];
  int tr = 0, j = 0;
  for (int a = 0; a < 4; a++)
    for (int b = a; b < 4; b++) {
      const int v = n * q[j++] - sm[a] * sm[b];
      if (a == b) tr += v;
      A[a][b] = A[b][a] = (float)v;
    }
  if (tr <= 0) return 0.0f;
  const float inv = 1.0f / (float)tr;
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++) A[a][b] *= inv;
  float f = 0.0f;
  for (int a = 0; a < 4; a++)
    for (int b = a; b < 4; b++) {
      const float v = A[a][0] * A[0][b] + A[a][1] * A[1][b] + A[a][2] * A[2][b] + A[a][3] * A[3][b];
      f += (a == b ? 1.0f : 2.0f) * v * v;
    }
  const float lam = sqrtf(sqrtf(f));
  float one = 1.0f - lam - 1e-5f;
  if (one < 0.0f) one = 0.0f;
  const float R = one * ((float)tr / (float)n);
  const float fn = (float)n;
  float lb = 0.0f;
  if (R >= fn) {
    lb = R - 2.0f * sqrtf(fn * R) - 1e-3f * R;
    if (lb < 0.0f) lb = 0.0f;
  }
  const float lv = g_level_bound ? level_bound(px, n, k, A) : 0.0f;
  return lv > lb ? lv : lb;
}

/* Records one fit of the traced block. For a fit that took FasTC's
 * single-colour shortcut the setup error and bound are its error. */
static void trace_fit(const mode_ctx *m, const cluster *c, int slot, int subset, int rot_im,
                      const fit_note *note, double final_err) {
  g_note = NULL;
  if (g_ntrace >= g_trace_cap) return;
  bc7o_fit_trace *t = &g_trace[g_ntrace++];
  t->mode = m->mode;
  t->slot = slot;
  t->subset = subset;
  t->rot_im = rot_im;
  t->n = c->n;
  t->annealed = note->annealed;
  t->final_err = final_err;
  if (note->annealed) {
    t->init_err = note->init + note->aerr;
    t->lower_bound =
        (m->metric ? 0.0 : (double)fit_lower_bound(c->px, c->n, 1 << bits_index(m, -1))) + note->aerr;
  } else {
    t->init_err = t->lower_bound = final_err;
  }
}

/* CompressionMode::Compress (CP:1300-1371). `slot` is the position of the
 * shape in the selection; it only keys the per-fit RNG. */
static double compress_mode(int mode, int shape, int slot,
                            const uint32_t block[16], const block_ctx *b,
                            params *pr) {
  mode_ctx m;
  init_ctx(&m, mode, b);
  const int nsub = m.a->subsets;
  memset(pr, 0, sizeof(*pr));
  pr->rot = -1;
  pr->idx_mode = -1;
  pr->shape = (uint16_t)shape;
  memset(pr->idx, 0xFF, sizeof(pr->idx));
  memset(pr->aidx, 0xFF, sizeof(pr->aidx));
  memset(pr->pbit, 0xFF, sizeof(pr->pbit));
  double total = 0.0;
  for (int ci = 0; ci < nsub; ci++) {
    uint8_t idx[16] = {0};
    cluster c;
    make_cluster(block, shape, nsub, ci, &c);
    if (m.a->has_rotation) {
      uint8_t aidx[16];
      double best = DBL_MAX;
      for (int rot = 0; rot < 4; rot++) {
        const int nim = mode == 4 ? 2 : 1;
        for (int im = 0; im < nim; im++) {
          m.rot = rot;
          m.idx_mode = im;
          uint32_t fit_lcg;
          if (b->s->rng_mode == BC7O_RNG_PER_FIT) {
            fit_lcg = bc7o_fit_seed(b->s->seed, b->bx, b->by,
                                    (uint32_t)((mode << 8) | (slot << 7) |
                                               (ci << 4) | (rot << 1) | im));
            m.lcg = &fit_lcg;
          }
          float v1[4], v2[4];
          fit_note note = {0.0, 0.0, 0};
          if (g_trace) g_note = &note;
          const double e = fit_alpha(&m, &c, v1, v2, idx, aidx);
          if (g_trace) trace_fit(&m, &c, slot, ci, (rot << 1) | im, &note, e);
          if (e < best) {
            best = e;
            memcpy(pr->idx[ci], idx, 16);
            memcpy(pr->aidx, aidx, 16);
            pr->rot = (int8_t)rot;
            pr->idx_mode = (int8_t)im;
            memcpy(pr->p1[ci], v1, sizeof(v1));
            memcpy(pr->p2[ci], v2, sizeof(v2));
          }
        }
      }
      total += best;
    } else {
      uint32_t fit_lcg;
      if (b->s->rng_mode == BC7O_RNG_PER_FIT) {
        fit_lcg = bc7o_fit_seed(b->s->seed, b->bx, b->by,
                                (uint32_t)((mode << 8) | (slot << 7) | (ci << 4)));
        m.lcg = &fit_lcg;
      }
      fit_note note = {0.0, 0.0, 0};
      if (g_trace) g_note = &note;
      const double e = fit_rgb(&m, &c, pr->p1[ci], pr->p2[ci], idx, &pr->pbit[ci]);
      if (g_trace) trace_fit(&m, &c, slot, ci, -1, &note, e);
      total += e;
      int k = 0;
      for (int i = 0; i < 16; i++)
        if (subset_of(i, shape, nsub) == ci) pr->idx[ci][i] = idx[k++];
    }
  }
  return total;
}

/* Debug hook: one mode compression with a single-stream LCG. */
double bc7o_compress_mode(const uint32_t px[16], int mode, int shape,
                          uint32_t steps, uint32_t exp_mode, uint32_t *lcg) {
  pthread_once(&gTablesOnce, build_tables);
  pthread_once(&gMetricOnce, build_metric);
  bc7o_settings s = {steps, 0xFF, 0, BC7O_RNG_SINGLE_STREAM, 0, exp_mode};
  block_ctx b = {&s, 0, 0, lcg};
  params p;
  return compress_mode(mode, shape, 0, px, &b, &p);
}

/* BitStream (BitStream.h:65-91): LSB-first writer, capped at 128 bits. */
typedef struct {
  uint8_t *buf;
  int pos;
} bitw;

static void put_bits(bitw *w, uint32_t val, int n) {
  for (int i = 0; i < n; i++) {
    if (w->pos >= 128) return;
    const uint32_t bit = i < 32 ? (val >> i) & 1 : 0;
    const int byte = w->pos >> 3, sh = w->pos & 7;
    w->buf[byte] = (uint8_t)((w->buf[byte] & ~(1u << sh)) | (bit << sh));
    w->pos++;
  }
}

/* CompressionMode::Pack (CP:1096-1298). */
static void pack(int mode, params *pr, uint8_t out[16]) {
  mode_ctx m;
  memset(&m, 0, sizeof(m));
  m.mode = mode;
  m.a = &kMode[mode];
  const mode_attr *a = m.a;
  const int nsub = a->subsets;
  bitw w = {out, 0};
  put_bits(&w, 1u << mode, mode + 1);
  put_bits(&w, pr->shape, a->part_bits);
  put_bits(&w, (uint32_t)pr->rot, a->has_rotation ? 2 : 0);
  put_bits(&w, (uint32_t)pr->idx_mode, a->has_idx_mode ? 1 : 0);
  const uint32_t qm = qmask_of(&m);
  uint32_t px1[3], px2[3];
  for (int i = 0; i < nsub; i++) {
    if (a->pbit == PB_NONE) {
      px1[i] = to_pixel(pr->p1[i], qm, -1);
      px2[i] = to_pixel(pr->p2[i], qm, -1);
    } else {
      px1[i] = to_pixel(pr->p1[i], qm, pbit_combo(&m, pr->pbit[i])[0]);
      px2[i] = to_pixel(pr->p2[i], qm, pbit_combo(&m, pr->pbit[i])[1]);
    }
  }
  const int nib = bits_index(&m, pr->idx_mode), nab = bits_alpha(&m, pr->idx_mode);
  for (int s = 0; s < nsub; s++) {
    const int anchor = anchor_of(s, pr->shape, nsub);
    if (pr->idx[s][anchor] >> (nib - 1)) {
      const uint32_t t = px1[s];
      px1[s] = px2[s];
      px2[s] = t;
      for (int i = 0; i < 16; i++)
        pr->idx[s][i] = (uint8_t)(((1 << nib) - 1) - pr->idx[s][i]);
      if (a->has_rotation)
        for (int i = 0; i < 16; i++)
          pr->aidx[i] = (uint8_t)(((1 << nab) - 1) - pr->aidx[i]);
    }
    if (a->has_rotation && (pr->aidx[anchor] >> (nab - 1)) > 0) {
      const uint32_t hi1 = px1[s] & 0xFF000000u, hi2 = px2[s] & 0xFF000000u;
      px1[s] = (px1[s] & 0x00FFFFFFu) | hi2;
      px2[s] = (px2[s] & 0x00FFFFFFu) | hi1;
      for (int i = 0; i < 16; i++)
        pr->aidx[i] = (uint8_t)(((1 << nab) - 1) - pr->aidx[i]);
    }
  }
  for (int ch = 0; ch < 4; ch++) {
    const int bits = ch == 3 ? a->alpha_bits : a->color_bits;
    for (int i = 0; i < nsub; i++) {
      put_bits(&w, ((px1[i] >> (8 * ch)) & 0xFF) >> (8 - bits), bits);
      put_bits(&w, ((px2[i] >> (8 * ch)) & 0xFF) >> (8 - bits), bits);
    }
  }
  if (a->pbit != PB_NONE)
    for (int s = 0; s < nsub; s++) {
      const int *pb = pbit_combo(&m, pr->pbit[s]);
      put_bits(&w, (uint32_t)pb[0], 1);
      if (a->pbit != PB_SHARED) put_bits(&w, (uint32_t)pb[1], 1);
    }
  if (a->has_idx_mode && pr->idx_mode == 1) {
    for (int i = 0; i < 16; i++) put_bits(&w, pr->aidx[i], i == 0 ? 1 : 2);
    for (int i = 0; i < 16; i++) put_bits(&w, pr->idx[0][i], i == 0 ? 2 : 3);
  } else {
    for (int i = 0; i < 16; i++) {
      const int s = subset_of(i, pr->shape, nsub);
      const int anchor = anchor_of(s, pr->shape, nsub);
      put_bits(&w, pr->idx[s][i], i == anchor ? nib - 1 : nib);
    }
    if (a->has_rotation)
      for (int i = 0; i < 16; i++) put_bits(&w, pr->aidx[i], i == 0 ? nab - 1 : nab);
  }
}

/* ------------------------------------------------------------------------ */
/* Shape selection (CP:1626-1750)                                            */
/* ------------------------------------------------------------------------ */

#define MODES_TWO ((1u << 1) | (1u << 3) | (1u << 7))
#define MODES_THREE ((1u << 0) | (1u << 2))
#define MODES_ALPHA ((1u << 4) | (1u << 5) | (1u << 6) | (1u << 7))

typedef struct {
  uint32_t nshapes;
  uint32_t shape[2];
  uint32_t nparts[2];
  uint32_t modes;
} selection;

static double estimate_error(const cluster *c, int nb, uint32_t metric) {
  float v[4];
  for (int k = 0; k < 4; k++) v[k] = c->mx[k] - c->mn[k];
  if (dot4(v, v) == 0) return 0.0;
  double e = 0.0001;
  e += quantized_error(c, c->mn, c->mx, nb, 0xFFFFFFFFu, gMetricW[metric], NULL,
                       NULL);
  return e;
}

static selection box_selection(const uint32_t px[16], uint32_t metric) {
  selection r;
  r.nshapes = 1;
  r.shape[0] = r.shape[1] = 0;
  r.nparts[0] = r.nparts[1] = 0;
  r.modes = 0xFF;
  int opaque = 1;
  for (int i = 0; i < 16; i++) opaque = opaque && (((px[i] >> 24) & 0xFF) >= 250);
  double best[2] = {DBL_MAX, DBL_MAX};
  for (int i = 0; i < 64; i++) {
    double err = 0.0;
    for (int ci = 0; ci < 2; ci++) {
      cluster c;
      make_cluster(px, i, 2, ci, &c);
      err += estimate_error(&c, 8, metric);
    }
    if (err < best[0]) {
      best[0] = err;
      r.shape[0] = (uint32_t)i;
      r.nparts[0] = 2;
    }
    if (err < 1e-9) {
      r.modes = MODES_TWO;
      return r;
    }
  }
  if (!opaque) {
    r.modes &= MODES_ALPHA;
    return r;
  }
  r.modes &= ~((1u << 4) | (1u << 5));
  r.nshapes++;
  for (int i = 0; i < 64; i++) {
    double err = 0.0;
    for (int ci = 0; ci < 3; ci++) {
      cluster c;
      make_cluster(px, i, 3, ci, &c);
      err += estimate_error(&c, 4, metric);
    }
    if (err < best[1]) {
      best[1] = err;
      r.shape[1] = (uint32_t)i;
      r.nparts[1] = 3;
    }
    if (err < 1e-9) {
      r.modes = MODES_THREE;
      return r;
    }
  }
  return r;
}

void bc7o_box_selection(const uint32_t px[16], uint32_t metric, uint32_t out[4]) {
  pthread_once(&gMetricOnce, build_metric);
  selection s = box_selection(px, metric);
  out[0] = s.nshapes;
  out[1] = s.shape[0];
  out[2] = s.nshapes > 1 ? s.shape[1] : 0xFFFFFFFFu;
  out[3] = s.modes;
}

/* ------------------------------------------------------------------------ */
/* Block driver (CP:1405-1458, 1752-1860)                                    */
/* ------------------------------------------------------------------------ */

static void write_single_color(uint32_t pixel, uint32_t wm, uint8_t out[16]) {
  bitw w = {out, 0};
  put_bits(&w, 1u << 5, 6);
  put_bits(&w, 0, 2);
  for (int c = 0; c < 3; c++) {
    const uint32_t v = (pixel >> (8 * c)) & 0xFF;
    put_bits(&w, gOpt7[v][0], 7);
    put_bits(&w, gOpt7[v][1], 7);
  }
  const uint32_t a = pixel >> 24;
  put_bits(&w, a, 8);
  put_bits(&w, a, 8);
  put_bits(&w, 0xaaaaaaabu, 31);
  put_bits(&w, kWatermark[wm % 9], 31);
}

static void write_transparent(uint8_t out[16]) {
  bitw w = {out, 0};
  put_bits(&w, 1u << 6, 7);
  put_bits(&w, 0, 121);
}

/* CompressClusters (CP:1752-1817): every selected mode over the searched
 * shapes in the order {0,2,1,3,7,4,5,6}, strict-< arg-min, Pack. Returns the
 * packed mode (8 when no mode applied: a transparent block is written). */
static int compress_clusters(const uint32_t px[16], const selection *sel, uint32_t modes,
                             const block_ctx *b, uint8_t out[16]) {
  static const int order[8] = {0, 2, 1, 3, 7, 4, 5, 6};
  double best = DBL_MAX;
  int best_mode = 8;
  params best_p, p;
  memset(&best_p, 0, sizeof(best_p));
  uint32_t nshapes = sel->nshapes < 5 ? sel->nshapes : 5;
  for (int oi = 0; oi < 8; oi++) {
    const int mode = order[oi];
    if (!(modes & (1u << mode))) continue;
    for (uint32_t si = 0; si < nshapes; si++) {
      const int np = kMode[mode].subsets;
      if (np != 1 && (uint32_t)np != sel->nparts[si]) continue;
      if (sel->shape[si] >= 16 && mode == 0) continue;
      const double e = compress_mode(mode, (int)sel->shape[si], (int)si, px, b, &p);
      if (e < best) {
        best = e;
        best_mode = mode;
        best_p = p;
      }
    }
  }
  if (best_mode == 8) { /* no mode applies to any searched shape */
    write_transparent(out);
    return 8;
  }
  pack(best_mode, &best_p, out);
  return best_mode;
}

void bc7o_compress_block(const uint32_t px[16], const bc7o_settings *s,
                         uint32_t bx, uint32_t by, uint32_t *wm, uint32_t *lcg,
                         uint8_t out[16]) {
  pthread_once(&gTablesOnce, build_tables);
  pthread_once(&gMetricOnce, build_metric);
  int same = 1;
  for (int i = 1; i < 16; i++) same = same && px[i] == px[0];
  if (same) {
    write_single_color(px[0], *wm, out);
    (*wm)++;
    return;
  }
  int transparent = 1;
  for (int i = 0; i < 16; i++)
    if ((px[i] >> 24) != 0) transparent = 0;
  if (transparent) {
    write_transparent(out);
    return;
  }
  selection sel = box_selection(px, s->metric);
  uint32_t modes = sel.modes & s->block_modes;
  /* An empty set is undefined behaviour in the reference (it packs mode 8);
   * fall back to the caller's mask so the block is always valid. */
  if (modes == 0) modes = s->block_modes & 0xFF;

  block_ctx b = {s, bx, by, lcg};
  compress_clusters(px, &sel, modes, &b, out);
}

int bc7o_trace_block(const uint32_t px[16], const bc7o_settings *s, uint32_t bx,
                     uint32_t by, uint32_t *wm, uint32_t *lcg, uint8_t out[16],
                     bc7o_fit_trace *fits, int cap) {
  g_trace = fits;
  g_trace_cap = cap;
  g_ntrace = 0;
  bc7o_compress_block(px, s, bx, by, wm, lcg, out);
  g_trace = NULL;
  g_note = NULL;
  return g_ntrace;
}

/* ------------------------------------------------------------------------ */
/* CompressWithStats: the logging block encoder (CP:1862-2183)               */
/* ------------------------------------------------------------------------ */

/* UpdateErrorEstimate (CP:1930-1936). */
static void update_estimate(double *est, int mode, double e) {
  if (est[mode] == -1.0 || e < est[mode]) est[mode] = e;
}

/* EstimateTwoClusterErrorStats / EstimateThreeClusterErrorStats
 * (CP:1862-1928): the subset's bounding box quantised with two grids (the
 * colour precisions of modes 1 and 3, or 0 and 2), each error recorded as
 * the candidate mode's estimate; the shape error takes the smaller. */
static double estimate_stats(const cluster *c, int three, uint32_t metric, double est[2]) {
  float v[4];
  for (int k = 0; k < 4; k++) v[k] = c->mx[k] - c->mn[k];
  if (dot4(v, v) == 0) {
    est[0] = est[1] = 0.0;
    return 0.0;
  }
  const int nb = three ? 4 : 8;
  const uint32_t m0 = three ? 0xFFF0F0F0u : 0xFFFCFCFCu;
  const uint32_t m1 = three ? 0xFFF8F8F8u : 0xFFFEFEFEu;
  const double bias = three ? 0.0001 : 0.0;
  const double e0 = bias + (double)quantized_error(c, c->mn, c->mx, nb, m0, gMetricW[metric], NULL, NULL);
  const double e1 = bias + (double)quantized_error(c, c->mn, c->mx, nb, m1, gMetricW[metric], NULL, NULL);
  est[0] = e0; /* never negative, so the reference's min() branch is dead */
  est[1] = e1;
  double err = 0.0001;
  err += e0 < e1 ? e0 : e1;
  return err;
}

/* One shape loop of the logging encoder: nsub 2 (CP:2066-2114) or 3
 * (CP:2118-2166). Returns 1 when a shape's estimate is below 1e-9. */
static int stats_shapes(const uint32_t px[16], int nsub, uint32_t metric, selection *sel,
                        bc7o_block_stats *st) {
  const int three = nsub == 3;
  const int slot = three ? 1 : 0;
  double best = DBL_MAX;
  for (int i = 0; i < 64; i++) {
    double err = 0.0;
    double acc[2] = {-1.0, -1.0};
    for (int ci = 0; ci < nsub; ci++) {
      cluster c;
      make_cluster(px, i, nsub, ci, &c);
      double e[2] = {-1.0, -1.0};
      err += estimate_stats(&c, three, metric, e);
      for (int k = 0; k < 2; k++)
        if (e[k] >= 0.0) acc[k] = acc[k] == -1.0 ? e[k] : acc[k] + e[k];
    }
    if (acc[0] != -1.0) update_estimate(st->estimate, three ? 0 : 1, acc[0]);
    if (acc[1] != -1.0) update_estimate(st->estimate, three ? 2 : 3, acc[1]);
    if (err < best) {
      if (three) st->three_shape[st->n_three++] = err;
      else st->two_shape[st->n_two++] = err;
      best = err;
      sel->shape[slot] = (uint32_t)i;
      sel->nparts[slot] = (uint32_t)nsub;
    }
    if (err < 1e-9) {
      sel->modes = three ? MODES_THREE : MODES_TWO;
      return 1;
    }
  }
  return 0;
}

/* CompressBC7Block with a BlockLogger (CP:1938-2183). Its shape selection
 * differs from BoxSelection: opaque means every alpha is exactly 255, the
 * modes are not narrowed by opacity (modes 4 and 5 stay on for opaque
 * blocks, 1, 3 and 6 for the others), the 3-subset shapes are searched
 * for opaque blocks even after an exact 2-subset shape, and the bounding
 * boxes are quantised before their QuantizedError. The per-mode errors it
 * logs stay -1: CompressClusters keeps min(error, -1) (CP:1801). */
void bc7o_compress_block_stats(const uint32_t px[16], const bc7o_settings *s, uint32_t bx,
                               uint32_t by, uint32_t *wm, uint32_t *lcg, uint8_t out[16],
                               bc7o_block_stats *st) {
  pthread_once(&gTablesOnce, build_tables);
  pthread_once(&gMetricOnce, build_metric);
  memset(st, 0, sizeof(*st));
  for (int i = 0; i < 8; i++) st->estimate[i] = st->error[i] = -1.0;
  int same = 1;
  for (int i = 1; i < 16; i++) same = same && px[i] == px[0];
  if (same) {
    write_single_color(px[0], *wm, out);
    (*wm)++;
    st->mode = 5;
    st->path = 0;
    return;
  }
  int opaque = 1, transparent = 1;
  for (int i = 0; i < 16; i++) {
    const uint32_t a = px[i] >> 24;
    if (a != 255) opaque = 0;
    if (a != 0) transparent = 0;
  }
  if (transparent) {
    write_transparent(out);
    st->mode = 6;
    st->path = 1;
    return;
  }
  { /* mode 6's estimate: the whole block's box, 4 buckets (CP:2046-2058) */
    cluster c;
    make_cluster(px, 0, 1, 0, &c);
    float v[4];
    for (int k = 0; k < 4; k++) v[k] = c.mx[k] - c.mn[k];
    if (dot4(v, v) == 0) {
      st->estimate[6] = 0.0;
    } else {
      const double e = 0.0001 + (double)quantized_error(&c, c.mn, c.mx, 4, 0xFEFEFEFEu,
                                                         gMetricW[s->metric], NULL, NULL);
      update_estimate(st->estimate, 6, e);
    }
  }
  selection sel;
  sel.nshapes = 1;
  sel.shape[0] = sel.shape[1] = 0;
  sel.nparts[0] = sel.nparts[1] = 0;
  sel.modes = 0xFF;
  int path = 0;
  if (stats_shapes(px, 2, s->metric, &sel, st)) path = 2;
  if (opaque) {
    sel.nshapes++;
    if (stats_shapes(px, 3, s->metric, &sel, st)) path = 2;
  }
  if (path == 0) path = 3;
  st->path = path;
  uint32_t modes = sel.modes & s->block_modes;
  if (modes == 0) modes = s->block_modes & 0xFF; /* as in bc7o_compress_block */
  block_ctx b = {s, bx, by, lcg};
  st->mode = compress_clusters(px, &sel, modes, &b, out);
}

/* ------------------------------------------------------------------------ */
/* Image drivers                                                             */
/* ------------------------------------------------------------------------ */

static void load_block(const uint8_t *rgba, uint32_t w, uint32_t x, uint32_t y,
                       uint32_t px[16]) {
  for (int r = 0; r < 4; r++)
    for (int c = 0; c < 4; c++) {
      const uint8_t *p = rgba + 4 * ((size_t)(y + r) * w + x + c);
      px[4 * r + c] = (uint32_t)p[0] | ((uint32_t)p[1] << 8) |
                      ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    }
}

/* BPTCC::Compress over a job rectangle (CP:1473-1520). */
int bc7o_compress(const uint8_t *rgba, uint8_t *out, uint32_t w, uint32_t h,
                  uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                  const bc7o_settings *s, uint32_t state[2]) {
  if ((w | h) & 3) return -1;
  if (x1 == 0) x1 = w;
  if (y1 == 0) y1 = h;
  if ((x0 | y0) & 3 || x0 > w || y0 > h) return -2;
  const uint32_t bw = w / 4;
  uint32_t start_x = x0;
  const uint32_t end_y = y1 < h - 4 ? y1 : h - 4;
  for (uint32_t y = y0; y <= end_y && h >= 4; y += 4) {
    const uint32_t end_x = (y == y1) ? x1 : w;
    for (uint32_t x = start_x; x < end_x; x += 4) {
      uint32_t px[16];
      load_block(rgba, w, x, y, px);
      uint8_t *dst = out + 16 * ((size_t)(y / 4) * bw + x / 4);
      bc7o_compress_block(px, s, x / 4, y / 4, &state[1], &state[0], dst);
    }
    start_x = 0;
  }
  return 0;
}

typedef struct {
  const uint8_t *rgba;
  uint8_t *out;
  uint32_t w;
  const bc7o_settings *s;
  const uint32_t *wm_rank;
  size_t b0, b1;
} mt_arg;

static void *mt_worker(void *p) {
  mt_arg *a = (mt_arg *)p;
  const uint32_t bw = a->w / 4;
  uint32_t dummy_lcg = 0;
  for (size_t b = a->b0; b < a->b1; b++) {
    const uint32_t bx = (uint32_t)(b % bw), by = (uint32_t)(b / bw);
    uint32_t px[16];
    load_block(a->rgba, a->w, bx * 4, by * 4, px);
    uint32_t wm = a->wm_rank[b];
    bc7o_compress_block(px, a->s, bx, by, &wm, &dummy_lcg, a->out + 16 * b);
  }
  return NULL;
}

int bc7o_compress_mt(const uint8_t *rgba, uint8_t *out, uint32_t w,
                     uint32_t h, const bc7o_settings *s, uint32_t wm_start,
                     int nthreads) {
  if ((w | h) & 3) return -1;
  if (s->rng_mode != BC7O_RNG_PER_FIT) return -3;
  pthread_once(&gTablesOnce, build_tables);
  pthread_once(&gMetricOnce, build_metric);
  const size_t nb = (size_t)(w / 4) * (h / 4);
  uint32_t *rank = (uint32_t *)malloc(nb * sizeof(uint32_t) + 1);
  if (!rank) return -4;
  uint32_t cnt = wm_start;
  for (size_t b = 0; b < nb; b++) {
    uint32_t px[16];
    load_block(rgba, w, (uint32_t)(b % (w / 4)) * 4, (uint32_t)(b / (w / 4)) * 4, px);
    int same = 1;
    for (int i = 1; i < 16; i++) same = same && px[i] == px[0];
    rank[b] = cnt;
    cnt += (uint32_t)same;
  }
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  mt_arg args[256];
  const size_t per = (nb + (size_t)nthreads - 1) / (size_t)nthreads;
  int started = 0;
  for (int t = 0; t < nthreads; t++) {
    size_t b0 = (size_t)t * per, b1 = b0 + per;
    if (b0 > nb) b0 = nb;
    if (b1 > nb) b1 = nb;
    args[t] = (mt_arg){rgba, out, w, s, rank, b0, b1};
    if (pthread_create(&th[t], NULL, mt_worker, &args[t]) == 0) started++;
    else mt_worker(&args[t]);
  }
  for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
  free(rank);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Decoder (DC:32-367)                                                       */
/* ------------------------------------------------------------------------ */

typedef struct {
  const uint8_t *buf;
  int pos;
} bitr;

static uint32_t get_bits(bitr *r, int n) {
  uint32_t v = 0;
  for (int i = 0; i < n; i++) {
    const uint32_t bit = (r->buf[r->pos >> 3] >> (r->pos & 7)) & 1;
    v |= bit << i;
    r->pos++;
  }
  return v;
}

static void decode_block(const uint8_t blk[16], uint32_t out[16]) {
  bitr r = {blk, 0};
  int mode = 0;
  while (mode < 8 && !get_bits(&r, 1)) mode++;
  if (mode >= 8) { /* reserved: the reference reads past the block */
    memset(out, 0, 16 * sizeof(uint32_t));
    return;
  }
  const mode_attr *a = &kMode[mode];
  const int nsub = a->subsets;
  int idx_mode = 0, rot = 0, shape = 0;
  if (nsub > 1) shape = (int)get_bits(&r, mode == 0 ? 4 : 6);
  else if (a->has_rotation) {
    rot = (int)get_bits(&r, 2);
    if (a->has_idx_mode) idx_mode = (int)get_bits(&r, 1);
  }
  uint32_t cp = (uint32_t)a->color_bits, ap = (uint32_t)a->alpha_bits;
  uint32_t eps[3][2][4];
  for (int ch = 0; ch < 3; ch++)
    for (int i = 0; i < nsub; i++)
      for (int e = 0; e < 2; e++) eps[i][e][ch] = (get_bits(&r, (int)cp) << (8 - cp)) & 0xFF;
  for (int i = 0; i < nsub; i++)
    for (int e = 0; e < 2; e++)
      eps[i][e][3] = ap == 0 ? 0xFF : ((get_bits(&r, (int)ap) << (8 - ap)) & 0xFF);
  if (a->pbit != PB_NONE) {
    cp++;
    ap++;
    for (int i = 0; i < nsub; i++) {
      if (a->pbit == PB_SHARED) {
        const uint32_t pb = get_bits(&r, 1);
        for (int e = 0; e < 2; e++)
          for (int ch = 0; ch < 4; ch++) eps[i][e][ch] |= pb << (8 - (ch == 3 ? ap : cp));
      } else {
        for (int e = 0; e < 2; e++) {
          const uint32_t pb = get_bits(&r, 1);
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
  uint32_t cidx[16], aidx[16];
  int cbits = a->idx_bits, abits = a->alpha_idx_bits;
  for (int i = 0; i < 16; i++) {
    const int s = subset_of(i, shape, nsub);
    cidx[i] = get_bits(&r, anchor_of(s, shape, nsub) == i ? cbits - 1 : cbits);
  }
  if (abits == 0) memcpy(aidx, cidx, sizeof(aidx));
  else {
    for (int i = 0; i < 16; i++) {
      const int s = subset_of(i, shape, nsub);
      aidx[i] = get_bits(&r, anchor_of(s, shape, nsub) == i ? abits - 1 : abits);
    }
    if (idx_mode) {
      for (int i = 0; i < 16; i++) {
        const uint32_t t = aidx[i];
        aidx[i] = cidx[i];
        cidx[i] = t;
      }
      const int t = abits;
      abits = cbits;
      cbits = t;
    }
  }
  /* The reference interpolates with the mode's nominal index widths even
   * when the index mode swapped the sets (DC:265-266), so a mode-4 block
   * with index mode 1 reads 3-bit colour indices through the 2-bit row. */
  const int nba = a->alpha_idx_bits, nbc = a->idx_bits;
  (void)cbits;
  (void)abits;
  for (int i = 0; i < 16; i++) {
    const int s = subset_of(i, shape, nsub);
    uint32_t px = 0;
    for (int ch = 0; ch < 4; ch++) {
      uint32_t ip;
      uint32_t w0, w1;
      if (ch == 3 && nba > 0) {
        weights_padded(nba, aidx[i], &w0, &w1);
        ip = ((eps[s][0][3] * w0 + eps[s][1][3] * w1) + 32) >> 6;
      } else {
        weights_padded(nbc, cidx[i], &w0, &w1);
        ip = ((eps[s][0][ch] * w0 + eps[s][1][ch] * w1) + 32) >> 6;
      }
      px |= (ip & 0xFF) << (8 * ch);
    }
    if (rot >= 1 && rot <= 3) {
      const int c = rot - 1;
      const uint32_t x = (px >> (8 * c)) & 0xFF, y = px >> 24;
      px = (px & ~(0xFFu << (8 * c)) & 0x00FFFFFFu) | (y << (8 * c)) | (x << 24);
    }
    out[i] = px;
  }
}

void bc7o_decompress(const uint8_t *blocks, uint8_t *rgba, uint32_t w,
                     uint32_t h) {
  for (uint32_t y = 0; y < h; y += 4)
    for (uint32_t x = 0; x < w; x += 4) {
      uint32_t px[16];
      decode_block(blocks, px);
      blocks += 16;
      const uint32_t dw = w - x < 4 ? w - x : 4, dh = h - y < 4 ? h - y : 4;
      for (uint32_t r = 0; r < dh; r++)
        for (uint32_t c = 0; c < dw; c++) {
          uint8_t *p = rgba + 4 * ((size_t)(y + r) * w + x + c);
          const uint32_t v = px[4 * r + c];
          p[0] = v & 0xFF;
          p[1] = (v >> 8) & 0xFF;
          p[2] = (v >> 16) & 0xFF;
          p[3] = v >> 24;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Quality metrics (Base/src/Image.cpp:206-255)                              */
/* ------------------------------------------------------------------------ */

static double px_sse(const uint8_t *a, const uint8_t *b) {
  const double ra = a[3] / 255.0, ua = b[3] / 255.0;
  double s = 0.0;
  for (int c = 0; c < 3; c++) {
    const double d = ra * (double)a[c] - ua * (double)b[c];
    s += d * d;
  }
  return s;
}

/* Each channel's squared difference goes into the running sum on its own,
   in FasTC's order (Image.cpp:244-247), so the sum is FasTC's to the last
   bit. */
double bc7o_psnr(const uint8_t *a, const uint8_t *b, uint32_t w, uint32_t h) {
  double mse = 0.0;
  const size_t n = (size_t)w * h;
  for (size_t i = 0; i < n; i++) {
    const uint8_t *pa = a + 4 * i, *pb = b + 4 * i;
    const double ra = pa[3] / 255.0, ua = pb[3] / 255.0;
    for (int c = 0; c < 3; c++) {
      const double d = ra * (double)pa[c] - ua * (double)pb[c];
      mse += d * d;
    }
  }
  mse /= (double)w * (double)h;
  return 10.0 * log10((3.0 * 255.0 * 255.0) / mse);
}

void bc7o_block_sse(const uint8_t *a, const uint8_t *b, uint32_t w, uint32_t h,
                    double *sse) {
  const uint32_t bw = w / 4;
  for (uint32_t by = 0; by < h / 4; by++)
    for (uint32_t bx = 0; bx < bw; bx++) {
      double s = 0.0;
      for (uint32_t r = 0; r < 4; r++)
        for (uint32_t c = 0; c < 4; c++) {
          const size_t o = 4 * ((size_t)(by * 4 + r) * w + bx * 4 + c);
          s += px_sse(a + o, b + o);
        }
      sse[(size_t)by * bw + bx] = s;
    }
}

void bc7o_tables(uint8_t opt7[512], uint8_t opt6[1536]) {
  pthread_once(&gTablesOnce, build_tables);
  memcpy(opt7, gOpt7, 512);
  memcpy(opt6, gOpt6, 1536);
}

void bc7o_partition(uint32_t shape, uint32_t nsub, uint8_t out[16]) {
  for (int i = 0; i < 16; i++) out[i] = (uint8_t)subset_of(i, (int)(shape & 63), (int)nsub);
}

uint32_t bc7o_anchor(uint32_t subset, uint32_t shape, uint32_t nsub) {
  return (uint32_t)anchor_of((int)subset, (int)(shape & 63), (int)nsub);
}
