/* DXT1 / DXT5 (BC1 / BC3) encoder and decoder restated in C.
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU kernels in
 * fastc_gb300/csrc/dxt.cu; nothing of the product links it.
 *
 * FasTC's DXT path (DXTEncoder/src/Compressor.cpp:44-93) runs the stb_dxt
 * v1.06 block encoder vendored in its tree (DXTEncoder/src/stb_dxt.h, public
 * domain, by Fabian Giesen and Sean Barrett) with dithering on and one
 * refinement pass, for every 4x4 block of the job: DXT1 the colour block
 * alone, DXT5 the alpha block then the colour block. That published
 * algorithm is restated here from its description:
 *   - colour: Floyd-Steinberg dither of the block to 565 (for the fit only);
 *     principal axis by four power iterations on the RGB covariance, the two
 *     texels with the extreme projections as endpoints; indices by
 *     projection onto the endpoint line with dithered error diffusion; one
 *     least-squares refinement of the endpoints for those indices, the
 *     indices re-matched when the endpoints change; a constant block (all
 *     16 RGBA texels equal) takes the optimal single-colour endpoint table;
 *   - alpha: endpoints min and max, indices by the bias rule of
 *     "DXT5 alpha block index determination" (F. Giesen, 2009).
 * The float and double steps keep the published operation order, so a
 * build without contraction (as FasTC's x86-64 SSE build) gives the same
 * bits. Decoding follows FasTC's decoder (DXTEncoder/src/Decompressor.cpp:
 * 26-155): 565 expanded by bit replication, 4-colour blocks when the first
 * endpoint word is larger (always for DXT5's colour), else 3 colours and
 * black, alpha 255 for DXT1, the 8-entry (or 6 + 0 + 255) alpha palette.
 * File:line citations are into the FasTC project. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "dxt_oracle.h"

static uint8_t gExp5[32], gExp6[64];
static uint8_t gMatch5[256][2], gMatch6[256][2]; /* [v][0] = high endpoint, [1] = low */
static uint8_t gQuantRB[256 + 16], gQuantG[256 + 16];
static int gInit;

static int mul8bit(int a, int b) {
  const int t = a * b + 128;
  return (t + (t >> 8)) >> 8;
}

static int lerp13(int a, int b) { return (2 * a + b) / 3; }

/* the single-colour table: the endpoint pair whose 1/3 interpolant lands
 * closest to each value, with 3 % of the endpoint distance as a penalty
 * (stb_dxt.h:121-147) */
static void match_table(uint8_t tab[256][2], const uint8_t *expand, int size) {
  for (int v = 0; v < 256; v++) {
    int best = 256;
    for (int lo = 0; lo < size; lo++)
      for (int hi = 0; hi < size; hi++) {
        const int mine = expand[lo], maxe = expand[hi];
        int err = abs(lerp13(maxe, mine) - v);
        err += abs(maxe - mine) * 3 / 100;
        if (err < best) {
          tab[v][0] = (uint8_t)hi;
          tab[v][1] = (uint8_t)lo;
          best = err;
        }
      }
  }
}

/* stb_dxt.h:603-621 */
static void init_tables(void) {
  if (gInit) return;
  for (int i = 0; i < 32; i++) gExp5[i] = (uint8_t)((i << 3) | (i >> 2));
  for (int i = 0; i < 64; i++) gExp6[i] = (uint8_t)((i << 2) | (i >> 4));
  for (int i = 0; i < 256 + 16; i++) {
    const int v = i < 8 ? 0 : (i - 8 > 255 ? 255 : i - 8);
    gQuantRB[i] = gExp5[mul8bit(v, 31)];
    gQuantG[i] = gExp6[mul8bit(v, 63)];
  }
  match_table(gMatch5, gExp5, 32);
  match_table(gMatch6, gExp6, 64);
  gInit = 1;
}

static uint16_t as565(int r, int g, int b) {
  return (uint16_t)((mul8bit(r, 31) << 11) + (mul8bit(g, 63) << 5) + mul8bit(b, 31));
}

static void from565(uint16_t v, int *c) {
  c[0] = gExp5[(v >> 11) & 31];
  c[1] = gExp6[(v >> 5) & 63];
  c[2] = gExp5[v & 31];
}

/* the four palette colours of endpoints c0, c1 (4-colour interpolation;
 * stb_dxt.h:149-157) */
static void palette(int col[4][3], uint16_t c0, uint16_t c1) {
  from565(c0, col[0]);
  from565(c1, col[1]);
  for (int k = 0; k < 3; k++) {
    col[2][k] = lerp13(col[0][k], col[1][k]);
    col[3][k] = lerp13(col[1][k], col[0][k]);
  }
}

/* Floyd-Steinberg dither of each RGB channel to its 565 grid, row by row;
 * px[i][c] are the block's texels, out the dithered ones (RGB only)
 * (stb_dxt.h:159-184) */
static void dither(const uint8_t px[16][4], uint8_t out[16][4]) {
  for (int ch = 0; ch < 3; ch++) {
    const uint8_t *q = (ch == 1 ? gQuantG : gQuantRB) + 8;
    int prev[4] = {0, 0, 0, 0}, cur[4];
    for (int y = 0; y < 4; y++) {
      const uint8_t *s0 = px[4 * y];
      int v;
      v = s0[ch] + ((3 * prev[1] + 5 * prev[0]) >> 4);
      out[4 * y + 0][ch] = q[v];
      cur[0] = px[4 * y + 0][ch] - out[4 * y + 0][ch];
      v = px[4 * y + 1][ch] + ((7 * cur[0] + 3 * prev[2] + 5 * prev[1] + prev[0]) >> 4);
      out[4 * y + 1][ch] = q[v];
      cur[1] = px[4 * y + 1][ch] - out[4 * y + 1][ch];
      v = px[4 * y + 2][ch] + ((7 * cur[1] + 3 * prev[3] + 5 * prev[2] + prev[1]) >> 4);
      out[4 * y + 2][ch] = q[v];
      cur[2] = px[4 * y + 2][ch] - out[4 * y + 2][ch];
      v = px[4 * y + 3][ch] + ((7 * cur[2] + 5 * prev[3] + prev[2]) >> 4);
      out[4 * y + 3][ch] = q[v];
      cur[3] = px[4 * y + 3][ch] - out[4 * y + 3][ch];
      memcpy(prev, cur, sizeof(prev));
    }
  }
}

/* indices: projections onto the endpoint direction, split at the midpoints
 * of the palette's projections, with the projection error diffused
 * (stb_dxt.h:186-281) */
static uint32_t match(const uint8_t px[16][4], int col[4][3]) {
  const int dr = col[0][0] - col[1][0], dg = col[0][1] - col[1][1], db = col[0][2] - col[1][2];
  int dots[16], stops[4];
  for (int i = 0; i < 16; i++) dots[i] = px[i][0] * dr + px[i][1] * dg + px[i][2] * db;
  for (int i = 0; i < 4; i++) stops[i] = col[i][0] * dr + col[i][1] * dg + col[i][2] * db;
  const int c0p = ((stops[1] + stops[3]) >> 1) << 4;
  const int half = ((stops[3] + stops[2]) >> 1) << 4;
  const int c3p = ((stops[2] + stops[0]) >> 1) << 4;
  int prev[4] = {0, 0, 0, 0}, cur[4];
  uint32_t mask = 0;
  for (int y = 0; y < 4; y++) {
    const int *dp = dots + 4 * y;
    uint32_t row = 0;
    for (int x = 0; x < 4; x++) {
      int diff;
      switch (x) {
        case 0: diff = 3 * prev[1] + 5 * prev[0]; break;
        case 1: diff = 7 * cur[0] + 3 * prev[2] + 5 * prev[1] + prev[0]; break;
        case 2: diff = 7 * cur[1] + 3 * prev[3] + 5 * prev[2] + prev[1]; break;
        default: diff = 7 * cur[2] + 5 * prev[3] + prev[2]; break;
      }
      const int dot = (dp[x] << 4) + diff;
      const int step = dot < half ? (dot < c0p ? 1 : 3) : (dot < c3p ? 2 : 0);
      cur[x] = dp[x] - stops[step];
      row |= (uint32_t)step << (2 * x);
    }
    mask |= row << (8 * y);
    memcpy(prev, cur, sizeof(prev));
  }
  return mask;
}

/* endpoints from the principal axis of the (dithered) texels
 * (stb_dxt.h:283-385) */
static void axis_endpoints(const uint8_t px[16][4], uint16_t *max16, uint16_t *min16) {
  int mu[3], mn[3], mx[3];
  for (int ch = 0; ch < 3; ch++) {
    int s = px[0][ch], lo = px[0][ch], hi = px[0][ch];
    for (int i = 1; i < 16; i++) {
      s += px[i][ch];
      if (px[i][ch] < lo) lo = px[i][ch];
      else if (px[i][ch] > hi) hi = px[i][ch];
    }
    mu[ch] = (s + 8) >> 4;
    mn[ch] = lo;
    mx[ch] = hi;
  }
  int cov[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 16; i++) {
    const int r = px[i][0] - mu[0], g = px[i][1] - mu[1], b = px[i][2] - mu[2];
    cov[0] += r * r;
    cov[1] += r * g;
    cov[2] += r * b;
    cov[3] += g * g;
    cov[4] += g * b;
    cov[5] += b * b;
  }
  float cf[6];
  for (int i = 0; i < 6; i++) cf[i] = (float)cov[i] / 255.0f;
  float vr = (float)(mx[0] - mn[0]), vg = (float)(mx[1] - mn[1]), vb = (float)(mx[2] - mn[2]);
  for (int it = 0; it < 4; it++) {
    const float r = vr * cf[0] + vg * cf[1] + vb * cf[2];
    const float g = vr * cf[1] + vg * cf[3] + vb * cf[4];
    const float b = vr * cf[2] + vg * cf[4] + vb * cf[5];
    vr = r;
    vg = g;
    vb = b;
  }
  double magn = fabs((double)vr);
  if (fabs((double)vg) > magn) magn = fabs((double)vg);
  if (fabs((double)vb) > magn) magn = fabs((double)vb);
  int ar, ag, ab;
  if (magn < 4.0) { /* too small: luma weights x 1000 */
    ar = 299;
    ag = 587;
    ab = 114;
  } else {
    magn = 512.0 / magn;
    ar = (int)((double)vr * magn);
    ag = (int)((double)vg * magn);
    ab = (int)((double)vb * magn);
  }
  int dmin = 0x7fffffff, dmax = -0x7fffffff, imin = 0, imax = 0;
  for (int i = 0; i < 16; i++) {
    const int d = px[i][0] * ar + px[i][1] * ag + px[i][2] * ab;
    if (d < dmin) {
      dmin = d;
      imin = i;
    }
    if (d > dmax) {
      dmax = d;
      imax = i;
    }
  }
  *max16 = as565(px[imax][0], px[imax][1], px[imax][2]);
  *min16 = as565(px[imin][0], px[imin][1], px[imin][2]);
}

static int clamp_trunc(float y, int hi) {
  const int x = (int)y;
  return x < 0 ? 0 : (x > hi ? hi : x);
}

/* least-squares endpoints for the indices in `mask`; 1 when they changed
 * (stb_dxt.h:387-475) */
static int refine(const uint8_t px[16][4], uint16_t *max16, uint16_t *min16, uint32_t mask) {
  const uint16_t old_min = *min16, old_max = *max16;
  uint16_t mn16, mx16;
  if ((mask ^ (mask << 2)) < 4) { /* one index for every texel: the mean's best pair */
    int r = 8, g = 8, b = 8;
    for (int i = 0; i < 16; i++) {
      r += px[i][0];
      g += px[i][1];
      b += px[i][2];
    }
    r >>= 4;
    g >>= 4;
    b >>= 4;
    mx16 = (uint16_t)((gMatch5[r][0] << 11) | (gMatch6[g][0] << 5) | gMatch5[b][0]);
    mn16 = (uint16_t)((gMatch5[r][1] << 11) | (gMatch6[g][1] << 5) | gMatch5[b][1]);
  } else {
    /* weight of the high endpoint per index (thirds), and the normal
     * equations' sums packed as xx << 16 | yy << 8 | xy */
    static const int w1[4] = {3, 0, 2, 1};
    static const int packed[4] = {0x090000, 0x000900, 0x040102, 0x010402};
    int acc = 0, a1[3] = {0, 0, 0}, a2[3] = {0, 0, 0};
    uint32_t m = mask;
    for (int i = 0; i < 16; i++, m >>= 2) {
      const int step = (int)(m & 3);
      acc += packed[step];
      for (int c = 0; c < 3; c++) {
        a1[c] += w1[step] * px[i][c];
        a2[c] += px[i][c];
      }
    }
    for (int c = 0; c < 3; c++) a2[c] = 3 * a2[c] - a1[c];
    const int xx = acc >> 16, yy = (acc >> 8) & 0xff, xy = acc & 0xff;
    const float frb = 3.0f * 31.0f / 255.0f / (float)(xx * yy - xy * xy);
    const float fg = frb * 63.0f / 31.0f;
    mx16 = (uint16_t)(clamp_trunc((float)(a1[0] * yy - a2[0] * xy) * frb + 0.5f, 31) << 11);
    mx16 |= (uint16_t)(clamp_trunc((float)(a1[1] * yy - a2[1] * xy) * fg + 0.5f, 63) << 5);
    mx16 |= (uint16_t)clamp_trunc((float)(a1[2] * yy - a2[2] * xy) * frb + 0.5f, 31);
    mn16 = (uint16_t)(clamp_trunc((float)(a2[0] * xx - a1[0] * xy) * frb + 0.5f, 31) << 11);
    mn16 |= (uint16_t)(clamp_trunc((float)(a2[1] * xx - a1[1] * xy) * fg + 0.5f, 63) << 5);
    mn16 |= (uint16_t)clamp_trunc((float)(a2[2] * xx - a1[2] * xy) * frb + 0.5f, 31);
  }
  *min16 = mn16;
  *max16 = mx16;
  return old_min != mn16 || old_max != mx16;
}

/* stb_dxt.h:477-549 */
static void color_block(const uint8_t px[16][4], uint8_t out[8]) {
  uint32_t mask;
  uint16_t mx16, mn16;
  int same = 1;
  for (int i = 1; i < 16; i++) same = same && memcmp(px[i], px[0], 4) == 0;
  if (same) {
    const int r = px[0][0], g = px[0][1], b = px[0][2];
    mask = 0xaaaaaaaau;
    mx16 = (uint16_t)((gMatch5[r][0] << 11) | (gMatch6[g][0] << 5) | gMatch5[b][0]);
    mn16 = (uint16_t)((gMatch5[r][1] << 11) | (gMatch6[g][1] << 5) | gMatch5[b][1]);
  } else {
    uint8_t d[16][4];
    memset(d, 0, sizeof(d));
    dither(px, d);
    axis_endpoints((const uint8_t(*)[4])d, &mx16, &mn16);
    int col[4][3];
    if (mx16 != mn16) {
      palette(col, mx16, mn16);
      mask = match(px, col);
    } else {
      mask = 0;
    }
    if (refine((const uint8_t(*)[4])d, &mx16, &mn16, mask)) {
      if (mx16 != mn16) {
        palette(col, mx16, mn16);
        mask = match(px, col);
      } else {
        mask = 0;
      }
    }
  }
  if (mx16 < mn16) {
    const uint16_t t = mn16;
    mn16 = mx16;
    mx16 = t;
    mask ^= 0x55555555u;
  }
  out[0] = (uint8_t)mx16;
  out[1] = (uint8_t)(mx16 >> 8);
  out[2] = (uint8_t)mn16;
  out[3] = (uint8_t)(mn16 >> 8);
  for (int k = 0; k < 4; k++) out[4 + k] = (uint8_t)(mask >> (8 * k));
}

/* stb_dxt.h:551-601 */
static void alpha_block(const uint8_t px[16][4], uint8_t out[8]) {
  int mn = px[0][3], mx = px[0][3];
  for (int i = 1; i < 16; i++) {
    if (px[i][3] < mn) mn = px[i][3];
    else if (px[i][3] > mx) mx = px[i][3];
  }
  out[0] = (uint8_t)mx;
  out[1] = (uint8_t)mn;
  const int dist = mx - mn, dist4 = dist * 4, dist2 = dist * 2;
  int bias = dist < 8 ? dist - 1 : dist / 2 + 2;
  bias -= mn * 7;
  uint64_t bits = 0;
  for (int i = 0; i < 16; i++) {
    int a = px[i][3] * 7 + bias, ind = 0;
    if (a >= dist4) {
      ind = 4;
      a -= dist4;
    }
    if (a >= dist2) {
      ind += 2;
      a -= dist2;
    }
    ind += a >= dist;
    ind = -ind & 7; /* the linear scale 0..7 to DXT5 order: 0 and 1 are the ends */
    ind ^= 2 > ind;
    bits |= (uint64_t)ind << (3 * i);
  }
  for (int k = 0; k < 6; k++) out[2 + k] = (uint8_t)(bits >> (8 * k));
}

/* stb_compress_dxt_block (stb_dxt.h:623-637) with STB_DXT_DITHER */
void dxto_compress_block(const uint8_t rgba[64], int alpha, uint8_t *out) {
  init_tables();
  uint8_t px[16][4];
  memcpy(px, rgba, 64);
  if (alpha) {
    alpha_block((const uint8_t(*)[4])px, out);
    out += 8;
  }
  color_block((const uint8_t(*)[4])px, out);
}

int dxto_compress(const uint8_t *rgba, uint8_t *out, uint32_t w, uint32_t h, int alpha) {
  if ((w | h) & 3) return -1;
  const uint32_t bsz = alpha ? 16 : 8, bw = w / 4;
  for (uint32_t by = 0; by < h / 4; by++)
    for (uint32_t bx = 0; bx < bw; bx++) {
      uint8_t blk[64];
      for (int r = 0; r < 4; r++)
        memcpy(blk + 16 * r, rgba + 4 * ((size_t)(4 * by + r) * w + 4 * bx), 16);
      dxto_compress_block(blk, alpha, out + bsz * ((size_t)by * bw + bx));
    }
  return 0;
}

/* DecompressDXT1Block (Decompressor.cpp:28-65) */
static void decode_colors(const uint8_t *b, int four, uint32_t out[16], int keep_alpha) {
  const uint16_t c0 = (uint16_t)(b[0] | (b[1] << 8)), c1 = (uint16_t)(b[2] | (b[3] << 8));
  int col[4][3];
  from565(c0, col[0]);
  from565(c1, col[1]);
  if (four || c0 > c1) {
    for (int k = 0; k < 3; k++) {
      col[2][k] = (2 * col[0][k] + col[1][k]) / 3;
      col[3][k] = (col[0][k] + 2 * col[1][k]) / 3;
    }
  } else {
    for (int k = 0; k < 3; k++) {
      col[2][k] = (col[0][k] + col[1][k]) / 2;
      col[3][k] = 0;
    }
  }
  const uint32_t m = (uint32_t)b[4] | ((uint32_t)b[5] << 8) | ((uint32_t)b[6] << 16) |
                     ((uint32_t)b[7] << 24);
  for (int i = 0; i < 16; i++) {
    const int *c = col[(m >> (2 * i)) & 3];
    const uint32_t rgb = (uint32_t)c[0] | ((uint32_t)c[1] << 8) | ((uint32_t)c[2] << 16);
    out[i] = keep_alpha ? (out[i] & 0xFF000000u) | rgb : 0xFF000000u | rgb;
  }
}

/* DecompressDXT5Block (Decompressor.cpp:67-96) */
static void decode_alpha(const uint8_t *b, uint32_t out[16]) {
  const int a0 = b[0], a1 = b[1];
  int pal[8] = {a0, a1, 0, 0, 0, 0, 0, 0};
  if (a0 > a1) {
    for (int i = 2; i < 8; i++) pal[i] = ((8 - i) * a0 + (i - 1) * a1) / 7;
  } else {
    for (int i = 2; i < 6; i++) pal[i] = ((6 - i) * a0 + (i - 1) * a1) / 5;
    pal[6] = 0;
    pal[7] = 255;
  }
  uint64_t m = 0;
  for (int k = 0; k < 6; k++) m |= (uint64_t)b[2 + k] << (8 * k);
  for (int i = 0; i < 16; i++) out[i] = (out[i] & 0x00FFFFFFu) | ((uint32_t)pal[(m >> (3 * i)) & 7] << 24);
}

void dxto_decompress(const uint8_t *blocks, uint8_t *rgba, uint32_t w, uint32_t h, int alpha) {
  init_tables();
  const uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4, bsz = alpha ? 16 : 8;
  for (uint32_t by = 0; by < bh; by++)
    for (uint32_t bx = 0; bx < bw; bx++) {
      const uint8_t *b = blocks + bsz * ((size_t)by * bw + bx);
      uint32_t px[16];
      for (int i = 0; i < 16; i++) px[i] = 0xFFFFFFFFu;
      if (alpha) {
        decode_alpha(b, px);
        decode_colors(b + 8, 1, px, 1);
      } else {
        decode_colors(b, 0, px, 0);
      }
      for (uint32_t y = 0; y < 4 && 4 * by + y < h; y++)
        for (uint32_t x = 0; x < 4 && 4 * bx + x < w; x++)
          memcpy(rgba + 4 * ((size_t)(4 * by + y) * w + 4 * bx + x), &px[4 * y + x], 4);
    }
}

void dxto_tables(uint8_t match5[512], uint8_t match6[512]) {
  init_tables();
  memcpy(match5, gMatch5, 512);
  memcpy(match6, gMatch6, 512);
}
