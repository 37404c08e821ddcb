// Block-level pieces of the BC7 search shared by the encoder kernels:
// FasTC's BoxSelection (shape estimate), the enumeration of the cluster fits
// CompressClusters runs, and the 128-bit packing. File:line citations are
// into FasTC's BPTCEncoder/src/Compressor.cpp (CP).
#pragma once

#include <cfloat>
#include <cstdint>

#include "bc7_encode.cuh"
#include "bc7_format.cuh"
#include "bc7_kernels.cuh"

namespace fastc {

constexpr uint32_t kModesTwo = (1u << 1) | (1u << 3) | (1u << 7);
constexpr uint32_t kModesThree = (1u << 0) | (1u << 2);
constexpr uint32_t kModesAlpha = (1u << 4) | (1u << 5) | (1u << 6) | (1u << 7);
// CompressClusters' mode order (CP:1757)
__host__ __device__ constexpr int mode_order(int i) {
  return i == 0 ? 0 : i == 1 ? 2 : i == 2 ? 1 : i == 3 ? 3 : i == 4 ? 7 : i == 5 ? 4 : i == 6 ? 5 : 6;
}

struct __align__(8) FitOut {
  double err;
  float p1[4], p2[4];
  uint64_t idx;   // 4 bits per texel
  uint64_t aidx;  // 4 bits per texel (rotation modes)
  uint32_t pbit;
  uint32_t pad;
};

struct Selection {
  uint32_t nshapes;
  uint32_t shape[2];
  uint32_t nparts[2];
  uint32_t modes;
};

struct Task {
  int mode, slot, subset, rot, im;
};

constexpr int kMaxTasks = 32;
constexpr uint32_t kStatusTaskOverflow = 2u;

// EstimateTwoClusterError / EstimateThreeClusterError (CP:1626-1655)
__device__ inline double estimate_shape(const uint32_t *px, uint32_t part, int nsub, int bits,
                                 const float *w) {
  double err = 0.0;
  for (int ci = 0; ci < nsub; ci++) {
    Cluster c;
    uint32_t buf[16];
    make_cluster(px, part, ci, buf, 1, c);
    float v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = __fsub_rn(c.mx[k], c.mn[k]);
    double e = 0.0;
    if (sqlen4(v) != 0.0f) {
      e = 0.0001;
      e = e + (double)quantized_error(c, c.mn, c.mx, bits, 0xFFFFFFFFu, w, -1, nullptr);
    }
    err = err + e;
  }
  return err;
}

__device__ __forceinline__ void argmin_pair(double &e, int &i, double oe, int oi) {
  if (oe < e || (oe == e && oi < i)) {
    e = oe;
    i = oi;
  }
}

// BoxSelection (CP:1670-1750), 64 shapes spread two per lane.
__device__ inline Selection box_selection_warp(const uint32_t *px, const uint32_t *part2,
                                        const uint32_t *part3, int metric, int lane) {
  Selection r;
  r.nshapes = 1;
  r.shape[0] = r.shape[1] = 0;
  r.nparts[0] = 2;
  r.nparts[1] = 0;
  r.modes = 0xFF;
  bool opaque = true;
  for (int i = 0; i < 16; i++) opaque = opaque && ((px[i] >> 24) >= 250);
  float w[4];
#pragma unroll
  for (int c = 0; c < 4; c++) w[c] = base_weight(metric, c);

  for (int pass = 0; pass < 2; pass++) {
    const uint32_t *part = pass ? part3 : part2;
    const int nsub = pass ? 3 : 2, bits = pass ? 2 : 3;
    const double e0 = estimate_shape(px, part[lane], nsub, bits, w);
    const double e1 = estimate_shape(px, part[lane + 32], nsub, bits, w);
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

// The cluster fits CompressClusters (CP:1752-1817) runs, in its order.
// Returns the number of tasks; fills `t` with task `want` if it exists.
__device__ inline int enumerate_tasks(const Selection &sel, uint32_t modes, int want, Task &t) {
  int n = 0;
  const uint32_t nshapes = sel.nshapes < 5 ? sel.nshapes : 5;
  for (int oi = 0; oi < 8; oi++) {
    const int mode = mode_order(oi);
    if (!(modes & (1u << mode))) continue;
    const ModeAttr a = mode_attr(mode);
    for (uint32_t s = 0; s < nshapes; s++) {
      if (a.subsets != 1 && (uint32_t)a.subsets != sel.nparts[s]) continue;
      if (sel.shape[s] >= 16 && mode == 0) continue;
      if (a.has_rotation) {
        const int nim = mode == 4 ? 2 : 1;
        for (int rot = 0; rot < 4; rot++)
          for (int im = 0; im < nim; im++) {
            if (n == want) t = Task{mode, (int)s, 0, rot, im};
            n++;
          }
      } else {
        for (int ci = 0; ci < a.subsets; ci++) {
          if (n == want) t = Task{mode, (int)s, ci, 0, 0};
          n++;
        }
      }
    }
  }
  return n;
}

__device__ inline void run_task(const Task &t, const Selection &sel, const uint32_t *px,
                         const uint32_t *part2, const uint32_t *part3, const uint32_t *opt6,
                         const JobDev &jb, uint32_t bx, uint32_t by, uint32_t *status,
                         FitOut &o) {
  ModeCtx m;
  m.mode = t.mode;
  m.a = mode_attr(t.mode);
  m.steps = (int)jb.steps;
  m.metric = (int)jb.metric;
  m.rot = t.rot;
  m.idx_mode = t.im;
  m.status = status;
  m.sct = nullptr;
  m.pal = nullptr;
  m.lcg = fit_seed(jb.seed, bx, by,
                   (uint32_t)((t.mode << 8) | (t.slot << 7) | (t.subset << 4) | (t.rot << 1) | t.im));
  const uint32_t shape = sel.shape[t.slot];
  const uint32_t part = m.a.subsets == 2 ? part2[shape] : (m.a.subsets == 3 ? part3[shape] : 0u);
  Cluster c;
  uint32_t buf[16], aux[16];
  make_cluster(px, part, t.subset, buf, 1, c);
  c.aux = aux;
  c.aux_stride = 1;
  o.idx = 0;
  o.aidx = 0;
  o.pbit = 0;
  if (m.a.has_rotation) {
    o.err = fit_alpha(m, c, opt6, o.p1, o.p2, o.idx, o.aidx);
  } else {
    uint32_t pb = 0xFF;
    o.err = fit_rgb(m, c, o.p1, o.p2, o.idx, pb);
    o.pbit = pb;
  }
}

struct BitWriter {
  uint32_t w[4];
  int pos;
  __device__ void put(uint32_t v, int n) {
    for (int i = 0; i < n && pos < 128; i++, pos++) {
      const uint32_t bit = i < 32 ? (v >> i) & 1u : 0u;
      w[pos >> 5] |= bit << (pos & 31);
    }
  }
};

// CompressionMode::Pack (CP:1096-1298) from the winning fits.
__device__ inline void pack_block(int mode, const Selection &sel, int slot, const FitOut *fits,
                           const uint8_t *anc2, const uint8_t *anc3, const uint32_t *part2,
                           const uint32_t *part3, int rot, int im, uint32_t out[4]) {
  const ModeAttr a = mode_attr(mode);
  const int nsub = a.subsets;
  const uint32_t shape = sel.shape[slot];
  const uint32_t part = nsub == 2 ? part2[shape] : (nsub == 3 ? part3[shape] : 0u);
  BitWriter bw;
  bw.w[0] = bw.w[1] = bw.w[2] = bw.w[3] = 0;
  bw.pos = 0;
  bw.put(1u << mode, mode + 1);
  bw.put(shape, a.part_bits);
  bw.put((uint32_t)rot, a.has_rotation ? 2 : 0);
  bw.put((uint32_t)im, a.has_idx_mode ? 1 : 0);
  const uint32_t qm = qmask_of(a);
  uint32_t px1[3], px2[3], idx[3];
  uint64_t idxs[3];
  uint64_t aidx = fits[0].aidx;
  for (int s = 0; s < nsub; s++) {
    const FitOut &f = fits[s];
    if (a.pbit == kPBitNone) {
      px1[s] = to_pixel(f.p1, qm, -1);
      px2[s] = to_pixel(f.p2, qm, -1);
    } else {
      const int pc = pbit_combo(a, (int)f.pbit);
      px1[s] = to_pixel(f.p1, qm, pb_first(pc));
      px2[s] = to_pixel(f.p2, qm, pb_second(pc));
    }
    idxs[s] = f.idx;
    (void)idx;
  }
  ModeCtx m0;
  m0.a = a;
  m0.idx_mode = 0;
  const int nib = bits_index(m0, im), nab = bits_alpha(m0, im);
  const uint64_t ones = 0x1111111111111111ull;
  for (int s = 0; s < nsub; s++) {
    const int anchor = s == 0 ? 0 : (nsub == 2 ? anc2[shape] : (s == 1 ? (anc3[shape] & 15) : (anc3[shape] >> 4)));
    if (get_nib(idxs[s], anchor) >> (nib - 1)) {
      const uint32_t t = px1[s];
      px1[s] = px2[s];
      px2[s] = t;
      idxs[s] = ones * (uint64_t)((1u << nib) - 1u) - idxs[s];
      if (a.has_rotation) aidx = ones * (uint64_t)((1u << nab) - 1u) - aidx;
    }
    if (a.has_rotation && (get_nib(aidx, anchor) >> (nab - 1)) > 0) {
      const uint32_t h1 = px1[s] & 0xFF000000u, h2 = px2[s] & 0xFF000000u;
      px1[s] = (px1[s] & 0x00FFFFFFu) | h2;
      px2[s] = (px2[s] & 0x00FFFFFFu) | h1;
      aidx = ones * (uint64_t)((1u << nab) - 1u) - aidx;
    }
  }
  for (int ch = 0; ch < 4; ch++) {
    const int bits = ch == 3 ? a.alpha_bits : a.color_bits;
    for (int s = 0; s < nsub; s++) {
      bw.put(((px1[s] >> (8 * ch)) & 0xFF) >> (8 - bits), bits);
      bw.put(((px2[s] >> (8 * ch)) & 0xFF) >> (8 - bits), bits);
    }
  }
  if (a.pbit != kPBitNone)
    for (int s = 0; s < nsub; s++) {
      const int pc = pbit_combo(a, (int)fits[s].pbit);
      bw.put((uint32_t)pb_first(pc), 1);
      if (a.pbit != kPBitShared) bw.put((uint32_t)pb_second(pc), 1);
    }
  if (a.has_idx_mode && im == 1) {
    for (int i = 0; i < 16; i++) bw.put(get_nib(aidx, i), i == 0 ? 1 : 2);
    for (int i = 0; i < 16; i++) bw.put(get_nib(idxs[0], i), i == 0 ? 2 : 3);
  } else {
    for (int i = 0; i < 16; i++) {
      const int s = (int)((part >> (2 * i)) & 3);
      const int anchor = s == 0 ? 0 : (nsub == 2 ? anc2[shape] : (s == 1 ? (anc3[shape] & 15) : (anc3[shape] >> 4)));
      bw.put(get_nib(idxs[s], i), i == anchor ? nib - 1 : nib);
    }
    if (a.has_rotation)
      for (int i = 0; i < 16; i++) bw.put(get_nib(aidx, i), i == 0 ? nab - 1 : nab);
  }
  out[0] = bw.w[0];
  out[1] = bw.w[1];
  out[2] = bw.w[2];
  out[3] = bw.w[3];
}

__device__ inline void single_color_block(uint32_t pixel, uint32_t wm, const uint32_t *opt7,
                                   const uint32_t *watermark, uint32_t out[4]) {
  BitWriter bw;
  bw.w[0] = bw.w[1] = bw.w[2] = bw.w[3] = 0;
  bw.pos = 0;
  bw.put(1u << 5, 6);
  bw.put(0, 2);
  for (int c = 0; c < 3; c++) {
    const uint32_t e = opt7[(pixel >> (8 * c)) & 0xFF];
    bw.put(e & 0xFF, 7);
    bw.put((e >> 8) & 0xFF, 7);
  }
  bw.put(pixel >> 24, 8);
  bw.put(pixel >> 24, 8);
  bw.put(0xaaaaaaabu, 31);
  bw.put(watermark[wm % 9], 31);
  for (int i = 0; i < 4; i++) out[i] = bw.w[i];
}


}  // namespace fastc
