/*
 * bc7_oracle.h -- CPU restatement of FasTC's BC7 (BPTC) encoder and decoder.
 *
 * TEST INFRASTRUCTURE ONLY. The product library never includes, links or
 * calls this code; tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline use it as the checker.
 *
 * Parity pin: at steps == 0 the blocks are checked byte-for-byte against the
 * reference library itself (oracle/_ref, built in place from the FasTC
 * sources) and against committed golden fixtures made from it. At steps > 0
 * with rng_mode == BC7O_RNG_SINGLE_STREAM and exp_mode == BC7O_EXP_LIBM the
 * oracle threads one LCG stream through every fit in the reference's order,
 * exactly as BPTCEncoder/src/Compressor.cpp does, and is checked
 * byte-for-byte against the reference with a pinned seed.
 */
#ifndef FASTC_BC7_ORACLE_H_
#define FASTC_BC7_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  /* One LCG stream per cluster fit, seeded from (seed, block x, block y,
   * fit id). Independent of scheduling; this is what the GPU encoder does. */
  BC7O_RNG_PER_FIT = 0,
  /* One LCG stream for the whole image, consumed in raster/mode order like
   * the reference's process-global g_seed (Compressor.cpp:358). */
  BC7O_RNG_SINGLE_STREAM = 1
};

enum {
  BC7O_EXP_PORTABLE = 0, /* the float exp the GPU encoder uses */
  BC7O_EXP_LIBM = 1      /* double exp() as in Compressor.cpp:531 */
};

typedef struct {
  uint32_t steps;       /* simulated-annealing steps (tc -q) */
  uint32_t block_modes; /* EBlockMode bit mask, 0xFF = all */
  uint32_t metric;      /* 0 uniform, 1 nonuniform */
  uint32_t rng_mode;    /* BC7O_RNG_* */
  uint32_t seed;        /* per-fit seed, or the initial LCG state */
  uint32_t exp_mode;    /* BC7O_EXP_* */
} bc7o_settings;

/* Compress the block-aligned rectangle [x0,x1) x [y0,y1) of a w x h RGBA8
 * image (x1/y1 == 0 mean w/h). Blocks land at their global block index in
 * `out` (w*h bytes). state[0] is the LCG state for the single-stream mode,
 * state[1] the watermark counter (number of single-colour blocks written so
 * far); both are read and updated. Returns 0 or a negative error. */
int bc7o_compress(const uint8_t *rgba, uint8_t *out, uint32_t w, uint32_t h,
                  uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                  const bc7o_settings *s, uint32_t state[2]);

/* Multi-threaded whole-image compression with the per-fit RNG (the result is
 * identical to bc7o_compress for any thread count). */
int bc7o_compress_mt(const uint8_t *rgba, uint8_t *out, uint32_t w,
                     uint32_t h, const bc7o_settings *s, uint32_t wm_start,
                     int nthreads);

/* One block: px = 16 RGBA8 texels (R in bits 0-7), bx/by = block coordinates
 * (keys the per-fit RNG), wm = watermark counter, lcg = single-stream state. */
void bc7o_compress_block(const uint32_t px[16], const bc7o_settings *s,
                         uint32_t bx, uint32_t by, uint32_t *wm, uint32_t *lcg,
                         uint8_t out[16]);

/* One cluster fit of a traced block, in CompressClusters' order. */
typedef struct {
  int32_t mode, slot, subset;
  int32_t rot_im;      /* rotation << 1 | index mode (modes 4, 5), else -1 */
  int32_t n, annealed; /* point count; 1 when the fit took the QuantizedError
                          path (not FasTC's single-colour shortcut) */
  double init_err;     /* its error before the annealing (alpha error included) */
  double final_err;    /* CompressCluster's return value */
  double lower_bound;  /* the GPU pipeline's bound (its error when not annealed) */
} bc7o_fit_trace;

/* bc7o_compress_block, also listing the block's cluster fits (at most cap;
 * returns how many were recorded). Diagnostic: checks the pipeline's
 * pruning rule against the whole algorithm. */
/* Diagnostic work counters summed over all threads since the last reset:
 * out[0] = QuantizedError calls, out[1] = texel-bucket evaluations (one per
 * palette entry a texel is compared with). reset != 0 zeroes them after
 * reading. */
void bc7o_qe_counters(uint64_t out[2], int reset);

/* Diagnostic: leave the palette-size term out of the traced bounds (0) or
 * put it back (1, the default). */
void bc7o_set_level_bound(int on);

int bc7o_trace_block(const uint32_t px[16], const bc7o_settings *s, uint32_t bx,
                     uint32_t by, uint32_t *wm, uint32_t *lcg, uint8_t out[16],
                     bc7o_fit_trace *fits, int cap);

/* What CompressWithStats logs for one block (Compressor.cpp:1938-2183):
 * the path (0 single colour, 1 transparent, 2 an exact shape, 3 searched),
 * the packed mode, each mode's error estimate and logged error (-1 when
 * unset), and every improving 2- and 3-subset shape estimate in order. */
typedef struct {
  int32_t path, mode;
  double estimate[8], error[8];
  int32_t n_two, n_three;
  double two_shape[64], three_shape[64];
} bc7o_block_stats;

/* One block through the logging encoder (its own shape selection). */
void bc7o_compress_block_stats(const uint32_t px[16], const bc7o_settings *s,
                               uint32_t bx, uint32_t by, uint32_t *wm,
                               uint32_t *lcg, uint8_t out[16],
                               bc7o_block_stats *st);

void bc7o_decompress(const uint8_t *blocks, uint8_t *rgba, uint32_t w,
                     uint32_t h);

/* Image::ComputePSNR (Base/src/Image.cpp:206-255). */
double bc7o_psnr(const uint8_t *a, const uint8_t *b, uint32_t w, uint32_t h);

/* Per-block sum of squared alpha-premultiplied RGB differences, in units of
 * 1/255^2 (the same metric as the PSNR), one double per 4x4 block. */
void bc7o_block_sse(const uint8_t *a, const uint8_t *b, uint32_t w,
                    uint32_t h, double *sse);

/* out[0] shapes searched, out[1] two-subset shape, out[2] three-subset
 * shape or 0xFFFFFFFF, out[3] selected modes (before the settings mask). */
void bc7o_box_selection(const uint32_t px[16], uint32_t metric,
                        uint32_t out[4]);

/* The two endpoint lookup tables, regenerated from their documented
 * generator (BCLookupTables.h:44-95 and :355-449). */
void bc7o_tables(uint8_t opt7[512], uint8_t opt6[1536]);

/* Partition table access: subset of each texel, and anchor texel of a
 * subset. */
void bc7o_partition(uint32_t shape, uint32_t nsubsets, uint8_t out[16]);
uint32_t bc7o_anchor(uint32_t subset, uint32_t shape, uint32_t nsubsets);

/* The per-fit LCG seed and the portable exp, exposed for tests. */
uint32_t bc7o_fit_seed(uint32_t seed, uint32_t bx, uint32_t by, uint32_t fit);
float bc7o_expf(float x);

#ifdef __cplusplus
}
#endif
#endif
