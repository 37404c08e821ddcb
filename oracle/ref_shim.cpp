// Test infrastructure only: never linked into the product library.
//
// Compiles FasTC's own BPTC encoder (BPTCEncoder/src/Compressor.cpp) in place,
// from the reference checkout named by the Makefile, and exposes a flat C ABI
// over it so the tests can use the unmodified reference as an oracle:
//
//   * ref_compress        -> BPTCC::Compress            (Compressor.cpp:1473)
//   * ref_decompress      -> BPTCC::Decompress          (Decompressor.cpp:345)
//   * ref_box_selection   -> BoxSelection               (Compressor.cpp:1670)
//   * ref_compress_block  -> CompressBC7Block           (Compressor.cpp:1819)
//   * ref_compress_stats  -> BPTCC::CompressWithStats   (Compressor.cpp:1577),
//                            with its per-block log captured as text
//   * ref_{get,set}_seed  -> g_seed, the annealing LCG  (Compressor.cpp:358)
//   * ref_{get,set}_wm    -> gWMVal, the single-colour watermark counter
//                            (Compressor.cpp:140)
//   * ref_tables          -> the two endpoint lookup tables used on the
//                            encode path (BCLookupTables.h:97,710)
//   * ref_dxt_compress    -> DXTC::CompressImageDXT1 / DXT5
//                            (DXTEncoder/src/Compressor.cpp:44-93, compiled
//                            from its own file by the Makefile)
//   * ref_dxt_decompress  -> DXTC::DecompressDXT1 / DXT5
//                            (DXTEncoder/src/Decompressor.cpp:94-155)
//
// g_seed is seeded from time(NULL) at load time, which makes q>0 output
// nondeterministic; the tests pin it with ref_set_seed before every call.
// The reference file is included, not copied: this translation unit only
// adds accessors for its file-static state.

#include "Compressor.cpp"

#include <cstdint>

#include "FasTC/DXTCompressor.h"

extern "C" {

void ref_set_seed(uint32_t s) { BPTCC::g_seed = s; }
uint32_t ref_get_seed(void) { return BPTCC::g_seed; }
void ref_set_wm(uint32_t v) { BPTCC::gWMVal = v; }
uint32_t ref_get_wm(void) { return BPTCC::gWMVal; }

static BPTCC::CompressionSettings MakeSettings(uint32_t steps, uint32_t modes,
                                               int metric) {
  BPTCC::CompressionSettings s;
  s.m_NumSimulatedAnnealingSteps = steps;
  s.m_BlockModes = modes;
  s.m_ErrorMetric = static_cast<BPTCC::ErrorMetric>(metric);
  return s;
}

void ref_compress(const uint8_t *rgba, uint8_t *out, uint32_t w, uint32_t h,
                  uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                  uint32_t steps, uint32_t modes, int metric) {
  FasTC::CompressionJob cj(FasTC::eCompressionFormat_BPTC, rgba, out, w, h,
                           x0, y0, x1, y1);
  BPTCC::Compress(cj, MakeSettings(steps, modes, metric));
}

void ref_compress_block(const uint32_t px[16], uint8_t out[16], uint32_t steps,
                        uint32_t modes, int metric) {
  BPTCC::CompressBC7Block(0, 0, px, out, MakeSettings(steps, modes, metric));
}

void ref_decompress(const uint8_t *blocks, uint8_t *rgba, uint32_t w,
                    uint32_t h) {
  FasTC::DecompressionJob dj(FasTC::eCompressionFormat_BPTC, blocks, rgba, w,
                             h);
  BPTCC::Decompress(dj);
}

// out[0] = number of shapes, out[1] = two-subset shape, out[2] = three-subset
// shape (or 0xFFFFFFFF), out[3] = selected mode mask.
void ref_box_selection(const uint32_t px[16], int metric, uint32_t out[4]) {
  BPTCC::ErrorMetric m = static_cast<BPTCC::ErrorMetric>(metric);
  BPTCC::ShapeSelection s = BPTCC::BoxSelection(0, 0, px, &m);
  out[0] = s.m_NumShapesToSearch;
  out[1] = s.m_Shapes[0].m_Index;
  out[2] = s.m_NumShapesToSearch > 1 ? s.m_Shapes[1].m_Index : 0xFFFFFFFFu;
  out[3] = s.m_SelectedModes;
}

// One CompressionMode::Compress call (Compressor.cpp:1300) for debugging:
// returns the error, leaves g_seed advanced.
double ref_compress_mode(const uint32_t px[16], int mode, int shape,
                         uint32_t steps) {
  BPTCC::CompressionSettings s = MakeSettings(steps, 0xFF, 0);
  RGBACluster cluster(px);
  const int nparts = BPTCC::CompressionMode::GetAttributesForMode(mode)->numSubsets;
  cluster.SetShapeIndex(shape, nparts);
  BPTCC::CompressionMode::Params params;
  return BPTCC::CompressionMode(mode, s).Compress(params, shape, cluster);
}

// CompressWithStats over a job rectangle with a log stream: returns the
// log's length and copies at most cap - 1 bytes of it, NUL-terminated.
size_t ref_compress_stats(const uint8_t *rgba, uint8_t *out, uint32_t w, uint32_t h,
                          uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                          uint32_t steps, uint32_t modes, int metric, char *log,
                          size_t cap) {
  FasTC::CompressionJob cj(FasTC::eCompressionFormat_BPTC, rgba, out, w, h,
                           x0, y0, x1, y1);
  std::stringstream ss;
  BPTCC::CompressWithStats(cj, &ss, MakeSettings(steps, modes, metric));
  const std::string text = ss.str();
  if (cap > 0) {
    const size_t n = text.size() < cap - 1 ? text.size() : cap - 1;
    memcpy(log, text.data(), n);
    log[n] = 0;
  }
  return text.size();
}

void ref_tables(uint8_t opt7[512], uint8_t opt6[1536]) {
  memcpy(opt7, ::Optimal7CompressBC7Mode5, 512);
  memcpy(opt6, ::Optimal6CompressDXT1, 1536);
}


void ref_dxt_compress(const uint8_t *rgba, uint8_t *out, uint32_t w, uint32_t h, int alpha) {
  FasTC::CompressionJob cj(alpha ? FasTC::eCompressionFormat_DXT5 : FasTC::eCompressionFormat_DXT1,
                           rgba, out, w, h);
  if (alpha) DXTC::CompressImageDXT5(cj);
  else DXTC::CompressImageDXT1(cj);
}

void ref_dxt_decompress(const uint8_t *blocks, uint8_t *rgba, uint32_t w, uint32_t h, int alpha) {
  FasTC::DecompressionJob dj(alpha ? FasTC::eCompressionFormat_DXT5 : FasTC::eCompressionFormat_DXT1,
                             blocks, rgba, w, h);
  if (alpha) DXTC::DecompressDXT5(dj);
  else DXTC::DecompressDXT1(dj);
}

}  // extern "C"
