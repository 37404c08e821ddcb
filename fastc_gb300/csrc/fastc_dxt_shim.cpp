// Drop-in replacement for FasTC's DXT library entry points.
//
// Compile this file against FasTC's own headers (Base/include,
// DXTEncoder/include) and link it, with libfastc_bc7.so, in place of
// DXTEncoder/src/Compressor.cpp and Decompressor.cpp. Core's format
// dispatch (Core/src/TexComp.cpp:130-134 picks DXTC::CompressImageDXT1 /
// CompressImageDXT5) and tc then encode DXT1 / DXT5 on the GPU without
// source changes, producing the same bytes.
//
// Each function keeps the reference signature from
// DXTEncoder/include/FasTC/DXTCompressor.h:22-29. The reference functions
// return void; these print the C-ABI status and abort on failure, so a
// failure is never silent.
#include <cstdio>
#include <cstdlib>

#include "FasTC/DXTCompressor.h"
#include "fastc_bc7.h"

namespace {

void Die(const char *where, fastc_bc7_status st) {
  std::fprintf(stderr, "fastc_dxt: %s failed: %s %s\n", where, fastc_bc7_status_string(st),
               fastc_bc7_last_error());
  std::abort();
}

void Compress(const FasTC::CompressionJob &cj, int format, const char *where) {
  fastc_bc7_job j;
  j.in = cj.InBuf();
  j.out = cj.OutBuf();
  j.width = cj.Width();
  j.height = cj.Height();
  j.x_start = cj.XStart();
  j.y_start = cj.YStart();
  j.x_end = cj.XEnd();
  j.y_end = cj.YEnd();
  const fastc_bc7_status st = fastc_dxt_compress(&j, format);
  if (st != FASTC_BC7_OK) Die(where, st);
}

void Decompress(const FasTC::DecompressionJob &dcj, int format, const char *where) {
  const fastc_bc7_status st =
      fastc_dxt_decompress(dcj.InBuf(), dcj.OutBuf(), dcj.Width(), dcj.Height(), format);
  if (st != FASTC_BC7_OK) Die(where, st);
}

}  // namespace

namespace DXTC {

void CompressImageDXT1(const FasTC::CompressionJob &cj) { Compress(cj, FASTC_DXT1, "CompressImageDXT1"); }

void CompressImageDXT5(const FasTC::CompressionJob &cj) { Compress(cj, FASTC_DXT5, "CompressImageDXT5"); }

void DecompressDXT1(const FasTC::DecompressionJob &dcj) { Decompress(dcj, FASTC_DXT1, "DecompressDXT1"); }

void DecompressDXT5(const FasTC::DecompressionJob &dcj) { Decompress(dcj, FASTC_DXT5, "DecompressDXT5"); }

}  // namespace DXTC
