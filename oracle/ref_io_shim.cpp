// Test infrastructure only: never linked into the product library.
//
// FasTC's own steps of `tc` after the encode, compiled in place from the
// reference checkout named by the Makefile (built into the same test library
// as ref_shim.cpp):
//
//   * ref_tc_psnr -> the PSNR tc prints: img.ComputePSNR(ci)
//                    (CLTool/src/tc.cpp:302), i.e. Image<Pixel>::ComputePSNR
//                    (Base/src/Image.cpp:206-255) against a CompressedImage
//                    that decodes itself with FasTC's BPTC / DXT decoders
//                    (Core/src/CompressedImage.cpp:86-134)
//   * ref_ktx     -> the KTX file tc writes for `-d out.ktx`
//                    (CLTool/src/tc.cpp:336-337 -> IO/src/ImageFile.cpp:132-160
//                    -> ImageWriterKTX::WriteImage, IO/src/ImageWriterKTX.cpp:69-161)
//   * ref_load_ktx -> the texels tc compresses for an uncompressed .ktx input
//                    (ImageLoaderKTX::LoadImage / ReadData,
//                    IO/src/ImageLoaderKTX.cpp:108-346)
//   * ref_load_tga -> the texels tc compresses for a .tga input
//                    (ImageLoaderTGA::ReadData, IO/src/ImageLoaderTGA.cpp:35-48,
//                    over IO/third_party/tga/targa.c, then ImageLoader::LoadImage,
//                    IO/src/ImageLoader.cpp:151-215)
//
// ImageWriterKTX keeps the image size in a function-local static
// (ImageWriterKTX.cpp:143,149,153), so only the first file a process writes per
// format group carries its own size; the fixture generator writes each KTX
// fixture from a fresh process, as one run of tc does.
//
// CompressedImage::DecompressImage also names the ETC1, PVRTC and ASTC
// decoders, which these tests never reach; the definitions at the end of this
// file satisfy the linker and abort if called.

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "FasTC/CompressedImage.h"
#include "FasTC/Image.h"
#include "FasTC/Pixel.h"
#include "FasTC/ASTCCompressor.h"
#include "FasTC/ETCCompressor.h"
#include "FasTC/PVRTCCompressor.h"
#include "ImageLoaderKTX.h"
#include "ImageLoaderTGA.h"
#include "ImageWriterKTX.h"

namespace {

// FasTC::ECompressionFormat from the container's format code (1 = DXT1,
// 5 = DXT5, 7 = BPTC); anything else is refused.
bool to_format(int code, FasTC::ECompressionFormat *f) {
  switch (code) {
    case 1: *f = FasTC::eCompressionFormat_DXT1; return true;
    case 5: *f = FasTC::eCompressionFormat_DXT5; return true;
    case 7: *f = FasTC::eCompressionFormat_BPTC; return true;
    default: return false;
  }
}

}  // namespace

extern "C" {

double ref_tc_psnr(const uint8_t *rgba, const uint8_t *blocks, uint32_t w,
                   uint32_t h, int format) {
  FasTC::ECompressionFormat f;
  if (!to_format(format, &f)) return -2.0;
  FasTC::Image<> img(w, h, reinterpret_cast<const uint32 *>(rgba));
  CompressedImage ci(w, h, f, blocks);
  return img.ComputePSNR(&ci);
}

// Writes the KTX file into out (capacity cap); returns its size, or minus the
// size needed when cap is too small, or 0 when the writer refused.
int64_t ref_ktx(const uint8_t *blocks, uint32_t w, uint32_t h, int format,
                uint8_t *out, uint64_t cap) {
  FasTC::ECompressionFormat f;
  if (!to_format(format, &f)) return 0;
  CompressedImage ci(w, h, f, blocks);
  ImageWriterKTX writer(ci);
  if (!writer.WriteImage()) return 0;
  const uint64_t n = writer.GetRawFileDataSz();
  if (n > cap) return -static_cast<int64_t>(n);
  memcpy(out, writer.GetRawFileData(), n);
  return static_cast<int64_t>(n);
}

// Loads a TGA file with FasTC's loader: returns the texel count with *w, *h
// set (RGBA8 texels written to out when cap holds them), or 0 when the
// loader refuses the file.
int64_t ref_load_tga(const uint8_t *data, int32_t n, uint8_t *out, uint64_t cap, uint32_t *w,
                     uint32_t *h) {
  ImageLoaderTGA loader(data, n);
  FasTC::Image<> *img = loader.LoadImage();
  if (!img) return 0;
  *w = img->GetWidth();
  *h = img->GetHeight();
  const uint64_t texels = (uint64_t)*w * *h;
  if (4 * texels <= cap)
    for (uint64_t i = 0; i < texels; i++) {
      const uint32 p = img->GetPixels()[i].Pack();
      memcpy(out + 4 * i, &p, 4);
    }
  delete img;
  return static_cast<int64_t>(texels);
}

// Loads a KTX file with FasTC's loader: returns the texel count with *w, *h
// set (RGBA8 texels written to out when cap holds them) for an uncompressed
// file, -1 for a compressed one (a CompressedImage), 0 when the loader
// refuses the file.
int64_t ref_load_ktx(const uint8_t *data, int32_t n, uint8_t *out, uint64_t cap, uint32_t *w,
                     uint32_t *h) {
  ImageLoaderKTX loader(data, n);
  FasTC::Image<> *img = loader.LoadImage();
  if (!img) return 0;
  if (dynamic_cast<CompressedImage *>(img)) {
    delete img;
    return -1;
  }
  *w = img->GetWidth();
  *h = img->GetHeight();
  const uint64_t texels = (uint64_t)*w * *h;
  if (4 * texels <= cap)
    for (uint64_t i = 0; i < texels; i++) {
      const uint32 p = img->GetPixels()[i].Pack();
      memcpy(out + 4 * i, &p, 4);
    }
  delete img;
  return static_cast<int64_t>(texels);
}

}  // extern "C"

// Link-only definitions of the decoders this test library does not compile.
static void not_built(const char *what) {
  fprintf(stderr, "%s is not part of the test build\n", what);
  abort();
}
namespace ETCC {
void Decompress(const FasTC::DecompressionJob &) { not_built("ETCC::Decompress"); }
}  // namespace ETCC
namespace PVRTCC {
void Decompress(const FasTC::DecompressionJob &, const EWrapMode, bool) {
  not_built("PVRTCC::Decompress");
}
}  // namespace PVRTCC
namespace ASTCC {
void Decompress(const FasTC::DecompressionJob &) { not_built("ASTCC::Decompress"); }
}  // namespace ASTCC
