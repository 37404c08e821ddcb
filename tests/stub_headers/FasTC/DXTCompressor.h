// Stand-in for FasTC's DXTEncoder/include/FasTC/DXTCompressor.h (:22-29).
// Test infrastructure only.
#ifndef FASTC_STUB_DXTCOMPRESSOR_H_
#define FASTC_STUB_DXTCOMPRESSOR_H_
#include "FasTC/CompressionJob.h"

namespace DXTC {
void CompressImageDXT1(const FasTC::CompressionJob &);
void CompressImageDXT5(const FasTC::CompressionJob &);
void DecompressDXT1(const FasTC::DecompressionJob &);
void DecompressDXT5(const FasTC::DecompressionJob &);
}  // namespace DXTC
#endif
