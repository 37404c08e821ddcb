// Stand-in for FasTC's Base/include/FasTC/Pixel.h: the channel accessors
// and bit-depth setter that the BPTC shim's DecompressLogical uses. Test
// infrastructure only.
#ifndef FASTC_STUB_PIXEL_H_
#define FASTC_STUB_PIXEL_H_
#include "FasTC/TexCompTypes.h"

namespace FasTC {

class Pixel {
 public:
  Pixel() : c_{0, 0, 0, 0}, depth_{8, 8, 8, 8} {}
  void ChangeBitDepth(const uint8 (&d)[4]) {
    for (int i = 0; i < 4; i++) depth_[i] = d[i];
  }
  int16 &A() { return c_[0]; }
  int16 &R() { return c_[1]; }
  int16 &G() { return c_[2]; }
  int16 &B() { return c_[3]; }
  const uint8 *Depth() const { return depth_; }

 private:
  int16 c_[4];
  uint8 depth_[4];
};

}  // namespace FasTC
#endif
