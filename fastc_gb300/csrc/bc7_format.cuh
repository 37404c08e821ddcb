// BC7 (BPTC) format constants shared by the encoder and decoder kernels.
//
// These tables are fixed by the BC7 block format, so their values have to be
// the ones FasTC uses; the representation is this project's own:
//   * partitions as one 32-bit word per shape, 2 bits per texel (texel i at
//     bits 2i..2i+1), so a lane reads all 16 subset ids with one load
//     (FasTC: BPTCEncoder/include/FasTC/Shapes.h:24-53, as 16-bit masks);
//   * anchors as bytes (FasTC: BPTCEncoder/src/AnchorTables.h:22-51);
//   * the mode table (FasTC: BPTCEncoder/src/Compressor.cpp:170-203);
//   * interpolation weights computed arithmetically, floor((64 j + h) / m)
//     with m = 2^bits - 1 and h = m / 2, which reproduces the BC7 weight rows
//     (FasTC: Compressor.cpp:159-168).
#pragma once

#include <cstdint>

namespace fastc {

enum PBitType : int { kPBitShared = 0, kPBitUnique = 1, kPBitNone = 2 };

struct ModeAttr {
  int part_bits, subsets, idx_bits, alpha_idx_bits, color_bits, alpha_bits;
  int has_rotation, has_idx_mode, pbit;
};

__host__ __device__ constexpr ModeAttr mode_attr(int mode) {
  switch (mode) {
    case 0: return {4, 3, 3, 0, 4, 0, 0, 0, kPBitUnique};
    case 1: return {6, 2, 3, 0, 6, 0, 0, 0, kPBitShared};
    case 2: return {6, 3, 2, 0, 5, 0, 0, 0, kPBitNone};
    case 3: return {6, 2, 2, 0, 7, 0, 0, 0, kPBitUnique};
    case 4: return {0, 1, 2, 3, 5, 6, 1, 1, kPBitNone};
    case 5: return {0, 1, 2, 2, 7, 8, 1, 0, kPBitNone};
    case 6: return {0, 1, 4, 0, 7, 7, 0, 0, kPBitUnique};
    default: return {6, 2, 2, 0, 5, 5, 0, 0, kPBitUnique};
  }
}

// Second-endpoint weight for a `bits`-bit index j (0 <= j < 2^bits).
__host__ __device__ __forceinline__ uint32_t weight1(int bits, uint32_t j) {
  switch (bits) {
    case 2: return (64u * j + 1u) / 3u;
    case 3: return (64u * j + 3u) / 7u;
    default: return (64u * j + 7u) / 15u;
  }
}

// Subset of every texel, 2 bits per texel, two-subset shapes.
#define FASTC_PART2_WORDS                                                    \
  0x50505050u, 0x40404040u, 0x54545454u, 0x54505040u, 0x50404000u,          \
      0x55545450u, 0x55545040u, 0x54504000u, 0x50400000u, 0x55555450u,      \
      0x55544000u, 0x54400000u, 0x55555440u, 0x55550000u, 0x55555500u,      \
      0x55000000u, 0x55150100u, 0x00004054u, 0x15010000u, 0x00405054u,      \
      0x00004050u, 0x15050100u, 0x05010000u, 0x40505054u, 0x00404050u,      \
      0x05010100u, 0x14141414u, 0x05141450u, 0x01155440u, 0x00555500u,      \
      0x15014054u, 0x05414150u, 0x44444444u, 0x55005500u, 0x11441144u,      \
      0x05055050u, 0x05500550u, 0x11114444u, 0x41144114u, 0x44111144u,      \
      0x15055054u, 0x01055040u, 0x05041050u, 0x05455150u, 0x14414114u,      \
      0x50050550u, 0x41411414u, 0x00141400u, 0x00041504u, 0x00105410u,      \
      0x10541000u, 0x04150400u, 0x50410514u, 0x41051450u, 0x05415014u,      \
      0x14054150u, 0x41050514u, 0x41505014u, 0x40011554u, 0x54150140u,      \
      0x50505500u, 0x00555050u, 0x15151010u, 0x54540404u

// Subset of every texel, 2 bits per texel, three-subset shapes.
#define FASTC_PART3_WORDS                                                    \
  0xaa685050u, 0x6a5a5040u, 0x5a5a4200u, 0x5450a0a8u, 0xa5a50000u,          \
      0xa0a05050u, 0x5555a0a0u, 0x5a5a5050u, 0xaa550000u, 0xaa555500u,      \
      0xaaaa5500u, 0x90909090u, 0x94949494u, 0xa4a4a4a4u, 0xa9a59450u,      \
      0x2a0a4250u, 0xa5945040u, 0x0a425054u, 0xa5a5a500u, 0x55a0a0a0u,      \
      0xa8a85454u, 0x6a6a4040u, 0xa4a45000u, 0x1a1a0500u, 0x0050a4a4u,      \
      0xaaa59090u, 0x14696914u, 0x69691400u, 0xa08585a0u, 0xaa821414u,      \
      0x50a4a450u, 0x6a5a0200u, 0xa9a58000u, 0x5090a0a8u, 0xa8a09050u,      \
      0x24242424u, 0x00aa5500u, 0x24924924u, 0x24499224u, 0x50a50a50u,      \
      0x500aa550u, 0xaaaa4444u, 0x66660000u, 0xa5a0a5a0u, 0x50a050a0u,      \
      0x69286928u, 0x44aaaa44u, 0x66666600u, 0xaa444444u, 0x54a854a8u,      \
      0x95809580u, 0x96969600u, 0xa85454a8u, 0x80959580u, 0xaa141414u,      \
      0x96960000u, 0xaaaa1414u, 0xa05050a0u, 0xa0a5a5a0u, 0x96000000u,      \
      0x40804080u, 0xa9a8a9a8u, 0xaaaaaa44u, 0x2a4a5254u

// Anchor texel of subset 1 for two-subset shapes.
#define FASTC_ANCHOR2_BYTES                                                  \
  15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 2, 8,  \
      2, 2, 8, 8, 15, 2, 8, 2, 2, 8, 8, 2, 2, 15, 15, 6, 8, 2, 8, 15, 15, 2,  \
      8, 2, 2, 2, 15, 15, 6, 6, 2, 6, 8, 15, 15, 2, 2, 15, 15, 15, 15, 15, 2, \
      2, 15

// Anchors of subsets 1 (low nibble) and 2 (high nibble), three-subset shapes.
#define FASTC_ANCHOR3_BYTES                                                  \
  0xf3, 0x83, 0x8f, 0x3f, 0xf8, 0xf3, 0x3f, 0x8f, 0xf8, 0xf8, 0xf6, 0xf6,   \
      0xf6, 0xf5, 0xf3, 0x83, 0xf3, 0x83, 0xf8, 0x3f, 0xf3, 0x83, 0xf6, 0x8a, \
      0x35, 0xf8, 0x68, 0xa6, 0xf8, 0xf5, 0xaf, 0x8f, 0xf8, 0x3f, 0xf3, 0xa5, \
      0xa6, 0x8a, 0x98, 0xaf, 0x6f, 0xf3, 0x8f, 0xf5, 0x3f, 0x6f, 0x6f, 0x8f, \
      0xf3, 0x3f, 0xf5, 0xf5, 0xf5, 0xf8, 0xf5, 0xfa, 0xf5, 0xfa, 0xf8, 0xfd, \
      0x3f, 0xfc, 0xf3, 0x83

// The 31 alpha-index bits FasTC writes into single-colour blocks, cycling
// through nine values (Compressor.cpp:135-139). They are part of the
// emitted bits, so they are reproduced as is.
#define FASTC_WATERMARK_WORDS                                                \
  0x32b92180u, 0x32ba3080u, 0x31103200u, 0x28103c80u, 0x32bb3080u,          \
      0x25903600u, 0x3530b900u, 0x3b32b180u, 0x34b5b98u

}  // namespace fastc
