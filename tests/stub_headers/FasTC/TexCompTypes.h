// Stand-in for FasTC's Base/include/FasTC/TexCompTypes.h: the fixed-width
// integer names the drop-in shims use. Test infrastructure: it lets the
// shims build and run against the GPU library where FasTC's own headers
// are absent.
#ifndef FASTC_STUB_TEXCOMPTYPES_H_
#define FASTC_STUB_TEXCOMPTYPES_H_
#include <cstdint>
typedef int8_t int8;
typedef uint8_t uint8;
typedef int16_t int16;
typedef uint16_t uint16;
typedef int32_t int32;
typedef uint32_t uint32;
typedef int64_t int64;
typedef uint64_t uint64;
#endif
