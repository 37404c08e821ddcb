/* DXT1 / DXT5 restatement of FasTC's DXT path (stb_dxt v1.06 with
 * dithering and one refinement, FasTC's decoder). TEST INFRASTRUCTURE
 * ONLY: the checker of the GPU kernels. */
#ifndef DXT_ORACLE_H_
#define DXT_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One 4x4 block of RGBA8 texels (row-major, 64 bytes): 8 bytes of DXT1
 * (alpha = 0) or 16 of DXT5 (alpha = 1). */
void dxto_compress_block(const uint8_t rgba[64], int alpha, uint8_t *out);
/* A whole image (width, height multiples of 4), blocks in raster order. */
int dxto_compress(const uint8_t *rgba, uint8_t *out, uint32_t w, uint32_t h, int alpha);
void dxto_decompress(const uint8_t *blocks, uint8_t *rgba, uint32_t w, uint32_t h, int alpha);
/* The single-colour endpoint tables: [value][0] = high, [1] = low. */
void dxto_tables(uint8_t match5[512], uint8_t match6[512]);

#ifdef __cplusplus
}
#endif
#endif
