// Stand-in for FasTC's BPTCEncoder/include/FasTC/BPTCCompressor.h
// (:54-216): the settings, logical block and entry points with FasTC's
// names and signatures. Test infrastructure only.
#ifndef FASTC_STUB_BPTCCOMPRESSOR_H_
#define FASTC_STUB_BPTCCOMPRESSOR_H_
#include <cstddef>
#include <ostream>
#include <vector>

#include "FasTC/CompressionJob.h"
#include "FasTC/Pixel.h"
#include "FasTC/TexCompTypes.h"

namespace BPTCC {

enum EBlockMode {
  eBlockMode_Zero = 1, eBlockMode_One = 2, eBlockMode_Two = 4, eBlockMode_Three = 8,
  eBlockMode_Four = 16, eBlockMode_Five = 32, eBlockMode_Six = 64, eBlockMode_Seven = 128,
};

enum ErrorMetric { eErrorMetric_Uniform, eErrorMetric_Nonuniform, kNumErrorMetrics };

struct Shape {
  uint32 m_NumPartitions;
  uint32 m_Index;
};

struct ShapeSelection {
  uint32 m_NumShapesToSearch;
  Shape m_Shapes[10];
  EBlockMode m_SelectedModes;
};

typedef ShapeSelection (*ShapeSelectionFn)(uint32 x, uint32 y, const uint32 pixels[16], const void *userData);

struct CompressionSettings {
  ShapeSelectionFn m_ShapeSelectionFn;
  const void *m_ShapeSelectionUserData;
  uint32 m_BlockModes;
  ErrorMetric m_ErrorMetric;
  uint32 m_NumSimulatedAnnealingSteps;
  CompressionSettings()
      : m_ShapeSelectionFn(NULL), m_ShapeSelectionUserData(NULL), m_BlockModes(static_cast<EBlockMode>(0xFF)),
        m_ErrorMetric(eErrorMetric_Uniform), m_NumSimulatedAnnealingSteps(50) {}
};

void Compress(const FasTC::CompressionJob &, CompressionSettings settings = CompressionSettings());
void CompressWithStats(const FasTC::CompressionJob &, std::ostream *logStream,
                       CompressionSettings settings = CompressionSettings());
void CompressAtomic(FasTC::CompressionJobList &);

struct LogicalBlock {
  EBlockMode m_Mode;
  Shape m_Shape;
  FasTC::Pixel m_Endpoints[3][2];
  uint32 m_Indices[16];
  uint32 m_AlphaIndices[16];
};

void DecompressLogical(const FasTC::DecompressionJob &, std::vector<LogicalBlock> *out);
void Decompress(const FasTC::DecompressionJob &);

}  // namespace BPTCC
#endif
