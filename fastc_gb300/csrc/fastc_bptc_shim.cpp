// Drop-in replacement for FasTC's BPTC encoder library entry points.
//
// Compile this file against FasTC's own headers (Base/include,
// BPTCEncoder/include and the generated BPTCConfig.h) and link it, with
// libfastc_bc7.so, in place of BPTCEncoder/src/Compressor.cpp and
// Decompressor.cpp. Core (TexComp.cpp's CompressBPTC plugin slot,
// ThreadGroup, WorkerQueue, the -a atomic path) and the tc tool then run
// on the GPU encoder without source changes.
//
// Each function keeps the reference signature from
// BPTCEncoder/include/FasTC/BPTCCompressor.h. The reference functions return
// void and only assert on bad input; these print the C-ABI status and abort,
// so a failure is never silent.
#include <sched.h>

#include <cstdio>
#include <cstdlib>
#include <ostream>
#include <string>
#include <vector>

#include "FasTC/BPTCCompressor.h"
#include "fastc_bc7.h"

namespace {

void Die(const char *where, fastc_bc7_status st) {
  std::fprintf(stderr, "fastc_bc7: %s failed: %s %s\n", where, fastc_bc7_status_string(st),
               fastc_bc7_last_error());
  std::abort();
}

fastc_bc7_settings ToC(const BPTCC::CompressionSettings &s) {
  fastc_bc7_settings c;
  fastc_bc7_settings_default(&c);
  c.shape_selection_fn = reinterpret_cast<const void *>(s.m_ShapeSelectionFn);
  c.shape_selection_user_data = s.m_ShapeSelectionUserData;
  c.block_modes = s.m_BlockModes;
  c.error_metric = static_cast<uint32_t>(s.m_ErrorMetric);
  c.steps = s.m_NumSimulatedAnnealingSteps;
  c.watermark_start = FASTC_BC7_WATERMARK_CONTINUE;  // FasTC's global gWMVal
  return c;
}

fastc_bc7_job ToC(const FasTC::CompressionJob &cj) {
  fastc_bc7_job j;
  j.in = cj.InBuf();
  j.out = cj.OutBuf();
  j.width = cj.Width();
  j.height = cj.Height();
  j.x_start = cj.XStart();
  j.y_start = cj.YStart();
  j.x_end = cj.XEnd();
  j.y_end = cj.YEnd();
  return j;
}

}  // namespace

namespace BPTCC {

// BPTCCompressor.h:166
void Compress(const FasTC::CompressionJob &cj, CompressionSettings settings) {
  const fastc_bc7_job j = ToC(cj);
  const fastc_bc7_settings s = ToC(settings);
  const fastc_bc7_status st = fastc_bc7_compress(&j, &s);
  if (st != FASTC_BC7_OK) Die("BPTCC::Compress", st);
}

// BPTCCompressor.h:173. Without a log stream FasTC encodes each block as
// Compress does (Compressor.cpp:1591-1596); with one it runs a logging
// encoder that selects shapes differently (Compressor.cpp:1862-2183) and
// writes each block's statistics to the stream: fastc_bc7_compress_stats
// runs that encoder on the GPU and fastc_bc7_stats_log formats the same
// text. Its block loop runs to y <= YEnd with no clamp to Height - 4
// (Compressor.cpp:1583-1584, unlike Compress at :1478), so for a job whose
// YEnd equals Height FasTC reads and writes one block row past the
// buffers; here the range is clamped as Compress clamps it.
void CompressWithStats(const FasTC::CompressionJob &cj, std::ostream *logStream,
                       CompressionSettings settings) {
  if (!logStream) {
    Compress(cj, settings);
    return;
  }
  const fastc_bc7_job j = ToC(cj);
  const fastc_bc7_settings s = ToC(settings);
  std::vector<fastc_bc7_block_stats> stats(fastc_bc7_job_blocks(&j) + 1);
  fastc_bc7_status st = fastc_bc7_compress_stats(&j, &s, stats.data());
  if (st != FASTC_BC7_OK) Die("BPTCC::CompressWithStats", st);
  size_t len = 0;
  st = fastc_bc7_stats_log(&j, stats.data(), nullptr, 0, &len);
  if (st != FASTC_BC7_OK) Die("BPTCC::CompressWithStats", st);
  std::string text(len, '\0');
  st = fastc_bc7_stats_log(&j, stats.data(), &text[0], len, &len);
  if (st != FASTC_BC7_OK) Die("BPTCC::CompressWithStats", st);
  logStream->write(text.data(), (std::streamsize)text.size());
}

#ifdef HAS_ATOMICS
// BPTCCompressor.h:189. Every calling thread returns once the whole list is
// compressed; the first one to arrive runs the batch on the GPU. Like the
// reference (Compressor.cpp:1542-1574), it uses the default settings.
void CompressAtomic(FasTC::CompressionJobList &cjl) {
  const uint32 n = cjl.GetNumJobs();
  if (__sync_lock_test_and_set(&cjl.m_CurrentBlockIndex, 1u) == 0u) {
    std::vector<fastc_bc7_job> jobs(n);
    for (uint32 i = 0; i < n; i++) {
      cjl.m_CurrentJobIndex = i;  // GetJob returns the current job
      jobs[i] = ToC(*cjl.GetJob(i));
    }
    fastc_bc7_settings s;
    fastc_bc7_settings_default(&s);  // CompressAtomic runs with default settings
    s.watermark_start = FASTC_BC7_WATERMARK_CONTINUE;
    const fastc_bc7_status st = fastc_bc7_compress_batch(jobs.data(), n, &s, 0);
    if (st != FASTC_BC7_OK) Die("BPTCC::CompressAtomic", st);
    for (uint32 i = 0; i < n; i++) *cjl.GetFinishedFlag(i) = 1;
    __sync_synchronize();
    cjl.m_CurrentJobIndex = n;
    __sync_synchronize();
    return;
  }
  while (*(volatile uint32 *)&cjl.m_CurrentJobIndex < n) sched_yield();
}
#endif

// BPTCCompressor.h:216
void Decompress(const FasTC::DecompressionJob &dj) {
  const fastc_bc7_status st =
      fastc_bc7_decompress(dj.InBuf(), dj.OutBuf(), dj.Width(), dj.Height(), 0);
  if (st != FASTC_BC7_OK) Die("BPTCC::Decompress", st);
}

// BPTCCompressor.h:212: the logical contents of every block (mode, shape,
// endpoints at their stored precision, indices).
void DecompressLogical(const FasTC::DecompressionJob &dj, std::vector<LogicalBlock> *out) {
  if (!out) return;
  const size_t n = (size_t)dj.Height() * dj.Width() / 16;
  std::vector<fastc_bc7_logical_block> lb(n);
  const fastc_bc7_status st = fastc_bc7_decode_logical(dj.InBuf(), n, lb.data());
  if (st != FASTC_BC7_OK) Die("BPTCC::DecompressLogical", st);
  out->clear();
  out->resize(n);
  for (size_t b = 0; b < n; b++) {
    const fastc_bc7_logical_block &c = lb[b];
    LogicalBlock &o = (*out)[b];
    if (c.mode >= 8) continue;
    o.m_Mode = static_cast<EBlockMode>(1 << c.mode);
    o.m_Shape.m_NumPartitions = c.subsets;
    o.m_Shape.m_Index = c.shape;
    for (uint32 s = 0; s < c.subsets; s++)
      for (int e = 0; e < 2; e++) {
        FasTC::Pixel p;
        p.ChangeBitDepth(c.depth);
        p.R() = c.endpoints[s][e][0];
        p.G() = c.endpoints[s][e][1];
        p.B() = c.endpoints[s][e][2];
        p.A() = c.depth[3] ? c.endpoints[s][e][3] : 0xFF;
        o.m_Endpoints[s][e] = p;
      }
    for (int i = 0; i < 16; i++) {
      o.m_Indices[i] = c.indices[i];
      o.m_AlphaIndices[i] = c.alpha_indices[i];
    }
  }
}

}  // namespace BPTCC
