// Stand-in for FasTC's Base/include/FasTC/CompressionJob.h (:40-210): the
// job, decompression job and job list with FasTC's names, constructors and
// accessors, defined inline. Test infrastructure only.
#ifndef FASTC_STUB_COMPRESSIONJOB_H_
#define FASTC_STUB_COMPRESSIONJOB_H_
#include <vector>

#include "FasTC/TexCompTypes.h"

namespace FasTC {

enum ECompressionFormat {
  eCompressionFormat_DXT1,
  eCompressionFormat_DXT5,
  eCompressionFormat_BPTC,
};

class CompressionJob {
 public:
  CompressionJob(ECompressionFormat fmt, const uint8 *in, unsigned char *out, uint32 w, uint32 h,
                 uint32 x0 = 0, uint32 y0 = 0)
      : fmt_(fmt), in_(in), out_(out), w_(w), h_(h), x0_(x0), x1_(w), y0_(y0), y1_(h) {}
  CompressionJob(ECompressionFormat fmt, const uint8 *in, unsigned char *out, uint32 w, uint32 h,
                 uint32 x0, uint32 y0, uint32 x1, uint32 y1)
      : fmt_(fmt), in_(in), out_(out), w_(w), h_(h), x0_(x0), x1_(x1), y0_(y0), y1_(y1) {}
  ECompressionFormat Format() const { return fmt_; }
  const uint8 *InBuf() const { return in_; }
  uint8 *OutBuf() const { return out_; }
  uint32 Width() const { return w_; }
  uint32 Height() const { return h_; }
  uint32 XStart() const { return x0_; }
  uint32 XEnd() const { return x1_; }
  uint32 YStart() const { return y0_; }
  uint32 YEnd() const { return y1_; }

 private:
  ECompressionFormat fmt_;
  const uint8 *in_;
  uint8 *out_;
  uint32 w_, h_, x0_, x1_, y0_, y1_;
};

class DecompressionJob {
 public:
  DecompressionJob(ECompressionFormat fmt, const uint8 *in, uint8 *out, uint32 w, uint32 h)
      : fmt_(fmt), in_(in), out_(out), w_(w), h_(h) {}
  const uint8 *InBuf() const { return in_; }
  uint8 *OutBuf() const { return out_; }
  uint32 Width() const { return w_; }
  uint32 Height() const { return h_; }
  ECompressionFormat Format() const { return fmt_; }

 private:
  ECompressionFormat fmt_;
  const uint8 *in_;
  uint8 *out_;
  uint32 w_, h_;
};

class CompressionJobList {
 public:
  explicit CompressionJobList(uint32 n) : total_(n), flags_(n, 0), m_CurrentJobIndex(0), m_CurrentBlockIndex(0) {}
  bool AddJob(const CompressionJob &j) {
    if (jobs_.size() >= total_) return false;
    jobs_.push_back(j);
    return true;
  }
  uint32 GetTotalNumJobs() const { return total_; }
  uint32 GetNumJobs() const { return (uint32)jobs_.size(); }
  const CompressionJob *GetJob(uint32 i) const { return &jobs_[i]; }
  uint32 *GetFinishedFlag(uint32 i) const { return const_cast<uint32 *>(&flags_[i]); }

 private:
  uint32 total_;
  std::vector<CompressionJob> jobs_;
  std::vector<uint32> flags_;

 public:
  uint32 m_CurrentJobIndex;
  uint32 m_CurrentBlockIndex;
};

}  // namespace FasTC
#endif
