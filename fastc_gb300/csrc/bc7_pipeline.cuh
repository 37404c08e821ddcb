// Data structures of the task-parallel BC7 encoder (bc7_pipeline.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "bc7_kernels.cuh"
#include "fastc_bc7.h"

namespace fastc {

// Cluster fits one block can need. BC7's mode table caps it at 32 (opaque
// block whose selection falls back to the caller's mask of modes 1,3-7);
// with all modes enabled it is 15 (block_task_bound() computes the bound of
// a mask). Scratch is sized by the bound of the launch's masks.
constexpr int kMaxBlockTasks = 32;
// The logging encoder of CompressWithStats keeps modes 4 and 5 on for
// opaque blocks, which then run once per shape slot: up to 38 fits (mode 4
// 2 x 8, mode 5 2 x 4, mode 6 2, modes 0 and 2 3 each, modes 1, 3 and 7 2
// each).
constexpr int kMaxStatsBlockTasks = 38;
// Blocks per pipeline chunk: scratch grows with chunk x task bound, and
// longer annealing lists keep more lanes busy, so the chunk is larger when
// the bound is small. Launches of more than one chunk use two scratch
// buffers so that the select stage of a chunk runs while the previous chunk
// anneals.
constexpr uint64_t kChunkTaskBudget = 16ull * 1024 * 1024;  // chunk blocks x task bound
// (a multiple of the watermark-rank chunk, so that each pipeline chunk
// ranks its own blocks)
__host__ __device__ constexpr uint64_t pipeline_chunk(int task_bound) {
  return kChunkTaskBudget / (uint64_t)(task_bound > 32 ? 48 : (task_bound > 16 ? 32 : 16)) /
         kRankChunk * kRankChunk;
}

// Per-block outcome of the select stage (16 bytes).
struct BlockSel {
  uint8_t shape0, shape1, nshapes;
  uint8_t modes;  // modes to search (CompressClusters' selectedModes)
  uint8_t done;   // 1: block already written (single colour / transparent)
  uint8_t pad[3];
  uint32_t job;   // index into the job table
  uint32_t lin;   // raster block index within the job's texture
};

constexpr uint8_t kTaskAnneal = 1u;      // the annealing loop has work
constexpr uint8_t kTaskNonuniform = 2u;  // nonuniform error metric

// State of one cluster fit between the stages (64 bytes).
struct __align__(16) TaskState {
  double err;     // CompressCluster's return value (colour part for modes 4/5)
  double aerr;    // alpha error (modes 4/5)
  // colour indices, 4 bits per texel; for a fit that anneals, until the
  // re-index stage writes its indices: the fit's error lower bound (float
  // bits 0-31), its position in the class's annealing list (bits 32-55) and
  // its point count (bits 56-63)
  uint64_t idx;
  uint64_t aidx;  // alpha indices, 4 bits per texel (modes 4/5)
  uint32_t p1, p2;  // endpoints as bytes (grid values)
  float a1, a2;     // alpha endpoints (modes 4/5), as FasTC keeps them
  uint32_t gl;      // block within the chunk
  uint8_t mode, slot, subset, rotim;  // rotim = rotation << 1 | index mode
  uint32_t lcg;     // annealing stream of this fit
  uint16_t steps;
  uint8_t pbit;
  uint8_t flags;
};

// Task classes: one per (BC7 mode, colour index width). Mode 4 anneals with
// 2-bit indices in index mode 0 and 3-bit indices in index mode 1, so it
// has two classes; every other mode has one.
constexpr int kClasses = 9;
__host__ __device__ constexpr int class_mode(int c) { return c < 4 ? c : (c <= 5 ? 4 : c - 1); }
__host__ __device__ constexpr int class_im(int c) { return c == 5 ? 1 : 0; }
__host__ __device__ constexpr int class_of(int mode, int im) {
  return mode < 4 ? mode : (mode == 4 ? 4 + im : mode + 1);
}

// A fit that anneals, as the setup stage hands it to its class's annealing
// list, or as a sparse warp hands an unfinished fit on (a continuation):
// everything the loop needs in one 128-byte record, so that taking the next
// fit is one atomic and eight 16-byte loads.
struct __align__(16) AnnealRec {
  uint32_t pts[16];  // the cluster's texels in texel order (first n used)
  uint64_t tex;      // texel index of each point, 4 bits per point
  uint32_t p1, p2;   // current endpoints (grid values, one byte per channel)
  float err;         // their QuantizedError
  uint32_t lcg;      // annealing stream of this fit
  uint32_t t;        // task index: where the result goes
  uint16_t steps;
  uint8_t n, pbit;   // point count, current p-bit combination
  uint8_t rot, flags;
  uint16_t energy;   // steps since the last improvement
  uint32_t b1, b2;   // best endpoints so far
  float best_err;
  uint8_t best_pbit, pad[15];
};
static_assert(sizeof(AnnealRec) == 128, "AnnealRec layout");

struct PipelineCounters {
  unsigned long long anneal_next[kClasses];  // refill cursors of the annealing lists
  uint32_t anneal_count[kClasses];           // fits of each class that anneal
  uint32_t tasks;                            // tasks in the current chunk
  unsigned long long cont_next[kClasses];    // refill cursors of the continuation lists
  uint32_t cont_count[kClasses];             // records in each continuation list (six used)
  uint32_t reindex_count[kClasses];          // annealed winning fits of each class
  uint32_t nhist[kClasses][17];              // fits left to anneal by point count
};
constexpr size_t kCountersSlot = 1024;
static_assert(sizeof(PipelineCounters) <= kCountersSlot, "PipelineCounters fits its slot");

// Side streams that run the classes' setup + annealing concurrently, forked
// from and joined back into the caller's stream with events (both are
// recorded into a CUDA graph when the caller's stream is being captured).
// Between the two, the per-block bound stage waits for every class's setup
// and the annealing of every class waits for it.
// One set must not be enqueued on by two threads at once.
// Chunks alternate between two sets, so that a class of chunk i + 1 starts
// while the same class of chunk i drains.
struct ClassStreams {
  cudaStream_t side[2][kClasses];
  cudaEvent_t fork[2];
  cudaEvent_t setup[2][kClasses];  // a class's setup stage is done
  cudaEvent_t bound[2];            // the block bounds are done
  cudaEvent_t join[2][kClasses];
};
cudaError_t class_streams_create(ClassStreams *cs);
void class_streams_destroy(ClassStreams *cs);

void upload_pipeline_tables(int device, const uint32_t opt7[256], const uint32_t opt6[256]);
// Most cluster fits a block can need when the caller enables `modes`
// (`stats`: under the logging encoder's shape selection).
int block_task_bound(uint32_t modes, bool stats = false);
// sm_count: of the device that runs the launch (bounds the continuation lists).
size_t pipeline_scratch_bytes(uint64_t total_blocks, int task_bound, int sm_count);
// The same with chunks of `chunk_blocks` (0: the default size; larger
// values are cut to it).
size_t pipeline_scratch_bytes(uint64_t total_blocks, int task_bound, int sm_count,
                              uint64_t chunk_blocks);
// Launch parameters the plan autotuner chooses (defaults: measured best on
// the mixed-size texture set).
struct PipelineTuning {
  int anneal_ctas_per_sm = 5;  // persistent annealing CTAs per SM (capped by residency)
  int yield_lanes = 12;        // a warp with at most this many lanes annealing hands its fits on
  int select_ctas_per_sm = 16; // grid of the select stage (grid-stride over the chunk's blocks)
  int setup_ctas_per_sm = 128; // grid cap of the setup stage (one thread per fit up to it)
  uint64_t chunk_blocks = 0;   // blocks per chunk, 0: pipeline_chunk(task bound); never more
  // the classes' setup kernels one after another on one stream (1) or
  // concurrently on the side streams (0); -1: one stream for a launch that
  // is a single chunk of at least kSerialSetupBlocks blocks
  int serial_setup = -1;
};
constexpr uint64_t kSerialSetupBlocks = 1ull << 18;
// Blocks per chunk a launch uses for this task bound and tuning.
uint64_t pipeline_chunk_blocks(int task_bound, const PipelineTuning &tune);

// `cls` null: every stage runs in order on `stream`. `task_bound`: the most
// block_task_bound() of the jobs' masks. `stats` not null: the logging
// encoder of CompressWithStats (its own shape selection), writing each
// block's statistics to stats[global block index] (the mode is left to the
// host, which reads it from the block).
// Events a caller can place between the pipeline's chunks (chunk k covers
// global blocks [k * pipeline_chunk(task_bound), ...)): before chunk k
// reads any texel the caller's stream waits for in_ready[k]; packed[k] is
// recorded on it once chunk k's blocks are written. Either array may be
// null; `count` is their length (chunks past it take no event).
struct ChunkEvents {
  const cudaEvent_t *in_ready = nullptr;
  const cudaEvent_t *packed = nullptr;
  int count = 0;
};

int launch_pipeline(const JobDev *jobs, int njobs, uint64_t total, const EncodeScratch &rank,
                    void *scratch, int sm_count, int task_bound, const ClassStreams *cls,
                    const PipelineTuning &tune, void *stream,
                    fastc_bc7_block_stats *stats = nullptr, const ChunkEvents *events = nullptr);

}  // namespace fastc
