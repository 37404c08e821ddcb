/*
 * fastc_bc7.h -- C ABI of the GB300 BC7 (BPTC) encoder, and of its DXT1 /
 * DXT5 encoder and decoder.
 *
 * Drop-in boundary for FasTC's BPTC encode path (and its DXT path, at the
 * end of this header). Every entry point takes
 * plain pointers and sizes and returns a status code; none throws, none
 * keeps a pointer after it returns (plans excepted, see below).
 *
 * Reference interfaces replaced (paths within the FasTC project):
 *   fastc_bc7_compress        BPTCC::Compress(const CompressionJob&,
 *                             CompressionSettings)
 *                             BPTCEncoder/include/FasTC/BPTCCompressor.h:166
 *                             (and the Core plugin slot CompressionFunc,
 *                             Core/src/CompressionFuncs.h:126, that
 *                             Core/src/TexComp.cpp:55-57 fills with it)
 *   fastc_bc7_compress_batch  BPTCC::CompressAtomic(CompressionJobList&)
 *                             BPTCEncoder/include/FasTC/BPTCCompressor.h:189
 *   fastc_bc7_compress_image  CompressImageData(...)
 *                             Core/include/FasTC/TexComp.h:81-88
 *   fastc_bc7_decompress      BPTCC::Decompress(const DecompressionJob&)
 *                             BPTCEncoder/include/FasTC/BPTCCompressor.h:216
 *   fastc_dxt_compress        DXTC::CompressImageDXT1 / CompressImageDXT5
 *                             (const CompressionJob&)
 *                             DXTEncoder/include/FasTC/DXTCompressor.h:24-25
 *                             (the Core plugin slot Core/src/TexComp.cpp:130-134)
 *   fastc_dxt_decompress      DXTC::DecompressDXT1 / DecompressDXT5
 *                             DXTEncoder/include/FasTC/DXTCompressor.h:27-28
 *
 * Differences a caller can observe:
 *   * steps > 0 draws annealing randomness from a per-fit stream seeded by
 *     `seed` and the block position, so results repeat exactly and do not
 *     depend on batching; FasTC seeds one global stream from time(NULL)
 *     (BPTCEncoder/src/Compressor.cpp:358).
 *   * A non-NULL shape_selection_fn (a host callback) is rejected with
 *     FASTC_BC7_ERR_UNSUPPORTED: the search runs on the GPU.
 *   * Where FasTC's selected mode set comes out empty (undefined behaviour
 *     there), the encoder searches the caller's block_modes instead.
 */
#ifndef FASTC_BC7_H_
#define FASTC_BC7_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FASTC_BC7_ABI_VERSION 2

#if defined(__GNUC__)
#define FASTC_BC7_API __attribute__((visibility("default")))
#else
#define FASTC_BC7_API
#endif

typedef enum {
  FASTC_BC7_OK = 0,
  FASTC_BC7_ERR_INVALID_ARGUMENT = 1, /* bad sizes, alignment or pointers */
  FASTC_BC7_ERR_UNSUPPORTED = 2,      /* e.g. a host shape-selection callback */
  FASTC_BC7_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed */
  FASTC_BC7_ERR_CUDA = 4,             /* CUDA runtime error; see fastc_bc7_last_error */
  FASTC_BC7_ERR_BUDGET = 5,           /* request larger than the server's memory budget */
  FASTC_BC7_ERR_TIMEOUT = 6,          /* wait gave up */
  FASTC_BC7_ERR_NOT_FOUND = 7,        /* unknown request id */
  FASTC_BC7_ERR_CANCELLED = 8,        /* request cancelled */
  FASTC_BC7_ERR_NO_DEVICE = 9,        /* no usable CUDA device */
  FASTC_BC7_ERR_INTERNAL = 10
} fastc_bc7_status;

/* watermark_start value that continues the process-wide single-colour
 * watermark counter, like FasTC's global gWMVal (Compressor.cpp:140): every
 * single-colour block of the call, in job and raster order, takes the next
 * entry. Host-memory entry points only. */
#define FASTC_BC7_WATERMARK_CONTINUE 0xFFFFFFFFu

/* EBlockMode (BPTCCompressor.h:56-65): bit m enables BC7 mode m. */
#define FASTC_BC7_ALL_MODES 0xFFu

/* Mirrors BPTCC::CompressionSettings (BPTCCompressor.h:123-158) plus the
 * GPU-side knobs. Use fastc_bc7_settings_default() to initialise. */
typedef struct {
  const void *shape_selection_fn;        /* m_ShapeSelectionFn: must be NULL */
  const void *shape_selection_user_data; /* m_ShapeSelectionUserData: ignored */
  uint32_t block_modes;                  /* m_BlockModes, default 0xFF */
  uint32_t error_metric;                 /* m_ErrorMetric: 0 uniform, 1 nonuniform */
  uint32_t steps;                        /* m_NumSimulatedAnnealingSteps (tc -q), default 50 */
  uint32_t seed;                         /* annealing seed, default 0 */
  uint32_t watermark_start;              /* watermark entry of the first single-colour
                                            block (FasTC's gWMVal + 1), default 0 */
  uint32_t reserved;
} fastc_bc7_settings;

/* One FasTC CompressionJob (Base/include/FasTC/CompressionJob.h:40-140):
 * `in` holds width*height RGBA8 texels (R in the lowest byte), `out`
 * receives width*height bytes of BC7 blocks in raster order. The job covers
 * the raster range of blocks from (x_start, y_start) up to, on row y_end,
 * x_end (exclusive); y_end > height - 4 means "to the end of the image".
 * All four are pixel coordinates and multiples of 4; width and height are
 * multiples of 4. Only the blocks of the range are written. */
typedef struct {
  const uint8_t *in;
  uint8_t *out;
  uint32_t width, height;
  uint32_t x_start, y_start, x_end, y_end;
} fastc_bc7_job;

FASTC_BC7_API void fastc_bc7_settings_default(fastc_bc7_settings *s);
FASTC_BC7_API const char *fastc_bc7_status_string(fastc_bc7_status st);
/* Text of the last CUDA error seen by this thread's calls (or ""). */
FASTC_BC7_API const char *fastc_bc7_last_error(void);
FASTC_BC7_API uint32_t fastc_bc7_abi_version(void);

/* Number of blocks a job covers (after validation), or 0 if invalid. */
FASTC_BC7_API uint64_t fastc_bc7_job_blocks(const fastc_bc7_job *job);

/* --- Host-memory entry points: copy in, encode, copy out, synchronise. --- */

/* BPTCC::Compress: one job, host buffers. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_compress(const fastc_bc7_job *job, const fastc_bc7_settings *s);

/* BPTCC::CompressAtomic: every job of a list compressed in one batched
 * launch (FasTC's CompressAtomic always runs with default settings; pass
 * NULL for the same behaviour). settings may be one entry for all jobs or,
 * with per_job_settings != 0, an array of n. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_compress_batch(const fastc_bc7_job *jobs, uint32_t n,
                                          const fastc_bc7_settings *settings,
                                          int per_job_settings);

/* CompressImageData for BC7: whole image, host buffers; cmp_size must be at
 * least width*height bytes. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_compress_image(const uint8_t *rgba, uint32_t width,
                                          uint32_t height, uint8_t *cmp, size_t cmp_size,
                                          const fastc_bc7_settings *s);

/* BPTCC::Decompress: host buffers; rgba receives width*height*4 bytes.
 * spec_semantics = 0 decodes exactly as FasTC's decoder, 1 follows the
 * BC7 specification for mode-4 blocks with index mode 1 (the only
 * difference). */
FASTC_BC7_API fastc_bc7_status fastc_bc7_decompress(const uint8_t *blocks, uint8_t *rgba, uint32_t width,
                                      uint32_t height, int spec_semantics);

/* Image quality of encoded blocks against the original texels, by FasTC's
 * Image::ComputePSNR metric (Base/src/Image.cpp:206-255): per texel the RGB
 * channels premultiplied by alpha / 255, squared differences summed over
 * R, G, B; PSNR = 10 log10(3 * 255^2 / (sum / (width * height))). The
 * blocks are decoded with FasTC's decoder semantics on the GPU and never
 * written out as an image.
 *
 * fastc_bc7_psnr: host buffers (blocks: width*height bytes for multiples of
 * 4; rgba: width*height*4 bytes). *psnr receives the PSNR (may be NULL);
 * block_sse, if not NULL, receives one double per 4x4 block in raster
 * order (the texels of the block in row order; texels outside the image
 * skipped). The PSNR equals FasTC's up to the order of the double sum
 * (per block, then a fixed tree over the blocks, instead of one pass over
 * the texels). */
FASTC_BC7_API fastc_bc7_status fastc_bc7_psnr(const uint8_t *blocks, const uint8_t *rgba,
                                              uint32_t width, uint32_t height, double *psnr,
                                              double *block_sse);
/* The same on device pointers, asynchronous on `stream`: block_sse (one
 * double per block, required) and, if sse_total is not NULL, their sum in
 * one device double (the same value on every run). Allocates nothing. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_block_error_device(const uint8_t *blocks,
                                                            const uint8_t *rgba, uint32_t width,
                                                            uint32_t height, double *block_sse,
                                                            double *sse_total, void *stream);

/* What BPTCC::CompressWithStats logs for one block through its BlockLogger
 * (BPTCEncoder/src/Compressor.cpp:1373-1389, 1938-2183). */
typedef struct {
  int32_t path;          /* 0 single colour, 1 transparent, 2 a shape with
                            estimate below 1e-9, 3 searched */
  int32_t mode;          /* BC7 mode of the block written */
  double estimate[8];    /* per-mode error estimate, -1 where none was made */
  double error[8];       /* per-mode error as FasTC logs it: always -1, since
                            its CompressClusters keeps min(error, -1) (:1801) */
  int32_t n_two, n_three;
  double two_shape[64];  /* each improving 2-subset shape estimate, in order */
  double three_shape[64];/* each improving 3-subset shape estimate, in order */
} fastc_bc7_block_stats;

/* BPTCC::CompressWithStats(job, logStream, settings) with a log stream
 * (BPTCEncoder/include/FasTC/BPTCCompressor.h:173; Compressor.cpp:1577-1624):
 * the logging encoder, whose shape selection differs from Compress's
 * (opaque means every alpha is 255, modes 4 and 5 stay on for opaque
 * blocks, 3-subset shapes are searched for opaque blocks even after an
 * exact 2-subset shape, bounding boxes are quantised to two colour grids).
 * Host buffers; the job's blocks are written to job->out and the
 * statistics of its fastc_bc7_job_blocks(job) blocks, in raster order, to
 * `stats`. FasTC's loop runs to y <= YEnd with no clamp to height - 4
 * (:1583-1584), reading and writing a row past the buffers when YEnd is
 * the height; here the range is clamped as Compress clamps it. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_compress_stats(const fastc_bc7_job *job,
                                                        const fastc_bc7_settings *s,
                                                        fastc_bc7_block_stats *stats);
/* FasTC's log text for the job's blocks: per block, "<block index>:
 * BlockStat_<name> -- <value>" lines (doubles as an ostream prints them, 6
 * significant digits), the improving shape estimates first, then Path, then
 * Mode and each mode's estimate and error. The block index is the block's
 * raster index in the whole texture (CompressionJob::CoordsToBlockIdx).
 * Writes at most cap bytes (no terminating zero); *len receives the full
 * length, so a call with cap 0 sizes the buffer. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_stats_log(const fastc_bc7_job *job,
                                                   const fastc_bc7_block_stats *stats,
                                                   char *buf, size_t cap, size_t *len);

/* BPTCC::LogicalBlock (BPTCCompressor.h:203-209): the stored fields of one
 * block. Endpoints are at their stored precision (p-bit appended as the
 * lowest bit), depth[] gives that precision per channel (0: channel absent,
 * reads as 255), indices are per texel after the index-mode swap. */
typedef struct {
  uint32_t mode;  /* 0..7, 8 = reserved block */
  uint32_t shape;
  uint32_t subsets;
  uint32_t rotation;
  uint32_t index_mode;
  uint8_t depth[4];
  uint8_t endpoints[3][2][4];
  uint8_t indices[16];
  uint8_t alpha_indices[16];
} fastc_bc7_logical_block;

/* BPTCC::DecompressLogical: parse n blocks on the host. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_decode_logical(const uint8_t *blocks, size_t n,
                                          fastc_bc7_logical_block *out);

/* --- Device-memory entry points: asynchronous on `stream`. ---
 * in/out of every job are device pointers to whole textures. Scratch is
 * taken from the stream-ordered allocator on `stream`. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_compress_device(const fastc_bc7_job *jobs, uint32_t n,
                                           const fastc_bc7_settings *settings,
                                           int per_job_settings, void *stream);
FASTC_BC7_API fastc_bc7_status fastc_bc7_decompress_device(const uint8_t *blocks, uint8_t *rgba,
                                             uint32_t width, uint32_t height,
                                             int spec_semantics, void *stream);

/* fastc_bc7_compress_device without any allocation inside the call: the job
 * table and scratch live in a fixed array in the library's device image
 * (about 2.1 MB). No counterpart in FasTC, whose encoder needs no device
 * memory; it serves callers that cannot let a library allocate (memory
 * budgeted up front, no allocator locks or device-wide synchronisation
 * while encoding). Same arguments and the same output bytes as
 * fastc_bc7_compress_device, with these differences:
 *   - at most FASTC_BC7_NOALLOC_MAX_JOBS jobs and FASTC_BC7_NOALLOC_MAX_BLOCKS
 *     4x4 blocks in total per call, else FASTC_BC7_ERR_INVALID_ARGUMENT with
 *     the limit in fastc_bc7_last_error;
 *   - the first call on each device does one-time set-up (looks the array
 *     up and uploads the encoder's tables, synchronising the device); make
 *     it before any stream capture;
 *   - every call reuses the one array, so calls that overlap on the device
 *     (different streams, or threads without ordering) race and corrupt
 *     each other's output; calls in order on one stream are safe;
 *   - the array is addressed in the runtime's primary context of the
 *     current device; a caller that makes its own driver-API context current
 *     instead (cuCtxCreate + cuCtxSetCurrent) must not use this entry point;
 *   - it always runs the warp-per-block engine, whose bytes equal the
 *     pipeline engine's (both are checked against the oracle bit for bit). */
#define FASTC_BC7_NOALLOC_MAX_BLOCKS (1u << 20)
#define FASTC_BC7_NOALLOC_MAX_JOBS 256u
FASTC_BC7_API fastc_bc7_status fastc_bc7_compress_device_noalloc(const fastc_bc7_job *jobs,
                                                   uint32_t n,
                                                   const fastc_bc7_settings *settings,
                                                   int per_job_settings, void *stream);

/* The process-wide watermark counter used by FASTC_BC7_WATERMARK_CONTINUE
 * (the entry the next single-colour block takes; FasTC starts at 0). */
FASTC_BC7_API void fastc_bc7_set_watermark_counter(uint32_t next_entry);
FASTC_BC7_API uint32_t fastc_bc7_get_watermark_counter(void);

/* --- Plans: a fixed set of device jobs captured once in a CUDA graph. ---
 * The job table, scratch and the graph are built at creation; each launch
 * replays the whole batch with one graph launch. The caller keeps the
 * jobs' device buffers alive until the plan is destroyed. */
typedef struct fastc_bc7_plan_s *fastc_bc7_plan;

FASTC_BC7_API fastc_bc7_status fastc_bc7_plan_create(const fastc_bc7_job *jobs, uint32_t n,
                                       const fastc_bc7_settings *settings,
                                       int per_job_settings, fastc_bc7_plan *out);
FASTC_BC7_API fastc_bc7_status fastc_bc7_plan_launch(fastc_bc7_plan plan, void *stream);
/* Device status bits of the plan's last completed launch (bit 0: a k-means
 * loop reached its iteration bound). Synchronises with the plan's work. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_plan_flags(fastc_bc7_plan plan, uint32_t *flags);
FASTC_BC7_API uint64_t fastc_bc7_plan_blocks(fastc_bc7_plan plan);
/* Kernel launches one fastc_bc7_plan_launch makes (kernel nodes of the
 * captured graph). */
FASTC_BC7_API uint64_t fastc_bc7_plan_kernels(fastc_bc7_plan plan);
/* Autotuner (replaces FasTC's fixed thread-count choice, Core/src/
 * TexComp.cpp:503-514): on the plan's own jobs, timing `launches` graph
 * launches per candidate on `stream`, a coordinate search over the
 * pipeline's launch parameters -- persistent CTAs per SM of the annealing
 * kernels, the lane count below which a warp hands its unfinished fits on,
 * blocks per chunk (the default, a half, a quarter), the select grid and
 * the setup grid -- and, for sets of at most 65,536 blocks, the
 * warp-per-block engine at 2, 4 or 8 warps per CTA; the fastest graph is
 * kept. The plan's outputs are rewritten with the same bytes (results do
 * not depend on the launch parameters or the engine). Synchronises
 * `stream`. A plan created under the warp-per-block engine is left as is. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_plan_autotune(fastc_bc7_plan plan, void *stream,
                                         uint32_t launches);
FASTC_BC7_API fastc_bc7_status fastc_bc7_plan_tuning(fastc_bc7_plan plan, int *anneal_ctas_per_sm,
                                       int *yield_lanes);
/* Every parameter the plan's graph was captured with. */
typedef struct {
  int32_t engine;             /* FASTC_BC7_ENGINE_PIPELINE or _WARP_PER_BLOCK */
  int32_t warps_per_cta;      /* warp-per-block engine */
  int32_t anneal_ctas_per_sm; /* pipeline: persistent annealing CTAs per SM */
  int32_t yield_lanes;        /* pipeline: hand-on threshold of the rotation classes */
  int32_t select_ctas_per_sm; /* pipeline: select grid */
  int32_t setup_ctas_per_sm;  /* pipeline: cap of the setup grid */
  uint64_t chunk_blocks;      /* pipeline: blocks per chunk */
} fastc_bc7_plan_tuning_info;
FASTC_BC7_API fastc_bc7_status fastc_bc7_plan_get_tuning(fastc_bc7_plan plan,
                                                         fastc_bc7_plan_tuning_info *out);
FASTC_BC7_API fastc_bc7_status fastc_bc7_plan_destroy(fastc_bc7_plan plan);

/* --- Request server: continuous batching under a device-memory budget. ---
 * A worker thread admits queued requests (host buffers, kept alive by the
 * caller until the request finishes) into up to max_inflight concurrent
 * batches, as budget and slots free up; each batch is one encoder launch on
 * its own stream. A request's blocks are the same alone or in any mix. */
typedef struct fastc_bc7_server_s *fastc_bc7_server;

typedef struct {
  size_t memory_budget;      /* device bytes for texels, blocks and scratch (8 GiB) */
  uint32_t max_inflight;     /* batches on the GPU at once (3) */
  uint32_t max_batch_blocks; /* blocks per batch (4 Mi) */
  uint32_t max_batch_jobs;   /* requests per batch (4096) */
  uint32_t reserved;
} fastc_bc7_server_config;

typedef struct {
  uint64_t submitted, completed, failed, cancelled, rejected, batches;
  uint64_t pixels_completed;
  size_t bytes_in_use, peak_bytes;
  double p50_latency_ms, p99_latency_ms, mean_latency_ms, max_latency_ms;
  double mpix_per_s; /* texels completed / time from first submit to last completion */
  double psnr_db;    /* FasTC's PSNR (Image::ComputePSNR) over every completed
                        request's texels, measured on the device */
} fastc_bc7_server_stats;

FASTC_BC7_API void fastc_bc7_server_config_default(fastc_bc7_server_config *cfg);
FASTC_BC7_API fastc_bc7_status fastc_bc7_server_create(const fastc_bc7_server_config *cfg,
                                                       fastc_bc7_server *out);
/* Queue one job (host buffers). FASTC_BC7_ERR_BUDGET when the request alone
 * exceeds the budget. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_server_submit(fastc_bc7_server s, const fastc_bc7_job *job,
                                                       const fastc_bc7_settings *settings,
                                                       uint64_t *request_id);
/* Queue one DXT1 / DXT5 job (format FASTC_DXT1 or FASTC_DXT5; the output
 * holds 8 or 16 bytes per block) on the same server: DXT requests share the
 * queue, the budget and the batches with BC7 requests (a batch runs its BC7
 * requests through the BC7 encoder and its DXT requests through the DXT
 * encoder on the same stream), and poll / wait / request_psnr / cancel /
 * release and the statistics cover them alike. The second compression
 * function of FasTC's plugin slot (DXTC::CompressImageDXT1 / DXT5,
 * DXTEncoder/include/FasTC/DXTCompressor.h:24-25) on the serving runtime. */
FASTC_BC7_API fastc_bc7_status fastc_dxt_server_submit(fastc_bc7_server s, const fastc_bc7_job *job,
                                                       int format, uint64_t *request_id);
/* OK when finished, TIMEOUT while queued or running, else the failure. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_server_poll(fastc_bc7_server s, uint64_t request_id);
/* Wait up to timeout_ms (negative: forever). */
FASTC_BC7_API fastc_bc7_status fastc_bc7_server_wait(fastc_bc7_server s, uint64_t request_id,
                                                     int64_t timeout_ms);
/* The PSNR of a finished request's blocks against its texels, by FasTC's
 * Image::ComputePSNR metric (Base/src/Image.cpp:206-255), computed on the
 * device after its encode; the request's status while it is not finished. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_server_request_psnr(fastc_bc7_server s,
                                                             uint64_t request_id, double *psnr);
/* Cancel a request that is still queued. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_server_cancel(fastc_bc7_server s, uint64_t request_id);
/* Forget a finished request. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_server_release(fastc_bc7_server s, uint64_t request_id);
FASTC_BC7_API fastc_bc7_status fastc_bc7_server_get_stats(fastc_bc7_server s,
                                                          fastc_bc7_server_stats *out);
/* Finish queued and running work, then free the server. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_server_destroy(fastc_bc7_server s);

/* Encoder organisation. PIPELINE (default): a per-block select stage, one
 * thread per cluster fit for the fit and the annealing (warps run 32 fits of
 * one mode, refilled from a queue), a per-block pack stage. WARP_PER_BLOCK:
 * one warp owns a block through the whole search, one lane per cluster fit.
 * Both give the same blocks. Applies to calls and plans created afterwards. */
#define FASTC_BC7_ENGINE_PIPELINE 0
#define FASTC_BC7_ENGINE_WARP_PER_BLOCK 1
FASTC_BC7_API fastc_bc7_status fastc_bc7_set_engine(int engine);
FASTC_BC7_API int fastc_bc7_get_engine(void);

/* Launch geometry of the warp-per-block engine: warps per CTA (1, 2, 4 or 8)
 * and CTAs per SM of the persistent encoder; 0 keeps the current value. */
FASTC_BC7_API fastc_bc7_status fastc_bc7_set_launch_shape(int warps_per_cta, int ctas_per_sm);
FASTC_BC7_API fastc_bc7_status fastc_bc7_get_launch_shape(int *warps_per_cta, int *ctas_per_sm);

/* ---- DXT1 / DXT5 (BC1 / BC3) ----
 * FasTC's DXT path: DXTC::CompressImageDXT1 / CompressImageDXT5
 * (DXTEncoder/include/FasTC/DXTCompressor.h:24-25, Compressor.cpp:47-93),
 * the stb_dxt block encoder with dithering, and DXTC::DecompressDXT1 /
 * DecompressDXT5 (DXTCompressor.h:27-28, Decompressor.cpp:98-155). A job is
 * the same fastc_bc7_job (width and height multiples of 4, the same
 * x/y start/end walk); only `in`, `out`, the sizes and the range are read.
 * Blocks are 8 bytes (DXT1) or 16 bytes (DXT5: alpha block, then colour
 * block) and land at out + block_index * size, block_index counted from the
 * texture's first block, as in FasTC. `in` and `out` must be 4-byte aligned.
 * The output equals FasTC's byte for byte. */
#define FASTC_DXT1 1
#define FASTC_DXT5 5
/* Host buffers; returns when `out` holds the blocks. */
FASTC_BC7_API fastc_bc7_status fastc_dxt_compress(const fastc_bc7_job *job, int format);
/* n jobs of host buffers in one call; returns when every `out` holds its
 * blocks. When every job's buffers are page-locked (cudaHostAlloc,
 * cudaHostRegister), the encoder reads the texels and writes the blocks
 * through the device's mapping of host memory, with no staging copies;
 * otherwise uploads, encodes and downloads of groups of jobs overlap. */
FASTC_BC7_API fastc_bc7_status fastc_dxt_compress_batch(const fastc_bc7_job *jobs, uint32_t n,
                                                       int format);
/* Device buffers, enqueued on `stream` (NULL: the legacy default stream);
 * allocates nothing. The first DXT call on a device uploads the encoder's
 * tables (a synchronous copy): make it outside stream capture. */
FASTC_BC7_API fastc_bc7_status fastc_dxt_compress_device(const fastc_bc7_job *jobs, uint32_t n,
                                                        int format, void *stream);
/* Blocks of a width x height image (rounded up to whole blocks) to RGBA8
 * texels (4-byte aligned); texels past the image edge are not written.
 * DXT1 blocks with c0 <= c1 decode as 3 colours and black, alpha 255. */
FASTC_BC7_API fastc_bc7_status fastc_dxt_decompress(const uint8_t *blocks, uint8_t *rgba,
                                                   uint32_t width, uint32_t height, int format);
FASTC_BC7_API fastc_bc7_status fastc_dxt_decompress_device(const uint8_t *blocks, uint8_t *rgba,
                                                          uint32_t width, uint32_t height,
                                                          int format, void *stream);
/* FasTC's Image::ComputePSNR (as fastc_bc7_psnr) of DXT1 / DXT5 blocks
 * against the original texels, decoded on the GPU. Host buffers: *psnr (may
 * be NULL) and, if not NULL, one double per block in block_sse. Device
 * buffers: block_sse (one double per block) and, if not NULL, their
 * fixed-order sum in *total, enqueued on `stream`. */
FASTC_BC7_API fastc_bc7_status fastc_dxt_psnr(const uint8_t *blocks, const uint8_t *rgba, uint32_t width,
                                             uint32_t height, int format, double *psnr,
                                             double *block_sse);
FASTC_BC7_API fastc_bc7_status fastc_dxt_block_error_device(const uint8_t *blocks, const uint8_t *rgba,
                                                           uint32_t width, uint32_t height, int format,
                                                           double *block_sse, double *total,
                                                           void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FASTC_BC7_H_ */
