"""Python mirror of FasTC's BPTC interface over the GB300 C ABI.

Names and argument meaning follow FasTC's BPTCEncoder/include/FasTC/
BPTCCompressor.h (CompressionSettings, Compress, CompressAtomic, Decompress)
and Base/include/FasTC/CompressionJob.h (CompressionJob, CompressionJobList);
CompressImageData follows Core/include/FasTC/TexComp.h:81-88. Errors raise
:class:`BC7Error` where FasTC would assert or return false.

Buffers may be numpy arrays (host memory: copied to the GPU and back) or
CUDA tensors (device memory: encoded in place on the current torch stream).
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass, field
from typing import Iterable, List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import BC7Error, Job, Settings, check, load

BLOCK_BYTES = 16
#: watermark_start value continuing FasTC's process-wide watermark counter
WATERMARK_CONTINUE = 0xFFFFFFFF


class ErrorMetric(enum.IntEnum):
    """BPTCC::ErrorMetric (BPTCCompressor.h:73-78)."""

    UNIFORM = 0
    NONUNIFORM = 1


class BlockMode(enum.IntFlag):
    """BPTCC::EBlockMode (BPTCCompressor.h:56-65)."""

    ZERO = 1
    ONE = 2
    TWO = 4
    THREE = 8
    FOUR = 16
    FIVE = 32
    SIX = 64
    SEVEN = 128
    ALL = 0xFF


class CompressionFormat(enum.IntEnum):
    """The formats of FasTC's ECompressionFormat (Base/include/FasTC/
    CompressionFormat.h) that this library encodes; values are the C ABI's
    format codes (FASTC_DXT1, FASTC_DXT5; 7 for BPTC)."""

    DXT1 = 1
    DXT5 = 5
    BPTC = 7


#: bytes per 4x4 block of each format
FORMAT_BLOCK_BYTES = {CompressionFormat.DXT1: 8, CompressionFormat.DXT5: 16, CompressionFormat.BPTC: 16}


@dataclass
class CompressionSettings:
    """BPTCC::CompressionSettings (BPTCCompressor.h:123-158) plus GPU knobs.

    ``seed`` keys the per-fit annealing streams; ``watermark_start`` is the
    watermark entry of the first single-colour block.
    """

    shape_selection_fn: object = None
    shape_selection_user_data: object = None
    block_modes: int = int(BlockMode.ALL)
    error_metric: ErrorMetric = ErrorMetric.UNIFORM
    num_simulated_annealing_steps: int = 50
    seed: int = 0
    watermark_start: int = 0

    def to_c(self) -> Settings:
        if self.shape_selection_fn is not None:
            raise BC7Error(_lib.ERR_UNSUPPORTED, "CompressionSettings",
                           "host shape-selection callbacks are not supported on the GPU path")
        return Settings(None, None, int(self.block_modes) & 0xFFFFFFFF, int(self.error_metric),
                        int(self.num_simulated_annealing_steps), int(self.seed) & 0xFFFFFFFF,
                        int(self.watermark_start) & 0xFFFFFFFF, 0)


def _is_cuda(t) -> bool:
    return hasattr(t, "is_cuda") and bool(t.is_cuda)


def _addr(buf) -> int:
    if _is_cuda(buf):
        return int(buf.data_ptr())
    arr = buf if isinstance(buf, np.ndarray) else np.frombuffer(buf, dtype=np.uint8)
    if not arr.flags["C_CONTIGUOUS"]:
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "CompressionJob", "buffers must be contiguous")
    return int(arr.ctypes.data)


def _nbytes(buf) -> int:
    if _is_cuda(buf):
        return int(buf.numel() * buf.element_size())
    return int(np.asarray(buf).nbytes)


@dataclass
class CompressionJob:
    """FasTC::CompressionJob: RGBA8 in (width*height*4 bytes), blocks out
    (width*height bytes for BPTC and DXT5, half that for DXT1), and the
    raster block range [start, end) in pixel coordinates; ``y_end`` past the
    last block row means the whole image. ``format`` is the job's
    ECompressionFormat (CompressionJob.h:42)."""

    in_buf: object
    out_buf: object
    width: int
    height: int
    x_start: int = 0
    y_start: int = 0
    x_end: Optional[int] = None
    y_end: Optional[int] = None
    format: CompressionFormat = CompressionFormat.BPTC

    def __post_init__(self):
        if self.x_end is None:
            self.x_end = self.width
        if self.y_end is None:
            self.y_end = self.height
        self.format = CompressionFormat(self.format)
        if _nbytes(self.in_buf) < self.width * self.height * 4:
            raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "CompressionJob", "input smaller than width*height*4")
        need = self.width * self.height * FORMAT_BLOCK_BYTES[self.format] // 16
        if _nbytes(self.out_buf) < need:
            raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "CompressionJob",
                           f"output smaller than {need} bytes for {self.format.name}")

    @property
    def on_device(self) -> bool:
        return _is_cuda(self.in_buf)

    def to_c(self) -> Job:
        if _is_cuda(self.in_buf) != _is_cuda(self.out_buf):
            raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "CompressionJob",
                           "input and output must both be host or both be device buffers")
        return Job(_addr(self.in_buf), _addr(self.out_buf), self.width, self.height, self.x_start,
                   self.y_start, self.x_end, self.y_end)

    def num_blocks(self) -> int:
        j = self.to_c()
        return int(load().fastc_bc7_job_blocks(C.byref(j)))

    # FasTC::CompressionJob::BlockIdxToCoords / CoordsToBlockIdx
    def block_idx_to_coords(self, block_idx: int):
        bw = self.width // 4
        return (block_idx % bw) * 4, (block_idx // bw) * 4

    def coords_to_block_idx(self, x: int, y: int) -> int:
        return (y // 4) * (self.width // 4) + x // 4


class CompressionJobList:
    """FasTC::CompressionJobList: a bounded list of jobs compressed together."""

    def __init__(self, n_jobs: int):
        self._total = n_jobs
        self._jobs: List[CompressionJob] = []

    def add_job(self, job: CompressionJob) -> bool:
        if len(self._jobs) >= self._total:
            return False
        self._jobs.append(job)
        return True

    def get_total_num_jobs(self) -> int:
        return self._total

    def get_num_jobs(self) -> int:
        return len(self._jobs)

    def get_job(self, idx: int) -> CompressionJob:
        return self._jobs[idx]

    def __iter__(self):
        return iter(self._jobs)


def _stream_handle(stream) -> Optional[int]:
    if stream is not None:
        return int(getattr(stream, "cuda_stream", stream))
    import torch

    return int(torch.cuda.current_stream().cuda_stream)


def _settings_array(settings: Sequence[CompressionSettings]):
    arr = (Settings * len(settings))()
    for i, s in enumerate(settings):
        arr[i] = s.to_c()
    return arr


def compress_jobs(jobs: Sequence[CompressionJob],
                  settings: "CompressionSettings | Sequence[CompressionSettings] | None" = None,
                  stream=None) -> None:
    """Compress a list of jobs in one batched launch (host or device buffers)."""
    lib = load()
    if not jobs:
        return
    per_job = isinstance(settings, (list, tuple))
    if per_job and len(settings) != len(jobs):
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "compress_jobs", "one settings entry per job")
    sarr = _settings_array(settings if per_job else [settings or CompressionSettings()])
    jarr = (Job * len(jobs))()
    for i, j in enumerate(jobs):
        if j.format != CompressionFormat.BPTC:
            raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "compress_jobs",
                           f"a {j.format.name} job: use fastc_gb300.dxt")
        jarr[i] = j.to_c()
    on_dev = {j.on_device for j in jobs}
    if len(on_dev) != 1:
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "compress_jobs", "mixed host and device jobs")
    if on_dev.pop():
        check(lib.fastc_bc7_compress_device(jarr, len(jobs), sarr, int(per_job),
                                            C.c_void_p(_stream_handle(stream))),
              "fastc_bc7_compress_device")
    else:
        check(lib.fastc_bc7_compress_batch(jarr, len(jobs), sarr, int(per_job)),
              "fastc_bc7_compress_batch")


def compress(job: CompressionJob, settings: Optional[CompressionSettings] = None, stream=None) -> None:
    """BPTCC::Compress (BPTCCompressor.h:166)."""
    compress_jobs([job], settings or CompressionSettings(), stream)


def compress_atomic(job_list: CompressionJobList, stream=None) -> None:
    """BPTCC::CompressAtomic (BPTCCompressor.h:189): every job of the list in
    one launch. Like FasTC's, it uses the default CompressionSettings."""
    compress_jobs(list(job_list), CompressionSettings(), stream)


def compress_with_stats(job: CompressionJob, settings: Optional[CompressionSettings] = None) -> str:
    """BPTCC::CompressWithStats (BPTCCompressor.h:173) with a log stream: the
    logging encoder writes the job's blocks to job.out (host arrays) and
    returns FasTC's log text for them (Compressor.cpp:1373-1389,
    1938-2183). Its shape selection differs from compress()'s."""
    if job.on_device:
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "compress_with_stats", "host buffers only")
    lib = load()
    cj = job.to_c()
    n = int(lib.fastc_bc7_job_blocks(C.byref(cj)))
    stats = (_lib.BlockStats * max(n, 1))()
    s = (settings or CompressionSettings()).to_c()
    check(lib.fastc_bc7_compress_stats(C.byref(cj), C.byref(s), C.cast(stats, C.c_void_p)),
          "fastc_bc7_compress_stats")
    size = C.c_size_t()
    check(lib.fastc_bc7_stats_log(C.byref(cj), C.cast(stats, C.c_void_p), None, 0, C.byref(size)),
          "fastc_bc7_stats_log")
    buf = C.create_string_buffer(max(size.value, 1))
    check(lib.fastc_bc7_stats_log(C.byref(cj), C.cast(stats, C.c_void_p), buf, size.value,
                                  C.byref(size)), "fastc_bc7_stats_log")
    return buf.raw[:size.value].decode()


def compress_image_data(data, width: int, height: int,
                        settings: Optional[CompressionSettings] = None,
                        format: CompressionFormat = CompressionFormat.BPTC) -> np.ndarray:
    """CompressImageData (Core/include/FasTC/TexComp.h:81-88; the format
    dispatch of Core/src/TexComp.cpp:110-134): returns the image's blocks,
    width*height bytes for BPTC and DXT5, half that for DXT1. `settings`
    applies to BPTC only."""
    data = np.ascontiguousarray(np.asarray(data, dtype=np.uint8))
    if width % 4 or height % 4:
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "compress_image_data",
                       "width or height is not a multiple of the block dimension")
    format = CompressionFormat(format)
    out = np.zeros(width * height * FORMAT_BLOCK_BYTES[format] // 16, dtype=np.uint8)
    job = CompressionJob(data, out, width, height, format=format)
    if format == CompressionFormat.BPTC:
        compress(job, settings)
    else:
        from . import dxt

        dxt.compress_dxt_jobs([job])
    return out


def decompress(blocks, width: int, height: int, spec_semantics: bool = False, out=None, stream=None):
    """BPTCC::Decompress (BPTCCompressor.h:216): RGBA8 [height, width, 4].

    With ``spec_semantics`` mode-4 blocks in index mode 1 decode as the BC7
    specification says instead of as FasTC's decoder does."""
    lib = load()
    if _is_cuda(blocks):
        import torch

        if out is None:
            out = torch.empty((height, width, 4), dtype=torch.uint8, device=blocks.device)
        check(lib.fastc_bc7_decompress_device(C.c_void_p(blocks.data_ptr()), C.c_void_p(out.data_ptr()),
                                              width, height, int(spec_semantics),
                                              C.c_void_p(_stream_handle(stream))),
              "fastc_bc7_decompress_device")
        return out
    blocks = np.ascontiguousarray(np.asarray(blocks, dtype=np.uint8))
    if out is None:
        out = np.zeros((height, width, 4), dtype=np.uint8)
    check(lib.fastc_bc7_decompress(blocks.ctypes.data_as(_lib.u8p), out.ctypes.data_as(_lib.u8p), width,
                                   height, int(spec_semantics)), "fastc_bc7_decompress")
    return out


def psnr(blocks, rgba, width: int, height: int, block_sse: bool = False, stream=None):
    """Image::ComputePSNR (Base/src/Image.cpp:206-255) of encoded `blocks`
    against the original `rgba`, computed on the GPU: the PSNR in dB, or
    (psnr, per-block SSE) with ``block_sse``. Host arrays go through
    fastc_bc7_psnr; CUDA tensors through fastc_bc7_block_error_device on
    `stream` (the result is read back, which synchronises that stream)."""
    import math

    lib = load()
    nb = ((width + 3) // 4) * ((height + 3) // 4)
    if _is_cuda(blocks):
        import torch

        sse = torch.empty(nb + 1, dtype=torch.float64, device=blocks.device)
        check(lib.fastc_bc7_block_error_device(
            C.c_void_p(blocks.data_ptr()), C.c_void_p(rgba.data_ptr()), width, height,
            C.c_void_p(sse.data_ptr() + 8), C.c_void_p(sse.data_ptr()),
            C.c_void_p(_stream_handle(stream))), "fastc_bc7_block_error_device")
        host = sse.cpu().numpy()
        total, per = float(host[0]), host[1:]
        db = 10.0 * math.log10(3.0 * 255.0 * 255.0 / (total / (width * height))) if total > 0 else math.inf
        return (db, per) if block_sse else db
    blocks = np.ascontiguousarray(np.asarray(blocks, dtype=np.uint8))
    rgba = np.ascontiguousarray(np.asarray(rgba, dtype=np.uint8))
    if blocks.size < nb * 16 or rgba.size < width * height * 4:
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "psnr: buffers smaller than the image")
    out = C.c_double()
    per = np.zeros(nb, dtype=np.float64) if block_sse else None
    check(lib.fastc_bc7_psnr(blocks.ctypes.data, rgba.ctypes.data, width, height, C.byref(out),
                             per.ctypes.data if per is not None else None), "fastc_bc7_psnr")
    return (out.value, per) if block_sse else out.value


class Plan:
    """A fixed set of device jobs captured once into a CUDA graph; each
    :meth:`launch` re-encodes the whole set with one graph launch."""

    def __init__(self, jobs: Sequence[CompressionJob],
                 settings: "CompressionSettings | Sequence[CompressionSettings] | None" = None):
        lib = load()
        if not jobs or not all(j.on_device for j in jobs):
            raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "Plan", "plans take device jobs")
        per_job = isinstance(settings, (list, tuple))
        sarr = _settings_array(settings if per_job else [settings or CompressionSettings()])
        jarr = (Job * len(jobs))()
        for i, j in enumerate(jobs):
            jarr[i] = j.to_c()
        self._jobs = list(jobs)  # keep the buffers alive
        h = C.c_void_p()
        check(lib.fastc_bc7_plan_create(jarr, len(jobs), sarr, int(per_job), C.byref(h)),
              "fastc_bc7_plan_create")
        self._h = h

    @property
    def num_blocks(self) -> int:
        return int(load().fastc_bc7_plan_blocks(self._h))

    def kernels(self) -> int:
        """Kernel launches one launch() makes (kernel nodes of the graph)."""
        return int(load().fastc_bc7_plan_kernels(self._h))

    def autotune(self, stream=None, launches: int = 2) -> dict:
        """Choose the launch parameters on this plan's own jobs (see
        fastc_bc7_plan_autotune); returns the chosen parameters."""
        check(load().fastc_bc7_plan_autotune(self._h, C.c_void_p(_stream_handle(stream)), int(launches)),
              "fastc_bc7_plan_autotune")
        return self.tuning()

    def tuning(self) -> dict:
        """Every parameter the plan's graph was captured with
        (fastc_bc7_plan_get_tuning)."""
        t = _lib.PlanTuning()
        check(load().fastc_bc7_plan_get_tuning(self._h, C.byref(t)), "fastc_bc7_plan_get_tuning")
        return {name: int(getattr(t, name)) for name, _ in _lib.PlanTuning._fields_}

    def launch(self, stream=None) -> None:
        check(load().fastc_bc7_plan_launch(self._h, C.c_void_p(_stream_handle(stream))),
              "fastc_bc7_plan_launch")

    def flags(self) -> int:
        f = C.c_uint32()
        check(load().fastc_bc7_plan_flags(self._h, C.byref(f)), "fastc_bc7_plan_flags")
        return int(f.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            load().fastc_bc7_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


ENGINE_PIPELINE = 0
ENGINE_WARP_PER_BLOCK = 1


def set_engine(engine: int) -> None:
    """Select the encoder organisation for later calls and plans."""
    check(load().fastc_bc7_set_engine(engine), "fastc_bc7_set_engine")


def get_engine() -> int:
    return int(load().fastc_bc7_get_engine())


def set_watermark_counter(next_entry: int) -> None:
    load().fastc_bc7_set_watermark_counter(next_entry)


def get_watermark_counter() -> int:
    return int(load().fastc_bc7_get_watermark_counter())


def set_launch_shape(warps_per_cta: int = 0, ctas_per_sm: int = 0):
    check(load().fastc_bc7_set_launch_shape(warps_per_cta, ctas_per_sm), "fastc_bc7_set_launch_shape")


def get_launch_shape():
    w, c = C.c_int(), C.c_int()
    check(load().fastc_bc7_get_launch_shape(C.byref(w), C.byref(c)), "fastc_bc7_get_launch_shape")
    return w.value, c.value
