"""DXT1 / DXT5 (BC1 / BC3) over the GB300 C ABI: FasTC's DXTC namespace
(DXTEncoder/include/FasTC/DXTCompressor.h:22-29).

CompressImageDXT1 / CompressImageDXT5 (Compressor.cpp:47-93) take a
:class:`CompressionJob` whose output holds 8 (DXT1) or 16 (DXT5) bytes per
block, indexed from the texture's first block; the blocks equal FasTC's byte
for byte. DecompressDXT1 / DecompressDXT5 (Decompressor.cpp:98-155) return
RGBA8 texels. Host arrays are copied to the GPU and back; CUDA tensors are
encoded in place on the given (or current torch) stream.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import BC7Error, Job, check, load
from .bptc import CompressionFormat, CompressionJob, _is_cuda, _stream_handle


def compress_dxt_jobs(jobs: Sequence[CompressionJob], stream=None) -> None:
    """Every job of one DXT format in one call: device jobs are encoded in
    place in launches of up to 32 jobs; host jobs go through the batched
    host entry point (copies overlapped with the encode)."""
    if not jobs:
        return
    fmts = {j.format for j in jobs}
    if len(fmts) != 1 or fmts & {CompressionFormat.BPTC}:
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "compress_dxt_jobs", "jobs of one DXT format")
    fmt = int(fmts.pop())
    on_dev = {j.on_device for j in jobs}
    if len(on_dev) != 1:
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "compress_dxt_jobs", "mixed host and device jobs")
    lib = load()
    jarr = (Job * len(jobs))(*[j.to_c() for j in jobs])
    if on_dev.pop():
        check(lib.fastc_dxt_compress_device(jarr, len(jobs), fmt, C.c_void_p(_stream_handle(stream))),
              "fastc_dxt_compress_device")
    else:
        check(lib.fastc_dxt_compress_batch(jarr, len(jobs), fmt), "fastc_dxt_compress_batch")


def _with_format(job: CompressionJob, fmt: CompressionFormat) -> CompressionJob:
    if job.format == fmt:
        return job
    return CompressionJob(job.in_buf, job.out_buf, job.width, job.height, job.x_start, job.y_start,
                          job.x_end, job.y_end, format=fmt)


def compress_image_dxt1(job: CompressionJob, stream=None) -> None:
    """DXTC::CompressImageDXT1 (DXTCompressor.h:24)."""
    compress_dxt_jobs([_with_format(job, CompressionFormat.DXT1)], stream)


def compress_image_dxt5(job: CompressionJob, stream=None) -> None:
    """DXTC::CompressImageDXT5 (DXTCompressor.h:25)."""
    compress_dxt_jobs([_with_format(job, CompressionFormat.DXT5)], stream)


def decompress(blocks, width: int, height: int, format: CompressionFormat, out=None, stream=None):
    """RGBA8 [height, width, 4] of DXT1 or DXT5 `blocks`."""
    format = CompressionFormat(format)
    if format == CompressionFormat.BPTC:
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "dxt.decompress", "a DXT format")
    lib = load()
    nbytes = ((width + 3) // 4) * ((height + 3) // 4) * (8 if format == CompressionFormat.DXT1 else 16)
    if _is_cuda(blocks):
        import torch

        if out is None:
            out = torch.empty((height, width, 4), dtype=torch.uint8, device=blocks.device)
        if blocks.numel() * blocks.element_size() < nbytes or out.numel() * out.element_size() < width * height * 4:
            raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "dxt.decompress", "buffers smaller than the image")
        check(lib.fastc_dxt_decompress_device(C.c_void_p(blocks.data_ptr()), C.c_void_p(out.data_ptr()),
                                              width, height, int(format),
                                              C.c_void_p(_stream_handle(stream))),
              "fastc_dxt_decompress_device")
        return out
    blocks = np.ascontiguousarray(np.asarray(blocks, dtype=np.uint8))
    if out is None:
        out = np.zeros((height, width, 4), dtype=np.uint8)
    if blocks.size < nbytes or out.nbytes < width * height * 4 or not out.flags["C_CONTIGUOUS"]:
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "dxt.decompress", "buffers smaller than the image")
    check(lib.fastc_dxt_decompress(blocks.ctypes.data_as(_lib.u8p), out.ctypes.data_as(_lib.u8p), width,
                                   height, int(format)), "fastc_dxt_decompress")
    return out


def decompress_dxt1(blocks, width: int, height: int, out=None, stream=None):
    """DXTC::DecompressDXT1 (DXTCompressor.h:27)."""
    return decompress(blocks, width, height, CompressionFormat.DXT1, out, stream)


def decompress_dxt5(blocks, width: int, height: int, out=None, stream=None):
    """DXTC::DecompressDXT5 (DXTCompressor.h:28)."""
    return decompress(blocks, width, height, CompressionFormat.DXT5, out, stream)


def psnr(blocks, rgba, width: int, height: int, format: CompressionFormat, block_sse: bool = False,
         stream=None):
    """Image::ComputePSNR (Base/src/Image.cpp:206-255) of DXT1 / DXT5
    `blocks` against the original `rgba`, decoded and compared on the GPU:
    the PSNR in dB, or (psnr, per-block SSE) with ``block_sse``. CUDA
    tensors are read on `stream` (the result is copied back, which
    synchronises it)."""
    import math

    format = CompressionFormat(format)
    if format == CompressionFormat.BPTC:
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "dxt.psnr", "a DXT format")
    lib = load()
    nb = ((width + 3) // 4) * ((height + 3) // 4)
    if _is_cuda(blocks):
        import torch

        sse = torch.empty(nb + 1, dtype=torch.float64, device=blocks.device)
        check(lib.fastc_dxt_block_error_device(
            C.c_void_p(blocks.data_ptr()), C.c_void_p(rgba.data_ptr()), width, height, int(format),
            C.c_void_p(sse.data_ptr() + 8), C.c_void_p(sse.data_ptr()),
            C.c_void_p(_stream_handle(stream))), "fastc_dxt_block_error_device")
        host = sse.cpu().numpy()
        total, per = float(host[0]), host[1:]
        db = 10.0 * math.log10(3.0 * 255.0 * 255.0 / (total / (width * height))) if total > 0 else math.inf
        return (db, per) if block_sse else db
    blocks = np.ascontiguousarray(np.asarray(blocks, dtype=np.uint8))
    rgba = np.ascontiguousarray(np.asarray(rgba, dtype=np.uint8))
    if blocks.size < nb * (8 if format == CompressionFormat.DXT1 else 16) or rgba.size < width * height * 4:
        raise BC7Error(_lib.ERR_INVALID_ARGUMENT, "dxt.psnr", "buffers smaller than the image")
    out = C.c_double()
    per = np.zeros(nb, dtype=np.float64) if block_sse else None
    check(lib.fastc_dxt_psnr(blocks.ctypes.data, rgba.ctypes.data, width, height, int(format), C.byref(out),
                             per.ctypes.data if per is not None else None), "fastc_dxt_psnr")
    return (out.value, per) if block_sse else out.value
