"""GB300-native BC7 (BPTC) texture encoder with FasTC's compression API.

The compute path is hand-written sm_103a CUDA in ``fastc_gb300/csrc`` behind
the C ABI in ``include/fastc_bc7.h``; this package is the Python mirror of
FasTC's BPTC interface (:mod:`fastc_gb300.bptc`) and of its DXT1/DXT5 path
(:mod:`fastc_gb300.dxt`), the batching/serving runtime, and the seeded
synthetic workloads.
"""
from . import dxt
from .bptc import (WATERMARK_CONTINUE, BC7Error, BlockMode, CompressionFormat, CompressionJob, CompressionJobList, CompressionSettings,
                   ErrorMetric, Plan, compress, compress_atomic, compress_image_data, compress_jobs,
                   compress_with_stats,
                   decompress, psnr, get_engine, get_launch_shape, get_watermark_counter, set_engine,
                   set_launch_shape, set_watermark_counter, ENGINE_PIPELINE, ENGINE_WARP_PER_BLOCK)

__all__ = [
    "BC7Error", "BlockMode", "CompressionFormat", "CompressionJob", "CompressionJobList", "CompressionSettings",
    "ErrorMetric", "Plan", "compress", "compress_atomic", "compress_image_data", "compress_jobs",
    "compress_with_stats",
    "decompress", "psnr", "get_launch_shape", "set_launch_shape", "WATERMARK_CONTINUE",
    "get_watermark_counter", "set_watermark_counter", "get_engine", "set_engine",
    "ENGINE_PIPELINE", "ENGINE_WARP_PER_BLOCK", "dxt",
]
