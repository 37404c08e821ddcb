"""Python front end of the continuous-batching BC7 (and DXT1 / DXT5)
request server.

The server itself (admission by device-memory budget, batches on several
streams, completion callbacks) is native code in the library; this module
keeps the request buffers alive and converts results and statistics.

    with Server(memory_budget=8 << 30) as srv:
        req = srv.submit(rgba, CompressionSettings(num_simulated_annealing_steps=16))
        blocks = srv.wait(req)          # numpy uint8, width*height bytes
        dxt = srv.submit(rgba, format=CompressionFormat.DXT1)  # same queue and batches
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib
from ._lib import BC7Error, Job, ServerConfig, ServerStats, check, load
from .bptc import FORMAT_BLOCK_BYTES, CompressionFormat, CompressionSettings


@dataclass
class Request:
    """A submitted request; holds its input and output buffers."""

    id: int
    rgba: np.ndarray
    out: np.ndarray
    width: int
    height: int


class Server:
    """fastc_bc7_server_* over ctypes."""

    def __init__(self, memory_budget: int = 8 << 30, max_inflight: int = 3,
                 max_batch_blocks: int = 1 << 22, max_batch_jobs: int = 4096):
        lib = load()
        cfg = ServerConfig()
        lib.fastc_bc7_server_config_default(C.byref(cfg))
        cfg.memory_budget = int(memory_budget)
        cfg.max_inflight = int(max_inflight)
        cfg.max_batch_blocks = int(max_batch_blocks)
        cfg.max_batch_jobs = int(max_batch_jobs)
        h = C.c_void_p()
        check(lib.fastc_bc7_server_create(C.byref(cfg), C.byref(h)), "fastc_bc7_server_create")
        self._h = h
        self._lib = lib

    def submit(self, rgba: np.ndarray, settings: Optional[CompressionSettings] = None,
               out: Optional[np.ndarray] = None,
               format: CompressionFormat = CompressionFormat.BPTC,
               rect: Optional[tuple] = None) -> Request:
        """Queue one texture: BC7 with `settings`, or DXT1 / DXT5 (settings
        do not apply) through fastc_dxt_server_submit. `rect` = (x_start,
        y_start, x_end, y_end) limits the request to a sub-job in FasTC's
        sense (blocks from (x_start, y_start) in raster order up to x_end on
        row y_end); its blocks go to their places in `out`."""
        rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
        h, w = rgba.shape[:2]
        fmt = CompressionFormat(format)
        if out is None:
            out = np.zeros(w * h * FORMAT_BLOCK_BYTES[fmt] // 16, dtype=np.uint8)
        x0, y0, x1, y1 = rect if rect is not None else (0, 0, w, h)
        job = Job(rgba.ctypes.data, out.ctypes.data, w, h, x0, y0, x1, y1)
        rid = C.c_uint64()
        if fmt == CompressionFormat.BPTC:
            s = (settings or CompressionSettings()).to_c()
            st = self._lib.fastc_bc7_server_submit(self._h, C.byref(job), C.byref(s), C.byref(rid))
            name = "fastc_bc7_server_submit"
        else:
            st = self._lib.fastc_dxt_server_submit(self._h, C.byref(job), int(fmt), C.byref(rid))
            name = "fastc_dxt_server_submit"
        if st != _lib.OK:
            raise BC7Error(st, name)
        return Request(int(rid.value), rgba, out, w, h)

    def poll(self, req: Request) -> bool:
        st = self._lib.fastc_bc7_server_poll(self._h, req.id)
        if st == _lib.ERR_TIMEOUT:
            return False
        check(st, "fastc_bc7_server_poll")
        return True

    def wait(self, req: Request, timeout_ms: int = -1) -> np.ndarray:
        check(self._lib.fastc_bc7_server_wait(self._h, req.id, int(timeout_ms)), "fastc_bc7_server_wait")
        return req.out

    def psnr(self, req: Request) -> float:
        """The PSNR of a finished request (FasTC's metric, measured on the
        device after its encode)."""
        v = C.c_double()
        check(self._lib.fastc_bc7_server_request_psnr(self._h, req.id, C.byref(v)),
              "fastc_bc7_server_request_psnr")
        return v.value

    def cancel(self, req: Request) -> None:
        check(self._lib.fastc_bc7_server_cancel(self._h, req.id), "fastc_bc7_server_cancel")

    def release(self, req: Request) -> None:
        check(self._lib.fastc_bc7_server_release(self._h, req.id), "fastc_bc7_server_release")

    def stats(self) -> dict:
        s = ServerStats()
        check(self._lib.fastc_bc7_server_get_stats(self._h, C.byref(s)), "fastc_bc7_server_get_stats")
        return {name: getattr(s, name) for name, _ in ServerStats._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fastc_bc7_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
