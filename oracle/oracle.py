"""ctypes bindings for the oracle libraries. TEST INFRASTRUCTURE ONLY.

* :class:`Port` -- the C restatement (oracle/bc7_oracle.c), built by
  ``make -C oracle port`` into ``oracle/_build/libbc7_oracle.so``.
* :class:`Reference` -- FasTC's own encoders, decoders, PSNR and KTX writer
  compiled in place by ``make -C oracle ref`` into
  ``oracle/_ref/libfastc_ref.so`` (only where the FasTC checkout is present).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libbc7_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfastc_ref.so")
# the FasTC checkout, where this machine has one (FASTC_REFERENCE overrides)
DEFAULT_REFERENCE = os.environ.get("FASTC_REFERENCE", "/root/reference")

RNG_PER_FIT = 0
RNG_SINGLE_STREAM = 1
EXP_PORTABLE = 0
EXP_LIBM = 1

_u8p = C.POINTER(C.c_uint8)
_u32p = C.POINTER(C.c_uint32)


class Settings(C.Structure):
    _fields_ = [("steps", C.c_uint32), ("block_modes", C.c_uint32), ("metric", C.c_uint32),
                ("rng_mode", C.c_uint32), ("seed", C.c_uint32), ("exp_mode", C.c_uint32)]


class BlockStats(C.Structure):
    """bc7o_block_stats: what CompressWithStats logs for one block."""
    _fields_ = [("path", C.c_int32), ("mode", C.c_int32), ("estimate", C.c_double * 8),
                ("error", C.c_double * 8), ("n_two", C.c_int32), ("n_three", C.c_int32),
                ("two_shape", C.c_double * 64), ("three_shape", C.c_double * 64)]


class FitTrace(C.Structure):
    """bc7o_fit_trace: one cluster fit of a traced block."""
    _fields_ = [("mode", C.c_int32), ("slot", C.c_int32), ("subset", C.c_int32),
                ("rot_im", C.c_int32), ("n", C.c_int32), ("annealed", C.c_int32),
                ("init_err", C.c_double), ("final_err", C.c_double), ("lower_bound", C.c_double)]


_MODE_NAMES = ["Zero", "One", "Two", "Three", "Four", "Five", "Six", "Seven"]


def stats_log(blocks) -> str:
    """The text CompressWithStats writes to its log stream for (block index,
    BlockStats) pairs in encode order: one "<index>: BlockStat_<name> --
    <value>" line per statistic (Compressor.cpp:1373-1389, 1951-1993), the
    improving shape estimates first, then the path, then (on return) the
    mode and each mode's estimate and error. Doubles print as an ostream's
    default 6 significant digits, i.e. printf's %g."""
    lines = []
    for idx, st in blocks:
        def put(name, v):
            lines.append(f"{idx}: BlockStat_{name} -- {v}\n")
        for k in range(st.n_two):
            put("TwoShapeEstimate", "%g" % st.two_shape[k])
        for k in range(st.n_three):
            put("ThreeShapeEstimate", "%g" % st.three_shape[k])
        put("Path", st.path)
        put("Mode", st.mode)
        for m in range(8):
            put(f"Mode{_MODE_NAMES[m]}Estimate", "%g" % st.estimate[m])
            put(f"Mode{_MODE_NAMES[m]}Error", "%g" % st.error[m])
    return "".join(lines)


def _ptr(a: np.ndarray, t=_u8p):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(t)


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def build_ref(reference: str = DEFAULT_REFERENCE) -> str | None:
    if not os.path.isdir(os.path.join(reference, "BPTCEncoder")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE={reference}"], check=True)
    return REF_SO


class Port:
    def __init__(self, path: str = PORT_SO):
        if not os.path.exists(path):
            build_port()
        lib = C.CDLL(path)
        lib.bc7o_compress.argtypes = [_u8p, _u8p] + [C.c_uint32] * 6 + [C.POINTER(Settings), _u32p]
        lib.bc7o_compress_mt.argtypes = [_u8p, _u8p, C.c_uint32, C.c_uint32, C.POINTER(Settings),
                                         C.c_uint32, C.c_int]
        lib.bc7o_compress_block.argtypes = [_u32p, C.POINTER(Settings), C.c_uint32, C.c_uint32,
                                            _u32p, _u32p, _u8p]
        lib.bc7o_decompress.argtypes = [_u8p, _u8p, C.c_uint32, C.c_uint32]
        lib.bc7o_psnr.argtypes = [_u8p, _u8p, C.c_uint32, C.c_uint32]
        lib.bc7o_psnr.restype = C.c_double
        lib.bc7o_block_sse.argtypes = [_u8p, _u8p, C.c_uint32, C.c_uint32, C.POINTER(C.c_double)]
        lib.bc7o_box_selection.argtypes = [_u32p, C.c_uint32, _u32p]
        lib.bc7o_tables.argtypes = [_u8p, _u8p]
        lib.bc7o_partition.argtypes = [C.c_uint32, C.c_uint32, _u8p]
        lib.bc7o_anchor.argtypes = [C.c_uint32] * 3
        lib.bc7o_anchor.restype = C.c_uint32
        lib.bc7o_fit_seed.argtypes = [C.c_uint32] * 4
        lib.bc7o_fit_seed.restype = C.c_uint32
        lib.bc7o_expf.argtypes = [C.c_float]
        lib.bc7o_expf.restype = C.c_float
        lib.bc7o_trace_block.argtypes = [_u32p, C.POINTER(Settings), C.c_uint32, C.c_uint32,
                                          _u32p, _u32p, _u8p, C.POINTER(FitTrace), C.c_int]
        lib.dxto_compress.argtypes = [_u8p, _u8p, C.c_uint32, C.c_uint32, C.c_int]
        lib.dxto_decompress.argtypes = [_u8p, _u8p, C.c_uint32, C.c_uint32, C.c_int]
        lib.dxto_tables.argtypes = [_u8p, _u8p]
        lib.bc7o_trace_block.restype = C.c_int
        lib.bc7o_compress_block_stats.argtypes = [_u32p, C.POINTER(Settings), C.c_uint32,
                                                  C.c_uint32, _u32p, _u32p, _u8p,
                                                  C.POINTER(BlockStats)]
        self.lib = lib

    def qe_counters(self, reset: bool = False):
        """(QuantizedError calls, texel-bucket evaluations) summed over all
        threads since the last reset (diagnostic work counters)."""
        out = np.zeros(2, dtype=np.uint64)
        self.lib.bc7o_qe_counters(out.ctypes.data_as(C.POINTER(C.c_uint64)), int(reset))
        return int(out[0]), int(out[1])

    def trace(self, img: np.ndarray, steps=0, modes=0xFF, metric=0, seed=0):
        """Every block's cluster fits (per-fit RNG), in raster block order:
        (blocks, [list of FitTrace per block])."""
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        out = np.zeros(w * h, dtype=np.uint8)
        s = self.settings(steps, modes, metric, RNG_PER_FIT, seed, EXP_PORTABLE)
        st = np.zeros(2, dtype=np.uint32)
        fits = (FitTrace * 64)()
        per_block = []
        bw = w // 4
        for by in range(h // 4):
            for bx in range(bw):
                px = np.ascontiguousarray(
                    img[4 * by:4 * by + 4, 4 * bx:4 * bx + 4].reshape(16, 4)).view(np.uint32).reshape(16)
                dst = np.zeros(16, dtype=np.uint8)
                n = self.lib.bc7o_trace_block(_ptr(px, _u32p), C.byref(s), bx, by,
                                              _ptr(st[1:2], _u32p), _ptr(st[0:1], _u32p), _ptr(dst),
                                              fits, 64)
                i = by * bw + bx
                out[16 * i:16 * i + 16] = dst
                per_block.append([FitTrace.from_buffer_copy(fits[k]) for k in range(n)])
        return out, per_block

    def compress_stats(self, img: np.ndarray, steps=0, modes=0xFF, metric=0,
                       rng_mode=RNG_PER_FIT, seed=0, exp_mode=EXP_PORTABLE, state=None):
        """The logging encoder (CompressWithStats with a log stream) over a
        whole image in raster block order: (blocks, [(block index,
        BlockStats)]). state = [LCG state, watermark counter], updated."""
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        out = np.zeros(w * h, dtype=np.uint8)
        st = np.zeros(2, dtype=np.uint32) if state is None else state
        s = self.settings(steps, modes, metric, rng_mode, seed, exp_mode)
        lcg = st[0:1]
        wm = st[1:2]
        blocks = []
        bw = w // 4
        for by in range(h // 4):
            for bx in range(bw):
                px = np.ascontiguousarray(
                    img[4 * by:4 * by + 4, 4 * bx:4 * bx + 4].reshape(16, 4)).view(np.uint32).reshape(16)
                dst = np.zeros(16, dtype=np.uint8)
                bs = BlockStats()
                self.lib.bc7o_compress_block_stats(_ptr(px, _u32p), C.byref(s), bx, by,
                                                   _ptr(wm, _u32p), _ptr(lcg, _u32p), _ptr(dst),
                                                   C.byref(bs))
                i = by * bw + bx
                out[16 * i:16 * i + 16] = dst
                blocks.append((i, bs))
        return out, blocks

    @staticmethod
    def settings(steps=0, modes=0xFF, metric=0, rng_mode=RNG_PER_FIT, seed=0,
                 exp_mode=EXP_PORTABLE) -> Settings:
        return Settings(steps, modes, metric, rng_mode, seed, exp_mode)

    def compress(self, img: np.ndarray, steps=0, modes=0xFF, metric=0, rng_mode=RNG_PER_FIT,
                 seed=0, exp_mode=EXP_PORTABLE, rect=(0, 0, 0, 0), state=None,
                 out=None) -> np.ndarray:
        """`out`: a w*h-byte buffer to write into (only the rect's blocks are
        written), e.g. reused across calls on sub-ranges of one image."""
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        if out is None:
            out = np.zeros(w * h, dtype=np.uint8)
        assert out.dtype == np.uint8 and out.size >= w * h and out.flags["C_CONTIGUOUS"]
        st = np.zeros(2, dtype=np.uint32) if state is None else state
        s = self.settings(steps, modes, metric, rng_mode, seed, exp_mode)
        rc = self.lib.bc7o_compress(_ptr(img), _ptr(out), w, h, *rect, C.byref(s), _ptr(st, _u32p))
        if rc:
            raise ValueError(f"bc7o_compress failed: {rc}")
        return out

    def compress_mt(self, img: np.ndarray, steps=0, modes=0xFF, metric=0, seed=0, wm_start=0,
                    threads=None) -> np.ndarray:
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        out = np.zeros(w * h, dtype=np.uint8)
        s = self.settings(steps, modes, metric, RNG_PER_FIT, seed, EXP_PORTABLE)
        rc = self.lib.bc7o_compress_mt(_ptr(img), _ptr(out), w, h, C.byref(s), wm_start,
                                       threads or os.cpu_count() or 1)
        if rc:
            raise ValueError(f"bc7o_compress_mt failed: {rc}")
        return out

    def decompress(self, blocks: np.ndarray, w: int, h: int) -> np.ndarray:
        blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
        out = np.zeros((h, w, 4), dtype=np.uint8)
        self.lib.bc7o_decompress(_ptr(blocks), _ptr(out), w, h)
        return out

    def psnr(self, a: np.ndarray, b: np.ndarray) -> float:
        a = np.ascontiguousarray(a, dtype=np.uint8)
        b = np.ascontiguousarray(b, dtype=np.uint8)
        return float(self.lib.bc7o_psnr(_ptr(a), _ptr(b), a.shape[1], a.shape[0]))

    def block_sse(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=np.uint8)
        b = np.ascontiguousarray(b, dtype=np.uint8)
        h, w = a.shape[:2]
        out = np.zeros((h // 4) * (w // 4), dtype=np.float64)
        self.lib.bc7o_block_sse(_ptr(a), _ptr(b), w, h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def dxt_compress(self, img: np.ndarray, alpha: bool) -> np.ndarray:
        """The DXT restatement (oracle/dxt_oracle.c): DXT5 when `alpha`."""
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        out = np.zeros((w // 4) * (h // 4) * (16 if alpha else 8), dtype=np.uint8)
        if self.lib.dxto_compress(_ptr(img), _ptr(out), w, h, int(alpha)):
            raise ValueError("dxto_compress: sizes must be multiples of 4")
        return out

    def dxt_decompress(self, blocks: np.ndarray, w: int, h: int, alpha: bool) -> np.ndarray:
        blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
        out = np.zeros((h, w, 4), dtype=np.uint8)
        self.lib.dxto_decompress(_ptr(blocks), _ptr(out), w, h, int(alpha))
        return out

    def dxt_tables(self):
        m5 = np.zeros(512, dtype=np.uint8)
        m6 = np.zeros(512, dtype=np.uint8)
        self.lib.dxto_tables(_ptr(m5), _ptr(m6))
        return m5, m6

    def box_selection(self, px: np.ndarray, metric=0):
        px = np.ascontiguousarray(px, dtype=np.uint32)
        out = np.zeros(4, dtype=np.uint32)
        self.lib.bc7o_box_selection(_ptr(px, _u32p), metric, _ptr(out, _u32p))
        return tuple(int(v) for v in out)

    def tables(self):
        o7 = np.zeros(512, dtype=np.uint8)
        o6 = np.zeros(1536, dtype=np.uint8)
        self.lib.bc7o_tables(_ptr(o7), _ptr(o6))
        return o7, o6

    def partition(self, shape: int, nsub: int) -> np.ndarray:
        out = np.zeros(16, dtype=np.uint8)
        self.lib.bc7o_partition(shape, nsub, _ptr(out))
        return out


class Reference:
    """FasTC's encoder itself, compiled in place (x86-64 container only)."""

    def __init__(self, path: str = REF_SO):
        lib = C.CDLL(path)
        lib.ref_set_seed.argtypes = [C.c_uint32]
        lib.ref_get_seed.restype = C.c_uint32
        lib.ref_set_wm.argtypes = [C.c_uint32]
        lib.ref_get_wm.restype = C.c_uint32
        lib.ref_compress.argtypes = [_u8p, _u8p] + [C.c_uint32] * 8 + [C.c_int]
        lib.ref_compress_block.argtypes = [_u32p, _u8p, C.c_uint32, C.c_uint32, C.c_int]
        lib.ref_decompress.argtypes = [_u8p, _u8p, C.c_uint32, C.c_uint32]
        lib.ref_box_selection.argtypes = [_u32p, C.c_int, _u32p]
        lib.ref_tables.argtypes = [_u8p, _u8p]
        lib.ref_compress_stats.argtypes = [_u8p, _u8p] + [C.c_uint32] * 8 + [C.c_int, C.c_char_p,
                                                                          C.c_size_t]
        lib.ref_compress_stats.restype = C.c_size_t
        lib.ref_dxt_compress.argtypes = [_u8p, _u8p, C.c_uint32, C.c_uint32, C.c_int]
        lib.ref_dxt_decompress.argtypes = [_u8p, _u8p, C.c_uint32, C.c_uint32, C.c_int]
        lib.ref_tc_psnr.argtypes = [_u8p, _u8p, C.c_uint32, C.c_uint32, C.c_int]
        lib.ref_tc_psnr.restype = C.c_double
        lib.ref_ktx.argtypes = [_u8p, C.c_uint32, C.c_uint32, C.c_int, _u8p, C.c_uint64]
        lib.ref_ktx.restype = C.c_int64
        self.lib = lib

    def dxt_compress(self, img: np.ndarray, alpha: bool) -> np.ndarray:
        """DXTC::CompressImageDXT1 / DXT5 over the whole image."""
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        out = np.zeros((w // 4) * (h // 4) * (16 if alpha else 8), dtype=np.uint8)
        self.lib.ref_dxt_compress(_ptr(img), _ptr(out), w, h, int(alpha))
        return out

    def dxt_decompress(self, blocks: np.ndarray, w: int, h: int, alpha: bool) -> np.ndarray:
        blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
        out = np.zeros((h, w, 4), dtype=np.uint8)
        self.lib.ref_dxt_decompress(_ptr(blocks), _ptr(out), w, h, int(alpha))
        return out

    def compress_stats(self, img: np.ndarray, steps=0, modes=0xFF, metric=0, seed=None, wm=0):
        """BPTCC::CompressWithStats with a log stream: (blocks, log text).
        Its block loop runs while the row is <= YEnd without Compress's clamp
        to height - 4 (Compressor.cpp:1583-1584), so a whole-image job
        (YEnd = height) reads and writes one block row past the buffers; the
        job here ends at the last block row (YEnd = height - 4)."""
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        out = np.zeros(w * h, dtype=np.uint8)
        if seed is not None:
            self.lib.ref_set_seed(seed)
        self.lib.ref_set_wm((wm - 1) & 0xFFFFFFFF if wm else 0xFFFFFFFF)
        cap = 1 << 16
        while True:
            buf = C.create_string_buffer(cap)
            n = self.lib.ref_compress_stats(_ptr(img), _ptr(out), w, h, 0, 0, w, h - 4, steps,
                                            modes, metric, buf, cap)
            if n < cap:
                return out, buf.value.decode()
            cap = n + 1
            if seed is not None:
                self.lib.ref_set_seed(seed)
            self.lib.ref_set_wm((wm - 1) & 0xFFFFFFFF if wm else 0xFFFFFFFF)

    def compress(self, img: np.ndarray, steps=0, modes=0xFF, metric=0, seed=None, wm=0,
                 rect=None) -> np.ndarray:
        """Fresh watermark counter (next single-colour block uses entry `wm`)."""
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        out = np.zeros(w * h, dtype=np.uint8)
        if seed is not None:
            self.lib.ref_set_seed(seed)
        self.lib.ref_set_wm((wm - 1) & 0xFFFFFFFF if wm else 0xFFFFFFFF)
        x0, y0, x1, y1 = rect if rect else (0, 0, w, h)
        self.lib.ref_compress(_ptr(img), _ptr(out), w, h, x0, y0, x1, y1, steps, modes, metric)
        return out

    def compress_threads(self, img: np.ndarray, steps=50, threads=1, seed=None) -> np.ndarray:
        """`tc -t N`: N threads compress disjoint block ranges of one image,
        split like Core/src/ThreadGroup.cpp:133-192 (they share FasTC's
        global RNG state, racing on it exactly as the reference does)."""
        import threading

        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        out = np.zeros(w * h, dtype=np.uint8)
        if seed is not None:
            self.lib.ref_set_seed(seed)
        bw = w // 4
        nb = bw * (h // 4)
        per = nb // threads + (1 if nb % threads else 0)
        ranges, done = [], 0
        while done < nb:
            e = min(done + per, nb)
            ranges.append(((done % bw) * 4, (done // bw) * 4, (e % bw) * 4, (e // bw) * 4))
            done = e
        ts = [threading.Thread(target=self.lib.ref_compress,
                               args=(_ptr(img), _ptr(out), w, h, *r, steps, 0xFF, 0)) for r in ranges]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        return out

    def decompress(self, blocks: np.ndarray, w: int, h: int) -> np.ndarray:
        blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
        out = np.zeros((h, w, 4), dtype=np.uint8)
        self.lib.ref_decompress(_ptr(blocks), _ptr(out), w, h)
        return out

    def tc_psnr(self, img: np.ndarray, blocks: np.ndarray, fmt: int = 7) -> float:
        """The PSNR FasTC's tc prints for these blocks of img (format code
        1 = DXT1, 5 = DXT5, 7 = BPTC), from FasTC's own CompressedImage
        decoder and Image::ComputePSNR."""
        img = np.ascontiguousarray(img, dtype=np.uint8)
        blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
        h, w = img.shape[:2]
        return float(self.lib.ref_tc_psnr(_ptr(img), _ptr(blocks), w, h, fmt))

    def ktx(self, blocks: np.ndarray, w: int, h: int, fmt: int = 7) -> bytes:
        """The KTX file FasTC's ImageWriterKTX writes for these blocks. Its
        image size is a function-local static, so only the first call per
        format group in a process gives the file one tc run writes."""
        blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
        out = np.zeros(len(blocks) + 4096, dtype=np.uint8)
        n = self.lib.ref_ktx(_ptr(blocks), w, h, fmt, _ptr(out), out.size)
        if n <= 0:
            raise RuntimeError(f"ImageWriterKTX refused ({n})")
        return out[:n].tobytes()

    def load_tga(self, raw: bytes):
        """The RGBA8 (h, w, 4) texels FasTC's TGA loader reads from a file,
        or None when it refuses the file."""
        lib = self.lib
        lib.ref_load_tga.argtypes = [C.c_char_p, C.c_int32, _u8p, C.c_uint64,
                                     C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        lib.ref_load_tga.restype = C.c_int64
        w, h = C.c_uint32(0), C.c_uint32(0)
        n = lib.ref_load_tga(raw, len(raw), None, 0, C.byref(w), C.byref(h))
        if n <= 0:
            return None
        out = np.zeros((h.value, w.value, 4), dtype=np.uint8)
        lib.ref_load_tga(raw, len(raw), _ptr(out), out.size, C.byref(w), C.byref(h))
        return out

    def load_ktx(self, raw: bytes):
        """The RGBA8 (h, w, 4) texels FasTC's KTX loader reads from an
        uncompressed file; "compressed" for a file it loads as a
        CompressedImage; None when it refuses the file."""
        lib = self.lib
        lib.ref_load_ktx.argtypes = [C.c_char_p, C.c_int32, _u8p, C.c_uint64,
                                     C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        lib.ref_load_ktx.restype = C.c_int64
        w, h = C.c_uint32(0), C.c_uint32(0)
        n = lib.ref_load_ktx(raw, len(raw), None, 0, C.byref(w), C.byref(h))
        if n == 0:
            return None
        if n < 0:
            return "compressed"
        out = np.zeros((h.value, w.value, 4), dtype=np.uint8)
        lib.ref_load_ktx(raw, len(raw), _ptr(out), out.size, C.byref(w), C.byref(h))
        return out

    def box_selection(self, px: np.ndarray, metric=0):
        px = np.ascontiguousarray(px, dtype=np.uint32)
        out = np.zeros(4, dtype=np.uint32)
        self.lib.ref_box_selection(_ptr(px, _u32p), metric, _ptr(out, _u32p))
        return tuple(int(v) for v in out)

    def tables(self):
        o7 = np.zeros(512, dtype=np.uint8)
        o6 = np.zeros(1536, dtype=np.uint8)
        self.lib.ref_tables(_ptr(o7), _ptr(o6))
        return o7, o6
