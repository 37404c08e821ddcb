"""The C-ABI library builds, loads and exports what include/fastc_bc7.h
declares; host-side validation works without a GPU. No kernel launches."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fastc_bc7.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fastc_(?:bc7|dxt)_\w+)\s*\(", src)))


def test_header_and_binding_agree():
    from fastc_gb300 import _lib

    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol(bc7lib):
    for name in declared_functions():
        assert hasattr(bc7lib, name), name


def test_exports_nothing_else(bc7lib):
    import subprocess

    from fastc_gb300 import _lib

    out = subprocess.run(["nm", "-D", "--defined-only", _lib.lib_path()], capture_output=True,
                         text=True).stdout
    ours = {l.split()[-1] for l in out.splitlines() if " T " in l and l.split()[-1].startswith("fastc")}
    assert ours == set(declared_functions())


def test_settings_defaults_mirror_fastc(bc7lib):
    from fastc_gb300._lib import Settings

    s = Settings()
    bc7lib.fastc_bc7_settings_default(C.byref(s))
    # BPTCCompressor.h:150-156: all modes, uniform metric, 50 steps
    assert (s.block_modes, s.error_metric, s.steps) == (0xFF, 0, 50)
    assert s.shape_selection_fn is None and s.seed == 0 and s.watermark_start == 0
    assert bc7lib.fastc_bc7_abi_version() == 2


def test_status_strings(bc7lib):
    for st in range(11):
        assert bc7lib.fastc_bc7_status_string(st)


@pytest.mark.parametrize("w,h,x0,y0,x1,y1,want", [
    (16, 16, 0, 0, 16, 16, 16),
    (16, 16, 0, 0, 0, 16, 16),      # y_end past the last row: whole image
    (16, 16, 4, 4, 8, 8, 3 + 2),    # FasTC raster range: rest of row 1, row 2 up to x=8
    (16, 16, 0, 4, 16, 4, 4),       # one full row
    (16, 12, 0, 0, 0, 8, 8),        # y_end on a row, x_end 0
    (8, 8, 0, 0, 8, 8, 4),
    (6, 8, 0, 0, 6, 8, 0),          # width not a multiple of 4
    (16, 16, 2, 0, 16, 16, 0),      # unaligned start
    (16, 16, 16, 0, 16, 16, 0),     # start past the row
])
def test_job_block_ranges(bc7lib, w, h, x0, y0, x1, y1, want):
    from fastc_gb300._lib import Job

    j = Job(1, 1, w, h, x0, y0, x1, y1)
    assert bc7lib.fastc_bc7_job_blocks(C.byref(j)) == want


def test_threadgroup_split_covers_image_once(bc7lib):
    """FasTC's ThreadGroup (Core/src/ThreadGroup.cpp:133-192) splits an image
    into sub-jobs by block index; their ranges must tile the image."""
    from fastc_gb300._lib import Job

    w, h = 64, 48
    nblocks = (w // 4) * (h // 4)
    for threads in (1, 2, 3, 5, 7, 16):
        per = nblocks // threads + (1 if nblocks % threads else 0)
        done = 0
        total = 0
        while done < nblocks:
            n = min(per, nblocks - done)
            sx, sy = (done % (w // 4)) * 4, (done // (w // 4)) * 4
            e = done + n
            ex, ey = (e % (w // 4)) * 4, (e // (w // 4)) * 4
            j = Job(1, 1, w, h, sx, sy, ex, ey)
            total += bc7lib.fastc_bc7_job_blocks(C.byref(j))
            done = e
        assert total == nblocks


def test_host_callback_rejected():
    from fastc_gb300 import BC7Error, CompressionJob, CompressionSettings, compress

    img = np.zeros((8, 8, 4), np.uint8)
    out = np.zeros(64, np.uint8)
    with pytest.raises(BC7Error) as e:
        compress(CompressionJob(img, out, 8, 8), CompressionSettings(shape_selection_fn=lambda *a: 0))
    assert e.value.status == 2


def test_invalid_arguments_rejected_before_any_device_work(bc7lib):
    from fastc_gb300._lib import Job, Settings

    s = Settings()
    bc7lib.fastc_bc7_settings_default(C.byref(s))
    buf = (C.c_uint8 * 1024)()
    addr = C.addressof(buf)
    assert bc7lib.fastc_bc7_compress(C.byref(Job(addr, addr, 6, 8, 0, 0, 6, 8)), C.byref(s)) == 1
    s.block_modes = 0
    assert bc7lib.fastc_bc7_compress(C.byref(Job(addr, addr, 8, 8, 0, 0, 8, 8)), C.byref(s)) == 1
    s.block_modes = 0xFF
    s.steps = 257
    assert bc7lib.fastc_bc7_compress(C.byref(Job(addr, addr, 8, 8, 0, 0, 8, 8)), C.byref(s)) == 1
    assert bc7lib.fastc_bc7_set_launch_shape(3, 0) == 1


def test_no_device_fails_loudly(bc7lib):
    from conftest import cuda_available

    if cuda_available():
        pytest.skip("a GPU is present")
    from fastc_gb300 import BC7Error, compress_image_data

    with pytest.raises(BC7Error):
        compress_image_data(np.zeros((8, 8, 4), np.uint8), 8, 8)


def test_dxt_invalid_arguments_rejected(bc7lib):
    from fastc_gb300._lib import Job

    buf = (C.c_uint8 * 4096)()
    addr = C.addressof(buf)
    ok = Job(addr, addr, 8, 8, 0, 0, 8, 8)
    assert bc7lib.fastc_dxt_compress(C.byref(ok), 3) == 1                      # no such format
    assert bc7lib.fastc_dxt_compress(C.byref(Job(addr, addr, 6, 8, 0, 0, 6, 8)), 1) == 1
    assert bc7lib.fastc_dxt_compress(C.byref(Job(addr + 2, addr, 8, 8, 0, 0, 8, 8)), 5) == 1
    assert bc7lib.fastc_dxt_compress(C.byref(Job(0, addr, 8, 8, 0, 0, 8, 8)), 1) == 1
    assert bc7lib.fastc_dxt_compress_device(None, 1, 1, None) == 1
    assert bc7lib.fastc_dxt_decompress(None, C.cast(addr, C.POINTER(C.c_uint8)), 8, 8, 5) == 1
    assert bc7lib.fastc_dxt_decompress_device(addr, addr, 0, 8, 1, None) == 1


def test_dxt_job_output_sizes():
    from fastc_gb300 import BC7Error, CompressionFormat, CompressionJob

    img = np.zeros((8, 8, 4), np.uint8)
    CompressionJob(img, np.zeros(32, np.uint8), 8, 8, format=CompressionFormat.DXT1)
    with pytest.raises(BC7Error):
        CompressionJob(img, np.zeros(32, np.uint8), 8, 8, format=CompressionFormat.DXT5)
    with pytest.raises(BC7Error):
        CompressionJob(img, np.zeros(32, np.uint8), 8, 8)


def test_bptc_entry_rejects_dxt_jobs():
    from fastc_gb300 import BC7Error, CompressionFormat, CompressionJob, compress

    img = np.zeros((8, 8, 4), np.uint8)
    with pytest.raises(BC7Error):
        compress(CompressionJob(img, np.zeros(64, np.uint8), 8, 8, format=CompressionFormat.DXT5))


def test_dxt_empty_ranges_need_no_device(bc7lib):
    """Jobs whose raster range holds no block (FasTC's walk writes nothing)
    return OK at once, on host and device entry points, without a GPU."""
    from fastc_gb300._lib import Job

    buf = (C.c_uint8 * 4096)()
    addr = C.addressof(buf)
    for rect in [(4, 4, 4, 4), (8, 4, 4, 4)]:
        j = Job(addr, addr, 16, 16, *rect)
        assert bc7lib.fastc_bc7_job_blocks(C.byref(j)) == 0
        for fmt in (1, 5):
            assert bc7lib.fastc_dxt_compress(C.byref(j), fmt) == 0
            assert bc7lib.fastc_dxt_compress_batch(C.byref(j), 1, fmt) == 0
    assert bc7lib.fastc_dxt_compress_batch(None, 0, 1) == 0
