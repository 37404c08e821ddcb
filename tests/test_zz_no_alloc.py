"""fastc_bc7_compress_device_noalloc, through the C ABI: two calls in a row
give the bytes fastc_bc7_compress_device gives, and sizes beyond the fixed
array are refused before any device work. Device buffers are made by the
test; the entry point itself takes its scratch from the library's array."""
import ctypes as C

import numpy as np
import pytest

from conftest import make_image

pytestmark = pytest.mark.gpu


def _jobs(pairs):
    from fastc_gb300._lib import Job

    arr = (Job * len(pairs))()
    for k, (din, dout, w, h) in enumerate(pairs):
        arr[k] = Job(din.data_ptr(), dout.data_ptr(), w, h, 0, 0, w, h)
    return arr


def _settings(q, seed):
    from fastc_gb300 import CompressionSettings

    return CompressionSettings(num_simulated_annealing_steps=q, seed=seed).to_c()


def test_noalloc_matches_compress_device_twice_in_a_row(gpu):
    import torch

    from fastc_gb300._lib import check, load

    lib = load()
    stream = torch.cuda.current_stream().cuda_stream
    calls = [
        ([(64, 64), (32, 128)], 16, 5),       # two jobs, annealing
        ([(128, 96)], 0, 9),                  # one job, no annealing
    ]
    for sizes, q, seed in calls:
        imgs = [make_image(f"tile_mix_radial_alpha({seed * 10 + i}, {w}, {h}, 0, 0, {w}, {h})")
                for i, (w, h) in enumerate(sizes)]
        din = [torch.from_numpy(im.reshape(-1)).to(gpu) for im in imgs]
        want = [torch.zeros(w * h, dtype=torch.uint8, device=gpu) for w, h in sizes]
        got = [torch.full((w * h,), 0xA5, dtype=torch.uint8, device=gpu) for w, h in sizes]
        s = _settings(q, seed)
        check(lib.fastc_bc7_compress_device(
            _jobs([(a, b, w, h) for a, b, (w, h) in zip(din, want, sizes)]), len(sizes),
            C.byref(s), 0, C.c_void_p(stream)), "fastc_bc7_compress_device")
        check(lib.fastc_bc7_compress_device_noalloc(
            _jobs([(a, b, w, h) for a, b, (w, h) in zip(din, got, sizes)]), len(sizes),
            C.byref(s), 0, C.c_void_p(stream)), "fastc_bc7_compress_device_noalloc")
        torch.cuda.synchronize()
        for a, b in zip(want, got):
            assert np.array_equal(a.cpu().numpy(), b.cpu().numpy())


def test_noalloc_refuses_sizes_beyond_its_array(gpu):
    import torch

    from fastc_gb300._lib import load

    lib = load()
    limit = 1 << 20  # FASTC_BC7_NOALLOC_MAX_BLOCKS
    # 4100 x 1024 texels = 262,400 blocks per job; four of them exceed the limit.
    w, h = 4100, 1024
    assert 4 * (w // 4) * (h // 4) > limit
    buf = torch.zeros(16, dtype=torch.uint8, device=gpu)  # never touched: refused first
    s = _settings(0, 1)
    jobs = _jobs([(buf, buf, w, h)] * 4)
    st = lib.fastc_bc7_compress_device_noalloc(jobs, 4, C.byref(s), 0, None)
    assert st == 1
    assert b"exceed the fixed scratch" in lib.fastc_bc7_last_error()
    many = _jobs([(buf, buf, 4, 4)] * 257)
    assert lib.fastc_bc7_compress_device_noalloc(many, 257, C.byref(s), 0, None) == 1
    assert b"job table" in lib.fastc_bc7_last_error()
