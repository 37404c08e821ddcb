"""fastc_bc7_compress_device_noalloc, through the C ABI: two calls in a row
give the bytes fastc_bc7_compress_device gives (under either engine, and on
a 1024 x 1024 texture at q50), calls after the first take nothing from the
device's memory pool, and sizes beyond the fixed array are refused before
any device work. Device buffers are made by the test; the entry point itself
takes its scratch from the library's array."""
import ctypes as C
import contextlib

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


@contextlib.contextmanager
def _engine(lib, engine):
    old = lib.fastc_bc7_get_engine()
    assert lib.fastc_bc7_set_engine(engine) == 0
    try:
        yield
    finally:
        lib.fastc_bc7_set_engine(old)


def _compare(lib, gpu, calls):
    import torch

    from fastc_gb300._lib import check

    stream = torch.cuda.current_stream().cuda_stream
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


def test_noalloc_matches_compress_device_twice_in_a_row(gpu):
    from fastc_gb300._lib import load

    lib = load()
    _compare(lib, gpu, [
        ([(64, 64), (32, 128)], 16, 5),       # two jobs, annealing
        ([(128, 96)], 0, 9),                  # one job, no annealing
    ])


def test_noalloc_matches_either_engine_and_a_large_texture(gpu):
    from fastc_gb300._lib import load

    lib = load()
    with _engine(lib, 1):  # FASTC_BC7_ENGINE_WARP_PER_BLOCK: the same engine on both sides
        _compare(lib, gpu, [([(96, 64), (16, 48)], 8, 3)])
    with _engine(lib, 0):  # FASTC_BC7_ENGINE_PIPELINE against the warp-per-block array path
        _compare(lib, gpu, [([(1024, 1024)], 50, 11), ([(256, 128)], 16, 12)])


def _cudart():
    """The CUDA runtime the library itself links (already loaded in this
    process), for the memory-pool queries."""
    from fastc_gb300._lib import load

    load()
    with open("/proc/self/maps") as f:
        paths = {ln.split()[-1] for ln in f if "libcudart.so" in ln}
    if not paths:
        pytest.skip("libcudart is not mapped in this process")
    return C.CDLL(sorted(paths)[0])


def test_noalloc_calls_take_no_device_memory(gpu):
    import torch

    from fastc_gb300._lib import check, load

    lib = load()
    rt = _cudart()
    RESERVED_CURRENT, USED_CURRENT, USED_HIGH = 5, 7, 8  # cudaMemPoolAttr values
    pool = C.c_void_p()
    assert rt.cudaDeviceGetMemPool(C.byref(pool), C.c_int(torch.cuda.current_device())) == 0

    def attr(a):
        v = C.c_uint64()
        assert rt.cudaMemPoolGetAttribute(pool, C.c_int(a), C.byref(v)) == 0
        return v.value

    stream = torch.cuda.current_stream().cuda_stream
    sizes = [(128, 64), (64, 256)]
    bufs = []
    for k, (w, h) in enumerate(sizes):
        img = make_image(f"tile_mix_radial_alpha({40 + k}, {w}, {h}, 0, 0, {w}, {h})")
        bufs.append((torch.from_numpy(img.reshape(-1)).to(gpu),
                     torch.zeros(w * h, dtype=torch.uint8, device=gpu), w, h))
    s = _settings(8, 2)

    def call(k):
        check(lib.fastc_bc7_compress_device_noalloc(_jobs([bufs[k]]), 1, C.byref(s), 0,
                                                    C.c_void_p(stream)),
              "fastc_bc7_compress_device_noalloc")

    call(0)  # first call: set-up, and every kernel of the path loaded once
    call(1)
    torch.cuda.synchronize()
    zero = C.c_uint64(0)
    assert rt.cudaMemPoolSetAttribute(pool, C.c_int(USED_HIGH), C.byref(zero)) == 0
    used0, reserved0 = attr(USED_CURRENT), attr(RESERVED_CURRENT)
    free0 = torch.cuda.mem_get_info()[0]
    call(0)
    call(1)
    torch.cuda.synchronize()
    assert attr(USED_HIGH) <= used0, "a call drew on the stream-ordered allocator"
    assert attr(RESERVED_CURRENT) == reserved0
    assert torch.cuda.mem_get_info()[0] == free0


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
