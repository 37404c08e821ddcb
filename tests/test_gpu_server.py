"""The continuous-batching request server on the GPU: results are the same
alone and in a concurrent mix, the memory budget is enforced, queued
requests can be cancelled, statistics (latency, PSNR per request and
overall) add up."""
import threading
import time

import numpy as np
import pytest

from conftest import make_image

pytestmark = pytest.mark.gpu


def settings(q, seed=11):
    from fastc_gb300 import CompressionSettings

    return CompressionSettings(num_simulated_annealing_steps=q, seed=seed)


def test_alone_equals_in_the_mix(gpu, port):
    from fastc_gb300.serve import Server

    rng = np.random.default_rng(3)
    reqs = []
    for i in range(24):
        w, h = (int(x) for x in 4 * rng.integers(2, 40, 2))
        q = int(rng.choice([0, 16, 50], p=[0.3, 0.4, 0.3]))
        reqs.append((make_image(f"tile_mix({400 + i}, {w}, {h})"), q))
    alone = []
    with Server(max_inflight=1) as srv:
        for img, q in reqs:
            alone.append(srv.wait(srv.submit(img, settings(q))).copy())
    with Server(max_inflight=3, max_batch_blocks=2048) as srv:
        # submitted from several threads while earlier batches run
        handles = [None] * len(reqs)

        def worker(k):
            for i in range(k, len(reqs), 4):
                handles[i] = srv.submit(reqs[i][0], settings(reqs[i][1]))
                time.sleep(0.001 * (i % 3))

        ts = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        mixed = [srv.wait(hd) for hd in handles]
        st = srv.stats()
        psnrs = [srv.psnr(hd) for hd in handles]
    for (img, q), a, m in zip(reqs, alone, mixed):
        assert np.array_equal(a, m)
    # and the same bytes as the oracle
    img, q = reqs[5]
    assert np.array_equal(alone[5], port.compress(img, steps=q, seed=11))
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batches"] >= 2
    assert st["p99_latency_ms"] >= st["p50_latency_ms"] > 0
    assert st["pixels_completed"] == sum(im.shape[0] * im.shape[1] for im, _ in reqs)
    # each request's quality, measured on the device, is the oracle's PSNR of
    # its blocks (FasTC's metric; the sums differ in order only), and the
    # server's overall PSNR is that of all requests' texels together
    sse = 0.0
    for (img, q), blocks, db in zip(reqs, mixed, psnrs):
        h, w = img.shape[:2]
        dec = port.decompress(blocks, w, h)
        assert abs(db - port.psnr(img, dec)) <= 1e-9
        sse += float(port.block_sse(img, dec).sum())
    px = st["pixels_completed"]
    assert abs(st["psnr_db"] - 10 * np.log10(3 * 255.0 ** 2 / (sse / px))) <= 1e-9


def test_budget_rejects_oversized_and_queues_the_rest(gpu):
    from fastc_gb300 import BC7Error
    from fastc_gb300.serve import Server

    small = make_image("tile_mix(7, 64, 64)")
    big = make_image("tile_mix(8, 1024, 1024)")
    with Server(memory_budget=96 << 20, max_inflight=2) as srv:
        with pytest.raises(BC7Error) as e:
            srv.submit(big, settings(0))
        assert e.value.status == 5
        hs = [srv.submit(small, settings(16)) for _ in range(8)]
        outs = [srv.wait(h) for h in hs]
        st = srv.stats()
    assert all(np.array_equal(outs[0], o) for o in outs)
    assert st["rejected"] == 1 and st["completed"] == 8
    assert st["peak_bytes"] <= 96 << 20


def test_cancel_queued_request(gpu):
    from fastc_gb300 import BC7Error
    from fastc_gb300.serve import Server

    imgs = [make_image(f"tile_mix({20 + i}, 256, 256)") for i in range(6)]
    with Server(max_inflight=1, max_batch_jobs=1) as srv:
        hs = [srv.submit(im, settings(50)) for im in imgs]
        cancelled = 0
        for h in hs[2:]:
            try:
                srv.cancel(h)
                cancelled += 1
            except BC7Error:
                pass
        for h in hs[:2]:
            srv.wait(h)
        for h in hs[2:]:
            try:
                srv.wait(h, timeout_ms=60000)
            except BC7Error as e:
                assert e.status == 8
        st = srv.stats()
    assert cancelled >= 1
    assert st["cancelled"] == cancelled
    assert st["completed"] + st["cancelled"] == len(imgs)


def test_wait_timeout_and_poll(gpu):
    from fastc_gb300 import BC7Error
    from fastc_gb300.serve import Server

    img = make_image("tile_mix(31, 512, 512)")
    with Server(max_inflight=1) as srv:
        h = srv.submit(img, settings(50))
        try:
            srv.wait(h, timeout_ms=0)
            finished_early = True
        except BC7Error as e:
            assert e.status == 6
            finished_early = False
        srv.wait(h)
        assert srv.poll(h)
        srv.release(h)
        with pytest.raises(BC7Error) as e:
            srv.poll(h)
        assert e.value.status == 7
    assert finished_early in (True, False)


def test_dxt_requests_share_the_server(gpu, port):
    """DXT1 / DXT5 requests (fastc_dxt_server_submit) in the same queue and
    batches as BC7 requests: each gives FasTC's DXT blocks (the oracle's,
    pinned to FasTC's) alone and in the mix, the BC7 requests among them are
    unchanged, and each request's PSNR is measured on the device."""
    from fastc_gb300 import CompressionFormat
    from fastc_gb300.serve import Server

    rng = np.random.default_rng(9)
    reqs = []
    for i in range(18):
        w, h = (int(x) for x in 4 * rng.integers(2, 30, 2))
        fmt = [CompressionFormat.BPTC, CompressionFormat.DXT1, CompressionFormat.DXT5][i % 3]
        reqs.append((make_image(f"tile_mix_radial_alpha({500 + i}, {w}, {h}, 3, 5)"), fmt))
    alone = []
    with Server(max_inflight=1) as srv:
        for img, fmt in reqs:
            alone.append(srv.wait(srv.submit(img, settings(8), format=fmt)).copy())
    with Server(max_inflight=3, max_batch_blocks=1024) as srv:
        handles = [srv.submit(img, settings(8), format=fmt) for img, fmt in reqs]
        mixed = [srv.wait(hd) for hd in handles]
        psnrs = [srv.psnr(hd) for hd in handles]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["batches"] >= 2
    for (img, fmt), a, m, db in zip(reqs, alone, mixed, psnrs):
        assert np.array_equal(a, m)
        h, w = img.shape[:2]
        if fmt == CompressionFormat.BPTC:
            assert np.array_equal(m, port.compress(img, steps=8, seed=11))
            dec = port.decompress(m, w, h)
        else:
            alpha = fmt == CompressionFormat.DXT5
            assert len(m) == w * h // (1 if alpha else 2)
            assert np.array_equal(m, port.dxt_compress(img, alpha))
            dec = port.dxt_decompress(m, w, h, alpha)
        assert abs(db - port.psnr(img, dec)) <= 1e-9


def test_dxt_submit_rejects_other_formats(gpu):
    import ctypes as C

    from fastc_gb300 import _lib
    from fastc_gb300.serve import Server

    img = make_image("tile_mix(5, 16, 16)")
    out = np.zeros(16 * 16, np.uint8)
    job = _lib.Job(img.ctypes.data, out.ctypes.data, 16, 16, 0, 0, 16, 16)
    rid = C.c_uint64()
    with Server() as srv:
        for fmt in (0, 3, 7):
            assert srv._lib.fastc_dxt_server_submit(srv._h, C.byref(job), fmt, C.byref(rid)) == \
                _lib.ERR_INVALID_ARGUMENT
        assert srv.stats()["submitted"] == 0


@pytest.mark.parametrize("fmt_name", ["BPTC", "DXT1", "DXT5"])
def test_sub_job_requests(gpu, port, fmt_name):
    """A request for a sub-job (FasTC's job rectangle: raster blocks from
    (x_start, y_start) to x_end on row y_end) writes exactly those blocks,
    equal to the whole image's, and its PSNR covers exactly those texels."""
    from fastc_gb300 import CompressionFormat
    from fastc_gb300.serve import Server

    fmt = CompressionFormat[fmt_name]
    img = make_image("tile_mix_radial_alpha(77, 48, 40, 9, 2)")
    bsz = 8 if fmt == CompressionFormat.DXT1 else 16
    if fmt == CompressionFormat.BPTC:
        whole = port.compress(img, steps=8, seed=11)
        dec = port.decompress(whole, 48, 40)
    else:
        whole = port.dxt_compress(img, fmt == CompressionFormat.DXT5)
        dec = port.dxt_decompress(whole, 48, 40, fmt == CompressionFormat.DXT5)
    sse = port.block_sse(img, dec).reshape(-1)
    rect = (8, 12, 20, 28)  # blocks 3 * 12 + 2 .. 7 * 12 + 5 (exclusive)
    first, end = 3 * 12 + 2, 7 * 12 + 5
    with Server(max_inflight=2) as srv:
        out = np.zeros(48 * 40 * bsz // 16, np.uint8)
        req = srv.submit(img, settings(8), out=out, format=fmt, rect=rect)
        srv.wait(req)
        db = srv.psnr(req)
    assert np.array_equal(out[first * bsz:end * bsz], whole[first * bsz:end * bsz])
    assert not out[:first * bsz].any() and not out[end * bsz:].any()
    want = 10 * np.log10(3 * 255.0 ** 2 / (float(sse[first:end].sum()) / ((end - first) * 16)))
    assert abs(db - want) <= 1e-9
