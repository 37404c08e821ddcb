"""GPU parity: the sm_103a encoder through the C ABI against FasTC's golden
outputs and against the oracle. Integer/byte results are compared bit for
bit; the only tolerance is the q>0 PSNR bar against the reference (0.05 dB)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_blocks, make_image

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[0, 1], ids=["pipeline", "warp_per_block"], autouse=True)
def engine(request, gpu):
    """Every parity test runs on both encoder organisations."""
    from fastc_gb300 import set_engine

    set_engine(request.param)
    yield request.param
    set_engine(0)


def gpu_compress(img, steps=0, metric=0, modes=0xFF, seed=0, wm=0):
    from fastc_gb300 import CompressionSettings, compress_image_data

    s = CompressionSettings(num_simulated_annealing_steps=steps, error_metric=metric, block_modes=modes,
                            seed=seed, watermark_start=wm)
    return compress_image_data(img, img.shape[1], img.shape[0], s)


def first_diff(a, b):
    bad = np.nonzero((a.reshape(-1, 16) != b.reshape(-1, 16)).any(1))[0]
    return bad.size, bad[:8]


@pytest.mark.parametrize("name", ["c1_q0", "tile_q0", "radial_q0", "c1_q0_nonuniform"])
def test_q0_matches_reference_golden(gpu, manifest, name):
    case = manifest["cases"][name]
    got = gpu_compress(make_image(case["image"]), 0, case["metric"])
    n, first = first_diff(got, golden_blocks(name))
    assert n == 0, f"{n} blocks differ from FasTC, first {first}"


@pytest.mark.parametrize("expr", [
    "tile_mix(31, 256, 256)",
    "tile_mix_radial_alpha(32, 256, 256, 5000, 700)",
    "gradient_noise_alpha_ramp(33, 192, 160)",
])
def test_q0_matches_oracle(gpu, port, expr):
    img = make_image(expr)
    n, first = first_diff(gpu_compress(img, 0), port.compress(img, steps=0))
    assert n == 0, f"{n} blocks differ, first {first}"


@pytest.mark.parametrize("expr,steps,metric", [
    ("tile_mix(41, 128, 128)", 50, 0),
    ("tile_mix_radial_alpha(42, 96, 96, 2000, 3000)", 16, 0),
    ("gradient_noise_alpha_ramp(43, 96, 96)", 8, 1),
    ("tile_mix(44, 64, 64)", 1, 0),
    ("tile_mix(45, 32, 32)", 256, 0),
])
def test_annealing_matches_oracle_bit_exact(gpu, port, expr, steps, metric):
    """Same per-fit streams, same float exp: the GPU and the oracle agree on
    every block at q>0."""
    img = make_image(expr)
    got = gpu_compress(img, steps, metric, seed=1234)
    want = port.compress(img, steps=steps, metric=metric, seed=1234)
    n, first = first_diff(got, want)
    assert n == 0, f"{n} blocks differ, first {first}"


@pytest.mark.parametrize("name", ["tile_q50_psnr", "radial_q50_psnr"])
def test_q50_psnr_within_0p05db_of_reference(gpu, port, manifest, name):
    case = manifest["quality"][name]
    img = make_image(case["image"])
    got = gpu_compress(img, case["steps"], seed=7)
    dec = port.decompress(got, img.shape[1], img.shape[0])
    psnr = port.psnr(img, dec)
    ref = float(np.mean(case["psnr"]))
    assert abs(psnr - ref) <= 0.05, (psnr, case["psnr"])


@pytest.mark.parametrize("name", ["tile_q50_psnr", "radial_q50_psnr"])
def test_q50_per_block_error_within_reference_seed_spread(gpu, port, manifest, name):
    """Per-block SSE (FasTC's premultiplied metric) against FasTC's own
    blocks at three pinned seeds. Annealing draws differ per seed, so FasTC
    against itself has about 7 % of blocks more than 1 % worse (16 SSE
    floor); ours must stay within that spread, and the total within 0.5 %."""
    case = manifest["quality"][name]
    img = make_image(case["image"])
    got = gpu_compress(img, case["steps"], seed=7)
    sse = port.block_sse(img, port.decompress(got, img.shape[1], img.shape[0])).astype(np.float64)
    ref = np.load(os.path.join(GOLDEN, name + "_sse.npy")).astype(np.float64)
    spread = max(np.mean((ref[i] + 16) / (ref[j] + 16) > 1.01) for i in range(3) for j in range(3) if i != j)
    for r in ref:
        assert np.mean((sse + 16) / (r + 16) > 1.01) <= spread + 0.01
        assert abs(sse.sum() / r.sum() - 1.0) <= 0.005


@pytest.mark.parametrize("mask", [0x41, 0xF0, 0x02, 0x80, 0x0C])
def test_mode_masks_match_oracle(gpu, port, mask):
    img = make_image("tile_mix(51, 64, 64)")
    n, first = first_diff(gpu_compress(img, 4, modes=mask, seed=3), port.compress(img, steps=4, modes=mask, seed=3))
    assert n == 0, f"{n} blocks differ, first {first}"


def test_single_colour_and_transparent_blocks(gpu, port):
    img = np.zeros((32, 64, 4), np.uint8)
    rng = np.random.default_rng(5)
    for by in range(8):
        for bx in range(16):
            kind = (bx + by) % 3
            blk = img[by * 4:by * 4 + 4, bx * 4:bx * 4 + 4]
            if kind == 0:
                blk[:] = rng.integers(0, 256, 4, dtype=np.uint8)  # one colour
            elif kind == 1:
                blk[..., :3] = rng.integers(0, 256, (4, 4, 3), dtype=np.uint8)
                blk[..., 3] = 0  # transparent, not one colour
            else:
                blk[:] = rng.integers(0, 256, (4, 4, 4), dtype=np.uint8)
    for wm in (0, 4, 17):
        n, first = first_diff(gpu_compress(img, 0, wm=wm), port.compress(img, steps=0, state=np.array([0, wm], np.uint32)))
        assert n == 0, (wm, n, first)


def test_batched_equals_alone(gpu):
    """A texture compressed inside a batch gives the same bytes as alone."""
    from fastc_gb300 import CompressionJob, CompressionSettings, compress_jobs

    imgs = [make_image(f"tile_mix({60 + i}, {w}, {h})") for i, (w, h) in
            enumerate([(16, 16), (64, 32), (8, 128), (96, 96), (4, 4)])]
    s = CompressionSettings(num_simulated_annealing_steps=16, seed=9)
    alone = [gpu_compress(im, 16, seed=9) for im in imgs]
    outs = [np.zeros(im.shape[0] * im.shape[1], np.uint8) for im in imgs]
    compress_jobs([CompressionJob(im, o, im.shape[1], im.shape[0]) for im, o in zip(imgs, outs)], s)
    for a, b in zip(alone, outs):
        assert np.array_equal(a, b)


def test_device_api_and_plan_match_host_api(gpu):
    import torch

    from fastc_gb300 import CompressionJob, CompressionSettings, Plan, compress_jobs

    imgs = [make_image(f"tile_mix_radial_alpha({70 + i}, {w}, {h}, 0, 0, {w}, {h})")
            for i, (w, h) in enumerate([(32, 32), (128, 64), (16, 256)])]
    s = CompressionSettings(num_simulated_annealing_steps=8, seed=21)
    host = [gpu_compress(im, 8, seed=21) for im in imgs]
    din = [torch.from_numpy(im).cuda() for im in imgs]
    dout = [torch.zeros(im.shape[0] * im.shape[1], dtype=torch.uint8, device="cuda") for im in imgs]
    jobs = [CompressionJob(a, b, im.shape[1], im.shape[0]) for a, b, im in zip(din, dout, imgs)]
    compress_jobs(jobs, s)
    torch.cuda.synchronize()
    for h, d in zip(host, dout):
        assert np.array_equal(h, d.cpu().numpy())
    for d in dout:
        d.zero_()
    plan = Plan(jobs, s)
    for _ in range(2):
        plan.launch()
    torch.cuda.synchronize()
    assert plan.flags() == 0
    for h, d in zip(host, dout):
        assert np.array_equal(h, d.cpu().numpy())
    plan.close()


def test_plan_autotune_keeps_the_bytes(gpu):
    """The autotuner swaps launch parameters, never results."""
    import torch

    from fastc_gb300 import CompressionJob, CompressionSettings, Plan, compress_jobs

    imgs = [make_image(f"tile_mix({90 + i}, {w}, {h})") for i, (w, h) in enumerate([(256, 128), (64, 64), (128, 512)])]
    s = CompressionSettings(num_simulated_annealing_steps=16, seed=5)
    din = [torch.from_numpy(im).cuda() for im in imgs]
    dout = [torch.zeros(im.shape[0] * im.shape[1], dtype=torch.uint8, device="cuda") for im in imgs]
    jobs = [CompressionJob(a, b, im.shape[1], im.shape[0]) for a, b, im in zip(din, dout, imgs)]
    compress_jobs(jobs, s)
    torch.cuda.synchronize()
    want = [d.cpu().numpy().copy() for d in dout]
    for d in dout:
        d.zero_()
    plan = Plan(jobs, s)
    t = plan.autotune(launches=1)
    assert t["engine"] in (0, 1)
    if t["engine"] == 0:  # the pipeline's parameters, from the candidate lists
        assert t["anneal_ctas_per_sm"] in (3, 4, 5, 6, 7) and t["yield_lanes"] in (8, 12, 16)
        assert t["select_ctas_per_sm"] in (8, 16, 32) and t["setup_ctas_per_sm"] in (6, 12, 24, 128)
        assert t["chunk_blocks"] > 0 and t["chunk_blocks"] % 1024 == 0
    else:  # 6,400 blocks: a small set, where the warp-per-block engine is a candidate
        assert t["warps_per_cta"] in (2, 4, 8)
    for d in dout:
        d.zero_()
    plan.launch()
    torch.cuda.synchronize()
    for w, d in zip(want, dout):
        assert np.array_equal(w, d.cpu().numpy())
    plan.close()


def test_sub_jobs_tile_the_image(gpu, port):
    """FasTC's ThreadGroup splits (Core/src/ThreadGroup.cpp:133-192), run one
    after another with the watermark counter continuing across calls like
    FasTC's global gWMVal, give the same bytes as one whole-image job."""
    from fastc_gb300 import WATERMARK_CONTINUE, CompressionJob, CompressionSettings, compress
    from fastc_gb300._lib import load

    lib = load()
    img = make_image("tile_mix(80, 64, 48)")
    w, h = 64, 48
    s = CompressionSettings(num_simulated_annealing_steps=4, seed=2, watermark_start=WATERMARK_CONTINUE)
    lib.fastc_bc7_set_watermark_counter(0)
    whole = np.zeros(w * h, np.uint8)
    compress(CompressionJob(img, whole, w, h), s)
    nsingle = sum(int((b == b[0]).all()) for b in __import__("fastc_gb300").synth.blocks_of(img))
    assert lib.fastc_bc7_get_watermark_counter() == nsingle % 9
    assert np.array_equal(whole, port.compress(img, steps=4, seed=2))
    lib.fastc_bc7_set_watermark_counter(0)
    out = np.zeros_like(whole)
    nblocks = (w // 4) * (h // 4)
    per = nblocks // 5 + 1
    done = 0
    while done < nblocks:
        e = min(done + per, nblocks)
        compress(CompressionJob(img, out, w, h, (done % 16) * 4, (done // 16) * 4, (e % 16) * 4, (e // 16) * 4), s)
        done = e
    assert np.array_equal(out, whole)


def test_unaligned_device_buffers(gpu):
    import torch

    from fastc_gb300 import CompressionJob, CompressionSettings, compress

    img = make_image("tile_mix(90, 32, 32)")
    want = gpu_compress(img, 0)
    raw_in = torch.zeros(img.size + 4, dtype=torch.uint8, device="cuda")
    raw_out = torch.zeros(want.size + 4, dtype=torch.uint8, device="cuda")
    din, dout = raw_in[4:], raw_out[4:]
    din.copy_(torch.from_numpy(img.reshape(-1)))
    compress(CompressionJob(din, dout, 32, 32), CompressionSettings(num_simulated_annealing_steps=0))
    torch.cuda.synchronize()
    assert np.array_equal(dout.cpu().numpy(), want)


@pytest.mark.parametrize("name", ["c1_q0", "radial_q0", "radial_q16_seed"])
def test_gpu_decoder_matches_fastc_decoder(gpu, port, manifest, name):
    from fastc_gb300 import decompress

    case = manifest["cases"][name]
    img = make_image(case["image"])
    blocks = golden_blocks(name)
    got = decompress(blocks, img.shape[1], img.shape[0])
    assert np.array_equal(got, port.decompress(blocks, img.shape[1], img.shape[0]))


def test_gpu_decoder_spec_mode_differs_only_on_mode4_index_mode1(gpu, port):
    from fastc_gb300 import decompress

    img = make_image("tile_mix_radial_alpha(95, 128, 128, 0, 0, 128, 128)")
    blocks = gpu_compress(img, 0)
    ref = decompress(blocks, 128, 128)
    spec = decompress(blocks, 128, 128, spec_semantics=True)
    b = blocks.reshape(-1, 16)
    mode4_im1 = (b[:, 0] & 0x1F) == 0x10
    mode4_im1 &= ((b[:, 0] >> 7) & 1) == 1
    diff = (ref != spec).reshape(32, 4, 32, 4, 4).any(axis=(1, 3, 4)).reshape(-1)
    assert not np.any(diff & ~mode4_im1)


def test_threads_encode_disjoint_sub_jobs(gpu, port):
    """FasTC's `tc -t N` path: N host threads call Compress at once, each on
    its own band of one image (disjoint sub-jobs into one output buffer).
    The image has no single-colour block, so FasTC's shared watermark
    counter plays no part; the blocks equal the whole image's."""
    import threading

    from fastc_gb300 import CompressionJob, CompressionSettings, compress, synth

    img = np.ascontiguousarray(make_image("gradient_noise_alpha_ramp(4, 96, 64)"))
    assert not any((b == b[0]).all() for b in synth.blocks_of(img))
    out = np.zeros(96 * 64, np.uint8)
    s = CompressionSettings(num_simulated_annealing_steps=8, seed=11)
    bands = [(0, y, 96, y + 12) for y in range(0, 64, 16)]
    errors = []

    def work(rect):
        try:
            for _ in range(3):
                compress(CompressionJob(img, out, 96, 64, *rect), s)
        except Exception as e:  # reported below
            errors.append(e)

    ts = [threading.Thread(target=work, args=(r,)) for r in bands]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors
    assert np.array_equal(out, port.compress(img, steps=8, seed=11))
