"""CompressWithStats with a log stream (the logging encoder behind tc -l) on
the GPU, through the C ABI: at q0 the blocks and the whole log text equal
FasTC's own (fixture tests/golden/tile_stats_q0.*, made by the reference);
at q>0 the blocks and log equal the oracle's logging encoder with the same
per-fit annealing streams; sub-jobs log their blocks under the blocks'
texture-wide indices."""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN, make_image

pytestmark = pytest.mark.gpu


def _gpu_stats(img, steps=0, seed=0, metric=0, rect=None):
    from fastc_gb300 import CompressionJob, CompressionSettings, compress_with_stats

    h, w = img.shape[:2]
    out = np.zeros(w * h, dtype=np.uint8)
    job = CompressionJob(img, out, w, h, *(rect or ()))
    log = compress_with_stats(job, CompressionSettings(num_simulated_annealing_steps=steps, seed=seed,
                                                       error_metric=metric))
    return out, log


def test_q0_blocks_and_log_match_fasTC(gpu, manifest):
    case = manifest["stats"]["tile_stats_q0"]
    img = make_image(case["image"])
    h = img.shape[0]
    # FasTC's fixture job ends at the last block row (its loop has no clamp)
    blocks, log = _gpu_stats(img, 0, rect=(0, 0, img.shape[1], h - 4))
    want = np.fromfile(os.path.join(GOLDEN, "tile_stats_q0.bin"), dtype=np.uint8)
    assert np.array_equal(blocks, want)
    assert len(log) == case["log_bytes"]
    assert hashlib.sha256(log.encode()).hexdigest() == case["log_sha256"]


@pytest.mark.parametrize("expr,steps,metric", [
    ("tile_mix_radial_alpha(4, 64, 64, 800, 1200)", 16, 0),
    ("tile_mix(73, 64, 48)", 8, 0),
    ("gradient_noise_alpha_ramp(5, 48, 64)", 0, 1),
])
def test_blocks_and_log_match_oracle(gpu, port, expr, steps, metric):
    from oracle import oracle as O

    img = make_image(expr)
    blocks, log = _gpu_stats(img, steps, seed=21, metric=metric)
    want, stats = port.compress_stats(img, steps=steps, metric=metric, seed=21)
    bad = np.nonzero((blocks.reshape(-1, 16) != want.reshape(-1, 16)).any(1))[0]
    assert bad.size == 0, (bad.size, bad[:8])
    assert log == O.stats_log(stats)


def test_sub_job_logs_texture_indices(gpu, port):
    from oracle import oracle as O

    img = make_image("tile_mix(74, 64, 64)")
    # blocks from (16, 8) on, raster order, to x = 32 on row 40
    blocks, log = _gpu_stats(img, 0, rect=(16, 8, 32, 40))
    bw = 16
    first, last = 2 * bw + 4, 10 * bw + 8  # exclusive end
    # the job's single-colour blocks take watermark entries from 0 on: start
    # the whole-image oracle so that its counter is at 0 (mod 9) at `first`
    _, pre = port.compress_stats(img, steps=0)
    before = sum(1 for i, s in pre if i < first and s.path == 0)
    want, stats = port.compress_stats(img, steps=0, state=np.array([0, (9 - before % 9) % 9], np.uint32))
    assert np.array_equal(blocks[16 * first:16 * last], want[16 * first:16 * last])
    assert not blocks[:16 * first].any() and not blocks[16 * last:].any()
    assert log == O.stats_log([(i, s) for i, s in stats if first <= i < last])
