"""CompressWithStats (the logging encoder behind tc -l) in the oracle, pinned
against FasTC: the blocks, the whole log text (by hash) and the parsed
per-block statistics of golden fixtures made by the reference itself
(tests/golden/make_golden.py), at q0 and at q16 with a pinned LCG seed.
Its shape selection differs from BPTCC::Compress, so its blocks differ too;
the statistics carry FasTC's quirks (per-mode errors stay -1)."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, make_image

import oracle.oracle as O


def _manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)["stats"]


def _run(port, case):
    img = make_image(case["image"])
    if case["lcg_seed"] is None:
        return img, port.compress_stats(img, steps=case["steps"])
    st = np.array([case["lcg_seed"], 0], np.uint32)
    return img, port.compress_stats(img, steps=case["steps"], rng_mode=O.RNG_SINGLE_STREAM,
                                    exp_mode=O.EXP_LIBM, state=st)


@pytest.mark.parametrize("name", ["tile_stats_q0", "radial_stats_q16_seed"])
def test_stats_blocks_and_log_match_fastc(port, name):
    case = _manifest()[name]
    img, (blocks, stats) = _run(port, case)
    assert hashlib.sha256(img.tobytes()).hexdigest() == case["input_sha256"]
    want = np.fromfile(os.path.join(GOLDEN, name + ".bin"), dtype=np.uint8)
    assert np.array_equal(blocks, want)
    log = O.stats_log(stats)
    assert len(log) == case["log_bytes"]
    assert hashlib.sha256(log.encode()).hexdigest() == case["log_sha256"]
    ref = np.load(os.path.join(GOLDEN, name + ".npz"))
    assert np.array_equal(ref["path"], [s.path for _, s in stats])
    assert np.array_equal(ref["mode"], [s.mode for _, s in stats])
    got_est = np.array([[float("%g" % v) for v in s.estimate] for _, s in stats])
    assert np.array_equal(ref["estimate"], got_est)
    assert (ref["error"] == -1).all()  # CompressClusters keeps min(error, -1)
    two = [float("%g" % s.two_shape[k]) for _, s in stats for k in range(s.n_two)]
    assert np.array_equal(ref["two"], two)


def test_stats_selection_differs_from_compress(port):
    """Modes 4 and 5 stay on for opaque blocks and the bounding boxes are
    quantised: the logging encoder picks other blocks than Compress."""
    case = _manifest()["tile_stats_q0"]
    img = make_image(case["image"])
    plain = port.compress(img, steps=0).reshape(-1, 16)
    logged = np.fromfile(os.path.join(GOLDEN, "tile_stats_q0.bin"), dtype=np.uint8).reshape(-1, 16)
    assert (plain != logged).any(1).sum() > 0


def test_stats_against_live_reference(port):
    """Fresh content straight against the reference library (x86 container)."""
    if not O.build_ref():
        pytest.skip("FasTC checkout not available")
    ref = O.Reference()
    img = make_image("tile_mix(91, 48, 48, 64, 32)")
    st = np.array([777, 0], np.uint32)
    blocks, stats = port.compress_stats(img, steps=12, rng_mode=O.RNG_SINGLE_STREAM,
                                        exp_mode=O.EXP_LIBM, state=st)
    want, log = ref.compress_stats(img, steps=12, seed=777)
    assert np.array_equal(blocks, want)
    assert O.stats_log(stats) == log
    assert int(st[0]) == int(ref.lib.ref_get_seed())
