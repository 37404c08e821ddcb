"""The oracle (C restatement of FasTC's encoder) against the reference's own
golden outputs, plus the generators the fixtures are made from. CPU only."""
import hashlib
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_blocks, make_image
from oracle import oracle as O


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_generators_reproduce_fixture_inputs(manifest):
    for name, case in manifest["cases"].items():
        assert sha(make_image(case["image"])) == case["input_sha256"], name
    for name, case in manifest["quality"].items():
        assert sha(make_image(case["image"])) == case["input_sha256"], name


@pytest.mark.parametrize("name", ["c1_q0", "tile_q0", "radial_q0", "c1_q0_nonuniform"])
def test_q0_blocks_bit_exact(port, manifest, name):
    case = manifest["cases"][name]
    img = make_image(case["image"])
    got = port.compress(img, steps=0, metric=case["metric"])
    want = golden_blocks(name)
    bad = np.nonzero((got.reshape(-1, 16) != want.reshape(-1, 16)).any(1))[0]
    assert bad.size == 0, f"{bad.size} blocks differ, first {bad[:8]}"


@pytest.mark.parametrize("name", ["c1_q8_seed", "tile_q50_seed", "radial_q16_seed"])
def test_annealing_single_stream_bit_exact(port, manifest, name):
    """With one LCG stream threaded through the fits in FasTC's order and
    double exp, the oracle reproduces the reference's q>0 blocks exactly."""
    case = manifest["cases"][name]
    img = make_image(case["image"])
    state = np.array([case["lcg_seed"], 0], dtype=np.uint32)
    got = port.compress(img, steps=case["steps"], metric=case["metric"], rng_mode=O.RNG_SINGLE_STREAM,
                        exp_mode=O.EXP_LIBM, state=state)
    assert np.array_equal(got, golden_blocks(name))


def test_endpoint_tables(port):
    g = np.load(os.path.join(GOLDEN, "endpoint_tables.npz"))
    o7, o6 = port.tables()
    assert np.array_equal(o7, g["opt7"])
    assert np.array_equal(o6, g["opt6"])


def test_box_selection(port, manifest):
    from fastc_gb300 import synth

    want = np.load(os.path.join(GOLDEN, "box_selection.npy"))
    img = make_image(manifest["box_selection"]["image"])
    got = np.array([port.box_selection(px) for px in synth.blocks_of(img)], dtype=np.uint32)
    assert np.array_equal(got, want)


def test_decoder_matches_reference_decoder(port, manifest):
    for name, case in manifest["cases"].items():
        img = make_image(case["image"])
        dec = port.decompress(golden_blocks(name), img.shape[1], img.shape[0])
        assert sha(dec) == case["decoded_sha256"], name


def test_partition_tables_consistent(port):
    for shape in range(64):
        for nsub in (2, 3):
            p = port.partition(shape, nsub)
            assert p[0] == 0 and set(p.tolist()) == set(range(nsub))
            for s in range(1, nsub):
                a = port.lib.bc7o_anchor(s, shape, nsub)
                assert p[a] == s
    assert port.lib.bc7o_anchor(0, 5, 2) == 0


def test_portable_exp(port):
    assert port.lib.bc7o_expf(0.0) == 1.0
    assert port.lib.bc7o_expf(-200.0) == 0.0
    for x in np.linspace(-100, 0, 2001):
        got = port.lib.bc7o_expf(float(x))
        want = math.exp(float(np.float32(x)))
        assert abs(got - want) <= 4e-7 * want + 1e-44, x
    assert math.isnan(port.lib.bc7o_expf(float("nan")))


def test_fit_seed_is_a_pure_function(port):
    a = [port.lib.bc7o_fit_seed(7, x, y, f) for x in range(4) for y in range(4) for f in (0, 0x180, 0x611)]
    b = [port.lib.bc7o_fit_seed(7, x, y, f) for x in range(4) for y in range(4) for f in (0, 0x180, 0x611)]
    assert a == b and len(set(a)) == len(a)


def test_multithreaded_equals_serial(port):
    img = make_image("tile_mix_radial_alpha(9, 64, 64, 500, 500)")
    serial = port.compress(img, steps=12, seed=99)
    for t in (1, 3, 8):
        assert np.array_equal(port.compress_mt(img, steps=12, seed=99, threads=t), serial)


def test_psnr_formula(port):
    a = np.zeros((4, 4, 4), np.uint8)
    b = a.copy()
    a[..., 3] = 255
    b[..., 3] = 255
    b[..., 0] = 255
    # one channel fully off on every pixel: mse = 255^2 -> 10 log10(3)
    assert abs(port.psnr(a, b) - 10 * math.log10(3.0)) < 1e-12


@pytest.mark.skipif(not os.path.isdir(os.path.join(O.DEFAULT_REFERENCE, "BPTCEncoder")),
                    reason="FasTC checkout not present")
def test_against_live_reference(port):
    """Fresh content straight against the reference library (x86 container)."""
    O.build_ref()
    ref = O.Reference()
    img = make_image("tile_mix_radial_alpha(77, 96, 96, 123 * 4, 456 * 4)")
    assert np.array_equal(port.compress(img, steps=0), ref.compress(img, steps=0))
    st = np.array([4242, 0], np.uint32)
    got = port.compress(img, steps=20, rng_mode=O.RNG_SINGLE_STREAM, exp_mode=O.EXP_LIBM, state=st)
    assert np.array_equal(got, ref.compress(img, steps=20, seed=4242))


def test_exact_projection_rounds_to_the_integer_index():
    """FasTC picks the palette indices around fl(fl(D / L) * k) (RGBAEndpoints.cpp:
    190-310). When D * k is a multiple of L, D / L equals j / k exactly, and the
    two float roundings give back j for every j < k, k in {3, 7, 15}: the GPU's
    integer quotient (j1 = j2 = j there) therefore needs no float path."""
    for k in (3, 7, 15):
        for j in range(1, k):
            sc = (np.float32(j) / np.float32(k)) * np.float32(k)
            assert sc.dtype == np.float32 and float(sc) == j, (k, j, sc)


def test_float_thresholds_equal_the_double_comparisons():
    """The PCA's tests against 1e-7, 1e-8 and 1e-10, which FasTC makes on
    floats widened to double, are made in single precision on the GPU with
    the float literals: 1e-7f and 1e-10f are the least floats above their
    doubles (x > 1e-7 iff x >= 1e-7f; x < 1e-10 iff x < 1e-10f), 1e-8f the
    greatest float below 1e-8 (x < 1e-8 iff x <= 1e-8f)."""
    def neighbours(c):
        f = np.float32(c)
        return float(np.nextafter(f, np.float32(0))), float(f), float(np.nextafter(f, np.float32(1)))

    for c in (1e-7, 1e-10):
        below, f, _ = neighbours(c)
        assert below < c < f
    below, f, above = neighbours(1e-8)
    assert f < 1e-8 < above
    # the comparisons themselves on the floats around each threshold
    for x in neighbours(1e-7):
        assert (x > 1e-7) == (np.float32(x) >= np.float32(1e-7))
    for x in neighbours(1e-10):
        assert (x < 1e-10) == (np.float32(x) < np.float32(1e-10))
    for x in neighbours(1e-8):
        assert (x < 1e-8) == (np.float32(x) <= np.float32(1e-8))


def test_quantized_error_call_count_matches_reference_profile(port):
    """The port runs FasTC's search: on the 256x256 gradient + noise + alpha
    ramp image at q0, QuantizedError is called about 320 times per block,
    the count a gprof profile of FasTC's own encoder gave on this content.
    The bench's work roofline counts texel-bucket evaluations the same way."""
    from conftest import make_image

    img = make_image("gradient_noise_alpha_ramp(1, 256, 256)")
    port.qe_counters(reset=True)
    port.compress(img, steps=0)
    calls, evals = port.qe_counters(reset=True)
    assert abs(calls / 4096 - 320) < 3, calls / 4096
    assert 10 * calls < evals < 16 * calls  # one to several palette entries per texel
