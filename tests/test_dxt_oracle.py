"""The DXT1 / DXT5 oracle (oracle/dxt_oracle.c, a restatement of the
stb_dxt encoder that FasTC's DXTEncoder/src/Compressor.cpp:47-93 runs, and
of DXTEncoder/src/Decompressor.cpp:26-155) against FasTC's own output: the
blocks and decoded texels of tests/golden/dxt*.bin, made by the reference
(tests/golden/make_golden.py). Bit-exact."""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_blocks, make_image


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def random_blocks(w, h, fmt, seed):
    n = ((w + 3) // 4) * ((h + 3) // 4) * (8 if fmt == 1 else 16)
    return np.random.default_rng(seed).integers(0, 256, n, dtype=np.uint8)


ENCODE = ["dxt1_tile", "dxt5_tile", "dxt1_gradient", "dxt5_radial", "dxt1_flat", "dxt5_flat"]


@pytest.mark.parametrize("name", ENCODE)
def test_port_blocks_equal_fasTC(port, manifest, name):
    case = manifest["dxt"][name]
    img = make_image(case["image"])
    assert sha(img) == case["input_sha256"]
    want = golden_blocks(name)
    assert sha(want) == case["blocks_sha256"]
    got = port.dxt_compress(img, case["format"] == 5)
    bsz = 8 if case["format"] == 1 else 16
    bad = np.nonzero((got.reshape(-1, bsz) != want.reshape(-1, bsz)).any(1))[0]
    assert bad.size == 0, (bad.size, bad[:8])


@pytest.mark.parametrize("name", ENCODE)
def test_port_decoder_equals_fasTC(port, manifest, name):
    case = manifest["dxt"][name]
    img = make_image(case["image"])
    dec = port.dxt_decompress(golden_blocks(name), img.shape[1], img.shape[0], case["format"] == 5)
    assert sha(dec) == case["decoded_sha256"]


@pytest.mark.parametrize("name", ["dxt1_random_decode", "dxt5_random_decode"])
def test_port_decoder_on_random_blocks(port, manifest, name):
    case = manifest["dxt"][name]
    blocks = random_blocks(case["width"], case["height"], case["format"], case["rng_seed"])
    assert sha(blocks) == case["blocks_sha256"]
    dec = port.dxt_decompress(blocks, case["width"], case["height"], case["format"] == 5)
    assert sha(dec) == case["decoded_sha256"]


def test_single_colour_tables_reproduce_values(port):
    """The single-colour tables hold, per value, the endpoint pair whose 1/3
    interpolant lands nearest (the 3 % endpoint-distance penalty aside)."""
    m5, m6 = port.dxt_tables()
    for tab, bits in ((m5.reshape(256, 2), 5), (m6.reshape(256, 2), 6)):
        exp = lambda q: (q << (8 - bits)) | (q >> (2 * bits - 8))
        hi, lo = exp(tab[:, 0].astype(int)), exp(tab[:, 1].astype(int))
        err = np.abs((2 * hi + lo) // 3 - np.arange(256))
        assert err.max() <= (2 if bits == 5 else 1)


def test_dxt1_is_colour_of_dxt5(port):
    """DXT5's second half is DXT1's colour block with the alpha ignored."""
    img = make_image("tile_mix_radial_alpha(7, 64, 32, 500, 700)")
    d1 = port.dxt_compress(img, False).reshape(-1, 8)
    d5 = port.dxt_compress(img, True).reshape(-1, 16)
    assert np.array_equal(d5[:, 8:], d1)


def test_alpha_block_endpoints_and_exact_ends(port):
    img = make_image("tile_mix_radial_alpha(9, 32, 32, 100, 100)")
    d5 = port.dxt_compress(img, True).reshape(-1, 16)
    dec = port.dxt_decompress(d5, 32, 32, True)
    blocks = img.reshape(8, 4, 8, 4, 4).transpose(0, 2, 1, 3, 4).reshape(-1, 16, 4)
    dblk = dec.reshape(8, 4, 8, 4, 4).transpose(0, 2, 1, 3, 4).reshape(-1, 16, 4)
    a = blocks[..., 3].astype(int)
    assert np.array_equal(d5[:, 0], a.max(1)) and np.array_equal(d5[:, 1], a.min(1))
    # 8 levels between min and max: each texel within half a step (+1 rounding)
    step = (a.max(1) - a.min(1)) / 7.0
    assert (np.abs(dblk[..., 3].astype(int) - a) <= step[:, None] / 2 + 1).all()
