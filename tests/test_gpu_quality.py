"""On-device image quality (fastc_bc7_psnr, fastc_bc7_block_error_device)
against the oracle's restatement of FasTC's Image::ComputePSNR
(Base/src/Image.cpp:206-255). Per-block SSE is summed in the same order on
both sides, so it is compared bit for bit; the image PSNR sums the blocks in
a different order than FasTC's single pass and is compared within 1e-9 dB."""
import numpy as np
import pytest

from conftest import golden_blocks, make_image

pytestmark = pytest.mark.gpu

CASES = [
    ("c1_q0", "gradient_noise_alpha_ramp(1, 256, 256)"),
    ("radial_q0", "tile_mix_radial_alpha(5, 128, 128, 1000, 2000)"),
    ("radial_q16_seed", "tile_mix_radial_alpha(5, 64, 64, 3000, 3000)"),
    ("tile_q50_seed", "tile_mix(2, 64, 64)"),
]


@pytest.mark.parametrize("name,expr", CASES)
def test_block_sse_and_psnr_match_oracle(gpu, port, manifest, name, expr):
    from fastc_gb300 import psnr

    assert manifest["cases"][name]["image"] == expr
    img = make_image(expr)
    blocks = golden_blocks(name)
    h, w = img.shape[:2]
    db, sse = psnr(blocks, img, w, h, block_sse=True)
    dec = port.decompress(blocks, w, h)
    want_sse = port.block_sse(img, dec)
    assert np.array_equal(sse, want_sse)
    assert abs(db - port.psnr(img, dec)) <= 1e-9


def test_device_entry_equals_host_entry(gpu, port):
    import torch

    from fastc_gb300 import CompressionSettings, compress_image_data, psnr

    img = make_image("tile_mix(61, 512, 256)")
    blocks = compress_image_data(img, 512, 256, CompressionSettings(num_simulated_annealing_steps=8, seed=2))
    host_db, host_sse = psnr(blocks, img, 512, 256, block_sse=True)
    dev_db, dev_sse = psnr(torch.from_numpy(blocks).to(gpu), torch.from_numpy(img).to(gpu), 512, 256,
                           block_sse=True)
    assert np.array_equal(host_sse, dev_sse)
    assert host_db == dev_db
    # twice in a row: the fixed-order sum repeats bit for bit
    assert psnr(blocks, img, 512, 256) == host_db
    assert abs(host_db - port.psnr(img, port.decompress(blocks, 512, 256))) <= 1e-9


def test_lossless_block_has_zero_error(gpu):
    from fastc_gb300 import CompressionSettings, compress_image_data, psnr

    img = np.zeros((8, 8, 4), np.uint8)
    img[..., 3] = 255
    blocks = compress_image_data(img, 8, 8, CompressionSettings(num_simulated_annealing_steps=0))
    db, sse = psnr(blocks, img, 8, 8, block_sse=True)
    assert db == float("inf") and not sse.any()
