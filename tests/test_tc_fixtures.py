"""What FasTC's tc prints and writes after the encode, pinned to FasTC
itself: the KTX files of its ImageWriterKTX (IO/src/ImageWriterKTX.cpp:69-161)
and the PSNR of its Image::ComputePSNR over its own decoders
(Base/src/Image.cpp:206-255, CLTool/src/tc.cpp:302), both recorded from the
reference build by tests/golden/make_golden.py."""
import hashlib

import numpy as np
import pytest

from conftest import golden_blocks, make_image

_FORMAT_NAMES = {1: "DXT1", 5: "DXT5", 7: "BPTC"}


@pytest.mark.parametrize("name", ["ktx_bptc_tile_q0", "ktx_dxt1_tile", "ktx_dxt5_tile"])
def test_ktx_bytes_are_fasTC_writer_file(manifest, name):
    from fastc_gb300 import imageio

    e = manifest["ktx"][name]
    raw = imageio.ktx_bytes(golden_blocks(e["blocks"]), e["width"], e["height"],
                            _FORMAT_NAMES[e["format"]])
    assert raw[:96].hex() == e["header_hex"]
    assert len(raw) == e["bytes"] and hashlib.sha256(raw).hexdigest() == e["sha256"]
    blocks, w, h, f = imageio.read_ktx(raw, with_format=True)
    assert (w, h, f) == (e["width"], e["height"], _FORMAT_NAMES[e["format"]])
    assert np.array_equal(blocks, golden_blocks(e["blocks"]))


def _psnr_cases(manifest):
    for group in ("cases", "dxt"):
        for name, e in sorted(manifest[group].items()):
            if "tc_psnr" in e:
                yield name, e


def test_oracle_psnr_is_fasTC_tc_psnr(port, manifest):
    """The oracle's PSNR sums FasTC's terms in FasTC's order: equal to
    FasTC's value to rounding of log10 (1e-12), and the same text in tc's
    "PSNR: %.3f" line, for every fixture."""
    seen = 0
    for name, e in _psnr_cases(manifest):
        img = make_image(e["image"])
        h, w = img.shape[:2]
        blocks = golden_blocks(name)
        fmt = e.get("format", 7)
        dec = port.decompress(blocks, w, h) if fmt == 7 else port.dxt_decompress(blocks, w, h, fmt == 5)
        got = port.psnr(img, dec)
        assert abs(got - e["tc_psnr"]) <= 1e-12, (name, got, e["tc_psnr"])
        assert f"{got:.3f}" == f"{e['tc_psnr']:.3f}"
        seen += 1
    assert seen >= 13
