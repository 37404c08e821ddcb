"""The tc-compatible command line on the GPU: PNG in, KTX out, the blocks
those of the library call, PSNR printed as FasTC's tc prints it."""
import hashlib
import re

import numpy as np
import pytest

from conftest import make_image

pytestmark = pytest.mark.gpu


def test_tc_png_to_ktx(gpu, tmp_path, capsys):
    from fastc_gb300 import CompressionJob, CompressionSettings, compress, imageio, tc

    img = make_image("tile_mix(41, 40, 24)")
    src = tmp_path / "in.png"
    src.write_bytes(imageio.png_bytes(img))
    out = tmp_path / "out.ktx"
    assert tc.main(["-q", "8", "-t", "4", "-d", str(out), str(src)]) == 0
    blocks, w, h = imageio.read_ktx(out.read_bytes())
    want = np.zeros(40 * 24, np.uint8)
    compress(CompressionJob(img, want, 40, 24), CompressionSettings(num_simulated_annealing_steps=8))
    assert (w, h) == (40, 24) and np.array_equal(blocks, want)
    line = [l for l in capsys.readouterr().out.splitlines() if l.startswith("PSNR: ")]
    assert line and float(line[0].split()[1]) > 20.0


@pytest.mark.parametrize("fmt,ktx", [("BPTC", "ktx_bptc_tile_q0"), ("DXT1", "ktx_dxt1_tile"),
                                     ("DXT5", "ktx_dxt5_tile")])
def test_tc_writes_fasTC_file_and_psnr_line(gpu, manifest, tmp_path, capsys, fmt, ktx):
    """`tc -q 0 -f FMT -d out.ktx` on a fixture image writes the very file
    FasTC's tc writes (its blocks, through its ImageWriterKTX) and prints
    FasTC's PSNR line (its Image::ComputePSNR of its decoder's texels)."""
    from fastc_gb300 import imageio, tc

    e = manifest["ktx"][ktx]
    src_case = manifest["cases" if fmt == "BPTC" else "dxt"][e["blocks"]]
    img = make_image(src_case["image"])
    src = tmp_path / "fixture.png"
    src.write_bytes(imageio.png_bytes(img))
    out = tmp_path / "out.ktx"
    assert tc.main(["-q", "0", "-f", fmt, "-d", str(out), str(src)]) == 0
    raw = out.read_bytes()
    assert len(raw) == e["bytes"] and hashlib.sha256(raw).hexdigest() == e["sha256"]
    # FasTC's stdout: the compression time (CompressImageData), then the PSNR
    lines = capsys.readouterr().out.splitlines()
    assert re.fullmatch(r"Compression time: \d+\.\d{3} ms", lines[0])
    assert lines[1:] == [f"PSNR: {src_case['tc_psnr']:.3f}"]


def test_tc_pads_odd_sizes_and_writes_decoded_png(gpu, tmp_path, capsys):
    """An image that is not whole blocks is zero-padded with FasTC's warning;
    the compressed image then has the padded size, so, as FasTC's tc, no
    PSNR is printed but the message that the sizes differ."""
    from fastc_gb300 import imageio, tc

    img = make_image("tile_mix(42, 16, 16)")[:14, :9].copy()
    src = tmp_path / "odd.npy"
    np.save(src, img)
    out = tmp_path / "odd-bptc.png"
    assert tc.main(["-q", "0", "-d", str(out), str(src)]) == 0
    dec = imageio.read_png(out.read_bytes())
    assert dec.shape == (16, 12, 4)
    cap = capsys.readouterr()
    assert "PSNR" not in cap.out
    assert cap.err.splitlines() == [
        "TexComp -- WARNING - Image size is not a multiple of block size. Padding with zeros...",
        "Cannot compute image metrics: compressed and uncompressed dimensions differ."]


def test_tc_log_is_compress_with_stats(gpu, tmp_path, monkeypatch):
    """-l writes FasTC's per-block log to <basename>.log, the blocks those
    of the logging encoder."""
    from fastc_gb300 import CompressionJob, CompressionSettings, compress_with_stats, imageio, tc

    img = make_image("tile_mix(43, 32, 24)")
    src = tmp_path / "logged.tex.png"
    src.write_bytes(imageio.png_bytes(img))
    monkeypatch.chdir(tmp_path)
    assert tc.main(["-l", "-q", "4", "-d", "out.ktx", str(src)]) == 0
    want = np.zeros(32 * 24, np.uint8)
    log = compress_with_stats(CompressionJob(img, want, 32, 24),
                              CompressionSettings(num_simulated_annealing_steps=4))
    assert (tmp_path / "logged.log").read_text() == log
    blocks, _, _ = imageio.read_ktx((tmp_path / "out.ktx").read_bytes())
    assert np.array_equal(blocks, want)


@pytest.mark.parametrize("fmt", ["DXT1", "DXT5"])
def test_tc_dxt_to_ktx_and_png(gpu, port, tmp_path, capsys, monkeypatch, fmt):
    """-f DXT1 / DXT5: the blocks in FasTC's KTX layout are the oracle's
    (FasTC's) blocks, the PSNR is FasTC's metric of their decode, the
    default output is <basename>-dxt1.png / -dxt5.png, and -l leaves an
    empty log (FasTC has no logging DXT encoder)."""
    from fastc_gb300 import imageio, tc

    img = make_image("tile_mix_radial_alpha(44, 48, 32, 100, 200)")
    src = tmp_path / "dxt_in.png"
    src.write_bytes(imageio.png_bytes(img))
    out = tmp_path / "out.ktx"
    assert tc.main(["-f", fmt, "-d", str(out), str(src)]) == 0
    blocks, w, h, f = imageio.read_ktx(out.read_bytes(), with_format=True)
    want = port.dxt_compress(img, fmt == "DXT5")
    assert (w, h, f) == (48, 32, fmt) and np.array_equal(blocks, want)
    dec = port.dxt_decompress(want, 48, 32, fmt == "DXT5")
    line = [l for l in capsys.readouterr().out.splitlines() if l.startswith("PSNR: ")]
    assert line and line[0] == f"PSNR: {port.psnr(img, dec):.3f}"
    monkeypatch.chdir(tmp_path)
    assert tc.main(["-f", fmt, "-l", str(src)]) == 0
    assert np.array_equal(imageio.read_png((tmp_path / f"dxt_in-{fmt.lower()}.png").read_bytes()), dec)
    assert (tmp_path / "dxt_in.log").read_text() == ""


@pytest.mark.parametrize("group,name,ext", [("tga", "tga24_raw", ".tga"), ("tga", "tga32_rle", ".tga"),
                                            ("tga", "tga16_raw", ".tga"), ("ktx_in", "ktxin_le", ".ktx"),
                                            ("ktx_in", "ktxin_be", ".ktx")])
def test_tc_tga_and_ktx_input_gives_fasTC_output(gpu, manifest, tmp_path, capsys, group, name, ext):
    """`tc -q 0 -d out.ktx file.tga|file.ktx`: the blocks FasTC's tc writes
    for the texels its loader reads, and its PSNR line."""
    import os
    import shutil

    from fastc_gb300 import imageio, tc

    e = manifest[group][name]
    src = tmp_path / ("in_" + name + ext)
    shutil.copy(os.path.join(os.path.dirname(__file__), "golden", name + ext), src)
    out = tmp_path / "out.ktx"
    assert tc.main(["-q", "0", "-d", str(out), str(src)]) == 0
    blocks, w, h = imageio.read_ktx(out.read_bytes())
    assert (w, h) == (e["width"], e["height"])
    assert hashlib.sha256(blocks.tobytes()).hexdigest() == e["q0_blocks_sha256"]
    line = [l for l in capsys.readouterr().out.splitlines() if l.startswith("PSNR: ")]
    assert line == [f"PSNR: {e['q0_tc_psnr']:.3f}"]
