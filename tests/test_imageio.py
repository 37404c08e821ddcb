"""The command-line tool's file formats, on the CPU: PNG round trips, the
KTX container byte for byte as FasTC's ImageWriterKTX lays it out, zero
padding to whole blocks, and the PSNR formula."""
import struct

import numpy as np
import pytest

from conftest import make_image


def test_png_round_trip_and_filters():
    from fastc_gb300 import imageio

    img = make_image("tile_mix(3, 20, 12)")
    assert np.array_equal(imageio.read_png(imageio.png_bytes(img)), img)


def test_png_reader_undoes_every_filter():
    import zlib

    from fastc_gb300 import imageio

    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (5, 7, 4), dtype=np.uint8)
    rows = []
    prev = np.zeros(28, dtype=np.int32)
    for y in range(5):
        f = y % 5
        line = img[y].reshape(-1).astype(np.int32)
        enc = np.zeros(28, dtype=np.int32)
        for x in range(28):
            a = line[x - 4] if x >= 4 else 0
            b = prev[x]
            c = prev[x - 4] if x >= 4 else 0
            pred = [0, a, b, (a + b) >> 1, int(imageio._paeth(np.int32(a), np.int32(b), np.int32(c)))][f]
            enc[x] = (line[x] - pred) & 0xFF
        rows.append(bytes([f]) + enc.astype(np.uint8).tobytes())
        prev = line

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body))

    png = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 7, 5, 8, 6, 0, 0, 0)) +
           chunk(b"IDAT", zlib.compress(b"".join(rows))) + chunk(b"IEND", b""))
    assert np.array_equal(imageio.read_png(png), img)


def test_ktx_layout_matches_fastc_writer():
    """IO/src/ImageWriterKTX.cpp: identifier, 13 words, the KTXorientation
    pair padded with the key's first byte, image size, blocks: 96 bytes of
    header for BC7."""
    from fastc_gb300 import imageio

    blocks = np.arange(64, dtype=np.uint8)
    raw = imageio.ktx_bytes(blocks, 8, 8)
    assert len(raw) == 96 + 64
    assert raw[:12] == bytes([0xAB, 0x4B, 0x54, 0x58, 0x20, 0x31, 0x31, 0xBB, 0x0D, 0x0A, 0x1A, 0x0A])
    words = struct.unpack("<13I", raw[12:64])
    assert words == (0x04030201, 0, 1, 0, 0x8E8C, 0x1908, 8, 8, 0, 0, 1, 1, 28)
    assert raw[64:68] == struct.pack("<I", 23)
    assert raw[68:92] == b"KTXorientation\0S=r,T=d\0K"
    assert raw[92:96] == struct.pack("<I", 64)
    b, w, h = imageio.read_ktx(raw)
    assert (w, h) == (8, 8) and np.array_equal(b, blocks)


@pytest.mark.parametrize("fmt,internal,base,size", [("DXT1", 0x83F0, 0x1907, 32), ("DXT5", 0x83F3, 0x1908, 64)])
def test_ktx_layout_for_dxt(fmt, internal, base, size):
    """ImageWriterKTX's DXT cases (IO/src/ImageWriterKTX.cpp:104-112,
    140-151): the S3TC internal formats, RGB base for DXT1, half a byte per
    texel for DXT1."""
    from fastc_gb300 import imageio

    blocks = np.arange(size, dtype=np.uint8)
    raw = imageio.ktx_bytes(blocks, 8, 8, fmt)
    assert len(raw) == 96 + size
    words = struct.unpack("<13I", raw[12:64])
    assert words[4:6] == (internal, base)
    assert raw[92:96] == struct.pack("<I", size)
    b, w, h, f = imageio.read_ktx(raw, with_format=True)
    assert (w, h, f) == (8, 8, fmt) and np.array_equal(b, blocks)
    with pytest.raises(ValueError):
        imageio.ktx_bytes(blocks[:-1], 8, 8, fmt)


def test_pad_to_blocks_and_basename():
    from fastc_gb300 import imageio, tc

    img = make_image("tile_mix(4, 16, 16)")[:13, :10]
    p = imageio.pad_to_blocks(img)
    assert p.shape == (16, 12, 4) and np.array_equal(p[:13, :10], img) and not p[13:].any()
    # FasTC's ExtractBasename: no directory, nothing from the first dot on
    assert tc.basename("dir/sub/tex.v2.png") == "tex"
    assert tc.basename("tex") == "tex"


def test_cli_refuses_what_it_does_not_do(capsys):
    from fastc_gb300 import tc

    assert tc.main(["-f", "ETC1", "x.png"]) == 1
    assert tc.main(["-f", "PVRTC", "x.png"]) == 1
    assert tc.main(["-f", "PVRTCLib", "x.png"]) == 1
    assert tc.main(["-q"]) == 1
    assert tc.main([]) == 1


def _tga_names():
    import json
    import os

    with open(os.path.join(os.path.dirname(__file__), "golden", "manifest.json")) as f:
        return sorted(json.load(f)["tga"])


@pytest.mark.parametrize("name", _tga_names())
def test_tga_reads_as_fasTC_loader(manifest, name):
    """TGA inputs decode to the texels FasTC's tc loads from them
    (ImageLoaderTGA over its targa reader, rows bottom-up whatever the
    descriptor says), and the files FasTC refuses are refused."""
    import hashlib
    import os

    from fastc_gb300 import imageio

    e = manifest["tga"][name]
    path = os.path.join(os.path.dirname(__file__), "golden", name + ".tga")
    with open(path, "rb") as f:
        raw = f.read()
    assert hashlib.sha256(raw).hexdigest() == e["file_sha256"]
    if e.get("refused"):
        with pytest.raises(ValueError):
            imageio.read_tga(raw)
        return
    img = imageio.read_tga(raw)
    assert img.shape == (e["height"], e["width"], 4) and img.dtype == np.uint8
    assert hashlib.sha256(img.tobytes()).hexdigest() == e["decoded_sha256"]
    assert np.array_equal(imageio.load_image(path), img)


def _ktx_in_names():
    import json
    import os

    with open(os.path.join(os.path.dirname(__file__), "golden", "manifest.json")) as f:
        return sorted(json.load(f)["ktx_in"])


@pytest.mark.parametrize("name", _ktx_in_names())
def test_uncompressed_ktx_reads_as_fasTC_loader(manifest, name):
    """Uncompressed KTX inputs give the texels FasTC's tc loads from them
    (ImageLoaderKTX: either byte order, key/value data skipped, texels in
    file order), the files it refuses are refused, and a compressed file
    (which FasTC loads as blocks) is refused as an input to compress."""
    import hashlib
    import os

    from fastc_gb300 import imageio

    e = manifest["ktx_in"][name]
    path = os.path.join(os.path.dirname(__file__), "golden", name + ".ktx")
    with open(path, "rb") as f:
        raw = f.read()
    assert hashlib.sha256(raw).hexdigest() == e["file_sha256"]
    if e.get("refused") or e.get("compressed"):
        with pytest.raises(ValueError):
            imageio.read_ktx_image(raw)
        return
    img = imageio.read_ktx_image(raw)
    assert img.shape == (e["height"], e["width"], 4)
    assert hashlib.sha256(img.tobytes()).hexdigest() == e["decoded_sha256"]
    assert np.array_equal(imageio.load_image(path), img)
