"""Image files for the command-line tool: PNG (8-bit RGB/RGBA/grey, no
interlace) read and written with zlib, TGA and uncompressed KTX read as
FasTC's loaders read them, raw RGBA8, numpy arrays, and the KTX container
FasTC writes for compressed images (BPTC, DXT1, DXT5).

The KTX layout follows FasTC's ImageWriterKTX (IO/src/ImageWriterKTX.cpp:
the 12-byte identifier, thirteen little-endian words, one key/value pair
"KTXorientation" = "S=r,T=d" padded to four bytes with the key's leading
bytes, the image size and the blocks), so files are byte-identical.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

KTX_IDENTIFIER = bytes([0xAB, 0x4B, 0x54, 0x58, 0x20, 0x31, 0x31, 0xBB, 0x0D, 0x0A, 0x1A, 0x0A])
GL_RGB = 0x1907
GL_RGBA = 0x1908
GL_COMPRESSED_RGBA_BPTC_UNORM = 0x8E8C
GL_COMPRESSED_RGB_S3TC_DXT1_EXT = 0x83F0
GL_COMPRESSED_RGBA_S3TC_DXT5_EXT = 0x83F3
# format -> (glInternalFormat, glBaseFormat, bytes per texel x 2), as
# ImageWriterKTX writes them (IO/src/ImageWriterKTX.cpp:93-113, 140-151)
_KTX_FORMATS = {
    "BPTC": (GL_COMPRESSED_RGBA_BPTC_UNORM, GL_RGBA, 2),
    "DXT1": (GL_COMPRESSED_RGB_S3TC_DXT1_EXT, GL_RGB, 1),
    "DXT5": (GL_COMPRESSED_RGBA_S3TC_DXT5_EXT, GL_RGBA, 2),
}
_ORIENT_KEY = b"KTXorientation"
_ORIENT_VALUE = b"S=r,T=d"


def ktx_bytes(blocks: np.ndarray, width: int, height: int, format: str = "BPTC") -> bytes:
    """A KTX file holding compressed blocks as FasTC writes it: BPTC and
    DXT5 width*height bytes, DXT1 half that."""
    internal, base, twice = _KTX_FORMATS[format]
    data = np.ascontiguousarray(blocks, dtype=np.uint8).tobytes()
    if len(data) != width * height * twice // 2:
        raise ValueError(f"{format} data must be {width * height * twice // 2} bytes")
    kv = len(_ORIENT_KEY) + 1 + len(_ORIENT_VALUE) + 1
    total_kv = (kv + 4 + 3) & ~3
    head = KTX_IDENTIFIER + struct.pack(
        "<13I", 0x04030201, 0, 1, 0, internal, base, width, height, 0, 0, 1, 1, total_kv)
    pad = (_ORIENT_KEY * 2)[: total_kv - kv - 4]
    body = struct.pack("<I", kv) + _ORIENT_KEY + b"\0" + _ORIENT_VALUE + b"\0" + pad
    return head + body + struct.pack("<I", len(data)) + data


def read_ktx(raw: bytes, with_format: bool = False):
    """(blocks, width, height) of a BPTC, DXT1 or DXT5 KTX file; with
    ``with_format`` also the format name."""
    if raw[:12] != KTX_IDENTIFIER:
        raise ValueError("not a KTX file")
    words = struct.unpack("<13I", raw[12:64])
    fmt = [k for k, v in _KTX_FORMATS.items() if v[0] == words[4]]
    if words[0] != 0x04030201 or not fmt:
        raise ValueError("not a little-endian BPTC / DXT1 / DXT5 KTX file")
    width, height, kv = words[6], words[7], words[12]
    off = 64 + kv
    (size,) = struct.unpack("<I", raw[off:off + 4])
    blocks = np.frombuffer(raw[off + 4:off + 4 + size], dtype=np.uint8).copy()
    return (blocks, width, height, fmt[0]) if with_format else (blocks, width, height)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def read_png(raw: bytes) -> np.ndarray:
    """RGBA8 (h, w, 4) of an 8-bit, non-interlaced PNG."""
    if raw[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, hdr = 8, [], None
    while pos < len(raw):
        (ln,) = struct.unpack(">I", raw[pos:pos + 4])
        kind = raw[pos + 4:pos + 8]
        body = raw[pos + 8:pos + 8 + ln]
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        pos += 12 + ln
    if hdr is None:
        raise ValueError("PNG without IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    chans = {0: 1, 2: 3, 4: 2, 6: 4}.get(ctype)
    if depth != 8 or chans is None or interlace:
        raise ValueError("only 8-bit grey/RGB/RGBA non-interlaced PNGs are supported")
    data = np.frombuffer(zlib.decompress(b"".join(idat)), dtype=np.uint8)
    stride = w * chans
    rows = data.reshape(h, stride + 1)
    out = np.zeros((h, stride), dtype=np.int32)
    prev = np.zeros(stride, dtype=np.int32)
    for y in range(h):
        f, line = rows[y, 0], rows[y, 1:].astype(np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 0xFF
        else:
            cur = np.zeros(stride, dtype=np.int32)
            for x in range(stride):
                a = cur[x - chans] if x >= chans else 0
                b = prev[x]
                c = prev[x - chans] if x >= chans else 0
                if f == 1:
                    pred = a
                elif f == 3:
                    pred = (a + b) >> 1
                else:
                    pred = int(_paeth(np.int32(a), np.int32(b), np.int32(c)))
                cur[x] = (line[x] + pred) & 0xFF
        out[y] = cur
        prev = cur
    img = out.astype(np.uint8).reshape(h, w, chans)
    if chans == 4:
        return img
    rgba = np.full((h, w, 4), 255, dtype=np.uint8)
    if chans == 3:
        rgba[..., :3] = img
    elif chans == 2:
        rgba[..., :3] = img[..., :1]
        rgba[..., 3] = img[..., 1]
    else:
        rgba[..., :3] = img
    return rgba


def png_bytes(rgba: np.ndarray) -> bytes:
    """An RGBA8 PNG (filter 0 on every row)."""
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = rgba.shape[:2]
    rows = np.concatenate([np.zeros((h, 1), dtype=np.uint8), rgba.reshape(h, w * 4)], axis=1)

    def chunk(kind: bytes, body: bytes) -> bytes:
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body))

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(rows.tobytes(), 6)) + chunk(b"IEND", b""))


GL_BYTE = 0x1400
GL_RGBA8 = 0x8058


def read_ktx_image(raw: bytes) -> np.ndarray:
    """RGBA8 (h, w, 4) from an uncompressed KTX file, read as FasTC's loader
    reads it (ImageLoaderKTX::ReadData, IO/src/ImageLoaderKTX.cpp:128-346):
    the identifier, the byte order from the endianness word (big-endian
    integers when its first byte is 4), the key/value data skipped; one
    mipmap level, one face, no array, depth 0 and a nonzero size; glType
    GL_BYTE (0x1400, the type FasTC's writer records for RGBA8) and
    glInternalFormat GL_RGBA8; then the image size word and the texels in
    file order, which must end the file. Compressed files (glType and
    glFormat 0) are refused: they hold blocks, not texels to encode."""
    if len(raw) < 68 or raw[:12] != KTX_IDENTIFIER:
        raise ValueError("KTX: not a KTX file")
    order = ">" if raw[12] == 0x04 else "<"
    (gl_type, _type_size, gl_format, internal, _base, w, h, depth, arrays, faces, mips,
     kv) = struct.unpack(order + "12I", raw[16:64])
    pos = 64 + kv
    if mips != 1:
        raise ValueError(f"KTX: unsupported mipmap levels: {mips}")
    if pos + 4 > len(raw):
        raise ValueError("KTX: truncated")
    if arrays > 1 or faces != 1 or depth != 0 or h == 0 or w == 0:
        raise ValueError("KTX: only single 2-D images are supported")
    if gl_type == 0 and gl_format == 0:
        raise ValueError("KTX: a compressed file holds blocks; decode it before compressing")
    if gl_type != GL_BYTE or internal != GL_RGBA8:
        raise ValueError(f"KTX: unsupported type 0x{gl_type:x} / internal format 0x{internal:x}")
    pos += 4  # the image size word
    n = w * h * 4
    if pos + n != len(raw):
        raise ValueError("KTX: the texels do not end the file")
    return np.frombuffer(raw, dtype=np.uint8, count=n, offset=pos).reshape(h, w, 4).copy()


def read_tga(raw: bytes) -> np.ndarray:
    """RGBA8 (h, w, 4) from a TGA file, read as FasTC's loader reads it
    (ImageLoaderTGA::ReadData, IO/src/ImageLoaderTGA.cpp:35-48, over
    targa_loadFromData, IO/third_party/tga/targa.c:262-571):

    * no colour maps; image types 0, 1 and 9 are refused, types 2 and 3 are
      read as uncompressed BGR(A) (type 3 too), every other type as
      run-length packets (targa.c:323-329, 436, 480);
    * 24- and 32-bit texels (alpha 255 at 24 bits), and 16-bit texels in
      uncompressed files only, red from the low five bits and blue from the
      high five, each shifted up by three, alpha 255 (targa.c:387-399,
      453-458); 8-bit files are refused;
    * the image descriptor is ignored: the rows are always taken bottom-up
      (ImageLoader::LoadFromPixelBuffer with flipY, IO/src/ImageLoader.cpp:
      122-149).

    Truncated files raise ValueError (FasTC refuses them too, apart from
    reading a few bytes past the end of a run-length file)."""
    if len(raw) < 18:
        raise ValueError("TGA: file shorter than its header")
    id_len, cmap, itype = raw[0], raw[1], raw[2]
    if cmap != 0:
        raise ValueError("TGA: colour-mapped files are not supported")
    if itype in (0, 1, 9):
        raise ValueError(f"TGA: unsupported image type {itype}")
    w, h = struct.unpack("<hh", raw[12:16])
    if w < 1 or h < 1:
        raise ValueError(f"TGA: invalid size {w}x{h}")
    depth = raw[16]
    if depth not in (16, 24, 32):
        raise ValueError(f"TGA: unsupported pixel depth of {depth} bits")
    rle = itype not in (2, 3)
    if depth == 16 and rle:
        raise ValueError("TGA: run-length files of 16-bit texels are not supported")
    pos = 18 + id_len
    if pos > len(raw):
        raise ValueError("TGA: truncated image ID")
    n = w * h
    out = np.empty((n, 4), dtype=np.uint8)
    if not rle:
        cm = 2 if depth == 16 else depth // 8
        if pos + n * cm > len(raw):
            raise ValueError("TGA: truncated pixel data")
        if depth == 16:
            v = np.frombuffer(raw, dtype="<u2", count=n, offset=pos)
            out[:, 0] = (v & 31) << 3
            out[:, 1] = ((v >> 5) & 31) << 3
            out[:, 2] = ((v >> 10) & 31) << 3
            out[:, 3] = 255
        else:
            px = np.frombuffer(raw, dtype=np.uint8, count=n * cm, offset=pos).reshape(n, cm)
            out[:, :3] = px[:, 2::-1]
            out[:, 3] = px[:, 3] if cm == 4 else 255
    else:
        cm = depth // 8
        buf = np.frombuffer(raw, dtype=np.uint8)
        k = 0
        while k < n:
            if pos >= len(raw):
                raise ValueError("TGA: truncated run-length data")
            hdr = raw[pos]
            pos += 1
            if hdr < 128:  # a packet of hdr + 1 literal texels
                cnt = min(hdr + 1, n - k)
                if pos + cnt * cm > len(raw):
                    raise ValueError("TGA: truncated run-length data")
                px = buf[pos:pos + cnt * cm].reshape(cnt, cm)
                pos += (hdr + 1) * cm
            else:  # a run of hdr - 127 copies of one texel
                cnt = min(hdr - 127, n - k)
                if pos + cm > len(raw):
                    raise ValueError("TGA: truncated run-length data")
                px = np.broadcast_to(buf[pos:pos + cm], (cnt, cm))
                pos += cm
            out[k:k + cnt, :3] = px[:, 2::-1]
            out[k:k + cnt, 3] = px[:, 3] if cm == 4 else 255
            k += cnt
    return np.ascontiguousarray(out.reshape(h, w, 4)[::-1])


def load_image(path: str, width: int = 0, height: int = 0) -> np.ndarray:
    """RGBA8 (h, w, 4) from .png, .tga, uncompressed .ktx, .npy or raw RGBA
    (.rgba, needs width/height)."""
    if path.endswith(".npy"):
        img = np.load(path)
    elif path.endswith(".rgba") or path.endswith(".raw"):
        if not (width and height):
            raise ValueError("raw RGBA input needs its size (-s WxH)")
        img = np.fromfile(path, dtype=np.uint8).reshape(height, width, 4)
    elif path.endswith(".tga"):
        with open(path, "rb") as f:
            img = read_tga(f.read())
    elif path.endswith(".ktx"):
        with open(path, "rb") as f:
            img = read_ktx_image(f.read())
    else:
        with open(path, "rb") as f:
            img = read_png(f.read())
    if img.ndim != 3 or img.shape[2] != 4 or img.dtype != np.uint8:
        raise ValueError("images must be RGBA8")
    return img


def pad_to_blocks(img: np.ndarray) -> np.ndarray:
    """Zero-pad to multiples of 4, as FasTC's CompressImage does
    (Core/src/TexComp.cpp:382-396)."""
    h, w = img.shape[:2]
    H, W = (h + 3) & ~3, (w + 3) & ~3
    if (H, W) == (h, w):
        return img
    out = np.zeros((H, W, 4), dtype=np.uint8)
    out[:h, :w] = img
    return out
