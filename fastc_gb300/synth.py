"""Seeded synthetic RGBA8 textures for the BC7 workloads.

FasTC's BC7 path has no public benchmark set, so every workload here is a
seeded synthetic image. All randomness comes from an integer hash of
(seed, stream, coordinates), so an image is a pure function of its seed and
geometry, identical on every machine and numpy version, and any
sub-rectangle of a large virtual image can be generated on its own.

Workloads (pixel data is uint8 [H, W, 4], R first):

* ``gradient_noise_alpha_ramp`` -- a bilinear gradient between four seeded
  corner colours plus 4-octave value noise (lattice periods 32/16/8/4 px,
  amplitude halving, +-24 levels in total per RGB channel); alpha is 255
  except one 64x64 block-aligned square holding a linear 0..255 ramp.
* ``tile_mix`` -- 8x8 tiles, each one of four kinds chosen uniformly: a
  smooth two-colour gradient in a random direction; uniform RGB noise; two
  flat colours split by a random straight edge; a gradient with per-texel
  random alpha in [0, 255].
* ``tile_mix_radial_alpha`` -- the tile_mix colours with alpha replaced by a
  seeded radial gradient plus noise, so every block carries alpha.
* ``texture_set`` -- many textures whose sides are drawn log-uniformly from
  {16, 32, ..., 2048} per axis, each filled with tile_mix.
"""
from __future__ import annotations

import numpy as np

_M32 = np.uint32(0xFFFFFFFF)


def _hash32(x: np.ndarray) -> np.ndarray:
    """lowbias32 integer hash (C. Wellons), vectorised over uint32."""
    x = np.asarray(x, dtype=np.uint32).copy()
    with np.errstate(over="ignore"):
        x ^= x >> np.uint32(16)
        x *= np.uint32(0x7FEB352D)
        x ^= x >> np.uint32(15)
        x *= np.uint32(0x846CA68B)
        x ^= x >> np.uint32(16)
    return x


def _h(seed: int, stream: int, *coords) -> np.ndarray:
    """Hash of (seed, stream, coords...) broadcast over array coordinates."""
    h = _hash32(np.uint32((seed * 0x9E3779B1 + stream * 0x85EBCA77) & 0xFFFFFFFF))
    for c in coords:
        c = np.asarray(c).astype(np.int64).astype(np.uint32)
        with np.errstate(over="ignore"):
            h = _hash32(h ^ (c * np.uint32(0x27D4EB2F) + np.uint32(0x165667B1)))
    return h


def _unit(seed: int, stream: int, *coords) -> np.ndarray:
    """Uniform float64 in [0, 1) from 24 hash bits."""
    return (_h(seed, stream, *coords) >> np.uint32(8)).astype(np.float64) / float(1 << 24)


def _grid(x0: int, y0: int, w: int, h: int):
    ys, xs = np.mgrid[y0:y0 + h, x0:x0 + w]
    return xs.astype(np.int64), ys.astype(np.int64)


def _value_noise(seed: int, stream: int, xs, ys, period: int) -> np.ndarray:
    """Bilinear value noise in [-1, 1) on a lattice of the given period."""
    gx, gy = xs // period, ys // period
    fx = (xs - gx * period) / period
    fy = (ys - gy * period) / period
    v00 = _unit(seed, stream, gx, gy)
    v10 = _unit(seed, stream, gx + 1, gy)
    v01 = _unit(seed, stream, gx, gy + 1)
    v11 = _unit(seed, stream, gx + 1, gy + 1)
    v = (v00 * (1 - fx) + v10 * fx) * (1 - fy) + (v01 * (1 - fx) + v11 * fx) * fy
    return 2.0 * v - 1.0


def _to_u8(x: np.ndarray) -> np.ndarray:
    return np.clip(np.floor(x + 0.5), 0, 255).astype(np.uint8)


def gradient_noise_alpha_ramp(seed: int = 1, width: int = 256, height: int = 256) -> np.ndarray:
    """Smooth gradient + value noise, opaque except one 64x64 alpha ramp."""
    xs, ys = _grid(0, 0, width, height)
    u = xs / max(width - 1, 1)
    v = ys / max(height - 1, 1)
    img = np.empty((height, width, 4), dtype=np.uint8)
    amp0 = 24.0 / (1 + 0.5 + 0.25 + 0.125)
    for ch in range(3):
        c = [255.0 * _unit(seed, 1, k, ch) for k in range(4)]
        base = (c[0] * (1 - u) + c[1] * u) * (1 - v) + (c[2] * (1 - u) + c[3] * u) * v
        noise = np.zeros_like(base)
        for octave, period in enumerate((32, 16, 8, 4)):
            noise += amp0 * 0.5 ** octave * _value_noise(seed, 10 + 4 * ch + octave, xs, ys, period)
        img[..., ch] = _to_u8(base + noise)
    img[..., 3] = 255
    side = 64
    if width >= side and height >= side:
        rx = int(_h(seed, 2, 0)) % ((width - side) // 4 + 1) * 4
        ry = int(_h(seed, 2, 1)) % ((height - side) // 4 + 1) * 4
        ramp = _to_u8(255.0 * np.arange(side) / (side - 1))
        img[ry:ry + side, rx:rx + side, 3] = ramp[None, :]
    return img


def _tile_params(seed: int, tx, ty):
    """Per-tile random parameters (all arrays shaped like tx)."""
    kind = (_h(seed, 100, tx, ty) % np.uint32(4)).astype(np.int64)
    c0 = np.stack([255.0 * _unit(seed, 101 + ch, tx, ty) for ch in range(3)], -1)
    c1 = np.stack([255.0 * _unit(seed, 104 + ch, tx, ty) for ch in range(3)], -1)
    ang = 2.0 * np.pi * _unit(seed, 107, tx, ty)
    off = _unit(seed, 108, tx, ty) * 6.0 - 3.0
    return kind, c0, c1, ang, off


def tile_mix(seed: int = 2, width: int = 2048, height: int = 2048, x0: int = 0, y0: int = 0,
             tile: int = 8) -> np.ndarray:
    """Four tile kinds on an 8x8 tile grid; any sub-rectangle of the virtual image."""
    xs, ys = _grid(x0, y0, width, height)
    tx, ty = xs // tile, ys // tile
    lx = (xs - tx * tile) - (tile - 1) / 2.0
    ly = (ys - ty * tile) - (tile - 1) / 2.0
    # per-tile parameters on the tile grid, then broadcast to the texels
    tx0, ty0 = x0 // tile, y0 // tile
    gtx, gty = np.mgrid[ty0:int(ty.max()) + 1, tx0:int(tx.max()) + 1][::-1]
    params = _tile_params(seed, gtx.astype(np.int64), gty.astype(np.int64))
    ix, iy = tx - tx0, ty - ty0
    kind, c0, c1, ang, off = (p[iy, ix] for p in params)
    ca, sa = np.cos(ang), np.sin(ang)
    proj = lx * ca + ly * sa
    t = np.clip(proj / (tile * 0.7071) + 0.5, 0.0, 1.0)[..., None]
    grad = c0 * (1 - t) + c1 * t
    noise = np.stack([255.0 * _unit(seed, 110 + ch, xs, ys) for ch in range(3)], -1)
    edge = np.where(((proj - off) > 0)[..., None], c1, c0)
    rgb = np.where((kind == 0)[..., None], grad,
          np.where((kind == 1)[..., None], noise,
          np.where((kind == 2)[..., None], edge, grad)))
    alpha = np.where(kind == 3, 255.0 * _unit(seed, 120, xs, ys) + 0.5, 255.0)
    img = np.empty((height, width, 4), dtype=np.uint8)
    img[..., :3] = _to_u8(rgb)
    img[..., 3] = np.clip(np.floor(alpha), 0, 255).astype(np.uint8)
    return img


def tile_mix_radial_alpha(seed: int = 5, width: int = 8192, height: int = 8192, x0: int = 0,
                          y0: int = 0, full_width: int = 8192, full_height: int = 8192) -> np.ndarray:
    """tile_mix colours; alpha = radial gradient + value noise over the full image."""
    img = tile_mix(seed, width, height, x0, y0)
    xs, ys = _grid(x0, y0, width, height)
    cx = full_width * (0.25 + 0.5 * float(_unit(seed, 200, 0)))
    cy = full_height * (0.25 + 0.5 * float(_unit(seed, 200, 1)))
    rmax = 0.75 * float(np.hypot(full_width, full_height))
    r = np.hypot(xs - cx, ys - cy) / rmax
    a = 255.0 * (1.0 - r) + 32.0 * _value_noise(seed, 201, xs, ys, 16)
    img[..., 3] = _to_u8(a)
    return img


def flat_blocks(seed: int = 0, width: int = 64, height: int = 64) -> np.ndarray:
    """Every 4x4 block one colour: block k has R = k, G = 255 - k, B = 37k,
    A = 91k (mod 256), offset by `seed`, so a 64x64 image walks every value
    of every channel once. Exercises single-colour encodings."""
    bx = np.arange(width // 4)[None, :]
    by = np.arange(height // 4)[:, None]
    k = (by * (width // 4) + bx + seed) % 256
    blk = np.stack([k, 255 - k, (37 * k) % 256, (91 * k) % 256], -1).astype(np.uint8)
    return np.ascontiguousarray(blk.repeat(4, 0).repeat(4, 1))


def texture_sides(seed: int, count: int, lo_log2: int = 4, hi_log2: int = 11):
    """Side lengths 2^U{lo..hi} drawn independently per axis."""
    n = hi_log2 - lo_log2 + 1
    ws = [1 << (lo_log2 + int(_h(seed, 300, i, 0)) % n) for i in range(count)]
    hs = [1 << (lo_log2 + int(_h(seed, 300, i, 1)) % n) for i in range(count)]
    return list(zip(ws, hs))


def texture_set(seed: int = 3, count: int = 512, lo_log2: int = 4, hi_log2: int = 11):
    """`count` tile_mix textures of log-uniform power-of-two sides."""
    out = []
    for i, (w, h) in enumerate(texture_sides(seed, count, lo_log2, hi_log2)):
        out.append(tile_mix(seed * 1000 + i, w, h))
    return out


def pack_u32(img: np.ndarray) -> np.ndarray:
    """[H, W, 4] uint8 -> [H, W] uint32 with R in bits 0-7."""
    return np.ascontiguousarray(img).view("<u4")[..., 0]


def blocks_of(img: np.ndarray) -> np.ndarray:
    """[H, W, 4] uint8 -> [H/4 * W/4, 16] uint32 texel rows, raster order."""
    h, w = img.shape[:2]
    p = pack_u32(img).reshape(h // 4, 4, w // 4, 4).transpose(0, 2, 1, 3)
    return np.ascontiguousarray(p.reshape(-1, 16))
