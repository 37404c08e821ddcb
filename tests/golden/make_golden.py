"""Regenerate the golden BC7 and DXT fixtures from FasTC's own encoders.

Runs only where the FasTC checkout is available (it builds
oracle/_ref/libfastc_ref.so from those sources in place):

    python tests/golden/make_golden.py [--reference /path/to/FasTC]

Every fixture is the reference's output on a seeded synthetic image from
fastc_gb300.synth; manifest.json records the input hashes, settings and
the reference's PSNR so the tests can check the generators too.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fastc_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

# name -> (generator call, steps, metric, pinned LCG seed or None)
CASES = {
    "c1_q0": ("gradient_noise_alpha_ramp(1, 256, 256)", 0, 0, None),
    "tile_q0": ("tile_mix(2, 128, 128)", 0, 0, None),
    "radial_q0": ("tile_mix_radial_alpha(5, 128, 128, 1000, 2000)", 0, 0, None),
    "c1_q0_nonuniform": ("gradient_noise_alpha_ramp(1, 128, 128)", 0, 1, None),
    "c1_q8_seed": ("gradient_noise_alpha_ramp(1, 128, 128)", 8, 0, 0x1234567),
    "tile_q50_seed": ("tile_mix(2, 64, 64)", 50, 0, 0xBEEF),
    "radial_q16_seed": ("tile_mix_radial_alpha(5, 64, 64, 3000, 3000)", 16, 0, 0xC0FFEE),
}

# CompressWithStats with a log stream: name -> (generator call, steps, pinned
# LCG seed or None); the blocks, the log's hash and the parsed statistics
STATS = {
    "tile_stats_q0": ("tile_mix(3, 64, 64)", 0, None),
    "radial_stats_q16_seed": ("tile_mix_radial_alpha(4, 64, 64, 800, 1200)", 16, 0xACE1),
}

# PSNR reference points at q50: the reference with several pinned seeds
QUALITY = {
    "tile_q50_psnr": ("tile_mix(21, 512, 512)", 50, [11, 22, 33]),
    "radial_q50_psnr": ("tile_mix_radial_alpha(5, 512, 512, 4096, 1024)", 50, [11, 22, 33]),
}


# The full-size configurations, FasTC at three pinned seeds each: PSNR and
# per-block SSE (premultiplied metric, float32, compressed). The 2048x2048
# tile mix at q50 is the single-launch configuration; the q100 radial-alpha
# case is the 8192x512 stripe of rows 3840..4351 (through the centre band
# of the radial gradient) of the 8192x8192 image, since FasTC takes about
# 20 minutes per seed on that stripe alone.
FULL_SIZE = {
    "c2_tile2048_q50": ("tile_mix(2, 2048, 2048)", 50, [11, 22, 33]),
    "c5_stripe8192x512_q100": ("tile_mix_radial_alpha(5, 8192, 512, 0, 3840)", 100, [11, 22, 33]),
}

# DXT1 / DXT5: name -> (generator call, format); FasTC's CompressImageDXT1 /
# CompressImageDXT5 blocks and its decoder's texels of them
DXT = {
    "dxt1_tile": ("tile_mix(2, 128, 128)", 1),
    "dxt5_tile": ("tile_mix(2, 128, 128)", 5),
    "dxt1_gradient": ("gradient_noise_alpha_ramp(1, 128, 64)", 1),
    "dxt5_radial": ("tile_mix_radial_alpha(5, 128, 128, 1000, 2000)", 5),
    "dxt1_flat": ("flat_blocks(0, 64, 64)", 1),
    "dxt5_flat": ("flat_blocks(3, 64, 64)", 5),
}
# random block bytes, numpy default_rng(seed).integers(0, 256), decoded by
# FasTC's decoder: name -> (width, height, format, seed); the sizes are not
# multiples of 4, so the decoder's edge clipping is covered too
DXT_DECODE = {
    "dxt1_random_decode": (62, 45, 1, 101),
    "dxt5_random_decode": (61, 46, 5, 102),
}


# The KTX files FasTC's tc writes (`-d out.ktx`) for fixture blocks: name ->
# (blocks fixture, format code). ImageWriterKTX keeps the image size in a
# function-local static, so each file is written by a fresh process, as by
# one run of tc.
KTX = {
    "ktx_bptc_tile_q0": ("tile_q0", 7),
    "ktx_dxt1_tile": ("dxt1_tile", 1),
    "ktx_dxt5_tile": ("dxt5_tile", 5),
}


# TGA inputs as FasTC's tc loads them (ImageLoaderTGA over the vendored
# targa reader): name -> (image, depth, image type, image ID, descriptor
# byte). The files are written here (rows bottom-up, run-length packets where
# the type asks for them) and FasTC's decoded texels recorded; the ones marked
# None are files FasTC refuses (a colour map, 8-bit texels, run-length 16-bit
# texels, image type 1, truncated texels).
TGA = {
    "tga32_raw": ("tile_mix_radial_alpha(6, 24, 20, 5, 3)[:17, :23]", 32, 2, b"fastc", 0x28),
    "tga24_raw": ("tile_mix(7, 20, 12)", 24, 2, b"", 0x00),
    "tga32_rle": ("flat_blocks(8, 40, 24)", 32, 10, b"", 0x08),
    "tga24_rle": ("tile_mix(9, 40, 12)[:9, :37]", 24, 10, b"id", 0x20),
    "tga32_bw_rle": ("flat_blocks(10, 16, 12)", 32, 11, b"", 0x08),
    "tga24_bw": ("tile_mix(11, 12, 8)", 24, 3, b"", 0x00),
    "tga16_raw": ("rng16(12, 16, 8)", 16, 2, b"", 0x00),
}
TGA_REFUSED = ["tga_colormap", "tga8_bw", "tga16_rle", "tga_type1", "tga32_truncated"]


def tga_file(img: np.ndarray, depth: int, itype: int, ident: bytes = b"", desc: int = 0) -> bytes:
    """A TGA file of img (RGBA8, or 16-bit words for depth 16), rows stored
    bottom-up; types 9-11 as run-length packets (runs of 2-128 equal texels,
    literal packets of up to 128)."""
    h, w = img.shape[:2]
    head = struct.pack("<BBBHHBHHHHBB", len(ident), 0, itype, 0, 0, 0, 0, 0, w, h, depth, desc)
    rows = img[::-1].reshape(h * w, -1)
    if depth == 16:
        texels = [int(v).to_bytes(2, "little") for v in rows[:, 0]]
    else:
        cm = depth // 8
        texels = [bytes(p[[2, 1, 0, 3][:cm]]) for p in rows]
    if itype in (2, 3):
        return head + ident + b"".join(texels)
    out, k = bytearray(), 0
    while k < len(texels):
        run = 1
        while k + run < len(texels) and run < 128 and texels[k + run] == texels[k]:
            run += 1
        if run >= 2:
            out += bytes([127 + run]) + texels[k]
            k += run
            continue
        lit = 1
        while (k + lit < len(texels) and lit < 128 and
               not (k + lit + 1 < len(texels) and texels[k + lit] == texels[k + lit + 1])):
            lit += 1
        out += bytes([lit - 1]) + b"".join(texels[k:k + lit])
        k += lit
    return head + ident + bytes(out)


def tga_refused(name: str) -> bytes:
    img = make("tile_mix(13, 8, 8)")
    raw = bytearray(tga_file(img, 32, 2))
    if name == "tga_colormap":
        raw[1] = 1
    elif name == "tga8_bw":
        raw = bytearray(tga_file(img, 32, 3))
        raw[16] = 8
    elif name == "tga16_rle":
        raw = bytearray(tga_file(np.zeros((8, 8, 1), np.uint16), 16, 10))
    elif name == "tga_type1":
        raw[2] = 1
    elif name == "tga32_truncated":
        raw = raw[:-5]
    return bytes(raw)


def rng16(seed: int, w: int, h: int) -> np.ndarray:
    """Random 16-bit texel words (h, w, 1)."""
    return np.random.default_rng(seed).integers(0, 1 << 16, (h, w, 1), dtype=np.uint16)


def make_tga(ref, manifest):
    manifest["tga"] = {}
    for name, (expr, depth, itype, ident, desc) in TGA.items():
        img = eval(expr, {"rng16": rng16}) if expr.startswith("rng16") else make(expr)
        raw = tga_file(np.ascontiguousarray(img), depth, itype, ident, desc)
        with open(os.path.join(HERE, name + ".tga"), "wb") as f:
            f.write(raw)
        dec = ref.load_tga(raw)
        e = manifest["tga"][name] = {"image": expr, "depth": depth, "type": itype,
                                     "file_sha256": hashlib.sha256(raw).hexdigest(),
                                     "width": int(dec.shape[1]), "height": int(dec.shape[0]),
                                     "decoded_sha256": sha(dec)}
        if dec.shape[0] % 4 == 0 and dec.shape[1] % 4 == 0:
            # what `tc -q 0` makes of the file: FasTC's blocks and PSNR line
            blocks = ref.compress(dec, steps=0)
            e["q0_blocks_sha256"] = sha(blocks)
            e["q0_tc_psnr"] = ref.tc_psnr(dec, blocks, 7)
        print(name, dec.shape, len(raw), "bytes")
    for name in TGA_REFUSED:
        raw = tga_refused(name)
        with open(os.path.join(HERE, name + ".tga"), "wb") as f:
            f.write(raw)
        assert ref.load_tga(raw) is None, name
        manifest["tga"][name] = {"file_sha256": hashlib.sha256(raw).hexdigest(), "refused": True}
        print(name, "refused")


# Uncompressed KTX inputs as FasTC's tc loads them (ImageLoaderKTX): name ->
# (image, integer byte order, key/value block, mipmap levels, glType,
# trailing bytes). FasTC reads the first two and refuses the next three;
# the last is a compressed (BPTC) file, which it loads as blocks.
KTX_IN = {
    "ktxin_le": ("tile_mix(14, 20, 12)", "<", True, 1, 0x1400, b""),
    "ktxin_be": ("tile_mix_radial_alpha(15, 16, 8, 7, 7)", ">", False, 1, 0x1400, b""),
    "ktxin_mips2": ("tile_mix(16, 8, 8)", "<", True, 2, 0x1400, b""),
    "ktxin_trailing": ("tile_mix(17, 8, 8)", "<", True, 1, 0x1400, b"\0\0\0\0"),
    "ktxin_ubyte": ("tile_mix(18, 8, 8)", "<", True, 1, 0x1401, b""),
}


def ktx_rgba_file(img: np.ndarray, order: str, kv: bool, mips: int, gl_type: int, tail: bytes) -> bytes:
    """An uncompressed RGBA8 KTX file laid out as FasTC's ImageWriterKTX
    writes one (IO/src/ImageWriterKTX.cpp:116-123, 127-160), with the given
    integer byte order, mipmap count, glType and trailing bytes."""
    h, w = img.shape[:2]
    kvb = b""
    if kv:
        body = b"KTXorientation\0S=r,T=d\0"
        kvb = struct.pack(order + "I", len(body)) + body
        kvb += b"K" * (-len(kvb) % 4)
    words = (0x04030201, gl_type, 1, 0x1908, 0x8058, 0x1908, w, h, 0, 0, 1, mips, len(kvb))
    ident = bytes([0xAB, 0x4B, 0x54, 0x58, 0x20, 0x31, 0x31, 0xBB, 0x0D, 0x0A, 0x1A, 0x0A])
    return (ident + struct.pack(order + "13I", *words) + kvb + struct.pack(order + "I", w * h * 4) +
            np.ascontiguousarray(img).tobytes() + tail)


def make_ktx_in(ref, manifest):
    manifest["ktx_in"] = {}
    files = {name: ktx_rgba_file(make(expr), *rest) for name, (expr, *rest) in KTX_IN.items()}
    bptc = np.fromfile(os.path.join(HERE, "tile_q0.bin"), np.uint8)
    from fastc_gb300 import imageio
    files["ktxin_compressed"] = imageio.ktx_bytes(bptc, 128, 128)
    for name, raw in files.items():
        with open(os.path.join(HERE, name + ".ktx"), "wb") as f:
            f.write(raw)
        got = ref.load_ktx(raw)
        e = {"file_sha256": hashlib.sha256(raw).hexdigest()}
        if got is None:
            e["refused"] = True
        elif isinstance(got, str):
            e["compressed"] = True
        else:
            e.update(width=int(got.shape[1]), height=int(got.shape[0]), decoded_sha256=sha(got))
            blocks = ref.compress(got, steps=0)  # what `tc -q 0` makes of the file
            e.update(q0_blocks_sha256=sha(blocks), q0_tc_psnr=ref.tc_psnr(got, blocks, 7))
        manifest["ktx_in"][name] = e
        print(name, e)


def dxt_random_blocks(w: int, h: int, fmt: int, seed: int) -> np.ndarray:
    n = ((w + 3) // 4) * ((h + 3) // 4) * (8 if fmt == 1 else 16)
    return np.random.default_rng(seed).integers(0, 256, n, dtype=np.uint8)


def make(expr: str) -> np.ndarray:
    return eval("synth." + expr, {"synth": synth})


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def parse_stats_log(text: str, nblocks: int):
    """The per-block statistics of a CompressWithStats log, as arrays."""
    path = np.full(nblocks, -1, np.int8)
    mode = np.full(nblocks, -1, np.int8)
    est = np.full((nblocks, 8), np.nan)
    err = np.full((nblocks, 8), np.nan)
    shapes = {2: ([], []), 3: ([], [])}  # (block index, estimate) of each improving shape
    names = ["Zero", "One", "Two", "Three", "Four", "Five", "Six", "Seven"]
    for line in text.splitlines():
        idx, rest = line.split(": ", 1)
        stat, val = rest.split(" -- ")
        i, stat = int(idx), stat[len("BlockStat_"):]
        if stat == "Path":
            path[i] = int(val)
        elif stat == "Mode":
            mode[i] = int(val)
        elif stat in ("TwoShapeEstimate", "ThreeShapeEstimate"):
            k = 2 if stat.startswith("Two") else 3
            shapes[k][0].append(i)
            shapes[k][1].append(float(val))
        else:
            m = names.index(stat[4:-8] if stat.endswith("Estimate") else stat[4:-5])
            (est if stat.endswith("Estimate") else err)[i, m] = float(val)
    return dict(path=path, mode=mode, estimate=est, error=err,
                two_block=np.array(shapes[2][0], np.int32), two=np.array(shapes[2][1]),
                three_block=np.array(shapes[3][0], np.int32), three=np.array(shapes[3][1]))


def make_stats(ref, manifest):
    manifest["stats"] = {}
    for name, (expr, steps, seed) in STATS.items():
        img = make(expr)
        blocks, log = ref.compress_stats(img, steps=steps, seed=seed)
        blocks.tofile(os.path.join(HERE, name + ".bin"))
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            **parse_stats_log(log, len(blocks) // 16))
        manifest["stats"][name] = {
            "image": expr, "steps": steps, "lcg_seed": seed, "input_sha256": sha(img),
            "blocks_sha256": sha(blocks),
            "log_sha256": hashlib.sha256(log.encode()).hexdigest(), "log_bytes": len(log),
        }
        print(name, len(blocks) // 16, "blocks,", len(log), "log bytes")


def _full_size_one(args):
    """One (case, seed) of the full-size fixtures, in a worker process (the
    reference's LCG seed is process-global, so each seed gets its own)."""
    name, expr, steps, seed = args
    ref, port = O.Reference(), O.Port()
    img = make(expr)
    blocks = ref.compress(img, steps=steps, seed=seed)
    dec = ref.decompress(blocks, img.shape[1], img.shape[0])
    return name, seed, port.psnr(img, dec), port.block_sse(img, dec).astype(np.float32)


def make_full_size(manifest, workers):
    import multiprocessing as mp

    work = [(name, expr, steps, s) for name, (expr, steps, seeds) in FULL_SIZE.items() for s in seeds]
    with mp.get_context("spawn").Pool(workers) as pool:
        res = pool.map(_full_size_one, work, chunksize=1)
    manifest["full_size"] = {}
    for name, (expr, steps, seeds) in FULL_SIZE.items():
        rows = sorted((r for r in res if r[0] == name), key=lambda r: seeds.index(r[1]))
        sse = np.stack([r[3] for r in rows]).astype(np.float64)
        # per-block SSE on a log scale, 1/1024 of an octave (0.07 %) per step:
        # the tests compare ratios against a 1 % bar
        np.savez_compressed(os.path.join(HERE, name + "_sse.npz"),
                            log2q=np.round(1024 * np.log2(sse + 16)).astype(np.uint16))
        manifest["full_size"][name] = {"image": expr, "steps": steps, "lcg_seeds": seeds,
                                       "input_sha256": sha(make(expr)),
                                       "psnr": [r[2] for r in rows],
                                       "sse_total": [float(x) for x in sse.sum(1)],
                                       "sse_encoding": "log2q = round(1024 * log2(sse + 16)), uint16"}
        print(name, [r[2] for r in rows])


def make_dxt(ref, manifest):
    manifest["dxt"] = {}
    for name, (expr, fmt) in DXT.items():
        img = make(expr)
        blocks = ref.dxt_compress(img, fmt == 5)
        blocks.tofile(os.path.join(HERE, name + ".bin"))
        dec = ref.dxt_decompress(blocks, img.shape[1], img.shape[0], fmt == 5)
        manifest["dxt"][name] = {"image": expr, "format": fmt, "input_sha256": sha(img),
                                 "blocks_sha256": sha(blocks), "decoded_sha256": sha(dec)}
        print(name, len(blocks), "bytes")
    for name, (w, h, fmt, seed) in DXT_DECODE.items():
        blocks = dxt_random_blocks(w, h, fmt, seed)
        dec = ref.dxt_decompress(blocks, w, h, fmt == 5)
        manifest["dxt"][name] = {"width": w, "height": h, "format": fmt, "rng_seed": seed,
                                 "blocks_sha256": sha(blocks), "decoded_sha256": sha(dec)}
        print(name)


def _ktx_one(args):
    """One KTX fixture, in a fresh worker process."""
    name, blocks, w, h, fmt = args
    return name, O.Reference().ktx(blocks, w, h, fmt)


def make_tc(ref, manifest):
    """What FasTC's tc prints and writes after the encode: its PSNR line for
    every fixture with an image (Image::ComputePSNR over FasTC's decoder),
    and the KTX files of KTX."""
    import multiprocessing as mp

    for group, fmt_of in (("cases", lambda e: 7), ("dxt", lambda e: e["format"])):
        for name, e in manifest[group].items():
            if "image" not in e:
                continue
            img = make(e["image"])
            blocks = np.fromfile(os.path.join(HERE, name + ".bin"), np.uint8)
            e["tc_psnr"] = ref.tc_psnr(img, blocks, fmt_of(e))
            print(name, "tc PSNR", e["tc_psnr"])
    work = []
    for name, (src, fmt) in KTX.items():
        e = manifest["cases" if fmt == 7 else "dxt"][src]
        h, w = make(e["image"]).shape[:2]
        work.append((name, np.fromfile(os.path.join(HERE, src + ".bin"), np.uint8), w, h, fmt))
    with mp.get_context("spawn").Pool(1, maxtasksperchild=1) as pool:
        files = dict(pool.map(_ktx_one, work, chunksize=1))
    manifest["ktx"] = {}
    for (name, _, w, h, fmt), (src, _) in zip(work, KTX.values()):
        raw = files[name]
        manifest["ktx"][name] = {"blocks": src, "format": fmt, "width": w, "height": h,
                                 "bytes": len(raw), "header_hex": raw[:96].hex(),
                                 "sha256": hashlib.sha256(raw).hexdigest()}
        print(name, len(raw), "bytes")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=O.DEFAULT_REFERENCE)
    ap.add_argument("--stats-only", action="store_true",
                    help="only (re)write the CompressWithStats fixtures")
    ap.add_argument("--full-size-only", action="store_true",
                    help="only (re)write the full-size PSNR / per-block SSE fixtures")
    ap.add_argument("--dxt-only", action="store_true",
                    help="only (re)write the DXT1 / DXT5 fixtures")
    ap.add_argument("--tc-only", action="store_true",
                    help="only (re)write tc's PSNR values and the KTX and TGA fixtures")
    ap.add_argument("--workers", type=int, default=6)
    args = ap.parse_args()
    if not O.build_ref(args.reference):
        sys.exit("FasTC checkout not found; cannot regenerate fixtures")
    ref = O.Reference()
    if args.stats_only or args.full_size_only or args.dxt_only or args.tc_only:
        with open(os.path.join(HERE, "manifest.json")) as f:
            manifest = json.load(f)
        if args.stats_only:
            make_stats(ref, manifest)
        elif args.dxt_only:
            make_dxt(ref, manifest)
            make_tc(ref, manifest)
        elif args.tc_only:
            make_tc(ref, manifest)
            make_tga(ref, manifest)
            make_ktx_in(ref, manifest)
        else:
            make_full_size(manifest, args.workers)
        with open(os.path.join(HERE, "manifest.json"), "w") as f:
            json.dump(manifest, f, indent=1, sort_keys=True)
        return
    manifest = {"cases": {}, "quality": {}}
    for name, (expr, steps, metric, seed) in CASES.items():
        img = make(expr)
        blocks = ref.compress(img, steps=steps, metric=metric, seed=seed)
        blocks.tofile(os.path.join(HERE, name + ".bin"))
        dec = ref.decompress(blocks, img.shape[1], img.shape[0])
        manifest["cases"][name] = {
            "image": expr, "steps": steps, "metric": metric, "lcg_seed": seed,
            "input_sha256": sha(img), "blocks_sha256": sha(blocks), "decoded_sha256": sha(dec),
        }
        print(name, len(blocks) // 16, "blocks")
    port = O.Port()
    for name, (expr, steps, seeds) in QUALITY.items():
        img = make(expr)
        psnrs, sses = [], []
        for s in seeds:
            blocks = ref.compress(img, steps=steps, seed=s)
            dec = ref.decompress(blocks, img.shape[1], img.shape[0])
            psnrs.append(port.psnr(img, dec))
            sses.append(port.block_sse(img, dec))
        np.save(os.path.join(HERE, name + "_sse.npy"), np.stack(sses).astype(np.float32))
        manifest["quality"][name] = {"image": expr, "steps": steps, "lcg_seeds": seeds,
                                     "input_sha256": sha(img), "psnr": psnrs}
        print(name, psnrs)
    sel_img = make("tile_mix(11, 128, 128)")
    sel = np.array([ref.box_selection(px) for px in synth.blocks_of(sel_img)], dtype=np.uint32)
    np.save(os.path.join(HERE, "box_selection.npy"), sel)
    manifest["box_selection"] = {"image": "tile_mix(11, 128, 128)", "input_sha256": sha(sel_img)}
    o7, o6 = ref.tables()
    np.savez(os.path.join(HERE, "endpoint_tables.npz"), opt7=o7, opt6=o6)
    make_stats(ref, manifest)
    make_dxt(ref, manifest)
    make_tc(ref, manifest)
    make_tga(ref, manifest)
    make_ktx_in(ref, manifest)
    make_full_size(manifest, args.workers)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
