"""tc-compatible command line: compress an image to BC7 (or DXT1 / DXT5) on
the GPU.

    python -m fastc_gb300.tc [-f BPTC|DXT1|DXT5] [-q N] [-n N] [-d OUT] [-nd] [-s WxH] IMAGE

Mirrors FasTC's CLTool (CLTool/src/tc.cpp): BPTC at quality -q (annealing
steps, default 50) or, with -f, DXT1 / DXT5 (quality has no effect, as in
FasTC), the image zero-padded to whole blocks, "PSNR: %.3f"
computed as FasTC's Image::ComputePSNR (alpha-premultiplied RGB, peak
3*255^2) on the decoded blocks (for a padded image, FasTC's message that
the sizes differ instead), and the output written to -d (or
<basename>-bptc.png, -dxt1.png, -dxt5.png): a .ktx name stores the
compressed blocks in FasTC's KTX layout, a .png name the decoded image. -nd writes nothing; -n N repeats the
compression; "Compression time: %.3f ms" (the mean) is printed before the PSNR, as FasTC prints it. Options that choose host threading (-t,
-j, -a, -simd) are accepted and have no effect: the work is distributed on
the GPU. -l runs CompressWithStats with a log stream and writes FasTC's
per-block log to <basename>.log (for DXT the log stays empty, as FasTC's
does: it has no logging DXT encoder); ETC1 and PVRTC are refused.
Inputs: PNG (8-bit), TGA and uncompressed KTX (as FasTC's loaders read them),
.npy RGBA8 arrays, raw RGBA (.rgba/.raw with -s WxH).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np


def usage(out=sys.stderr) -> None:
    print(__doc__.strip(), file=out)


def basename(path: str) -> str:
    """ExtractBasename (CLTool/src/tc.cpp:57-79): the file name without its
    directory and without everything from its first dot."""
    return os.path.basename(path).split(".", 1)[0]


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    if not argv:
        usage()
        return 1
    quality, repeats, out_name, write_out, save_log, fmt = 50, 1, "", True, False, "BPTC"
    width = height = 0
    i = 0
    while i < len(argv) and argv[i].startswith("-"):
        opt = argv[i]
        if opt in ("-h", "--help"):
            usage(sys.stdout)
            return 0
        if opt in ("-q", "-n", "-t", "-j", "-s", "-d", "-f"):
            if i + 1 >= len(argv):
                usage()
                return 1
            val = argv[i + 1]
            if opt == "-q":
                quality = int(val)
            elif opt == "-n":
                repeats = max(1, int(val))
            elif opt == "-s":
                width, height = (int(x) for x in val.lower().split("x"))
            elif opt == "-d":
                out_name = val
            elif opt == "-f":
                # FasTC's names (CLTool/src/tc.cpp:121-148); a name it does
                # not know leaves the format as it was
                if val in ("PVRTC", "PVRTCLib", "ETC1"):
                    print(f"format {val} is not supported: this build encodes BPTC, DXT1 and DXT5",
                          file=sys.stderr)
                    return 1
                if val in ("DXT1", "DXT5"):
                    fmt = val
                elif val == "BPTCLib":
                    fmt = "BPTC"
            i += 2
            continue
        if opt == "-nd":
            write_out = False
        elif opt == "-l":
            save_log = True
        elif opt not in ("-a", "-v", "-simd"):
            usage()
            return 1
        i += 1
    if i >= len(argv) or quality < 0:
        usage()
        return 1
    path = argv[i]

    from . import dxt, imageio
    from .bptc import (CompressionFormat, CompressionJob, CompressionSettings, compress, compress_with_stats,
                       decompress, psnr)

    src = imageio.load_image(path, width, height)
    img = imageio.pad_to_blocks(src)
    h, w = img.shape[:2]
    padded = img.shape != src.shape
    if padded:  # CompressImage's warning (Core/src/TexComp.cpp:157-158, 383)
        print("TexComp -- WARNING - Image size is not a multiple of block size. Padding with zeros...",
              file=sys.stderr)
    cf = CompressionFormat[fmt]
    blocks = np.zeros(w * h // (2 if cf == CompressionFormat.DXT1 else 1), dtype=np.uint8)
    settings = CompressionSettings(num_simulated_annealing_steps=quality)
    logs = []
    t0 = time.perf_counter()
    for _ in range(repeats):
        job = CompressionJob(img, blocks, w, h, format=cf)
        if cf != CompressionFormat.BPTC:
            dxt.compress_dxt_jobs([job])
        elif save_log:  # the log stream sees every compression, as FasTC's does
            logs.append(compress_with_stats(job, settings))
        else:
            compress(job, settings)
    dt = (time.perf_counter() - t0) / repeats
    # CompressImageData reports the mean time of the -n compressions on
    # every run (Core/src/TexComp.cpp:516-517)
    print(f"Compression time: {dt * 1e3:.3f} ms")
    if save_log:
        with open(basename(path) + ".log", "w") as f:
            f.write("".join(logs))
    if padded:
        # the compressed image has the padded size, so tc compares nothing
        # (CLTool/src/tc.cpp:297-299)
        print("Cannot compute image metrics: compressed and uncompressed dimensions differ.",
              file=sys.stderr)
    else:
        if cf == CompressionFormat.BPTC:
            db = psnr(blocks, img, w, h)
        else:
            db = dxt.psnr(blocks, img, w, h, cf)
        print(f"PSNR: {db:.3f}")
    if write_out:
        if not out_name:
            out_name = basename(path) + ("-bptc.png" if cf == CompressionFormat.BPTC else f"-{fmt.lower()}.png")
        with open(out_name, "wb") as f:
            if out_name.endswith(".ktx"):
                f.write(imageio.ktx_bytes(blocks, w, h, fmt))
            elif cf == CompressionFormat.BPTC:
                f.write(imageio.png_bytes(decompress(blocks, w, h)))
            else:
                f.write(imageio.png_bytes(dxt.decompress(blocks, w, h, cf)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
