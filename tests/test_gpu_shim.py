"""The C++ drop-ins (fastc_gb300/csrc/fastc_bptc_shim.cpp and
fastc_dxt_shim.cpp) producing bytes on the GPU. A FasTC-style caller is
built against stand-in copies of FasTC's interface headers
(tests/stub_headers/FasTC: FasTC's class and function names and
signatures, nothing else), linked with the shims and libfastc_bc7.so, and
run: BPTCC::Compress at q0 gives FasTC's golden blocks, CompressWithStats
with a log stream gives FasTC's blocks and log text, CompressAtomic called
from two threads gives the library's batch result, Decompress gives
FasTC's decoded texels, and DXTC::CompressImageDXT1/5 and DecompressDXT5
give FasTC's DXT bytes."""
import hashlib
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_blocks, make_image

pytestmark = pytest.mark.gpu

CALLER = r"""
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <sstream>
#include <thread>
#include <vector>

#include "FasTC/BPTCCompressor.h"
#include "FasTC/DXTCompressor.h"

static std::vector<unsigned char> slurp(const char *p) {
  std::ifstream f(p, std::ios::binary);
  return std::vector<unsigned char>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

static void spit(const std::string &p, const void *d, size_t n) {
  std::ofstream f(p, std::ios::binary);
  f.write(static_cast<const char *>(d), (std::streamsize)n);
}

// op input width height output [arg]
int main(int argc, char **argv) {
  if (argc < 6) return 2;
  const std::string op = argv[1];
  std::vector<unsigned char> in = slurp(argv[2]);
  const uint32 w = (uint32)atoi(argv[3]), h = (uint32)atoi(argv[4]);
  const std::string outp = argv[5];
  const int arg = argc > 6 ? atoi(argv[6]) : 0;
  std::vector<unsigned char> out;
  if (op == "compress") {
    out.assign(w * h, 0);
    FasTC::CompressionJob cj(FasTC::eCompressionFormat_BPTC, in.data(), out.data(), w, h);
    BPTCC::CompressionSettings s;
    s.m_NumSimulatedAnnealingSteps = (uint32)arg;
    BPTCC::Compress(cj, s);
  } else if (op == "stats") {  // the job ends at the last block row
    out.assign(w * h, 0);
    FasTC::CompressionJob cj(FasTC::eCompressionFormat_BPTC, in.data(), out.data(), w, h, 0, 0, w, h - 4);
    BPTCC::CompressionSettings s;
    s.m_NumSimulatedAnnealingSteps = (uint32)arg;
    std::ostringstream log;
    BPTCC::CompressWithStats(cj, &log, s);
    const std::string t = log.str();
    spit(outp + ".log", t.data(), t.size());
  } else if (op == "atomic") {  // `arg` images of w x h, stacked
    out.assign((size_t)arg * w * h, 0);
    FasTC::CompressionJobList list((uint32)arg);
    for (int k = 0; k < arg; k++)
      list.AddJob(FasTC::CompressionJob(FasTC::eCompressionFormat_BPTC, in.data() + (size_t)k * w * h * 4,
                                        out.data() + (size_t)k * w * h, w, h));
    std::thread t1([&] { BPTCC::CompressAtomic(list); });
    std::thread t2([&] { BPTCC::CompressAtomic(list); });
    t1.join();
    t2.join();
    for (int k = 0; k < arg; k++)
      if (*list.GetFinishedFlag((uint32)k) != 1) return 3;
  } else if (op == "decompress") {
    out.assign((size_t)w * h * 4, 0);
    BPTCC::Decompress(FasTC::DecompressionJob(FasTC::eCompressionFormat_BPTC, in.data(), out.data(), w, h));
  } else if (op == "dxt1" || op == "dxt5") {
    out.assign(op == "dxt1" ? w * h / 2 : w * h, 0);
    FasTC::CompressionJob cj(op == "dxt1" ? FasTC::eCompressionFormat_DXT1 : FasTC::eCompressionFormat_DXT5,
                             in.data(), out.data(), w, h);
    if (op == "dxt1") DXTC::CompressImageDXT1(cj);
    else DXTC::CompressImageDXT5(cj);
  } else if (op == "dxt5_decode") {
    out.assign((size_t)w * h * 4, 0);
    DXTC::DecompressDXT5(FasTC::DecompressionJob(FasTC::eCompressionFormat_DXT5, in.data(), out.data(), w, h));
  } else {
    return 2;
  }
  spit(outp, out.data(), out.size());
  return 0;
}
"""


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def caller(bc7lib, tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("shim")
    src = d / "caller.cpp"
    src.write_text(CALLER)
    exe = str(d / "caller")
    libdir = os.path.join(ROOT, "fastc_gb300", "lib")
    csrc = os.path.join(ROOT, "fastc_gb300", "csrc")
    cmd = ["g++", "-std=c++11", "-O1", "-w", "-pthread", "-DHAS_ATOMICS",
           "-I" + os.path.join(ROOT, "tests", "stub_headers"), "-I" + os.path.join(ROOT, "include"),
           str(src), os.path.join(csrc, "fastc_bptc_shim.cpp"), os.path.join(csrc, "fastc_dxt_shim.cpp"),
           "-L" + libdir, "-lfastc_bc7", "-Wl,-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]

    def run(op, data, w, h, arg=None):
        inp = d / f"{op}.in"
        outp = d / f"{op}.out"
        np.ascontiguousarray(data, dtype=np.uint8).tofile(inp)
        args = [exe, op, str(inp), str(w), str(h), str(outp)] + ([str(arg)] if arg is not None else [])
        r = subprocess.run(args, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        res = np.fromfile(outp, dtype=np.uint8)
        log = (d / f"{op}.out.log").read_text() if op == "stats" else None
        return res, log

    return run


def test_compress_q0_gives_fasTC_blocks(caller, manifest):
    case = manifest["cases"]["c1_q0"]
    img = make_image(case["image"])
    blocks, _ = caller("compress", img, img.shape[1], img.shape[0], 0)
    assert np.array_equal(blocks, golden_blocks("c1_q0"))


def test_compress_q16_equals_the_library(caller, port):
    img = make_image("tile_mix(2, 64, 64)")
    blocks, _ = caller("compress", img, 64, 64, 16)
    assert np.array_equal(blocks, port.compress(img, steps=16, seed=0))


def test_compress_with_stats_gives_fasTC_blocks_and_log(caller, manifest):
    case = manifest["stats"]["tile_stats_q0"]
    img = make_image(case["image"])
    blocks, log = caller("stats", img, img.shape[1], img.shape[0], 0)
    h = img.shape[0]
    want = golden_blocks("tile_stats_q0")
    assert np.array_equal(blocks[:len(want)], want) and not blocks[len(want):].any()
    assert len(log) == case["log_bytes"]
    assert hashlib.sha256(log.encode()).hexdigest() == case["log_sha256"]
    assert h == 64


def test_compress_atomic_from_two_threads_equals_one_batch(caller):
    from fastc_gb300 import (WATERMARK_CONTINUE, CompressionJob, CompressionSettings, compress_jobs,
                             set_watermark_counter)

    imgs = [make_image(f"tile_mix({51 + k}, 64, 64)") for k in range(3)]
    blocks, _ = caller("atomic", np.stack(imgs), 64, 64, 3)
    # CompressAtomic runs FasTC's default settings with the process-wide
    # watermark counter, which starts at 0 in the caller
    set_watermark_counter(0)
    outs = [np.zeros(64 * 64, np.uint8) for _ in imgs]
    compress_jobs([CompressionJob(i, o, 64, 64) for i, o in zip(imgs, outs)],
                  CompressionSettings(num_simulated_annealing_steps=50, watermark_start=WATERMARK_CONTINUE))
    assert np.array_equal(blocks, np.concatenate(outs))


def test_decompress_gives_fasTC_texels(caller, manifest):
    case = manifest["cases"]["c1_q0"]
    img = make_image(case["image"])
    dec, _ = caller("decompress", golden_blocks("c1_q0"), img.shape[1], img.shape[0])
    assert sha(dec) == case["decoded_sha256"]


@pytest.mark.parametrize("name", ["dxt1_tile", "dxt5_tile", "dxt5_radial"])
def test_dxt_compress_gives_fasTC_blocks(caller, manifest, name):
    case = manifest["dxt"][name]
    img = make_image(case["image"])
    blocks, _ = caller("dxt1" if case["format"] == 1 else "dxt5", img, img.shape[1], img.shape[0])
    assert np.array_equal(blocks, golden_blocks(name))


def test_dxt5_decompress_gives_fasTC_texels(caller, manifest):
    case = manifest["dxt"]["dxt5_random_decode"]
    w, h = case["width"], case["height"]
    n = ((w + 3) // 4) * ((h + 3) // 4) * 16
    blocks = np.random.default_rng(case["rng_seed"]).integers(0, 256, n, dtype=np.uint8)
    dec, _ = caller("dxt5_decode", blocks, w, h)
    assert sha(dec) == case["decoded_sha256"]
