"""The C++ drop-in (fastc_gb300/csrc/fastc_bptc_shim.cpp) compiled against
FasTC's own headers and linked with the library and the FasTC Base sources
it uses, the way a maintainer would swap FasTC's BPTC encoder: a
FasTC-style caller builds and links, and without a GPU each entry point
aborts with the C ABI's message instead of returning silently (FasTC's
functions return void). CompressWithStats
without a log stream encodes like Compress (as in FasTC); with one it runs
the logging encoder (fastc_bc7_compress_stats), which needs the device too.
Needs the FasTC checkout, so it runs in the x86 container only; objects go
under oracle/_ref/."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

import oracle.oracle as O

CALLER = r"""
#include <cstring>
#include <iostream>
#include <vector>

#include "FasTC/BPTCCompressor.h"
#include "FasTC/CompressionJob.h"

int main(int argc, char **argv) {
  std::vector<unsigned char> in(16 * 16 * 4, 7), out(16 * 16, 0);
  FasTC::CompressionJob cj(FasTC::eCompressionFormat_BPTC, in.data(), out.data(), 16, 16);
  BPTCC::CompressionSettings s;
  s.m_NumSimulatedAnnealingSteps = 8;
  const char *what = argc > 1 ? argv[1] : "";
  if (!std::strcmp(what, "compress")) BPTCC::Compress(cj, s);
  if (!std::strcmp(what, "stats_null")) BPTCC::CompressWithStats(cj, NULL, s);
  if (!std::strcmp(what, "stats_log")) BPTCC::CompressWithStats(cj, &std::cout, s);
  return 0;
}
"""


@pytest.fixture(scope="module")
def shim_exe(bc7lib):
    if not shutil.which("g++") or not O.build_ref():
        pytest.skip("FasTC checkout or g++ not available")
    ref = O.DEFAULT_REFERENCE
    out = os.path.join(ROOT, "oracle", "_ref", "shimtest")
    os.makedirs(out, exist_ok=True)
    src = os.path.join(out, "caller.cpp")
    with open(src, "w") as f:
        f.write(CALLER)
    exe = os.path.join(out, "caller")
    libdir = os.path.join(ROOT, "fastc_gb300", "lib")
    cmd = ["g++", "-std=c++11", "-O1", "-w",
           "-I" + os.path.join(ROOT, "oracle", "_ref", "gen"),
           "-I" + os.path.join(ref, "Base", "include"),
           "-I" + os.path.join(ref, "BPTCEncoder", "include"),
           "-I" + os.path.join(ROOT, "include"),
           src, os.path.join(ROOT, "fastc_gb300", "csrc", "fastc_bptc_shim.cpp"),
           os.path.join(ref, "Base", "src", "CompressionJob.cpp"),
           os.path.join(ref, "Base", "src", "Pixel.cpp"),
           "-L" + libdir, "-lfastc_bc7", "-Wl,-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def _run(exe, what):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    return subprocess.run([exe, what], capture_output=True, text=True, env=env, timeout=120)


def test_shim_builds_against_fastc_headers(shim_exe):
    assert _run(shim_exe, "nothing").returncode == 0


def test_compress_fails_loudly_without_a_device(shim_exe):
    r = _run(shim_exe, "compress")
    assert r.returncode != 0
    assert "fastc_bc7: BPTCC::Compress failed" in r.stderr


def test_compress_with_stats_without_a_log_encodes_like_compress(shim_exe):
    r = _run(shim_exe, "stats_null")
    assert r.returncode != 0
    assert "fastc_bc7: BPTCC::Compress failed" in r.stderr  # it went to Compress


def test_compress_with_stats_with_a_log_runs_the_logging_encoder(shim_exe):
    r = _run(shim_exe, "stats_log")
    assert r.returncode != 0
    assert "fastc_bc7: BPTCC::CompressWithStats failed" in r.stderr
    assert "unsupported" not in r.stderr.lower()  # it reached the device path


DXT_CALLER = r"""
#include <cstring>
#include <vector>

#include "FasTC/CompressionJob.h"
#include "FasTC/DXTCompressor.h"

int main(int argc, char **argv) {
  std::vector<unsigned char> in(16 * 16 * 4, 7), out(16 * 16, 0), dec(16 * 16 * 4, 0);
  FasTC::CompressionJob cj(FasTC::eCompressionFormat_DXT5, in.data(), out.data(), 16, 16);
  FasTC::DecompressionJob dj(FasTC::eCompressionFormat_DXT1, out.data(), dec.data(), 16, 16);
  const char *what = argc > 1 ? argv[1] : "";
  if (!std::strcmp(what, "dxt5")) DXTC::CompressImageDXT5(cj);
  if (!std::strcmp(what, "dxt1_decode")) DXTC::DecompressDXT1(dj);
  return 0;
}
"""


@pytest.fixture(scope="module")
def dxt_shim_exe(bc7lib):
    """The DXT drop-in (fastc_gb300/csrc/fastc_dxt_shim.cpp) against FasTC's
    DXTEncoder headers, as a maintainer would swap FasTC's DXT library."""
    if not shutil.which("g++") or not O.build_ref():
        pytest.skip("FasTC checkout or g++ not available")
    ref = O.DEFAULT_REFERENCE
    out = os.path.join(ROOT, "oracle", "_ref", "shimtest")
    os.makedirs(out, exist_ok=True)
    src = os.path.join(out, "dxt_caller.cpp")
    with open(src, "w") as f:
        f.write(DXT_CALLER)
    exe = os.path.join(out, "dxt_caller")
    libdir = os.path.join(ROOT, "fastc_gb300", "lib")
    cmd = ["g++", "-std=c++11", "-O1", "-w",
           "-I" + os.path.join(ROOT, "oracle", "_ref", "gen"),
           "-I" + os.path.join(ref, "Base", "include"),
           "-I" + os.path.join(ref, "DXTEncoder", "include"),
           "-I" + os.path.join(ROOT, "include"),
           src, os.path.join(ROOT, "fastc_gb300", "csrc", "fastc_dxt_shim.cpp"),
           os.path.join(ref, "Base", "src", "CompressionJob.cpp"),
           os.path.join(ref, "Base", "src", "Pixel.cpp"),
           "-L" + libdir, "-lfastc_bc7", "-Wl,-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def test_dxt_shim_builds_against_fastc_headers(dxt_shim_exe):
    assert _run(dxt_shim_exe, "nothing").returncode == 0


@pytest.mark.parametrize("what,where", [("dxt5", "CompressImageDXT5"), ("dxt1_decode", "DecompressDXT1")])
def test_dxt_entry_points_fail_loudly_without_a_device(dxt_shim_exe, what, where):
    r = _run(dxt_shim_exe, what)
    assert r.returncode != 0
    assert f"fastc_dxt: {where} failed" in r.stderr
