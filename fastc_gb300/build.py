"""Build the GB300 BC7 library in-tree with nvcc (sm_103a only).

    python -m fastc_gb300.build            # -> fastc_gb300/lib/libfastc_bc7.so

The encoder translation unit is compiled with -fmad=false (no FMA
contraction) and IEEE division/square root, which is what makes the float
arithmetic round exactly like FasTC's x86-64 build.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libfastc_bc7.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]
# (source, object name, extra flags). bc7_kernels.cu is compiled once per warp
# count of the warp-per-block encoder, one encode_kernel instantiation each,
# so that the four long compiles run in parallel.
SOURCES = [("bc7_kernels.cu", "bc7_kernels", []),
           ("bc7_kernels.cu", "bc7_wpb_w1", ["-DFASTC_WPB_WARPS=1"]),
           ("bc7_kernels.cu", "bc7_wpb_w2", ["-DFASTC_WPB_WARPS=2"]),
           ("bc7_kernels.cu", "bc7_wpb_w8", ["-DFASTC_WPB_WARPS=8"]),
           ("bc7_pipeline.cu", "bc7_pipeline", []),
           ("bc7_api.cu", "bc7_api", []),
           ("bc7_server.cu", "bc7_server", []),
           ("bc7_static.cu", "bc7_static", []),
           ("dxt.cu", "dxt", [])]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fastc_gb300")


def _compile(item, extra) -> str:
    src, name, flags = item
    obj = os.path.join(BUILD, name + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *flags, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def sources_newer_than(path: str) -> bool:
    if not os.path.exists(path):
        return True
    t = os.path.getmtime(path)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "fastc_bc7.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and not sources_newer_than(LIB):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
