import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as O

    O.build_port()
    return O.Port()


@pytest.fixture(scope="session")
def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def golden_blocks(name: str) -> np.ndarray:
    return np.fromfile(os.path.join(GOLDEN, name + ".bin"), dtype=np.uint8)


def make_image(expr: str) -> np.ndarray:
    from fastc_gb300 import synth

    return eval("synth." + expr, {"synth": synth})


@pytest.fixture(scope="session")
def bc7lib():
    """The built C-ABI library (builds it if needed; no GPU required)."""
    from fastc_gb300 import _lib, build

    build.build()
    return _lib.load()


def cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(bc7lib):
    if not cuda_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    import torch

    torch.cuda.init()
    return torch.device("cuda:0")
