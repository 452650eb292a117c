import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def manifest_multi():
    """Frames of several outputs, one input hash per output."""
    with open(os.path.join(GOLDEN, "manifest_multi.json")) as f:
        return json.load(f)


def read_frame(case):
    with open(os.path.join(GOLDEN, case + ".zl"), "rb") as f:
        return f.read()


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the GPU library; requires a CUDA device."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from openzl_gb300 import build

    build.build()
    import openzl_gb300

    return openzl_gb300.library()
