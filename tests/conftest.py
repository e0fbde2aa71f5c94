import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a); runs through the C ABI")


@pytest.fixture(scope="session")
def ylib():
    import yukawacolourednoise_gb300 as yk
    yk.lib()
    return yk


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a visible CUDA device")
    torch.cuda.set_device(0)
    return torch


def golden_files():
    return sorted(GOLDEN.glob("ref_*.npz"))
