from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built extension")


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def th():
    import torchhull_gb300

    return torchhull_gb300


@pytest.fixture(scope="session")
def ref(cuda):
    """torchhull's own CUDA extension, built from its unmodified sources by oracle/ref_build.py.

    Skipped where the sources were not staged into oracle/_ref/src; a staged
    tree that fails to build is an error, not a skip.
    """
    from oracle import ref_build

    if not ref_build.staged():
        pytest.skip("reference sources not staged (oracle/_ref/src)")
    return ref_build.build(verbose=False)
