"""CPU checks of the C ABI library: it loads and exports every declared symbol."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions() -> list[str]:
    names = []
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w\*\s]+?\b(th_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from torchhull_gb300 import build

    if not build.LIB.exists():
        pytest.skip("library not built")
    return ctypes.CDLL(str(build.LIB))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("th_visual_hull", "th_visual_hull_export", "th_visual_hull_export_candidates",
                     "th_gaussian_blur", "th_context_create", "th_context_destroy"):
        assert required in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(lib):
    lib.th_status_string.restype = ctypes.c_char_p
    lib.th_status_string.argtypes = [ctypes.c_int]
    assert lib.th_status_string(0) == b"ok"
    assert lib.th_status_string(2) == b"unsupported dtype"


def test_context_without_gpu_reports_no_device(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ctx = ctypes.c_void_p()
    lib.th_context_create.restype = ctypes.c_int
    assert lib.th_context_create(0, ctypes.byref(ctx)) == 6  # TH_ERR_NO_DEVICE
    assert not ctx.value


def test_product_does_not_use_the_oracle():
    """The package neither imports, loads nor includes anything from oracle/."""
    pattern = re.compile(r"(^\s*(from|import)\s+oracle\b)|liboracle|oracle\.(h|cpp)|oracle/", re.M)
    for path in (ROOT / "torchhull_gb300").rglob("*"):
        if path.suffix in (".py", ".cu", ".cuh", ".cpp", ".h") and "_build" not in path.parts:
            assert not pattern.search(path.read_text()), path
