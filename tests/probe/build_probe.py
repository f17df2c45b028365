"""Builds the test-only arithmetic probe (arith_probe.cu) into tests/probe/_build/.

The probe is not part of the library: only tests/test_gpu_hull.py loads it.
Compiled for sm_103a with nvcc's default flags (-fmad=true), like the
reference's own build, because it checks how nvcc treats the reference's
spelling of the world-coordinate expression.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "arith_probe.cu"
LIB = HERE / "_build" / "libarith_probe.so"


def build() -> Path:
    if LIB.exists() and LIB.stat().st_mtime > SRC.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(parents=True, exist_ok=True)
    nvcc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    cmd = [str(nvcc) if nvcc.exists() else (shutil.which("nvcc") or "nvcc"), "-gencode",
           "arch=compute_103a,code=sm_103a", "-O3", "-shared", "-Xcompiler", "-fPIC", "-o", str(LIB), str(SRC)]
    subprocess.run(cmd, check=True, capture_output=True)
    return LIB
