"""Recipe for the reference's own CUDA extension (test infrastructure only).

torchhull's CUDA sources (``src/torchhull/_C/src/*.{cpp,cu}``, the headers in
``_C/include/torchhull`` and ``_C/python/bindings.cpp``) are compiled
**unmodified** with ``torch.utils.cpp_extension`` for sm_103a. The two
libraries its CMake build fetches over the network (glm 1.0.1 and stdgpu
d7c07d05, ``_C/CMakeLists.txt:26-60``) are replaced by the project-written
stand-ins under ``oracle/ref_shims/`` (the vector and hash-map surface those
sources touch); charonload, its build driver, is replaced by this script.

Two steps, because the GPU machine is a different architecture and has no
copy of the reference tree:

* ``stage()`` (only where the reference tree exists) copies those sources,
  byte for byte, into ``oracle/_ref/src/``. ``oracle/_ref/`` is git-ignored:
  the copy never enters the repository's history; it only travels with the
  working tree so the other machine can compile it.
* ``build()`` compiles ``oracle/_ref/src/`` into ``oracle/_ref/build/`` as the
  Python module ``torchhull_ref_C`` (the reference's ``_c_torchhull``).

The module is used by the parity tests (the reference build against this
library's CUDA path and against the CPU oracle) and by ``bench.py``'s
reference-CUDA timing leg. Nothing in the product imports it.
"""

from __future__ import annotations

import filecmp
import os
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_TREE = Path(os.environ.get("TH_REFERENCE_TREE", "/root/reference")) / "src" / "torchhull" / "_C"
STAGE = HERE / "_ref" / "src"
BUILD = HERE / "_ref" / "build"
SHIMS = HERE / "ref_shims"
MODULE = "torchhull_ref_C"

# Relative to the reference's _C directory.
_SOURCES = [
    "src/gaussian_blur.cpp",
    "src/gaussian_blur_cuda.cu",
    "src/io.cpp",
    "src/marching_cubes.cpp",
    "src/marching_cubes_cuda.cu",
    "src/visual_hull.cpp",
    "src/visual_hull_cuda.cu",
    "python/bindings.cpp",
]
_OTHER = ["src/marching_cubes_table.h"]
_HEADER_DIR = "include/torchhull"


def staged() -> bool:
    return all((STAGE / s).exists() for s in _SOURCES)


def stage() -> bool:
    """Copies the reference sources into oracle/_ref/src when the reference tree is present."""
    if not REF_TREE.is_dir():
        return staged()
    files = _SOURCES + _OTHER + [f"{_HEADER_DIR}/{p.name}" for p in sorted((REF_TREE / _HEADER_DIR).iterdir())]
    for rel in files:
        src = REF_TREE / rel
        dst = STAGE / rel
        dst.parent.mkdir(parents=True, exist_ok=True)
        if not dst.exists() or not filecmp.cmp(src, dst, shallow=False):
            shutil.copyfile(src, dst)
    return True


def build(verbose: bool = False):
    """Compiles the staged reference sources; returns the module, or None when nothing is staged."""
    stage()
    if not staged():
        return None
    import torch.utils.cpp_extension as ce

    BUILD.mkdir(parents=True, exist_ok=True)
    os.environ.setdefault("MAX_JOBS", str(max(1, min(16, os.cpu_count() or 1))))
    common = ["-O3", "-DNDEBUG", "-D__CUDA_NO_HALF_OPERATORS__"]
    return ce.load(
        name=MODULE,
        sources=[str(STAGE / s) for s in _SOURCES],
        extra_include_paths=[str(STAGE / "include"), str(SHIMS)],
        extra_cflags=common,
        extra_cuda_cflags=[
            "-gencode",
            "arch=compute_103a,code=sm_103a",
            "--extended-lambda",
            "--expt-relaxed-constexpr",
            *common,
        ],
        build_directory=str(BUILD),
        with_cuda=True,
        verbose=verbose,
    )


def load():
    """The built module, or None when it has not been staged or built on this machine."""
    if not staged():
        return None
    try:
        return build(verbose=False)
    except Exception as exc:  # a failed build is reported by the caller
        print(f"reference build failed: {exc}", file=sys.stderr)
        return None


if __name__ == "__main__":
    mod = build(verbose=True)
    print("reference extension:", getattr(mod, "__file__", None))
