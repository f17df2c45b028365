"""Build recipe: CUDA library (C ABI) and the thin torch extension, in-tree.

* ``csrc/*.cu`` -> ``_build/obj/*.o`` with nvcc for sm_103a only (parallel),
  linked into ``_build/libtorchhull_gb300.so`` (static cudart, C ABI of
  ``include/torchhull_gb300.h``).
* ``csrc/torch_ext.cpp`` -> ``_build/ext/torchhull_gb300_C*.so`` through
  torch.utils.cpp_extension, linked against the library above.

Everything lands under ``torchhull_gb300/_build/`` (git-ignored); nothing is
installed into site-packages.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
OBJ = BUILD / "obj"
EXT_DIR = BUILD / "ext"
LIB = BUILD / "libtorchhull_gb300.so"
EXT_NAME = "torchhull_gb300_C"
CU_SOURCES = ["sat.cu", "carve.cu", "batch.cu", "mesh.cu", "mc.cu", "wire.cu", "blur.cu", "blur_noalloc.cu", "capi.cu"]
HEADERS = ["th_common.cuh", "th_hull.cuh", "th_classify.cuh", "th_batch.cuh", "th_mc.cuh", "th_internal.h", "mc_tables.h"]

NVCC_FLAGS = [
    "-gencode",
    "arch=compute_103a,code=sm_103a",
    "-lineinfo",
    "-O3",
    "-std=c++20",
    "-Xcompiler",
    "-fPIC",
    "-Xptxas",
    "-warn-spills",
]


def _defines() -> list[str]:
    """Extra preprocessor definitions from TH_NVCC_DEFINES (space-separated NAME=VALUE), for tuning builds."""
    return [f"-D{d}" for d in os.environ.get("TH_NVCC_DEFINES", "").split() if d]


def _nvcc() -> str:
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda_home) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found")
    return found


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: str) -> Path:
    out = OBJ / (Path(src).stem + ".o")
    deps = [CSRC / src] + [CSRC / h for h in HEADERS] + [PKG.parent / "include" / "torchhull_gb300.h"]
    if _stale(out, deps):
        cmd = [_nvcc(), *NVCC_FLAGS, *_defines(), "-c", str(CSRC / src), "-o", str(out)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return out


def build_library(verbose: bool = False) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    # objects built with other definitions are stale
    stamp = OBJ / "defines.txt"
    defines = " ".join(_defines())
    if not stamp.exists() or stamp.read_text() != defines:
        for o in OBJ.glob("*.o"):
            o.unlink()
        stamp.write_text(defines)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(CU_SOURCES)) as ex:
        objs = list(ex.map(_compile, CU_SOURCES))
    if _stale(LIB, objs):
        cmd = [_nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", str(LIB), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


def build_extension(verbose: bool = False):
    import torch.utils.cpp_extension as ce

    EXT_DIR.mkdir(parents=True, exist_ok=True)
    return ce.load(
        name=EXT_NAME,
        sources=[str(CSRC / "torch_ext.cpp")],
        extra_cflags=["-O2"],
        extra_ldflags=[f"-L{BUILD}", "-ltorchhull_gb300", f"-Wl,-rpath,{BUILD}"],
        extra_include_paths=[str(PKG.parent / "include")],
        build_directory=str(EXT_DIR),
        with_cuda=True,
        verbose=verbose,
    )


def build(verbose: bool = False) -> None:
    """Builds both artefacts; the extension build may run while nvcc compiles."""
    with concurrent.futures.ThreadPoolExecutor(max_workers=1) as ex:
        lib_future = ex.submit(build_library, verbose)
        lib_future.result()
    build_extension(verbose)


def extension_path() -> Path | None:
    hits = sorted(EXT_DIR.glob(f"{EXT_NAME}*.so"))
    return hits[0] if hits else None


if __name__ == "__main__":
    build(verbose=True)
