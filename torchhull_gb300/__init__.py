"""GB300 (sm_103a) implementation of torchhull's visual-hull and blur path.

Drop-in for ``torchhull.visual_hull``, ``torchhull.visual_hull_with_candidate_voxels``,
``torchhull.sparse_visual_hull_field``, ``torchhull.marching_cubes``,
``torchhull.candidate_voxels_to_wireframes``, ``torchhull.store_curve_network``
and ``torchhull.gaussian_blur`` (the reference's whole public API): same
argument names, defaults, outputs and errors.  The work runs in hand-written
CUDA behind the C ABI of ``include/torchhull_gb300.h``; there is no CPU path,
and CPU tensors raise the reference's "No backend implementation" error.

Build once with ``python -c "import __graft_entry__ as g; g.build()"`` (or
``python -m torchhull_gb300.build``); importing an unbuilt tree raises
ImportError.
"""

from __future__ import annotations

import importlib.machinery
import importlib.util

import torch

from . import build as _build

__all__ = [
    "candidate_voxels_to_wireframes",
    "gaussian_blur",
    "integral_image",
    "marching_cubes",
    "sparse_visual_hull_field",
    "store_curve_network",
    "visual_hull",
    "visual_hull_blurred",
    "visual_hull_with_candidate_voxels",
]


def _load_extension():
    path = _build.extension_path()
    if path is None or not _build.LIB.exists():
        raise ImportError(
            "torchhull_gb300 CUDA extension is not built (expected under torchhull_gb300/_build/); "
            "run `python -m torchhull_gb300.build` first"
        )
    loader = importlib.machinery.ExtensionFileLoader(_build.EXT_NAME, str(path))
    spec = importlib.util.spec_from_file_location(_build.EXT_NAME, str(path), loader=loader)
    module = importlib.util.module_from_spec(spec)
    loader.exec_module(module)
    return module


_ext = None

# The names re-exported from the extension (the reference's public API plus
# the fused blur -> hull request of its second benchmark configuration).
_EXPORTS = (
    "visual_hull",
    "visual_hull_with_candidate_voxels",
    "gaussian_blur",
    "integral_image",
    "marching_cubes",
    "candidate_voxels_to_wireframes",
    "store_curve_network",
    "visual_hull_blurred",
)


def _extension():
    """The CUDA extension, loaded on first use (ImportError when it is not built)."""
    global _ext
    if _ext is None:
        _ext = _load_extension()
    return _ext


def __getattr__(name: str):
    # Loading on first use keeps the scene generator (``torchhull_gb300.scenes``)
    # importable without the CUDA extension; every operation still fails loudly
    # when the extension is missing.
    if name == "_C":
        return _extension()
    if name in _EXPORTS:
        return getattr(_extension(), name)
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")


def sparse_visual_hull_field(
    masks: torch.Tensor,
    transforms: torch.Tensor,
    level: int,
    cube_corner_bfl: tuple[float, float, float],
    cube_length: float,
    masks_partial: bool,
    transforms_convention: str,
) -> torch.Tensor:
    """Sparse hull field as a coalesced COO tensor of size (1, R, R, R), R = 2^level + 1.

    Indices are (0, z, y, x), values the product of the views' mask samples
    (reference: visual_hull_cuda.cu:522-580, :896-914).
    """
    idx, values, r = _extension().sparse_visual_hull_field_raw(
        masks, transforms, level, cube_corner_bfl, cube_length, masks_partial, transforms_convention
    )
    z = idx // (r * r)
    y = idx // r % r
    x = idx % r
    indices = torch.stack([torch.zeros_like(idx), z, y, x])
    return torch.sparse_coo_tensor(indices, values, (1, r, r, r)).coalesce()
