"""ctypes front end of the CPU oracle (oracle.cpp): TEST INFRASTRUCTURE ONLY.

Used by the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` as the checker.  The product path never imports this module.
See oracle.h for the parity status of the oracle.
"""

from __future__ import annotations

import ctypes
import dataclasses
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

DTYPE_CODES = {
    np.dtype(np.bool_): 0,
    np.dtype(np.uint8): 1,
    np.dtype(np.int8): 2,
    np.dtype(np.int16): 3,
    np.dtype(np.int32): 4,
    np.dtype(np.int64): 5,
    np.dtype(np.float16): 6,
    np.dtype(np.float32): 7,
    np.dtype(np.float64): 8,
}
CODE_DTYPES = {v: k for k, v in DTYPE_CODES.items()}

_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        vp, i64, i32, f32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_float
        L.oracle_visual_hull.restype = vp
        L.oracle_visual_hull.argtypes = [vp, i32, i64, i64, i64, vp, i32, i32, f32, f32, f32, f32, i32, i32, i32, i32,
                                         ctypes.c_char_p, i32]
        for name in ("oracle_hull_num_levels", "oracle_hull_field_size", "oracle_hull_num_verts",
                     "oracle_hull_num_faces"):
            getattr(L, name).restype = i64
            getattr(L, name).argtypes = [vp]
        L.oracle_hull_level_size.restype = i64
        L.oracle_hull_level_size.argtypes = [vp, i64]
        L.oracle_hull_level_copy.argtypes = [vp, i64, vp]
        L.oracle_hull_field_copy.argtypes = [vp, vp, vp]
        L.oracle_hull_mesh_copy.argtypes = [vp, vp, vp]
        L.oracle_hull_free.argtypes = [vp]
        L.oracle_integral_image.restype = i32
        L.oracle_integral_image.argtypes = [vp, i32, i64, i64, i64, vp, i32]
        L.oracle_gaussian_blur.restype = i32
        L.oracle_gaussian_blur.argtypes = [vp, i32, i64, i64, i64, i32, f32, i32, vp, i32, i32, ctypes.c_char_p, i32]
        L.oracle_marching_cubes.restype = vp
        L.oracle_marching_cubes.argtypes = [vp, vp, i32, i64, i64, i64, i64, f32, i32, i32, i32, ctypes.c_char_p, i32]
        for name in ("oracle_mesh_num_verts", "oracle_mesh_num_faces"):
            getattr(L, name).restype = i64
            getattr(L, name).argtypes = [vp]
        L.oracle_mesh_copy.argtypes = [vp, vp, vp]
        L.oracle_mesh_free.argtypes = [vp]
        L.oracle_candidate_wireframe.argtypes = [vp, i64, i32, f32, f32, f32, f32, vp, vp]
        L.oracle_bilerp_ones_failures.restype = i64
        L.oracle_bilerp_ones_failures.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        _lib = L
    return _lib


@dataclasses.dataclass
class HullResult:
    verts: np.ndarray  # [V,3] float32
    faces: np.ndarray  # [F,3] int64
    levels: list[np.ndarray]  # per-level ravelled candidates, reference order
    field_indices: np.ndarray  # [C] int64 ascending
    field_values: np.ndarray  # [C] float32


def _as_array(x) -> np.ndarray:
    if hasattr(x, "detach"):
        x = x.detach().cpu().contiguous().numpy()
    return np.ascontiguousarray(x)


def visual_hull(masks, transforms, level, cube_corner_bfl, cube_length, masks_partial, transforms_convention,
                unique_verts=True, nthreads=0) -> HullResult:
    m = _as_array(masks)
    t = _as_array(transforms)
    if m.ndim != 4 or m.shape[3] != 1:
        raise ValueError("masks must be [B,H,W,1]")
    if transforms_convention not in ("opengl", "opencv"):
        raise ValueError(f'Unsupported transforms_convention "{transforms_convention}".')
    err = ctypes.create_string_buffer(256)
    B, H, W, _ = m.shape
    h = lib().oracle_visual_hull(
        m.ctypes.data, DTYPE_CODES[m.dtype], B, H, W, t.ctypes.data, DTYPE_CODES[t.dtype], int(level),
        float(cube_corner_bfl[0]), float(cube_corner_bfl[1]), float(cube_corner_bfl[2]), float(cube_length),
        int(bool(masks_partial)), int(transforms_convention == "opengl"), int(bool(unique_verts)), int(nthreads),
        err, len(err))
    if not h:
        raise RuntimeError(err.value.decode())
    L = lib()
    try:
        levels = []
        for i in range(L.oracle_hull_num_levels(h)):
            a = np.empty(L.oracle_hull_level_size(h, i), dtype=np.int64)
            L.oracle_hull_level_copy(h, i, a.ctypes.data)
            levels.append(a)
        n = L.oracle_hull_field_size(h)
        fi = np.empty(n, dtype=np.int64)
        fv = np.empty(n, dtype=np.float32)
        L.oracle_hull_field_copy(h, fi.ctypes.data, fv.ctypes.data)
        v = np.empty((L.oracle_hull_num_verts(h), 3), dtype=np.float32)
        f = np.empty((L.oracle_hull_num_faces(h), 3), dtype=np.int64)
        L.oracle_hull_mesh_copy(h, v.ctypes.data, f.ctypes.data)
    finally:
        L.oracle_hull_free(h)
    return HullResult(v, f, levels, fi, fv)


def integral_image(masks, nthreads=0) -> np.ndarray:
    m = _as_array(masks)
    B, H, W = m.shape[:3]
    out = np.empty((B, H, W), dtype=np.float32)
    lib().oracle_integral_image(m.ctypes.data, DTYPE_CODES[m.dtype], B, H, W, out.ctypes.data, int(nthreads))
    return out


def gaussian_blur(images, kernel_size, sigma, sparse=True, dtype=None, nthreads=0) -> np.ndarray:
    m = _as_array(images)
    out_dtype = np.dtype(dtype) if dtype is not None else m.dtype
    B, H, W, _ = m.shape
    out = np.empty(m.shape, dtype=out_dtype)
    err = ctypes.create_string_buffer(256)
    rc = lib().oracle_gaussian_blur(m.ctypes.data, DTYPE_CODES[m.dtype], B, H, W, int(kernel_size), float(sigma),
                                    int(bool(sparse)), out.ctypes.data, DTYPE_CODES.get(out_dtype, -1),
                                    int(nthreads), err, len(err))
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return out


def marching_cubes(volume=None, isolevel=0.0, return_local_coords=True, unique_verts=True, *, indices=None,
                   values=None, size=None, nthreads=0) -> tuple[np.ndarray, np.ndarray]:
    """Dense volume [1,D,H,W], or a coalesced sparse one as indices [4,N] (rows 0, z, y, x), values [N] and
    size (1, D, H, W).  Returns (verts [V,3] float32, faces [F,3] int64)."""
    if volume is not None:
        v = _as_array(volume)
        _, D, H, W = v.shape
        vals = np.ascontiguousarray(v.reshape(-1))
        ids = np.arange(vals.size, dtype=np.int64)
    else:
        idx = _as_array(indices).astype(np.int64)
        vals = _as_array(values)
        _, D, H, W = size
        ids = np.ascontiguousarray(idx[3] + W * (idx[2] + H * idx[1]), dtype=np.int64)
    err = ctypes.create_string_buffer(256)
    L = lib()
    h = L.oracle_marching_cubes(ids.ctypes.data, vals.ctypes.data, DTYPE_CODES.get(vals.dtype, -1), ids.size, D, H,
                                W, float(isolevel), int(bool(return_local_coords)), int(bool(unique_verts)),
                                int(nthreads), err, len(err))
    if not h:
        raise RuntimeError(err.value.decode())
    try:
        verts = np.empty((L.oracle_mesh_num_verts(h), 3), dtype=np.float32)
        faces = np.empty((L.oracle_mesh_num_faces(h), 3), dtype=np.int64)
        L.oracle_mesh_copy(h, verts.ctypes.data, faces.ctypes.data)
    finally:
        L.oracle_mesh_free(h)
    return verts, faces


def candidate_voxels_to_wireframes(candidate_voxels, cube_corner_bfl, cube_length):
    out = []
    for i, c in enumerate(candidate_voxels):
        ids = np.ascontiguousarray(_as_array(c), dtype=np.int64)
        n = ids.size
        verts = np.empty((8 * n, 3), dtype=np.float32)
        edges = np.empty((12 * n, 2), dtype=np.int64)
        lib().oracle_candidate_wireframe(ids.ctypes.data, n, i, float(cube_corner_bfl[0]), float(cube_corner_bfl[1]),
                                         float(cube_corner_bfl[2]), float(cube_length), verts.ctypes.data,
                                         edges.ctypes.data)
        out.append((verts, edges))
    return out


def nthreads_default() -> int:
    return os.cpu_count() or 1
