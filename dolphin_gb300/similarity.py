"""Phase-similarity raster on the GPU: drop-in for ``dolphin.similarity``.

``get_circle_idxs``, ``median_similarity`` and ``max_similarity`` keep the reference's
arguments, outputs and in-place mask update (similarity.py:31-254); the rasters are
computed by ``dpl_similarity_prep`` and ``dpl_similarity`` in ``libdpl.so``.
``stack_similarity`` is the per-block computation of ``create_similarities``
(similarity.py:258-352) without its raster I/O: the optional nearest-n differences
(similarity.py:355-375), then the median or max similarity.

Inputs are host arrays (numpy) or CUDA tensors; complex128 / float64 stacks are
computed in complex64 / float32.  ``phase_similarity`` (similarity.py:21-28) is the
reference's per-pair helper on two 1-D vectors; it runs on the host and is not part of
the raster path.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _device as D
from . import _lib

__all__ = [
    "get_circle_idxs",
    "max_similarity",
    "median_similarity",
    "nearest_n_pair_count",
    "phase_similarity",
    "stack_similarity",
]


def get_circle_idxs(max_radius: int, min_radius: int = 0, sort_output: bool = True) -> np.ndarray:
    """(K, 2) int64 (row, col) offsets of the search circle, as the reference returns them
    (an empty float array when there are none)."""
    max_radius, min_radius = int(max_radius), int(min_radius)
    if max_radius < 0:
        raise ValueError("negative dimensions are not allowed")
    if max_radius == 0:
        raise IndexError("index 0 is out of bounds for axis 0 with size 0")
    lib = _lib.load()
    count = C.c_int64()
    _lib.check(lib.dpl_circle_offsets(max_radius, min_radius, int(bool(sort_output)), None, 0, C.byref(count)),
               "dpl_circle_offsets")
    if count.value == 0:
        return np.array([])
    buf = np.empty((count.value, 2), dtype=np.int32)
    _lib.check(lib.dpl_circle_offsets(max_radius, min_radius, int(bool(sort_output)), buf.ctypes.data, count.value,
                                      C.byref(count)), "dpl_circle_offsets")
    return buf.astype(np.int64)


def phase_similarity(x1, x2) -> float:
    """Mean over the vectors of Re(x1 conj x2) (host helper on two 1-D vectors)."""
    x1, x2 = np.asarray(x1), np.asarray(x2)
    n = len(x1)
    total = 0.0
    for a, b in zip(x1, x2):
        total += float(np.real(a * np.conj(b)))
    return total / n


def nearest_n_pair_count(num_layers: int, n: int) -> int:
    """Number of nearest-n pairs (i, j), i < j <= i + n, over num_layers + 1 dates."""
    return sum(min(n, num_layers - i) for i in range(num_layers + 1))


def _run(ifg_stack, search_radius, mask, kind, nearest_n=0):
    on_device = D.is_device_tensor(ifg_stack)
    shape = tuple(int(v) for v in ifg_stack.shape)
    if len(shape) != 3:
        raise ValueError(f"ifg_stack must be (n_ifg, rows, cols), got shape {shape}")
    n, rows, cols = shape
    if mask is not None and tuple(mask.shape) != (rows, cols):
        raise ValueError(f"ifg_stack.shape = {shape}, but mask.shape = {tuple(mask.shape)}")
    if on_device:
        is_complex = ifg_stack.is_complex()
    else:
        is_complex = np.iscomplexobj(ifg_stack)
    stack = D.to_device(ifg_stack, np.complex64 if is_complex else np.float32)
    mask_dev = None if mask is None else D.to_device(mask, np.uint8)
    m = nearest_n_pair_count(n, nearest_n) if nearest_n else n
    unit = D.empty((m, rows, cols), np.complex64, device=stack.device)
    valid = D.empty((rows, cols), np.uint8, device=stack.device)
    out = D.empty((rows, cols), np.float32, device=stack.device)
    lib = _lib.load()
    sh = D.stream_handle()
    _lib.check(lib.dpl_similarity_prep(D.ptr(stack), int(is_complex), n, rows, cols, D.ptr(mask_dev),
                                       int(nearest_n), D.ptr(unit), m, D.ptr(valid), sh), "dpl_similarity_prep")
    _lib.check(lib.dpl_similarity(D.ptr(unit), m, rows, cols, int(search_radius), kind, D.ptr(out), sh),
               "dpl_similarity")
    if mask is not None:
        # the reference clears the caller's mask on invalid pixels, in place
        if D.is_device_tensor(mask):
            mask.copy_(valid.to(mask.dtype))
        else:
            np.copyto(mask, D.to_host(valid).astype(mask.dtype, copy=False))
    return out if on_device else D.to_host(out)


def _radius(search_radius):
    r = int(search_radius)
    if r < 0:
        raise ValueError("negative dimensions are not allowed")
    if r == 0:
        raise IndexError("index 0 is out of bounds for axis 0 with size 0")
    return r


def median_similarity(ifg_stack, search_radius: int, mask=None):
    """Median similarity of each pixel with its neighbours (Wang 2022, eq. 5)."""
    return _run(ifg_stack, _radius(search_radius), mask, 0)


def max_similarity(ifg_stack, search_radius: int, mask=None):
    """Largest similarity of each pixel with any neighbour (Wang 2022, eq. 6)."""
    return _run(ifg_stack, _radius(search_radius), mask, 1)


def stack_similarity(ifg_stack, search_radius: int = 7, sim_type: str = "median", nearest_n: int | None = None,
                     mask=None):
    """``create_similarities``' block computation: with ``nearest_n``, the phases of the
    nearest-n pairs of the single-reference stack (layer t = date t + 1 against date 0)
    replace the layers; then the median or max similarity."""
    if sim_type == "median":
        kind = 0
    elif sim_type == "max":
        kind = 1
    else:
        raise ValueError(f"Unrecognized sim_type = {sim_type!r}")
    nn = 0 if nearest_n is None else int(nearest_n)
    if nn < 0:
        raise ValueError("nearest_n must be positive")
    return _run(ifg_stack, _radius(search_radius), mask, kind, nn)
