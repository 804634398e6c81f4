"""SHP selection on the GPU (drop-in for ``dolphin.shp.estimate_neighbors``)."""

from __future__ import annotations

import logging
import math
from typing import Optional

import numpy as np

from . import _device as D
from . import _lib
from ._types import ShpMethod, Strides

logger = logging.getLogger("dolphin_gb300")

__all__ = ["estimate_neighbors", "glrt_threshold", "ks_critical_distance"]


def glrt_threshold(alpha: float) -> float:
    """chi-square(1) quantile at 1 - alpha (shp/_glrt.py:78)."""
    from scipy import stats

    return float(stats.chi2.ppf(1 - alpha, df=1))


def ks_critical_distance(nslc: int, alpha: float) -> float:
    """Critical ECDF distance: the reference's scan (shp/_ks.py:221-239).

    Scans distances from 0.01 in steps of 0.001 and returns the first whose
    Kolmogorov-series p-value (100 terms, N/2 effective samples) is <= alpha.
    """
    n_eff = nslc / 2.0
    cur = 0.01
    crit = 0.1
    sq = math.sqrt(n_eff)
    while cur <= 1.0:
        value = cur * (sq + 0.12 + 0.11 / sq)
        pvalue = 0
        for t in range(1, 101):
            pvalue += ((-1) ** (t - 1)) * math.exp(-2 * (value**2) * (t**2))
        pvalue = max(0.0, min(1.0, 2 * pvalue))
        if pvalue <= alpha:
            crit = cur
            break
        cur += 0.001
    return crit


def _method_name(method) -> str:
    return str(getattr(method, "value", method)).lower()


def estimate_neighbors(
    *,
    halfwin_rowcol: tuple[int, int],
    alpha: float,
    strides: Optional[Strides] = None,
    mean=None,
    var=None,
    nslc: Optional[int] = None,
    amp_stack=None,
    is_sorted: bool = False,
    method: ShpMethod = ShpMethod.GLRT,
    prune_disconnected: bool = False,
):
    """Statistically homogeneous neighbours of each pixel (shp/__init__.py:19-116).

    Same keyword-only arguments, return value and errors as the reference:
    ``None`` for RECT, else a bool array ``(rows // sy, cols // sx, 2hy+1, 2hx+1)``.
    Host inputs give a numpy array; CUDA-tensor inputs give a uint8 CUDA tensor.
    """
    if strides is None:
        strides = Strides(x=1, y=1)
    if prune_disconnected:
        logger.warning("`prune_disconnected` is deprecated: ignoring")
    name = _method_name(method)
    if name == "rect":
        return None
    hy, hx = (int(v) for v in halfwin_rowcol)
    sy, sx = (int(v) for v in strides)
    if name == "glrt":
        if nslc is None:
            raise ValueError("`nslc` must be provided for GLRT method")
        on_device = any(D.is_device_tensor(x) for x in (mean, var, amp_stack))
        if mean is None or var is None:
            if amp_stack is None:
                raise ValueError("GLRT needs `mean` and `var` (or `amp_stack`)")
            if D.is_device_tensor(amp_stack):
                a = amp_stack.float()
                mean = a.mean(0) if mean is None else mean
                var = a.var(0, unbiased=False) if var is None else var
            else:
                a = np.asarray(amp_stack)
                mean = np.mean(a, axis=0) if mean is None else mean
                var = np.var(a, axis=0) if var is None else var
        shape = tuple(mean.shape)
        rows, cols = shape
        out = D.empty((rows // sy, cols // sx, 2 * hy + 1, 2 * hx + 1), np.uint8)
        lib = _lib.load()
        ws = D.workspace(lib.dpl_shp_glrt_workspace_size(rows, cols))
        m = D.to_device(mean, np.float32)
        v = D.to_device(var, np.float32)
        thr = float(np.float32(glrt_threshold(alpha)))
        st = lib.dpl_shp_glrt(D.ptr(m), D.ptr(v), rows, cols, hy, hx, sy, sx, int(nslc), thr, D.ptr(out),
                              D.ptr(ws), ws.numel(), D.stream_handle())
        _lib.check(st, "dpl_shp_glrt")
        return out if on_device else D.to_host(out).astype(bool)
    if name == "ks":
        if amp_stack is None:
            raise ValueError("amp_stack must be provided for KS method")
        on_device = D.is_device_tensor(amp_stack)
        n, rows, cols = tuple(amp_stack.shape)
        out = D.empty((rows // sy, cols // sx, 2 * hy + 1, 2 * hx + 1), np.uint8)
        lib = _lib.load()
        ws = D.workspace(lib.dpl_shp_ks_workspace_size(n, rows, cols))
        a = D.to_device(amp_stack, np.float32)
        cutoff = ks_critical_distance(n, alpha)
        st = lib.dpl_shp_ks(D.ptr(a), n, rows, cols, hy, hx, sy, sx, cutoff, int(bool(is_sorted)), D.ptr(out),
                            D.ptr(ws), ws.numel(), D.stream_handle())
        _lib.check(st, "dpl_shp_ks")
        return out if on_device else D.to_host(out).astype(bool)
    raise ValueError(f"SHP method {method} is not implemented")
