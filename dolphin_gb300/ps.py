"""Amplitude-dispersion PS selection on the GPU (drop-in for ``ps.calc_ps_block``)."""

from __future__ import annotations

from typing import Optional

import numpy as np

from . import _device as D
from . import _lib

__all__ = ["calc_ps_block"]


def calc_ps_block(stack_mag, amp_dispersion_threshold: float = 0.25, min_count: Optional[int] = None):
    """Amplitude mean, dispersion and PS mask of a block (ps.py:169-244).

    Same arguments, outputs and dtypes as the reference: ``(mean float32,
    amp_disp float32, ps bool)``.  The float32 arithmetic reproduces numpy's
    ``nanmean``/``nanstd`` bit for bit.  A host (numpy) input returns numpy arrays;
    a CUDA tensor input returns CUDA tensors (``ps`` as uint8).
    """
    on_device = D.is_device_tensor(stack_mag)
    if on_device:
        if stack_mag.is_complex():
            raise ValueError("The input `stack_mag` must be real-valued.")
        shape = tuple(stack_mag.shape)
    else:
        stack_mag = np.asarray(stack_mag)
        if np.iscomplexobj(stack_mag):
            raise ValueError("The input `stack_mag` must be real-valued.")
        shape = stack_mag.shape
    nslc = shape[0]
    spatial = shape[1:]
    npix = int(np.prod(spatial)) if len(spatial) else 1
    if min_count is None:
        min_count = int(0.9 * nslc)
    thr_is_f64 = isinstance(amp_dispersion_threshold, np.floating) and np.dtype(
        type(amp_dispersion_threshold)) == np.float64
    mag = D.to_device(stack_mag, np.float32)
    mean = D.empty((npix,), np.float32)
    disp = D.empty((npix,), np.float32)
    ps = D.empty((npix,), np.uint8)
    lib = _lib.load()
    st = lib.dpl_ps_block(D.ptr(mag), nslc, npix, float(np.float32(amp_dispersion_threshold)),
                          int(thr_is_f64), float(amp_dispersion_threshold), int(min_count),
                          D.ptr(mean), D.ptr(disp), D.ptr(ps), D.stream_handle())
    _lib.check(st, "dpl_ps_block")
    if on_device:
        return mean.reshape(spatial), disp.reshape(spatial), ps.reshape(spatial)
    return (D.to_host(mean).reshape(spatial), D.to_host(disp).reshape(spatial),
            D.to_host(ps).astype(bool).reshape(spatial))
