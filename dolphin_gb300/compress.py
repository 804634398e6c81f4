"""Compressed SLC on the GPU: drop-in for ``dolphin.phase_link.compress``.

Same arguments, output and in-place behaviour as the reference
(phase_link/_compress.py:11-65); the compute runs in ``libdpl.so``.
"""

from __future__ import annotations

import numpy as np

from . import _device as D
from . import _lib

__all__ = ["compress"]


def compress(slc_stack, pl_cpx_phase, first_real_slc_idx: int = 0, slc_mean=None, reference_idx=None):
    """Project the SLCs on the phase-linked phase: mean |z| x exp(i angle(sum_t z_t conj(pl_t))).

    ``pl_cpx_phase`` is re-referenced to ``reference_idx`` (if not None) before the
    compressed layers (index < ``first_real_slc_idx``) are dropped, and upsampled to the
    SLC grid by block repetition (zero beyond).  Where the projected phase is exactly
    0 the output is NaN and a given ``slc_mean`` is set to NaN in place.  Host inputs
    give a host (rows, cols) complex64 array; CUDA tensors give a CUDA tensor.
    """
    on_device = D.is_device_tensor(slc_stack)
    nslc, rows, cols = (int(v) for v in slc_stack.shape)
    pn, prow, pcol = (int(v) for v in pl_cpx_phase.shape)
    if pn != nslc:
        raise ValueError(f"pl_cpx_phase has {pn} layers, slc_stack {nslc}")
    ref = None if reference_idx is None else int(reference_idx)
    if ref is not None and ref < 0:
        ref += nslc
    if ref is not None and not 0 <= ref < nslc:
        raise IndexError(f"reference_idx {reference_idx} out of range for {nslc} layers")
    slc = D.to_device(slc_stack, np.complex64)
    pl = D.to_device(pl_cpx_phase, np.complex64)
    mean_dev = None
    if slc_mean is not None:
        mean_dev = D.to_device(slc_mean, np.float32)
        if D.is_device_tensor(slc_mean) and mean_dev.data_ptr() != slc_mean.data_ptr():
            mean_dev = mean_dev.clone()
    out = D.empty((rows, cols), np.complex64)
    lib = _lib.load()
    st = lib.dpl_compress(D.ptr(slc), nslc, rows, cols, D.ptr(pl), prow, pcol, int(first_real_slc_idx),
                          D.ptr(mean_dev), int(ref is not None), int(ref or 0), D.ptr(out), D.stream_handle())
    _lib.check(st, "dpl_compress")
    if slc_mean is not None:
        # the reference modifies the given mean in place (NaN where the phase is 0)
        if D.is_device_tensor(slc_mean):
            if mean_dev.data_ptr() != slc_mean.data_ptr():
                slc_mean.copy_(mean_dev.to(slc_mean.dtype))
        else:
            np.copyto(slc_mean, D.to_host(mean_dev).astype(slc_mean.dtype, copy=False))
    return out if on_device else D.to_host(out)
