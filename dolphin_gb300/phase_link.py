"""Phase linking on the GPU: drop-in for ``dolphin.phase_link.run_phase_linking``.

``run_phase_linking`` keeps the reference's signature, defaults, output
``PhaseLinkOutput`` and exceptions (phase_link/_core.py:67-249).  All compute runs
in ``libdpl.so``; this module only moves arrays and maps status codes to
exceptions.
"""

from __future__ import annotations

import contextlib
import math
import threading
from enum import IntEnum
from typing import NamedTuple, Optional

import numpy as np

from . import _device as D
from . import _lib
from ._types import HalfWindow, Strides

__all__ = [
    "EstimatorType",
    "PhaseLinkOutput",
    "PhaseLinkRuntimeError",
    "deferred_checks",
    "estimate_stack_covariance",
    "process_coherence_matrices",
    "run_phase_linking",
]

DEFAULT_STRIDES = Strides(1, 1)


class PhaseLinkRuntimeError(Exception):
    """Exception raised while running the MLE solver."""


class EstimatorType(IntEnum):
    """Type of estimator used for phase linking."""

    EVD = 0
    EMI = 1


class PhaseLinkOutput(NamedTuple):
    """Output of the MLE solver (same fields and order as the reference)."""

    cpx_phase: object
    temp_coh: object
    shp_counts: object
    eigenvalues: object
    estimator: object
    crlb_std_dev: object
    closure_phases: object


_deferred = threading.local()


@contextlib.contextmanager
def deferred_checks():
    """Defer the status checks of device-resident ``run_phase_linking`` calls.

    Inside the block, a call on CUDA tensors enqueues its pipeline and a copy of its
    three status words into pinned host memory, and returns without waiting for the
    GPU, so that a block loop keeps the host ahead of the device.  On leaving the
    block, each deferred status is waited for and checked in call order: the first
    failure raises the exception that the synchronous call would have raised (e.g.
    ``PhaseLinkRuntimeError`` for an all-NaN SLC).  The outputs of a failed call are
    undefined.  Calls on host (numpy) arrays are not affected.  Not in the reference,
    whose calls are synchronous.
    """
    prev = getattr(_deferred, "pending", None)
    pending = []
    _deferred.pending = pending
    try:
        yield
    finally:
        _deferred.pending = prev
    lib = _lib.load()
    for nslc, words, event in pending:
        event.synchronize()
        _lib.check(lib.dpl_phase_link_status_words(nslc, words.data_ptr()), "dpl_phase_link")


@contextlib.contextmanager
def _captured_checks(calls):
    """Inside the block (a CUDA-graph capture of device-resident calls), each
    ``run_phase_linking`` call enqueues its pipeline without a host copy or event and
    appends ``(params, workspace)`` to ``calls``; after a replay, ``check_captured``
    reports the first failure in call order."""
    prev = getattr(_deferred, "pending", None)
    prev_graph = getattr(_deferred, "graph", None)
    _deferred.pending = []
    _deferred.graph = calls
    try:
        yield calls
    finally:
        _deferred.pending = prev
        _deferred.graph = prev_graph


def check_captured(calls):
    """Status of the captured calls after a replay (synchronises the stream), raising
    the exception the first failing synchronous call would have raised."""
    lib = _lib.load()
    for prm, ws in calls:
        _lib.check(lib.dpl_phase_link_status(prm, D.ptr(ws), ws.numel(), D.stream_handle()), "dpl_phase_link")


def _is_complex(x) -> bool:
    if D.is_device_tensor(x):
        return x.is_complex()
    return np.iscomplexobj(x)


def _host_all_nan_check(slc):
    nans = np.isnan(slc)
    bad = np.where(np.all(nans, axis=(1, 2)))[0]
    if bad.size > 0:
        raise PhaseLinkRuntimeError(f"slc_stack[{bad}] out of {len(slc)} are all NaNs.")


def run_phase_linking(
    slc_stack,
    half_window: HalfWindow,
    strides: Strides = DEFAULT_STRIDES,
    use_evd: bool = False,
    beta: float = 0.0,
    zero_correlation_threshold: float = 0.0,
    reference_idx: int = 0,
    nodata_mask=None,
    mask_input_ps: bool = False,
    ps_mask=None,
    use_max_ps: bool = True,
    neighbor_arrays=None,
    avg_mag=None,
    use_slc_amp: bool = False,
    baseline_lag: Optional[int] = None,
    first_real_slc_idx: int = 0,
    compute_crlb: bool = True,
    *,
    covariance_form: str = "tensor",
    solver_slots: int = 0,
    solver_lanes: int = 0,
    eigh_fallback: bool = True,
    nonconverged=None,
) -> PhaseLinkOutput:
    """Estimate the linked phase for a stack of SLCs (phase_link/_core.py:67-249).

    Host (numpy) inputs give numpy outputs; if ``slc_stack`` is a CUDA tensor, all
    outputs stay on the device as tensors (``estimator`` uint8, masks uint8).

    ``covariance_form`` (keyword-only, not in the reference): ``"tensor"`` computes
    the coherence matrices on the tensor cores (bf16 hi/lo split, fp32
    accumulation); ``"tf32"`` the same contraction with tf32 operands (one product,
    fp32 accumulation); ``"simt"`` uses fp32 CUDA-core arithmetic throughout; ``"fp64"``
    computes the covariance and the solve in double precision (a reference form: GB300's
    FP64 rate is low), writing the same float32 outputs.

    ``solver_slots`` / ``solver_lanes`` (keyword-only, not in the reference): the
    register solver's row slots (even, >= N) and threads per pixel (8, 16, 32); 0 picks
    the smallest that fit.  A tuner's choices (``dolphin_gb300.tune_forms``); the results
    are the same.

    ``eigh_fallback`` (keyword-only, not in the reference): pixels whose eigen-iteration
    misses the stopping rule within 49 steps are solved again by a dense Hermitian
    eigensolver (tensor-core form); ``False`` keeps the last iterate, as the reference
    does.  ``nonconverged``: an optional (rows', cols') uint8 array (a CUDA tensor for
    device inputs) that receives 1 on those pixels.
    """
    on_device = D.is_device_tensor(slc_stack)
    shape = tuple(slc_stack.shape)
    if len(shape) != 3:
        raise ValueError(f"slc_stack must be 3-D (n_images, rows, cols), got {shape}")
    nslc, rows, cols = shape
    hy, hx = (int(v) for v in half_window)
    sy, sx = (int(v) for v in strides)
    # mask shapes are checked before launching; the reference raises its all-NaN
    # error first, so that check runs on the host in this (error) path only
    for name, m in (("nodata_mask", nodata_mask), ("ps_mask", ps_mask)):
        if m is not None and tuple(m.shape) != (rows, cols):
            if not on_device:
                _host_all_nan_check(np.asarray(slc_stack))
            nd = None if nodata_mask is None else tuple(nodata_mask.shape)
            pm = None if ps_mask is None else tuple(ps_mask.shape)
            raise ValueError(f"nodata_mask.shape={nd}, ps_mask.shape={pm}, but != SLC (rows, cols) {rows, cols}")
    if not _is_complex(slc_stack):
        raise ValueError("The SLC stack must be complex.")
    out_rows, out_cols = rows // sy, cols // sx
    wy, wx = 2 * hy + 1, 2 * hx + 1
    if neighbor_arrays is not None and tuple(neighbor_arrays.shape) != (out_rows, out_cols, wy, wx):
        raise ValueError(
            f"neighbor_arrays.shape={tuple(neighbor_arrays.shape)} != {(out_rows, out_cols, wy, wx)}"
        )

    slc = D.to_device(slc_stack, np.complex64)
    nodata = None if nodata_mask is None else D.to_device(nodata_mask, np.uint8)
    ps = None if ps_mask is None else D.to_device(ps_mask, np.uint8)
    nb = None if neighbor_arrays is None else D.to_device(neighbor_arrays, np.uint8)
    am = None if avg_mag is None else D.to_device(avg_mag, np.float32)

    prm = _lib.PlParams(
        nslc=nslc, rows=rows, cols=cols, hy=hy, hx=hx, sy=sy, sx=sx, use_evd=int(bool(use_evd)),
        beta=float(beta), zero_correlation_threshold=float(zero_correlation_threshold),
        reference_idx=int(reference_idx), mask_input_ps=int(bool(mask_input_ps)),
        use_max_ps=int(bool(use_max_ps)), use_slc_amp=int(bool(use_slc_amp)),
        baseline_lag=int(baseline_lag) if baseline_lag else 0,
        first_real_slc_idx=int(first_real_slc_idx), compute_crlb=int(bool(compute_crlb)),
        cov_form=_form_code(covariance_form), solver_slots=int(solver_slots), solver_lanes=int(solver_lanes),
        nonconverged_mode=0 if eigh_fallback else 1,
    )
    cpx = D.empty((nslc, out_rows, out_cols), np.complex64)
    tcoh = D.empty((out_rows, out_cols), np.float32)
    counts = D.empty((out_rows, out_cols), np.int32) if nb is not None else None
    eig = D.empty((out_rows, out_cols), np.float32)
    est = D.empty((out_rows, out_cols), np.uint8)
    crlb = D.empty((nslc, out_rows, out_cols), np.float32)
    clos = D.empty((out_rows, out_cols, max(nslc - 2, 0)), np.float32)
    lib = _lib.load()
    ws = D.workspace(lib.dpl_phase_link_workspace_size(prm))
    inp = _lib.PlInputs(slc=D.ptr(slc), nodata_mask=D.ptr(nodata), ps_mask=D.ptr(ps), neighbors=D.ptr(nb),
                        avg_mag=D.ptr(am))
    ncflag = None
    if nonconverged is not None:
        if tuple(nonconverged.shape) != (out_rows, out_cols):
            raise ValueError(f"nonconverged.shape={tuple(nonconverged.shape)} != {(out_rows, out_cols)}")
        ncflag = D.empty((out_rows, out_cols), np.uint8)
    outp = _lib.PlOutputs(cpx_phase=D.ptr(cpx), temp_coh=D.ptr(tcoh), shp_counts=D.ptr(counts),
                          eigenvalues=D.ptr(eig), estimator=D.ptr(est), crlb_std_dev=D.ptr(crlb),
                          closure_phases=D.ptr(clos) if nslc > 2 else None, nonconverged=D.ptr(ncflag))
    pending = getattr(_deferred, "pending", None) if on_device else None
    captured = getattr(_deferred, "graph", None) if on_device else None
    if captured is not None:
        _lib.check(lib.dpl_phase_link_async(prm, inp, outp, D.ptr(ws), ws.numel(), D.stream_handle()),
                   "dpl_phase_link_async")
        captured.append((prm, ws))
    elif pending is None:
        st = lib.dpl_phase_link(prm, inp, outp, D.ptr(ws), ws.numel(), D.stream_handle())
        _lib.check(st, "dpl_phase_link")
    else:
        torch = D.torch()
        _lib.check(lib.dpl_phase_link_async(prm, inp, outp, D.ptr(ws), ws.numel(), D.stream_handle()),
                   "dpl_phase_link_async")
        words = torch.empty(3, dtype=torch.int32, pin_memory=True)
        _lib.check(lib.dpl_phase_link_status_copy(prm, D.ptr(ws), ws.numel(), words.data_ptr(), D.stream_handle()),
                   "dpl_phase_link_status_copy")
        event = torch.cuda.Event()
        event.record()
        pending.append((nslc, words, event))
    if ncflag is not None:
        if D.is_device_tensor(nonconverged):
            nonconverged.copy_(ncflag)
        else:
            nonconverged[...] = D.to_host(ncflag)
    if on_device:
        if counts is None:
            counts = D.require_cuda().zeros((out_rows, out_cols), dtype=D.torch().int16, device=cpx.device)
        return PhaseLinkOutput(cpx, tcoh, counts, eig, est, crlb, clos)
    return PhaseLinkOutput(
        cpx_phase=D.to_host(cpx),
        temp_coh=D.to_host(tcoh),
        shp_counts=D.to_host(counts) if counts is not None else np.zeros((out_rows, out_cols), np.int16),
        eigenvalues=D.to_host(eig),
        estimator=D.to_host(est),
        crlb_std_dev=D.to_host(crlb),
        closure_phases=D.to_host(clos),
    )


def _form_code(form: str) -> int:
    codes = {"tensor": 0, "simt": 1, "fp64": 2, "tf32": 3}
    if form not in codes:
        raise ValueError(f"covariance_form must be one of {sorted(codes)}, got {form!r}")
    return codes[form]


def estimate_stack_covariance(slc_stack, half_window: HalfWindow, strides: Strides = DEFAULT_STRIDES,
                              neighbor_arrays=None, *, covariance_form: str = "tensor"):
    """SHP-masked coherence matrices (covariance.py:24-107): (rows', cols', N, N) complex64."""
    if not _is_complex(slc_stack):
        raise ValueError("The SLC stack must be complex.")
    on_device = D.is_device_tensor(slc_stack)
    nslc, rows, cols = tuple(slc_stack.shape)
    hy, hx = (int(v) for v in half_window)
    sy, sx = (int(v) for v in strides)
    out_rows, out_cols = rows // sy, cols // sx
    slc = D.to_device(slc_stack, np.complex64)
    nb = None if neighbor_arrays is None else D.to_device(neighbor_arrays, np.uint8)
    C = D.empty((out_rows, out_cols, nslc, nslc), np.complex64)
    lib = _lib.load()
    ws = D.workspace(lib.dpl_covariance_workspace_size(nslc, rows, cols))
    st = lib.dpl_covariance(D.ptr(slc), nslc, rows, cols, hy, hx, sy, sx, D.ptr(nb), _form_code(covariance_form),
                            D.ptr(C), D.ptr(ws), ws.numel(), D.stream_handle())
    _lib.check(st, "dpl_covariance")
    return C if on_device else D.to_host(C)


def process_coherence_matrices(C_arrays, use_evd: bool = False, beta: float = 0.0,
                               zero_correlation_threshold: float = 0.0, reference_idx: int = 0,
                               num_looks: float = 1, first_real_slc_idx: int = 0, compute_crlb: bool = True,
                               return_metrics: bool = False):
    """EVD/EMI on given coherence matrices (phase_link/_core.py:379-534).

    Returns ``(eig_vecs (rows, cols, N) referenced, eig_vals, estimator uint8,
    crlb_std_dev (rows, cols, N))``; with ``return_metrics`` also the temporal
    coherence (metrics.py:10-40) and the closure phases (_closure_phase.py:23-40).
    """
    on_device = D.is_device_tensor(C_arrays)
    shape = tuple(C_arrays.shape)
    n = shape[-1]
    batch = shape[:-2]
    npix = int(np.prod(batch)) if batch else 1
    Cd = D.to_device(C_arrays, np.complex64)
    vec = D.empty((npix, n), np.complex64)
    val = D.empty((npix,), np.float32)
    est = D.empty((npix,), np.uint8)
    crlb = D.empty((npix, n), np.float32)
    tc = D.empty((npix,), np.float32)
    clos = D.empty((npix, max(n - 2, 0)), np.float32)
    lib = _lib.load()
    ref = reference_idx + n if reference_idx < 0 else reference_idx
    ws = D.workspace(lib.dpl_process_coherence_workspace_size(npix))
    st = lib.dpl_process_coherence(D.ptr(Cd), npix, n, int(bool(use_evd)), float(beta),
                                   float(zero_correlation_threshold), int(ref), float(num_looks),
                                   int(first_real_slc_idx), int(bool(compute_crlb)), D.ptr(vec), D.ptr(val),
                                   D.ptr(est), D.ptr(crlb), D.ptr(tc), D.ptr(clos) if n > 2 else None,
                                   D.ptr(ws), ws.numel(), D.stream_handle())
    _lib.check(st, "dpl_process_coherence")
    outs = [vec.reshape(*batch, n), val.reshape(batch), est.reshape(batch), crlb.reshape(*batch, n)]
    if return_metrics:
        outs += [tc.reshape(batch), clos.reshape(*batch, max(n - 2, 0))]
    if on_device:
        return tuple(outs)
    return tuple(D.to_host(o) for o in outs)


def num_looks_for(half_window) -> float:
    """The CRLB's number of looks, sqrt(hy * hx) (phase_link/_core.py:342)."""
    return math.sqrt(half_window[0] * half_window[1])
