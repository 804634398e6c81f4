"""ctypes binding of ``libdpl.so`` (declared in ``include/dpl.h``).

The library is loaded on first use.  There is no CPU fallback: if the library
is missing, cannot be loaded, or no CUDA device is present, calls raise
``RuntimeError``.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libdpl.so"

DPL_OK = 0
DPL_ERR_INVALID_ARGUMENT = 1
DPL_ERR_ALL_NAN_SLC = 2
DPL_ERR_CUDA = 3
DPL_ERR_WORKSPACE = 4
DPL_ERR_UNSUPPORTED = 5
DPL_ERR_TIMEOUT = 6

# every function declared in include/dpl.h: name -> (restype, argtypes)
_p = C.c_void_p
_i64 = C.c_int64
_i = C.c_int
_f = C.c_float
_d = C.c_double
_sz = C.c_size_t


class PlParams(C.Structure):
    _fields_ = [
        ("nslc", _i64), ("rows", _i64), ("cols", _i64),
        ("hy", _i), ("hx", _i), ("sy", _i), ("sx", _i),
        ("use_evd", _i), ("beta", _d), ("zero_correlation_threshold", _d),
        ("reference_idx", _i), ("mask_input_ps", _i), ("use_max_ps", _i), ("use_slc_amp", _i),
        ("baseline_lag", _i), ("first_real_slc_idx", _i), ("compute_crlb", _i), ("cov_form", _i),
        ("solver_slots", _i), ("solver_lanes", _i), ("nonconverged_mode", _i),
    ]


class PlInputs(C.Structure):
    _fields_ = [("slc", _p), ("nodata_mask", _p), ("ps_mask", _p), ("neighbors", _p), ("avg_mag", _p)]


class PlOutputs(C.Structure):
    _fields_ = [
        ("cpx_phase", _p), ("temp_coh", _p), ("shp_counts", _p), ("eigenvalues", _p),
        ("estimator", _p), ("crlb_std_dev", _p), ("closure_phases", _p), ("nonconverged", _p),
    ]


SIGNATURES = {
    "dpl_last_error_message": (C.c_char_p, []),
    "dpl_version": (_i, []),
    "dpl_max_nslc": (_i, []),
    "dpl_ps_block": (_i, [_p, _i64, _i64, _f, _i, _d, _i64, _p, _p, _p, _p]),
    "dpl_shp_glrt_workspace_size": (_sz, [_i64, _i64]),
    "dpl_shp_glrt": (_i, [_p, _p, _i64, _i64, _i, _i, _i, _i, _i, _f, _p, _p, _sz, _p]),
    "dpl_shp_ks_workspace_size": (_sz, [_i64, _i64, _i64]),
    "dpl_shp_ks": (_i, [_p, _i64, _i64, _i64, _i, _i, _i, _i, _d, _i, _p, _p, _sz, _p]),
    "dpl_phase_link_workspace_size": (_sz, [C.POINTER(PlParams)]),
    "dpl_phase_link": (_i, [C.POINTER(PlParams), C.POINTER(PlInputs), C.POINTER(PlOutputs), _p, _sz, _p]),
    "dpl_phase_link_async": (_i, [C.POINTER(PlParams), C.POINTER(PlInputs), C.POINTER(PlOutputs), _p, _sz, _p]),
    "dpl_phase_link_status": (_i, [C.POINTER(PlParams), _p, _sz, _p]),
    "dpl_phase_link_status_copy": (_i, [C.POINTER(PlParams), _p, _sz, _p, _p]),
    "dpl_phase_link_status_words": (_i, [_i64, _p]),
    "dpl_phase_link_batch_workspace_size": (_sz, [C.POINTER(PlParams), _i]),
    "dpl_phase_link_batch": (_i, [C.POINTER(PlParams), C.POINTER(PlInputs), C.POINTER(PlOutputs), _i, _p, _sz, _p]),
    "dpl_phase_link_batch_status": (_i, [C.POINTER(PlParams), _i, _p, _sz, _p]),
    "dpl_covariance_workspace_size": (_sz, [_i64, _i64, _i64]),
    "dpl_covariance": (_i, [_p, _i64, _i64, _i64, _i, _i, _i, _i, _p, _i, _p, _p, _sz, _p]),
    "dpl_process_coherence_workspace_size": (_sz, [_i64]),
    "dpl_process_coherence": (_i, [_p, _i64, _i, _i, _d, _d, _i, _d, _i, _i, _p, _p, _p, _p, _p, _p, _p, _sz, _p]),
    "dpl_compress": (_i, [_p, _i64, _i64, _i64, _p, _i64, _i64, _i, _p, _i, _i, _p, _p]),
    "dpl_circle_offsets": (_i, [_i, _i, _i, _p, _i64, C.POINTER(C.c_int64)]),
    "dpl_similarity_max_radius": (_i, []),
    "dpl_similarity_prep": (_i, [_p, _i, _i64, _i64, _i64, _p, _i, _p, _i64, _p, _p]),
    "dpl_similarity": (_i, [_p, _i64, _i64, _i64, _i, _i, _p, _p]),
    "dpl_grow_nodata_region": (_i, [_p, _p, _i, _i64, _i64, _d, _i, _i, _p]),
    "dpl_process_coherence_warm": (_i, [_p, _i64, _i, _i, _d, _d, _i, _d, _i, _i, _p, _p, _p, _p, _p, _p, _p, _p,
                                        _p, _sz, _p]),
    "dpl_mlp_features": (_i, [_p, _i, _i64, _i, _p, _p]),
    "dpl_mlp_frame": (_i, [_p, _i, _i64, _p, _i, _p, _p]),
    "dpl_gemm_f32": (_i, [_i, _i, _i, _p, _i64, _i64, _p, _i64, _i64, _p, _i64, _p, _f, _f, _i, _p]),
    "dpl_relu_grad": (_i, [_p, _p, _i64, _p]),
    "dpl_mse_grad": (_i, [_p, _p, _p, _i64, _p, _p]),
    "dpl_colsum": (_i, [_p, _i, _i, _p, _p]),
    "dpl_adam": (_i, [_p, _p, _p, _p, _i64, _f, _f, _f, _f, _i, _p]),
    "dpl_mlp_packed_bytes": (_sz, [_i, _i]),
    "dpl_mlp_pack": (_i, [_p, _i, _i, _p, _p]),
    "dpl_mlp_forward_tc": (_i, [_p, _i64, _i, _i, _i, _i, _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    "dpl_process_coherence_noalloc_max_pixels": (_i64, []),
    "dpl_process_coherence_noalloc": (_i, [_p, _i64, _i, _i, _d, _d, _i, _d, _i, _i, _p, _p, _p, _p, _p, _p, _p]),
    "dpl_kernel_timing": (_i, [_i, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "dpl_fp32_fma_probe": (_i, [_p, _i, _i, _p]),
    "dpl_fp64_fma_probe": (_i, [_p, _i, _i, _p]),
}

_lock = threading.Lock()
_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load libdpl.so and declare its signatures (raises if it is missing)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path is not None else LIB_PATH
        if not p.exists():
            raise RuntimeError(
                f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(there is no CPU fallback)"
            )
        lib = C.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


class DplError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def check(status: int, what: str = ""):
    """Raise the Python exception that corresponds to a dpl_status."""
    if status == DPL_OK:
        return
    msg = load().dpl_last_error_message().decode(errors="replace")
    if status == DPL_ERR_ALL_NAN_SLC:
        from .phase_link import PhaseLinkRuntimeError

        raise PhaseLinkRuntimeError(msg)
    if status == DPL_ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    raise DplError(status, f"{what}: {msg}" if what else msg)
