"""Device-memory plumbing: numpy <-> CUDA tensors and the current stream.

PyTorch supplies the device allocator and streams; the compute is in libdpl.so.
"""

from __future__ import annotations

import numpy as np


def torch():
    import torch as _t

    return _t


def require_cuda():
    t = torch()
    if not t.cuda.is_available():
        raise RuntimeError("dolphin_gb300 needs a CUDA GPU (there is no CPU fallback)")
    return t


def is_device_tensor(x) -> bool:
    try:
        t = torch()
    except ImportError:  # pragma: no cover
        return False
    return isinstance(x, t.Tensor) and x.is_cuda


def to_device(x, dtype=None, device=None):
    """numpy array (or CUDA tensor) -> contiguous CUDA tensor of ``dtype`` (a numpy dtype)."""
    t = require_cuda()
    if is_device_tensor(x):
        out = x
        if dtype is not None:
            out = out.to(_torch_dtype(np.dtype(dtype)))
        return out.contiguous()
    arr = np.asarray(x)
    if dtype is not None:
        arr = arr.astype(dtype, copy=False)
    arr = np.ascontiguousarray(arr)
    host = t.from_numpy(arr)
    if host.dtype == t.bool:
        host = host.view(t.uint8)
    host = host.pin_memory()
    return host.to(device or "cuda", non_blocking=True)


def empty(shape, dtype, device=None):
    t = require_cuda()
    return t.empty(tuple(int(s) for s in shape), dtype=_torch_dtype(np.dtype(dtype)), device=device or "cuda")


def workspace(nbytes: int, device=None):
    t = require_cuda()
    return t.empty(max(int(nbytes), 256), dtype=t.uint8, device=device or "cuda")


def ptr(x):
    return None if x is None else int(x.data_ptr())


def stream_handle():
    t = require_cuda()
    return int(t.cuda.current_stream().cuda_stream)


def to_host(x, dtype=None):
    arr = x.cpu().numpy()
    if dtype is not None and arr.dtype != np.dtype(dtype):
        arr = arr.view(dtype) if arr.dtype.itemsize == np.dtype(dtype).itemsize else arr.astype(dtype)
    return arr


_MAP = None


def _torch_dtype(dt: np.dtype):
    global _MAP
    t = torch()
    if _MAP is None:
        _MAP = {
            np.dtype(np.float32): t.float32,
            np.dtype(np.float64): t.float64,
            np.dtype(np.complex64): t.complex64,
            np.dtype(np.uint8): t.uint8,
            np.dtype(np.bool_): t.uint8,
            np.dtype(np.int16): t.int16,
            np.dtype(np.int32): t.int32,
            np.dtype(np.int64): t.int64,
            np.dtype(np.uint32): t.int32,
        }
    return _MAP[dt]
