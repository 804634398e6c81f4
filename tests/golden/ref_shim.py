"""Run the reference's own phase-linking source without jax or numba.

This module is fixture-generation infrastructure only.  It is imported by
``make_golden.py`` in a container that holds the reference checkout; nothing
on the GPU side, in ``smoke()`` or in ``bench.py`` imports it.

The reference (dolphin) computes its hot path with ``jax.numpy`` (under
``jit``/``vmap``) and ``numba.njit``.  Neither package is installable here, so
this module registers stand-ins in ``sys.modules`` before the reference
modules are loaded from their source files:

* ``jax`` / ``jax.numpy`` / ``jax.lax`` / ``jax.scipy.linalg``: numpy and
  scipy with JAX's 32-bit canonicalisation (``jax_enable_x64`` off: float64 ->
  float32, complex128 -> complex64, int64 -> int32), ``jit`` as the identity,
  ``vmap`` as a Python loop, ``lax.dynamic_slice`` with JAX's start clamping,
  ``lax.while_loop`` as a Python loop, immutable ``.at[...].set`` updates, and
  LAPACK-backed ``cho_factor``/``solve`` that return NaNs on failure (as
  jaxlib does) instead of raising;
* ``numba``: ``njit``/``cuda.jit`` as the identity and ``prange`` as ``range``
  (so the numba kernels run as the plain Python they are written in);
* ``osgeo`` and the I/O parts of ``dolphin`` that the hot-path modules import
  at top level but never call on this path.

What this does NOT reproduce is XLA's own float32 kernels: sums, dots and
transcendental functions are numpy's.  Fixtures made this way pin the
reference's semantics (window clamping, masks, iteration caps, NaN rules,
output layout) and its float32 results to within rounding.
"""

from __future__ import annotations

import functools
import importlib.util
import os
import sys
import types
from pathlib import Path

import numpy as np
import scipy.linalg as sla

# the reference checkout: DOLPHIN_REF_ROOT, else where this container mounts it
REF_ROOT = Path(os.environ.get("DOLPHIN_REF_ROOT", "/root/reference"))
REF_SRC = REF_ROOT / "src" / "dolphin"

# --------------------------------------------------------------------------------------
# dtype canonicalisation (jax_enable_x64 = False)
# --------------------------------------------------------------------------------------
_CANON = {
    np.dtype(np.float64): np.dtype(np.float32),
    np.dtype(np.complex128): np.dtype(np.complex64),
    np.dtype(np.int64): np.dtype(np.int32),
    np.dtype(np.uint64): np.dtype(np.uint32),
}


def _canon(x):
    """Cast 64-bit numpy arrays/scalars to their 32-bit JAX counterparts."""
    if isinstance(x, np.ndarray):
        dt = _CANON.get(x.dtype)
        out = x.astype(dt) if dt is not None else x
        return out.view(JArr)
    if isinstance(x, np.generic):
        dt = _CANON.get(x.dtype)
        out = np.asarray(x.astype(dt) if dt is not None else x)
        return out.view(JArr)
    if isinstance(x, tuple):
        return tuple(_canon(v) for v in x)
    if isinstance(x, list):
        return [_canon(v) for v in x]
    return x


def _canon_input(x):
    """Canonicalise strongly-typed numpy inputs; Python scalars stay weak."""
    if isinstance(x, (np.ndarray, np.generic)):
        dt = _CANON.get(x.dtype)
        if dt is not None:
            return np.asarray(x).astype(dt)
        return np.asarray(x) if isinstance(x, np.generic) else x.view(np.ndarray)
    return x


class _AtIndexer:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtSetter(self._arr, idx)


class _AtSetter:
    def __init__(self, arr, idx):
        self._arr = arr
        self._idx = idx

    def set(self, value):
        out = np.array(self._arr, copy=True)
        out[self._idx] = value
        return _canon(out)


class JArr(np.ndarray):
    """ndarray view with JAX-like dtype canonicalisation and ``.at`` updates."""

    @property
    def at(self):
        return _AtIndexer(self)

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        ins = [_canon_input(i) for i in inputs]
        if "out" in kwargs:
            kwargs["out"] = tuple(
                o.view(np.ndarray) if isinstance(o, np.ndarray) else o
                for o in kwargs["out"]
            )
        res = getattr(ufunc, method)(*ins, **kwargs)
        return _canon(res)

    def __array_function__(self, func, types_, args, kwargs):
        def strip(v):
            if isinstance(v, JArr):
                return v.view(np.ndarray)
            if isinstance(v, (list, tuple)):
                return type(v)(strip(x) for x in v)
            return v

        res = func(*strip(args), **{k: strip(v) for k, v in kwargs.items()})
        return _canon(res)


def _wrap_np(fn):
    @functools.wraps(fn)
    def inner(*args, **kwargs):
        args = [_canon_input(a) if isinstance(a, (np.ndarray, np.generic)) else a for a in args]
        return _canon(fn(*args, **kwargs))

    return inner


class _JnpModule(types.ModuleType):
    """``jax.numpy`` stand-in: numpy functions with canonicalised outputs."""

    def __getattr__(self, name):
        obj = getattr(np, name)
        if callable(obj) and not isinstance(obj, type):
            return _wrap_np(obj)
        return obj


def _asarray(x, dtype=None):
    a = np.asarray(x, dtype=dtype)
    return _canon(a)


# --------------------------------------------------------------------------------------
# jax transformations
# --------------------------------------------------------------------------------------
def jit(fun=None, **_kw):
    if fun is None:
        return lambda f: f
    return fun


def vmap(fun, in_axes=0, out_axes=0):
    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        sizes = {np.shape(a)[0] for a, ax in zip(args, axes) if ax is not None}
        (n,) = sizes
        outs = []
        for k in range(n):
            call = [a[k] if ax is not None else a for a, ax in zip(args, axes)]
            outs.append(fun(*call))
        if isinstance(outs[0], tuple):
            return tuple(_canon(np.stack([np.asarray(o[i]) for o in outs])) for i in range(len(outs[0])))
        return _canon(np.stack([np.asarray(o) for o in outs]))

    return mapped


def _clamp(lo, x, hi):
    return np.minimum(np.maximum(x, lo), hi)


def _dynamic_slice(arr, start_indices, slice_sizes):
    """``lax.dynamic_slice``: each start is clamped into [0, dim - size]."""
    arr = np.asarray(arr)
    idx = []
    for dim, st, sz in zip(arr.shape, start_indices, slice_sizes):
        if sz > dim:
            raise TypeError("slice size larger than operand")
        st = int(np.clip(int(st), 0, dim - sz))
        idx.append(slice(st, st + sz))
    return _canon(arr[tuple(idx)])


def _select(pred, on_true, on_false):
    return _canon(np.where(np.asarray(pred), np.asarray(on_true), np.asarray(on_false)))


def _while_loop(cond_fun, body_fun, init_val):
    val = init_val
    while bool(np.asarray(cond_fun(val))):
        val = body_fun(val)
    return val


# --------------------------------------------------------------------------------------
# jax.scipy.linalg (batched, NaN on failure like jaxlib)
# --------------------------------------------------------------------------------------
def _batched(fn, a, *rest):
    a = np.asarray(a)
    if a.ndim == 2:
        return fn(a, *rest)
    flat = a.reshape(-1, *a.shape[-2:])
    outs = [fn(flat[i], *[np.asarray(r).reshape(-1, *np.asarray(r).shape[-2:])[i] for r in rest]) for i in range(flat.shape[0])]
    return np.stack(outs).reshape(*a.shape[:-2], *outs[0].shape)


def _cho_factor_single(a, lower):
    try:
        c, _ = sla.cho_factor(a, lower=lower, check_finite=False)
        if lower:
            c = np.tril(c)
        else:
            c = np.triu(c)
        if not np.all(np.isfinite(c)):
            return np.full_like(a, np.nan)
        return c
    except (np.linalg.LinAlgError, sla.LinAlgError):
        return np.full_like(a, np.nan)


def cho_factor(a, lower=False, **_kw):
    a = _canon_input(np.asarray(a))
    return _canon(_batched(lambda m: _cho_factor_single(m, lower), a)), lower


def cho_solve(c_and_lower, b, **_kw):
    c, lower = c_and_lower
    c = np.asarray(c)
    b = _canon_input(np.asarray(b))

    def single(cm, bm):
        if not np.all(np.isfinite(cm)):
            return np.full(bm.shape, np.nan, dtype=np.result_type(cm, bm))
        return sla.cho_solve((cm, lower), bm, check_finite=False)

    return _canon(_batched(single, c, b))


def solve(a, b, assume_a="gen", **_kw):
    a = _canon_input(np.asarray(a))
    b = _canon_input(np.asarray(b))

    def single(am, bm):
        try:
            return sla.solve(am, bm, assume_a=assume_a, check_finite=False)
        except (np.linalg.LinAlgError, sla.LinAlgError, ValueError):
            return np.full(bm.shape, np.nan, dtype=np.result_type(am, bm))

    return _canon(_batched(single, a, b))


def lu_factor(a, **_kw):
    a = _canon_input(np.asarray(a))
    lu, piv = sla.lu_factor(a, check_finite=False)
    return _canon(lu), _canon(piv)


def lu_solve(lu_and_piv, b, **_kw):
    lu, piv = lu_and_piv
    return _canon(sla.lu_solve((np.asarray(lu), np.asarray(piv)), _canon_input(np.asarray(b)), check_finite=False))


# --------------------------------------------------------------------------------------
# registration
# --------------------------------------------------------------------------------------
def _module(name, **attrs):
    m = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    sys.modules[name] = m
    return m


def _install_jax():
    jnp = _JnpModule("jax.numpy")
    jnp.asarray = _asarray
    jnp.array = _asarray
    jnp.linalg = types.SimpleNamespace(norm=_wrap_np(np.linalg.norm))
    sys.modules["jax.numpy"] = jnp
    lax = _module(
        "jax.lax",
        clamp=_clamp,
        dynamic_slice=_dynamic_slice,
        select=_select,
        while_loop=_while_loop,
    )
    linalg = _module(
        "jax.scipy.linalg",
        cho_factor=cho_factor,
        cho_solve=cho_solve,
        solve=solve,
        lu_factor=lu_factor,
        lu_solve=lu_solve,
    )
    jscipy = _module("jax.scipy", linalg=linalg)
    jtyping = _module("jax.typing", ArrayLike=object)
    _module(
        "jax",
        numpy=jnp,
        lax=lax,
        scipy=jscipy,
        typing=jtyping,
        jit=jit,
        vmap=vmap,
        Array=np.ndarray,
    )


def _install_numba():
    def njit(*args, **_kw):
        if len(args) == 1 and callable(args[0]):
            return args[0]
        return lambda f: f

    cuda = _module("numba.cuda", jit=njit, grid=None)
    _module("numba", njit=njit, jit=njit, prange=range, cuda=cuda)


def _install_osgeo():
    gdal = _module("osgeo.gdal", UseExceptions=lambda: None)
    _module("osgeo", gdal=gdal, gdal_array=_module("osgeo.gdal_array"), gdalconst=_module("osgeo.gdalconst"))


def _load_file(modname, path):
    spec = importlib.util.spec_from_file_location(modname, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[modname] = mod
    spec.loader.exec_module(mod)
    return mod


def _package(modname, path):
    pkg = types.ModuleType(modname)
    pkg.__path__ = [str(path)]
    sys.modules[modname] = pkg
    return pkg


def load_function(path, name, **names):
    """One top-level function of a reference source file, run from its own source text
    with ``numpy`` and ``names`` as its globals (for modules whose imports are out of
    reach here, such as ``timeseries.py``)."""
    import ast

    text = Path(path).read_text()
    for node in ast.parse(text).body:
        if isinstance(node, ast.FunctionDef) and node.name == name:
            ns = {"np": np, "annotations": None, **names}
            code = "from __future__ import annotations\n" + ast.get_source_segment(text, node)
            exec(compile(code, str(path), "exec"), ns)
            return ns[name]
    raise KeyError(f"{name} not found in {path}")


_LOADED = None


def load_reference():
    """Return a namespace with the reference's hot-path modules, loaded from source."""
    global _LOADED
    if _LOADED is not None:
        return _LOADED
    if not REF_SRC.exists():
        raise FileNotFoundError(f"reference checkout not found at {REF_SRC}")
    _install_jax()
    _install_numba()
    _install_osgeo()

    dolphin = _package("dolphin", REF_SRC)
    types_mod = _load_file("dolphin._types", REF_SRC / "_types.py")
    dolphin.Strides = types_mod.Strides
    dolphin.HalfWindow = types_mod.HalfWindow
    utils = _load_file("dolphin.utils", REF_SRC / "utils.py")
    dolphin.utils = utils
    enums = _load_file("dolphin._ref_enums", REF_SRC / "workflows" / "config" / "_enums.py")
    _module("dolphin.workflows", ShpMethod=enums.ShpMethod)
    # dolphin.io is only needed for names imported at the top of ps.py
    _module(
        "dolphin.io",
        EagerLoader=object,
        StackReader=object,
        repack_raster=lambda *a, **k: None,
    )
    dolphin.io = sys.modules["dolphin.io"]

    pl = _package("dolphin.phase_link", REF_SRC / "phase_link")
    cov = _load_file("dolphin.phase_link.covariance", REF_SRC / "phase_link" / "covariance.py")
    crlb = _load_file("dolphin.phase_link.crlb", REF_SRC / "phase_link" / "crlb.py")
    metrics = _load_file("dolphin.phase_link.metrics", REF_SRC / "phase_link" / "metrics.py")
    closure = _load_file("dolphin.phase_link._closure_phase", REF_SRC / "phase_link" / "_closure_phase.py")
    eigs = _load_file("dolphin.phase_link._eigenvalues", REF_SRC / "phase_link" / "_eigenvalues.py")
    fill = _load_file("dolphin.phase_link._ps_filling", REF_SRC / "phase_link" / "_ps_filling.py")
    pl.covariance, pl.crlb, pl.metrics = cov, crlb, metrics
    core = _load_file("dolphin.phase_link._core", REF_SRC / "phase_link" / "_core.py")
    compress = _load_file("dolphin.phase_link._compress", REF_SRC / "phase_link" / "_compress.py")

    shp = _package("dolphin.shp", REF_SRC / "shp")
    _load_file("dolphin.shp._common", REF_SRC / "shp" / "_common.py")
    glrt = _load_file("dolphin.shp._glrt", REF_SRC / "shp" / "_glrt.py")
    ks = _load_file("dolphin.shp._ks", REF_SRC / "shp" / "_ks.py")
    shp._glrt, shp._ks = glrt, ks
    shp_init = _load_file("dolphin.shp.__init__", REF_SRC / "shp" / "__init__.py")

    ps = _load_file("dolphin.ps", REF_SRC / "ps.py")
    similarity = _load_file("dolphin.similarity", REF_SRC / "similarity.py")
    # the block manager and the ministack planner (file names and dates only; the
    # date parser of opera_utils is never reached for real SLCs given as dates)
    blocks = _load_file("dolphin.io._blocks", REF_SRC / "io" / "_blocks.py")
    dolphin.io.DEFAULT_DATETIME_FORMAT = "%Y%m%d"
    _module("opera_utils", get_dates=lambda *a, **k: (_ for _ in ()).throw(NotImplementedError("get_dates")))
    stack = _load_file("dolphin.stack", REF_SRC / "stack.py")
    incidence = load_function(REF_SRC / "timeseries.py", "get_incidence_matrix", flatten=utils.flatten)

    _LOADED = types.SimpleNamespace(
        types=types_mod,
        utils=utils,
        covariance=cov,
        crlb=crlb,
        metrics=metrics,
        closure=closure,
        eigs=eigs,
        fill=fill,
        core=core,
        compress=compress,
        glrt=glrt,
        ks=ks,
        shp=shp_init,
        ps=ps,
        similarity=similarity,
        get_incidence_matrix=incidence,
        blocks=blocks,
        stack=stack,
        ShpMethod=enums.ShpMethod,
    )
    return _LOADED
