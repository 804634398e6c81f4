"""Numpy restatement of dolphin's phase-linking hot path (ORACLE, test infrastructure).

Every function cites the reference file:line it restates (paths are relative
to the dolphin checkout, ``src/dolphin/...``).  Precision is a parameter:

* ``dtype=np.float32`` (default) follows the reference's arithmetic: jax runs
  with x64 disabled, so the reference computes in float32/complex64;
* ``dtype=np.float64`` is the same algorithm in float64/complex128, used as
  the high-precision oracle that every GPU result's error is stated against.

The functions are vectorised over pixels (loops only over the matrix order N
or the window), so a few hundred thousand pixels run in seconds to minutes.
Linear algebra that the reference delegates to LAPACK through jax
(``cho_factor``/``cho_solve``, ``lu_factor``/``lu_solve``, ``solve``) is
restated here with the same algorithms (Cholesky; LU with partial pivoting
choosing the first maximum of ``|re|+|im|`` as ``icamax`` does), returning
NaNs on failure as jaxlib does.
"""

from __future__ import annotations

import math
import warnings
from typing import NamedTuple, Optional

import numpy as np

__all__ = [
    "PhaseLinkOutput",
    "PhaseLinkRuntimeError",
    "calc_ps_block",
    "closure_phases",
    "compress",
    "compute_out_shape",
    "decimate",
    "estimate_neighbors",
    "estimate_neighbors_glrt",
    "estimate_neighbors_ks",
    "estimate_stack_covariance",
    "estimate_temp_coh",
    "fill_ps_pixels",
    "get_max_idxs",
    "glrt_threshold",
    "ks_critical_distance",
    "ks_max_cdf_dist",
    "process_coherence_matrices",
    "run_phase_linking",
    "take_looks",
    "upsample_nearest",
]


class PhaseLinkRuntimeError(Exception):
    """Mirror of ``PhaseLinkRuntimeError`` (phase_link/_core.py:29-30)."""


class PhaseLinkOutput(NamedTuple):
    """Mirror of ``PhaseLinkOutput`` (phase_link/_core.py:40-64)."""

    cpx_phase: np.ndarray
    temp_coh: np.ndarray
    shp_counts: np.ndarray
    eigenvalues: np.ndarray
    estimator: np.ndarray
    crlb_std_dev: np.ndarray
    closure_phases: np.ndarray


def _cdt(dtype):
    return np.complex64 if np.dtype(dtype) == np.float32 else np.complex128


# --------------------------------------------------------------------------------------
# index helpers  (utils.py:99-107, 172-278, 528-564; phase_link/_core.py:537-561)
# --------------------------------------------------------------------------------------
def compute_out_shape(shape, strides):
    """utils.py:528-564: ``(rows // sy, cols // sx)``."""
    return (shape[0] // strides[0], shape[1] // strides[1])


def _make_dims_multiples(arr, ry, rx, how):
    """utils.py:253-278."""
    rows, cols = arr.shape[-2:]
    rc, cc = rows % ry, cols % rx
    if how == "cutoff":
        return arr[..., : rows - rc, : cols - cc]
    if how == "pad":
        pr, pc = (ry - rc) % ry, (rx - cc) % rx
        if pr or pc:
            pad_val = False if arr.dtype == bool else np.nan
            widths = [(0, 0)] * (arr.ndim - 2) + [(0, pr), (0, pc)]
            arr = np.pad(arr, widths, mode="constant", constant_values=pad_val)
        return arr
    raise ValueError(f"Invalid edge strategy: {how}")


def take_looks(arr, row_looks, col_looks, func_type="nansum", edge_strategy="cutoff"):
    """utils.py:172-250 (2-D or stacked 3-D input)."""
    if row_looks == 1 and col_looks == 1:
        return arr
    arr = _make_dims_multiples(arr, row_looks, col_looks, edge_strategy)
    rows, cols = arr.shape[-2:]
    nr, nc = rows // row_looks, cols // col_looks
    shaped = arr.reshape(*arr.shape[:-2], nr, row_looks, nc, col_looks)
    func = getattr(np, func_type)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", category=RuntimeWarning)
        return func(shaped, axis=(-1, -3))


def decimate(arr, strides):
    """phase_link/_core.py:537-561."""
    ys, xs = strides
    rows, cols = arr.shape[-2:]
    return arr[..., ys // 2 : (rows // ys) * ys + 1 : ys, xs // 2 : (cols // xs) * xs + 1 : xs]


def _window_starts(centers, half, size, dim):
    """Start of a ``lax.dynamic_slice`` window (covariance.py:159-170, shp/_glrt.py:204-208).

    The start ``c - half`` is clamped into ``[0, dim - size]``: windows near an edge
    are shifted inwards, not truncated.
    """
    return np.clip(centers - half, 0, dim - size)


# --------------------------------------------------------------------------------------
# PS selection  (ps.py:169-244)
# --------------------------------------------------------------------------------------
def calc_ps_block(stack_mag, amp_dispersion_threshold=0.25, min_count=None):
    """ps.py:169-244: amplitude mean, dispersion and PS mask."""
    stack_mag = np.asarray(stack_mag)
    if np.iscomplexobj(stack_mag):
        raise ValueError("The input `stack_mag` must be real-valued.")
    if min_count is None:
        min_count = int(0.9 * stack_mag.shape[0])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", category=RuntimeWarning)
        mean = np.nanmean(stack_mag, axis=0)
        std_dev = np.nanstd(stack_mag, axis=0)
        count = np.count_nonzero(~np.isnan(stack_mag), axis=0)
        amp_disp = std_dev / mean
    amp_disp[count < min_count] = np.nan
    mean = np.nan_to_num(mean, nan=0, posinf=0, neginf=0, copy=False)
    amp_disp = np.nan_to_num(amp_disp, nan=0, posinf=0, neginf=0, copy=False)
    ps = amp_disp < amp_dispersion_threshold
    ps[amp_disp == 0] = False
    return mean, amp_disp, ps


# --------------------------------------------------------------------------------------
# SHP: GLRT  (shp/_glrt.py:13-130) and KS  (shp/_ks.py:22-239)
# --------------------------------------------------------------------------------------
def glrt_threshold(alpha):
    """shp/_glrt.py:78: chi-square(1) quantile at 1 - alpha (float64)."""
    from scipy import stats

    return float(stats.chi2.ppf(1 - alpha, df=1))


def _out_centers(out_n, stride):
    return stride // 2 + np.arange(out_n) * stride


def estimate_neighbors_glrt(
    mean, var, halfwin_rowcol, strides=(1, 1), nslc=1, alpha=0.001, dtype=np.float32,
    return_stat=False, exact=False,
):
    """shp/_glrt.py:13-130.

    Rayleigh scale^2 = (var + mean^2)/2; statistic
    ``T = nslc * (2 log((s1+s2)/2) - log s1 - log s2)``; SHP where ``threshold > T``.
    The comparison window is ``dynamic_slice``-clamped (shifted at edges), while the
    validity mask is taken from the unshifted window origin; the window centre
    ``[hy, hx]`` is always False.

    ``exact``: decide on the statistic evaluated in float64 from the ``dtype`` scale^2,
    as ``nslc * log1p((s1 - s2)^2 / (4 s1 s2))`` (algebraically the same, without the
    cancellation of the three logs), against the ``dtype`` threshold.  The returned
    statistic is then that float64 value.
    """
    dt = np.dtype(dtype)
    mean = np.asarray(mean, dtype=dt)
    var = np.asarray(var, dtype=dt)
    rows, cols = mean.shape
    hy, hx = halfwin_rowcol
    sy, sx = strides
    wy, wx = 2 * hy + 1, 2 * hx + 1
    out_rows, out_cols = compute_out_shape((rows, cols), (sy, sx))
    scale2 = (var + mean**2) / 2
    thr = dt.type(glrt_threshold(alpha))

    in_r = _out_centers(out_rows, sy)
    in_c = _out_centers(out_cols, sx)
    r0 = _window_starts(in_r, hy, wy, rows)
    c0 = _window_starts(in_c, hx, wx, cols)
    rr = r0[:, None] + np.arange(wy)[None, :]  # (R', wy)
    cc = c0[:, None] + np.arange(wx)[None, :]  # (C', wx)
    s2 = scale2[rr[:, None, :, None], cc[None, :, None, :]]  # (R', C', wy, wx)
    s1 = scale2[in_r[:, None], in_c[None, :]][:, :, None, None]
    with np.errstate(all="ignore"):
        pooled = (s1 + s2) / 2
        stat = nslc * (2 * np.log(pooled) - np.log(s1) - np.log(s2))
        if exact:
            a1, a2 = s1.astype(np.float64), s2.astype(np.float64)
            stat = float(nslc) * np.log1p((a1 - a2) ** 2 / (4.0 * a1 * a2))
            thr = np.float64(thr)
    is_shp = thr > stat
    ur0 = in_r - hy
    uc0 = in_c - hx
    wr = np.arange(wy)
    wc = np.arange(wx)
    valid_r = (wr[None, :] >= -ur0[:, None]) & (wr[None, :] < rows - ur0[:, None])
    valid_c = (wc[None, :] >= -uc0[:, None]) & (wc[None, :] < cols - uc0[:, None])
    valid = valid_r[:, None, :, None] & valid_c[None, :, None, :]
    is_shp &= valid
    is_shp[:, :, hy, hx] = False
    if return_stat:
        return is_shp, stat, thr
    return is_shp


def ks_critical_distance(nslc, alpha):
    """shp/_ks.py:221-239: scan from 0.01 in 0.001 steps of the Kolmogorov series."""
    n_eff = nslc / 2.0
    cur_dist = 0.01
    critical_distance = 0.1
    sqrt_n = math.sqrt(n_eff)
    while cur_dist <= 1.0:
        value = cur_dist * (sqrt_n + 0.12 + 0.11 / sqrt_n)
        pvalue = 0
        for t in range(1, 101):
            pvalue += ((-1) ** (t - 1)) * math.exp(-2 * (value**2) * (t**2))
        pvalue = max(0.0, min(1.0, 2 * pvalue))
        if pvalue <= alpha:
            critical_distance = cur_dist
            break
        cur_dist += 0.001
    return critical_distance


def ks_max_cdf_dist(x1, x2):
    """shp/_ks.py:164-218, vectorised over leading axes.

    ``x1``, ``x2``: sorted samples along the last axis (same length n).  Walks the
    merge exactly as the reference does: one step per sample, both arrays stepping
    together on a tie (a comparison with NaN counts as a tie), ECDFs accumulated by
    repeated float64 additions of ``1/n``.
    """
    x1 = np.asarray(x1)
    x2 = np.asarray(x2)
    x1, x2 = np.broadcast_arrays(x1, x2)
    n = x1.shape[-1]
    shape = x1.shape[:-1]
    a = x1.reshape(-1, n)
    b = x2.reshape(-1, n)
    m = a.shape[0]
    i1 = np.zeros(m, np.int64)
    i2 = np.zeros(m, np.int64)
    i_out = np.zeros(m, np.int64)
    cdf1 = np.zeros(m, np.float64)
    cdf2 = np.zeros(m, np.float64)
    max_dist = np.zeros(m, np.float64)
    step = 1 / n
    rows = np.arange(m)
    pad_a = np.concatenate([a, np.zeros((m, 1), a.dtype)], axis=1)
    pad_b = np.concatenate([b, np.zeros((m, 1), b.dtype)], axis=1)
    while True:
        act = i_out < 2 * n
        if not act.any():
            break
        va = pad_a[rows, i1]
        vb = pad_b[rows, i2]
        c_end1 = act & (i1 == n)
        rest = act & ~c_end1
        with np.errstate(invalid="ignore"):
            c_adv1 = rest & ((i2 == n) | (va < vb))
            rest2 = rest & ~c_adv1
            c_adv2 = rest2 & (va > vb)
        c_tie = rest2 & ~c_adv2
        cdf2 = np.where(c_end1 | c_adv2 | c_tie, cdf2 + step, cdf2)
        cdf1 = np.where(c_adv1 | c_tie, cdf1 + step, cdf1)
        i2 = i2 + (c_end1 | c_adv2 | c_tie)
        i1 = i1 + (c_adv1 | c_tie)
        i_out = i_out + act + c_tie
        max_dist = np.where(act, np.maximum(max_dist, np.abs(cdf1 - cdf2)), max_dist)
    return max_dist.reshape(shape)


def estimate_neighbors_ks(amp_stack, halfwin_rowcol, strides=(1, 1), alpha=0.001, is_sorted=False):
    """shp/_ks.py:22-98, 139-161.

    Windows are truncated at the image edge (utils.py:99-107); a truncated window
    gets no neighbours at all.  Centre is False.
    """
    amp = np.asarray(amp_stack)
    sorted_amp = amp if is_sorted else np.sort(amp, axis=0)
    n, rows, cols = sorted_amp.shape
    cutoff = ks_critical_distance(n, alpha)
    hy, hx = halfwin_rowcol
    sy, sx = strides
    wy, wx = 2 * hy + 1, 2 * hx + 1
    out_rows, out_cols = compute_out_shape((rows, cols), (sy, sx))
    is_shp = np.zeros((out_rows, out_cols, wy, wx), dtype=bool)
    in_r = _out_centers(out_rows, sy)
    in_c = _out_centers(out_cols, sx)
    full_r = (in_r - hy >= 0) & (in_r + hy + 1 <= rows)
    full_c = (in_c - hx >= 0) & (in_c + hx + 1 <= cols)
    ors = np.nonzero(full_r)[0]
    ocs = np.nonzero(full_c)[0]
    if len(ors) == 0 or len(ocs) == 0:
        return is_shp
    px = np.moveaxis(sorted_amp, 0, -1)  # (rows, cols, n)
    for a in range(wy):
        for b in range(wx):
            if a == hy and b == hx:
                continue
            x1 = px[in_r[ors][:, None], in_c[ocs][None, :]]
            x2 = px[(in_r[ors] - hy + a)[:, None], (in_c[ocs] - hx + b)[None, :]]
            d = ks_max_cdf_dist(x1, x2)
            is_shp[ors[:, None], ocs[None, :], a, b] = d < cutoff
    return is_shp


def estimate_neighbors(
    *, halfwin_rowcol, alpha, strides=None, mean=None, var=None, nslc=None,
    amp_stack=None, is_sorted=False, method="glrt", prune_disconnected=False,
):
    """shp/__init__.py:19-116 (dispatcher).  ``prune_disconnected`` is ignored."""
    if strides is None:
        strides = (1, 1)
    method = str(getattr(method, "value", method)).lower()
    if method == "rect":
        return None
    if method == "glrt":
        if nslc is None:
            raise ValueError("`nslc` must be provided for GLRT method")
        if mean is None:
            mean = np.mean(amp_stack, axis=0)
        if var is None:
            var = np.var(amp_stack, axis=0)
        return estimate_neighbors_glrt(mean, var, halfwin_rowcol, tuple(strides), nslc, alpha)
    if method == "ks":
        if amp_stack is None:
            raise ValueError("amp_stack must be provided for KS method")
        return estimate_neighbors_ks(amp_stack, halfwin_rowcol, tuple(strides), alpha, is_sorted)
    raise ValueError(f"SHP method {method} is not implemented")


# --------------------------------------------------------------------------------------
# covariance  (phase_link/covariance.py:24-170)
# --------------------------------------------------------------------------------------
def estimate_stack_covariance(slc_stack, half_window, strides=(1, 1), neighbor_arrays=None,
                              dtype=np.float32, chunk=2048, out_pixels=None):
    """covariance.py:24-170: SHP-masked sample coherence matrix per output pixel.

    Returns ``(out_rows, out_cols, N, N)`` (or ``(len(out_pixels), N, N)`` when
    ``out_pixels`` -- a pair of flat row/col index arrays into the output grid --
    restricts the computation to a subset of pixels).
    """
    slc = np.asarray(slc_stack)
    if not np.iscomplexobj(slc):
        raise ValueError("The SLC stack must be complex.")
    cdt = _cdt(dtype)
    rdt = np.dtype(dtype)
    slc = slc.astype(cdt, copy=False)
    n, rows, cols = slc.shape
    hy, hx = half_window
    sy, sx = strides
    wy, wx = 2 * hy + 1, 2 * hx + 1
    if wy > rows or wx > cols:
        raise ValueError(f"window {(wy, wx)} larger than the SLC stack {(rows, cols)}")
    out_rows, out_cols = compute_out_shape((rows, cols), (sy, sx))
    if out_pixels is None:
        orr, occ = np.meshgrid(np.arange(out_rows), np.arange(out_cols), indexing="ij")
        orr, occ = orr.ravel(), occ.ravel()
        grid = True
    else:
        orr, occ = (np.asarray(v).ravel() for v in out_pixels)
        grid = False
    npx = orr.size
    out = np.zeros((npx, n, n), dtype=cdt)
    wr = np.arange(wy)
    wc = np.arange(wx)
    for s in range(0, npx, chunk):
        r_o = orr[s : s + chunk]
        c_o = occ[s : s + chunk]
        in_r = sy // 2 + r_o * sy
        in_c = sx // 2 + c_o * sx
        r0 = _window_starts(in_r, hy, wy, rows)
        c0 = _window_starts(in_c, hx, wx, cols)
        rr = (r0[:, None] + wr[None, :])[:, :, None]
        cc = (c0[:, None] + wc[None, :])[:, None, :]
        z = slc[:, rr, cc]  # (N, P, wy, wx)
        z = np.moveaxis(z, 0, 1).reshape(len(r_o), n, wy * wx)
        valid = ~np.isnan(z)
        if neighbor_arrays is not None:
            nb = np.asarray(neighbor_arrays)[r_o, c_o].reshape(len(r_o), 1, wy * wx)
            valid &= nb.astype(bool)
        zm = np.where(valid, z, cdt(0))
        numer = np.matmul(zm, np.conj(np.swapaxes(zm, -1, -2)))
        amp_vec = np.sum(np.abs(zm) ** 2, axis=-1, dtype=rdt)
        amp_mat = np.sqrt(amp_vec[:, :, None] * amp_vec[:, None, :])
        with np.errstate(all="ignore"):
            out[s : s + chunk] = np.where(amp_mat > 1e-6, numer / amp_mat, cdt(0))
    if grid:
        return out.reshape(out_rows, out_cols, n, n)
    return out


# --------------------------------------------------------------------------------------
# dense per-pixel linear algebra (restating the LAPACK routines the reference calls)
# --------------------------------------------------------------------------------------
def _cholesky_lower(a):
    """Batched Cholesky (potrf semantics): lower factor, NaN matrix on failure."""
    a = np.array(a, copy=True)
    bsz, n, _ = a.shape
    L = np.zeros_like(a)
    ok = np.ones(bsz, dtype=bool)
    with np.errstate(all="ignore"):
        for j in range(n):
            d = a[:, j, j] - np.sum(L[:, j, :j] * L[:, j, :j], axis=-1)
            ok &= d > 0
            ljj = np.sqrt(np.where(d > 0, d, 1))
            L[:, j, j] = ljj
            if j + 1 < n:
                s = a[:, j + 1 :, j] - np.einsum("bik,bk->bi", L[:, j + 1 :, :j], L[:, j, :j])
                L[:, j + 1 :, j] = s / ljj[:, None]
    L[~ok] = np.nan
    return L


def _cho_inverse(L):
    """``cho_solve((L, lower), I)``: inverse of L L^T by two triangular solves."""
    bsz, n, _ = L.shape
    eye = np.broadcast_to(np.eye(n, dtype=L.dtype), L.shape)
    y = np.zeros_like(L)
    with np.errstate(all="ignore"):
        for i in range(n):
            s = eye[:, i, :] - np.einsum("bk,bkj->bj", L[:, i, :i], y[:, :i, :])
            y[:, i, :] = s / L[:, i, i][:, None]
        x = np.zeros_like(L)
        for i in range(n - 1, -1, -1):
            s = y[:, i, :] - np.einsum("bk,bkj->bj", L[:, i + 1 :, i], x[:, i + 1 :, :])
            x[:, i, :] = s / L[:, i, i][:, None]
    return x


def _lu_factor(a):
    """Batched LU with partial pivoting (getrf semantics, pivot = first max |re|+|im|)."""
    lu = np.array(a, copy=True)
    bsz, n, _ = lu.shape
    piv = np.zeros((bsz, n), dtype=np.int64)
    b = np.arange(bsz)
    with np.errstate(all="ignore"):
        for k in range(n):
            col = lu[:, k:, k]
            p = k + np.argmax(np.abs(col.real) + np.abs(col.imag), axis=1)
            piv[:, k] = p
            rk = lu[b, k, :].copy()
            lu[b, k, :] = lu[b, p, :]
            lu[b, p, :] = rk
            pv = lu[:, k, k]
            nz = pv != 0
            recip = np.where(nz, 1 / np.where(nz, pv, 1), 0).astype(lu.dtype)
            if k + 1 < n:
                lu[:, k + 1 :, k] = np.where(nz[:, None], lu[:, k + 1 :, k] * recip[:, None], lu[:, k + 1 :, k])
                lu[:, k + 1 :, k + 1 :] -= lu[:, k + 1 :, k][:, :, None] * lu[:, k, k + 1 :][:, None, :]
    return lu, piv


def _lu_solve(lu, piv, rhs):
    """Batched ``lu_solve``: apply row swaps, unit-lower then upper triangular solves."""
    bsz, n, _ = lu.shape
    x = np.array(rhs, copy=True)
    b = np.arange(bsz)
    for k in range(n):
        p = piv[:, k]
        xk = x[b, k].copy()
        x[b, k] = x[b, p]
        x[b, p] = xk
    with np.errstate(all="ignore"):
        for i in range(1, n):
            x[:, i] = x[:, i] - np.sum(lu[:, i, :i] * x[:, :i], axis=-1)
        for i in range(n - 1, -1, -1):
            x[:, i] = (x[:, i] - np.sum(lu[:, i, i + 1 :] * x[:, i + 1 :], axis=-1)) / lu[:, i, i]
    return x


def _norm(v):
    return np.sqrt(np.sum((v.real * v.real + v.imag * v.imag), axis=-1))


def power_iteration(A, tol=1e-5, max_iters=50, return_active=False):
    """phase_link/_eigenvalues.py:93-136, batched over pixels (A: (B, n, n)); with
    ``return_active`` also the pixels that missed the stopping rule."""
    bsz, n, _ = A.shape
    cdt = A.dtype
    v = np.ones((bsz, n), dtype=cdt)
    v = v / _norm(v)[:, None]
    active = np.ones(bsz, dtype=bool)
    iters = 1
    with np.errstate(all="ignore"):
        while active.any() and iters < max_iters:
            av = np.einsum("bij,bj->bi", A[active], v[active])
            nv = av / _norm(av)[:, None]
            diff = _norm(nv - v[active])
            v[active] = nv
            still = diff > tol
            idx = np.nonzero(active)[0]
            active[idx[~still]] = False
            iters += 1
        lam = np.einsum("bi,bij,bj->b", np.conj(v), A, v)
    if return_active:
        return lam.real, v, active
    return lam.real, v


def inverse_iteration(A, mu, tol=1e-5, max_iters=50, return_active=False):
    """phase_link/_eigenvalues.py:139-205, batched over pixels."""
    bsz, n, _ = A.shape
    cdt = A.dtype
    v = np.ones((bsz, n), dtype=cdt)
    v = v / _norm(v)[:, None]
    shifted = A - cdt.type(mu) * np.eye(n, dtype=cdt)
    lu, piv = _lu_factor(shifted)
    active = np.ones(bsz, dtype=bool)
    iters = 1
    with np.errstate(all="ignore"):
        while active.any() and iters < max_iters:
            x = _lu_solve(lu[active], piv[active], v[active])
            nv = x / _norm(x)[:, None]
            diff = _norm(nv - v[active])
            v[active] = nv
            still = diff > tol
            idx = np.nonzero(active)[0]
            active[idx[~still]] = False
            iters += 1
        lam = np.einsum("bi,bij,bj->b", np.conj(v), A, v)
    if return_active:
        return lam.real, v, active
    return lam.real, v


def eigh_fallback_vectors(A, target):
    """The fallback for pixels whose eigen-iteration missed its stopping rule (not in the
    reference): the eigenvector of the Hermitian A (B, n, n), in float64, whose eigenvalue
    is nearest 0.99 (``target="emi"``, the shifted inverse iteration's limit) or largest in
    magnitude (``"evd"``, power iteration's limit); returns (eigenvalues, unit vectors)."""
    A64 = np.asarray(A).astype(np.complex128)
    w, V = np.linalg.eigh(A64)
    k = np.argmin(np.abs(w - 0.99), axis=-1) if target == "emi" else np.argmax(np.abs(w), axis=-1)
    b = np.arange(A64.shape[0])
    return w[b, k], V[b, :, k]


def _crlb(gamma, gamma_inv, num_looks, ref, fim_jitter=1e-6):
    """phase_link/crlb.py:132-189 (``aps_variance`` = 0 path)."""
    bsz, n, _ = gamma.shape
    eye = np.eye(n, dtype=gamma.dtype)
    X = 2.0 * num_looks * (gamma * gamma_inv - eye)
    X = X.astype(gamma.dtype)
    idx = np.concatenate([np.arange(ref), np.arange(ref + 1, n)])
    fim = X[:, idx[:, None], idx[None, :]]
    if fim_jitter != 0.0:
        fim = fim + gamma.dtype.type(fim_jitter) * np.eye(n - 1, dtype=gamma.dtype)
    L = _cholesky_lower(fim)
    sigma = _cho_inverse(L)
    with np.errstate(all="ignore"):
        sig = np.sqrt(np.diagonal(sigma, axis1=-2, axis2=-1))
    return np.insert(sig, ref, 0.0, axis=-1)


def process_coherence_matrices(C, use_evd=False, beta=0.0, zero_correlation_threshold=0.0,
                               reference_idx=0, num_looks=1.0, first_real_slc_idx=0,
                               compute_crlb=True, eigh_fallback=False, nonconverged=None):
    """phase_link/_core.py:379-534 on a batch of matrices C: (B, n, n).

    Returns (referenced eigenvector (B, n), eigenvalue (B,), estimator (B,) uint8,
    crlb (B, n)).  ``eigh_fallback`` (not in the reference): pixels whose iteration for
    the chosen estimator missed the stopping rule get the float64 dense eigenvector
    (``eigh_fallback_vectors``; for EMI with |Gamma| inverted in float64); their mask is
    written to ``nonconverged`` (a (B,) bool array) when given.
    """
    C = np.asarray(C)
    bsz, n, _ = C.shape
    rdt = C.real.dtype
    evd_vals, evd_vecs, evd_active = power_iteration(C * np.abs(C), return_active=True)
    gamma = np.abs(C)
    eye = np.eye(n, dtype=rdt)
    if beta > 0:
        gamma = ((1 - beta) * gamma + beta * eye).astype(rdt)
    gamma = np.where(gamma < zero_correlation_threshold, rdt.type(0), gamma)
    L = _cholesky_lower(gamma + rdt.type(1e-6) * eye)
    gamma_inv = _cho_inverse(L)
    if eigh_fallback and evd_active.any():
        w, V = eigh_fallback_vectors((C * np.abs(C))[evd_active], "evd")
        evd_vals = evd_vals.copy()
        evd_vecs = evd_vecs.copy()
        evd_vals[evd_active] = w
        evd_vecs[evd_active] = V.astype(C.dtype)
    if use_evd:
        vals, vecs = evd_vals, evd_vecs
        estimator = np.zeros(bsz, dtype=np.uint8)
        active = evd_active
    else:
        emi_vals, emi_vecs, emi_active = inverse_iteration((gamma_inv * C).astype(C.dtype), 0.99,
                                                           return_active=True)
        bad = np.any(np.isnan(gamma_inv), axis=(-1, -2))
        fix = emi_active & ~bad
        if eigh_fallback and fix.any():
            g64 = gamma[fix].astype(np.float64) + 1e-6 * np.eye(n)
            A64 = np.linalg.inv(g64) * C[fix].astype(np.complex128)
            w, V = eigh_fallback_vectors(A64, "emi")
            emi_vals = emi_vals.copy()
            emi_vecs = emi_vecs.copy()
            emi_vals[fix] = w
            emi_vecs[fix] = V.astype(C.dtype)
        with np.errstate(all="ignore"):
            emi_vecs = (np.sqrt(rdt.type(n)) * emi_vecs / _norm(emi_vecs)[:, None]).astype(C.dtype)
        vecs = np.where(bad[:, None], evd_vecs, emi_vecs)
        vals = np.where(bad, evd_vals, emi_vals)
        estimator = np.where(bad, 0, 1).astype(np.uint8)
        active = np.where(bad, evd_active, emi_active)
    if nonconverged is not None:
        nonconverged[...] = active
    if compute_crlb:
        crlb = _crlb(gamma, gamma_inv, num_looks, max(first_real_slc_idx - 1, 0))
    else:
        crlb = np.zeros((bsz, n), dtype=rdt)
    ref = vecs[:, reference_idx]
    with np.errstate(all="ignore"):
        out = vecs * np.exp(-1j * np.angle(ref))[:, None].astype(C.dtype)
    return out.astype(C.dtype), vals.astype(rdt), estimator, crlb.astype(rdt)


def estimate_temp_coh(cpx_phase, C):
    """phase_link/metrics.py:10-97 with unit weights; cpx_phase (B, n), C (B, n, n)."""
    n = C.shape[-1]
    iu, ju = np.triu_indices(n, k=1)
    with np.errstate(all="ignore"):
        outer = cpx_phase[:, :, None] * np.conj(cpx_phase[:, None, :])
        reformed = np.angle(outer)
        diffs = np.exp(1j * np.angle(C)) * np.exp(-1j * reformed)
        up = diffs[:, iu, ju]
        isnan = np.isnan(up)
        total = np.sum(np.where(isnan, 0, up), axis=-1)
        count = np.sum(~isnan, axis=-1)
        out = np.abs(total / count)
    return np.nan_to_num(out, nan=0, posinf=0, neginf=0).astype(C.real.dtype)


def closure_phases(C):
    """phase_link/_closure_phase.py:6-40: angle(C[i,i+1] C[i+1,i+2] conj C[i,i+2])."""
    n = C.shape[-1]
    i = np.arange(n - 2)
    d1a = C[..., i, i + 1]
    d1b = C[..., i + 1, i + 2]
    d2 = C[..., i, i + 2]
    return np.angle(d1a * d1b * np.conj(d2)).astype(C.real.dtype)


# --------------------------------------------------------------------------------------
# PS filling  (phase_link/_ps_filling.py:16-153)
# --------------------------------------------------------------------------------------
def get_max_idxs(arr, row_looks, col_looks):
    """_ps_filling.py:118-153: brightest non-NaN pixel per look window (row-major,
    first maximum wins); windows that are all NaN are skipped."""
    arr = np.asarray(arr)
    h, w = arr.shape
    nh, nw = h // row_looks, w // col_looks
    if nh == 0 or nw == 0:
        return np.array([], dtype=np.int64), np.array([], dtype=np.int64)
    win = arr[: nh * row_looks, : nw * col_looks].reshape(nh, row_looks, nw, col_looks)
    win = win.transpose(0, 2, 1, 3).reshape(nh, nw, row_looks * col_looks).astype(np.float64)
    filled = np.where(np.isnan(win), -np.inf, win)
    k = np.argmax(filled, axis=-1)
    has = np.take_along_axis(filled, k[..., None], axis=-1)[..., 0] > -np.inf
    ii, jj = np.nonzero(has)
    kk = k[ii, jj]
    return ii * row_looks + kk // col_looks, jj * col_looks + kk % col_looks


def fill_ps_pixels(cpx_phase, temp_coh, slc_stack, ps_mask, strides, avg_mag,
                   reference_idx=0, use_max_ps=True):
    """_ps_filling.py:16-97 (mutates ``cpx_phase`` and ``temp_coh`` in place)."""
    if avg_mag is None:
        with warnings.catch_warnings():
            warnings.simplefilter("ignore", category=RuntimeWarning)
            avg_mag = np.nanmean(np.abs(slc_stack), axis=0)
    mag = np.array(avg_mag, copy=True)
    mag[~ps_mask] = np.nan
    ps_looked = take_looks(ps_mask, *strides, func_type="any", edge_strategy="pad")
    ps_looked = ps_looked[: cpx_phase.shape[1], : cpx_phase.shape[2]]
    if use_max_ps:
        r_idx, c_idx = get_max_idxs(mag, *strides)
        ref = np.exp(-1j * np.angle(slc_stack[reference_idx][r_idx, c_idx]))
        for i in range(len(slc_stack)):
            slc_phase = np.angle(slc_stack[i][r_idx, c_idx])
            cur_amp = np.abs(cpx_phase[i][ps_looked])
            cpx_phase[i][ps_looked] = cur_amp * (np.exp(1j * slc_phase) * ref)
    else:
        nanned = np.array(slc_stack, copy=True)
        nanned[:, ~ps_mask] = np.nan
        nanned[:, ps_mask] *= np.exp(-1j * np.angle(nanned[0, ps_mask]))[None]
        avg_ps = take_looks(nanned, *strides, func_type="nanmean", edge_strategy="pad")
        avg_ps = avg_ps[:, : cpx_phase.shape[1], : cpx_phase.shape[2]]
        ps_phases = np.angle(avg_ps[:, ps_looked])
        cpx_phase[:, ps_looked] = np.abs(cpx_phase[:, ps_looked]) * np.exp(1j * ps_phases)
    temp_coh[ps_looked] = 1


# --------------------------------------------------------------------------------------
# driver  (phase_link/_core.py:67-376)
# --------------------------------------------------------------------------------------
def _raise_if_all_nan(slc_stack):
    """phase_link/_core.py:564-571."""
    nans = np.isnan(slc_stack)
    bad = np.where(np.all(nans, axis=(1, 2)))[0]
    if bad.size > 0:
        raise PhaseLinkRuntimeError(f"slc_stack[{bad}] out of {len(slc_stack)} are all NaNs.")


def gamma_min_eig(C, beta=0.0, zero_correlation_threshold=0.0):
    """Smallest eigenvalue (float64) of the jittered ``|Gamma|`` that the EMI step factors.

    Not part of the reference: a diagnostic.  Where it is within rounding of zero,
    whether the float32 Cholesky (phase_link/_core.py:466-472) succeeds -- and so
    whether the pixel uses EMI or falls back to EVD -- is decided by rounding.
    """
    n = C.shape[-1]
    g = np.abs(np.asarray(C, dtype=np.complex128))
    eye = np.eye(n)
    if beta > 0:
        g = (1 - beta) * g + beta * eye
    g = np.where(g < zero_correlation_threshold, 0.0, g)
    return np.linalg.eigvalsh(g + 1e-6 * eye)[..., 0]


def run_cpl(slc_stack, half_window, strides, use_evd=False, beta=0.0,
            zero_correlation_threshold=0.0, reference_idx=0, neighbor_arrays=None,
            baseline_lag=None, first_real_slc_idx=0, compute_crlb=True, dtype=np.float32,
            chunk=2048, diagnostics=None, eigh_fallback=False):
    """phase_link/_core.py:252-376 (pixel-chunked so C is never held whole).

    ``diagnostics`` (a dict, optional) receives ``gamma_min_eig`` and ``nonconverged``
    (the iteration missed its stopping rule) per output pixel.
    """
    slc = np.asarray(slc_stack).astype(_cdt(dtype), copy=False)
    n, rows, cols = slc.shape
    hy, hx = half_window
    out_rows, out_cols = compute_out_shape((rows, cols), strides)
    npx = out_rows * out_cols
    rdt = np.dtype(dtype)
    cdt = _cdt(dtype)
    cpx = np.zeros((npx, n), cdt)
    temp_coh = np.zeros(npx, rdt)
    eig = np.zeros(npx, rdt)
    est = np.zeros(npx, np.uint8)
    crlb = np.zeros((npx, n), rdt)
    clos = np.zeros((npx, max(n - 2, 0)), rdt)
    num_looks = math.sqrt(hy * hx)
    reference_idx = n + reference_idx if reference_idx < 0 else reference_idx
    orr, occ = np.meshgrid(np.arange(out_rows), np.arange(out_cols), indexing="ij")
    orr, occ = orr.ravel(), occ.ravel()
    if baseline_lag:
        ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
        lag_zero = np.abs(ii - jj) >= baseline_lag
    ncv = np.zeros(npx, bool)
    if diagnostics is not None:
        diagnostics["gamma_min_eig"] = np.zeros((out_rows, out_cols), np.float64)
    for s in range(0, npx, chunk):
        sl = slice(s, s + chunk)
        C = estimate_stack_covariance(slc, half_window, strides, neighbor_arrays, dtype=dtype,
                                      chunk=chunk, out_pixels=(orr[sl], occ[sl]))
        if baseline_lag:
            C[:, lag_zero] = 0
        clos[sl] = closure_phases(C)
        if diagnostics is not None:
            diagnostics["gamma_min_eig"].reshape(-1)[sl] = gamma_min_eig(C, beta, zero_correlation_threshold)
        v, lam, e, cr = process_coherence_matrices(
            C, use_evd=use_evd, beta=beta, zero_correlation_threshold=zero_correlation_threshold,
            reference_idx=reference_idx, num_looks=num_looks,
            first_real_slc_idx=first_real_slc_idx, compute_crlb=compute_crlb,
            eigh_fallback=eigh_fallback, nonconverged=ncv[sl])
        cpx[sl], eig[sl], est[sl], crlb[sl] = v, lam, e, cr
        temp_coh[sl] = estimate_temp_coh(v, C)
    if diagnostics is not None:
        diagnostics["nonconverged"] = ncv.reshape(out_rows, out_cols)
    if neighbor_arrays is None:
        shp_counts = np.zeros((out_rows, out_cols), dtype=np.int16)
    else:
        shp_counts = np.sum(np.asarray(neighbor_arrays), axis=(-2, -1)).astype(np.int32)
    return PhaseLinkOutput(
        cpx_phase=np.moveaxis(cpx.reshape(out_rows, out_cols, n), -1, 0),
        temp_coh=temp_coh.reshape(out_rows, out_cols),
        shp_counts=shp_counts,
        eigenvalues=eig.reshape(out_rows, out_cols),
        estimator=est.reshape(out_rows, out_cols),
        crlb_std_dev=np.moveaxis(crlb.reshape(out_rows, out_cols, n), -1, 0),
        closure_phases=clos.reshape(out_rows, out_cols, max(n - 2, 0)),
    )


def run_phase_linking(slc_stack, half_window, strides=(1, 1), use_evd=False, beta=0.0,
                      zero_correlation_threshold=0.0, reference_idx=0, nodata_mask=None,
                      mask_input_ps=False, ps_mask=None, use_max_ps=True, neighbor_arrays=None,
                      avg_mag=None, use_slc_amp=False, baseline_lag=None,
                      first_real_slc_idx=0, compute_crlb=True, dtype=np.float32,
                      diagnostics=None, eigh_fallback=False):
    """phase_link/_core.py:67-249 (``diagnostics``, ``eigh_fallback``: see :func:`run_cpl`
    and :func:`process_coherence_matrices`)."""
    slc_stack = np.asarray(slc_stack)
    _, rows, cols = slc_stack.shape
    strides = tuple(strides)
    half_window = tuple(half_window)
    nodata_mask = np.zeros((rows, cols), bool) if nodata_mask is None else np.asarray(nodata_mask).astype(bool)
    ps_mask = np.zeros((rows, cols), bool) if ps_mask is None else np.asarray(ps_mask).astype(bool)
    _raise_if_all_nan(slc_stack)
    if nodata_mask.shape != (rows, cols) or ps_mask.shape != (rows, cols):
        raise ValueError(
            f"nodata_mask.shape={nodata_mask.shape}, ps_mask.shape={ps_mask.shape},"
            f" but != SLC (rows, cols) {rows, cols}"
        )
    nodata_mask |= np.any(np.isnan(slc_stack), axis=0)
    ps_mask[nodata_mask] = False
    masked = slc_stack.copy()
    if mask_input_ps:
        masked[:, nodata_mask | ps_mask] = np.nan
    else:
        masked[:, nodata_mask] = np.nan
    cpl = run_cpl(masked, half_window, strides, use_evd=use_evd, beta=beta,
                  zero_correlation_threshold=zero_correlation_threshold,
                  reference_idx=reference_idx, neighbor_arrays=neighbor_arrays,
                  baseline_lag=baseline_lag, first_real_slc_idx=first_real_slc_idx,
                  compute_crlb=compute_crlb, dtype=dtype, diagnostics=diagnostics,
                  eigh_fallback=eigh_fallback)
    mask_looked = take_looks(nodata_mask, *strides, func_type="all")
    temp_coh = np.array(cpl.temp_coh)
    cdt = _cdt(dtype)
    with np.errstate(all="ignore"):
        cpx_phase = np.exp(1j * np.angle(cpl.cpx_phase)).astype(cdt)
    if np.any(ps_mask):
        fill_ps_pixels(cpx_phase, temp_coh, slc_stack, ps_mask, strides, avg_mag,
                       reference_idx, use_max_ps=use_max_ps)
    if use_slc_amp:
        with np.errstate(all="ignore"):
            cpx_phase = (np.exp(1j * np.angle(cpx_phase)) * np.abs(decimate(slc_stack, strides))).astype(cdt)
    cpx_phase[:, mask_looked] = np.nan
    temp_coh[mask_looked] = np.nan
    return PhaseLinkOutput(
        cpx_phase=cpx_phase,
        temp_coh=temp_coh,
        shp_counts=np.asarray(cpl.shp_counts),
        eigenvalues=np.asarray(cpl.eigenvalues),
        estimator=np.asarray(cpl.estimator),
        crlb_std_dev=np.array(cpl.crlb_std_dev),
        closure_phases=np.asarray(cpl.closure_phases),
    )


# --------------------------------------------------------------------------------------
# compressed SLC (phase_link/_compress.py:11-65)
# --------------------------------------------------------------------------------------
def upsample_nearest(arr, output_shape, looks=None):
    """Block repetition to `output_shape`, zero where the repeats do not reach (utils.py:281-324)."""
    in_rows, in_cols = arr.shape[-2:]
    out_rows, out_cols = output_shape[-2:]
    if (in_rows, in_cols) == (out_rows, out_cols):
        return arr
    ry, rx = (out_rows // in_rows, out_cols // in_cols) if looks is None else looks
    up = np.repeat(np.repeat(arr, ry, axis=-2), rx, axis=-1)
    r, c = min(out_rows, up.shape[-2]), min(out_cols, up.shape[-1])
    out = np.zeros(arr.shape[:-2] + (out_rows, out_cols), dtype=arr.dtype)
    out[..., :r, :c] = up[..., :r, :c]
    return out


def compress(slc_stack, pl_cpx_phase, first_real_slc_idx=0, slc_mean=None, reference_idx=None):
    """Compressed SLC: mean amplitude x phase of sum_t z_t conj(pl_t) (phase_link/_compress.py:11-65).

    The phase-linked phases are re-referenced to `reference_idx` (if given) before the
    compressed layers (index < first_real_slc_idx) are dropped; NaN products are
    skipped (nansum); where that phase is exactly 0 the magnitude becomes NaN, and a
    given `slc_mean` is modified in place accordingly, as in the reference.
    """
    pl = np.asarray(pl_cpx_phase)
    if reference_idx is not None:
        pl = pl * pl[reference_idx][None, :, :].conj()
    pl = pl[first_real_slc_idx:]
    slcs = np.asarray(slc_stack)[first_real_slc_idx:]
    pl_up = upsample_nearest(pl, slcs.shape[1:])
    with warnings.catch_warnings():
        warnings.filterwarnings("ignore", message="invalid value encountered")
        phase = np.angle(np.nansum(slcs * np.conjugate(pl_up), axis=0))
    if slc_mean is None:
        slc_mean = np.mean(np.abs(slcs), axis=0)
    slc_mean[phase == 0] = np.nan
    return slc_mean * np.exp(1j * phase)
