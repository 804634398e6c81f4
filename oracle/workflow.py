"""Numpy restatement of the wrapped-phase block loop and the sequential ministack chain
(ORACLE, test infrastructure).

Follows workflows/single.py:188-368 (per block: SHP selection by GLRT on the given
amplitude mean and dispersion or by KS on the block's amplitudes, phase linking, NaN -> 0, the compressed SLC of the real
SLCs with their mean and dispersion, trimmed results placed at the block's output
position, the strided ones eroded by grow_nodata_region, 2 pixels; then the median
similarity, radius 7), io/_blocks.py:59-348 (the block grid) and
stack.py:446-562 / workflows/sequential.py:105-207 (ministacks of real SLCs led by the
compressed SLCs of the earlier ones; averages of the temporal coherence and SHP counts
with 0 as nodata; the radius-11 similarity of the last ministack).  Raster I/O,
repacking and file bookkeeping are not restated.
"""

from __future__ import annotations

import numpy as np
from scipy import ndimage

from . import phase_link as P
from . import similarity as S

__all__ = ["blocks", "grow_nodata_region", "plan", "sequential", "single"]


def _grid(shape, block, start, end):
    r = start[0]
    while r < shape[0] - end[0]:
        c = start[1]
        while c < shape[1] - end[1]:
            yield r, min(r + block[0], shape[0] - end[0]), c, min(c + block[1], shape[1] - end[1])
            c += block[1]
        r += block[0]


def blocks(shape, block_shape, strides, half_window):
    """[(out, out_trim, in, in_no_pad, in_trim)] as (r0, r1, c0, c1) with None for open ends."""
    sy, sx = strides
    my, mx = round(half_window[0] / sy), round(half_window[1] / sx)
    oshape = (shape[0] // sy, shape[1] // sx)
    oblock = (block_shape[0] // sy, block_shape[1] // sx)
    trim = (my, -my if my else None, mx, -mx if mx else None)
    res = []
    for r0, r1, c0, c1 in _grid(oshape, oblock, (my, mx), (my, mx)):
        npd = (r0 * sy, r1 * sy, c0 * sx, c1 * sx)
        pad = (npd[0] - sy * my, npd[1] + sy * my, npd[2] - sx * mx, npd[3] + sx * mx)
        if pad[0] < 0 or pad[2] < 0:
            raise ValueError("block padding below 0")
        itrim = (npd[0] - pad[0], (npd[1] - pad[1]) or None, npd[2] - pad[2], (npd[3] - pad[3]) or None)
        res.append(((r0, r1, c0, c1), trim, pad, npd, itrim))
    return res


def grow_nodata_region(arr, nodata, n_pixels=1):
    arr = np.asarray(arr)
    mask = np.isnan(arr) if (isinstance(nodata, float) and np.isnan(nodata)) else arr == nodata
    grown = ndimage.binary_dilation(mask, structure=np.ones((2 * n_pixels + 1, 2 * n_pixels + 1)))
    out = arr.copy()
    out[grown] = nodata
    return out


def plan(n, size, max_comp=5, kind="always_first", out_ref=None):
    """[(layers, is_compressed, out_ref, comp_ref)] with layers >= 0 the input SLCs and
    -(1 + j) the j-th compressed SLC (one per earlier ministack)."""
    if size < 2:
        raise ValueError("Cannot create ministacks with size < 2")
    res = []
    for k, start in enumerate(range(0, n, size)):
        comp = list(range(k))[-max_comp:]
        nc = len(comp)
        comp_ref = max(0, nc - 1) if kind == "always_first" else -1
        oref = out_ref if out_ref is not None else max(0, nc - 1)
        layers = [-(1 + j) for j in comp] + list(range(start, min(start + size, n)))
        res.append((layers, [True] * nc + [False] * (len(layers) - nc), oref, comp_ref))
    return res


def _sl(a, b):
    return slice(a, b)


def single(stack, hw, strides, block_shape, first_real, out_ref, comp_ref, nodata, ps, amp_mean, amp_disp,
           shp_nslc, alpha, radius=7, method="glrt", dtype=np.float32):
    """One ministack's block loop; ``dtype`` is the precision of the phase linking (the
    SHP and PS selection stay float32, as the reference's)."""
    stack = np.asarray(stack)
    n, rows, cols = stack.shape
    sy, sx = strides
    orow, ocol = rows // sy, cols // sx
    nreal = n - first_real
    out = {"pl": np.zeros((nreal, orow, ocol), np.complex64), "crlb": np.zeros((nreal, orow, ocol), np.float32),
           "clos": np.zeros((orow, ocol, n - 2), np.float32), "comp": np.zeros((rows, cols), np.complex64),
           "disp": np.zeros((rows, cols), np.float32), "tc": np.zeros((orow, ocol), np.float32),
           "counts": np.zeros((orow, ocol), np.int32), "eig": np.zeros((orow, ocol), np.float32),
           "est": np.zeros((orow, ocol), np.uint8)}
    var = (amp_disp * amp_mean) ** 2
    for (o, t, i, p, f) in blocks((rows, cols), block_shape, strides, hw):
        ir, ic = _sl(i[0], i[1]), _sl(i[2], i[3])
        if nodata[ir, ic].all():
            continue
        cur = stack[:, ir, ic].astype(np.complex64)
        if np.all(cur == 0) or np.isnan(cur).all():
            continue
        nb = P.estimate_neighbors(halfwin_rowcol=hw, alpha=alpha, strides=strides, mean=amp_mean[ir, ic],
                                  var=var[ir, ic], nslc=shp_nslc,
                                  amp_stack=np.abs(cur) if method == "ks" else None, method=method)
        try:
            res = P.run_phase_linking(cur, hw, strides, reference_idx=out_ref, nodata_mask=nodata[ir, ic],
                                      ps_mask=ps[ir, ic].copy(), neighbor_arrays=nb, avg_mag=amp_mean[ir, ic],
                                      first_real_slc_idx=first_real, compute_crlb=True, dtype=dtype)
        except P.PhaseLinkRuntimeError:
            continue
        tr, tc = _sl(t[0], t[1]), _sl(t[2], t[3])
        fr, fc = _sl(f[0], f[1]), _sl(f[2], f[3])
        cpx = np.nan_to_num(np.asarray(res.cpx_phase))
        m_, d_, _ = P.calc_ps_block(np.abs(cur[first_real:, fr, fc]))
        comp = P.compress(cur[:, fr, fc], cpx[:, tr, tc], first_real_slc_idx=first_real, slc_mean=m_,
                          reference_idx=comp_ref)
        part = cpx[first_real:, tr, tc]
        h, w = part.shape[-2:]
        sl = (slice(o[0], o[0] + h), slice(o[2], o[2] + w))
        out["pl"][(slice(None),) + sl] = part
        out["crlb"][(slice(None),) + sl] = np.nan_to_num(np.asarray(res.crlb_std_dev))[first_real:, tr, tc]
        out["clos"][sl] = np.asarray(res.closure_phases)[tr, tc]
        out["comp"][p[0]:p[0] + comp.shape[0], p[2]:p[2] + comp.shape[1]] = comp
        out["disp"][p[0]:p[0] + comp.shape[0], p[2]:p[2] + comp.shape[1]] = d_
        for key, src, nd in (("tc", np.nan_to_num(np.asarray(res.temp_coh)), 0), ("counts", res.shp_counts, 0),
                             ("eig", res.eigenvalues, 0), ("est", res.estimator, 255)):
            out[key][sl] = grow_nodata_region(np.asarray(src)[tr, tc], nd, 2)
    out["sim"] = S.median_similarity(out["pl"], radius)
    return out


def sequential(stack, size, hw, strides, block_shape, nodata, ps, amp_mean, amp_disp, alpha=0.05, max_comp=100,
               method="glrt", dtype=np.float32):
    """Per-ministack outputs, then the averages and the last ministack's radius-11 similarity."""
    stack = np.asarray(stack)
    comps, outs = [], []
    for layers, flags, oref, cref in plan(len(stack), size, max_comp):
        cur = np.stack([comps[-l - 1] if l < 0 else stack[l] for l in layers])
        res = single(cur, hw, strides, block_shape, flags.index(False), oref, cref, nodata, ps, amp_mean, amp_disp,
                     len(stack), alpha, method=method, dtype=dtype)
        comps.append(res["comp"])
        outs.append(res)
    extra = {}
    if len(outs) > 1:
        for key in ("tc", "counts"):
            a = np.stack([o[key].astype(np.float32) for o in outs])
            m = np.where((a == 0).any(0), 0, np.nanmean(a, 0))
            extra[key + "_avg"] = m.astype(np.float32 if key == "tc" else np.int16)
        extra["sim_full"] = S.median_similarity(outs[-1]["pl"], 11)
    return outs, extra
