"""Generate the golden fixtures in this folder from the reference's own code.

Run from the repository root in a container that has the reference checkout:

    python tests/golden/make_golden.py

The reference's hot-path modules are loaded from their source files through
``ref_shim`` (numpy stand-ins for jax/numba; see its docstring for what that does
and does not reproduce) and run on small seeded inputs.  Inputs and outputs are
written to ``tests/golden/*.npz``; the tests only read those files, so neither the
reference nor this script is needed to run them.
"""

from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

import ref_shim  # noqa: E402

from dolphin_gb300.simulate import StackConfig, make_stack  # noqa: E402

R = ref_shim.load_reference()
HW = R.types.HalfWindow
ST = R.types.Strides


def _save(name, **arrays):
    path = HERE / f"{name}.npz"
    np.savez_compressed(path, **arrays)
    print(f"wrote {path.name}: {path.stat().st_size / 1024:.0f} KiB")


def make_ps():
    rng = np.random.default_rng(101)
    n, rows, cols = 12, 17, 23
    mag = rng.lognormal(0.0, 0.5, size=(n, rows, cols)).astype(np.float32)
    # low-dispersion pixels (PS-like), a constant pixel (dispersion 0), NaN patterns
    mag[:, 2, 3] = (10 * (1 + 0.01 * rng.normal(size=n))).astype(np.float32)
    mag[:, 5, 5] = (8 * (1 + 0.2 * rng.normal(size=n))).astype(np.float32)
    mag[:, 7, 9] = np.float32(4.0)
    mag[0, 1, 1] = np.nan
    mag[:3, 4, 4] = np.nan
    mag[:, 6, 6] = np.nan
    mag[:, 10:12, 14:18] = (5 * (1 + 0.05 * rng.normal(size=(n, 2, 4)))).astype(np.float32)
    cases = [(0.25, None), (0.4, n), (0.35, 9), (1e5, None), (0.0, None)]
    out = {"mag": mag, "thr": np.array([c[0] for c in cases]),
           "min_count": np.array([-1 if c[1] is None else c[1] for c in cases])}
    for k, (thr, mc) in enumerate(cases):
        mean, disp, ps = R.ps.calc_ps_block(mag.copy(), thr, mc)
        out[f"mean_{k}"], out[f"disp_{k}"], out[f"ps_{k}"] = mean, disp, ps
    _save("ps_block", **out)


def _amp_field(seed, n, rows, cols):
    rng = np.random.default_rng(seed)
    amp = rng.rayleigh(scale=10.0, size=(n, rows, cols)).astype(np.float32)
    amp[:, : rows // 3, :] *= np.float32(3.0)  # a bright region with a sharp edge
    amp[:, :, cols - 4 :] *= np.float32(0.4)
    return amp


def make_glrt():
    out = {}
    cases = [
        # (seed, n, rows, cols, hw, strides, nslc, alpha)
        (201, 30, 24, 30, (3, 5), (1, 1), 30, 0.001),
        (202, 20, 22, 26, (5, 5), (2, 2), 20, 0.005),
        (203, 12, 19, 27, (2, 4), (2, 3), 12, 0.05),
        (204, 30, 16, 40, (5, 11), (1, 1), 30, 0.001),
    ]
    for k, (seed, n, rows, cols, hw, st, nslc, alpha) in enumerate(cases):
        amp = _amp_field(seed, n, rows, cols)
        mean = np.mean(amp, axis=0)
        var = np.var(amp, axis=0)
        mean[:3, :4] = 0  # nodata convention: mean 0 gives no SHPs
        nb = np.asarray(
            R.shp.estimate_neighbors(
                mean=mean, var=var, halfwin_rowcol=hw, strides=ST(*st), nslc=nslc,
                alpha=alpha, method="glrt",
            )
        )
        out[f"mean_{k}"], out[f"var_{k}"], out[f"nb_{k}"] = mean, var, nb
        out[f"params_{k}"] = np.array([*hw, *st, nslc, alpha], dtype=np.float64)
    _save("glrt", ncases=np.array(len(cases)), **out)


def make_ks():
    out = {}
    cases = [
        (301, 16, 14, 18, (2, 3), (1, 1), 0.05),
        (302, 11, 13, 15, (3, 3), (2, 2), 0.01),
        (303, 30, 11, 11, (5, 5), (1, 1), 1e-6),
    ]
    for k, (seed, n, rows, cols, hw, st, alpha) in enumerate(cases):
        amp = _amp_field(seed, n, rows, cols)
        if k == 0:
            amp[:, 6, 8] = amp[:, 6, 7]  # exact ties between two pixels
            amp[3, 5, 5] = np.nan
        nb = np.asarray(
            R.shp.estimate_neighbors(
                amp_stack=amp, halfwin_rowcol=hw, strides=ST(*st), nslc=n, alpha=alpha,
                method="ks",
            )
        )
        out[f"amp_{k}"], out[f"nb_{k}"] = amp, nb
        out[f"params_{k}"] = np.array([*hw, *st, alpha], dtype=np.float64)
    crit = []
    for n in (5, 8, 10, 15, 20, 30, 45, 64):
        for alpha in (1e-6, 0.001, 0.01, 0.05, 0.5):
            crit.append((n, alpha, R.ks._get_ecdf_critical_distance(n, alpha)))
    out["crit"] = np.array(crit, dtype=np.float64)
    # the reference's own doctest vectors for the ECDF distance (shp/_ks.py:180-194)
    x1 = np.array([1, 2, 3, 4, 5], dtype=np.float64)
    pairs = [x1, np.array([2, 3, 4, 5, 6.0]), np.array([6, 7, 8, 9, 10.0])]
    out["cdf_x"] = np.stack(pairs)
    out["cdf_d"] = np.array([R.ks._get_max_cdf_dist(x1, p) for p in pairs])
    _save("ks", ncases=np.array(len(cases)), **out)


def make_covariance():
    out = {}
    z = make_stack(StackConfig(nslc=8, rows=14, cols=17, seed=401, ps_frac=0.0))
    z[2, 3, 4] = np.nan
    z[:, 9, 10] = np.nan
    amp = np.abs(z)
    nb = np.asarray(
        R.shp.estimate_neighbors(
            mean=np.nanmean(amp, 0), var=np.nanvar(amp, 0), halfwin_rowcol=(3, 4),
            strides=ST(1, 1), nslc=8, alpha=0.05, method="glrt",
        )
    )
    out["slc"] = z
    out["nb"] = nb
    out["C_rect"] = np.asarray(R.covariance.estimate_stack_covariance(z, HW(3, 4), ST(1, 1)))
    out["C_nb"] = np.asarray(
        R.covariance.estimate_stack_covariance(z, HW(3, 4), ST(1, 1), neighbor_arrays=nb)
    )
    out["C_strided"] = np.asarray(R.covariance.estimate_stack_covariance(z, HW(3, 4), ST(2, 3)))
    _save("covariance", **out)


def _pl_case(idx, z, hw, strides, **kw):
    t0 = time.time()
    res = R.core.run_phase_linking(z.copy(), HW(*hw), ST(*strides), **kw)
    print(f"  case {idx}: {time.time() - t0:.1f}s")
    out = {f"{idx}_{k}": np.asarray(v) for k, v in res._asdict().items()}
    return out


def make_phase_link():
    cfg = StackConfig(nslc=10, rows=18, cols=22, seed=501, ps_frac=0.04)
    z, ps_truth, _ = make_stack(cfg, return_truth=True)
    amp = np.abs(z)
    mean, disp, ps = R.ps.calc_ps_block(amp.copy(), 0.25, cfg.nslc)
    var = (disp * mean) ** 2
    nodata = np.zeros(z.shape[1:], bool)
    nodata[0, :3] = True
    zn = z.copy()
    zn[4, 15:, 19:] = np.nan  # a corner that is NaN in one SLC -> nodata
    nb11 = np.asarray(
        R.shp.estimate_neighbors(mean=mean, var=var, halfwin_rowcol=(3, 4), strides=ST(1, 1),
                                 nslc=cfg.nslc, alpha=0.001, method="glrt"))
    nb23 = np.asarray(
        R.shp.estimate_neighbors(mean=mean, var=var, halfwin_rowcol=(3, 4), strides=ST(2, 3),
                                 nslc=cfg.nslc, alpha=0.001, method="glrt"))
    out = {"slc": z, "slc_nan": zn, "ps": ps, "nodata": nodata, "mean": mean, "nb11": nb11,
           "nb23": nb23}
    specs = {
        0: dict(z="slc", hw=(3, 4), strides=(1, 1), kw={}),
        1: dict(z="slc_nan", hw=(3, 4), strides=(1, 1),
                kw=dict(ps_mask="ps", nodata_mask="nodata", neighbor_arrays="nb11")),
        2: dict(z="slc_nan", hw=(3, 4), strides=(2, 3),
                kw=dict(ps_mask="ps", neighbor_arrays="nb23", use_max_ps=False, reference_idx=2,
                        first_real_slc_idx=3, use_slc_amp=True)),
        3: dict(z="slc", hw=(3, 4), strides=(1, 1),
                kw=dict(use_evd=True, baseline_lag=3, beta=0.1, zero_correlation_threshold=0.05,
                        ps_mask="ps", neighbor_arrays="nb11")),
        4: dict(z="slc", hw=(3, 4), strides=(1, 1),
                kw=dict(mask_input_ps=True, ps_mask="ps", avg_mag="mean", compute_crlb=False,
                        reference_idx=-1)),
        5: dict(z="slc", hw=(2, 2), strides=(3, 2),
                kw=dict(ps_mask="ps", beta=0.05, first_real_slc_idx=1, baseline_lag=4)),
    }
    for idx, spec in specs.items():
        kw = {k: (out[v] if isinstance(v, str) else v) for k, v in spec["kw"].items()}
        if "ps_mask" in kw:
            kw["ps_mask"] = kw["ps_mask"].copy()
        if "nodata_mask" in kw:
            kw["nodata_mask"] = kw["nodata_mask"].copy()
        out.update(_pl_case(idx, out[spec["z"]], spec["hw"], spec["strides"], **kw))
    meta = np.array([repr({k: (v["z"], v["hw"], v["strides"], v["kw"]) for k, v in specs.items()})])
    _save("phase_link", specs=meta, **out)


def make_config1_crop():
    """Config-1 generator (N=10, gamma0=0.7, gamma_inf=0.1, tau=36 d) on a 40x48 crop."""
    cfg = StackConfig(nslc=10, rows=40, cols=48, seed=20261204, ps_frac=0.05)
    z = make_stack(cfg)
    amp = np.abs(z)
    mean, disp, ps = R.ps.calc_ps_block(amp.copy(), 0.25, cfg.nslc)
    var = (disp * mean) ** 2
    nb = np.asarray(
        R.shp.estimate_neighbors(mean=mean, var=var, halfwin_rowcol=(5, 5), strides=ST(1, 1),
                                 nslc=cfg.nslc, alpha=0.001, method="glrt"))
    out = {"slc": z, "ps": ps, "mean": mean, "disp": disp, "var": var, "nb": nb}
    out.update(_pl_case("emi", z, (5, 5), (1, 1), ps_mask=ps.copy(), neighbor_arrays=nb, avg_mag=mean))
    _save("config1_crop", **out)


def make_ps_fill():
    """get_max_idxs/fill_ps_pixels known answers, incl. the reference's strides-(3,6) regression layout."""
    out = {}
    ka = [
        (np.array([[5, 1, 3], [4, 9, 2], [8, 7, 6]], dtype=np.float64), 1, 1),
        (np.arange(16, dtype=np.float64).reshape(4, 4) + 1, 2, 2),
        (np.array([[1, 5, 3], [4, 20, 2], [8, 0, 6]], dtype=np.float64), 2, 2),
        (np.arange(9 * 11, dtype=np.float64).reshape(9, 11), 2, 3),
    ]
    for n in range(10, 15):
        for looks in (2, 3):
            ka.append((np.arange(n * n, dtype=np.float64).reshape(n, n), looks, looks))
    for k, (arr, ry, rx) in enumerate(ka):
        r, c = R.fill.get_max_idxs(arr, ry, rx)
        out[f"ka_arr_{k}"], out[f"ka_looks_{k}"] = arr, np.array([ry, rx])
        out[f"ka_r_{k}"], out[f"ka_c_{k}"] = np.asarray(r), np.asarray(c)
    out["n_ka"] = np.array(len(ka))
    # regression layout: PS positions of the reference's ps-fix fixture on a 522x534 grid
    d = np.load(ref_shim.REF_ROOT / "tests" / "data" / "ps-fix" / "failing_data_idxs.npz")
    rows, cols = d["not_nan_rows"], d["not_nan_cols"]
    rng = np.random.default_rng(601)
    mags = (rng.normal(size=(522, 534)) ** 2).astype(np.float64)
    avg_mag = np.full_like(mags, np.nan)
    avg_mag[rows, cols] = mags[rows, cols]
    r, c = R.fill.get_max_idxs(avg_mag, 3, 6)
    out["fix_rows"], out["fix_cols"] = rows.astype(np.int16), cols.astype(np.int16)
    out["fix_mags"] = mags[rows, cols]
    out["fix_r"], out["fix_c"] = np.asarray(r).astype(np.int16), np.asarray(c).astype(np.int16)
    _save("ps_fill", **out)


def make_compress():
    """compress() on seeded stacks: strides 1 and 3, referencing, compressed layers, NaNs."""
    out = {}
    cases = [
        # (seed, n, rows, cols, strides, first_real, ref, with_mean)
        (701, 10, 11, 11, (1, 1), 0, -1, False),
        (702, 10, 11, 11, (3, 3), 0, -1, False),
        (703, 14, 12, 17, (2, 3), 2, 1, True),
        (704, 8, 9, 10, (1, 1), 0, 3, True),
    ]
    for k, (seed, n, rows, cols, st, first, ref, with_mean) in enumerate(cases):
        rng = np.random.default_rng(seed)
        z = make_stack(StackConfig(nslc=n, rows=rows, cols=cols, seed=seed, ps_frac=0.0))
        z[1, 2, 3] = np.nan + 1j * np.nan  # one NaN sample
        z[:, 4, 5] = np.nan  # a pixel with no valid sample
        orow, ocol = rows // st[0], cols // st[1]
        ph = rng.uniform(-np.pi, np.pi, size=(n, orow, ocol))
        pl = np.exp(1j * ph).astype(np.complex64)
        pl[:, 0, 0] = np.nan  # a NaN phase-linked pixel
        mean = (np.abs(z[first:]).mean(axis=0) * 1.5).astype(np.float32) if with_mean else None
        mean_in = None if mean is None else mean.copy()
        comp = R.compress.compress(z.copy(), pl.copy(), first_real_slc_idx=first,
                                   slc_mean=mean, reference_idx=None if ref < 0 else ref)
        out[f"slc_{k}"], out[f"pl_{k}"], out[f"out_{k}"] = z, pl, np.asarray(comp)
        out[f"params_{k}"] = np.array([first, ref, int(with_mean)])
        if with_mean:
            out[f"mean_in_{k}"], out[f"mean_after_{k}"] = mean_in, mean
    _save("compress", ncases=np.array(len(cases)), **out)


def make_similarity():
    """similarity.py: circle offsets, phase_similarity, median/max rasters (masks, NaNs,
    zeros, real phase input, clipping at the edges) and the nearest-n differences."""
    S = R.similarity
    out = {}
    for radius in range(1, 26):
        out[f"circle_{radius}"] = np.asarray(S.get_circle_idxs(radius)).reshape(-1, 2).astype(np.int16)
    for radius, rmin in [(5, 0), (7, 2), (9, 4)]:
        out[f"circle_raw_{radius}_{rmin}"] = np.asarray(
            S.get_circle_idxs(radius, min_radius=rmin, sort_output=False)).reshape(-1, 2).astype(np.int16)
    # phase_similarity on the reference's known-answer vectors and a random pair
    rng = np.random.default_rng(801)
    x1 = np.exp(1j * rng.uniform(0, 2 * np.pi, 50)).astype(np.complex64)
    x2 = np.exp(1j * rng.uniform(0, 2 * np.pi, 50)).astype(np.complex64)
    out["ps_x1"], out["ps_x2"] = x1, x2
    out["ps_val"] = np.array([S.phase_similarity(x1, x2), S.phase_similarity(x1, x1),
                              S.phase_similarity(np.zeros(10, np.complex64), np.zeros(10, np.complex64))])

    def ifgs(seed, n, rows, cols):
        z = make_stack(StackConfig(nslc=n + 1, rows=rows, cols=cols, seed=seed, ps_frac=0.0))
        return (z[1:] * np.conj(z[:1])).astype(np.complex64)

    cases = []
    a = ifgs(802, 8, 13, 17)
    a[:, 2, 3] = np.nan  # a pixel with no data
    a[:, 5, 0] = 0  # an all-zero pixel (invalid)
    a[3, 7, 9] = np.nan  # one NaN layer: its similarities are NaN
    cases += [("cpx", a, r, None) for r in (2, 3, 5)]
    b = ifgs(803, 6, 5, 10)
    mask = np.array(
        [[1, 0, 0, 1, 0, 0, 0, 0, 1, 1], [0, 1, 1, 1, 1, 1, 1, 1, 0, 1], [1, 0, 0, 0, 0, 1, 1, 0, 1, 0],
         [1, 1, 1, 1, 1, 0, 1, 0, 0, 0], [0, 0, 1, 1, 1, 1, 1, 1, 0, 1]], dtype=bool)
    cases += [("masked", b, r, mask) for r in (2, 5, 9)]
    ph = np.angle(ifgs(804, 5, 9, 11)).astype(np.float32)
    ph[:, 4, 4] = 0.0  # zero phase everywhere: invalid
    cases += [("real", ph, 4, None)]
    cases += [("row", ifgs(805, 4, 1, 12), 3, None), ("col", ifgs(806, 4, 11, 1), 3, None)]
    cases += [("zeros", np.zeros((10, 4, 5), np.complex64), 2, None),
              ("nans", np.full((10, 4, 5), np.nan, np.complex64), 2, None)]
    for k, (name, stack, radius, m) in enumerate(cases):
        m_med = None if m is None else m.copy()
        m_max = None if m is None else m.copy()
        med = S.median_similarity(stack.copy(), search_radius=radius, mask=m_med)
        mx = S.max_similarity(stack.copy(), search_radius=radius, mask=m_max)
        out[f"case_{k}_stack"], out[f"case_{k}_radius"] = stack, np.array(radius)
        out[f"case_{k}_median"], out[f"case_{k}_max"] = np.asarray(med), np.asarray(mx)
        if m is not None:
            out[f"case_{k}_mask_in"], out[f"case_{k}_mask_after"] = m, m_med
        print(f"  similarity case {k} ({name}, radius {radius})")
    out["ncases"] = np.array(len(cases))
    # nearest-n differences of a single-reference stack (3 nearest dates, 7 + 1 dates)
    c = ifgs(807, 7, 10, 12)
    c[:, 1, 1] = np.nan
    c[2, 3, 4] = np.nan
    c[:, 6, 6] = 0
    pairs = S._create_nearest_n_pairs(c.shape[0] + 1, n=3)
    A = R.get_incidence_matrix(pairs)
    d = S._calc_nearest_diffs(c.copy(), A)
    out["nn_stack"], out["nn_pairs"], out["nn_diffs"] = c, np.array(pairs), np.asarray(d)
    out["nn_median"] = np.asarray(S.median_similarity(d.copy(), search_radius=3))
    _save("similarity", **out)


NONE_IDX = -(2**31)  # a None slice bound


def _enc(b):
    return [NONE_IDX if v is None else int(v) for v in (b.row_start, b.row_stop, b.col_start, b.col_stop)]


def _ref_single(stack, hw, strides, block_shape, first_real, out_ref, comp_ref, nodata, ps, amp_mean, amp_disp,
                shp_nslc, alpha):
    """workflows/single.py:188-368 on arrays, with the reference's own functions; no files."""
    rows, cols = stack.shape[1:]
    mgr = R.blocks.StridedBlockManager(arr_shape=(rows, cols), block_shape=block_shape, strides=ST(*strides),
                                       half_window=HW(*hw))
    orow, ocol = rows // strides[0], cols // strides[1]
    n = len(stack)
    nreal = n - first_real
    out = {
        "pl": np.zeros((nreal, orow, ocol), np.complex64), "crlb": np.zeros((nreal, orow, ocol), np.float32),
        "clos": np.zeros((orow, ocol, n - 2), np.float32), "comp": np.zeros((rows, cols), np.complex64),
        "disp": np.zeros((rows, cols), np.float32), "tc": np.zeros((orow, ocol), np.float32),
        "counts": np.zeros((orow, ocol), np.int32), "eig": np.zeros((orow, ocol), np.float32),
        "est": np.zeros((orow, ocol), np.uint8),
    }
    var = (amp_disp * amp_mean) ** 2
    for (o_r, o_c), (t_r, t_c), (i_r, i_c), (p_r, p_c), (f_r, f_c) in mgr.iter_blocks():
        if nodata[i_r, i_c].all():
            continue
        cur = stack[:, i_r, i_c]
        if np.all(cur == 0) or np.isnan(cur).all():
            continue
        cur = cur.astype(np.complex64)
        nb = R.shp.estimate_neighbors(halfwin_rowcol=hw, alpha=alpha, strides=ST(*strides), mean=amp_mean[i_r, i_c],
                                      var=var[i_r, i_c], nslc=shp_nslc, method=R.ShpMethod.GLRT)
        try:
            res = R.core.run_phase_linking(cur.copy(), HW(*hw), ST(*strides), reference_idx=out_ref,
                                           nodata_mask=nodata[i_r, i_c], ps_mask=ps[i_r, i_c], neighbor_arrays=nb,
                                           avg_mag=amp_mean[i_r, i_c], first_real_slc_idx=first_real,
                                           compute_crlb=True)
        except R.core.PhaseLinkRuntimeError:
            continue
        cpx = np.nan_to_num(np.asarray(res.cpx_phase))
        crlb = np.nan_to_num(np.asarray(res.crlb_std_dev))
        tcoh = np.nan_to_num(np.asarray(res.temp_coh))
        m_, d_, _ = R.ps.calc_ps_block(np.abs(cur[first_real:, f_r, f_c]))
        comp = np.asarray(R.compress.compress(cur[:, f_r, f_c], cpx[:, t_r, t_c], first_real_slc_idx=first_real,
                                              slc_mean=m_, reference_idx=comp_ref))
        part = cpx[first_real:, t_r, t_c]
        h, w = part.shape[-2:]
        sl = (slice(o_r.start, o_r.start + h), slice(o_c.start, o_c.start + w))
        out["pl"][(slice(None),) + sl] = part
        out["crlb"][(slice(None),) + sl] = crlb[first_real:, t_r, t_c]
        out["clos"][sl] = np.asarray(res.closure_phases)[t_r, t_c]
        ch, cw = comp.shape
        out["comp"][p_r.start:p_r.start + ch, p_c.start:p_c.start + cw] = comp
        out["disp"][p_r.start:p_r.start + ch, p_c.start:p_c.start + cw] = d_
        for key, src, nd in (("tc", tcoh, 0), ("counts", np.asarray(res.shp_counts), 0),
                             ("eig", np.asarray(res.eigenvalues), 0), ("est", np.asarray(res.estimator), 255)):
            out[key][sl] = R.utils.grow_nodata_region(src[t_r, t_c], nodata=nd, n_pixels=2, copy=True)
    out["sim"] = np.asarray(R.similarity.median_similarity(out["pl"].copy(), search_radius=7))
    return out


def make_workflow():
    """Block manager, ministack planner and grow_nodata_region known answers, and a
    two-ministack sequential run built from the reference's own per-block functions."""
    import json
    from datetime import datetime, timedelta

    out = {}
    cfgs = [((40, 50), (16, 16), (2, 2), (3, 5)), ((37, 41), (10, 12), (1, 1), (2, 3)), ((64, 64), (32, 32), (1, 1),
                                                                                       (0, 0)),
            ((50, 30), (20, 20), (3, 2), (4, 4)), ((25, 25), (512, 512), (1, 1), (5, 11))]
    for k, (shape, block, strides, hw) in enumerate(cfgs):
        mgr = R.blocks.StridedBlockManager(arr_shape=shape, block_shape=block, strides=ST(*strides),
                                           half_window=HW(*hw))
        rows = [sum((_enc(b) for b in blk), []) for blk in mgr.iter_blocks()]
        out[f"blocks_{k}"] = np.array(rows, dtype=np.int64).reshape(-1, 20)
        out[f"blocks_cfg_{k}"] = np.array(list(shape) + list(block) + list(strides) + list(hw))
    out["nblock_cfgs"] = np.array(len(cfgs))

    plans = []
    for (n, size, max_comp, plan, out_ref) in [(11, 4, 2, "always_first", None), (10, 5, 100, "always_first", None),
                                               (9, 3, 1, "always_first", 0), (6, 6, 5, "last_per_ministack", None),
                                               (7, 10, 5, "always_first", 2), (15, 4, 0, "always_first", None)]:
        files = [f"slc_{(datetime(2020, 1, 1) + timedelta(days=12 * i)).strftime('%Y%m%d')}.tif" for i in range(n)]
        dates = [[datetime(2020, 1, 1) + timedelta(days=12 * i)] for i in range(n)]
        planner = R.stack.MiniStackPlanner(file_list=files, dates=dates, is_compressed=[False] * n,
                                           output_folder="ms", max_num_compressed=max_comp,
                                           output_reference_idx=out_ref, compressed_slc_plan=plan)
        made, comp_paths = [], []
        for ms in planner.plan(size):
            layers = []
            for f in ms.file_list:
                f = str(f)
                layers.append(files.index(f) if f in files else -(1 + comp_paths.index(f)))
            made.append({"layers": layers, "is_compressed": list(map(bool, ms.is_compressed)),
                         "out_ref": int(ms.output_reference_idx), "comp_ref": int(ms.compressed_reference_idx),
                         "first_real": int(ms.first_real_slc_idx)})
            comp_paths.append(str(ms.get_compressed_slc_info().path))
        plans.append({"n": n, "size": size, "max_comp": max_comp, "plan": plan, "out_ref": out_ref, "ministacks": made})
    out["plans"] = np.array(json.dumps(plans))

    rng = np.random.default_rng(901)
    g = rng.normal(size=(14, 17)).astype(np.float32)
    g[g < -1.2] = 0
    g[3, 5] = 0
    e = (rng.random((9, 11)) > 0.5).astype(np.uint8)
    e[4, 4] = 255
    gn = g.copy()
    gn[7, 7] = np.nan
    for k, (arr, nd, npx) in enumerate([(g, 0, 2), (g, 0, 1), (e, 255, 2), (gn, np.nan, 1), (e, 0, 0)]):
        out[f"grow_in_{k}"] = arr
        out[f"grow_nd_{k}"] = np.array(nd, dtype=np.float64)
        out[f"grow_n_{k}"] = np.array(npx)
        out[f"grow_out_{k}"] = R.utils.grow_nodata_region(arr, nodata=nd, n_pixels=npx, copy=True)
    out["ngrow"] = np.array(5)

    # two ministacks of 4 SLCs (the second led by the first one's compressed SLC)
    cfg = StackConfig(nslc=8, rows=20, cols=26, seed=902, ps_frac=0.04)
    z = make_stack(cfg)
    amp_mean, amp_disp, ps = R.ps.calc_ps_block(np.abs(z), 0.25, cfg.nslc)
    amp_mean, amp_disp, ps = (np.asarray(a) for a in (amp_mean, amp_disp, ps))
    nodata = np.zeros(z.shape[1:], bool)
    nodata[:3, :4] = True
    hw, strides, block = (2, 3), (1, 1), (12, 12)
    comp_list = []
    files = [f"slc_{(datetime(2020, 1, 1) + timedelta(days=12 * i)).strftime('%Y%m%d')}.tif" for i in range(8)]
    dates = [[datetime(2020, 1, 1) + timedelta(days=12 * i)] for i in range(8)]
    planner = R.stack.MiniStackPlanner(file_list=files, dates=dates, is_compressed=[False] * 8, output_folder="ms",
                                       max_num_compressed=100)
    for k, ms in enumerate(planner.plan(4)):
        real = [files.index(str(f)) for f in ms.file_list if str(f) in files]
        layers = ([c for c in comp_list] if comp_list else []) + [z[i] for i in real]
        cur = np.stack(layers).astype(np.complex64)
        res = _ref_single(cur, hw, strides, block, int(ms.first_real_slc_idx), int(ms.output_reference_idx),
                          int(ms.compressed_reference_idx), nodata, ps, amp_mean, amp_disp, 8, 0.05)
        comp_list.append(res["comp"])
        for key, val in res.items():
            out[f"seq{k}_{key}"] = val
        print(f"  sequential ministack {k}: {len(cur)} layers")
    out["seq_slc"], out["seq_nodata"], out["seq_ps"] = z, nodata, ps
    out["seq_amp_mean"], out["seq_amp_disp"] = amp_mean, amp_disp
    out["seq_cfg"] = np.array(list(hw) + list(strides) + list(block) + [4])
    _save("workflow", **out)


if __name__ == "__main__":
    which = sys.argv[1:] or ["ps", "glrt", "ks", "covariance", "phase_link", "config1", "ps_fill", "compress",
                             "similarity", "workflow"]
    for w in which:
        print(f"[{w}]")
        {"ps": make_ps, "glrt": make_glrt, "ks": make_ks, "covariance": make_covariance,
         "phase_link": make_phase_link, "config1": make_config1_crop, "ps_fill": make_ps_fill,
         "compress": make_compress, "similarity": make_similarity, "workflow": make_workflow}[w]()
