"""Pin the CPU oracle against golden vectors produced by the reference's own code.

The fixtures in ``tests/golden`` come from ``tests/golden/make_golden.py``, which ran
dolphin's phase-linking modules from source (numpy stand-ins for jax/numba).  These
tests need no GPU and no reference checkout.
"""

import ast

import numpy as np
import pytest

from oracle import phase_link as O


def _phase_err(a, b):
    return np.abs(np.angle(a * np.conj(b)))


def test_ps_block_bit_exact(golden):
    g = golden("ps_block")
    mag = g["mag"]
    for k, (thr, mc) in enumerate(zip(g["thr"], g["min_count"])):
        mean, disp, ps = O.calc_ps_block(mag.copy(), float(thr), None if mc < 0 else int(mc))
        assert mean.dtype == disp.dtype == np.float32
        np.testing.assert_array_equal(mean, g[f"mean_{k}"])
        np.testing.assert_array_equal(disp, g[f"disp_{k}"])
        np.testing.assert_array_equal(ps, g[f"ps_{k}"])


def test_ps_block_rejects_complex():
    with pytest.raises(ValueError):
        O.calc_ps_block(np.ones((3, 2, 2), np.complex64))


def test_glrt_bit_exact(golden):
    g = golden("glrt")
    for k in range(int(g["ncases"])):
        hy, hx, sy, sx, nslc, alpha = g[f"params_{k}"]
        nb = O.estimate_neighbors_glrt(g[f"mean_{k}"], g[f"var_{k}"], (int(hy), int(hx)),
                                       (int(sy), int(sx)), int(nslc), alpha)
        np.testing.assert_array_equal(nb, g[f"nb_{k}"])


def test_ks_bit_exact(golden):
    g = golden("ks")
    for k in range(int(g["ncases"])):
        hy, hx, sy, sx, alpha = g[f"params_{k}"]
        nb = O.estimate_neighbors_ks(g[f"amp_{k}"], (int(hy), int(hx)), (int(sy), int(sx)), alpha)
        np.testing.assert_array_equal(nb, g[f"nb_{k}"])
    for n, alpha, d in g["crit"]:
        assert O.ks_critical_distance(int(n), alpha) == d
    x = g["cdf_x"]
    d = O.ks_max_cdf_dist(np.broadcast_to(x[0], x.shape), x)
    np.testing.assert_array_equal(d, g["cdf_d"])


def test_covariance(golden):
    g = golden("covariance")
    z = g["slc"]
    np.testing.assert_allclose(O.estimate_stack_covariance(z, (3, 4), (1, 1)), g["C_rect"], atol=2e-6)
    np.testing.assert_allclose(O.estimate_stack_covariance(z, (3, 4), (1, 1), g["nb"]), g["C_nb"], atol=2e-6)
    np.testing.assert_allclose(O.estimate_stack_covariance(z, (3, 4), (2, 3)), g["C_strided"], atol=2e-6)


def _run_case(g, idx, spec):
    zname, hw, strides, kw = spec
    kw = dict(kw)
    for key in ("ps_mask", "nodata_mask", "neighbor_arrays", "avg_mag"):
        if key in kw:
            kw[key] = np.array(g[kw[key]])
    return O.run_phase_linking(np.array(g[zname]), hw, strides, **kw)


def compare_pl(out, g, prefix, tc_min=0.3, phase_tol=1e-3, tc_tol=1e-4, borderline=None):
    """Compare a PhaseLinkOutput with golden outputs ``{prefix}_{field}`` in ``g``.

    ``borderline``: pixels whose EMI-vs-EVD choice is decided by rounding (the
    jittered |Gamma| is within rounding of singular); they are left out.
    """
    ref = {k: g[f"{prefix}_{k}"] for k in O.PhaseLinkOutput._fields}
    if borderline is not None and borderline.any():
        keep = ~borderline
        ref = {k: (v[..., keep] if k in ("cpx_phase", "crlb_std_dev") else v[keep]) if v.ndim >= 2 else v
               for k, v in ref.items()}
        ref["closure_phases"] = g[f"{prefix}_closure_phases"][keep]
        out = O.PhaseLinkOutput(**{k: (v[..., keep] if k in ("cpx_phase", "crlb_std_dev") else v[keep])
                                   for k, v in out._asdict().items()})
    for k in O.PhaseLinkOutput._fields:
        assert out._asdict()[k].shape == ref[k].shape, k
        assert out._asdict()[k].dtype == ref[k].dtype, k
    np.testing.assert_array_equal(out.estimator, ref["estimator"])
    np.testing.assert_array_equal(out.shp_counts, ref["shp_counts"])
    nan_ref = np.isnan(ref["temp_coh"])
    np.testing.assert_array_equal(np.isnan(out.temp_coh), nan_ref)
    np.testing.assert_array_equal(np.isnan(out.cpx_phase), np.isnan(ref["cpx_phase"]))
    good = (~nan_ref) & (ref["temp_coh"] > tc_min) & np.all(np.isfinite(ref["cpx_phase"]), axis=0)
    assert good.sum() > 0
    err = _phase_err(out.cpx_phase[:, good], ref["cpx_phase"][:, good])
    assert err.max() <= phase_tol, err.max()
    assert np.abs(out.temp_coh[good] - ref["temp_coh"][good]).max() <= tc_tol
    np.testing.assert_allclose(np.abs(out.cpx_phase[:, ~nan_ref]), np.abs(ref["cpx_phase"][:, ~nan_ref]), rtol=1e-5)
    # Eigenvalues and CRLB are only well posed where C has full rank: with fewer SHP
    # samples than SLCs, |C|^-1 is huge and v^H A v cancels catastrophically.
    n = out.cpx_phase.shape[0]
    posed = (ref["shp_counts"] >= n) | (ref["shp_counts"].dtype == np.int16)
    posed = posed & ~nan_ref
    fin = np.isfinite(ref["eigenvalues"]) & posed
    np.testing.assert_allclose(out.eigenvalues[fin], ref["eigenvalues"][fin], rtol=1e-3, atol=1e-4)
    fin = np.isfinite(ref["crlb_std_dev"]) & posed[None]
    np.testing.assert_array_equal(np.isfinite(out.crlb_std_dev)[..., posed], np.isfinite(ref["crlb_std_dev"])[..., posed])
    np.testing.assert_allclose(out.crlb_std_dev[fin], ref["crlb_std_dev"][fin], rtol=2e-3, atol=1e-5)
    cl_err = _phase_err(np.exp(1j * out.closure_phases), np.exp(1j * ref["closure_phases"]))
    assert cl_err.max() < 1e-4


def test_run_phase_linking_cases(golden):
    g = golden("phase_link")
    specs = ast.literal_eval(str(g["specs"][0]))
    for idx, spec in specs.items():
        out = _run_case(g, idx, spec)
        compare_pl(out, g, idx)


def test_config1_crop(golden):
    g = golden("config1_crop")
    diag = {}
    out = O.run_phase_linking(g["slc"], (5, 5), (1, 1), ps_mask=g["ps"].copy(),
                              neighbor_arrays=g["nb"], avg_mag=g["mean"], diagnostics=diag)
    borderline = diag["gamma_min_eig"] < 1e-4
    assert borderline.sum() <= 0.1 * borderline.size
    compare_pl(out, g, "emi", borderline=borderline)
    mean, disp, ps = O.calc_ps_block(np.abs(g["slc"]), 0.25, 10)
    np.testing.assert_array_equal(ps, g["ps"])
    np.testing.assert_array_equal(mean, g["mean"])


def test_get_max_idxs_known_answers(golden):
    g = golden("ps_fill")
    for k in range(int(g["n_ka"])):
        ry, rx = g[f"ka_looks_{k}"]
        r, c = O.get_max_idxs(g[f"ka_arr_{k}"], int(ry), int(rx))
        np.testing.assert_array_equal(r, g[f"ka_r_{k}"])
        np.testing.assert_array_equal(c, g[f"ka_c_{k}"])
    avg = np.full((522, 534), np.nan)
    avg[g["fix_rows"], g["fix_cols"]] = g["fix_mags"]
    r, c = O.get_max_idxs(avg, 3, 6)
    np.testing.assert_array_equal(r, g["fix_r"])
    np.testing.assert_array_equal(c, g["fix_c"])


def test_all_nan_slc_raises():
    z = np.ones((3, 8, 8), np.complex64)
    z[1] = np.nan
    with pytest.raises(O.PhaseLinkRuntimeError, match="are all NaNs"):
        O.run_phase_linking(z, (1, 1))
