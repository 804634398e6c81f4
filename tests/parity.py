"""Comparison helpers shared by the oracle and GPU parity tests."""

import numpy as np

from oracle import phase_link as O


def phase_err(a, b):
    """|angle(a * conj(b))| -- phase difference in radians."""
    return np.abs(np.angle(a * np.conj(b)))


_phase_err = phase_err


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


def compare_workflow(out, ref, tc_min=0.3, phase_tol=1e-3, tc_tol=1e-4, sim_tol=2e-3, est_mismatch=0.01,
                     eig_rtol=1e-3, crlb_rtol=2e-3):
    """Compare one ministack's block-loop rasters (dicts with keys pl, crlb, clos, comp,
    disp, tc, counts, eig, est, sim) with a reference run.

    SHP counts and the nodata (zero) patterns must match exactly; the estimator may
    differ on a small share of pixels whose |Gamma| is within rounding of singular.
    Phases (linked, closure, compressed) within ``phase_tol`` rad and the temporal
    coherence within ``tc_tol`` on pixels with coherence > ``tc_min``.
    """
    np.testing.assert_array_equal(np.asarray(out["counts"]).astype(np.int64), np.asarray(ref["counts"]).astype(np.int64))
    np.testing.assert_array_equal(out["tc"] == 0, ref["tc"] == 0)
    np.testing.assert_array_equal(out["pl"] == 0, ref["pl"] == 0)
    good = (ref["tc"] > tc_min) & (out["tc"] > tc_min)
    assert good.sum() > 0
    assert np.max(np.abs(out["tc"][good] - ref["tc"][good])) <= tc_tol
    assert np.max(phase_err(out["pl"][:, good], ref["pl"][:, good])) <= phase_tol
    if ref["clos"].size:
        d = np.angle(np.exp(1j * (out["clos"][good] - ref["clos"][good])))
        assert np.max(np.abs(d)) <= phase_tol
    mism = np.mean(np.asarray(out["est"]) != np.asarray(ref["est"]))
    assert mism <= est_mismatch, mism
    # eigenvalues and CRLB only where C has full rank (at least as many SHP samples as
    # layers), as for a single phase-linking call
    n_layers = ref["clos"].shape[-1] + 2
    posed = good & (np.asarray(out["est"]) == np.asarray(ref["est"])) & (np.asarray(ref["counts"]) >= n_layers)
    np.testing.assert_allclose(out["eig"][posed], ref["eig"][posed], rtol=eig_rtol, atol=1e-4)
    np.testing.assert_allclose(out["crlb"][:, posed], ref["crlb"][:, posed], rtol=crlb_rtol, atol=1e-5)
    # compressed SLC: mean amplitude and the phase of the projection on the linked phases
    np.testing.assert_array_equal(np.isnan(out["comp"]), np.isnan(ref["comp"]))
    np.testing.assert_allclose(out["disp"], ref["disp"], rtol=1e-5, atol=1e-6)
    ok = np.isfinite(ref["comp"]) & (np.abs(ref["comp"]) > 0)
    np.testing.assert_allclose(np.abs(out["comp"][ok]), np.abs(ref["comp"][ok]), rtol=1e-5)
    assert np.max(phase_err(out["comp"][ok], ref["comp"][ok])) <= 5 * phase_tol
    np.testing.assert_array_equal(np.isnan(out["sim"]), np.isnan(ref["sim"]))
    fin = ~np.isnan(ref["sim"])
    if fin.any():
        assert np.max(np.abs(out["sim"][fin] - ref["sim"][fin])) <= sim_tol
