"""Comparison helpers shared by the oracle and GPU parity tests."""

import numpy as np

from oracle import phase_link as O


def phase_err(a, b):
    """|angle(a * conj(b))| -- phase difference in radians."""
    return np.abs(np.angle(a * np.conj(b)))


_phase_err = phase_err


def judge_flips(out, ref, fp64, label="", tc_min=0.3, phase_tol=1e-3, tc_tol=1e-4):
    """Pixels whose EMI/EVD choice differs from the float32 reference ``ref`` are judged
    against the FP64 answer ``fp64``: where its temporal coherence is above ``tc_min``,
    the phase must be within ``phase_tol`` rad and the coherence within ``tc_tol`` of it.
    Returns the flip mask; prints the count and the worst errors."""
    flip = np.asarray(out.estimator) != np.asarray(ref.estimator)
    if not flip.any():
        return flip
    assert fp64 is not None, f"{label}: {int(flip.sum())} estimator flips and no FP64 answer to judge them"
    fgood = flip & (fp64.temp_coh > tc_min) & np.all(np.isfinite(fp64.cpx_phase), axis=0)
    perr = phase_err(out.cpx_phase[:, fgood], fp64.cpx_phase[:, fgood].astype(np.complex64)) if fgood.any() else np.zeros(1)
    terr = np.abs(out.temp_coh[fgood] - fp64.temp_coh[fgood]) if fgood.any() else np.zeros(1)
    same64 = int((np.asarray(out.estimator)[flip] == np.asarray(fp64.estimator)[flip]).sum())
    print(f"{label}: {int(flip.sum())} estimator flips against the float32 reference ({same64} agree with the "
          f"FP64 answer); on the {int(fgood.sum())} coherent ones: phase error vs FP64 {float(perr.max()):.2e} rad, "
          f"coherence {float(terr.max()):.2e}")
    assert perr.max() <= phase_tol, perr.max()
    assert terr.max() <= tc_tol, terr.max()
    return flip


def judge_nonconverged(out, flags, fp64, label="", tc_min=0.3, phase_tol=1e-3, tc_tol=1e-4):
    """Pixels the dense eigensolver solved again (``flags``: the iteration missed its
    stopping rule, where the reference returns its last iterate) are judged against the
    FP64 answer ``fp64`` computed with the same fallback.  Returns the flag mask."""
    f = np.zeros(out.temp_coh.shape, bool) if flags is None else np.asarray(flags).astype(bool)
    if not f.any():
        return f
    assert fp64 is not None, f"{label}: {int(f.sum())} re-solved pixels and no FP64 answer to judge them"
    fgood = f & (fp64.temp_coh > tc_min) & np.all(np.isfinite(fp64.cpx_phase), axis=0)
    perr = phase_err(out.cpx_phase[:, fgood], fp64.cpx_phase[:, fgood].astype(np.complex64)) if fgood.any() else np.zeros(1)
    terr = np.abs(out.temp_coh[fgood] - fp64.temp_coh[fgood]) if fgood.any() else np.zeros(1)
    print(f"{label}: {int(f.sum())} pixels solved by the dense eigensolver; on the {int(fgood.sum())} coherent "
          f"ones: phase error vs FP64 {float(perr.max()):.2e} rad, coherence {float(terr.max()):.2e}")
    assert perr.max() <= phase_tol, perr.max()
    assert terr.max() <= tc_tol, terr.max()
    return f


def compare_pl(out, g, prefix, tc_min=0.3, phase_tol=1e-3, tc_tol=1e-4, fp64=None, label=None, nonconverged=None):
    """Compare a PhaseLinkOutput with golden outputs ``{prefix}_{field}`` in ``g``.

    Pixels whose EMI-vs-EVD choice differs from the golden one (|Gamma| within rounding
    of singular) are judged against the FP64 answer ``fp64`` (see ``judge_flips``), and
    so are the pixels flagged in ``nonconverged`` (``judge_nonconverged``); both are
    left out of the comparison with the golden outputs.
    """
    ref = {k: g[f"{prefix}_{k}"] for k in O.PhaseLinkOutput._fields}
    borderline = judge_flips(out, O.PhaseLinkOutput(**ref), fp64, label or str(prefix), tc_min, phase_tol, tc_tol)
    borderline = borderline | judge_nonconverged(out, nonconverged, fp64, label or str(prefix), tc_min, phase_tol,
                                                 tc_tol)
    if borderline.any():
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


def compare_workflow(out, ref, tc_min=0.3, phase_tol=1e-3, tc_tol=1e-4, sim_tol=2e-3, ref64=None,
                     eig_rtol=1e-3, crlb_rtol=2e-3, label="ministack"):
    """Compare one ministack's block-loop rasters (dicts with keys pl, crlb, clos, comp,
    disp, tc, counts, eig, est, sim) with a reference run.

    SHP counts and the nodata (zero) patterns must match exactly.  Phases (linked,
    closure, compressed) within ``phase_tol`` rad and the temporal coherence within
    ``tc_tol`` on pixels with coherence > ``tc_min``.  Where the EMI/EVD choice differs
    from the reference run (|Gamma| within rounding of singular), the linked phase and
    the coherence are judged against ``ref64``, the same run with the phase linking in
    float64, instead; the flips are counted and printed.
    """
    np.testing.assert_array_equal(np.asarray(out["counts"]).astype(np.int64), np.asarray(ref["counts"]).astype(np.int64))
    np.testing.assert_array_equal(out["tc"] == 0, ref["tc"] == 0)
    np.testing.assert_array_equal(out["pl"] == 0, ref["pl"] == 0)
    flip = np.asarray(out["est"]) != np.asarray(ref["est"])
    if flip.any():
        assert ref64 is not None, f"{label}: {int(flip.sum())} estimator flips and no float64 run to judge them"
        fgood = flip & (ref64["tc"] > tc_min)
        perr = phase_err(out["pl"][:, fgood], ref64["pl"][:, fgood]).max() if fgood.any() else 0.0
        terr = np.abs(out["tc"][fgood] - ref64["tc"][fgood]).max() if fgood.any() else 0.0
        print(f"{label}: {int(flip.sum())} estimator flips against the float32 run; on the {int(fgood.sum())} "
              f"coherent ones: phase error vs float64 {perr:.2e} rad, coherence {terr:.2e}")
        assert perr <= phase_tol, perr
        assert terr <= tc_tol, terr
    good = (ref["tc"] > tc_min) & (out["tc"] > tc_min) & ~flip
    assert good.sum() > 0
    assert np.max(np.abs(out["tc"][good] - ref["tc"][good])) <= tc_tol
    assert np.max(phase_err(out["pl"][:, good], ref["pl"][:, good])) <= phase_tol
    if ref["clos"].size:
        d = np.angle(np.exp(1j * (out["clos"][good] - ref["clos"][good])))
        assert np.max(np.abs(d)) <= phase_tol
    # eigenvalues and CRLB only where C has full rank (at least as many SHP samples as
    # layers), as for a single phase-linking call
    n_layers = ref["clos"].shape[-1] + 2
    posed = good & (np.asarray(out["est"]) == np.asarray(ref["est"])) & (np.asarray(ref["counts"]) >= n_layers)
    e_out, e32 = np.asarray(out["eig"])[posed], np.asarray(ref["eig"])[posed]
    off = ~np.isclose(e_out, e32, rtol=eig_rtol, atol=1e-4)
    if off.any() and ref64 is not None:
        # where the float32 runs disagree the float64 run decides (an ill-conditioned
        # |Gamma| amplifies float32 rounding in the eigenvalue)
        e64 = np.asarray(ref64["eig"])[posed]
        print(f"{label}: {int(off.sum())} eigenvalues off the float32 run: got {e_out[off]}, float32 {e32[off]}, "
              f"float64 {e64[off]}")
        off &= ~np.isclose(e_out, e64, rtol=eig_rtol, atol=1e-4)
    assert not off.any(), (e_out[off], e32[off])
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
