"""FP64 form (covariance and solver in double on the GPU) against the float64 oracle.

Both compute in double; the GPU writes float32 outputs, so phases agree to float32
rounding (~1e-7 rad) and the temporal coherence to ~1e-7.  Pixels whose |Gamma| +
1e-6 I has a smallest eigenvalue below 1e-9 (where even double rounding decides the
Cholesky outcome) are left out of the estimator comparison; eigenvalues and CRLB are
compared where C has full rank.  Both solve the pixels whose iteration misses the
stopping rule again with a dense eigensolver in double (the default of both).
"""

import numpy as np
import pytest

from oracle import phase_link as O
from parity import phase_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import dolphin_gb300 as dp  # noqa: E402
from dolphin_gb300.simulate import StackConfig, make_stack  # noqa: E402


def _compare(out, ref, diag, counts_ok, phase_tol=2e-6, tc_tol=2e-6):
    keep = diag["gamma_min_eig"] >= 1e-9
    np.testing.assert_array_equal(out.estimator[keep], ref.estimator[keep])
    np.testing.assert_array_equal(np.isnan(out.temp_coh), np.isnan(ref.temp_coh))
    fin = keep & np.isfinite(ref.temp_coh) & np.all(np.isfinite(ref.cpx_phase), axis=0)
    assert fin.sum() > 0
    err = phase_err(out.cpx_phase[:, fin], ref.cpx_phase[:, fin].astype(np.complex64))
    assert err.max() <= phase_tol, err.max()
    assert np.abs(out.temp_coh[fin] - ref.temp_coh[fin]).max() <= tc_tol
    posed = fin & counts_ok
    np.testing.assert_allclose(out.eigenvalues[posed], ref.eigenvalues[posed], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(out.crlb_std_dev[:, posed], ref.crlb_std_dev[:, posed], rtol=1e-4, atol=1e-6)
    if ref.closure_phases.size:
        cl = phase_err(np.exp(1j * out.closure_phases[fin]), np.exp(1j * ref.closure_phases[fin]))
        assert cl.max() <= 1e-5


def test_fp64_precision_case():
    hw = (7, 7)
    cfg = StackConfig(nslc=40, rows=40 + 14, cols=44 + 14, seed=20261206, gamma_inf=0.02, disk_gamma0=0.95,
                      disk_radius=0.3, ps_frac=0.0)
    z = make_stack(cfg)
    mean, disp, _ps = dp.calc_ps_block(np.abs(z), 0.25, cfg.nslc)
    nb = dp.estimate_neighbors(halfwin_rowcol=hw, alpha=0.001, mean=mean, var=(disp * mean) ** 2, nslc=cfg.nslc)
    diag = {}
    ref = O.run_phase_linking(z, hw, neighbor_arrays=nb, dtype=np.float64, diagnostics=diag, eigh_fallback=True)
    flags = np.zeros(z.shape[1:], np.uint8)
    out = dp.run_phase_linking(z, hw, neighbor_arrays=nb, covariance_form="fp64", nonconverged=flags)
    np.testing.assert_array_equal(out.shp_counts, ref.shp_counts)
    np.testing.assert_array_equal(flags.astype(bool), diag["nonconverged"])
    _compare(out, ref, diag, ref.shp_counts >= cfg.nslc)
    # the float32 forms against it: the precision table's denominator on the GPU.  The
    # SIMT form (fused, the coherence never stored) keeps the last iterate: it is compared
    # with the FP64 form doing the same.
    last = dp.run_phase_linking(z, hw, neighbor_arrays=nb, covariance_form="fp64", eigh_fallback=False)
    # the eigenvector's own conditioning, |A| / gap (A = |Gamma|^{-1} o C in float64, the
    # gap to the eigenvalue next to the one nearest the 0.99 shift)
    C64 = O.estimate_stack_covariance(z, hw, neighbor_arrays=nb, dtype=np.float64)
    G = np.abs(C64) + 1e-6 * np.eye(cfg.nslc)
    with np.errstate(all="ignore"):
        w = np.linalg.eigvalsh(np.linalg.inv(G) * C64)
    k = np.argmin(np.abs(w - 0.99), axis=-1)[..., None]
    d = np.abs(w - np.take_along_axis(w, k, -1))
    d.sort(axis=-1)
    cond = np.abs(w).max(-1) / d[..., 1]
    # relative rounding of each form's covariance sums: bf16 hi/lo products (about
    # 2^-17), fp32 SIMT sums (a few ulp)
    eps = {"tensor": 2.0 ** -17, "simt": 2.0 ** -22}
    for form, ref_form in (("tensor", out), ("simt", last)):
        f32 = np.zeros(z.shape[1:], np.uint8)
        o32 = dp.run_phase_linking(z, hw, neighbor_arrays=nb, covariance_form=form, nonconverged=f32)
        good = (ref_form.temp_coh > 0.3) & (diag["gamma_min_eig"] >= 1e-3)
        err = phase_err(o32.cpx_phase[:, good], ref_form.cpx_phase[:, good]).max(0)
        tol = np.maximum(2e-3, eps[form] * cond[good])
        above = err > 1e-3
        differ = (f32.astype(bool) != flags.astype(bool))[good]
        worst = int(np.argmax(err / tol))
        print(f"[fp64] form={form:6s} vs GPU float64: phase err max {err.max():.2e} rad on {good.sum()} pixels, "
              f"{int(above.sum())} above 1e-3 ({int((above & differ).sum())} of them where only one of the two "
              f"forms met the stopping rule); {int(f32.sum())} / {int(flags.sum())} dense-eigensolver pixels; "
              f"worst against its bound: {err[worst]:.2e} rad, |A|/gap {cond[good][worst]:.2e}")
        # slowly converging pixels (contraction near 1 per step) carry the stopping rule's
        # own error, |step| / (1 - ratio), up to ~1e-3 rad in either form; where the
        # eigenvalue gap is small the covariance's rounding moves the eigenvector by about
        # eps |A| / gap, whatever solves it
        assert np.all(err <= tol) and above.mean() <= 1e-3


@pytest.mark.parametrize("kw", [
    dict(),
    dict(strides=(2, 3)),
    dict(use_evd=True),
    dict(beta=0.1, zero_correlation_threshold=0.05),
    dict(baseline_lag=4),
    dict(reference_idx=3, first_real_slc_idx=2),
])
def test_fp64_options_against_oracle(kw):
    cfg = StackConfig(nslc=10, rows=30, cols=34, seed=20261204, ps_frac=0.05)
    z = make_stack(cfg)
    z[2, 4, 5] = np.nan
    z[:, 10, 11] = np.nan
    mean, disp, ps = dp.calc_ps_block(np.abs(z), 0.25, cfg.nslc)
    hw = (5, 5)
    strides = kw.pop("strides", (1, 1))
    nb = dp.estimate_neighbors(halfwin_rowcol=hw, alpha=0.001, strides=strides, mean=mean, var=(disp * mean) ** 2,
                               nslc=cfg.nslc)
    diag = {}
    ref = O.run_phase_linking(z, hw, strides, ps_mask=ps, neighbor_arrays=nb, avg_mag=mean, dtype=np.float64,
                              diagnostics=diag, eigh_fallback=True, **kw)
    out = dp.run_phase_linking(z, hw, strides, ps_mask=ps, neighbor_arrays=nb, avg_mag=mean,
                               covariance_form="fp64", **kw)
    np.testing.assert_array_equal(out.shp_counts, ref.shp_counts)
    _compare(out, ref, diag, ref.shp_counts >= cfg.nslc)


def test_fp64_rejected_by_covariance_entry():
    z = make_stack(StackConfig(nslc=4, rows=8, cols=8, seed=1, ps_frac=0.0))
    with pytest.raises(ValueError):
        dp.estimate_stack_covariance(z, (1, 1), covariance_form="fp64")
