"""GPU parity: each CUDA stage through the C ABI against the golden vectors and the oracle.

Masks (PS, GLRT, KS) must be bit-exact; phases within 1e-3 rad and temporal
coherence within 1e-4 on pixels with coherence > 0.3 (the benchmark spec's tolerances).
"""

import ast

import numpy as np
import pytest

from oracle import phase_link as O
from parity import compare_pl, judge_flips, phase_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import dolphin_gb300 as dp  # noqa: E402
from dolphin_gb300.simulate import StackConfig, make_stack  # noqa: E402

PHASE_TOL = 1e-3  # rad
TC_TOL = 1e-4


# ---------------------------------------------------------------------------------
# PS selection
# ---------------------------------------------------------------------------------
def test_ps_block_golden(golden):
    g = golden("ps_block")
    mag = g["mag"]
    for k, (thr, mc) in enumerate(zip(g["thr"], g["min_count"])):
        mean, disp, ps = dp.calc_ps_block(mag, float(thr), None if mc < 0 else int(mc))
        assert mean.dtype == disp.dtype == np.float32 and ps.dtype == bool
        np.testing.assert_array_equal(mean, g[f"mean_{k}"])
        np.testing.assert_array_equal(disp, g[f"disp_{k}"])
        np.testing.assert_array_equal(ps, g[f"ps_{k}"])


@pytest.mark.parametrize("n", [1, 5, 30, 45, 70])
def test_ps_block_bit_exact_random(n):
    rng = np.random.default_rng(n)
    mag = rng.lognormal(0, 0.6, size=(n, 37, 53)).astype(np.float32)
    mag[rng.random(mag.shape) < 0.02] = np.nan
    mag[:, 3, 4] = np.nan
    mag[:, 5, 6] = 2.5
    for thr, mc in ((0.25, None), (0.5, n), (np.float64(0.3), 1)):
        got = dp.calc_ps_block(mag, thr, mc)
        want = O.calc_ps_block(mag.copy(), thr, mc)
        for a, b in zip(got, want):
            np.testing.assert_array_equal(a, b)


def test_ps_block_rejects_complex():
    with pytest.raises(ValueError):
        dp.calc_ps_block(np.ones((3, 2, 2), np.complex64))


def test_ps_block_empty_and_device_roundtrip():
    mean, disp, ps = dp.calc_ps_block(np.zeros((4, 0, 3), np.float32))
    assert mean.shape == (0, 3)
    mag = torch.rand(6, 8, 9, device="cuda")
    m, d, p = dp.calc_ps_block(mag)
    assert m.is_cuda and p.dtype == torch.uint8
    ref = O.calc_ps_block(mag.cpu().numpy())
    np.testing.assert_array_equal(m.cpu().numpy(), ref[0])


# ---------------------------------------------------------------------------------
# SHP
# ---------------------------------------------------------------------------------
def test_glrt_golden(golden):
    g = golden("glrt")
    for k in range(int(g["ncases"])):
        hy, hx, sy, sx, nslc, alpha = g[f"params_{k}"]
        nb = dp.estimate_neighbors(halfwin_rowcol=(int(hy), int(hx)), strides=(int(sy), int(sx)),
                                   mean=g[f"mean_{k}"], var=g[f"var_{k}"], nslc=int(nslc), alpha=alpha)
        np.testing.assert_array_equal(nb, g[f"nb_{k}"])


@pytest.mark.parametrize("hw,strides", [((5, 5), (1, 1)), ((5, 11), (1, 1)), ((3, 7), (2, 3)), ((7, 7), (4, 1)),
                                        ((0, 0), (1, 1)), ((10, 31), (1, 2))])
def test_glrt_vs_oracle(hw, strides):
    rng = np.random.default_rng(17)
    amp = rng.rayleigh(10.0, size=(20, 67, 141)).astype(np.float32)
    amp[:, 10:30, 40:90] *= 2.5
    mean, var = amp.mean(0), amp.var(0)
    mean[:2, :3] = 0
    var[5, 7] = np.nan
    nb = dp.estimate_neighbors(halfwin_rowcol=hw, strides=strides, mean=mean, var=var, nslc=20, alpha=0.001)
    check_glrt_masks(nb, mean, var, hw, strides, 20, 0.001, f"GLRT {hw} {strides}")


def check_glrt_masks(nb, mean, var, hw, strides, nslc, alpha, label):
    """GLRT masks against the oracle: equal to the exact decision (the statistic in
    float64 on the float32 scale^2) apart from tests within 1e-6 (relative) of the
    cutoff, which are counted; against the float32 evaluation (the reference's
    arithmetic) they differ only where float32 rounding flips that evaluation itself."""
    ref, _stat, _thr = O.estimate_neighbors_glrt(mean, var, hw, strides, nslc, alpha, return_stat=True)
    exact, xstat, xthr = O.estimate_neighbors_glrt(mean, var, hw, strides, nslc, alpha, return_stat=True,
                                                   exact=True)
    near = np.abs(xstat - xthr) <= 1e-6 * xthr
    diff = nb != exact
    assert not (diff & ~near).any(), np.argwhere(diff & ~near)[:5]
    flipped32 = ref != exact
    diff32 = nb != ref
    assert not (diff32 & ~(flipped32 | near)).any()
    print(f"{label}: {int(near.sum())} tests within 1e-6 of the cutoff ({int((diff & near).sum())} of them "
          f"differ from the exact decision); {int(flipped32.sum())} float32 decisions flipped by rounding")
    return int(near.sum()), int((diff & near).sum()), int(flipped32.sum())


def test_glrt_near_cutoff_is_exact():
    """Neighbours whose statistic sits 1e-9 .. 1e-4 (relative) from the cutoff: every
    GPU decision is the exact one."""
    from scipy import stats

    nslc, alpha = 20, 0.001
    thr = float(np.float32(stats.chi2.ppf(1 - alpha, df=1)))
    c = np.expm1(thr / nslc)
    r_star = ((2 + 4 * c) + np.sqrt((2 + 4 * c) ** 2 - 4)) / 2  # T(1, r*) = thr
    deltas = np.concatenate([-np.logspace(-9, -4, 400), np.logspace(-9, -4, 400)])
    s = np.ones(2 * deltas.size + 1, np.float64)
    s[1::2] = r_star * (1 + deltas)
    s = s.astype(np.float32)
    # mean 0: scale^2 = var / 2 exactly
    var = np.tile(2 * s, (3, 1)).astype(np.float32)
    mean = np.zeros_like(var)
    nb = dp.estimate_neighbors(halfwin_rowcol=(0, 1), mean=mean, var=var, nslc=nslc, alpha=alpha)
    near, near_diff, flipped = check_glrt_masks(nb, mean, var, (0, 1), (1, 1), nslc, alpha, "GLRT near the cutoff")
    # exact even within 1e-6 of the cutoff (how many float32 evaluations flip depends on
    # the host's float32 log; check_glrt_masks prints it)
    assert near > 0 and near_diff == 0


def test_glrt_window_larger_than_image():
    with pytest.raises(ValueError):
        dp.estimate_neighbors(halfwin_rowcol=(5, 5), mean=np.ones((4, 20), np.float32),
                              var=np.ones((4, 20), np.float32), nslc=3, alpha=0.01)


def test_glrt_requires_nslc():
    with pytest.raises(ValueError):
        dp.estimate_neighbors(halfwin_rowcol=(1, 1), mean=np.ones((4, 4)), var=np.ones((4, 4)), alpha=0.01)


def test_shp_rect_and_unknown():
    assert dp.estimate_neighbors(halfwin_rowcol=(1, 1), alpha=0.1, method="rect") is None
    with pytest.raises(ValueError):
        dp.estimate_neighbors(halfwin_rowcol=(1, 1), alpha=0.1, method="nope", nslc=3,
                              mean=np.ones((4, 4)), var=np.ones((4, 4)))


def test_ks_golden(golden):
    g = golden("ks")
    for k in range(int(g["ncases"])):
        hy, hx, sy, sx, alpha = g[f"params_{k}"]
        nb = dp.estimate_neighbors(halfwin_rowcol=(int(hy), int(hx)), strides=(int(sy), int(sx)),
                                   amp_stack=g[f"amp_{k}"], alpha=alpha, method="ks")
        np.testing.assert_array_equal(nb, g[f"nb_{k}"])


@pytest.mark.parametrize("n", [7, 30, 64])
def test_ks_vs_oracle(n):
    rng = np.random.default_rng(n)
    amp = rng.rayleigh(5.0, size=(n, 23, 29)).astype(np.float32)
    amp[:, :8] *= 1.7
    amp[:, 12, 12] = amp[:, 12, 13]  # exact ties
    nb = dp.estimate_neighbors(halfwin_rowcol=(2, 3), amp_stack=amp, alpha=0.05, method="ks")
    ref = O.estimate_neighbors_ks(amp, (2, 3), (1, 1), 0.05)
    np.testing.assert_array_equal(nb, ref)
    srt = np.sort(amp, axis=0)
    nb2 = dp.estimate_neighbors(halfwin_rowcol=(2, 3), amp_stack=srt, alpha=0.05, method="ks", is_sorted=True)
    np.testing.assert_array_equal(nb2, ref)


def test_ks_requires_amp_stack():
    with pytest.raises(ValueError):
        dp.estimate_neighbors(halfwin_rowcol=(1, 1), alpha=0.1, method="ks")


# ---------------------------------------------------------------------------------
# covariance
# ---------------------------------------------------------------------------------
# fp32 SIMT sums vs bf16 hi/lo products with fp32 accumulation
# tf32 operands carry 11 significant bits: 2^-11 relative per sample product
COV_ATOL = {"simt": 5e-6, "tensor": 3e-5, "tf32": 2e-3}


@pytest.mark.parametrize("form", ["tensor", "simt"])
def test_covariance_golden(golden, form):
    g = golden("covariance")
    z = g["slc"]
    tol = COV_ATOL[form]
    kw = dict(covariance_form=form)
    np.testing.assert_allclose(dp.estimate_stack_covariance(z, (3, 4), (1, 1), **kw), g["C_rect"], atol=tol)
    np.testing.assert_allclose(dp.estimate_stack_covariance(z, (3, 4), (1, 1), g["nb"], **kw), g["C_nb"], atol=tol)
    np.testing.assert_allclose(dp.estimate_stack_covariance(z, (3, 4), (2, 3), **kw), g["C_strided"], atol=tol)


@pytest.mark.parametrize("form", ["tensor", "simt", "tf32"])
@pytest.mark.parametrize("n", [3, 20, 30, 33, 64])
def test_covariance_vs_float64(n, form):
    z = make_stack(StackConfig(nslc=n, rows=19, cols=27, seed=n, ps_frac=0.0))
    z[1, 4, 5] = np.nan
    got = dp.estimate_stack_covariance(z, (2, 3), (1, 2), covariance_form=form)
    ref = O.estimate_stack_covariance(z.astype(np.complex128), (2, 3), (1, 2), dtype=np.float64)
    np.testing.assert_allclose(got, ref, atol=COV_ATOL[form])


@pytest.mark.parametrize("form", ["tensor", "simt", "tf32"])
def test_covariance_with_shp_masks(form):
    """Masks with holes and a PS-like bright pixel, large window (5, 11), tile edges."""
    z = make_stack(StackConfig(nslc=30, rows=37, cols=70, seed=9, ps_frac=0.03))
    amp = np.abs(z)
    mean, disp, ps = O.calc_ps_block(amp, 0.25, 30)
    nb = O.estimate_neighbors_glrt(mean, (disp * mean) ** 2, (5, 11), (1, 1), 30, 0.001)
    got = dp.estimate_stack_covariance(z, (5, 11), (1, 1), nb, covariance_form=form)
    ref = O.estimate_stack_covariance(z.astype(np.complex128), (5, 11), (1, 1), nb, dtype=np.float64)
    np.testing.assert_allclose(got, ref, atol=COV_ATOL[form])


def test_covariance_form_rejects_unknown():
    with pytest.raises(ValueError):
        dp.estimate_stack_covariance(np.ones((3, 5, 5), np.complex64), (1, 1), covariance_form="nope")


def test_covariance_rejects_real():
    with pytest.raises(ValueError, match="complex"):
        dp.estimate_stack_covariance(np.ones((3, 5, 5), np.float32), (1, 1))


# ---------------------------------------------------------------------------------
# eigen-solvers (process_coherence_matrices), tests modelled on the reference's
# eigen tests: simulated coherence matrices, compared with numpy eigh
# ---------------------------------------------------------------------------------
def _sim_C(n, seed, rows=6, cols=7):
    rng = np.random.default_rng(seed)
    gamma = (0.99 - 0.95) * np.exp(-np.abs(np.subtract.outer(np.arange(n), np.arange(n))) * 12 / 72) + 0.95
    np.fill_diagonal(gamma, 1.0)
    out = np.empty((rows, cols, n, n), np.complex64)
    for r in range(rows):
        for c in range(cols):
            ph = rng.normal(scale=0.5, size=n)
            out[r, c] = gamma * np.exp(1j * np.subtract.outer(ph, ph))
    return out


def test_evd_matches_eigh():
    C = _sim_C(20, 1)
    vec, val, est, _ = dp.process_coherence_matrices(C, use_evd=True, compute_crlb=False)
    w, v = np.linalg.eigh(C * np.abs(C))
    np.testing.assert_allclose(val, w[..., -1], rtol=2e-5)
    ref = v[..., -1] * np.exp(-1j * np.angle(v[..., :1, -1]))
    assert phase_err(vec, ref).max() < 5e-3
    assert (est == 0).all()


def test_emi_matches_eigh():
    C = _sim_C(20, 2)
    vec, val, est, _ = dp.process_coherence_matrices(C, compute_crlb=False)
    A = C * np.linalg.inv(np.abs(C).astype(np.float64) + 1e-6 * np.eye(20))
    w, v = np.linalg.eigh(A)
    np.testing.assert_allclose(val, w[..., 0], atol=2e-4)
    ref = v[..., 0] * np.exp(-1j * np.angle(v[..., :1, 0]))
    assert phase_err(vec, ref).max() < 1e-3
    assert (est == 1).all()


@pytest.mark.parametrize("n,kw", [
    (10, dict()),
    (30, dict(beta=0.1, zero_correlation_threshold=0.05, reference_idx=3, first_real_slc_idx=4)),
    (45, dict(use_evd=True)),
    (64, dict(reference_idx=-1)),
])
def test_process_coherence_vs_oracle(n, kw):
    z = make_stack(StackConfig(nslc=n, rows=18, cols=20, seed=100 + n, ps_frac=0.0))
    C = O.estimate_stack_covariance(z, (5, 5), (1, 1))
    vec, val, est, crlb, tc, clos = dp.process_coherence_matrices(C, num_looks=5.0, return_metrics=True, **kw)
    okw = dict(kw)
    ref_idx = okw.pop("reference_idx", 0)
    ref_idx = ref_idx + n if ref_idx < 0 else ref_idx
    rv, rl, re_, rc = O.process_coherence_matrices(C.reshape(-1, n, n), num_looks=5.0, reference_idx=ref_idx, **okw)
    rtc = O.estimate_temp_coh(rv, C.reshape(-1, n, n))
    np.testing.assert_array_equal(est.ravel(), re_)
    good = rtc > 0.3
    assert phase_err(vec.reshape(-1, n)[good], rv[good]).max() < PHASE_TOL
    np.testing.assert_allclose(np.abs(vec.reshape(-1, n)), np.abs(rv), rtol=1e-3, atol=1e-4)
    np.testing.assert_allclose(val.ravel(), rl, rtol=1e-3)
    assert np.abs(tc.ravel() - rtc)[good].max() < TC_TOL
    np.testing.assert_allclose(crlb.reshape(-1, n), rc, rtol=3e-3, atol=1e-5)
    rcl = O.closure_phases(C.reshape(-1, n, n))
    assert phase_err(np.exp(1j * clos.reshape(rcl.shape)), np.exp(1j * rcl)).max() < 1e-5


def test_singular_gamma_falls_back_to_evd():
    # duplicate SLC -> rank-deficient C -> the Cholesky of |C| fails -> EVD, estimator 0
    n = 8
    C = np.ones((1, n, n), np.complex64) * 0.999
    C[0][np.diag_indices(n)] = 1
    C[0, :, 3] = C[0, :, 2]
    C[0, 3, :] = C[0, 2, :]
    vec, val, est, crlb = dp.process_coherence_matrices(C)
    rv, rl, re_, rc = O.process_coherence_matrices(C)
    np.testing.assert_array_equal(est, re_)
    np.testing.assert_array_equal(np.isnan(crlb), np.isnan(rc))


# ---------------------------------------------------------------------------------
# run_phase_linking end to end
# ---------------------------------------------------------------------------------
@pytest.mark.parametrize("form", ["tensor", "simt"])
def test_run_phase_linking_golden_cases(golden, form):
    g = golden("phase_link")
    specs = ast.literal_eval(str(g["specs"][0]))
    for idx, (zname, hw, strides, kw) in specs.items():
        kw = dict(kw)
        for key in ("ps_mask", "nodata_mask", "neighbor_arrays", "avg_mag"):
            if key in kw:
                kw[key] = np.array(g[kw[key]])
        okw = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in kw.items()}
        ref64 = O.run_phase_linking(np.array(g[zname]), hw, strides, dtype=np.float64, eigh_fallback=True, **okw)
        z = np.array(g[zname])
        flags = np.zeros((z.shape[1] // strides[0], z.shape[2] // strides[1]), np.uint8)
        out = dp.run_phase_linking(z, hw, strides, covariance_form=form, nonconverged=flags, **kw)
        compare_pl(out, g, idx, fp64=ref64, label=f"golden case {idx} ({form})", nonconverged=flags)


@pytest.mark.parametrize("form", ["tensor", "simt"])
def test_config1_crop_golden(golden, form):
    g = golden("config1_crop")
    ref64 = O.run_phase_linking(g["slc"], (5, 5), (1, 1), ps_mask=g["ps"].copy(), neighbor_arrays=g["nb"],
                                avg_mag=g["mean"], dtype=np.float64, eigh_fallback=True)
    flags = np.zeros(g["slc"].shape[1:], np.uint8)
    out = dp.run_phase_linking(g["slc"], (5, 5), ps_mask=g["ps"], neighbor_arrays=g["nb"], avg_mag=g["mean"],
                               covariance_form=form, nonconverged=flags)
    compare_pl(out, g, "emi", fp64=ref64, label=f"config-1 crop ({form})", nonconverged=flags)


@pytest.mark.parametrize("strides", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("half_window", [5, 11])
@pytest.mark.parametrize("shape", [(10, 11), (15, 20), (50, 75)])
def test_strides_window_sizes(strides, half_window, shape):
    """Mirror of the reference's smoke test over shapes, windows and strides."""
    rng = np.random.default_rng(0)
    data = rng.normal(0, 1, size=(4, *shape)).astype(np.complex64)
    if 2 * half_window + 1 > shape[0]:
        with pytest.raises(ValueError):
            dp.run_phase_linking(data, dp.HalfWindow(half_window, half_window), dp.Strides(strides, strides))
        return
    out = dp.run_phase_linking(data, dp.HalfWindow(half_window, half_window), dp.Strides(strides, strides))
    assert out.cpx_phase.shape == (4, shape[0] // strides, shape[1] // strides)


@pytest.mark.parametrize("form", ["tensor", "simt"])
def test_config1_full_vs_oracle_f32_and_f64(form):
    """Config 1 (N=10, 128x128, hw 5x5, GLRT 0.001, EMI, PS 0.25) against both oracles."""
    z = make_stack(StackConfig())
    amp = np.abs(z)
    mean, disp, ps = dp.calc_ps_block(amp, 0.25, 10)
    var = (disp * mean) ** 2
    nb = dp.estimate_neighbors(halfwin_rowcol=(5, 5), alpha=0.001, mean=mean, var=var, nslc=10)
    out = dp.run_phase_linking(z, (5, 5), ps_mask=ps, neighbor_arrays=nb, avg_mag=mean, covariance_form=form)
    ref = O.run_phase_linking(z, (5, 5), ps_mask=ps.copy(), neighbor_arrays=nb, avg_mag=mean)
    ref64 = O.run_phase_linking(z, (5, 5), ps_mask=ps.copy(), neighbor_arrays=nb, avg_mag=mean, dtype=np.float64)
    flip = judge_flips(out, ref, ref64, f"config 1 ({form})")
    # against the FP64 oracle on every coherent pixel, flips included
    good64 = (ref64.temp_coh > 0.3) & np.all(np.isfinite(ref64.cpx_phase), axis=0)
    e64 = phase_err(out.cpx_phase[:, good64], ref64.cpx_phase[:, good64]).max()
    assert e64 < PHASE_TOL, e64
    assert np.abs(out.temp_coh[good64] - ref64.temp_coh[good64]).max() < TC_TOL
    # against the float32 oracle where both chose the same estimator
    good = (ref.temp_coh > 0.3) & ~flip & np.all(np.isfinite(ref.cpx_phase), axis=0)
    assert good.mean() > 0.5
    e32 = phase_err(out.cpx_phase[:, good], ref.cpx_phase[:, good]).max()
    assert e32 < PHASE_TOL, e32
    assert np.abs(out.temp_coh[good] - ref.temp_coh[good]).max() < TC_TOL
    print(f"config 1 ({form}): max phase error {e32:.2e} rad vs float32, {e64:.2e} rad vs float64 oracle")


def test_all_nan_slc_raises():
    z = make_stack(StackConfig(nslc=5, rows=12, cols=12))
    z[2] = np.nan
    with pytest.raises(dp.PhaseLinkRuntimeError, match=r"slc_stack\[\[2\]\] out of 5 are all NaNs."):
        dp.run_phase_linking(z, (2, 2))


def test_deferred_checks_same_outputs_and_errors():
    """Device calls inside deferred_checks() return the synchronous call's outputs, and
    a failing call raises the synchronous call's exception when the block ends."""
    z = torch.from_numpy(make_stack(StackConfig(nslc=8, rows=20, cols=22, seed=31, ps_frac=0.05))).cuda()
    sync = [dp.run_phase_linking(z, (2, 3)), dp.run_phase_linking(z, (2, 3), use_evd=True)]
    with dp.deferred_checks():
        deferred = [dp.run_phase_linking(z, (2, 3)), dp.run_phase_linking(z, (2, 3), use_evd=True)]
    for a, b in zip(sync, deferred):
        for x, y in zip(a, b):
            assert torch.equal(x, y)
    bad = z.clone()
    bad[2] = float("nan")
    with pytest.raises(dp.PhaseLinkRuntimeError, match=r"slc_stack\[\[2\]\] out of 8 are all NaNs."):
        with dp.deferred_checks():
            dp.run_phase_linking(z, (2, 3))
            dp.run_phase_linking(bad, (2, 3))  # returns; the error comes at the end of the block
            dp.run_phase_linking(z, (2, 3))


def test_mask_shape_and_dtype_errors():
    z = make_stack(StackConfig(nslc=5, rows=12, cols=12))
    with pytest.raises(ValueError, match="nodata_mask.shape"):
        dp.run_phase_linking(z, (2, 2), nodata_mask=np.zeros((3, 3), bool))
    with pytest.raises(ValueError, match="complex"):
        dp.run_phase_linking(np.abs(z), (2, 2))


def test_too_many_slcs_is_unsupported():
    z = np.ones((65, 8, 8), np.complex64)
    with pytest.raises(RuntimeError):
        dp.run_phase_linking(z, (1, 1))


def test_shift_nan_edges():
    """Reference test_run_phase_linking_with_shift: NaN rows become nodata rows."""
    z = make_stack(StackConfig(nslc=30, rows=11, cols=11, seed=3, ps_frac=0))
    z[0, 0, :] = np.nan
    z[1, -1, :] = np.nan
    out = dp.run_phase_linking(z, (5, 5))
    assert np.isnan(out.cpx_phase[:, [0, -1], :]).all()
    assert np.isnan(out.temp_coh[[0, -1], :]).all()
    assert np.all(~np.isnan(out.cpx_phase[:, 1:-1, :]))


@pytest.mark.parametrize("use_max_ps", [True, False])
@pytest.mark.parametrize("strides", [1, 2, 3])
def test_ps_fill(use_max_ps, strides):
    """Reference test_run_phase_linking_ps_fill: PS phase copied from the SLCs."""
    z = make_stack(StackConfig(nslc=30, rows=11, cols=11, seed=4, ps_frac=0))
    ps_mask = np.zeros((11, 11), bool)
    ps_mask[2, 2] = True
    out = dp.run_phase_linking(z, (5, 5), (strides, strides), ps_mask=ps_mask, use_max_ps=use_max_ps)
    ps_phase = z[:, 2, 2] * np.conj(z[0, 2, 2])
    o = 2 // strides
    np.testing.assert_allclose(np.angle(out.cpx_phase[:, o, o] * np.conj(ps_phase)), 0, atol=1e-5)
    assert out.temp_coh[o, o] == 1


@pytest.mark.parametrize("use_slc_amp", [False, True])
def test_use_slc_amp(use_slc_amp):
    z = make_stack(StackConfig(nslc=30, rows=11, cols=11, seed=5, ps_frac=0))
    ps_mask = np.zeros((11, 11), bool)
    ps_mask[1, 1] = True
    out = dp.run_phase_linking(z, (5, 5), ps_mask=ps_mask, use_slc_amp=use_slc_amp)
    expected = np.abs(z) if use_slc_amp else 1
    np.testing.assert_allclose(np.abs(out.cpx_phase), expected, rtol=1e-5)


def test_device_tensors_stay_on_device():
    z = make_stack(StackConfig(nslc=8, rows=16, cols=16))
    zt = torch.from_numpy(z).cuda()
    out = dp.run_phase_linking(zt, (2, 2))
    assert out.cpx_phase.is_cuda and out.temp_coh.is_cuda
    host = dp.run_phase_linking(z, (2, 2))
    np.testing.assert_array_equal(out.cpx_phase.cpu().numpy(), host.cpx_phase)


def test_config2_crop_tensor_vs_float64():
    """Config 2 parameters (N=30, half-window (5, 11), GLRT 0.001, EMI, PS 0.25, CRLB) on a
    64 x 96 crop: chosen (tensor) form against the float64 oracle, 1e-3 rad / 1e-4."""
    z = make_stack(StackConfig(nslc=30, rows=64 + 10, cols=96 + 22, seed=20261205, ps_frac=0.03))
    mean, disp, ps = dp.calc_ps_block(np.abs(z), 0.25, 30)
    nb = dp.estimate_neighbors(halfwin_rowcol=(5, 11), alpha=0.001, mean=mean, var=(disp * mean) ** 2, nslc=30)
    out = dp.run_phase_linking(z, (5, 11), ps_mask=ps, neighbor_arrays=nb, avg_mag=mean)
    ref64 = O.run_phase_linking(z, (5, 11), ps_mask=ps.copy(), neighbor_arrays=nb, avg_mag=mean, dtype=np.float64)
    # every coherent pixel against the float64 oracle, estimator flips included
    good = (ref64.temp_coh > 0.3) & np.all(np.isfinite(ref64.cpx_phase), axis=0)
    assert good.mean() > 0.8
    err = phase_err(out.cpx_phase[:, good], ref64.cpx_phase[:, good].astype(np.complex64))
    assert err.max() < PHASE_TOL, err.max()
    assert np.abs(out.temp_coh[good] - ref64.temp_coh[good]).max() < TC_TOL
    flip = out.estimator != ref64.estimator
    # the estimator differs only on PS pixels, whose phase PS filling replaces (their
    # |Gamma| is near rank one, within float32 rounding of singular)
    assert not (flip & ~ps.astype(bool)).any()
    print(f"config-2 crop: max phase error {err.max():.2e} rad vs float64; {int(flip.sum())} estimator flips, "
          f"all on PS pixels")


# ---------------------------------------------------------------------------------
# compressed SLC (phase_link/_compress.py:11-65)
# ---------------------------------------------------------------------------------
def test_compress_golden(golden):
    g = golden("compress")
    for k in range(int(g["ncases"])):
        first, ref, with_mean = (int(x) for x in g[f"params_{k}"])
        mean = g[f"mean_in_{k}"].copy() if with_mean else None
        out = dp.compress(g[f"slc_{k}"], g[f"pl_{k}"], first_real_slc_idx=first, slc_mean=mean,
                          reference_idx=None if ref < 0 else ref)
        want = g[f"out_{k}"]
        assert out.dtype == np.complex64 and out.shape == want.shape
        np.testing.assert_array_equal(np.isnan(out), np.isnan(want))
        ok = ~np.isnan(want)
        np.testing.assert_allclose(np.abs(out[ok]), np.abs(want[ok]), rtol=2e-6)
        assert phase_err(out[ok], want[ok]).max() < 1e-5
        if with_mean:
            np.testing.assert_array_equal(np.isnan(mean), np.isnan(g[f"mean_after_{k}"]))


@pytest.mark.parametrize("strides", [1, 3])
def test_compress_magnitude_is_stack_mean(strides):
    # the reference's own property test (tests/test_phase_link_compress.py): with the
    # stack's phase-linked phase, |compressed| is the mean amplitude, NaN beyond the
    # upsampled area
    z = make_stack(StackConfig(nslc=10, rows=11, cols=11, seed=77, ps_frac=0.0))
    out = dp.run_phase_linking(z, (3, 3), (strides, strides), compute_crlb=False)
    comp = dp.compress(z, out.cpx_phase)
    vr, vc = 11 // strides * strides, 11 // strides * strides
    np.testing.assert_allclose(np.abs(comp)[:vr, :vc], np.abs(z).mean(axis=0)[:vr, :vc], rtol=1e-5)
    assert np.isnan(np.abs(comp)[vr:, :]).all() and np.isnan(np.abs(comp)[:, vc:]).all()
    rc = O.compress(z, out.cpx_phase)
    assert phase_err(comp[:vr, :vc], rc[:vr, :vc]).max() < 1e-5


def test_compress_device_tensors_and_errors():
    z = make_stack(StackConfig(nslc=6, rows=8, cols=9, seed=78, ps_frac=0.0))
    pl = np.exp(1j * np.angle(z)).astype(np.complex64)
    mean = torch.from_numpy(np.abs(z).mean(axis=0).astype(np.float32)).cuda()
    comp = dp.compress(torch.from_numpy(z).cuda(), torch.from_numpy(pl).cuda(), slc_mean=mean, reference_idx=-1)
    assert comp.is_cuda and comp.dtype == torch.complex64
    rc = O.compress(z, pl, slc_mean=np.abs(z).mean(axis=0).astype(np.float32), reference_idx=5)
    assert phase_err(comp.cpu().numpy(), rc).max() < 1e-5
    with pytest.raises(IndexError):
        dp.compress(z, pl, reference_idx=6)
    with pytest.raises(ValueError):
        dp.compress(z, pl[:3])
