"""Ministack batch: PS + GLRT + phase linking of uneven-depth stacks as one CUDA graph."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import dolphin_gb300 as dp  # noqa: E402
from dolphin_gb300.batch import PhaseLinkBatch, tune_forms  # noqa: E402
from dolphin_gb300.simulate import StackConfig, make_stack  # noqa: E402

from parity import phase_err  # noqa: E402

HW = (3, 4)


def _stacks(seed0, depths=(8, 20, 36)):
    return [torch.from_numpy(make_stack(StackConfig(nslc=n, rows=40, cols=48, seed=seed0 + n, ps_frac=0.02,
                                                    outlier_frac=0.3))).cuda() for n in depths]


def _single(z, form):
    n = z.shape[0]
    mean, disp, ps = dp.calc_ps_block(z.abs(), 0.25, n)
    nb = dp.estimate_neighbors(halfwin_rowcol=HW, alpha=0.001, mean=mean, var=(disp * mean) ** 2, nslc=n)
    return dp.run_phase_linking(z, HW, ps_mask=ps, neighbor_arrays=nb, avg_mag=mean, covariance_form=form)


@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_single_calls(graph):
    stacks = _stacks(900)
    forms = {8: "tensor", 20: "simt", 36: "tensor"}
    batch = PhaseLinkBatch(stacks, HW, forms=forms, graph=graph)
    for rep in range(2):  # with graph=True the second run is a replay
        outs = batch.run()
        for z, out in zip(stacks, outs):
            want = _single(z, forms[int(z.shape[0])])
            good = torch.isfinite(want.cpx_phase).all(0).cpu().numpy()
            err = phase_err(out.cpx_phase.cpu().numpy()[:, good], want.cpx_phase.cpu().numpy()[:, good])
            assert err.max() < 1e-5, (rep, z.shape[0], err.max())
            assert torch.equal(out.estimator, want.estimator)
            assert torch.equal(out.shp_counts, want.shp_counts)
            np.testing.assert_allclose(out.temp_coh.cpu().numpy(), want.temp_coh.cpu().numpy(), atol=1e-6)


def test_graph_replay_reads_updated_inputs():
    stacks = _stacks(950, depths=(10, 24))
    batch = PhaseLinkBatch(stacks, HW, forms={10: "tensor", 24: "tensor"}, graph=True)
    batch.run()
    fresh = _stacks(990, depths=(10, 24))
    for z, f in zip(stacks, fresh):
        z.copy_(f)
    outs = batch.run()
    for z, out in zip(stacks, outs):
        want = _single(z, "tensor")
        good = torch.isfinite(want.cpx_phase).all(0).cpu().numpy()
        assert phase_err(out.cpx_phase.cpu().numpy()[:, good], want.cpx_phase.cpu().numpy()[:, good]).max() < 1e-5


def test_batch_reports_all_nan_slc_after_replay():
    stacks = _stacks(970, depths=(8, 12))
    batch = PhaseLinkBatch(stacks, HW, forms={8: "tensor", 12: "tensor"}, graph=True)
    batch.run()
    stacks[1][3] = float("nan")
    with pytest.raises(dp.PhaseLinkRuntimeError, match="are all NaNs"):
        batch.run()


def test_tune_forms_table(tmp_path):
    path = tmp_path / "forms.json"
    forms = tune_forms([8, 20], HW, table_path=path, sample=32, reps=1)
    assert set(forms) == {8, 20}
    for n, c in forms.items():
        assert c["form"] in {"tensor", "simt"}
        assert c["slots"] >= n and c["slots"] % 2 == 0 and c["lanes"] in (8, 16, 32) and c["lanes"] >= c["slots"]
    assert path.exists() and tune_forms([8], HW, table_path=path) == {8: forms[8]}


@pytest.mark.parametrize("n", [6, 8, 12, 20, 30, 45])
def test_solver_instances_agree(n):
    """Every register-solver instance the tuner can pick (row slots, threads per pixel)
    gives the default instance's results, up to the order of the group reductions."""
    from dolphin_gb300.batch import _solver_candidates

    z = _stacks(990 + n, depths=(n,))[0]
    mean, disp, ps = dp.calc_ps_block(z.abs(), 0.25, n)
    nb = dp.estimate_neighbors(halfwin_rowcol=HW, alpha=0.001, mean=mean, var=(disp * mean) ** 2, nslc=n)
    kw = dict(ps_mask=ps, neighbor_arrays=nb, avg_mag=mean)
    ref = dp.run_phase_linking(z, HW, **kw)
    for k, g in _solver_candidates(n):
        out = dp.run_phase_linking(z, HW, solver_slots=k, solver_lanes=g, **kw)
        assert torch.equal(out.estimator, ref.estimator), (k, g)
        good = torch.isfinite(ref.cpx_phase).all(0) & (ref.temp_coh > 0.3)
        err = torch.angle(out.cpx_phase[:, good] * ref.cpx_phase[:, good].conj()).abs().max()
        assert float(err) < 1e-5, (k, g, float(err))
        assert float((out.temp_coh - ref.temp_coh)[good].abs().max()) < 1e-5
        fin = torch.isfinite(ref.crlb_std_dev)
        assert torch.equal(fin, torch.isfinite(out.crlb_std_dev))


@pytest.mark.parametrize("graph", [False, True])
def test_persistent_batch_n8_n45(graph):
    """The persistent path (one work-queue covariance launch for every stack): N = 8 and
    45 with the bf16 and the tf32 covariance, bit-identical to the per-stack path, and
    against the oracle."""
    from oracle import phase_link as O

    hw = (5, 5)  # 121 samples: full-rank coherence at N = 45
    stacks = [torch.from_numpy(make_stack(StackConfig(nslc=n, rows=44, cols=52, seed=960 + k, ps_frac=0.02,
                                                      outlier_frac=0.3))).cuda() for k, n in enumerate((8, 45, 12, 45))]
    forms = {8: "tensor", 45: "tensor", 12: "tf32"}
    per = PhaseLinkBatch(stacks, hw, forms=forms, graph=False, persistent=False).run()
    outs = PhaseLinkBatch(stacks, hw, forms=forms, graph=graph, persistent=True).run()
    for z, a, b in zip(stacks, outs, per):
        for x, y in zip(a, b):
            assert torch.equal(torch.nan_to_num(x.float() if not x.is_complex() else torch.view_as_real(x), 7.0),
                               torch.nan_to_num(y.float() if not y.is_complex() else torch.view_as_real(y), 7.0))
    for k in (0, 1):  # N = 8 and 45 against the oracle
        z = stacks[k].cpu().numpy()
        n = z.shape[0]
        mean, disp, ps = O.calc_ps_block(np.abs(z), 0.25, n)
        nb = O.estimate_neighbors_glrt(mean, (disp * mean) ** 2, hw, (1, 1), n, 0.001)
        ref = O.run_phase_linking(z, hw, ps_mask=ps.copy(), neighbor_arrays=nb, avg_mag=mean, dtype=np.float64,
                                  eigh_fallback=True)
        out = outs[k]
        # well-conditioned pixels: at least twice as many SHP samples as SLCs (near N
        # samples the sample coherence is close to singular and float32 rounding of C
        # moves the eigenvector by more than 1e-3 rad)
        good = (ref.temp_coh > 0.3) & np.all(np.isfinite(ref.cpx_phase), axis=0) & \
            (out.estimator.cpu().numpy() == ref.estimator) & (ref.shp_counts >= 2 * n)
        assert good.sum() > 0
        err = phase_err(out.cpx_phase.cpu().numpy()[:, good], ref.cpx_phase[:, good].astype(np.complex64))
        print(f"persistent batch N={n}: max phase error {err.max():.2e} rad vs the float64 oracle on "
              f"{int(good.sum())} pixels")
        assert err.max() < 1e-3
