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
