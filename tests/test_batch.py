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
    assert set(forms) == {8, 20} and set(forms.values()) <= {"tensor", "simt"}
    assert path.exists() and tune_forms([8], HW, table_path=path) == {8: forms[8]}
