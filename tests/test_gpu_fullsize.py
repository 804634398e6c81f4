"""The workload's full block size (N=30, a 1024x1024 block with its (5, 11) halo, GLRT
alpha 0.001, EMI, PS fill, CRLB): size-independent properties of every output, and
parity with the oracle on a crop.

SHP selection, the covariance window and the PS fill are local, so on pixels at least a
half-window inside a crop the crop gives the same inputs to every step as the full
block: there the oracle run on the crop and the GPU run on the full block must agree
(SHP counts exactly; phases within 1e-3 rad and temporal coherence within 1e-4 where the
coherence is above 0.3).
"""

import numpy as np
import pytest

from oracle import phase_link as O
from parity import judge_flips, phase_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import dolphin_gb300 as dp  # noqa: E402
from dolphin_gb300.simulate import StackConfig, make_stack_torch  # noqa: E402

N, HALF, ALPHA, PS_THR = 30, (5, 11), 0.001, 0.25
ROWS, COLS = 1024 + 2 * HALF[0], 1024 + 2 * HALF[1]


@pytest.fixture(scope="module")
def block():
    z = make_stack_torch(StackConfig(nslc=N, rows=ROWS, cols=COLS, seed=20261210, ps_frac=0.03))
    mean, disp, ps = dp.calc_ps_block(z.abs(), PS_THR, N)
    nb = dp.estimate_neighbors(halfwin_rowcol=HALF, alpha=ALPHA, mean=mean, var=(disp * mean) ** 2, nslc=N)
    out = dp.run_phase_linking(z, HALF, ps_mask=ps, neighbor_arrays=nb, avg_mag=mean)
    torch.cuda.synchronize()
    return z, ps, nb, out


def test_full_block_properties(block):
    z, ps, nb, out = block
    cpx = out.cpx_phase.cpu().numpy()
    tc = out.temp_coh.cpu().numpy()
    assert cpx.shape == (N, ROWS, COLS) and tc.shape == (ROWS, COLS)
    assert np.isfinite(cpx).all() and np.isfinite(tc).all()  # no nodata in this stack
    np.testing.assert_allclose(np.abs(cpx), 1.0, atol=1e-5)  # unit phasors
    assert np.abs(np.angle(cpx[0])).max() < 1e-5  # referenced to SLC 0 (up to the rounding of the product)
    assert tc.min() >= 0.0 and tc.max() <= 1.0 + 1e-6
    assert (tc[ps.cpu().numpy().astype(bool)] == 1.0).all()  # PS pixels
    est = out.estimator.cpu().numpy()
    assert set(np.unique(est)) <= {0, 1}
    assert np.isfinite(out.eigenvalues.cpu().numpy()).mean() > 0.999
    # SHP counts are the popcount of each pixel's neighbour mask
    counts = out.shp_counts.cpu().numpy()
    np.testing.assert_array_equal(counts, nb.reshape(ROWS, COLS, -1).sum(dim=-1).cpu().numpy())
    assert counts.max() <= (2 * HALF[0] + 1) * (2 * HALF[1] + 1) - 1
    crlb = out.crlb_std_dev.cpu().numpy()
    # 0 at the reference date; NaN where |Gamma|^-1 or the Fisher matrix fails (as in the
    # reference; the crop test below checks where); otherwise non-negative
    assert (crlb[0] == 0).all() and np.isfinite(crlb).mean() > 0.9 and (crlb[np.isfinite(crlb)] >= 0).all()


@pytest.mark.parametrize("r0, c0", [(0, 0), (500, 480), (ROWS - 44, COLS - 66)])
def test_full_block_crop_matches_oracle(block, r0, c0):
    z, ps, nb, out = block
    hy, hx = HALF
    crop = z[:, r0:r0 + 44, c0:c0 + 66].cpu().numpy()
    mean, disp, ps_c = O.calc_ps_block(np.abs(crop), PS_THR, N)
    nb_c = O.estimate_neighbors_glrt(mean, (disp * mean) ** 2, HALF, (1, 1), N, ALPHA)
    ref = O.run_phase_linking(crop, HALF, ps_mask=ps_c.copy(), neighbor_arrays=nb_c, avg_mag=mean)
    ref64 = O.run_phase_linking(crop, HALF, ps_mask=ps_c.copy(), neighbor_arrays=nb_c, avg_mag=mean,
                                dtype=np.float64)
    # interior of the crop, except where the crop touches the block's own edge
    ir0 = 0 if r0 == 0 else hy
    ic0 = 0 if c0 == 0 else hx
    ir1 = 44 if r0 + 44 == ROWS else 44 - hy
    ic1 = 66 if c0 + 66 == COLS else 66 - hx
    sl = (slice(r0 + ir0, r0 + ir1), slice(c0 + ic0, c0 + ic1))
    rs = (slice(ir0, ir1), slice(ic0, ic1))
    np.testing.assert_array_equal(ps.cpu().numpy()[sl].astype(bool), ps_c[rs])
    np.testing.assert_array_equal(out.shp_counts.cpu().numpy()[sl], ref.shp_counts[rs])
    est_g, est_r = out.estimator.cpu().numpy()[sl], ref.estimator[rs]
    # EMI or EVD per pixel hangs on whether |Gamma| + 1e-6 I is positive definite, which
    # rounding decides where |Gamma| is within rounding of singular (PS pixels, whose few
    # SHPs give a near rank-one |Gamma|): those pixels are judged against the float64 answer
    mine = O.PhaseLinkOutput(*(np.asarray(x.cpu().numpy())[(slice(None),) * (x.dim() - 2) + sl]
                               for x in out[:6]), None)
    crop_ref = O.PhaseLinkOutput(*(np.asarray(x)[(slice(None),) * (x.ndim - 2) + rs] for x in ref[:6]), None)
    crop_64 = O.PhaseLinkOutput(*(np.asarray(x)[(slice(None),) * (x.ndim - 2) + rs] for x in ref64[:6]), None)
    flip = judge_flips(mine, crop_ref, crop_64, f"full-block crop ({r0}, {c0})")
    assert not (flip & ~ps_c[rs]).any()
    tc_g, tc_r = out.temp_coh.cpu().numpy()[sl], ref.temp_coh[rs]
    good = (tc_r > 0.3) & (est_g == est_r)
    assert good.sum() > 0
    err = phase_err(out.cpx_phase.cpu().numpy()[(slice(None),) + sl][:, good], ref.cpx_phase[(slice(None),) + rs][:, good])
    assert err.max() <= 1e-3, err.max()
    assert np.abs(tc_g[good] - tc_r[good]).max() <= 1e-4
    # CRLB where C has full rank (at least N SHP samples): the same NaN pattern, and values
    # within 2e-3 relative
    posed = good & (ref.shp_counts[rs] >= N)
    cr_g = out.crlb_std_dev.cpu().numpy()[(slice(None),) + sl][:, posed]
    cr_r = ref.crlb_std_dev[(slice(None),) + rs][:, posed]
    np.testing.assert_array_equal(np.isfinite(cr_g), np.isfinite(cr_r))
    fin = np.isfinite(cr_r)
    np.testing.assert_allclose(cr_g[fin], cr_r[fin], rtol=2e-3, atol=1e-5)
