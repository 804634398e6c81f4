"""Phase-similarity raster on the GPU against the golden vectors of the reference's own
similarity.py and against the oracle on seeded stacks.

Tolerance: the GPU sums the float32 products of a pixel pair in float32 (fused
multiply-adds), the reference in float64; over n <= 64 layers of unit phasors the
similarities agree to 5e-6, and a median or a maximum of values that agree to e
agrees to e.  NaN patterns and the in-place mask update are exact.
"""

import numpy as np
import pytest

from oracle import similarity as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import dolphin_gb300 as dp  # noqa: E402
from dolphin_gb300 import _lib  # noqa: E402
from dolphin_gb300.simulate import StackConfig, make_stack  # noqa: E402

TOL = 5e-6


def _same(a, b, tol=TOL):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    nan_a, nan_b = np.isnan(a), np.isnan(b)
    assert np.array_equal(nan_a, nan_b), f"NaN pattern differs at {np.argwhere(nan_a != nan_b)[:5].tolist()}"
    ok = ~nan_b
    if ok.any():
        err = np.max(np.abs(a[ok].astype(np.float64) - b[ok]))
        assert err <= tol, err


def _ifgs(seed, n, rows, cols):
    z = make_stack(StackConfig(nslc=n + 1, rows=rows, cols=cols, seed=seed, ps_frac=0.0))
    return (z[1:] * np.conj(z[:1])).astype(np.complex64)


def test_golden_cases(golden):
    g = golden("similarity")
    for k in range(int(g["ncases"])):
        stack, radius = g[f"case_{k}_stack"], int(g[f"case_{k}_radius"])
        masked = f"case_{k}_mask_in" in g
        m1 = g[f"case_{k}_mask_in"].copy() if masked else None
        m2 = g[f"case_{k}_mask_in"].copy() if masked else None
        med = dp.median_similarity(stack, radius, mask=m1)
        mx = dp.max_similarity(stack, radius, mask=m2)
        assert med.dtype == np.float32 and med.shape == stack.shape[1:]
        _same(med, g[f"case_{k}_median"])
        _same(mx, g[f"case_{k}_max"])
        if masked:
            assert np.array_equal(m1, g[f"case_{k}_mask_after"])
            assert np.array_equal(m2, g[f"case_{k}_mask_after"])


def test_golden_nearest_n(golden):
    g = golden("similarity")
    got = dp.stack_similarity(g["nn_stack"], search_radius=3, sim_type="median", nearest_n=3)
    _same(got, g["nn_median"])


@pytest.mark.parametrize("radius", [2, 3, 4, 7, 9, 11, 12, 16])
def test_oracle_seeded(radius):
    rng = np.random.default_rng(900 + radius)
    a = _ifgs(900 + radius, 17, 37, 70)
    a[:, 3, 4] = np.nan
    a[:, 10, 60] = 0
    a[5, 20, 20] = np.nan
    mask = rng.random(a.shape[1:]) > 0.15
    for kind in ("median", "max"):
        m_gpu, m_ref = mask.copy(), mask.copy()
        got = getattr(dp, f"{kind}_similarity")(a, radius, mask=m_gpu)
        ref = getattr(O, f"{kind}_similarity")(a, radius, m_ref)
        _same(got, ref)
        assert np.array_equal(m_gpu, m_ref)


@pytest.mark.parametrize("n", [1, 2, 5, 33, 64])
def test_layer_counts_and_real_phase(n):
    a = _ifgs(950 + n, n, 21, 45)
    _same(dp.median_similarity(a, 7), O.median_similarity(a, 7))
    ph = np.angle(a).astype(np.float32)
    ph[:, 2, 2] = 0.0
    _same(dp.max_similarity(ph, 5), O.max_similarity(ph, 5))


@pytest.mark.parametrize("shape", [(1, 1), (1, 40), (40, 1), (2, 3), (33, 31), (65, 97)])
def test_edges_and_small_images(shape):
    a = _ifgs(970, 6, *shape)
    for radius in (2, 5, 7, 11, 16):
        _same(dp.median_similarity(a, radius), O.median_similarity(a, radius))
        _same(dp.max_similarity(a, radius), O.max_similarity(a, radius))


def test_nearest_n_against_oracle():
    a = _ifgs(980, 11, 30, 41)
    a[:, 4, 4] = np.nan
    a[2, 9, 9] = np.nan
    for nn in (1, 3, 5):
        ref = O.median_similarity(O.nearest_diffs(a, nn), 5)
        _same(dp.stack_similarity(a, 5, "median", nearest_n=nn), ref)
        ref_max = O.max_similarity(O.nearest_diffs(a, nn), 5)
        _same(dp.stack_similarity(a, 5, "max", nearest_n=nn), ref_max)


def test_device_tensors_and_mask_in_place():
    a = _ifgs(990, 9, 26, 33)
    mask = np.ones(a.shape[1:], bool)
    mask[::3, ::4] = False
    a[:, 1, 1] = 0
    ref_mask = mask.copy()
    ref = O.median_similarity(a, 7, ref_mask)
    dm = torch.from_numpy(mask.copy()).cuda()
    got = dp.median_similarity(torch.from_numpy(a).cuda(), 7, mask=dm)
    assert got.is_cuda and got.dtype == torch.float32
    _same(got.cpu().numpy(), ref)
    assert np.array_equal(dm.cpu().numpy(), ref_mask)


def test_no_offsets_no_layers_and_limits():
    a = _ifgs(991, 4, 6, 7)
    assert np.isnan(dp.median_similarity(a, 1)).all()  # radius 1: empty circle
    assert np.isnan(dp.max_similarity(np.zeros((0, 6, 7), np.complex64), 3)).all()
    assert np.isnan(dp.median_similarity(np.zeros((5, 4, 5), np.complex64), 2)).all()
    assert np.isnan(dp.median_similarity(np.full((5, 4, 5), np.nan, np.complex64), 2)).all()
    with pytest.raises(_lib.DplError):
        dp.median_similarity(a, dp.similarity._lib.load().dpl_similarity_max_radius() + 1)


def test_large_frame_interior_against_oracle_crop():
    """A 1000 x 1200 frame, 30 layers, radius 7 and 11: the oracle on two crops; pixels
    farther than the radius from a crop edge see the same neighbours in both."""
    a = _ifgs(992, 30, 1000, 1200)
    rng = np.random.default_rng(5)
    a[:, rng.integers(0, 1000, 300), rng.integers(0, 1200, 300)] = np.nan
    for radius in (7, 11):
        got = dp.median_similarity(a, radius)
        h = radius - 1
        for r0, c0 in [(0, 0), (500, 700)]:
            crop = a[:, r0:r0 + 60, c0:c0 + 80]
            ref = O.median_similarity(crop, radius)
            rs = slice(0 if r0 == 0 else h, 60 - h)
            cs = slice(0 if c0 == 0 else h, 80 - h)
            _same(got[r0:r0 + 60, c0:c0 + 80][rs, cs], ref[rs, cs])
