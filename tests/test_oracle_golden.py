"""Pin the CPU oracle against golden vectors produced by the reference's own code.

The fixtures in ``tests/golden`` come from ``tests/golden/make_golden.py``, which ran
dolphin's phase-linking modules from source (numpy stand-ins for jax/numba).  These
tests need no GPU and no reference checkout.
"""

import ast

import numpy as np
import pytest

from oracle import phase_link as O
from parity import compare_pl


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


def test_run_phase_linking_cases(golden):
    g = golden("phase_link")
    specs = ast.literal_eval(str(g["specs"][0]))
    for idx, spec in specs.items():
        out = _run_case(g, idx, spec)
        compare_pl(out, g, idx)


def test_config1_crop(golden):
    g = golden("config1_crop")
    out = O.run_phase_linking(g["slc"], (5, 5), (1, 1), ps_mask=g["ps"].copy(),
                              neighbor_arrays=g["nb"], avg_mag=g["mean"])
    ref64 = O.run_phase_linking(g["slc"], (5, 5), (1, 1), ps_mask=g["ps"].copy(),
                                neighbor_arrays=g["nb"], avg_mag=g["mean"], dtype=np.float64)
    compare_pl(out, g, "emi", fp64=ref64, label="oracle, config-1 crop")
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


def test_compress_matches_reference(golden):
    g = golden("compress")
    for k in range(int(g["ncases"])):
        first, ref, with_mean = (int(x) for x in g[f"params_{k}"])
        mean = g[f"mean_in_{k}"].copy() if with_mean else None
        out = O.compress(g[f"slc_{k}"], g[f"pl_{k}"], first_real_slc_idx=first, slc_mean=mean,
                         reference_idx=None if ref < 0 else ref)
        np.testing.assert_array_equal(np.isnan(out), np.isnan(g[f"out_{k}"]))
        np.testing.assert_allclose(out, g[f"out_{k}"], rtol=1e-6, atol=1e-6, equal_nan=True)
        if with_mean:  # the given mean is modified in place, as the reference does
            np.testing.assert_array_equal(np.isnan(mean), np.isnan(g[f"mean_after_{k}"]))
