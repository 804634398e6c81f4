"""Phase similarity, CPU side: the oracle against the golden vectors made from the
reference's own similarity.py, and the library's host-side pieces (the search circle,
the per-pair helper, the nearest-n pair count) against the same vectors."""

import numpy as np
import pytest

from oracle import similarity as O


@pytest.fixture(scope="module")
def g(golden):
    return golden("similarity")


@pytest.fixture(scope="module")
def sim():
    from dolphin_gb300 import _build

    _build.build_library()
    from dolphin_gb300 import similarity

    return similarity


def _same(a, b, tol):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.array_equal(np.isnan(a), np.isnan(b))
    ok = ~np.isnan(b)
    if ok.any():
        assert np.max(np.abs(a[ok].astype(np.float64) - b[ok])) <= tol


def test_oracle_circle_matches_reference(g):
    for radius in range(1, 26):
        assert np.array_equal(O.circle_offsets(radius).reshape(-1, 2), g[f"circle_{radius}"]), radius
    for radius, rmin in [(5, 0), (7, 2), (9, 4)]:
        raw = O.circle_offsets(radius, min_radius=rmin, sort_output=False).reshape(-1, 2)
        assert np.array_equal(raw, g[f"circle_raw_{radius}_{rmin}"])


def test_oracle_rasters_match_reference(g):
    for k in range(int(g["ncases"])):
        stack, radius = g[f"case_{k}_stack"], int(g[f"case_{k}_radius"])
        masked = f"case_{k}_mask_in" in g
        m1 = g[f"case_{k}_mask_in"].copy() if masked else None
        m2 = g[f"case_{k}_mask_in"].copy() if masked else None
        _same(O.median_similarity(stack, radius, m1), g[f"case_{k}_median"], 1e-6)
        _same(O.max_similarity(stack, radius, m2), g[f"case_{k}_max"], 1e-6)
        if masked:
            assert np.array_equal(m1, g[f"case_{k}_mask_after"])


def test_oracle_nearest_n_matches_reference(g):
    pairs = O.nearest_n_pairs(g["nn_stack"].shape[0] + 1, 3)
    assert pairs == [tuple(p) for p in g["nn_pairs"].tolist()]
    d = O.nearest_diffs(g["nn_stack"], 3)
    _same(d.real, g["nn_diffs"].real, 0)
    _same(O.median_similarity(d, 3), g["nn_median"], 1e-6)


def test_oracle_phase_similarity(g):
    assert abs(O.phase_similarity(g["ps_x1"], g["ps_x2"]) - g["ps_val"][0]) < 1e-6
    assert abs(O.phase_similarity(g["ps_x1"], g["ps_x1"]) - 1.0) < 1e-6
    assert O.phase_similarity(np.zeros(10, np.complex64), np.zeros(10, np.complex64)) == 0
    assert np.isnan(O.phase_similarity(np.full(10, np.nan, np.complex64), np.full(10, np.nan, np.complex64)))


def test_library_circle_matches_reference(g, sim):
    for radius in range(1, 26):
        got = sim.get_circle_idxs(radius)
        ref = g[f"circle_{radius}"]
        if len(ref) == 0:
            assert got.shape == (0,)
        else:
            assert got.dtype == np.int64
            assert np.array_equal(got, ref), radius
    for radius, rmin in [(5, 0), (7, 2), (9, 4)]:
        assert np.array_equal(sim.get_circle_idxs(radius, rmin, False), g[f"circle_raw_{radius}_{rmin}"])
    with pytest.raises(IndexError):
        sim.get_circle_idxs(0)
    with pytest.raises(ValueError):
        sim.get_circle_idxs(-2)


def test_library_host_helpers(g, sim):
    assert abs(sim.phase_similarity(g["ps_x1"], g["ps_x2"]) - g["ps_val"][0]) < 1e-6
    assert sim.phase_similarity(np.ones(10, np.complex64), np.ones(10, np.complex64)) == 1
    n = g["nn_stack"].shape[0]
    assert sim.nearest_n_pair_count(n, 3) == len(g["nn_pairs"])
    for layers in range(0, 12):
        for nn in range(1, 5):
            assert sim.nearest_n_pair_count(layers, nn) == len(O.nearest_n_pairs(layers + 1, nn))


def test_similarity_errors_before_any_device_work(sim):
    stack = np.zeros((3, 4, 5), np.complex64)
    with pytest.raises(ValueError):
        sim.median_similarity(stack, 3, mask=np.ones((4, 4), bool))
    with pytest.raises(ValueError):
        sim.median_similarity(np.zeros((4, 5), np.complex64), 3)
    with pytest.raises(ValueError):
        sim.stack_similarity(stack, 3, sim_type="mean")
    with pytest.raises(IndexError):
        sim.max_similarity(stack, 0)
