"""The warm-start network's numpy oracle: gradients against finite differences."""

import numpy as np

from oracle import mlp as M


def _net(rng, sizes):
    Ws = [rng.normal(scale=1 / np.sqrt(a), size=(b, a)) for a, b in zip(sizes[:-1], sizes[1:])]
    bs = [rng.normal(scale=0.1, size=b) for b in sizes[1:]]
    return Ws, bs


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(5)
    sizes = [7, 9, 6, 4]
    Ws, bs = _net(rng, sizes)
    X = rng.normal(size=(11, sizes[0]))
    T = rng.normal(size=(11, sizes[-1]))
    gW, gb = M.backward(X, T, Ws, bs)
    h = 1e-6
    for k in range(len(Ws)):
        for (a, b) in [(0, 0), (sizes[k + 1] - 1, sizes[k] - 1), (1, 2)]:
            Wp = [w.copy() for w in Ws]
            Wp[k][a, b] += h
            Wm = [w.copy() for w in Ws]
            Wm[k][a, b] -= h
            fd = (M.mse(M.forward(X, Wp, bs)[-1], T) - M.mse(M.forward(X, Wm, bs)[-1], T)) / (2 * h)
            assert abs(fd - gW[k][a, b]) < 1e-6 * max(1.0, abs(fd))
        bp = [b.copy() for b in bs]
        bp[k][0] += h
        bm = [b.copy() for b in bs]
        bm[k][0] -= h
        fd = (M.mse(M.forward(X, Ws, bp)[-1], T) - M.mse(M.forward(X, Ws, bm)[-1], T)) / (2 * h)
        assert abs(fd - gb[k][0]) < 1e-6 * max(1.0, abs(fd))


def test_features_order():
    C = np.arange(2 * 4 * 4).reshape(2, 4, 4).astype(np.complex64)
    f = M.features(C)
    assert f.shape == (2, 6)
    np.testing.assert_array_equal(f[0], [4, 8, 9, 12, 13, 14])  # (1,0), (2,0), (2,1), (3,0), (3,1), (3,2)


def test_adam_step_moves_against_gradient():
    w = np.ones(3)
    m, v = np.zeros(3), np.zeros(3)
    M.adam_step(w, np.array([1.0, -1.0, 0.0]), m, v, 0.1, 0.9, 0.999, 1e-8, 1)
    np.testing.assert_allclose(w, [0.9, 1.1, 1.0], atol=1e-6)
