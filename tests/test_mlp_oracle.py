"""The learned warm start's CPU oracle: analytic gradients against finite
differences (float64, no bf16 rounding), and the feature restatement's basic
invariants.  No GPU."""
import numpy as np

from ncollide_gb300 import workloads as W
from oracle import mlp_oracle as M


def _random_params(rng):
    p = np.zeros(M.N_PARAMS)
    p[M.OFF_W1:M.OFF_B1] = (rng.standard_normal((128, 48)) * 0.2 * (np.arange(48) < M.NF)).flatten()
    p[M.OFF_B1:M.OFF_W2] = rng.standard_normal(128) * 0.1
    p[M.OFF_W2:M.OFF_B2] = rng.standard_normal(128 * 128) * 0.1
    p[M.OFF_B2:M.OFF_W3] = rng.standard_normal(128) * 0.1
    p[M.OFF_W3:M.OFF_B3] = rng.standard_normal(4 * 128) * 0.1
    p[M.OFF_B3:] = rng.standard_normal(4) * 0.1
    return p


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = _random_params(rng)
    X = np.zeros((16, 48))
    X[:, :M.NF] = rng.standard_normal((16, M.NF))
    d = rng.standard_normal((16, 3))
    Y = np.concatenate([d / np.linalg.norm(d, axis=1, keepdims=True), rng.integers(0, 2, (16, 1))], 1)
    g, _, _ = M.forward_backward(p, X, Y, emulate_bf16=False)
    idx = np.concatenate([rng.integers(M.OFF_W1, M.OFF_B1, 6), rng.integers(M.OFF_B1, M.OFF_W2, 3),
                          rng.integers(M.OFF_W2, M.OFF_B2, 6), rng.integers(M.OFF_B2, M.OFF_W3, 3),
                          rng.integers(M.OFF_W3, M.OFF_B3, 6), np.arange(M.OFF_B3, M.N_PARAMS)])
    idx = idx[(idx < M.OFF_B1) & ((idx - M.OFF_W1) % 48 >= M.NF) == False]  # noqa: E712  (skip padded inputs)
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (M.forward_backward(pp, X, Y, emulate_bf16=False)[1][0] -
              M.forward_backward(pm, X, Y, emulate_bf16=False)[1][0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.140625], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5 and r[4] == 3.140625


def test_features_shape_and_invariants():
    b = W.mixed_convex(256, seed=9)
    X = M.pair_features(b)
    assert X.shape == (256, 48)
    assert np.all(X[:, 39:] == 0)
    assert np.allclose(np.linalg.norm(X[:, 3:7], axis=1), 1.0, atol=1e-5)
    assert np.all(X[:, 6] >= 0)
    onehot = X[:, 7:13]
    assert np.all(onehot.sum(1) == 1)
