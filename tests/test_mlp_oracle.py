"""The warm-start network's CPU oracle: BF16 rounding and analytic gradients
(checked against central finite differences), before it judges the GPU."""
import numpy as np

from oracle import mlp as M


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.14159, 0.0, 65504.0], dtype=np.float32)
    r = M.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa -> 1
    assert r[0] == 1.0 and r[1] == 1.0
    # 1 + 1.5 * 2^-8 rounds up to 1 + 2^-7
    assert r[2] == np.float32(1.0078125) and r[3] == np.float32(1.0078125)
    assert r[4] == np.float32(-3.140625) and r[5] == 0.0
    assert r[6] == np.float32(65536.0)
    # idempotent and within half an ulp of 8 bits
    assert np.array_equal(M.bf16(r), r)
    z = np.random.default_rng(0).normal(size=10000).astype(np.float32)
    assert np.max(np.abs(M.bf16(z) - z) / np.abs(z)) <= 2.0 ** -8


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(1)
    B = 16
    X = rng.normal(size=(B, M.N_IN)).astype(np.float32)
    y = rng.normal(size=B).astype(np.float32)
    theta = M.he_init(3).astype(np.float64)
    _, _, g = M.forward_backward(X, y, theta, round_weights=False)
    idx = np.concatenate([rng.choice(np.arange(M.OFF_W1, M.OFF_B1), 12, replace=False),
                          rng.choice(np.arange(M.OFF_B1, M.OFF_W2), 6, replace=False),
                          rng.choice(np.arange(M.OFF_W2, M.OFF_B2), 12, replace=False),
                          rng.choice(np.arange(M.OFF_B2, M.OFF_W3), 6, replace=False),
                          rng.choice(np.arange(M.OFF_W3, M.OFF_B3), 6, replace=False), [M.OFF_B3]])
    h = 1e-6
    for i in idx:
        tp = theta.copy()
        tm = theta.copy()
        tp[i] += h
        tm[i] -= h
        # float64 parameters: forward in float64 without rounding
        lp = _loss64(X, y, tp)
        lm = _loss64(X, y, tm)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, fd, g[i])


def _loss64(X, y, theta):
    W1 = theta[M.OFF_W1:M.OFF_B1].reshape(M.N_IN, M.N_H)
    b1 = theta[M.OFF_B1:M.OFF_W2]
    W2 = theta[M.OFF_W2:M.OFF_B2].reshape(M.N_H, M.N_H)
    b2 = theta[M.OFF_B2:M.OFF_W3]
    w3 = theta[M.OFF_W3:M.OFF_B3]
    b3 = theta[M.OFF_B3]
    A1 = np.maximum(X.astype(np.float64) @ W1 + b1, 0)
    A2 = np.maximum(A1 @ W2 + b2, 0)
    e = A2 @ w3 + b3 - y
    return float(np.mean(e * e))
