"""CPU checks of the FP64 surrogate oracle (oracle/mlp_oracle.py): its analytic loss gradient
against central finite differences, its force against -dU/dr by finite differences, and the
bfloat16 rounding rule."""

import numpy as np

from oracle import mlp_oracle as M


def setup(n_pairs=6, B=40, seed=3):
    rng = np.random.default_rng(seed)
    theta = M.init_params(n_pairs, seed).astype(np.float64)
    theta[3072:3136] = rng.normal(0, 0.3, 64)
    theta[7232:7296] = rng.normal(0, 0.3, 64)
    p = rng.integers(0, n_pairs, B)
    r = rng.uniform(0.8, 3.0, B)
    return theta, p, r, rng.normal(0, 1, B), rng.normal(0, 3, B)


def test_loss_gradient_matches_finite_differences():
    theta, p, r, Ut, Ft = setup()
    L, g = M.loss_and_grad(theta, p, r, Ut, Ft, 0.3, 0.8, 3.0, 6)
    rng = np.random.default_rng(1)
    idx = np.concatenate([rng.choice(7424, 60, replace=False), 7424 + rng.choice(96, 20, replace=False),
                          [7360]])
    eps = 1e-6
    for k in idx:
        t1, t2 = theta.copy(), theta.copy()
        t1[k] += eps
        t2[k] -= eps
        fd = (M.loss_and_grad(t1, p, r, Ut, Ft, 0.3, 0.8, 3.0, 6)[0]
              - M.loss_and_grad(t2, p, r, Ut, Ft, 0.3, 0.8, 3.0, 6)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def test_force_is_minus_energy_derivative():
    theta, p, r, _, _ = setup()
    U, dU, _ = M.forward(theta, p, r, 0.8, 3.0, 6)
    h = 1e-6
    Up, _, _ = M.forward(theta, p, r + h, 0.8, 3.0, 6)
    Um, _, _ = M.forward(theta, p, r - h, 0.8, 3.0, 6)
    assert np.allclose((Up - Um) / (2 * h), dU, rtol=1e-6, atol=1e-6)


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.14159], np.float32)
    y = M.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0  # tie to even
    assert y[2] == 1.0 + 2 ** -7
    assert y[3] == -2.5
    assert abs(y[4] - 3.140625) < 1e-12
    assert np.all(M.bf16x2(x) - x.astype(np.float64) == 0.0)


def test_pair_index_enumerates_upper_triangle():
    n = 5
    seen = sorted(int(M.pair_index(a, b, n)) for a in range(n) for b in range(a, n))
    assert seen == list(range(n * (n + 1) // 2))
    assert M.pair_index(3, 1, n) == M.pair_index(1, 3, n)
