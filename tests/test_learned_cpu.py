"""CPU checks of the learned-initial-iterate pieces: the network oracle (its
backward formulas against finite differences, its bfloat16 rounding) and the
Gaussian random field sampler (variance and correlation)."""
import numpy as np

import mlp_oracle as mo


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 1.5 * 2.0 ** -8, 1.0 + 3.0 * 2.0 ** -8, -2.5, 0.0], dtype=np.float32)
    want = np.array([1.0, 1.0, 1.0 + 2.0 ** -7, 1.0 + 2.0 ** -6, -2.5, 0.0], dtype=np.float32)
    assert np.array_equal(mo.bf16(x), want)


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    sizes = [5, 7, 6, 3]
    n = sum(a * b + b for a, b in zip(sizes[:-1], sizes[1:]))
    theta = rng.normal(size=n) * 0.5
    X, T = rng.normal(size=(4, 5)), rng.normal(size=(4, 3))
    _, g = mo.loss_and_gradients(theta, sizes, X, T, exact=True)
    fd = np.empty(n)
    h = 1e-6
    for i in range(n):
        e = np.zeros(n)
        e[i] = h
        fd[i] = (mo.loss_and_gradients(theta + e, sizes, X, T, True)[0]
                 - mo.loss_and_gradients(theta - e, sizes, X, T, True)[0]) / (2 * h)
    assert np.max(np.abs(fd - g)) <= 1e-7 * max(1.0, np.max(np.abs(g)))


def test_oracle_adam_first_step_is_signed_lr():
    g = np.array([0.5, -2.0, 1e-3])
    theta, m, v = mo.adam(np.zeros(3), g, np.zeros(3), np.zeros(3), 1, 1e-2)
    assert np.allclose(theta, -1e-2 * np.sign(g), rtol=1e-4)


def test_grf_variance_and_correlation(vfvm):
    from vfvm_gb300.learned import grf_logkappa, kappa_instance
    n, S = 65, 300
    G = np.array([grf_logkappa(n, s) for s in range(S)]).reshape(S, n, n)
    assert abs(G.var(axis=0).mean() - 1.0) < 0.08
    for lag in (3, 6, 13):
        r = lag / (n - 1)
        c = (G[:, :, :-lag] * G[:, :, lag:]).mean()
        assert abs(c - np.exp(-r * r / (2 * 0.1 ** 2))) < 0.05
    # seeded: the same seed gives the same instance
    a, fa = kappa_instance(33, 5)
    b, fb = kappa_instance(33, 5)
    assert np.array_equal(a, b) and fa == fb and -1.0 <= fa <= 1.0
