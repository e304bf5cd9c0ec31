"""The warm-start network's CPU oracle and host logic (no GPU).

The oracle (oracle/mlp_oracle.py) is what the GPU forward, gradient and Adam kernels are checked
against; here it is pinned itself: its gradient against central finite differences in FP64, its
BF16 rounding against the bit-level rounding of the synthetic-input module, its Adam step against
the closed form of the first step, and a training run that lowers the loss. The feature layout
and the seeded run sampler of epspectral_gb300.warmstart are checked as host logic.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as MO


def _net(dims, seed):
    rng = np.random.default_rng(seed)
    return np.concatenate([np.concatenate([rng.normal(0, 1 / np.sqrt(a), a * b), rng.normal(0, 0.1, b)])
                           for a, b in zip(dims[:-1], dims[1:])])


def test_nparams_and_unflatten():
    dims = [5, 4, 3]
    p = np.arange(MO.nparams(dims), dtype=float)
    (W0, b0), (W1, b1) = MO.unflatten(p, dims)
    assert W0.shape == (4, 5) and b0.shape == (4,) and W1.shape == (3, 4) and b1.shape == (3,)
    assert W0[1, 0] == 5 and b0[0] == 20 and W1[0, 0] == 24
    with pytest.raises(ValueError):
        MO.unflatten(p[:-1], dims)


def test_gradient_matches_finite_differences():
    dims = [6, 8, 7, 3]
    p = _net(dims, 1)
    rng = np.random.default_rng(2)
    X, Y = rng.normal(size=(9, 6)), rng.normal(size=(9, 3))
    loss, g = MO.loss_and_grad(p, dims, X, Y, round_bf16=False)
    h = 1e-6
    fd = np.empty_like(p)
    for k in range(len(p)):
        e = np.zeros_like(p)
        e[k] = h
        fd[k] = (MO.loss_and_grad(p + e, dims, X, Y, round_bf16=False)[0]
                 - MO.loss_and_grad(p - e, dims, X, Y, round_bf16=False)[0]) / (2 * h)
    assert np.max(np.abs(fd - g)) <= 1e-8 * max(1.0, np.max(np.abs(g)))
    assert loss == pytest.approx(np.mean((MO.predict(p, dims, X, round_bf16=False) - Y) ** 2), rel=1e-14)


def test_bf16_rounding_matches_bit_rounding():
    from epspectral_gb300 import synthetic
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.normal(size=1000).astype(np.float32),
                        np.array([1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -1.5, 0.0], dtype=np.float32)])
    ref = synthetic.bf16_bits_to_float32(synthetic.float32_to_bf16_bits(x)).astype(np.float64)
    assert np.array_equal(MO.bf16_round(x), ref)
    # ties go to even: 1 + 2^-8 -> 1, 1 + 3 * 2^-8 -> 1 + 2^-6
    assert MO.bf16_round(np.float32([1.0 + 2.0 ** -8]))[0] == 1.0
    assert MO.bf16_round(np.float32([1.0 + 3 * 2.0 ** -8]))[0] == 1.0 + 2.0 ** -6


def test_adam_first_step_is_signed_learning_rate():
    g = np.array([0.3, -2.0, 1e-3])
    p, m, v = MO.adam_step(np.zeros(3), g, np.zeros(3), np.zeros(3), 1, 0.01)
    assert np.allclose(p, -0.01 * np.sign(g) * np.abs(g) / (np.abs(g) + 1e-8), rtol=0, atol=1e-15)


def test_training_lowers_the_loss():
    dims = [4, 16, 16, 2]
    rng = np.random.default_rng(4)
    X = rng.normal(size=(128, 4))
    Y = np.stack([np.sin(X[:, 0]) + X[:, 1] * X[:, 2], np.cos(X[:, 3])], axis=1)
    p0 = _net(dims, 5)
    l0 = MO.loss_and_grad(p0, dims, X, Y)[0]
    p, hist = MO.train(p0, dims, X, Y, epochs=60, batch=32, lr=3e-3)
    assert hist[-1] < 0.5 * hist[0] and MO.loss_and_grad(p, dims, X, Y)[0] < 0.3 * l0


def test_feature_layout_and_targets():
    from epspectral_gb300 import warmstart as W
    nw, ni = 7, 3
    rng = np.random.default_rng(6)
    S0 = rng.normal(size=(nw, ni)) + 1j * rng.normal(size=(nw, ni))
    S = S0 + 0.1 * (rng.normal(size=(nw, ni)) + 1j * rng.normal(size=(nw, ni)))
    eps = np.array([-0.2, 0.0, 0.3])
    X = W.features(S0, 0.025, 0.1, 1.5, eps)
    assert X.shape == (ni, 2 * nw + W.N_SCALARS)
    assert np.array_equal(X[1, :nw], S0[:, 1].real) and np.array_equal(X[2, nw:2 * nw], S0[:, 2].imag)
    assert np.allclose(X[:, 2 * nw:], [[0.025, 0.1, 1.5, e - 0.1] for e in eps])
    Y = W.targets(S0, S)
    D = (Y[:, :nw] + 1j * Y[:, nw:]).T
    assert np.allclose(S0 + D, S, rtol=0, atol=1e-15)


def test_sample_runs_is_seeded_and_in_range():
    from epspectral_gb300 import warmstart as W
    a = W.sample_runs(20, 7)
    assert a == W.sample_runs(20, 7) and a != W.sample_runs(20, 8)
    assert all(100 <= r["T_K"] <= 800 and 0.5 <= r["filling"] <= 1.5 and 0.5 <= r["scale"] <= 2.0 for r in a)
    assert len({r["scale"] for r in a[:8]}) == 1 and a[8]["scale"] != a[0]["scale"]
