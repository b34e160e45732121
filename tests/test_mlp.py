"""The surrogate network's training kernels against the CPU oracle.

CPU: the oracle's FP64 backward pass agrees with central finite differences
(pins the oracle), and its bf16 rounding helper is round-to-nearest-even.
GPU: the tensor-core gradients equal the oracle's (same bf16 rounding
points) within 1e-2 relative L2 per parameter block and the loss within
1e-3; the captured training step applies Adam as the oracle's gradients
give it; training lowers the loss; prediction is batch-size independent.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as MO


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1.0 + 2 ** -9], np.float32)
    r = MO.bf16(x)
    assert list(r) == [1.0, 1.0, 1.0 + 4 * 2 ** -8, -2.5, 1.0]


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = MO.init_like_device(5)
    X = rng.standard_normal((12, MO.IN))
    t = rng.standard_normal(12)
    loss, g = MO.loss_and_grad(p, X, t, emulate_bf16=False)
    picks = []
    for key in ("W0", "b0", "W1", "b1", "W2", "W3", "b3", "w5", "b5"):
        o, s = MO.OFFSETS[key]
        size = int(np.prod(s))
        for _ in range(3):
            j = int(rng.integers(size))
            if key == "W0":
                j = int(rng.integers(s[0])) * s[1] + int(rng.integers(MO.IN))
            picks.append(o + j)
    h = 1e-6
    for i in picks:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (MO.loss_and_grad(pp, X, t, False)[0] - MO.loss_and_grad(pm, X, t, False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def _blocks():
    return [(k, o, int(np.prod(s))) for k, (o, s) in MO.OFFSETS.items()]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [128, 300, 1024])
def test_tensor_core_gradients_match_oracle(n):
    import pticm
    m = pticm.MLP(seed=7, batch=1024)
    assert m.n_params == MO.PARAM_COUNT
    rng = np.random.default_rng(n)
    p = MO.init_like_device(11).astype(np.float32)
    m.params = p
    X = rng.standard_normal((n, MO.IN)).astype(np.float32)
    t = rng.standard_normal(n).astype(np.float32)
    loss, g = m.gradients(X, t)
    ol, og = MO.loss_and_grad(p.astype(np.float64), X, t, emulate_bf16=True)
    assert abs(loss - ol) <= 1e-3 * abs(ol)
    for key, o, size in _blocks():
        a, b = g[o:o + size].astype(np.float64), og[o:o + size]
        if key == "W0":   # the padding columns get gradient but stay unused
            a = a.reshape(MO.H, MO.K0)[:, :MO.IN]
            b = b.reshape(MO.H, MO.K0)[:, :MO.IN]
        err = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30)
        assert err < 1e-2, (key, err)


@pytest.mark.gpu
def test_captured_adam_steps_match_oracle_adam():
    """Three one-step training calls on a dataset smaller than the batch (each
    step sees every row): the captured step's update equals Adam applied to
    the oracle's gradients at the device's parameters, with the bias
    corrections of steps 1, 2, 3 (the step counter outlives a call)."""
    import pticm
    rng = np.random.default_rng(4)
    n, lr = 300, 1e-3
    X = rng.standard_normal((n, MO.IN)).astype(np.float32)
    t = rng.standard_normal(n).astype(np.float32)
    m = pticm.MLP(seed=2, batch=1024)
    m.params = MO.init_like_device(13).astype(np.float32)
    mom = np.zeros(MO.PARAM_COUNT)
    vel = np.zeros(MO.PARAM_COUNT)
    for k in range(1, 4):
        p0 = m.params.astype(np.float64)
        ol, g = MO.loss_and_grad(p0, X, t, emulate_bf16=True)
        losses = m.train(X, t, steps=1, lr=lr, seed=k)
        assert abs(losses[0] - ol) <= 1e-3 * abs(ol)
        mom = 0.9 * mom + 0.1 * g
        vel = 0.999 * vel + 0.001 * g * g
        want = -lr * (mom / (1 - 0.9 ** k)) / (np.sqrt(vel / (1 - 0.999 ** k)) + 1e-8)
        got = m.params.astype(np.float64) - p0
        err = np.abs(got - want) / lr
        # gradients agree to ~1e-2; entries with near-zero gradient may differ
        assert np.median(err) < 0.02, (k, np.median(err))
        assert np.mean(err < 0.25) > 0.97, (k, np.mean(err < 0.25))


@pytest.mark.gpu
def test_training_lowers_loss_and_prediction_is_batch_independent():
    import pticm
    rng = np.random.default_rng(1)
    n = 4096
    X = rng.uniform(-1, 1, (n, MO.IN)).astype(np.float32)
    y = (np.sin(2 * X[:, 0]) * X[:, 1] + 0.5 * X[:, 6] ** 2).astype(np.float32)
    m = pticm.MLP(seed=3, batch=512)
    losses = m.train(X, y, steps=600, lr=1e-3, seed=5)
    assert losses[-50:].mean() < 0.05 * losses[:5].mean(), (losses[:5], losses[-50:].mean())
    pred = m.predict(X)
    assert np.sqrt(np.mean((pred - y) ** 2)) < 0.1
    m2 = pticm.MLP(seed=9, batch=128)
    m2.params = m.params
    assert np.array_equal(m2.predict(X[:700]), pred[:700])
    # the device forward equals the oracle's bf16 forward
    yo, _ = MO.forward(m.params.astype(np.float64), X[:256], emulate_bf16=True)
    assert np.max(np.abs(yo - pred[:256])) < 2e-2 * (np.abs(yo).max() + 1)
