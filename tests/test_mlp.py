"""The warm-start MLP: forward pass, gradients and Adam steps of the device
kernels against the FP64 restatement (tests/mlp_ref.py), which is itself
checked against finite differences; training reduces the loss."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import mlp_ref  # noqa: E402


def _points(rng, n):
    x = np.stack([rng.choice([16, 24, 32, 48, 64, 72, 96, 128], n) / 128.0, rng.uniform(0.4, 0.8, n),
                  rng.uniform(1.5, 1.99, n), rng.uniform(0, 1, n)], 1).astype(np.float32)
    t = (np.sin(3 * x[:, 3]) * (1 + x[:, 1]) - 0.5 * x[:, 0]).astype(np.float32)
    return x, t


def _init(seed=0):
    rng = np.random.default_rng(seed)
    return mlp_ref.pack([(rng.uniform(-1, 1, (o, i)) / np.sqrt(i), rng.uniform(-1, 1, o) / np.sqrt(i))
                         for o, i in mlp_ref.SIZES])


def test_reference_gradient_vs_finite_differences():
    rng = np.random.default_rng(1)
    p = _init(1)
    x, t = _points(rng, 40)
    _, g = mlp_ref.loss_and_grad(p, x, t)
    for k in rng.choice(p.size, 60, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (mlp_ref.loss_and_grad(pp, x, t)[0] - mlp_ref.loss_and_grad(pm, x, t)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(g[k]), k


def test_param_count_and_features():
    from muca_gb300 import build as b
    b.build()
    import muca_gb300 as m
    assert int(m.lib().muca_mlp_param_count()) == 33793 == mlp_ref.pack(mlp_ref.unpack(np.zeros(33793))).size
    lnw = np.cumsum(np.linspace(-1, 1, 65))
    x, t = m.mlp_features(8, 0.5, 1.96, lnw)
    assert x.shape == (65, 4) and np.allclose(x[:, 3], np.arange(65) / 64)
    np.testing.assert_allclose(t, (lnw - lnw.mean()) / 64, rtol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1000, 999, 33, 4096])
def test_forward_and_gradient_vs_reference(muca, n):
    rng = np.random.default_rng(2)
    p = _init(2).astype(np.float32)
    x, t = _points(rng, n)  # 1000, 999, 33: not multiples of the 32-point tile; odd sizes shift the scratch
    with muca.MLP(seed=5) as net:
        net.set_params(p)
        y = net.predict(x)
        loss, g = net.grad(x, t)
    yr, _, _ = mlp_ref.forward(p.astype(np.float64), x)
    np.testing.assert_allclose(y, yr, rtol=2e-5, atol=2e-6)
    lr, gr = mlp_ref.loss_and_grad(p.astype(np.float64), x, t)
    assert abs(loss - lr) <= 1e-5 * lr
    off = 0
    for o, i in mlp_ref.SIZES:  # per layer: FP32 sums against FP64
        n = o * i + o
        scale = np.abs(gr[off:off + n]).max()
        np.testing.assert_allclose(g[off:off + n], gr[off:off + n], rtol=0, atol=2e-5 * scale)
        off += n


@pytest.mark.gpu
def test_adam_steps_vs_reference(muca, orc):
    rng = np.random.default_rng(3)
    p = _init(3)
    x, t = _points(rng, 500)
    B, steps, lr, seed = 64, 4, 1e-3, 11
    with muca.MLP() as net:
        net.set_params(p.astype(np.float32))
        net.set_data(x, t)
        losses = net.train(steps, batch=B, lr=lr, seed=seed)
        pd = net.params()
    q = p.astype(np.float32).astype(np.float64)
    mm = np.zeros_like(q)
    vv = np.zeros_like(q)
    for s in range(steps):
        idx = mlp_ref.minibatch(orc, x.shape[0], B, s, seed)
        loss, g = mlp_ref.loss_and_grad(q, x[idx], t[idx])
        assert abs(losses[s] - loss) <= 1e-4 * loss + 1e-7, s
        q, mm, vv = mlp_ref.adam_step(q, g, mm, vv, s + 1, lr)
    # early Adam steps move every parameter by about lr; FP32 rounding of
    # tiny gradients can flip a step's sign, so compare in units of lr
    diff = np.abs(pd - q) / lr
    assert np.mean(diff > 1e-2) < 1e-3 and diff.max() < 2 * steps


@pytest.mark.gpu
def test_training_reduces_loss(muca):
    rng = np.random.default_rng(4)
    x, t = _points(rng, 20000)
    with muca.MLP(seed=1) as net:
        net.set_data(x, t)
        losses = net.train(1500, batch=1024, lr=1e-3, seed=2)
        y = net.predict(x)
    assert np.all(np.isfinite(losses))
    assert losses[-50:].mean() < 0.02 * losses[:10].mean()
    assert np.mean((y - t) ** 2) < 0.02 * np.var(t)
