"""The warm-start MLP on the GPU: gradients against the CPU oracle
(oracle/mlp_oracle.py, float64 replaying the BF16 roundings) and training
that actually fits a smooth target."""
import os
import sys

import numpy as np
import pytest

from fvs2d_gb300.mlp import MLP

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("engine", ["tcgen05", "mma.sync"])
@pytest.mark.parametrize("n,n_in,width,depth,n_out", [(64, 5, 32, 2, 4), (300, 5, 256, 4, 4), (257, 7, 48, 1, 3)])
def test_gradients_match_cpu_oracle(n, n_in, width, depth, n_out, engine):
    rng = np.random.default_rng(11)
    m = MLP(n_in, width, depth, n_out, seed=3)
    m.set_engine(engine)
    x = rng.standard_normal((n, n_in)).astype(np.float32)
    y = rng.standard_normal((n, n_out)).astype(np.float32) * 0.3
    p = m.get_params()
    loss, g = m.loss_grad(x, y)
    ref_loss, ref_g = mlp_oracle.loss_grad(p, x.astype(np.float64), y.astype(np.float64), n_in, width, depth, n_out)
    # The oracle replays the BF16 roundings of the activations; only the FP32
    # accumulation order differs.  Where an activation lies next to a BF16
    # rounding boundary, that order decides its rounding, and one flip moves
    # the activation by 2^-8 relative.  Measured on GB300 over these cases
    # (both engines): loss 9.3e-6, gradient 1.3e-4 overall and 2.5e-4 for
    # the worst layer (width 256, depth 4); without flips (width <= 48)
    # ~1e-7.  Bars: 4-5x the measured worst case.
    assert abs(loss - ref_loss) <= 5e-5 * abs(ref_loss)
    err = np.linalg.norm(g - ref_g) / np.linalg.norm(ref_g)
    assert err < 5e-4, err
    # every layer's gradient, not only the largest
    off = 0
    dims_in = [n_in] + [width] * depth
    dims_out = [width] * depth + [n_out]
    for i, o in zip(dims_in, dims_out):
        k = i * o + o
        e = np.linalg.norm(g[off:off + k] - ref_g[off:off + k]) / max(np.linalg.norm(ref_g[off:off + k]), 1e-30)
        assert e < 1e-3, (i, o, e)
        off += k


def test_params_roundtrip():
    m = MLP(5, 64, 2, 4, seed=1)
    p = m.get_params()
    q = p * 0.5 + 0.01
    m.set_params(q)
    assert np.array_equal(m.get_params(), q.astype(np.float32))


def test_training_fits_smooth_target():
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (65536, 5)).astype(np.float32)
    y = np.stack([np.sin(2 * x[:, 0]) * x[:, 1], x[:, 2] ** 2 - x[:, 3], np.cos(x[:, 4] + x[:, 0]),
                  0.5 * x[:, 1] * x[:, 2]], 1).astype(np.float32)
    m = MLP(5, 256, 4, 4, seed=2)
    base = float(((m.predict(x[:4096]) - y[:4096]) ** 2).mean())
    losses = m.train(x, y, batch=2048, epochs=12, lr=2e-3, seed=1)
    assert np.all(np.isfinite(losses))
    pred = m.predict(x[:4096])
    mse = float(((pred - y[:4096]) ** 2).mean())
    assert mse < 0.02 * base and mse < 2e-3, (base, mse, losses)


def test_engines_agree():
    """tcgen05 and mma.sync multiply the same BF16 operands with FP32
    accumulation; only the accumulation order differs."""
    rng = np.random.default_rng(3)
    x = rng.standard_normal((5000, 5)).astype(np.float32)
    y = rng.standard_normal((5000, 4)).astype(np.float32)
    m = MLP(5, 256, 4, 4, seed=7)
    a = m.predict(x)
    la, ga = m.loss_grad(x[:3000], y[:3000])
    m.set_engine("mma.sync")
    b = m.predict(x)
    lb, gb = m.loss_grad(x[:3000], y[:3000])
    assert np.abs(a - b).max() <= 1e-3 * np.abs(b).max(), np.abs(a - b).max()
    assert abs(la - lb) <= 1e-4 * abs(lb)
    assert np.linalg.norm(ga - gb) <= 1e-2 * np.linalg.norm(gb)
