"""The warm-start MLP's CUDA kernels (forward, backward, Adam) against the numpy
restatement in oracle/mlp_ref.py."""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def model(dims, seed=0):
    from ansatzevolve_gb300.warmstart import Mlp
    return Mlp(dims[0], dims[2], hidden=dims[1], seed=seed)


@pytest.mark.parametrize("dims,n", [((200, 512, 81), 37), ((20, 96, 7), 130)])
def test_loss_gradient_and_prediction_match_oracle(dims, n):
    rng = np.random.default_rng(5)
    X = rng.normal(size=(n, dims[0])).astype(np.float32)
    T = rng.normal(size=(n, dims[2])).astype(np.float32)
    sc = (rng.normal(size=dims[0]), rng.uniform(0.5, 2, dims[0]), rng.normal(size=dims[2]),
          rng.uniform(0.5, 2, dims[2]))
    sc = tuple(np.asarray(a, dtype=np.float32) for a in sc)
    m = model(dims)
    p = mlp_ref.init_params(*dims, seed=6)
    m.set_params(p)
    m.set_scaling(*sc)
    assert np.array_equal(m.get_params(), p)
    sc64 = tuple(a.astype(np.float64) for a in sc)
    loss, g = m.loss_grad(X, T)
    lo, go = mlp_ref.loss_grad(p, X, T, dims, sc64)
    assert abs(loss - lo) < 1e-5 * lo
    # FP32 accumulation against float64: relative to each tensor's largest entry
    n_in, H, n_out = dims
    offs = np.cumsum([0, H * n_in, H, H * H, H, n_out * H, n_out])
    for t in range(6):
        a, b = g[offs[t]:offs[t + 1]], go[offs[t]:offs[t + 1]]
        assert np.max(np.abs(a - b)) <= 1e-4 * np.max(np.abs(b)) + 1e-9, t
    y = m.predict(X)
    yo = mlp_ref.predict(p, X, dims, sc64)
    assert np.max(np.abs(y - yo)) <= 1e-4 * np.max(np.abs(yo))
    m.close()


def test_training_fits_a_smooth_map():
    dims = (16, 128, 5)
    rng = np.random.default_rng(8)
    A = rng.normal(size=(16, 5)) / 4
    X = rng.normal(size=(512, 16)).astype(np.float32)
    T = np.sin(X @ A).astype(np.float32)
    m = model(dims, seed=3)
    m.fit_scaling(X, T)
    l0, _ = m.loss_grad(X, T)
    hist = m.train(X, T, epochs=150, batch=64, lr=1e-3, seed=1)
    assert hist.shape == (150,)
    l1, _ = m.loss_grad(X, T)
    assert l1 < 0.05 * l0, (l0, l1, hist[::30])
    # the same seeds give the same trained weights
    m2 = model(dims, seed=3)
    m2.fit_scaling(X, T)
    m2.train(X, T, epochs=150, batch=64, lr=1e-3, seed=1)
    assert np.array_equal(m.get_params(), m2.get_params())
    m.close()
    m2.close()
