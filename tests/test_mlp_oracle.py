"""The numpy restatement of the warm-start MLP (the reference for its CUDA kernels):
gradients against finite differences, bf16 rounding against known values."""
import numpy as np

from oracle import mlp_ref


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3, 65504.0], dtype=np.float32)
    r = mlp_ref.bf16_round(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: ties go to the even mantissa (1.0)
    assert r[0] == 1.0 and r[1] == 1.0
    assert r[2] == np.float32(1.0078125)
    assert r[3] == -2.5
    assert abs(r[4] - 3.0e-3) < 3.0e-3 * 2 ** -8
    assert (r.view(np.uint32) & 0xFFFF).max() == 0


def test_gradient_matches_central_differences():
    dims = (6, 8, 3)
    rng = np.random.default_rng(1)
    X = rng.normal(size=(5, 6))
    T = rng.normal(size=(5, 3))
    sc = (rng.normal(size=6), rng.uniform(0.5, 2, 6), rng.normal(size=3), rng.uniform(0.5, 2, 3))
    p = mlp_ref.init_params(*dims, seed=2).astype(np.float64)
    loss, g = mlp_ref.loss_grad(p, X, T, dims, sc, quantise=False)
    assert loss > 0
    h = 1e-5
    for i in range(0, p.size, 7):
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp_ref.loss_grad(pp, X, T, dims, sc, quantise=False)[0] -
              mlp_ref.loss_grad(pm, X, T, dims, sc, quantise=False)[0]) / (2 * h)
        assert abs(fd - g[i]) < 1e-7 + 1e-6 * abs(fd), (i, fd, g[i])


def test_quantised_model_on_bf16_weights_is_the_plain_model():
    dims = (6, 8, 3)
    p = mlp_ref.bf16_round(mlp_ref.init_params(*dims, seed=3))
    X = np.random.default_rng(4).normal(size=(4, 6))
    np.testing.assert_array_equal(mlp_ref.forward(p, X, dims)["y"], mlp_ref.forward(p, X, dims, quantise=False)["y"])
