"""Test infrastructure only: a numpy restatement of the warm-start MLP (the aegpu_mlp_*
kernels) used to check their forward pass and gradients.  Nothing in the
product imports it.

Model: x' = (x - in_mean) / in_scale; z1 = x' W1^T + b1, a1 = gelu(z1);
z2 = a1 W2^T + b2, a2 = gelu(z2); y' = a2 W3^T + b3; y = y' * out_scale + out_mean.
The weight matrices are used after rounding to bfloat16 (round to nearest even), as
the kernels do; everything else is float64 here.  Loss: mean over rows and outputs
of (y' - (t - out_mean) / out_scale)^2.  Parameter layout: W1[H][n_in], b1[H],
W2[H][H], b2[H], W3[n_out][H], b3[n_out].  GELU is the exact erf form.
"""
import math

import numpy as np

_erf = np.vectorize(math.erf)


def bf16_round(x):
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(params, n_in, H, n_out):
    p = np.asarray(params, dtype=np.float32)
    sizes = [H * n_in, H, H * H, H, n_out * H, n_out]
    out, o = [], 0
    for s in sizes:
        out.append(p[o:o + s])
        o += s
    W1, b1, W2, b2, W3, b3 = out
    return W1.reshape(H, n_in), b1, W2.reshape(H, H), b2, W3.reshape(n_out, H), b3


def unpack64(params, n_in, H, n_out):
    p = np.asarray(params, dtype=np.float64)
    sizes = [H * n_in, H, H * H, H, n_out * H, n_out]
    out, o = [], 0
    for s in sizes:
        out.append(p[o:o + s])
        o += s
    W1, b1, W2, b2, W3, b3 = out
    return W1.reshape(H, n_in), b1, W2.reshape(H, H), b2, W3.reshape(n_out, H), b3


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward(params, X, dims, scaling=None, quantise=True):
    """quantise=False skips the bf16 rounding (pure float64 model, for derivative checks)."""
    n_in, H, n_out = dims
    if quantise:
        W1, b1, W2, b2, W3, b3 = unpack(params, n_in, H, n_out)
        W1, W2, W3 = (bf16_round(w).astype(np.float64) for w in (W1, W2, W3))
    else:
        W1, b1, W2, b2, W3, b3 = unpack64(params, n_in, H, n_out)
    X = np.asarray(X, dtype=np.float64)
    if scaling is not None:
        X = (X - scaling[0]) / scaling[1]
    z1 = X @ W1.T + b1
    a1 = gelu(z1)
    z2 = a1 @ W2.T + b2
    a2 = gelu(z2)
    y = a2 @ W3.T + b3
    return dict(x=X, z1=z1, a1=a1, z2=z2, a2=a2, y=y, W1=W1, W2=W2, W3=W3)


def predict(params, X, dims, scaling=None):
    y = forward(params, X, dims, scaling)["y"]
    if scaling is not None:
        y = y * scaling[3] + scaling[2]
    return y


def loss_grad(params, X, T, dims, scaling=None, quantise=True):
    """Loss and gradients with respect to the parameters; with quantise=True the
    weight gradients are those of the rounded weights (what the kernels compute)."""
    n_in, H, n_out = dims
    f = forward(params, X, dims, scaling, quantise)
    T = np.asarray(T, dtype=np.float64)
    if scaling is not None:
        T = (T - scaling[2]) / scaling[3]
    n = T.shape[0]
    d = f["y"] - T
    loss = float(np.mean(d * d))
    dy = 2.0 * d / (n * n_out)
    gW3 = dy.T @ f["a2"]
    gb3 = dy.sum(axis=0)
    dz2 = (dy @ f["W3"]) * gelu_grad(f["z2"])
    gW2 = dz2.T @ f["a1"]
    gb2 = dz2.sum(axis=0)
    dz1 = (dz2 @ f["W2"]) * gelu_grad(f["z1"])
    gW1 = dz1.T @ f["x"]
    gb1 = dz1.sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def init_params(n_in, H, n_out, seed):
    """Any reasonable parameter vector for the checks (not the kernels' initialiser)."""
    rng = np.random.default_rng(seed)
    parts = [rng.uniform(-1, 1, H * n_in) / math.sqrt(n_in), rng.uniform(-1, 1, H) / math.sqrt(n_in),
             rng.uniform(-1, 1, H * H) / math.sqrt(H), rng.uniform(-1, 1, H) / math.sqrt(H),
             rng.uniform(-1, 1, n_out * H) / math.sqrt(H), rng.uniform(-1, 1, n_out) / math.sqrt(H)]
    return np.concatenate(parts).astype(np.float32)
