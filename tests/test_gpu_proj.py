"""Projected sweep (evolveDerivativeProj) on the GPU against the oracle."""
import numpy as np
import pytest

import ansatzevolve_gb300 as ae
from tests.fixtures import oracle_synthetic, synthetic_problem

pytestmark = pytest.mark.gpu


def test_projected_gradient_batch_vs_oracle():
    pb = synthetic_problem(8, 4, 4, 2, 0)
    o = oracle_synthetic(pb, csr=False)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    nb = 3
    e = ae.Engine(16, ae.BASIS_SZ, 8, 4, 4, ops0)
    init = np.zeros(e.D)
    init[np.searchsorted(e.states(), pb["hf"])] = 1.0
    e.set_initial(init)
    e.set_batch(nb)
    rng = np.random.default_rng(4)
    ang = rng.uniform(-0.3, 0.3, (nb, len(ops0)))
    proj = rng.normal(size=(nb, e.D))
    ov, g = e.gradient_proj(ang, proj)
    for b in range(nb):
        ovo, go = o.gradient_proj_ops(ang[b], proj[b])
        assert abs(ov[b] - ovo) < 1e-12
        np.testing.assert_allclose(g[b], go, atol=1e-12, rtol=0)
    # the energy gradient still works after a projected sweep (H psi recomputed)
    e.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    E, gE = e.gradient(ang)
    Eo, gEo = o.energy_gradient_ops(ang[1])
    assert abs(E[1] - Eo) < 1e-10
    np.testing.assert_allclose(gE[1], gEo, atol=1e-9, rtol=0)
    e.close()


def test_projected_hessian_vs_oracle_differences():
    """evolveHessianProj: gradient and overlap against the oracle's projected sweep,
    the Hessian against central differences of it (compressed parameters)."""
    pb = synthetic_problem(8, 4, 4, 2, 1)
    o = oracle_synthetic(pb, csr=False)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    p0 = np.asarray(pb["order_1b"]) - 1
    scale = np.asarray(pb["scale"])
    P = int(p0.max()) + 1
    e = ae.Engine(16, ae.BASIS_SZ, 8, 4, 4, ops0)
    init = np.zeros(e.D)
    init[np.searchsorted(e.states(), pb["hf"])] = 1.0
    e.set_initial(init)
    rng = np.random.default_rng(6)
    x = rng.uniform(-0.3, 0.3, P)
    proj = rng.normal(size=e.D)

    def comp_grad(xx):
        ov, go = o.gradient_proj_ops(scale * xx[p0], proj)
        g = np.zeros(P)
        np.add.at(g, p0, scale * go)
        return ov, g

    ov, g, H = e.hessian_proj(scale * x[p0], p0, scale, proj)
    ovo, go = comp_grad(x)
    assert abs(ov - ovo) < 1e-12
    np.testing.assert_allclose(g, go, atol=1e-12, rtol=0)
    np.testing.assert_allclose(H, H.T, atol=1e-12, rtol=0)
    h = 1e-5
    for mu in range(P):
        d = np.zeros(P)
        d[mu] = h
        fd = (comp_grad(x + d)[1] - comp_grad(x - d)[1]) / (2 * h)
        np.testing.assert_allclose(H[mu], fd, atol=1e-8, rtol=0)
    e.close()
