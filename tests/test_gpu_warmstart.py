"""The learned warm start on a small Hamiltonian family (8 orbitals, 4a+4b, 2 layers):
what the trained network gains over the same batched optimiser without it, with the
converged energies decided by the engine."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_network_warm_start_gain_and_same_minima():
    from ansatzevolve_gb300 import HAM_STORED
    from ansatzevolve_gb300 import warmstart as ws
    spec = ws.FamilySpec(8, 4, 2, seed=3)
    x0, E0, _, _, _ = ws.scan_newton(spec, [0.0], np.zeros(spec.P))
    x0 = x0[0]
    s_tr = np.sort(np.random.default_rng(1).uniform(0, 1, 300))
    s_ho = np.sort(np.random.default_rng(2).uniform(0, 1, 24))
    xtr, Etr, gtr, its = ws.scan_bfgs_chain(spec, s_tr, x0, gtol=1e-8)
    assert gtr.max() < 1e-8
    model, hist = ws.train_warmstart(spec.features(s_tr), xtr, hidden=256, epochs=300, batch=64)
    assert hist[-1] < 0.05 * hist[0]
    warm = ws.scan_batched_warm(spec, s_ho, model, x0, gtol=1e-6, n_anchor=2, mode=HAM_STORED)
    # without the network: every instance starts from the s = 0 angles
    e = spec.engine(len(s_ho), [spec.integrals(s) for s in s_ho], HAM_STORED)
    xz, Ez, gz, itz, rz = e.optimise_batch(np.tile(x0, (len(s_ho), 1)), spec.param0, spec.scale, gtol=1e-6)
    e.close()
    assert warm["gnorm"].max() < 1e-6 and gz.max() < 1e-6
    # the plain scan (reference Newton from the previous instance) finds the same minima
    xp, Ep, tp, nh, ne = ws.scan_newton(spec, s_ho, x0, gtol=1e-6)
    np.testing.assert_allclose(warm["E"], Ep, atol=1e-8, rtol=0)
    np.testing.assert_allclose(Ez, Ep, atol=1e-8, rtol=0)
    # the network's gain: fewer lockstep rounds and iterations than the same optimiser
    # started without it
    assert warm["used"].sum() >= len(s_ho) // 2
    assert np.median(warm["iters"]) < np.median(itz)
    assert warm["rounds"] < rz
    model.close()
