"""Host side of the Hamiltonian-family scans: the batched integrals and network features
agree bit for bit with the one-instance-at-a-time forms the plain path uses."""
import numpy as np
import pytest

from ansatzevolve_gb300 import warmstart as ws


@pytest.mark.parametrize("n_orb,pert", [(6, 1.0), (10, 0.25)])
def test_family_batches_bit_identical(n_orb, pert):
    spec = ws.FamilySpec(n_orb, n_orb // 2, 2, seed=3, pert=pert)
    s = np.random.default_rng(11).uniform(0, 1, 17)
    h, g = spec.integrals_batch(s)
    F = spec.features(s)
    assert h.shape == (17, n_orb, n_orb) and g.shape == (17,) + (n_orb,) * 4
    for i, x in enumerate(s):
        a, b = spec.integrals(x)
        assert np.array_equal(a, h[i]) and np.array_equal(b, g[i])
        assert np.array_equal(ws.features(a, b), F[i])
    # an empty batch is empty
    h0, g0 = spec.integrals_batch(np.zeros(0))
    assert h0.shape == (0, n_orb, n_orb) and g0.shape == (0,) + (n_orb,) * 4
