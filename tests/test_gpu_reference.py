"""The engine against the reference's own outputs on the benchmark's 10-, 12- and
14-orbital inputs (tests/golden/ref10.npz, ref12.npz, ref14.npz, produced by the
reference build through its stateAnsatzManager API): energy at 1e-10, gradient and
Hessian entries at 1e-9, sampled final-state amplitudes at 1e-12.  At 14 orbitals
(7a+7b, 4 layers, 11,778,624 determinants) the reference applies its operator list on
the fly, and so does the engine."""
import numpy as np
import pytest

import ansatzevolve_gb300 as ae
from ansatzevolve_gb300.synthetic import synthetic_integrals

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,mode", [("ref10", ae.HAM_STORED), ("ref10", ae.HAM_ON_THE_FLY),
                                       ("ref12", ae.HAM_STORED), ("ref12", ae.HAM_ON_THE_FLY),
                                       ("ref14", ae.HAM_ON_THE_FLY)])
def test_engine_matches_reference_outputs(golden, name, mode):
    fx = golden(name)
    N, na, nb = int(fx["N"]), int(fx["na"]), int(fx["nb"])
    ops0 = np.asarray(fx["ops_1b"]) - 1
    p0 = np.asarray(fx["order_1b"]) - 1
    scale = np.asarray(fx["scale"])
    P = int(p0.max()) + 1
    e = ae.Engine(2 * N, ae.BASIS_SZ, na + nb, na, nb, ops0)
    init = np.zeros(e.D)
    init[np.searchsorted(e.states(), int(fx["hf"]))] = 1.0
    e.set_initial(init)
    h1, g2 = synthetic_integrals(N, int(fx["seed"]))
    e.set_ham_integrals(h1, g2, mode)
    ang = scale * np.asarray(fx["x"])[p0]
    E, gops = e.gradient(ang)
    g = np.zeros(P)
    np.add.at(g, p0, scale * gops)
    assert abs(E - float(fx["E"])) < 1e-10
    np.testing.assert_allclose(g, fx["G"], atol=1e-9, rtol=0)
    psi = e.evolve(ang)
    states = e.states()
    assert np.array_equal(states[fx["sample_rank"]], fx["sample_bits"])
    np.testing.assert_allclose(psi[fx["sample_rank"]], fx["sample_amp"], atol=1e-12, rtol=0)
    assert abs(np.dot(psi, psi) - float(fx["norm"])) < 1e-12
    if "H" in fx and mode == ae.HAM_STORED:
        Eh, gh, H = e.hessian(ang, p0, scale)
        np.testing.assert_allclose(H, fx["H"], atol=1e-9, rtol=0)
        np.testing.assert_allclose(gh, fx["G"], atol=1e-9, rtol=0)
    e.close()
