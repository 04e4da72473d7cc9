"""LUCJ ansatz (exp(-K) exp(iJ) exp(K) in the reference's Givens + phase operator
forms) on the engine in complex mode."""
import numpy as np
import pytest

import ansatzevolve_gb300 as ae
from ansatzevolve_gb300.lucj import lucj_operators, random_lucj
from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals
from tests.test_lucj_host import dense_lucj_state, sector_states

pytestmark = pytest.mark.gpu


def lucj_engine(N, na, K, J, mode=ae.HAM_STORED):
    ops, ang = lucj_operators(K, J)
    e = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops, complex_mode=True)
    init = np.zeros(2 * e.D)
    init[2 * np.searchsorted(e.states(), hartree_fock_index(N, na, na))] = 1.0
    e.set_initial(init)
    h1, g2 = synthetic_integrals(N, 7)
    e.set_ham_integrals(h1, g2, mode)
    return e, ops, ang, h1, g2


def test_lucj_state_matches_dense_exponentials_6_orbitals():
    N, na = 6, 3
    K, J = random_lucj(N, 5)
    e, ops, ang, h1, g2 = lucj_engine(N, na, K, J)
    want, _ = dense_lucj_state(N, na, K, J, sector_states(N, na, na))
    got = e.evolve(ang)
    got = got[0::2] + 1j * got[1::2]
    assert np.max(np.abs(got - want)) < 1e-12
    e.close()


@pytest.mark.parametrize("mode", [ae.HAM_STORED, ae.HAM_ON_THE_FLY])
def test_lucj_energy_gradient_vs_oracle_8_orbitals(mode):
    from oracle.oracle import Oracle
    N, na = 8, 4
    K, J = random_lucj(N, 2)
    e, ops, ang, h1, g2 = lucj_engine(N, na, K, J, mode)
    o = Oracle(2 * N, 2, 2 * na, na, na, cplx=True)
    o.set_initial([hartree_fock_index(N, na, na)], [1.0])
    o.set_ops(ops, np.arange(len(ops)), np.ones(len(ops)))
    o.set_ham_integrals(h1, g2, csr=True)
    E, g = e.gradient(ang)
    Eo, go = o.energy_gradient_ops(ang)
    assert abs(E - Eo) < 1e-10
    np.testing.assert_allclose(g, go, atol=1e-9, rtol=0)
    s = e.evolve(ang)
    np.testing.assert_allclose(s, o.evolve_ops(ang), atol=1e-12, rtol=0)
    e.close()


def test_lucj_14_orbitals_on_the_fly_energy_gradient():
    """14 orbitals, 7a+7b, complex128 (188 MB state), H on the fly: the gradient is
    checked against a central difference of the energy along a random direction, and
    the norm of the state stays 1."""
    N, na = 14, 7
    K, J = random_lucj(N, 3)
    e, ops, ang, h1, g2 = lucj_engine(N, na, K, J, ae.HAM_ON_THE_FLY)
    assert e.D == 11778624
    E, g = e.gradient(ang)
    psi = e.evolve(ang)
    assert abs(np.dot(psi, psi) - 1.0) < 1e-12
    rng = np.random.default_rng(1)
    d = rng.normal(size=len(ang))
    d /= np.linalg.norm(d)
    h = 1e-4
    Ep = e.energy(ang + h * d)
    Em = e.energy(ang - h * d)
    assert abs((Ep - Em) / (2 * h) - g @ d) < 1e-7 * max(1.0, abs(g @ d))
    e.close()


def test_lucj_14_orbitals_matches_reference(golden):
    """The complex LUCJ circuit at 14 orbitals (7a+7b, 11,778,624 determinants, 1214
    operators, each its own parameter) against the reference's own complex build
    (tests/golden/lucj14.npz): energy at 1e-10, every operator's gradient at 1e-9,
    sampled final-state amplitudes at 1e-12, H on the fly in both.  The operators and
    angles are the fixture's own (the inputs the reference ran): the decomposition of
    exp(K) goes through a LAPACK eigensolver, whose phase choices can differ between
    machines by multiples of 2 pi in individual angles."""
    fx = golden("lucj14")
    N, na = int(fx["N"]), int(fx["na"])
    ops, ang = np.asarray(fx["ops"]), np.asarray(fx["x"])
    K, J = random_lucj(N, int(fx["lucj_seed"]))
    ops_here, ang_here = lucj_operators(K, J)
    np.testing.assert_array_equal(ops_here, ops)
    # the same circuit: angles agree modulo 2 pi
    d = np.angle(np.exp(1j * (ang_here - ang)))
    assert np.max(np.abs(d)) < 1e-12
    e = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops, complex_mode=True)
    init = np.zeros(2 * e.D)
    init[2 * np.searchsorted(e.states(), hartree_fock_index(N, na, na))] = 1.0
    e.set_initial(init)
    h1, g2 = synthetic_integrals(N, int(fx["ham_seed"]))
    e.set_ham_integrals(h1, g2, ae.HAM_ON_THE_FLY)
    E, g = e.gradient(ang)
    assert abs(E - float(fx["E"])) < 1e-10
    np.testing.assert_allclose(g, fx["G"], atol=1e-9, rtol=0)
    psi = e.evolve(ang)
    assert np.array_equal(e.states()[fx["sample_rank"]], fx["sample_bits"])
    amp = psi[2 * fx["sample_rank"]] + 1j * psi[2 * fx["sample_rank"] + 1]
    np.testing.assert_allclose(amp, fx["sample_amp"], atol=1e-12, rtol=0)
    assert abs(np.dot(psi, psi) - float(fx["norm"])) < 1e-12
    e.close()
