"""Spin-flip half product of the energy's H psi.  With as many alpha as beta electrons,
an integral Hamiltonian and a state with psi(a, b) = psi(b, a) for every pair of alpha
and beta strings (tUPS through its compressed parameters, from the closed-shell start),
H psi has the same symmetry, and the engine computes only the rows with a <= b.  The
tests check that the half path is taken exactly when the state passes the device test,
that it agrees with the full product (knob off) to rounding and with the oracle, for
coded stored rows and on the fly, real and complex, single and batched, and that a
state without the symmetry takes the full path bit for bit."""
import numpy as np
import pytest

import ansatzevolve_gb300 as ae
from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals
from tests.fixtures import oracle_synthetic, synthetic_problem

pytestmark = pytest.mark.gpu


def make_engine(pb, nb=1):
    N = pb["N"]
    e = ae.Engine(2 * N, ae.BASIS_SZ, pb["na"] + pb["nb"], pb["na"], pb["nb"], np.asarray(pb["ops_1b"]) - 1)
    init = np.zeros(e.D)
    init[np.searchsorted(e.states(), pb["hf"])] = 1.0
    e.set_initial(init)
    if nb > 1:
        e.set_batch(nb)
    return e


def compressed_angles(pb, x):
    return np.asarray(pb["scale"], dtype=float) * x[np.asarray(pb["order_1b"]) - 1]


@pytest.mark.parametrize("N,mode", [(8, ae.HAM_STORED), (8, ae.HAM_ON_THE_FLY), (10, ae.HAM_STORED),
                                    (10, ae.HAM_ON_THE_FLY)])
def test_half_product_matches_full_and_oracle(N, mode):
    na = N // 2
    pb = synthetic_problem(N, na, na, 2, 4)
    P = int(np.max(pb["order_1b"]))
    rng = np.random.default_rng(N)
    ang = compressed_angles(pb, rng.uniform(-0.5, 0.5, P))
    e = make_engine(pb)
    e.set_ham_integrals(pb["h1"], pb["g2"], mode)
    assert e.get_tuning(ae.TUNE_FLIP) == 1
    E1, g1 = e.gradient(ang)
    assert e.flip_status()[0]
    e.set_tuning(ae.TUNE_FLIP, 0)
    E0, g0 = e.gradient(ang)
    assert not e.flip_status()[0]
    assert abs(E1 - E0) < 1e-12 * max(1.0, abs(E0))
    np.testing.assert_allclose(g1, g0, atol=1e-11, rtol=0)
    # FP64 work of the half product: rows with a <= b, the energy FMAs, the test
    D, nA = e.D, int(round(e.D ** 0.5))
    width = e.info()["nnz"] // D
    wh, wf = e.fp64_work(half=True)[0], e.fp64_work(half=False)[0]
    assert wf == D * width + D
    assert wh == nA * (nA + 1) // 2 * width + 2 * D + (D - nA) // 2
    assert wh < 0.6 * wf
    o = oracle_synthetic(pb, csr=False)
    Eo, go = o.energy_gradient_ops(ang)
    assert abs(E1 - Eo) < 1e-10
    np.testing.assert_allclose(g1, go, atol=1e-9, rtol=0)
    # independent angles break the symmetry: the full product, bit for bit
    ang2 = rng.uniform(-0.3, 0.3, len(ang))
    e.set_tuning(ae.TUNE_FLIP, 1)
    Ea, ga = e.gradient(ang2)
    assert not e.flip_status()[0]
    e.set_tuning(ae.TUNE_FLIP, 0)
    Eb, gb = e.gradient(ang2)
    assert Ea == Eb and np.array_equal(ga, gb)
    e.close()


@pytest.mark.parametrize("mode", [ae.HAM_STORED, ae.HAM_ON_THE_FLY])
def test_half_product_batched_per_instance(mode):
    """A batch with per-instance integrals whose instances alternate between invariant
    and broken states: each instance takes its own path and equals its own engine's
    result bit for bit; the energy through the captured graph agrees too."""
    N, na, nb = 8, 4, 4
    pb = synthetic_problem(N, na, na, 2, 5)
    P = int(np.max(pb["order_1b"]))
    rng = np.random.default_rng(3)
    nops = len(pb["ops_1b"])
    ang = np.stack([compressed_angles(pb, rng.uniform(-0.5, 0.5, P)) if b % 2 == 0 else rng.uniform(-0.3, 0.3, nops)
                    for b in range(nb)])
    ints = [synthetic_integrals(N, 30 + b) for b in range(nb)]
    bat = make_engine(pb, nb)
    bat.set_ham_integrals_batch(np.stack([h for h, _ in ints]), np.stack([g for _, g in ints]), mode)
    Eb, gb = bat.gradient(ang)
    assert list(bat.flip_status()) == [True, False, True, False]
    for b in range(nb):
        one = make_engine(pb)
        one.set_ham_integrals(*ints[b], mode)
        E, g = one.gradient(ang[b])
        assert Eb[b] == E and np.array_equal(gb[b], g)
        assert one.flip_status()[0] == (b % 2 == 0)
        one.close()
    assert np.array_equal(bat.energy(ang), Eb)
    bat.close()


def test_half_product_hessian():
    """The analytic Hessian (its energy and gradient through the half product, its
    tangent products full) agrees with the knob off."""
    N, na = 8, 4
    pb = synthetic_problem(N, na, na, 2, 6)
    P = int(np.max(pb["order_1b"]))
    p0 = np.asarray(pb["order_1b"]) - 1
    sc = np.asarray(pb["scale"], dtype=float)
    x = np.random.default_rng(7).uniform(-0.5, 0.5, P)
    e = make_engine(pb)
    e.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    E1, g1, H1 = e.hessian(sc * x[p0], p0, sc)
    e.set_tuning(ae.TUNE_FLIP, 0)
    E0, g0, H0 = e.hessian(sc * x[p0], p0, sc)
    assert abs(E1 - E0) < 1e-12 * max(1.0, abs(E0))
    np.testing.assert_allclose(g1, g0, atol=1e-11, rtol=0)
    np.testing.assert_allclose(H1, H0, atol=1e-10, rtol=0)
    e.close()


@pytest.mark.parametrize("mode", [ae.HAM_STORED, ae.HAM_ON_THE_FLY])
def test_half_product_complex_lucj(mode):
    """Complex LUCJ (the same rotation and Jastrow for both spins) from the closed-shell
    start: the state is flip-invariant, the half product agrees with the full one and
    with the oracle."""
    from oracle.oracle import Oracle
    from ansatzevolve_gb300.lucj import lucj_operators, random_lucj
    N, na = 8, 4
    K, J = random_lucj(N, 2)
    ops, ang = lucj_operators(K, J)
    e = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops, complex_mode=True)
    init = np.zeros(2 * e.D)
    init[2 * np.searchsorted(e.states(), hartree_fock_index(N, na, na))] = 1.0
    e.set_initial(init)
    h1, g2 = synthetic_integrals(N, 7)
    e.set_ham_integrals(h1, g2, mode)
    E1, g1 = e.gradient(ang)
    assert e.flip_status()[0]
    e.set_tuning(ae.TUNE_FLIP, 0)
    E0, g0 = e.gradient(ang)
    assert abs(E1 - E0) < 1e-12 * max(1.0, abs(E0))
    np.testing.assert_allclose(g1, g0, atol=1e-11, rtol=0)
    o = Oracle(2 * N, 2, 2 * na, na, na, cplx=True)
    o.set_initial([hartree_fock_index(N, na, na)], [1.0])
    o.set_ops(ops, np.arange(len(ops)), np.ones(len(ops)))
    o.set_ham_integrals(h1, g2, csr=True)
    Eo, go = o.energy_gradient_ops(ang)
    assert abs(E1 - Eo) < 1e-10
    np.testing.assert_allclose(g1, go, atol=1e-9, rtol=0)
    e.close()


def test_flip_knob_checks():
    pb = synthetic_problem(6, 3, 3, 1, 0)
    e = make_engine(pb)
    with pytest.raises(ae.AegpuError):
        e.set_tuning(ae.TUNE_FLIP, 2)
    e.set_tuning(ae.TUNE_FLIP, 0)
    assert e.get_tuning(ae.TUNE_FLIP) == 0
    assert not e.flip_status()[0]  # nothing evaluated yet
    e.close()


@pytest.mark.parametrize("mode", [ae.HAM_STORED, ae.HAM_ON_THE_FLY])
def test_half_product_several_vectors(mode):
    """aegpu_apply_dev over a batch of vectors in one launch (several right-hand sides per
    thread with stored rows, the Hessian's form): invariant vectors, a zero one among
    them, share the half product, a group holding a broken vector takes the full one,
    and every result agrees with the full product."""
    torch = pytest.importorskip("torch")
    N, na, nb = 8, 4, 6
    pb = synthetic_problem(N, na, na, 2, 1)
    e = make_engine(pb, nb)
    e.set_ham_integrals(pb["h1"], pb["g2"], mode)
    D, nA = e.D, int(round(e.D ** 0.5))
    r = np.random.default_rng(9).normal(size=(nb, nA, nA))
    X = r + r.transpose(0, 2, 1)
    X[1] = 0.0
    X[4] = r[4]
    x = torch.tensor(X.reshape(nb, D), dtype=torch.float64, device="cuda")
    ys = []
    s = torch.cuda.Stream()
    for flip in (1, 0):
        e.set_tuning(ae.TUNE_FLIP, flip)
        y = torch.zeros_like(x)
        with torch.cuda.stream(s):
            e.apply_dev(x.data_ptr(), y.data_ptr(), None, s.cuda_stream)
        s.synchronize()
        ys.append(y.cpu().numpy())
    y1, y0 = ys
    assert np.max(np.abs(y1 - y0)) <= 1e-12 * np.max(np.abs(y0))
    assert not np.any(y1[1]) and np.array_equal(y1[4], y0[4])
    e.close()
