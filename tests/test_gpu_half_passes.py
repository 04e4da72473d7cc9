"""Spin-flip half passes of the forward and adjoint sweeps.  A tUPS circuit holds the
mirror of every excitation (alpha and beta orbitals exchanged) in the same pass, and
its compressed parameters give mirrors the same angle, so from the closed-shell start
the state keeps psi(a, b) = psi(b, a) through every pass: the engine visits one orbit
of every mirror pair, keeps the amplitudes with a <= b current and sums each gradient
over the excitation and its mirror.  The tests check that the half passes are taken
exactly when the angles and the start state allow them, that they agree with the full
passes (knob off) to rounding and with the oracle, single and batched, through the
captured graph and the host path, and that the projected gradient (whose bra has no
symmetry) and the Hessian still run the full passes after a half evaluation at the
same angles."""
import numpy as np
import pytest

import ansatzevolve_gb300 as ae
from tests.fixtures import oracle_synthetic, synthetic_problem

pytestmark = pytest.mark.gpu


def make_engine(pb, nb=1, cplx=False):
    N = pb["N"]
    e = ae.Engine(2 * N, ae.BASIS_SZ, pb["na"] + pb["nb"], pb["na"], pb["nb"], np.asarray(pb["ops_1b"]) - 1,
                  complex_mode=cplx)
    W = 2 if cplx else 1
    init = np.zeros(e.D * W)
    init[W * np.searchsorted(e.states(), pb["hf"])] = 1.0
    e.set_initial(init)
    if nb > 1:
        e.set_batch(nb)
    return e


def compressed_angles(pb, x):
    return np.asarray(pb["scale"], dtype=float) * x[np.asarray(pb["order_1b"]) - 1]


@pytest.mark.parametrize("N,L,mode", [(8, 2, ae.HAM_STORED), (10, 3, ae.HAM_ON_THE_FLY), (12, 1, ae.HAM_STORED)])
def test_half_passes_match_full_and_oracle(N, L, mode):
    na = N // 2
    pb = synthetic_problem(N, na, na, L, 3)
    P = int(np.max(pb["order_1b"]))
    rng = np.random.default_rng(N + L)
    ang = compressed_angles(pb, rng.uniform(-0.6, 0.6, P))
    e = make_engine(pb)
    e.set_ham_integrals(pb["h1"], pb["g2"], mode)
    info = e.half_info()
    assert info["available"] and 0 < info["active"] < e.info()["active"]
    assert e.get_tuning(ae.TUNE_HALF) == 1
    E1, g1 = e.gradient(ang)
    assert e.half_status()[0]
    psi1 = e.evolve(ang)
    M = psi1.reshape(int(round(e.D ** 0.5)), -1)
    assert np.array_equal(M, M.T)  # the state is completed from its a <= b half
    e.set_tuning(ae.TUNE_HALF, 0)
    E0, g0 = e.gradient(ang)
    assert not e.half_status()[0]
    psi0 = e.evolve(ang)
    assert abs(E1 - E0) < 1e-12 * max(1.0, abs(E0))
    np.testing.assert_allclose(g1, g0, atol=1e-11, rtol=0)
    np.testing.assert_allclose(psi1, psi0, atol=1e-13, rtol=0)
    if N <= 10:  # 12 orbitals: against the reference's own output in test_gpu_reference.py
        o = oracle_synthetic(pb, csr=False)
        Eo, go = o.energy_gradient_ops(ang)
        assert abs(E1 - Eo) < 1e-10
        np.testing.assert_allclose(g1, go, atol=1e-9, rtol=0)
    e.close()


def test_half_passes_off_without_the_symmetry():
    """Independent angles, or a start state without psi(a,b) = psi(b,a): the full passes,
    bit for bit the results with the knob off."""
    N, na = 8, 4
    pb = synthetic_problem(N, na, na, 2, 6)
    rng = np.random.default_rng(7)
    e = make_engine(pb)
    e.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    ang = rng.uniform(-0.4, 0.4, len(pb["ops_1b"]))
    Ea, ga = e.gradient(ang)
    assert not e.half_status()[0]
    e.set_tuning(ae.TUNE_HALF, 0)
    Eb, gb = e.gradient(ang)
    assert Ea == Eb and np.array_equal(ga, gb)
    o = oracle_synthetic(pb, csr=False)
    Eo, go = o.energy_gradient_ops(ang)
    assert abs(Ea - Eo) < 1e-10
    np.testing.assert_allclose(ga, go, atol=1e-9, rtol=0)
    # an unsymmetric start state (two determinants, (a, b) and not (b, a))
    e.set_tuning(ae.TUNE_HALF, 1)
    states = e.states()
    lo = (1 << N) - 1
    a_str, b_str = [s for s in range(1 << N) if bin(s).count("1") == na][:2]
    d1 = (a_str << N) | b_str
    init = np.zeros(e.D)
    init[np.searchsorted(states, pb["hf"])] = 0.8
    init[np.searchsorted(states, d1)] = 0.6
    assert (d1 & lo) != (d1 >> N)
    e.set_initial(init)
    angc = compressed_angles(pb, rng.uniform(-0.4, 0.4, int(np.max(pb["order_1b"]))))
    Ec, gc = e.gradient(angc)
    assert not e.half_status()[0]
    o.set_initial(states[init != 0], init[init != 0])
    Eo, go = o.energy_gradient_ops(angc)
    assert abs(Ec - Eo) < 1e-10
    np.testing.assert_allclose(gc, go, atol=1e-9, rtol=0)
    e.close()


def test_half_passes_batched_graph_and_host_paths():
    """A batch whose instances alternate between symmetric and independent angles: each
    takes its own passes and equals its own batch-of-one evaluation bit for bit, on the
    host path and through the captured graph."""
    N, na, nb = 8, 4, 4
    pb = synthetic_problem(N, na, na, 2, 8)
    P = int(np.max(pb["order_1b"]))
    rng = np.random.default_rng(9)
    angs = []
    for b in range(nb):
        angs.append(compressed_angles(pb, rng.uniform(-0.5, 0.5, P)) if b % 2 == 0
                    else rng.uniform(-0.5, 0.5, len(pb["ops_1b"])))
    angs = np.array(angs)
    e = make_engine(pb, nb)
    e.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    E, g = e.gradient(angs)
    assert list(e.half_status()) == [True, False, True, False]
    e.io_put_angles(angs)
    e.launch_io()
    Eg, gg = e.io_get_results()
    assert np.array_equal(E, Eg) and np.array_equal(g, gg)
    one = make_engine(pb)
    one.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    for b in range(nb):
        E1, g1 = one.gradient(angs[b])
        assert E1 == E[b] and np.array_equal(g1, g[b])
    one.close()
    e.close()


def test_projected_gradient_and_hessian_after_half_evaluation():
    """The projected gradient's bra has no mirror symmetry and the Hessian's sweeps carry
    tangents: both run the full passes, also right after a half evaluation at the same
    angles (whose checkpoints are laid out for the half passes)."""
    N, na = 8, 4
    pb = synthetic_problem(N, na, na, 2, 10)
    P = int(np.max(pb["order_1b"]))
    rng = np.random.default_rng(11)
    ang = compressed_angles(pb, rng.uniform(-0.5, 0.5, P))
    e = make_engine(pb)
    e.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    E, g = e.gradient(ang)
    assert e.half_status()[0]
    proj = rng.normal(size=e.D)
    proj /= np.linalg.norm(proj)
    ov, gp = e.gradient_proj(ang, proj)
    o = oracle_synthetic(pb, csr=False)
    ovo, gpo = o.gradient_proj_ops(ang, proj)
    assert abs(ov - ovo) < 1e-12
    np.testing.assert_allclose(gp, gpo, atol=1e-10, rtol=0)
    # the energy gradient again at the same angles (state cached): still right
    E2, g2 = e.gradient(ang)
    assert abs(E2 - E) < 1e-12
    np.testing.assert_allclose(g2, g, atol=1e-11, rtol=0)
    x = rng.uniform(-0.5, 0.5, P)
    _, _, H = e.hessian(compressed_angles(pb, x), np.asarray(pb["order_1b"]) - 1, pb["scale"])
    Ho = o.hessian_comp(x)
    np.testing.assert_allclose(H, Ho, atol=1e-9, rtol=0)
    e.close()


@pytest.mark.parametrize("mode", [ae.HAM_STORED, ae.HAM_ON_THE_FLY])
def test_half_passes_complex_lucj(mode):
    """The complex LUCJ circuit: its Givens and phase operators come in alpha/beta
    mirror pairs with equal angles, its density-density operators are their own mirrors
    or pairs, so rotation and diagonal passes both run halved; the results match the
    full passes and the oracle."""
    from oracle.oracle import Oracle
    from ansatzevolve_gb300.lucj import lucj_operators, random_lucj
    from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals
    N, na = 8, 4
    K, J = random_lucj(N, 2)
    ops, ang = lucj_operators(K, J)
    e = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops, complex_mode=True)
    init = np.zeros(2 * e.D)
    init[2 * np.searchsorted(e.states(), hartree_fock_index(N, na, na))] = 1.0
    e.set_initial(init)
    h1, g2 = synthetic_integrals(N, 7)
    e.set_ham_integrals(h1, g2, mode)
    assert e.half_info()["available"]
    E1, g1 = e.gradient(ang)
    assert e.half_status()[0]
    s1 = e.evolve(ang)
    e.set_tuning(ae.TUNE_HALF, 0)
    E0, g0 = e.gradient(ang)
    s0 = e.evolve(ang)
    assert abs(E1 - E0) < 1e-12 * max(1.0, abs(E0))
    np.testing.assert_allclose(g1, g0, atol=1e-11, rtol=0)
    np.testing.assert_allclose(s1, s0, atol=1e-13, rtol=0)
    o = Oracle(2 * N, 2, 2 * na, na, na, cplx=True)
    o.set_initial([hartree_fock_index(N, na, na)], [1.0])
    o.set_ops(ops, np.arange(len(ops)), np.ones(len(ops)))
    o.set_ham_integrals(h1, g2, csr=True)
    Eo, go = o.energy_gradient_ops(ang)
    assert abs(E1 - Eo) < 1e-10
    np.testing.assert_allclose(g1, go, atol=1e-9, rtol=0)
    e.close()


@pytest.mark.parametrize("N,L,mode", [(8, 2, ae.HAM_STORED), (10, 2, ae.HAM_ON_THE_FLY)])
def test_hessian_half_tangents_match_full(N, L, mode):
    """With the half passes' symmetry the Hessian carries one tangent of every mirror
    pair and counts each second-derivative pair for its mirror pair too; it matches the
    full computation (knob off) and the oracle."""
    na = N // 2
    pb = synthetic_problem(N, na, na, L, 13)
    P = int(np.max(pb["order_1b"]))
    rng = np.random.default_rng(N + 7)
    x = rng.uniform(-0.5, 0.5, P)
    ang = compressed_angles(pb, x)
    p0, sc = np.asarray(pb["order_1b"]) - 1, pb["scale"]
    e = make_engine(pb)
    e.set_ham_integrals(pb["h1"], pb["g2"], mode)
    E1, g1, H1 = e.hessian(ang, p0, sc)
    e.gradient(ang)
    assert e.half_status()[0]
    e.set_tuning(ae.TUNE_HALF, 0)
    E0, g0, H0 = e.hessian(ang, p0, sc)
    assert abs(E1 - E0) < 1e-12 * max(1.0, abs(E0))
    np.testing.assert_allclose(g1, g0, atol=1e-11, rtol=0)
    np.testing.assert_allclose(H1, H0, atol=1e-10, rtol=0)
    o = oracle_synthetic(pb, csr=False)
    np.testing.assert_allclose(H1, o.hessian_comp(x), atol=1e-9, rtol=0)
    e.close()


def test_diagonal_half_pass_counts():
    """The work accounting of the diagonal passes (the bench's FP64 and HBM figures of
    the LUCJ sweeps): the amplitudes with an active slot and the slot activations over
    every determinant (full passes) and over a <= b (half passes), against a count over
    the basis with the engine's own pass layout."""
    from ansatzevolve_gb300.lucj import lucj_operators, random_lucj
    N, na = 8, 4
    K, J = random_lucj(N, 2)
    ops, _ = lucj_operators(K, J)
    dops = np.array([o for o in ops if o[0] == o[1] or o[2] >= 0], dtype=np.int32)
    e = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, dops, complex_mode=True)
    hi = e.half_info()
    assert hi["available"]
    passes, diag, mirrored = ae.host_pass_layout(2 * N, dops, e.get_tuning(ae.TUNE_PASS_OPS), True)
    assert mirrored and all(diag) and len(passes) == e.info()["blocks"]
    bits = e.states().astype(np.int64)
    nA = int(round(len(bits) ** 0.5))
    a, b = np.divmod(np.arange(len(bits)), nA)
    tri = a <= b
    ann = np.array([(1 << int(o[0])) | (1 << int(o[1])) for o in dops], dtype=np.int64)
    act = act_h = slots = slots_h = 0
    for p in passes:
        n = ((bits[:, None] & ann[p][None, :]) == ann[p][None, :]).sum(axis=1)
        act += int(np.count_nonzero(n))
        slots += int(n.sum())
        act_h += int(np.count_nonzero(n[tri]))
        slots_h += int(n[tri].sum())
    assert hi["active"] == len(passes) * nA * (nA + 1) // 2
    assert hi["fwd_fp64"] == 4 * act_h and hi["adj_fp64"] == 6 * act_h + slots_h
    _, fwd, adj = e.fp64_work(half=False, half_passes=False)
    assert fwd == 4 * act and adj == 6 * act + slots
    e.close()


@pytest.mark.parametrize("half", [1, 0])
def test_task_orders_agree(half, monkeypatch):
    """The sweeps' two task orders (warp-major where a launch fits one wave, the default;
    CTA-major everywhere with AEGPU_TASK_ORDER=0) visit every warp task once: the same
    state, energy and gradient up to the order of the gradient sums, with and without
    the half passes, real and complex."""
    from ansatzevolve_gb300.lucj import lucj_operators, random_lucj
    from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals
    N, na = 10, 5
    pb = synthetic_problem(N, na, na, 2, 21)
    P = int(np.max(pb["order_1b"]))
    ang = compressed_angles(pb, np.random.default_rng(22).uniform(-0.5, 0.5, P))
    K, J = random_lucj(8, 4)
    lops, lang = lucj_operators(K, J)
    h1, g2 = synthetic_integrals(8, 9)
    out = []
    for order in ("1", "0"):
        monkeypatch.setenv("AEGPU_TASK_ORDER", order)
        e = make_engine(pb)
        e.set_tuning(ae.TUNE_HALF, half)
        e.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_ON_THE_FLY)
        E, g = e.gradient(ang)
        assert bool(e.half_status()[0]) == bool(half)
        psi = e.evolve(ang)
        e.close()
        c = ae.Engine(16, ae.BASIS_SZ, 8, 4, 4, lops, complex_mode=True)
        init = np.zeros(2 * c.D)
        init[2 * np.searchsorted(c.states(), hartree_fock_index(8, 4, 4))] = 1.0
        c.set_initial(init)
        c.set_tuning(ae.TUNE_HALF, half)
        c.set_ham_integrals(h1, g2, ae.HAM_STORED)
        Ec, gc = c.gradient(lang)
        psic = c.evolve(lang)
        c.close()
        out.append((E, g, psi, Ec, gc, psic))
    (E1, g1, p1, Ec1, gc1, pc1), (E0, g0, p0, Ec0, gc0, pc0) = out
    for a, b in ((E1, E0), (Ec1, Ec0)):
        assert abs(a - b) < 1e-12 * max(1.0, abs(b))
    for a, b in ((g1, g0), (gc1, gc0)):
        np.testing.assert_allclose(a, b, atol=1e-12, rtol=0)
    for a, b in ((p1, p0), (pc1, pc0)):
        np.testing.assert_allclose(a, b, atol=1e-14, rtol=0)
