"""Batched evaluation (nb instances per call) against one-at-a-time evaluation and the
oracle.  A batch runs the same kernels with an instance index, so every instance's
energy, gradient and state must be bit-identical to evaluating it alone."""
import numpy as np
import pytest

import ansatzevolve_gb300 as ae
from ansatzevolve_gb300.synthetic import family_integrals
from tests.fixtures import oracle_synthetic, sector_of, synthetic_problem

pytestmark = pytest.mark.gpu
TOL_E, TOL_G = 1e-10, 1e-9


def make_engine(pb, nb=1):
    ops0 = np.asarray(pb["ops_1b"]) - 1
    N = pb["N"]
    eng = ae.Engine(2 * N, ae.BASIS_SZ, pb["na"] + pb["nb"], pb["na"], pb["nb"], ops0)
    init = np.zeros(eng.D)
    init[np.searchsorted(eng.states(), pb["hf"])] = 1.0
    eng.set_initial(init)
    if nb > 1:
        eng.set_batch(nb)
    return eng


@pytest.mark.parametrize("mode", [ae.HAM_STORED, ae.HAM_ON_THE_FLY])
def test_batch_shared_hamiltonian_bit_identical(mode):
    pb = synthetic_problem(8, 4, 4, 2, 0)
    nb = 6
    rng = np.random.default_rng(21)
    nops = len(pb["ops_1b"])
    ang = rng.uniform(-0.3, 0.3, (nb, nops))
    one = make_engine(pb)
    one.set_ham_integrals(pb["h1"], pb["g2"], mode)
    bat = make_engine(pb, nb)
    assert bat.nb == nb
    bat.set_ham_integrals(pb["h1"], pb["g2"], mode)
    Eb, gb = bat.gradient(ang)
    psib = bat.evolve(ang)
    assert gb.shape == (nb, nops) and psib.shape == (nb, one.D)
    for b in range(nb):
        E, g = one.gradient(ang[b])
        assert Eb[b] == E
        assert np.array_equal(gb[b], g)
        assert np.array_equal(psib[b], one.evolve(ang[b]))
    assert np.array_equal(bat.energy(ang), Eb)
    # one instance against the oracle
    o = oracle_synthetic(pb, csr=False)
    Eo, go = o.energy_gradient_ops(ang[3])
    assert abs(Eb[3] - Eo) < TOL_E
    np.testing.assert_allclose(gb[3], go, atol=TOL_G, rtol=0)
    one.close()
    bat.close()


@pytest.mark.parametrize("mode", [ae.HAM_STORED, ae.HAM_ON_THE_FLY])
def test_batch_per_instance_integrals(mode):
    """Instance b carries its own integrals (a Hamiltonian family): each must agree
    bit for bit with an engine holding only that Hamiltonian."""
    pb = synthetic_problem(8, 4, 4, 2, 0)
    nb = 5
    s = np.linspace(0.0, 1.0, nb)
    fam = [family_integrals(8, float(si), seed=3) for si in s]
    h1s = np.stack([f[0] for f in fam])
    g2s = np.stack([f[1] for f in fam])
    rng = np.random.default_rng(5)
    ang = rng.uniform(-0.3, 0.3, (nb, len(pb["ops_1b"])))
    bat = make_engine(pb, nb)
    bat.set_ham_integrals_batch(h1s, g2s, mode)
    Eb, gb = bat.gradient(ang)
    one = make_engine(pb)
    for b in range(nb):
        one.set_ham_integrals(h1s[b], g2s[b], mode)
        E, g = one.gradient(ang[b])
        assert Eb[b] == E, (b, Eb[b], E)
        assert np.array_equal(gb[b], g)
    # the last instance against the oracle
    pb_last = dict(pb, h1=h1s[-1], g2=g2s[-1])
    Eo, go = oracle_synthetic(pb_last, csr=False).energy_gradient_ops(ang[-1])
    assert abs(Eb[-1] - Eo) < TOL_E
    np.testing.assert_allclose(gb[-1], go, atol=TOL_G, rtol=0)
    # changing the batch size drops per-instance Hamiltonians
    bat.set_batch(nb + 1)
    with pytest.raises(ae.AegpuError, match="no Hamiltonian"):
        bat.energy(np.zeros((nb + 1, len(pb["ops_1b"]))))
    one.close()
    bat.close()


def test_batch_10_orbital_family_on_the_fly_vs_oracle():
    pb = synthetic_problem(10, 5, 5, 3, 0)
    nb = 3
    fam = [family_integrals(10, si, seed=11) for si in (0.1, 0.5, 0.9)]
    bat = make_engine(pb, nb)
    bat.set_ham_integrals_batch(np.stack([f[0] for f in fam]), np.stack([f[1] for f in fam]), ae.HAM_ON_THE_FLY)
    rng = np.random.default_rng(3)
    ang = rng.uniform(-0.3, 0.3, (nb, len(pb["ops_1b"])))
    Eb, gb = bat.gradient(ang)
    b = 1
    Eo, go = oracle_synthetic(dict(pb, h1=fam[b][0], g2=fam[b][1]), csr=False).energy_gradient_ops(ang[b])
    assert abs(Eb[b] - Eo) < TOL_E
    np.testing.assert_allclose(gb[b], go, atol=TOL_G, rtol=0)
    bat.close()


def test_batch_graph_path_matches_host_path():
    torch = pytest.importorskip("torch")
    pb = synthetic_problem(8, 4, 4, 2, 0)
    nb = 7
    nops = len(pb["ops_1b"])
    bat = make_engine(pb, nb)
    fam = [family_integrals(8, float(si), seed=4) for si in np.linspace(0, 1, nb)]
    bat.set_ham_integrals_batch(np.stack([f[0] for f in fam]), np.stack([f[1] for f in fam]), ae.HAM_STORED)
    rng = np.random.default_rng(17)
    for k in range(3):
        ang = rng.uniform(-0.3, 0.3, (nb, nops))
        E, g = bat.gradient(ang)
        a = torch.tensor(ang, dtype=torch.float64, device="cuda")
        Ed = torch.zeros(nb, dtype=torch.float64, device="cuda")
        gd = torch.zeros((nb, nops), dtype=torch.float64, device="cuda")
        bat.gradient_dev(a.data_ptr(), Ed.data_ptr(), gd.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert np.array_equal(Ed.cpu().numpy(), E)
        assert np.array_equal(gd.cpu().numpy(), g)
    bat.close()


def test_batch_complex_with_number_operators(golden):
    """Complex mode with diagonal (number) passes, one Hamiltonian shared by the batch."""
    fx = golden("h4c")
    nq = int(fx["nq"])
    ops0 = np.asarray(fx["ops_1b"]) - 1
    kind, ne, na, nbe = sector_of(nq, fx["init_idx"], ops0)
    assert kind == ae.BASIS_SZ
    order = np.asarray(fx["order_1b"]) - 1
    scale = np.asarray(fx["scale"])

    def build(nb):
        eng = ae.Engine(nq, kind, ne, na, nbe, ops0, complex_mode=True)
        init = np.zeros(2 * eng.D)
        pos = np.searchsorted(eng.states(), np.asarray(fx["init_idx"]))
        init[2 * pos] = fx["init_re"]
        init[2 * pos + 1] = fx["init_im"]
        eng.set_initial(init)
        if nb > 1:
            eng.set_batch(nb)
        eng.set_ham_integrals(fx["h1"], fx["g2"], ae.HAM_STORED)
        return eng

    nb = 4
    rng = np.random.default_rng(2)
    P = int(order.max()) + 1
    xs = rng.uniform(-0.5, 0.5, (nb, P))
    ang = scale * xs[:, order]
    one, bat = build(1), build(nb)
    Eb, gb = bat.gradient(ang)
    for b in range(nb):
        E, g = one.gradient(ang[b])
        assert Eb[b] == E
        assert np.array_equal(gb[b], g)
    # every instance at the fixture's angles reproduces the reference energy
    for k in range(len(fx["angles"])):
        angk = np.tile(scale * np.asarray(fx["angles"][k])[:P][order], (nb, 1))
        np.testing.assert_allclose(bat.energy(angk), fx["E"][k] - float(fx["nuclear"]), atol=TOL_E, rtol=0)
    one.close()
    bat.close()


def test_group_launch_mixed_sizes():
    """Two batches of different determinant-space sizes evaluated by one graph launch
    give the same results as each engine's own evaluation."""
    p8 = synthetic_problem(8, 4, 4, 2, 0)
    p6 = synthetic_problem(6, 3, 3, 2, 1)
    e8 = make_engine(p8, 3)
    fam = [family_integrals(8, float(si), seed=6) for si in (0.0, 0.4, 0.8)]
    e8.set_ham_integrals_batch(np.stack([f[0] for f in fam]), np.stack([f[1] for f in fam]), ae.HAM_ON_THE_FLY)
    e6 = make_engine(p6, 2)
    e6.set_ham_integrals(p6["h1"], p6["g2"], ae.HAM_STORED)
    grp = ae.Group([e8, e6])
    assert grp.launch_count() > 0
    rng = np.random.default_rng(23)
    for k in range(2):
        a8 = rng.uniform(-0.3, 0.3, (3, e8.nops))
        a6 = rng.uniform(-0.3, 0.3, (2, e6.nops))
        e8.io_put_angles(a8)
        e6.io_put_angles(a6)
        for e in (e8, e6):  # uploads ran on the engines' streams: finish them
            e.io_get_results()
        grp.launch()
        grp.sync()
        E8, g8 = e8.io_get_results()
        E6, g6 = e6.io_get_results()
        R8, G8 = e8.gradient(a8)
        R6, G6 = e6.gradient(a6)
        assert np.array_equal(E8, R8) and np.array_equal(g8, G8)
        assert np.array_equal(E6, R6) and np.array_equal(g6, G6)
    # a member that changes invalidates the group
    e6.set_batch(3)
    with pytest.raises(ae.AegpuError):
        grp.launch()
    grp.close()
    e8.close()
    e6.close()


@pytest.mark.parametrize("tpr", [1, 2, 4, 8])
def test_stored_product_threads_per_row(tpr):
    """Every threads-per-row shape of the stored-H product gives H x (against the
    oracle's operator-list product) and the same energy."""
    pb = synthetic_problem(8, 4, 4, 2, 0)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    e = ae.Engine(16, ae.BASIS_SZ, 8, 4, 4, ops0, tuning={ae.TUNE_SPMV_TPR: tpr})
    init = np.zeros(e.D)
    init[np.searchsorted(e.states(), pb["hf"])] = 1.0
    e.set_initial(init)
    e.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    assert e.tuning()[ae.TUNE_SPMV_TPR] == tpr
    o = oracle_synthetic(pb, csr=False)
    x = np.random.default_rng(tpr).normal(size=e.D)
    np.testing.assert_allclose(e.apply_h(x), o.apply_h(x), atol=1e-11, rtol=1e-12)
    ang = np.random.default_rng(1).uniform(-0.3, 0.3, len(ops0))
    E, g = e.gradient(ang)
    Eo, go = o.energy_gradient_ops(ang)
    assert abs(E - Eo) < TOL_E
    np.testing.assert_allclose(g, go, atol=TOL_G, rtol=0)
    e.close()


def test_out_of_order_calls_are_refused():
    """A second problem on one engine, a batch size out of range, a Hessian of a batch
    and a group launch without a Hamiltonian return status codes (no trap)."""
    pb = synthetic_problem(6, 3, 3, 1, 0)
    ops0 = np.ascontiguousarray(np.asarray(pb["ops_1b"]) - 1, dtype=np.int32)
    e = ae.Engine(12, ae.BASIS_SZ, 6, 3, 3, ops0)
    rc = e.L.aegpu_set_problem(e.h, 12, ae.BASIS_SZ, 6, 3, 3, 0, len(ops0), ae.iptr(ops0.reshape(-1)))
    assert rc == 2 and "already set" in e.L.aegpu_last_error(e.h).decode()
    assert e.L.aegpu_set_batch(e.h, 0) == 1
    assert e.L.aegpu_set_batch(e.h, 70000) == 1
    with pytest.raises(ae.AegpuError):
        ae.Group([e])  # no Hamiltonian yet
    e.set_batch(2)
    e.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    p0 = np.asarray(pb["order_1b"]) - 1
    with pytest.raises(ae.AegpuError, match="batch size of 1"):
        e.hessian(np.zeros(len(ops0)), p0, np.asarray(pb["scale"]))
    e.close()


def test_instance_mask_skips_and_keeps_results():
    """Masked instances are skipped (their results stay as they were); the others are
    bit-identical to the unmasked evaluation, through both the host and graph paths."""
    pb = synthetic_problem(8, 4, 4, 2, 0)
    nb = 5
    e = make_engine(pb, nb)
    fam = [family_integrals(8, float(si), seed=8) for si in np.linspace(0, 1, nb)]
    e.set_ham_integrals_batch(np.stack([f[0] for f in fam]), np.stack([f[1] for f in fam]), ae.HAM_ON_THE_FLY)
    rng = np.random.default_rng(30)
    a1 = rng.uniform(-0.3, 0.3, (nb, e.nops))
    a2 = rng.uniform(-0.3, 0.3, (nb, e.nops))
    E1, g1 = e.gradient(a1)
    E2, g2 = e.gradient(a2)
    mask = np.array([1, 0, 1, 0, 1])
    E1, g1 = e.gradient(a1)  # all active: results at a1
    e.set_active(mask)
    Em, gm = e.gradient(a2)
    for b in range(nb):
        if mask[b]:
            assert Em[b] == E2[b] and np.array_equal(gm[b], g2[b])
        else:
            assert Em[b] == E1[b] and np.array_equal(gm[b], g1[b])
    e.set_active(None)
    Ea, ga = e.gradient(a2)
    assert np.array_equal(Ea, E2) and np.array_equal(ga, g2)
    e.close()


def test_allocation_failures_return_status_codes():
    """Host-side fault injection: whichever set-up allocation fails, the call returns a
    status (out of memory) instead of trapping, and a later engine works normally."""
    pb = synthetic_problem(6, 3, 3, 1, 0)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    L = ae.lib()
    seen_fail = 0
    try:
        for n in (0, 2, 5, 9, 14, 20, 30, 45):
            L.aegpu_debug_fail_alloc_after(n)
            try:
                e = ae.Engine(12, ae.BASIS_SZ, 6, 3, 3, ops0)
                e.set_batch(3)
                e.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
                e.gradient(np.zeros((3, e.nops)))
                e.close()
            except ae.AegpuError as err:
                assert "error 4" in str(err) or "allocation" in str(err), err
                seen_fail += 1
    finally:
        L.aegpu_debug_fail_alloc_after(-1)
    assert seen_fail >= 4
    e = ae.Engine(12, ae.BASIS_SZ, 6, 3, 3, ops0)
    e.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    E, g = e.gradient(np.zeros(e.nops))
    assert np.isfinite(E)
    e.close()


def test_batched_hessian_columns_and_line_search_points():
    """One batched energy + gradient launch over an instance's Hessian columns (central
    differences of the analytic gradient at x +- h e_i) and its line-search points
    x + t d: the columns reproduce the analytic Hessian, and every point's energy and
    gradient equal a batch-of-one evaluation at that point."""
    from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals, tups_operators
    N, na, L = 8, 4, 2
    ops, param, scale = tups_operators(N, L)
    p0, P = param - 1, int(param.max())
    h1, g2 = synthetic_integrals(N, 3)
    x = np.random.default_rng(4).uniform(-0.3, 0.3, P)
    e1 = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops - 1)
    init = np.zeros(e1.D)
    init[np.searchsorted(e1.states(), hartree_fock_index(N, na, na))] = 1.0
    e1.set_initial(init)
    e1.set_ham_integrals(h1, g2, ae.HAM_STORED)
    _, g0, Hx = e1.hessian(scale * x[p0], p0, scale)
    h = 1e-4
    ts = np.linspace(0.2, 1.5, 6)
    X = np.vstack([x + h * np.eye(P), x - h * np.eye(P), x[None, :] + ts[:, None] * (-g0)[None, :]])
    e = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops - 1)
    e.set_initial(init)
    e.set_batch(len(X))
    e.set_ham_integrals(h1, g2, ae.HAM_STORED)
    e.io_put_angles(scale[None, :] * X[:, p0])
    e.launch_io()
    E, gops = e.io_get_results()
    G = np.zeros((len(X), P))
    for k in range(len(X)):
        np.add.at(G[k], p0, scale * gops[k])
    Hfd = (G[:P] - G[P:2 * P]) / (2 * h)
    np.testing.assert_allclose(Hfd, Hx, atol=1e-6, rtol=0)
    for k in (0, P, 2 * P, len(X) - 1):
        Ek, gk = e1.gradient(scale * X[k][p0])
        assert abs(Ek - E[k]) < 1e-12
        np.testing.assert_allclose(gk, gops[k], atol=1e-12, rtol=0)
    e.close()
    e1.close()


@pytest.mark.parametrize("mode", [ae.HAM_STORED, ae.HAM_ON_THE_FLY])
def test_new_integral_values_refresh_in_place(mode):
    """Setting new integrals of the same shape on an engine that already has some
    (a family scan) gives exactly what a fresh engine gives for them, for a batch with
    per-instance integrals too, and a captured evaluation graph keeps working."""
    from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals, tups_operators
    N, na = 8, 4
    ops, param, scale = tups_operators(N, 2)
    ang = np.random.default_rng(2).uniform(-0.3, 0.3, len(ops))

    def fresh(ints, nb):
        e = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops - 1)
        init = np.zeros(e.D)
        init[np.searchsorted(e.states(), hartree_fock_index(N, na, na))] = 1.0
        e.set_initial(init)
        if nb > 1:
            e.set_batch(nb)
            e.set_ham_integrals_batch(np.stack([a for a, _ in ints]), np.stack([b for _, b in ints]), mode)
        else:
            e.set_ham_integrals(*ints[0], mode)
        return e

    for nb in (1, 3):
        first = [synthetic_integrals(N, 10 + b) for b in range(nb)]
        second = [synthetic_integrals(N, 20 + b) for b in range(nb)]
        e = fresh(first, nb)
        A = np.tile(ang, (nb, 1)) if nb > 1 else ang
        e.gradient(A)
        if nb > 1:
            e.set_ham_integrals_batch(np.stack([a for a, _ in second]), np.stack([b for _, b in second]), mode)
        else:
            e.set_ham_integrals(*second[0], mode)
        E1, g1 = e.gradient(A)
        ref = fresh(second, nb)
        E2, g2 = ref.gradient(A)
        assert np.array_equal(np.atleast_1d(E1), np.atleast_1d(E2))
        assert np.array_equal(g1, g2)
        ref.close()
        e.close()


@pytest.mark.parametrize("N,na,L,s0,mode", [(8, 4, 2, 0, ae.HAM_STORED), (10, 5, 3, 256, ae.HAM_ON_THE_FLY),
                                            (12, 6, 3, 448, ae.HAM_ON_THE_FLY)])
def test_batched_classes_match_reference(golden, N, na, L, s0, mode):
    """Instance 0 of each size class of the benchmark's batched launch (its integrals and
    angles) inside a batch with per-instance integrals, against the reference's own
    energy and gradient (tests/golden/batched4.npz)."""
    from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals, tups_operators
    fx = golden("batched4")
    ops, param, scale = tups_operators(N, L)
    e = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops - 1)
    init = np.zeros(e.D)
    init[np.searchsorted(e.states(), hartree_fock_index(N, na, na))] = 1.0
    e.set_initial(init)
    e.set_batch(2)
    ints = [synthetic_integrals(N, s0), synthetic_integrals(N, s0 + 1)]
    e.set_ham_integrals_batch(np.stack([a for a, _ in ints]), np.stack([b for _, b in ints]), mode)
    x = np.asarray(fx["x%d" % N])
    E, g = e.gradient(np.vstack([x, np.random.default_rng(1).uniform(-0.3, 0.3, len(x))]))
    gc = np.zeros(int(param.max()))
    np.add.at(gc, param - 1, scale * g[0])
    assert abs(E[0] - float(fx["E%d" % N])) < 1e-10
    np.testing.assert_allclose(gc, fx["G%d" % N], atol=1e-9, rtol=0)
    e.close()
