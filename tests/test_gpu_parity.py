"""GPU parity of the product path against the reference's outputs and the oracle.

Everything here calls the CUDA extension through its C ABIs: the reference-compatible
AnsatzSynthInterface functions (via the Python mirror of PyAnsatzEvolve) and the
aegpu engine ABI.  Tolerances are the target's: energies 1e-10 Ha, gradient and
Hessian entries 1e-9, statevector entries 1e-12.
"""
import os
import tempfile

import numpy as np
import pytest

import ansatzevolve_gb300 as ae
from ansatzevolve_gb300.synthetic import write_integrals
from tests.fixtures import oracle_synthetic, synthetic_problem

pytestmark = pytest.mark.gpu
TOL_E, TOL_G, TOL_S = 1e-10, 1e-9, 1e-12


def manager_from_fixture(fx, integrals_mode=None):
    m = ae.stateAnsatzManager()
    nq = int(fx["nq"])
    if "init_im" in fx and np.any(np.asarray(fx["init_im"]) != 0):
        coeff = np.asarray(fx["init_re"]) + 1j * np.asarray(fx["init_im"])
    else:
        coeff = np.asarray(fx["init_re"], dtype=float)
    assert m.storeInitial(nq, np.asarray(fx["init_idx"]), coeff)
    assert m.storeOperators(np.asarray(fx["ops_1b"]).tolist())
    assert m.storeParameterDependencies(list(zip(np.asarray(fx["order_1b"]) - 1, fx["scale"])))
    if "h1" in fx:
        assert m.storeIntegrals(fx["h1"], fx["g2"], 0 if integrals_mode is None else integrals_mode)
    else:
        assert m.storeHamiltonian(np.asarray(fx["ham_i_1b"]) - 1, np.asarray(fx["ham_j_1b"]) - 1, fx["ham_v"])
    if "nuclear" in fx:
        assert m.storeNuclearEnergy(float(fx["nuclear"]))
    return m


@pytest.mark.parametrize("name", ["f90", "ferm", "h4", "h4c"])
def test_c_abi_matches_reference_fixture(golden, name):
    fx = golden(name)
    m = manager_from_fixture(fx)
    cplx = name == "h4c"
    for k, x in enumerate(fx["angles"]):
        E = m.getExpectationValue(x)
        assert abs(E - fx["E"][k]) < TOL_E, (name, k, E, fx["E"][k])
        g = m.getGradientComp(x)
        np.testing.assert_allclose(g, fx["G"][k], atol=TOL_G, rtol=0)
        H = m.getHessianComp(x)
        np.testing.assert_allclose(H, fx["H"][k], atol=TOL_G, rtol=0)
        s = m.getFinalState(x, complex_state=cplx)
        want = fx["S"][k]
        if cplx:
            want = want[0::2] + 1j * want[1::2]
        np.testing.assert_allclose(s, want, atol=TOL_S, rtol=0)


@pytest.mark.parametrize("name", ["syn6", "syn8"])
@pytest.mark.parametrize("mode", [ae.HAM_STORED, ae.HAM_ON_THE_FLY])
def test_synthetic_tups_matches_reference(golden, name, mode):
    fx = golden(name)
    N, na, nb = int(fx["N"]), int(fx["na"]), int(fx["nb"])
    pb = synthetic_problem(N, na, nb, int(fx["layers"]), int(fx["seed"]))
    m = ae.stateAnsatzManager()
    assert m.storeInitial(2 * N, [int(fx["hf"])], [1.0])
    assert m.storeOperators(np.asarray(fx["ops_1b"]).tolist())
    assert m.storeParameterDependencies(list(zip(np.asarray(fx["order_1b"]) - 1, fx["scale"])))
    assert m.storeIntegrals(pb["h1"], pb["g2"], mode)
    for k, x in enumerate(fx["angles"]):
        assert abs(m.getExpectationValue(x) - fx["E"][k]) < TOL_E
        np.testing.assert_allclose(m.getGradientComp(x), fx["G"][k], atol=TOL_G, rtol=0)
        s = m.getFinalState(x)
        np.testing.assert_allclose(s[fx["sector"]], fx["S_sector"][k], atol=TOL_S, rtol=0)
    H = m.getHessianComp(fx["angles"][0])
    np.testing.assert_allclose(H, fx["H"][0], atol=TOL_G, rtol=0)


def test_run_path_integral_files_and_optimise(golden):
    """Integrals read from <prefix>_oneEInts.bin / _twoEInts.bin like the reference's
    storeRunPath; Newton from the Parameters file's first set reaches the H4 L1
    minimum of Benchmarks.md:13 (electronic energy -2.838345804245581)."""
    fx = golden("h4")
    m = ae.stateAnsatzManager()
    assert m.storeInitial(int(fx["nq"]), np.asarray(fx["init_idx"]), np.asarray(fx["init_re"], dtype=float))
    assert m.storeOperators(np.asarray(fx["ops_1b"]).tolist())
    assert m.storeParameterDependencies(list(zip(np.asarray(fx["order_1b"]) - 1, fx["scale"])))
    assert m.storeNuclearEnergy(float(fx["nuclear"]))
    with tempfile.TemporaryDirectory() as td:
        prefix = os.path.join(td, "H4")
        write_integrals(prefix, fx["h1"], fx["g2"])
        assert m.storeRunPath(prefix)
        E0 = m.getExpectationValue(fx["angles"][2])
    assert abs(E0 - fx["E"][2]) < TOL_E
    E, x = m.optimise(fx["angles"][2])
    assert abs(E - float(fx["nuclear"]) - (-2.838345804245581)) < 1e-8
    assert abs(E - float(fx["opt_E"])) < 1e-8
    assert np.linalg.norm(m.getGradientComp(x)) < 1e-6


def test_hamiltonian_representations_agree(golden):
    """Stored ELL rows, on-the-fly rows and the oracle's CSR give the same H x."""
    pb = synthetic_problem(8, 4, 4, 2, 0)
    o = oracle_synthetic(pb, csr=True)
    rp, col, val = o.csr()
    rng = np.random.default_rng(3)
    x = rng.normal(size=o.D)
    want = o.apply_h(x)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    for mode in ("csr", ae.HAM_STORED, ae.HAM_ON_THE_FLY):
        eng = ae.Engine(16, ae.BASIS_SZ, 8, 4, 4, ops0)
        if mode == "csr":
            eng.set_ham_csr(rp, col, val)
        else:
            eng.set_ham_integrals(pb["h1"], pb["g2"], mode)
        np.testing.assert_allclose(eng.apply_h(x), want, atol=1e-12, rtol=0)
        eng.close()


@pytest.mark.parametrize("N,na,nb,layers,mode", [(10, 5, 5, 3, ae.HAM_STORED), (10, 5, 5, 3, ae.HAM_ON_THE_FLY),
                                                 (12, 6, 6, 3, ae.HAM_STORED)])
def test_large_energy_gradient_vs_oracle(N, na, nb, layers, mode):
    pb = synthetic_problem(N, na, nb, layers, 0)
    o = oracle_synthetic(pb, csr=False)
    rng = np.random.default_rng(1)
    P = int(np.max(pb["order_1b"]))
    x = rng.uniform(-0.1, 0.1, P)
    Eo, go = o.gradient_comp(x)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    eng = ae.Engine(2 * N, ae.BASIS_SZ, na + nb, na, nb, ops0)
    init = np.zeros(eng.D)
    init[np.searchsorted(eng.states(), pb["hf"])] = 1.0
    eng.set_initial(init)
    eng.set_ham_integrals(pb["h1"], pb["g2"], mode)
    ang = pb["scale"] * x[np.asarray(pb["order_1b"]) - 1]
    E, gops = eng.gradient(ang)
    g = np.zeros(P)
    np.add.at(g, np.asarray(pb["order_1b"]) - 1, pb["scale"] * gops)
    assert abs(E - Eo) < TOL_E
    np.testing.assert_allclose(g, go, atol=TOL_G, rtol=0)
    psi = eng.evolve(ang)
    np.testing.assert_allclose(psi, o.evolve_ops(ang), atol=TOL_S, rtol=0)
    # determinism: the same call twice is bit-identical
    E2, g2 = eng.gradient(ang)
    assert E2 == E and np.array_equal(g2, gops)
    eng.close()


def test_hessian_matches_finite_differences_10_orbitals():
    """Size-independent property at 10 orbitals: the analytic Hessian equals central
    differences of the analytic gradient, and is symmetric."""
    pb = synthetic_problem(10, 5, 5, 1, 2)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    p0 = np.asarray(pb["order_1b"]) - 1
    P = int(p0.max()) + 1
    eng = ae.Engine(20, ae.BASIS_SZ, 10, 5, 5, ops0)
    init = np.zeros(eng.D)
    init[np.searchsorted(eng.states(), pb["hf"])] = 1.0
    eng.set_initial(init)
    eng.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    x = np.random.default_rng(4).uniform(-0.3, 0.3, P)

    def grad(xx):
        _, go = eng.gradient(pb["scale"] * xx[p0])
        g = np.zeros(P)
        np.add.at(g, p0, pb["scale"] * go)
        return g

    E, g, H = eng.hessian(pb["scale"] * x[p0], p0, pb["scale"])
    np.testing.assert_allclose(g, grad(x), atol=1e-9, rtol=0)
    np.testing.assert_allclose(H, H.T, atol=1e-9, rtol=0)
    h = 1e-5
    for mu in range(0, P, 3):
        d = np.zeros(P)
        d[mu] = h
        fd = (grad(x + d) - grad(x - d)) / (2 * h)
        np.testing.assert_allclose(H[mu], fd, atol=2e-6, rtol=0)
    eng.close()


def test_device_resident_graph_path_matches_host_path():
    """aegpu_gradient_dev (one captured CUDA graph per evaluation, inputs in HBM)
    gives bit-identical results to the host-buffer path, call after call."""
    torch = pytest.importorskip("torch")
    pb = synthetic_problem(8, 4, 4, 2, 0)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    eng = ae.Engine(16, ae.BASIS_SZ, 8, 4, 4, ops0)
    init = np.zeros(eng.D)
    init[np.searchsorted(eng.states(), pb["hf"])] = 1.0
    eng.set_initial(init)
    eng.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    rng = np.random.default_rng(9)
    for k in range(3):
        ang = rng.uniform(-0.3, 0.3, len(ops0))
        E, g = eng.gradient(ang)
        a = torch.tensor(ang, dtype=torch.float64, device="cuda")
        Ed = torch.zeros(1, dtype=torch.float64, device="cuda")
        gd = torch.zeros(len(ops0), dtype=torch.float64, device="cuda")
        eng.gradient_dev(a.data_ptr(), Ed.data_ptr(), gd.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert float(Ed.item()) == E
        assert np.array_equal(gd.cpu().numpy(), g)
    eng.close()


@pytest.mark.parametrize("N,layers,batch", [(10, 3, 1), (12, 3, 1), (8, 2, 16)])
def test_programmatic_dependent_launch_is_bit_identical(N, layers, batch):
    """With the pass kernels launched as programmatic dependents (AEGPU_TUNE_PDL) the
    host path, the captured-graph path and a batch give bit-identical energies and
    gradients to the plain launches."""
    torch = pytest.importorskip("torch")
    pb = synthetic_problem(N, N // 2, N // 2, layers, 0)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    rng = np.random.default_rng(N)
    angs = rng.uniform(-0.3, 0.3, (batch, len(ops0)))
    out = []
    for pdl in (0, 1):
        eng = ae.Engine(2 * N, ae.BASIS_SZ, N, N // 2, N // 2, ops0, tuning={ae.TUNE_PDL: pdl})
        eng.set_batch(batch)
        init = np.zeros(eng.D)
        init[np.searchsorted(eng.states(), pb["hf"])] = 1.0
        eng.set_initial(init)
        eng.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
        E, g = eng.gradient(angs.ravel())
        a = torch.tensor(angs.ravel(), dtype=torch.float64, device="cuda")
        Ed = torch.zeros(batch, dtype=torch.float64, device="cuda")
        gd = torch.zeros(batch * len(ops0), dtype=torch.float64, device="cuda")
        for _ in range(3):
            eng.gradient_dev(a.data_ptr(), Ed.data_ptr(), gd.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        out.append((np.atleast_1d(E), np.ravel(g), Ed.cpu().numpy(), gd.cpu().numpy()))
        eng.close()
    for x, y in zip(out[0], out[1]):
        assert np.array_equal(x, y)
    assert np.array_equal(out[1][0], out[1][2]) and np.array_equal(out[1][1], out[1][3])


def test_14_orbital_on_the_fly_rows_and_gradient():
    """14 orbitals, 7a+7b (11,778,624 determinants), H applied on the fly.  The oracle
    checks H x on sampled rows (a full apply would take minutes on the host); the
    analytic gradient is checked against a central difference of the energy along a
    random direction (size-independent property)."""
    from tests.fixtures import oracle_synthetic
    pb = synthetic_problem(14, 7, 7, 1, 5)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    p0 = np.asarray(pb["order_1b"]) - 1
    P = int(p0.max()) + 1
    eng = ae.Engine(28, ae.BASIS_SZ, 14, 7, 7, ops0)
    assert eng.D == 11778624
    init = np.zeros(eng.D)
    init[np.searchsorted(eng.states(), pb["hf"])] = 1.0
    eng.set_initial(init)
    eng.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_ON_THE_FLY)
    rng = np.random.default_rng(8)
    x = rng.normal(size=eng.D)
    y = eng.apply_h(x)
    o = oracle_synthetic(pb, csr=False)
    rows = np.sort(rng.choice(eng.D, 64, replace=False))
    np.testing.assert_allclose(y[rows], o.apply_h_rows(x, rows), atol=1e-11, rtol=1e-12)
    th = rng.uniform(-0.2, 0.2, P)
    E, gops = eng.gradient(pb["scale"] * th[p0])
    g = np.zeros(P)
    np.add.at(g, p0, pb["scale"] * gops)
    d = rng.normal(size=P)
    d /= np.linalg.norm(d)
    h = 1e-4
    Ep = eng.energy(pb["scale"] * (th + h * d)[p0])
    Em = eng.energy(pb["scale"] * (th - h * d)[p0])
    assert abs((Ep - Em) / (2 * h) - g @ d) < 1e-7 * max(1.0, abs(g @ d))
    eng.close()


def test_fp64_work_and_peak_probe():
    """The FP64 work model counts one DFMA per stored element (the stored H's
    nonzeros) and the DFMA probe reports a plausible GB300 rate."""
    pb = synthetic_problem(8, 4, 4, 2, 0)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    eng = ae.Engine(16, ae.BASIS_SZ, 8, 4, 4, ops0)
    eng.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    w = eng.fp64_work()
    info = eng.info()
    assert w[0] == info["nnz"] + info["D"]
    assert w[1] > info["active"] and w[2] > 2 * (w[1] - info["active"])
    t = ae.fp64_peak()
    assert 0.2 < t < 20.0, t
    eng.close()


def test_hessian_12_orbitals_directional_derivative():
    """Config-2 size (12 orbitals, 853,776 determinants, 99 parameters, stored H): the
    analytic Hessian is symmetric and H d equals the central difference of the analytic
    gradient along a random direction d (size-independent property)."""
    pb = synthetic_problem(12, 6, 6, 3, 0)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    p0 = np.asarray(pb["order_1b"]) - 1
    P = int(p0.max()) + 1
    eng = ae.Engine(24, ae.BASIS_SZ, 12, 6, 6, ops0)
    init = np.zeros(eng.D)
    init[np.searchsorted(eng.states(), pb["hf"])] = 1.0
    eng.set_initial(init)
    eng.set_ham_integrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    rng = np.random.default_rng(12)
    x = rng.uniform(-0.1, 0.1, P)

    def grad(xx):
        _, go = eng.gradient(pb["scale"] * xx[p0])
        g = np.zeros(P)
        np.add.at(g, p0, pb["scale"] * go)
        return g

    E, g, H = eng.hessian(pb["scale"] * x[p0], p0, pb["scale"])
    np.testing.assert_allclose(g, grad(x), atol=1e-9, rtol=0)
    np.testing.assert_allclose(H, H.T, atol=1e-9, rtol=0)
    d = rng.normal(size=P)
    d /= np.linalg.norm(d)
    h = 1e-5
    fd = (grad(x + h * d) - grad(x - h * d)) / (2 * h)
    np.testing.assert_allclose(H @ d, fd, atol=5e-6, rtol=0)
    eng.close()


@pytest.mark.parametrize("name", ["h4", "h4c", "syn8"])
def test_get_expectation_values_batched(golden, name):
    """getExpectationValues evaluates its rows as one batch (evolveMultiple +
    getEnergies): bit-identical to the row-by-row energies, compressed or per-operator
    rows, and the manager keeps working with a batch of one afterwards (Hessian)."""
    fx = golden(name)
    if name.startswith("syn"):
        N = int(fx["N"])
        pb = synthetic_problem(N, int(fx["na"]), int(fx["nb"]), int(fx["layers"]), int(fx["seed"]))
        m = ae.stateAnsatzManager()
        assert m.storeInitial(2 * N, [int(fx["hf"])], [1.0])
        assert m.storeOperators(np.asarray(fx["ops_1b"]).tolist())
        assert m.storeParameterDependencies(list(zip(np.asarray(fx["order_1b"]) - 1, fx["scale"])))
        assert m.storeIntegrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    else:
        m = manager_from_fixture(fx)
    P = int(np.asarray(fx["order_1b"]).max())
    rows = np.random.default_rng(2).uniform(-0.5, 0.5, (7, P))
    single = np.array([m.getExpectationValue(r) for r in rows])
    batch = m.getExpectationValues(rows)
    assert np.array_equal(batch, single)
    p0, sc = np.asarray(fx["order_1b"]) - 1, np.asarray(fx["scale"])
    ops_rows = sc * rows[:, p0]
    assert np.array_equal(m.getExpectationValues(ops_rows), single)
    H = m.getHessianComp(np.asarray(fx["angles"][0])[:P])
    if "H" in fx:
        np.testing.assert_allclose(H, fx["H"][0], atol=TOL_G, rtol=0)
    assert abs(m.getExpectationValue(np.asarray(fx["angles"][0])[:P]) - fx["E"][0]) < TOL_E


@pytest.mark.parametrize("name", ["h4", "h4c"])
def test_python_binding_current_angles_and_per_operator_derivatives(golden, name):
    """The reference binding's surface (PyAnsatzEvolve.cpp:17-96): setAngles / getAngles,
    getters without angles evaluate at the current angles, getGradient / getHessian per
    operator (compressing them gives the reference's compressed values), compressed
    getters accept per-operator angles, optimise() starts from the current angles."""
    fx = golden(name)
    m = manager_from_fixture(fx)
    P = int(np.asarray(fx["order_1b"]).max())
    p0, sc = np.asarray(fx["order_1b"]) - 1, np.asarray(fx["scale"])
    x = np.asarray(fx["angles"][1])[:P]
    assert m.setAngles(x)
    assert np.array_equal(m.getAngles(), x)
    E = m.getExpectationValue()
    assert abs(E - fx["E"][1]) < TOL_E and E == m.getExpectationValue(x)
    np.testing.assert_allclose(m.getGradientComp(), fx["G"][1], atol=TOL_G, rtol=0)
    np.testing.assert_allclose(m.getHessianComp(), fx["H"][1], atol=TOL_G, rtol=0)
    C = np.zeros((P, len(p0)))
    C[p0, np.arange(len(p0))] = sc
    g_ops, H_ops = m.getGradient(), m.getHessian()
    np.testing.assert_allclose(C @ g_ops, fx["G"][1], atol=TOL_G, rtol=0)
    np.testing.assert_allclose(C @ H_ops @ C.T, fx["H"][1], atol=TOL_G, rtol=0)
    np.testing.assert_allclose(H_ops, H_ops.T, atol=1e-12, rtol=0)
    # per-operator angles (the decompressed x) through the compressed getters
    th = sc * x[p0]
    np.testing.assert_allclose(m.getGradientComp(th), fx["G"][1], atol=TOL_G, rtol=0)
    np.testing.assert_allclose(m.getHessianComp(th), fx["H"][1], atol=TOL_G, rtol=0)
    # a parameter whose operators all have scale 0 cannot be recovered (its angle reads 0,
    # like the reference's normalised compression)
    recoverable = np.zeros(P, dtype=bool)
    recoverable[p0[sc != 0]] = True
    np.testing.assert_allclose(m.getAngles(), np.where(recoverable, x, 0.0), atol=1e-15, rtol=0)
    s = m.getFinalState(complex_state=name == "h4c")
    want = fx["S"][1] if name != "h4c" else fx["S"][1][0::2] + 1j * fx["S"][1][1::2]
    np.testing.assert_allclose(s, want, atol=TOL_S, rtol=0)
    if name == "h4":
        m.setAngles(np.asarray(fx["angles"][2])[:P])
        Eopt, xopt = m.optimise()
        assert abs(Eopt - float(fx["nuclear"]) - (-2.838345804245581)) < 1e-8
        assert np.array_equal(m.getAngles(), xopt)


@pytest.mark.parametrize("cplx", [False, True])
def test_coded_and_uncoded_stored_rows_agree(cplx, monkeypatch):
    """The two stored row formats (coded doubles with a value table, and uncoded rows,
    AEGPU_CODED_ROWS=0) give the same H x, energy, gradient and Hessian up to summation
    order, real and complex."""
    from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals, tups_operators
    N, na = 8, 4
    ops, param, scale = tups_operators(N, 2)
    h1, g2 = synthetic_integrals(N, 5)
    ang = np.random.default_rng(6).uniform(-0.3, 0.3, len(ops))
    out = []
    for coded in ("1", "0"):
        monkeypatch.setenv("AEGPU_CODED_ROWS", coded)
        e = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops - 1, complex_mode=cplx)
        W = 2 if cplx else 1
        init = np.zeros(e.D * W)
        init[W * np.searchsorted(e.states(), hartree_fock_index(N, na, na))] = 1.0
        e.set_initial(init)
        e.set_ham_integrals(h1, g2, ae.HAM_STORED)
        x = np.random.default_rng(7).normal(size=e.D * W)
        Hx = e.apply_h(x)
        E, g = e.gradient(ang)
        _, _, H = e.hessian(ang, param - 1, scale) if not cplx else (None, None, None)
        out.append((Hx, E, g, H))
        e.close()
    (Hx1, E1, g1, H1), (Hx0, E0, g0, H0) = out
    np.testing.assert_allclose(Hx1, Hx0, atol=1e-11, rtol=0)
    assert abs(E1 - E0) < 1e-12
    np.testing.assert_allclose(g1, g0, atol=1e-12, rtol=0)
    if H1 is not None:
        np.testing.assert_allclose(H1, H0, atol=1e-11, rtol=0)
