"""The properties entry points on the GPU (aegpu_lowest_eigenpair, aegpu_ground_overlap,
aegpu_hessian_metric, aegpu_path_properties, aegpu_subspace_eigenvalues) against the
reference's own writeProperties / doSubspaceDiagonalisation output
(tests/golden/props_*.npz) and, at sizes without a reference fixture, against the
oracle: the lowest eigenvalue of the oracle's Hamiltonian, the metric by central
differences of the oracle's states, and the variational bound at 12 orbitals."""
import time

import numpy as np
import pytest

import ansatzevolve_gb300 as ae
from tests.fixtures import oracle_synthetic, sector_of, synthetic_problem

pytestmark = pytest.mark.gpu


def engine_for(golden, tag):
    px = golden(tag)
    base = str(px["base"])
    fx = golden(base)
    if base.startswith("syn"):
        pb = synthetic_problem(int(fx["N"]), int(fx["na"]), int(fx["nb"]), int(fx["layers"]), int(fx["seed"]))
        nq, init_idx, init_c = pb["nq"], [pb["hf"]], np.array([1.0])
        h1, g2, nuclear = pb["h1"], pb["g2"], 0.0
    else:
        nq, init_idx = int(fx["nq"]), np.asarray(fx["init_idx"])
        init_c = np.asarray(fx["init_re"]) + 1j * np.asarray(fx.get("init_im", np.zeros(len(init_idx))))
        h1, g2, nuclear = fx["h1"], fx["g2"], float(fx["nuclear"])
    ops0 = np.asarray(fx["ops_1b"]) - 1
    kind, ne, na, nbe = sector_of(nq, init_idx, ops0)
    cplx = base == "h4c"
    e = ae.Engine(nq, kind, ne, na, nbe, ops0, complex_mode=cplx)
    pos = np.searchsorted(e.states(), init_idx)
    if cplx:
        init = np.zeros(2 * e.D)
        init[2 * pos], init[2 * pos + 1] = init_c.real, init_c.imag
    else:
        init = np.zeros(e.D)
        init[pos] = init_c.real
    e.set_initial(init)
    e.set_ham_integrals(h1, g2, ae.HAM_STORED)
    p0 = np.asarray(fx["order_1b"]) - 1
    paths = [np.zeros(int(p0.max()) + 1)] + list(px["sets"])
    return e, paths, p0, np.asarray(fx["scale"]), nuclear, px


@pytest.mark.parametrize("tag", ["props_h4", "props_h4c", "props_syn6"])
def test_properties_match_reference(golden, tag):
    e, paths, p0, scale, nuclear, px = engine_for(golden, tag)
    lam, res, nprod = e.lowest_eigenpair(tol=1e-11)
    assert res < 1e-10 and nprod >= 2
    ours = []
    for k, x in enumerate(paths):
        row, H, M = e.path_properties(scale * x[p0], p0, scale, nuclear, hessian=True, overlap=True)
        ref = px["rows"][:, k]
        np.testing.assert_allclose(row[:3], ref[:3], atol=1e-10, rtol=0)
        assert np.array_equal(row[3:12], ref[3:12]), (k, row[3:12], ref[3:12])
        assert abs(row[12] - ref[12]) < 1e-9
        assert abs(row[15] - ref[14]) < 1e-9
        np.testing.assert_allclose(H, px["hess"][k], atol=1e-9, rtol=0)
        np.testing.assert_allclose(M, px["metric"][k], atol=1e-9, rtol=0)
        ours.append(row[13] + 1j * row[14])
    ours, ref = np.array(ours), px["overlap"]
    # the reference's eigenvector has an arbitrary phase; ours has <start|v> >= 0
    assert ours[0].real >= 0 and abs(ours[0].imag) < 1e-12
    ph = ours[0] / ref[0]
    ph /= abs(ph)
    np.testing.assert_allclose(ours, ph * ref, atol=1e-9, rtol=0)
    w, null = e.subspace_eigenvalues([scale * x[p0] for x in px["sets"]])
    np.testing.assert_allclose(w, px["subspace_eigs"], atol=1e-10, rtol=0)
    assert null == int(px["subspace_null_rank"])
    e.close()


def test_lanczos_restarts_reach_the_same_eigenpair(golden):
    """A basis of 4 vectors forces many explicit restarts; the eigenvalue and the
    eigenvector agree with the unrestarted run."""
    e, paths, p0, scale, nuclear, px = engine_for(golden, "props_syn6")
    lam, res, _ = e.lowest_eigenpair(tol=1e-11)
    v = e.ground_state()
    lam4, res4, n4 = e.lowest_eigenpair(tol=1e-9, basis=4, max_products=20000)
    assert res4 < 1e-9 and n4 > 4
    assert abs(lam4 - lam) < 1e-12 * max(1.0, abs(lam)) + 1e-15
    assert abs(abs(np.vdot(v, e.ground_state())) - 1.0) < 1e-12
    e.close()


def _synthetic_engine(N, mode, layers=2, seed=0):
    pb = synthetic_problem(N, N // 2, N // 2, layers, seed)
    ops0 = np.asarray(pb["ops_1b"]) - 1
    e = ae.Engine(2 * N, ae.BASIS_SZ, N, N // 2, N // 2, ops0)
    init = np.zeros(e.D)
    init[np.searchsorted(e.states(), [pb["hf"]])] = 1.0
    e.set_initial(init)
    e.set_ham_integrals(pb["h1"], pb["g2"], mode)
    return e, pb


@pytest.mark.parametrize("mode", [ae.HAM_STORED, ae.HAM_ON_THE_FLY])
def test_lowest_eigenpair_8_orbitals_vs_oracle(mode):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    e, pb = _synthetic_engine(8, mode)
    lam, res, nprod = e.lowest_eigenpair(tol=1e-10)
    o = oracle_synthetic(pb)
    rp, col, val = o.csr()
    Hs = sp.csr_matrix((val, col, rp), shape=(o.D, o.D))
    w, V = sla.eigsh(Hs, k=2, which="SA", tol=1e-14)
    assert res < 1e-10
    assert abs(lam - w[0]) < 1e-10 * max(1.0, abs(w[0]))
    v = e.ground_state()
    gap = w[1] - w[0]
    assert abs(abs(v @ V[:, 0]) - 1.0) < max(1e-12, (1e-10 / gap) ** 2 * 10)
    # the overlap entry point is <psi(theta)|v>
    x = np.random.default_rng(3).uniform(-0.3, 0.3, int(pb["order_1b"].max()))
    th = np.asarray(pb["scale"]) * x[np.asarray(pb["order_1b"]) - 1]
    ov = e.ground_overlap(th)
    assert abs(ov - o.evolve_ops(th) @ v) < 1e-12
    e.close()


def test_metric_8_orbitals_matches_finite_differences():
    from oracle.properties_ref import metric_fd
    e, pb = _synthetic_engine(8, ae.HAM_STORED)
    p0, scale = np.asarray(pb["order_1b"]) - 1, np.asarray(pb["scale"])
    x = np.random.default_rng(4).uniform(-0.4, 0.4, int(p0.max()) + 1)
    E, g, H, M = e.hessian_metric(scale * x[p0], p0, scale)
    o = oracle_synthetic(pb)
    Mfd = metric_fd(o, x, p0, scale)
    np.testing.assert_allclose(M, Mfd, atol=1e-8, rtol=0)
    np.testing.assert_allclose(M, M.T, atol=1e-14, rtol=0)
    E2, g2, H2 = e.hessian(scale * x[p0], p0, scale)
    assert E == E2 and np.array_equal(g, g2) and np.array_equal(H, H2)
    e.close()


def test_lowest_eigenpair_12_orbitals_is_a_variational_bound():
    """12 orbitals (D = 853,776), stored H: the Rayleigh quotient of the converged
    vector lies below every ansatz energy (here the HF state and the benchmark's
    angles), and its residual meets the tolerance."""
    e, pb = _synthetic_engine(12, ae.HAM_STORED, layers=3)
    t0 = time.perf_counter()
    lam, res, nprod = e.lowest_eigenpair(tol=1e-8, basis=100, max_products=3000)
    dt = time.perf_counter() - t0
    assert res <= 1e-8, (res, nprod)
    p0, scale = np.asarray(pb["order_1b"]) - 1, np.asarray(pb["scale"])
    x = np.random.default_rng(1).uniform(-0.1, 0.1, int(p0.max()) + 1)
    for th in (np.zeros(len(p0)), scale * x[p0]):
        E = e.energy(th)
        assert lam < E
        ov = e.ground_overlap(th)
        assert 0.0 < abs(ov) <= 1.0 + 1e-12
    print("12-orbital lowest eigenpair: %.12f, residual %.1e, %d products, %.2f s" % (lam, res, nprod, dt))
    e.close()


def test_writeproperties_verb_on_run_files(golden, tmp_path):
    """The reference driver's writeproperties verb through the C ABI extensions: run
    files of the H4 L1 inputs, table rows equal the reference's."""
    from ansatzevolve_gb300.runfiles import properties_run
    from tests.test_gpu_runfiles import write_fixture
    px = golden("props_h4")
    fx = golden("h4")
    prefix = str(tmp_path / "H4")
    write_fixture(prefix, fx, px["sets"])
    table, w, nr, lam, text = properties_run(prefix)
    rows = np.array([table[n] for n in ae.PROPERTY_NAMES])
    np.testing.assert_allclose(rows[:3], px["rows"][:3], atol=1e-10, rtol=0)
    assert np.array_equal(rows[3:12], px["rows"][3:12])
    np.testing.assert_allclose(rows[12], px["rows"][12], atol=1e-9, rtol=0)
    np.testing.assert_allclose(rows[15], px["rows"][14], atol=1e-9, rtol=0)
    np.testing.assert_allclose(w, px["subspace_eigs"], atol=1e-10, rtol=0)
    assert nr == int(px["subspace_null_rank"])
    assert "Elec. Energy" in text and "MagOfOverlapWithState_0" in text
    assert lam < rows[0].min()


def test_writeproperties_verb_complex_and_extracted_min(golden, tmp_path):
    """The writeproperties verb on the complex H4 inputs (diagonal phase operators),
    with the angle sets read from an extractedmin file instead of the Parameters file:
    rows equal the reference's for the same sets."""
    from ansatzevolve_gb300.runfiles import properties_run, write_extracted_min
    from tests.test_gpu_runfiles import write_fixture
    px = golden("props_h4c")
    fx = golden("h4c")
    prefix = str(tmp_path / "H4c")
    P = int(np.asarray(fx["order_1b"]).max())
    write_fixture(prefix, fx, [np.zeros(P)])  # Parameters: one set, P angles (sizes extractedmin)
    write_extracted_min(prefix + "_extractedmin", px["sets"])
    table, w, nr, lam, text = properties_run(prefix, extracted_min=True)
    rows = np.array([table[n] for n in ae.PROPERTY_NAMES])
    np.testing.assert_allclose(rows[:3], px["rows"][:3], atol=1e-10, rtol=0)
    assert np.array_equal(rows[3:12], px["rows"][3:12])
    np.testing.assert_allclose(rows[15], px["rows"][14], atol=1e-9, rtol=0)
    np.testing.assert_allclose(w, px["subspace_eigs"], atol=1e-10, rtol=0)
    assert nr == int(px["subspace_null_rank"])


def test_generate_paths_for_subspace(golden):
    """generatePathsForSubspace: distinct Newton minima from the seeded random starts
    and the subspace diagonalisation over them.  H4 L1 has one minimum reachable from
    them (one path: the subspace eigenvalue is that energy; asking for more fails
    cleanly after the bounded number of starts); on the 6-orbital synthetic inputs three
    are found, and the lowest subspace eigenvalue lies between H's lowest eigenvalue and
    the lowest minimum.  The call is repeatable (seeded)."""
    from tests.test_gpu_parity import manager_from_fixture
    fx = golden("h4")
    m = manager_from_fixture(fx)
    w, nr, E = m.generatePathsForSubspace(1)
    assert abs(w[0] - (E[0] - float(fx["nuclear"]))) < 1e-10 and nr == 0
    with pytest.raises(ae.AegpuError):
        m.generatePathsForSubspace(2)
    m.close()
    fx = golden("syn6")
    N = int(fx["N"])
    pb = synthetic_problem(N, int(fx["na"]), int(fx["nb"]), int(fx["layers"]), int(fx["seed"]))
    m = ae.stateAnsatzManager()
    assert m.storeInitial(2 * N, [int(fx["hf"])], [1.0])
    assert m.storeOperators(np.asarray(fx["ops_1b"]).tolist())
    assert m.storeParameterDependencies(list(zip(np.asarray(fx["order_1b"]) - 1, fx["scale"])))
    assert m.storeIntegrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    w, nr, E = m.generatePathsForSubspace(3)
    assert len(set(np.round(E, 9))) == 3
    lam, res = m.getLowestEigenvalue()
    assert lam - 1e-9 <= w[0] <= E.min() + 1e-9
    assert np.all(np.diff(w) >= -1e-12)
    w2, nr2, E2 = m.generatePathsForSubspace(3)
    np.testing.assert_allclose(w2, w, atol=1e-9, rtol=0)
    np.testing.assert_allclose(E2, E, atol=1e-9, rtol=0)
    m.close()


@pytest.mark.parametrize("name", ["h4", "h4c"])
def test_writeproperties_files(golden, tmp_path, capfd, name):
    """writeProperties' files next to the run files, in the reference's formats: per
    path the Hessian (.Matbin) and the metric (.Matbin, or .CMatbin for complex runs),
    and the ground-state overlap magnitudes (.Vecbin), equal to the reference's own; its
    table goes to stdout."""
    from ansatzevolve_gb300.runfiles import properties_run
    from tests.test_gpu_runfiles import write_fixture
    px = golden("props_" + name)
    fx = golden(name)
    prefix = str(tmp_path / "H4")
    write_fixture(prefix, fx, px["sets"])
    properties_run(prefix, write_files=True)
    assert "Results:" in capfd.readouterr().out
    P = int(np.asarray(fx["order_1b"]).max())
    for k in range(len(px["sets"]) + 1):
        H = np.fromfile("%s_Path_%d_Hessian.Matbin" % (prefix, k)).reshape(P, P)
        np.testing.assert_allclose(H, px["hess"][k], atol=1e-9, rtol=0)
        if name == "h4c":
            M = np.fromfile("%s_Path_%d_Metric.CMatbin" % (prefix, k)).reshape(P, P, 2)[..., 0]
        else:
            M = np.fromfile("%s_Path_%d_Metric.Matbin" % (prefix, k)).reshape(P, P)
        np.testing.assert_allclose(M, px["metric"][k], atol=1e-9, rtol=0)
    mag = np.fromfile(prefix + "_MagOfOverlapWithGroundState_0.Vecbin")
    np.testing.assert_allclose(mag, px["rows"][14], atol=1e-9, rtol=0)
    assert open(prefix + "_MagOfOverlapWithGroundState_0.ColVeccsv").read().count("\n") == len(mag)


@pytest.mark.parametrize("tag", ["overlaps_syn6", "overlaps_h4c"])
def test_overlaps_with_several_eigenstates_match_reference(golden, tag):
    """The overlaps of every path with the k lowest eigenstates of H (the reference's
    numberOfOverlapsToCompute, from its dense eigensolver): magnitudes at 1e-9, values up
    to one sign per eigenstate (the eigensolvers choose signs independently).  States of
    another spin symmetry than the paths (zero overlap) must appear in their place in the
    spectrum, so the Lanczos has to find them too."""
    e, paths, p0, scale, nuclear, px = engine_for(golden, tag)
    k = int(px["k"])
    lam, res, nprod = e.lowest_eigenpairs(k, tol=1e-11, basis=200)
    assert np.all(res < 1e-10), res
    assert np.all(np.diff(lam) > 1e-8)
    got = np.array([e.ground_overlaps(scale * x[p0], k) for x in paths]).T  # [state][path]
    np.testing.assert_allclose(np.abs(got), px["mag"], atol=1e-9, rtol=0)
    for i in range(k):
        ref = px["overlap"][i]
        j = int(np.argmax(np.abs(ref)))
        if abs(ref[j]) < 1e-8:
            continue
        sgn = np.sign((ref[j] / got[i][j]).real)
        np.testing.assert_allclose(sgn * got[i], ref, atol=1e-9, rtol=0)
    # the single-state entry point afterwards still gives the lowest eigenpair
    lam1, res1, _ = e.lowest_eigenpair(tol=1e-11)
    assert abs(lam1 - lam[0]) < 1e-9 or abs(px["mag"][0]).max() < 1e-8
    e.close()


def test_writeproperties_number_of_overlaps(golden, tmp_path, capfd):
    """The manager's writeProperties with setNumberOfOverlapsToCompute(4): one
    OverlapWithState_i / MagOfOverlapWithState_i row pair and one
    _MagOfOverlapWithGroundState_i file per state, equal to the reference's."""
    px = golden("overlaps_syn6")
    fx = golden("syn6")
    pb = synthetic_problem(int(fx["N"]), int(fx["na"]), int(fx["nb"]), int(fx["layers"]), int(fx["seed"]))
    m = ae.stateAnsatzManager()
    assert m.storeInitial(pb["nq"], [pb["hf"]], [1.0])
    assert m.storeOperators(np.asarray(fx["ops_1b"]).tolist())
    assert m.storeParameterDependencies(list(zip(np.asarray(fx["order_1b"]) - 1, fx["scale"])))
    assert m.storeIntegrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    assert m.setNumberOfOverlapsToCompute(4)
    P = int(np.asarray(fx["order_1b"]).max())
    paths = np.vstack([np.zeros(P)] + list(px["sets"]))
    prefix = str(tmp_path / "syn6")
    m.writeProperties(paths, runPath=prefix, hessian=False)
    out = capfd.readouterr().out
    for i in range(4):
        assert "OverlapWithState_%d " % i in out and "MagOfOverlapWithState_%d " % i in out
        mag = np.fromfile("%s_MagOfOverlapWithGroundState_%d.Vecbin" % (prefix, i))
        np.testing.assert_allclose(mag, px["mag"][i], atol=1e-9, rtol=0)
    m.close()
