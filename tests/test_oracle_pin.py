"""Pins the C restatement (oracle/oracle.c) against the reference's own outputs.

The fixtures in tests/golden/ were produced by the reference built from source
(oracle/build_ref.sh + tests/golden/make_golden.py); the known answers printed by
the reference's Fortran binding test (src/test.F90:70-109) and the H4 L1 minimum of
Benchmarks.md:13 are checked as well.  CPU only.
"""
import numpy as np
import pytest

from tests.fixtures import oracle_from_golden, synthetic_problem, oracle_synthetic
from oracle.oracle import exc_apply


def _sector_state(o, full, cplx=False):
    st = o.states()
    if cplx:
        full = np.asarray(full).reshape(-1, 2)
        return full[st].reshape(-1)
    return np.asarray(full)[st]


@pytest.mark.parametrize("name,cplx", [("f90", False), ("ferm", False), ("h4", False), ("h4c", True)])
def test_oracle_matches_reference_fixture(golden, name, cplx):
    fx = golden(name)
    o = oracle_from_golden(fx, cplx)
    nuc = float(fx.get("nuclear", 0.0))
    for k, x in enumerate(fx["angles"]):
        E, g = o.gradient_comp(x)
        assert abs(E + nuc - fx["E"][k]) < 1e-10
        np.testing.assert_allclose(g, fx["G"][k], atol=1e-9, rtol=0)
        H = o.hessian_comp(x)
        np.testing.assert_allclose(H, fx["H"][k], atol=1e-9, rtol=0)
        ang = np.zeros(o.nops)
        scale = np.asarray(fx["scale"])
        param = np.asarray(fx["order_1b"]) - 1
        ang = scale * np.asarray(x)[param]
        psi = o.evolve_ops(ang)
        np.testing.assert_allclose(psi, _sector_state(o, fx["S"][k], cplx), atol=1e-12, rtol=0)


def test_fortran_known_answers(golden):
    fx = golden("f90")
    o = oracle_from_golden(fx)
    E0, g0 = o.gradient_comp(np.zeros(9))
    Em, gm = o.gradient_comp(fx["angles"][1])
    assert abs(E0 - (-2.2506796656654822)) < 1e-12
    assert abs(np.linalg.norm(g0) - 0.56168441173471617) < 1e-12
    assert abs(Em - (-2.844887240192931)) < 1e-12
    assert np.linalg.norm(gm) < 1e-10
    np.testing.assert_allclose(fx["known_E"][:2], [-2.2506796656654822, -2.844887240192931])


def test_h4_benchmark_minimum(golden):
    fx = golden("h4")
    # Benchmarks.md:13 quotes the electronic minimum; the manager adds the nuclear energy
    assert abs(fx["opt_E"] - float(fx["nuclear"]) - (-2.838345804245581)) < 1e-9
    o = oracle_from_golden(fx)
    E, g = o.gradient_comp(fx["opt_angles"])
    assert abs(E + float(fx["nuclear"]) - fx["opt_E"]) < 1e-10
    assert np.linalg.norm(g) < 1e-6


@pytest.mark.parametrize("name", ["f90", "syn6"])
def test_excitation_rule_bit_exact(golden, name):
    fx = golden(name)
    ops0 = np.asarray(fx["ops_1b"]) - 1
    partner, sign = fx["pair_partner"], fx["pair_sign"]
    n = partner.shape[1]
    step = 1 if n <= 256 else 7
    for e in range(len(ops0)):
        for s in range(0, n, step):
            k, p, sg = exc_apply(s, ops0[e])
            if k == 1:
                assert p == partner[e, s] and sg == sign[e, s]
            elif k == 0:
                # the reference returns the state itself, sign false, for inactive states
                assert partner[e, s] == s


def test_synthetic_tups_matches_reference(golden):
    fx = golden("syn8")
    pb = synthetic_problem(int(fx["N"]), int(fx["na"]), int(fx["nb"]), int(fx["layers"]), int(fx["seed"]))
    np.testing.assert_array_equal(pb["ops_1b"], fx["ops_1b"])
    for csr in (True, False):
        o = oracle_synthetic(pb, csr=csr)
        st = o.states()
        np.testing.assert_array_equal(st, fx["sector"])
        for k, x in enumerate(fx["angles"]):
            E, g = o.gradient_comp(x)
            assert abs(E - fx["E"][k]) < 1e-10
            np.testing.assert_allclose(g, fx["G"][k], atol=1e-9, rtol=0)
            psi = o.evolve_ops(pb["scale"] * np.asarray(x)[np.asarray(pb["order_1b"]) - 1])
            np.testing.assert_allclose(psi, fx["S_sector"][k], atol=1e-12, rtol=0)
    o = oracle_synthetic(pb, csr=True)
    H = o.hessian_comp(fx["angles"][0])
    np.testing.assert_allclose(H, fx["H"][0], atol=1e-9, rtol=0)


def test_projected_gradient_is_the_derivative_of_the_overlap():
    """The oracle's projected sweep (evolveDerivativeProj) against central differences
    of <proj|psi(theta)>, real and complex."""
    pb = synthetic_problem(6, 3, 3, 2, 4)
    o = oracle_synthetic(pb)
    rng = np.random.default_rng(3)
    ang = rng.uniform(-0.4, 0.4, o.nops)
    proj = rng.normal(size=o.D)
    ov, g = o.gradient_proj_ops(ang, proj)
    assert abs(ov - proj @ o.evolve_ops(ang)) < 1e-13
    h = 1e-6
    for k in range(0, o.nops, 5):
        d = np.zeros(o.nops)
        d[k] = h
        fd = (proj @ o.evolve_ops(ang + d) - proj @ o.evolve_ops(ang - d)) / (2 * h)
        assert abs(fd - g[k]) < 1e-8


@pytest.mark.parametrize("name", ["ref10", "ref12"])
def test_oracle_matches_reference_at_benchmark_sizes(golden, name):
    """The benchmark's own 10- and 12-orbital inputs: the oracle's energy, gradient and
    sampled final-state amplitudes against the reference's (tests/golden/ref*.npz)."""
    import numpy as np
    from tests.fixtures import oracle_synthetic
    fx = golden(name)
    N = int(fx["N"])
    pb = dict(N=N, nq=2 * N, na=int(fx["na"]), nb=int(fx["nb"]), hf=int(fx["hf"]), ops_1b=fx["ops_1b"],
              order_1b=fx["order_1b"], scale=fx["scale"])
    from ansatzevolve_gb300.synthetic import synthetic_integrals
    pb["h1"], pb["g2"] = synthetic_integrals(N, int(fx["seed"]))
    o = oracle_synthetic(pb, csr=False)
    E, g = o.gradient_comp(fx["x"])
    assert abs(E - float(fx["E"])) < 1e-10
    np.testing.assert_allclose(g, fx["G"], atol=1e-9, rtol=0)
    p0 = np.asarray(fx["order_1b"]) - 1
    psi = o.evolve_ops(np.asarray(fx["scale"]) * np.asarray(fx["x"])[p0])
    np.testing.assert_allclose(psi[fx["sample_rank"]], fx["sample_amp"], atol=1e-12, rtol=0)
    assert abs(np.dot(psi, psi) - float(fx["norm"])) < 1e-12


def props_inputs(golden, tag):
    """(oracle, compressed paths incl. the zero path, param0, scale, nuclear, fixture)."""
    px = golden(tag)
    base = str(px["base"])
    fx = golden(base)
    if base.startswith("syn"):
        pb = synthetic_problem(int(fx["N"]), int(fx["na"]), int(fx["nb"]), int(fx["layers"]), int(fx["seed"]))
        o, nuclear = oracle_synthetic(pb), 0.0
    else:
        o, nuclear = oracle_from_golden(fx, cplx=base == "h4c"), float(fx["nuclear"])
    p0 = np.asarray(fx["order_1b"]) - 1
    paths = [np.zeros(int(p0.max()) + 1)] + list(px["sets"])
    return o, paths, p0, np.asarray(fx["scale"]), nuclear, px


@pytest.mark.parametrize("tag", ["props_h4", "props_h4c", "props_syn6"])
def test_properties_restatement_matches_reference(golden, tag):
    """The numpy restatement of writeProperties / doSubspaceDiagonalisation
    (oracle/properties_ref.py) reproduces the reference's own table, Hessians, metrics
    (here by finite differences) and subspace eigenvalues."""
    from oracle.properties_ref import decompress, lowest_eigenpair, path_row, subspace_eigenvalues
    o, paths, p0, scale, nuclear, px = props_inputs(golden, tag)
    lam, v0 = lowest_eigenpair(o)
    v0 = v0.astype(complex)
    ours = []
    for k, x in enumerate(paths):
        row, H, M = path_row(o, x, p0, scale, nuclear, v0)
        ref = px["rows"][:, k]
        np.testing.assert_allclose(row[:3], ref[:3], atol=1e-10, rtol=0)
        assert np.array_equal(row[3:12], ref[3:12]), (k, row[3:12], ref[3:12])
        assert abs(row[12] - ref[12]) < 1e-9
        assert abs(row[15] - ref[14]) < 1e-9
        np.testing.assert_allclose(H, px["hess"][k], atol=1e-9, rtol=0)
        np.testing.assert_allclose(M, px["metric"][k], atol=1e-7, rtol=0)
        ours.append(row[13] + 1j * row[14])
    # the eigenvector's phase is arbitrary: one phase for all paths
    ours, ref = np.array(ours), px["overlap"]
    ph = ours[0] / ref[0]
    ph /= abs(ph)
    np.testing.assert_allclose(ours, ph * ref, atol=1e-9, rtol=0)
    eigs, null = subspace_eigenvalues(o, [decompress(x, p0, scale) for x in px["sets"]])
    np.testing.assert_allclose(eigs, px["subspace_eigs"], atol=1e-12, rtol=0)
    assert null == int(px["subspace_null_rank"])
