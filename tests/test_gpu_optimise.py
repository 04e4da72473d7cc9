"""Optimisers over the engine: the reference's Newton method (one instance at a time,
analytic Hessian) and the lockstep batched BFGS agree on the minima they share."""
import numpy as np
import pytest

import ansatzevolve_gb300 as ae
from ansatzevolve_gb300.synthetic import family_integrals
from tests.fixtures import synthetic_problem

pytestmark = pytest.mark.gpu


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


def test_batched_bfgs_and_newton_share_minima_on_a_family():
    """Newton from zero angles finds a minimum per family member; the batched BFGS
    started from perturbed copies of those minima returns to them (same energies to
    1e-8), every instance at |g| < gtol.  Which minimum an optimiser finds from a far
    start depends on its path, so the comparison is made inside the basins."""
    pb = synthetic_problem(8, 4, 4, 2, 0)
    p0 = np.asarray(pb["order_1b"]) - 1
    scale = np.asarray(pb["scale"])
    P = int(p0.max()) + 1
    fam = [family_integrals(8, float(s), seed=7) for s in np.linspace(0.0, 1.0, 4)]
    gtol = 1e-6
    newton = []
    one = make_engine(pb)
    for h1, g2 in fam:
        one.set_ham_integrals(h1, g2, ae.HAM_STORED)
        x, E, gn, nh, ne = one.optimise_newton(np.zeros(P), p0, scale, gtol=gtol)
        assert gn < gtol and nh > 0 and ne > 0
        newton.append((x, E))
    bat = make_engine(pb, len(fam))
    bat.set_ham_integrals_batch(np.stack([f[0] for f in fam]), np.stack([f[1] for f in fam]), ae.HAM_STORED)
    rng = np.random.default_rng(3)
    x0 = np.stack([x for x, _ in newton]) + rng.uniform(-2e-3, 2e-3, (len(fam), P))
    xb, Eb, gb, it, rounds = bat.optimise_batch(x0, p0, scale, gtol=gtol)
    assert np.all(gb < gtol), gb
    assert rounds > 0 and np.all(it > 0)
    En = np.array([E for _, E in newton])
    np.testing.assert_allclose(Eb, En, atol=1e-8, rtol=0)
    # the returned energies are the engine's own at the returned angles
    np.testing.assert_allclose(bat.energy(scale * xb[:, p0]), Eb, atol=1e-12, rtol=0)
    one.close()
    bat.close()


def test_projected_iteration_reaches_a_stationary_point(golden):
    """The reference's iterativeTups on the H4 L1 fixture (integrals from the
    reference's own Hams/ inputs): it stops at a projected gradient below 1e-5, which is
    half the energy gradient at a renewed bra, so the energy gradient there is below
    2e-5, and the reported energy is the engine's energy at the returned angles; Newton
    from there stays at that energy."""
    from tests.fixtures import sector_of
    fx = golden("h4")
    nq = int(fx["nq"])
    ops0 = np.asarray(fx["ops_1b"]) - 1
    kind, ne, na, nbe = sector_of(nq, fx["init_idx"], ops0)
    p0 = np.asarray(fx["order_1b"]) - 1
    scale = np.asarray(fx["scale"])
    P = int(p0.max()) + 1
    e = ae.Engine(nq, kind, ne, na, nbe, ops0)
    init = np.zeros(e.D)
    init[np.searchsorted(e.states(), np.asarray(fx["init_idx"]))] = fx["init_re"]
    e.set_initial(init)
    e.set_ham_integrals(fx["h1"], fx["g2"], ae.HAM_STORED)
    x0 = np.asarray(fx["angles"][1])[:P]
    x, E, gp, nh, nev, outer = e.optimise_projected(x0, p0, scale, gtol=1e-5)
    assert gp < 1e-5 and nh > 0 and outer >= 1
    Ee, gops = e.gradient(scale * x[p0])
    g = np.zeros(P)
    np.add.at(g, p0, scale * gops)
    assert abs(Ee - E) < 1e-12
    assert np.linalg.norm(g) < 2.0001e-5
    xn, En, gn, _, _ = e.optimise_newton(x, p0, scale, gtol=1e-10)
    assert abs(En - E) < 1e-8
    e.close()


def _h4_engine(golden):
    from tests.fixtures import sector_of
    fx = golden("h4")
    nq = int(fx["nq"])
    ops0 = np.asarray(fx["ops_1b"]) - 1
    kind, ne, na, nbe = sector_of(nq, fx["init_idx"], ops0)
    p0 = np.asarray(fx["order_1b"]) - 1
    e = ae.Engine(nq, kind, ne, na, nbe, ops0)
    init = np.zeros(e.D)
    init[np.searchsorted(e.states(), np.asarray(fx["init_idx"]))] = fx["init_re"]
    e.set_initial(init)
    e.set_ham_integrals(fx["h1"], fx["g2"], ae.HAM_STORED)
    return e, fx, p0, np.asarray(fx["scale"])


def test_projected_iteration_with_diis(golden):
    """DIIS over the renewals (iterativeTups with doDIIS): a history of one vector
    extrapolates to the last angles (coefficient 1 up to rounding), so the run follows
    the plain iteration; EDIIS (15, the reference's setting) and Pulay DIIS runs return
    angles whose energy is the one reported."""
    e, fx, p0, scale = _h4_engine(golden)
    P = int(p0.max()) + 1
    x0 = np.asarray(fx["angles"][1])[:P]
    plain = e.optimise_projected(x0, p0, scale, gtol=1e-5)
    for ediis in (True, False):
        one = e.optimise_projected(x0, p0, scale, gtol=1e-5, diis=1, ediis=ediis)
        np.testing.assert_allclose(one[0], plain[0], atol=1e-9, rtol=0)
        assert abs(one[1] - plain[1]) < 1e-12 and one[2] < 1e-5
    for size, ediis in ((15, True), (6, False)):
        x, E, gp, nh, nev, outer = e.optimise_projected(x0, p0, scale, gtol=1e-5, max_outer=200, diis=size,
                                                         ediis=ediis)
        assert outer >= 1 and np.isfinite(gp)
        assert abs(e.energy(scale * x[p0]) - E) < 1e-12
        print("DIIS %d %s: E %.12f |g_proj| %.2e after %d renewals (plain: %d)" %
              (size, "EDIIS" if ediis else "Pulay", E, gp, outer, plain[5]))
    e.close()
