"""The reference's run files end to end on the GPU: every golden fixture's inputs
written in the reference's formats (Initial / Operators / Order / Parameters /
Nuclear_Energy files plus integrals or a sparse Hamiltonian), set up with setRunFiles
(the command-line driver's loading, main.cpp:235-386) and evaluated through the C
ABI against the reference's outputs; and the driver's `optimise` verb on the H4 L1
inputs, which starts from the Parameters file's first set and reaches the minimum of
Benchmarks.md:13 (electronic energy -2.838345804245581)."""
import os

import numpy as np
import pytest

import ansatzevolve_gb300 as ae
from ansatzevolve_gb300.runfiles import load_run_files, optimise_run, write_run_files

pytestmark = pytest.mark.gpu
TOL_E, TOL_G = 1e-10, 1e-9


def write_fixture(prefix, fx, sets):
    coeff = np.asarray(fx["init_re"]) + 1j * np.asarray(fx.get("init_im", 0.0))
    kw = dict(nq=int(fx["nq"]), initial_index=fx["init_idx"], initial_coeff=coeff, operators_1b=fx["ops_1b"],
              order0=np.asarray(fx["order_1b"]) - 1, scale=fx["scale"], parameter_sets=sets,
              energies=np.zeros(len(sets)))
    if float(fx.get("nuclear", 0.0)) != 0.0:
        kw["nuclear_energy"] = float(fx["nuclear"])
    if "h1" in fx:
        kw.update(h1=fx["h1"], g2=fx["g2"])
    else:
        kw["ham_triplets"] = (np.asarray(fx["ham_i_1b"]) - 1, np.asarray(fx["ham_j_1b"]) - 1, fx["ham_v"])
    write_run_files(prefix, **kw)


@pytest.mark.parametrize("name", ["f90", "ferm", "h4", "h4c"])
def test_set_run_files_matches_reference_fixture(golden, tmp_path, name):
    fx = golden(name)
    prefix = str(tmp_path / name)
    write_fixture(prefix, fx, fx["angles"])
    m = ae.stateAnsatzManager()
    rf = m.storeRunFiles(prefix)
    assert len(rf.parameter_sets) == len(fx["angles"])
    for k, x in enumerate(rf.parameter_sets):
        assert abs(m.getExpectationValue(x) - fx["E"][k]) < TOL_E, (name, k)
        np.testing.assert_allclose(m.getGradientComp(x), fx["G"][k], atol=TOL_G, rtol=0)
    m.close()


def test_optimise_verb_reaches_the_h4_minimum(golden, tmp_path):
    fx = golden("h4")
    prefix = str(tmp_path / "H4")
    # the reference's H4 L1 Parameters file: the seed set first, then the minimum
    write_fixture(prefix, fx, [fx["angles"][2], fx["angles"][0]])
    out = str(tmp_path / "opt_Parameters.dat")
    E, x, rf = optimise_run(prefix, out=out)
    assert rf.nuclear_energy == float(fx["nuclear"])
    assert abs(E - rf.nuclear_energy - (-2.838345804245581)) < 1e-8
    assert abs(E - float(fx["opt_E"])) < 1e-8
    # the written set is read back by the same readers and evaluates to the same energy
    os.replace(out, prefix + "_Parameters.dat")
    m = ae.stateAnsatzManager()
    rf2 = m.storeRunFiles(prefix)
    assert np.array_equal(rf2.parameter_sets[0], x)
    assert rf2.energies[0] == E
    assert abs(m.getExpectationValue(rf2.parameter_sets[0]) - E) < 1e-12
    assert np.linalg.norm(m.getGradientComp(rf2.parameter_sets[0])) < 1e-6
    m.close()
    assert load_run_files(prefix).n_params == len(x)


def test_iterative_optimise_verb(golden, tmp_path):
    """The driver's iterativeOptimise verb on the H4 L1 run files: the projected
    iteration then Newton from the Parameters file's first set ends at a stationary
    point whose energy is the engine's at the returned angles."""
    from ansatzevolve_gb300.runfiles import iterative_optimise_run
    fx = golden("h4")
    prefix = str(tmp_path / "H4")
    write_fixture(prefix, fx, [fx["angles"][2], fx["angles"][0]])
    E, x, rf = iterative_optimise_run(prefix)
    m = ae.stateAnsatzManager()
    m.storeRunFiles(prefix)
    assert abs(m.getExpectationValue(x) - E) < 1e-12
    assert np.linalg.norm(m.getGradientComp(x)) < 1e-6
    m.close()
