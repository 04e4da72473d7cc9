"""The run-file readers (include/aegpu_runfiles.h; TUPSLoadingUtils.cpp:10-360) and the
writers of ansatzevolve_gb300.runfiles, on the CPU:
* written files read back exactly (every format, real and complex initial states);
* the reference parser's rules: a bitstring alone has coefficient 1, a repeated
  bitstring keeps its last value, the qubit count is the longest bitstring, an order
  entry without a scale has scale 1, parameters past the file's last set are 0, a
  missing Parameters or Nuclear_Energy file is not an error;
* malformed files are refused with the file named;
* setRunFiles' status codes (setup only, no GPU work);
* where the reference checkout is present, its own Hams/ fixtures parse to the inputs
  recorded in the golden fixtures (which an independent parser extracted)."""
import ctypes
import os

import numpy as np
import pytest

from ansatzevolve_gb300 import AegpuError, lib
from ansatzevolve_gb300.runfiles import (load_run_files, write_extracted_min, write_initial, write_order,
                                         write_run_files)
from ansatzevolve_gb300.checkpoint import write_parameters

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference checkout (only its Hams/ fixtures are read; tests skip without it)
REF = os.environ.get("AE_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")


def _case(tmp_path, **kw):
    prefix = str(tmp_path / "run")
    rng = np.random.default_rng(1)
    ops = np.array([[1, 2, 0, 0], [5, 6, 0, 0], [1, 5, 2, 6], [3, 4, 0, 0], [7, 8, 0, 0]])
    order0 = np.array([0, 0, 1, 2, 2])
    scale = np.array([1.0, -1.0, 1.0, 0.5, 1.0])
    args = dict(nq=8, initial_index=[0b01010101, 0b00110011], initial_coeff=[0.6, 0.8],
                operators_1b=ops, order0=order0, scale=scale,
                parameter_sets=rng.uniform(-1, 1, (3, 3)), energies=[-1.5, -2.25, np.pi], nuclear_energy=0.7)
    args.update(kw)
    write_run_files(prefix, **args)
    return prefix, args


def test_round_trip_real(tmp_path):
    prefix, a = _case(tmp_path)
    rf = load_run_files(prefix)
    assert rf.nq == 8
    assert list(rf.initial_index) == a["initial_index"]
    assert np.array_equal(rf.initial_coeff, np.array(a["initial_coeff"], dtype=complex))
    assert np.array_equal(rf.operators, a["operators_1b"])
    assert np.array_equal(rf.order, a["order0"]) and np.array_equal(rf.scale, a["scale"])
    assert rf.n_params == 3 and rf.n_unique == 3
    assert np.array_equal(rf.parameter_sets, a["parameter_sets"])
    assert np.array_equal(rf.energies, a["energies"])
    assert rf.nuclear_energy == 0.7


def test_round_trip_complex_initial(tmp_path):
    c = np.array([0.6 + 0.0j, 0.0 + 0.8j])
    prefix, a = _case(tmp_path, initial_coeff=c)
    rf = load_run_files(prefix)
    assert np.array_equal(rf.initial_coeff, c)


def test_reference_parser_rules(tmp_path):
    prefix, _ = _case(tmp_path, parameter_sets=None, nuclear_energy=None)
    # bitstring alone -> 1; repeated bitstring -> last; nq = longest bitstring
    with open(prefix + "_Initial.dat", "w") as f:
        f.write("0011\n00000101,0.25\n0011,-0.5,0.125\n")
    # an entry without a scale has scale 1
    with open(prefix + "_Order.dat", "w") as f:
        f.write("1\n1,-1\n2\n3,0.5\n  3\n")
    rf = load_run_files(prefix)
    assert rf.nq == 8
    assert list(rf.initial_index) == [3, 5]
    assert np.array_equal(rf.initial_coeff, [-0.5 + 0.125j, 0.25])
    assert np.array_equal(rf.scale, [1, -1, 1, 0.5, 1]) and np.array_equal(rf.order, [0, 0, 1, 2, 2])
    # no Parameters / Nuclear_Energy file: no angle sets, no nuclear energy
    assert rf.parameter_sets.shape == (0, 3) and rf.nuclear_energy is None and rf.n_unique == 3


def test_parameters_past_the_last_set_are_zero(tmp_path):
    prefix, _ = _case(tmp_path, parameter_sets=None)
    # first set has 4 angles, last only 2: the reference assigns parameter p only
    # when p < the last set's count (TUPSLoadingUtils.cpp:275)
    with open(prefix + "_Parameters.dat", "w") as f:
        f.write("4\nEnergy of minimum 1= -1.0 x\n0.1\n0.2\n0.3\n0.4\n")
        f.write("2\nEnergy of minimum 2= -2.0 y\n0.5 0.6\n")
    rf = load_run_files(prefix)
    assert rf.n_unique == 3  # max(largest order, 2)
    assert np.array_equal(rf.parameter_sets, [[0.1, 0.2, 0.0], [0.5, 0.6, 0.0]])
    assert np.array_equal(rf.energies, [-1.0, -2.0])
    # more angles than parameters: n_unique follows the file (the reference's count)
    write_parameters(prefix + "_Parameters.dat", [np.arange(5.0)], [0.0])
    rf = load_run_files(prefix)
    assert rf.n_unique == 5 and np.array_equal(rf.parameter_sets, [[0.0, 1.0, 2.0]])


def test_extracted_min_sets(tmp_path):
    prefix, _ = _case(tmp_path, parameter_sets=[np.zeros(4)])  # n_unique = 4
    write_extracted_min(prefix + "_extractedmin", np.arange(8.0).reshape(2, 4))
    rf = load_run_files(prefix, extracted_min=True)
    assert np.array_equal(rf.parameter_sets, [[0, 1, 2], [4, 5, 6]])
    assert np.isnan(rf.energies).all()
    write_extracted_min(prefix + "_extractedmin", np.arange(6.0))
    with pytest.raises(AegpuError, match="extractedmin"):
        load_run_files(prefix, extracted_min=True)


@pytest.mark.parametrize("fname,text,match", [
    ("_Initial.dat", "abc,1\n", "missing bitstring"),
    ("_Initial.dat", "1" * 32 + ",1\n", "31 qubits"),
    ("_Operators.dat", "1 2 0 0\n5 6 0\n", "four integers"),
    ("_Order.dat", "1\n1\n2\n3\n", "More operators in path than relations given"),
    ("_Order.dat", "1\n1\n0\n3\n3\n", "negative"),
    ("_Parameters.dat", "3\nno energy here\n", "'='"),
    ("_Parameters.dat", "3\nE= 1\n0.1\n0.2\n", "fewer than 3"),
])
def test_malformed_files_are_refused(tmp_path, fname, text, match):
    prefix, _ = _case(tmp_path)
    with open(prefix + fname, "w") as f:
        f.write(text)
    with pytest.raises(AegpuError, match=match):
        load_run_files(prefix)


def test_missing_required_file(tmp_path):
    prefix, _ = _case(tmp_path)
    os.remove(prefix + "_Operators.dat")
    with pytest.raises(AegpuError, match="_Operators.dat"):
        load_run_files(prefix)


def test_set_run_files_status_codes(tmp_path):
    L = lib()
    prefix, _ = _case(tmp_path)
    assert L.setRunFiles(prefix.encode(), None) == 1
    ctx = ctypes.c_void_p(L.init())
    try:
        assert L.setRunFiles(None, ctx) == 2
        assert L.setRunFiles(str(tmp_path / "absent").encode(), ctx) == 3
        assert L.setRunFiles(prefix.encode(), ctx) == 0
    finally:
        L.cleanup(ctypes.byref(ctx))


def test_writers_match_the_manual_examples(tmp_path):
    p = str(tmp_path / "x")
    write_initial(p, 8, [0b01010101], [1.0])
    assert open(p).read() == "01010101,1.0\n"
    write_order(p, [0, 0, 1, 0, 0], [1, 1, 1, -1, -1])
    assert open(p).read() == "1\n1\n2\n1,-1.0\n1,-1.0\n"


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "Hams")), reason="reference checkout not present")
@pytest.mark.parametrize("sub,name", [("H4/L1/H4", "h4"), ("TestFermionic/TestFermionic", "ferm"),
                                      ("H4_Complex/L1/H4", "h4c")])
def test_reference_fixtures_parse_like_the_golden_inputs(golden, sub, name):
    fx = golden(name)
    rf = load_run_files(os.path.join(REF, "Hams", sub))
    assert rf.nq == int(fx["nq"])
    assert np.array_equal(rf.initial_index, fx["init_idx"])
    assert np.array_equal(rf.initial_coeff, fx["init_re"] + 1j * fx["init_im"])
    assert np.array_equal(rf.operators, fx["ops_1b"])
    assert np.array_equal(rf.order + 1, fx["order_1b"]) and np.array_equal(rf.scale, fx["scale"])
    assert (rf.nuclear_energy or 0.0) == float(fx["nuclear"])
    # the golden's first angle set is the Parameters file's last set
    assert np.array_equal(rf.parameter_sets[-1], fx["angles"][0])


def test_round_trip_random_files(tmp_path):
    """Randomised round trips through the writers and the C++ readers: every value
    comes back exactly (17 significant digits), for many shapes of input."""
    rng = np.random.default_rng(11)
    for case in range(40):
        nq = 2 * int(rng.integers(2, 8))
        nops = int(rng.integers(1, 30))
        ops = np.zeros((nops, 4), dtype=np.int64)
        for k in range(nops):
            a, b = rng.choice(nq, 2, replace=False) + 1
            ops[k] = (a, b, 0, 0) if rng.random() < 0.5 else tuple(rng.choice(nq, 4, replace=False) + 1)
        P = int(rng.integers(1, nops + 1))
        order0 = np.concatenate([np.arange(P), rng.integers(0, P, nops - P)]) if nops > P else np.arange(nops)
        scale = np.where(rng.random(nops) < 0.5, 1.0, rng.normal(size=nops))
        ninit = int(rng.integers(1, 5))
        idx = rng.choice(1 << nq, ninit, replace=False)
        coeff = rng.normal(size=ninit) + (1j * rng.normal(size=ninit) if rng.random() < 0.5 else 0)
        sets = rng.normal(size=(int(rng.integers(0, 4)), P)) * 10.0 ** rng.integers(-12, 3)
        nuc = float(rng.normal()) if rng.random() < 0.5 else None
        prefix = str(tmp_path / ("r%d" % case))
        write_run_files(prefix, nq, idx, coeff, ops, order0, scale,
                        parameter_sets=sets if len(sets) else None, energies=rng.normal(size=len(sets)),
                        nuclear_energy=nuc)
        rf = load_run_files(prefix)
        assert rf.nq == nq
        got = dict(zip(rf.initial_index.tolist(), rf.initial_coeff))
        for i, c in zip(idx.tolist(), np.asarray(coeff, dtype=complex)):
            assert got[i] == c
        assert np.array_equal(rf.operators, ops)
        assert np.array_equal(rf.order, order0) and np.array_equal(rf.scale, scale)
        assert rf.n_params == int(order0.max()) + 1
        if len(sets):
            assert np.array_equal(rf.parameter_sets, sets[:, :rf.n_params])
        else:
            assert rf.parameter_sets.shape[0] == 0
        assert rf.nuclear_energy == nuc


def test_reference_named_loaders(tmp_path):
    """The reference binding's module functions (PyAnsatzEvolve.cpp:101-147): loadOperators
    (1-based lists), loadPath ((0, 0.0) per operator), loadNuclearEnergy (0 when missing),
    readCsvState (dense real vector), loadParameters (template path first, then one path
    per angle set with angle = set[order] * scale)."""
    import ansatzevolve_gb300 as ae
    prefix, a = _case(tmp_path)
    assert ae.loadOperators(prefix + "_Operators.dat") == a["operators_1b"].tolist()
    assert ae.loadPath(prefix + "_Operators.dat") == [(0, 0.0)] * len(a["operators_1b"])
    assert ae.loadNuclearEnergy(prefix) == 0.7
    assert ae.loadNuclearEnergy(str(tmp_path / "none")) == 0.0
    dense = ae.readCsvState(prefix + "_Initial.dat")
    want = np.zeros(256)
    want[a["initial_index"]] = a["initial_coeff"]
    assert np.array_equal(dense, want)
    template = [(3, 0.25)] * 5
    paths, order, nuniq = ae.loadParameters(prefix + "_Order.dat", prefix + "_Parameters.dat", template)
    assert order == [(int(p), float(c)) for p, c in zip(a["order0"], a["scale"])] and nuniq == 3
    assert paths[0] == template and len(paths) == 1 + len(a["parameter_sets"])
    for x, path in zip(a["parameter_sets"], paths[1:]):
        assert path == [(3, float(x[p] * c)) for p, c in order]
    with pytest.raises(AegpuError, match="relations"):
        ae.loadParameters(prefix + "_Order.dat", prefix + "_Parameters.dat", template[:3])


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "Hams")), reason="reference checkout not present")
def test_reference_named_loaders_on_fixtures(golden):
    import ansatzevolve_gb300 as ae
    fx = golden("h4")
    base = os.path.join(REF, "Hams", "H4", "L1", "H4")
    assert ae.loadOperators(base + "_Operators.dat") == np.asarray(fx["ops_1b"]).tolist()
    assert ae.loadNuclearEnergy(base) == float(fx["nuclear"])
    st = ae.readCsvState(base + "_Initial.dat")
    assert len(st) == 256 and [i for i, v in enumerate(st) if v] == list(fx["init_idx"])
    paths, order, nuniq = ae.loadParameters(base + "_Order.dat", base + "_Parameters.dat",
                                            ae.loadPath(base + "_Operators.dat"))
    assert nuniq == 9 and len(paths) == 3
    p0, sc = np.asarray(fx["order_1b"]) - 1, np.asarray(fx["scale"])
    assert np.array_equal([a for _, a in paths[2]], sc * np.asarray(fx["angles"][0])[p0])
