"""The reference's run files: the inputs its command-line driver reads from a path
prefix (src/main.cpp:221-386), and the driver's ``optimise`` verb on top of them.

Reading is done by the library's C++ readers (``include/aegpu_runfiles.h``, restating
src/TUPSLoadingUtils.cpp:10-360); this module wraps them and adds writers for the same
formats, so inputs made here are read unchanged by the reference and the other way
round:

    <prefix>_Initial.dat         "bitstring,re[,im]" per line (bit i = i-th char from the right)
    <prefix>_Operators.dat       "a b c d", 1-based, 0 = absent
    <prefix>_Order.dat           "parameter[,scale]", 1-based
    <prefix>_Parameters.dat      count, "... = energy ..." line, angles; repeated
    <prefix>_Nuclear_Energy.dat  one number
    <prefix>_extractedmin        bare angles, n_unique per set
    <prefix>_oneEInts.bin / _twoEInts.bin   integrals (``synthetic.write_integrals``)
    <prefix>_Ham_Coeff.dat / _Ham_Index.dat  sparse Hamiltonian (``write_sparse_hamiltonian``)
"""
import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import PROPERTY_NAMES, AegpuError, _DP, _IP, _P, lib, stateAnsatzManager
from .checkpoint import write_parameters


@dataclass
class RunFiles:
    nq: int
    initial_index: np.ndarray   # int32, 0-based into the 2^nq space
    initial_coeff: np.ndarray   # complex128
    operators: np.ndarray       # int32 (n_ops, 4), 1-based, 0 = absent (the file's form)
    order: np.ndarray           # int32, 0-based parameter of each operator
    scale: np.ndarray           # float64
    n_unique: int               # the reference driver's parameter count (sizes extractedmin sets)
    parameter_sets: np.ndarray  # (n_sets, n_params) compressed angle sets
    energies: np.ndarray        # the energy written with each set (NaN if none)
    nuclear_energy: Optional[float]

    @property
    def n_params(self):
        return int(self.order.max()) + 1 if len(self.order) else 0


def _read(opener, what):
    """Open a run-files handle through `opener(ctypes.byref(handle))` and copy out every
    field (the ones the opener did not fill come back empty)."""
    L = lib()
    h = _P()
    rc = opener(ctypes.byref(h))
    if rc:
        raise AegpuError("run files %s: %s" % (what, L.aegpu_run_files_error().decode()))
    try:
        n = [ctypes.c_int() for _ in range(6)]
        L.aegpu_run_files_sizes(h, *[ctypes.byref(v) for v in n])
        nq, ninit, nops, P, nuniq, nsets = (v.value for v in n)
        idx = np.zeros(ninit, dtype=np.int32)
        coeff = np.zeros(2 * ninit)
        ops = np.zeros(4 * nops, dtype=np.int32)
        order = np.zeros(nops, dtype=np.int32)
        scale = np.zeros(nops)
        sets = np.zeros(max(nsets * P, 1))
        energies = np.zeros(max(nsets, 1))
        nuc = np.zeros(1)
        ip = lambda a: a.ctypes.data_as(_IP)  # noqa: E731
        dp = lambda a: a.ctypes.data_as(_DP)  # noqa: E731
        L.aegpu_run_files_get(h, ip(idx), dp(coeff), ip(ops), ip(order), dp(scale), dp(sets), dp(energies), dp(nuc))
    finally:
        L.aegpu_run_files_free(h)
    return RunFiles(nq=nq, initial_index=idx, initial_coeff=coeff[0::2] + 1j * coeff[1::2],
                    operators=ops.reshape(nops, 4), order=order - 1, scale=scale, n_unique=nuniq,
                    parameter_sets=sets[:nsets * P].reshape(nsets, P), energies=energies[:nsets],
                    nuclear_energy=None if np.isnan(nuc[0]) else float(nuc[0]))


def load_run_files(prefix, extracted_min=False):
    """All run files of `prefix`; raises AegpuError naming the file that is missing or
    malformed.  The Parameters and Nuclear_Energy files are optional."""
    L = lib()
    return _read(lambda h: L.aegpu_run_files_load(str(prefix).encode(), int(bool(extracted_min)), h), prefix)


def write_initial(path, nq, index, coeff):
    """One "bitstring,re[,im]" line per basis state (the imaginary part only when some
    coefficient has one)."""
    c = np.asarray(coeff)
    cplx = np.iscomplexobj(c) and np.any(np.imag(c) != 0)
    with open(path, "w") as f:
        for i, v in zip(np.asarray(index, dtype=np.int64), c):
            bits = format(int(i), "0%db" % nq)
            if cplx:
                f.write("%s,%r,%r\n" % (bits, float(np.real(v)), float(np.imag(v))))
            else:
                f.write("%s,%r\n" % (bits, float(np.real(v))))


def write_operators(path, operators_1b):
    with open(path, "w") as f:
        for o in np.asarray(operators_1b, dtype=np.int64).reshape(-1, 4):
            f.write("%d %d %d %d\n" % tuple(o))


def write_order(path, order0, scale=None):
    order0 = np.asarray(order0, dtype=np.int64)
    scale = np.ones(len(order0)) if scale is None else np.asarray(scale, dtype=np.float64)
    with open(path, "w") as f:
        for p, c in zip(order0, scale):
            f.write("%d\n" % (p + 1) if c == 1.0 else "%d,%r\n" % (p + 1, float(c)))


def write_nuclear_energy(prefix, e):
    with open(prefix + "_Nuclear_Energy.dat", "w") as f:
        f.write("%r\n" % float(e))


def write_extracted_min(path, sets):
    with open(path, "w") as f:
        for a in np.atleast_2d(sets):
            for v in a:
                f.write("%r\n" % float(v))


def write_sparse_hamiltonian(prefix, i0, j0, coeff):
    """<prefix>_Ham_Coeff.dat (one coefficient per line) and <prefix>_Ham_Index.dat
    ("i j" per line, 1-based indices into the 2^nq space)."""
    with open(prefix + "_Ham_Coeff.dat", "w") as f:
        for v in np.asarray(coeff, dtype=np.float64):
            f.write("%r\n" % float(v))
    with open(prefix + "_Ham_Index.dat", "w") as f:
        for i, j in zip(np.asarray(i0, dtype=np.int64), np.asarray(j0, dtype=np.int64)):
            f.write("%d %d\n" % (i + 1, j + 1))


def write_run_files(prefix, nq, initial_index, initial_coeff, operators_1b, order0, scale=None,
                    parameter_sets=None, energies=None, nuclear_energy=None, h1=None, g2=None,
                    ham_triplets=None):
    """Everything `load_run_files` / ``setRunFiles`` read, in the reference's formats."""
    write_initial(prefix + "_Initial.dat", nq, initial_index, initial_coeff)
    write_operators(prefix + "_Operators.dat", operators_1b)
    write_order(prefix + "_Order.dat", order0, scale)
    if parameter_sets is not None:
        write_parameters(prefix + "_Parameters.dat", parameter_sets, energies)
    if nuclear_energy is not None:
        write_nuclear_energy(prefix, nuclear_energy)
    if h1 is not None:
        from .synthetic import write_integrals
        write_integrals(prefix, h1, g2)
    if ham_triplets is not None:
        write_sparse_hamiltonian(prefix, *ham_triplets)


def iterative_optimise_run(prefix, extracted_min=False, out=None):
    """The driver's ``iterativeOptimise`` verb (src/main.cpp:502-515): the projected
    iteration then Newton-Raphson from the first angle set; as `optimise_run`."""
    return optimise_run(prefix, extracted_min, out, iterative=True)


def optimise_run(prefix, extracted_min=False, out=None, iterative=False):
    """The reference driver's ``optimise`` verb (src/main.cpp:489-500): set up from the
    run files, Newton-Raphson (TUPSQuantities::OptimiseTups) from the first angle set
    (zero angles when the files hold none), on the GPU.  Returns (energy, compressed
    angles, RunFiles); with `out`, also writes the optimised set as a Parameters file."""
    m = stateAnsatzManager()
    try:
        rf = m.storeRunFiles(prefix)
        if extracted_min:
            rf = load_run_files(prefix, extracted_min=True)
        x0 = rf.parameter_sets[0] if len(rf.parameter_sets) else np.zeros(rf.n_params)
        E, x = m.iterativeOptimise(x0) if iterative else m.optimise(x0)
    finally:
        m.close()
    if out is not None:
        write_parameters(out, [x], [E])
    return E, x, rf


def format_properties(table, have_hf=True):
    """The table in the reference's text layout (printOutputHeaders / printOutputLine,
    tupsquantities.cpp:2158-2205): a 40-character name column, then one 26-character
    column per path ("HF" first when the zero path is included)."""
    npath = len(next(iter(table.values())))
    out = ["", "%-40s %40s " % ("Results:", "Path Number")]
    head = "%-40s" % ""
    labels = (["HF"] if have_hf else []) + [str(i) for i in range(1, npath + (0 if have_hf else 1))]
    out.append(head + "".join("%-26s" % c for c in labels))
    for name in PROPERTY_NAMES:
        vals = np.asarray(table[name])
        if np.all(np.isnan(vals)):
            continue
        out.append("%-40s" % name + "".join("%-26.16g" % v for v in vals))
    return "\n".join(out) + "\n"


def properties_run(prefix, extracted_min=False, no_hf_path=False, no_hess=False, lowest_eigenvalue=True,
                   optimise=False, write_files=False):
    """The reference driver's ``writeproperties`` verb (src/main.cpp:520-529; with
    ``optimise`` first, as ``optimise writeproperties`` runs them, :489-500): the
    properties table over the zero path (unless no_hf_path) and the run files' angle
    sets (plus the optimised set).  Returns (table dict, subspace eigenvalues, null
    rank, lowest eigenvalue or None, text); write_files also writes the reference's
    per-path Hessian / metric files and overlap vector next to the run files."""
    m = stateAnsatzManager()
    try:
        rf = m.storeRunFiles(prefix)
        if extracted_min:
            rf = load_run_files(prefix, extracted_min=True)
        sets = [np.asarray(x) for x in rf.parameter_sets]
        if optimise:
            x0 = sets[0] if sets else np.zeros(rf.n_params)
            sets.append(m.optimise(x0)[1])
        paths = ([] if no_hf_path else [np.zeros(rf.n_params)]) + sets
        table = m.getProperties(paths, hessian=not no_hess, overlap=lowest_eigenvalue)
        if write_files:  # the reference's files beside the run files, and its printout
            m.writeProperties(paths, runPath=prefix, hessian=not no_hess, overlap=lowest_eigenvalue,
                              hf_path=not no_hf_path)
        lam = m.getLowestEigenvalue()[0] if lowest_eigenvalue else None
        w, nr = m.getSubspaceEigenvalues(sets) if sets else (np.zeros(0), 0)
    finally:
        m.close()
    return table, w, nr, lam, format_properties(table, have_hf=not no_hf_path)


# ------------------------------------------------------------------------------
# The reference binding's module functions (PyAnsatzEvolve.cpp:101-147), same names and
# return shapes, over the C++ readers.  A rotation path is a list of (operator index,
# angle) pairs; the reference's module fills the index with 0 (loadPath without an
# operator pool).


def loadOperators(filepath):
    """Operators of an Operators file, 1-based [a, b, c, d] lists (0 = absent)."""
    L = lib()
    rf = _read(lambda h: L.aegpu_run_file_read(str(filepath).encode(), 2, h), filepath)
    return [list(map(int, o)) for o in rf.operators]


def loadPath(filepath):
    """One (0, 0.0) rotation element per operator of an Operators file."""
    return [(0, 0.0) for _ in loadOperators(filepath)]


def loadNuclearEnergy(filepath):
    """The number in <filepath>_Nuclear_Energy.dat, 0.0 when the file is missing."""
    L = lib()
    rf = _read(lambda h: L.aegpu_run_file_read(str(filepath).encode(), 3, h), filepath)
    return 0.0 if rf.nuclear_energy is None else rf.nuclear_energy


def readCsvState(filepath):
    """The Initial file as a dense real vector of 2^(longest bitstring) entries (the
    reference's real readCsvState drops imaginary parts)."""
    L = lib()
    rf = _read(lambda h: L.aegpu_run_file_read(str(filepath).encode(), 1, h), filepath)
    out = np.zeros(1 << rf.nq)
    out[rf.initial_index] = rf.initial_coeff.real
    return out.tolist()


def loadParameters(orderFilePath, parameterFilepath, templatePath):
    """(rotationPaths, order, numberOfUniqueParameters) as the reference binding returns
    them: the template path first (its own angles), then one path per angle set of the
    Parameters file with angle = set[order] * scale (0 where the file's last set has no
    such parameter); order is [(parameter, scale)], 0-based."""
    L = lib()
    template = [(int(i), float(a)) for i, a in templatePath]
    rf = _read(lambda h: L.aegpu_run_files_parameters(str(orderFilePath).encode(), str(parameterFilepath).encode(),
                                                      len(template), h), orderFilePath)
    order = [(int(p), float(c)) for p, c in zip(rf.order, rf.scale)]
    paths = [list(template)]
    for x in rf.parameter_sets:
        paths.append([(template[k][0], float(x[p] * c)) for k, (p, c) in enumerate(order)])
    return paths, order, rf.n_unique
