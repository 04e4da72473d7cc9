"""Generates the committed golden fixtures in tests/golden/ from the reference itself.

Run here (where the reference checkout and oracle/_ref exist):
    oracle/build_ref.sh && python tests/golden/make_golden.py
Every fixture records the inputs (initial state, excitations, order, Hamiltonian as
triplets or integrals, angles) and the reference's outputs for them, produced by
oracle/_ref/ref_driver through the reference's public stateAnsatzManager API.
Sources of the inputs:
  f90      -- the Fortran binding test's arrays, parsed from src/test.F90
  ferm     -- Hams/TestFermionic (sparse Hamiltonian, number-only sector)
  h4       -- Hams/H4/L1 integrals / operators / order / parameters (+ optimise)
  h4c      -- Hams/H4_Complex/L1 (complex build, diagonal U3 operators)
  syn8     -- synthetic 8-orbital TUPS, seed 0 (ansatzevolve_gb300.synthetic)
  syn6     -- synthetic 6-orbital TUPS, seed 3, plus the excitation rule table
  ref10    -- the benchmark's 10-orbital inputs (seed 0, 3 layers): E, gradient, Hessian,
              sampled final-state amplitudes
  ref12    -- the benchmark's 12-orbital inputs (seed 0, 3 layers): E, gradient, Hessian,
              sampled final-state amplitudes
  ref14    -- the benchmark's 14-orbital inputs (7a+7b, seed 0, 4 layers; the reference
              picks its on-the-fly H here): E, gradient, sampled final-state amplitudes
  lucj14   -- the complex LUCJ circuit exp(-K) exp(iJ) exp(K) at 14 orbitals (K, J of
              ansatzevolve_gb300.lucj.random_lucj(14, 3), integrals of seed 7), every
              operator its own parameter: E, gradient, sampled final-state amplitudes
  overlaps_syn6, overlaps_h4c
           -- writeProperties with numberOfOverlapsToCompute = 4 / 3 over the zero path and
              the syn6 / h4c angle sets: overlaps with the lowest eigenstates
  batched4 -- instance 0 of each size class of the benchmark's batched launch (8, 10, 12
              orbitals, its own integrals and angles): energy and gradient
  pairs12  -- the excitation rule of every operator of the 12-orbital, 3-layer TUPS circuit
              over every determinant of the 6a+6b sector: SHA-256 digests of the partner
              bitstrings and signs, active counts and a seeded sample of raw entries
  props_h4, props_h4c, props_syn6
           -- the reference's own TUPSQuantities::writeProperties table (energies,
              Hessian / metric eigenvalue and diagonal counts, gradient norms, overlaps
              with the lowest eigenvector), its Hessian and metric matrices per path, and
              doSubspaceDiagonalisation's eigenvalues, over the zero path and the angle
              sets of the h4 / h4c / syn6 inputs plus a repeat of the first set
Only the ref10 / ref12 / ref14 / lucj14 / pairs12 / overlaps_* / batched4 / props_* cases can be regenerated alone:
    python tests/golden/make_golden.py ref10 ref12 ref14 lucj14 pairs12 overlaps_syn6 overlaps_h4c batched4 props_h4 props_h4c props_syn6
The reference checkout is AE_REFERENCE (default: a `reference` directory beside this
repository).
"""
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from ansatzevolve_gb300.synthetic import (hartree_fock_index, synthetic_integrals,  # noqa: E402
                                          tups_operators, write_integrals)

REF = os.environ.get("AE_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
DRV = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
OUT = os.path.dirname(os.path.abspath(__file__))


def run(spec_lines, cplx=False, threads=4):
    with tempfile.TemporaryDirectory(dir=os.environ.get("AE_GOLDEN_TMP")) as td:
        sp, op = os.path.join(td, "spec"), os.path.join(td, "out")
        open(sp, "w").write("\n".join(spec_lines) + "\nend\n")
        drv = DRV + ("_cplx" if cplx else "")
        subprocess.run([drv, sp, op], check=True, stderr=subprocess.DEVNULL, stdout=subprocess.DEVNULL,
                       env=dict(os.environ, OMP_NUM_THREADS=str(threads)))
        return np.fromfile(op, dtype="<f8")


def spec(nq, init, ops0, param0, scale, ham, anglesets, want=(1, 1, 1, 1), pairs=0, optimise=0, nuclear=0.0):
    s = [f"nqubits {nq}", f"initial {len(init)}"]
    s += [f"{i} {re!r} {im!r}" for i, re, im in init]
    s += [f"ops {len(ops0)}"] + [" ".join(str(int(v)) for v in o) for o in ops0]
    s += [f"order {len(param0)}"] + [f"{int(p)} {float(c)!r}" for p, c in zip(param0, scale)]
    s += ham
    s += [f"nuclear {float(nuclear)!r}"]
    s += [f"anglesets {len(anglesets)} {len(anglesets[0])}"] + [" ".join(repr(float(a)) for a in A) for A in anglesets]
    s += ["want " + " ".join(str(w) for w in want), f"pairs {pairs}", f"optimise {optimise}"]
    return s


def split_outputs(d, nsets, P, nstate, want, cplx=False):
    out = {"E": [], "G": [], "H": [], "S": []}
    w = 2 if cplx else 1
    k = 0
    for _ in range(nsets):
        if want[0]:
            out["E"].append(d[k]); k += 1
        if want[1]:
            out["G"].append(d[k:k + P]); k += P
        if want[2]:
            out["H"].append(d[k:k + P * P].reshape(P, P, order="F")); k += P * P
        if want[3]:
            out["S"].append(d[k:k + nstate * w]); k += nstate * w
    return {key: np.array(v) for key, v in out.items() if v}, d[k:]


def fortran_case():
    src = open(os.path.join(REF, "src", "test.F90")).read()

    def arr(pat):
        m = re.search(pat + r"\s*=\s*(?:transpose\(reshape\()?\[([^\]]*)\]", src)
        return [t.strip() for t in m.group(1).split(",")]

    hi = np.array([int(x) for x in arr("HamiIndexes")], dtype=np.int32)
    hj = np.array([int(x) for x in arr("HamjIndexes")], dtype=np.int32)
    hv = np.array([float(x.replace("_dp", "")) for x in arr("HamCoeffs")])
    ops = np.array([int(x) for x in arr(r"dimension\(15, 4\) :: operators")], dtype=np.int32).reshape(15, 4)
    order = np.array([int(x) for x in arr(r"dimension\(15\) :: order")], dtype=np.int32)
    angmin = np.array([float(x.replace("_dp", "")) for x in re.findall(
        r"angles\s*=\s*\[([^\]]*)\]", src)[1].split(",")])
    expected = {}
    for key, pat in [("E0", r'"Expected:", (-?[0-9.]+)_dp'), ("G0", r'"gradient Norm Expected:", ([0-9.E-]+)_dp')]:
        expected[key] = [float(v) for v in re.findall(pat, src)]
    rng = np.random.default_rng(11)
    sets = [np.zeros(9), angmin, rng.uniform(-1, 1, 9)]
    ops0 = ops - 1
    s = spec(8, [(170, 1.0, 0.0)], ops0, order - 1, np.ones(15),
             [f"ham triplets {len(hv)}"] + [f"{a - 1} {b - 1} {float(c)!r}" for a, b, c in zip(hi, hj, hv)],
             sets, pairs=1)
    d = run(s)
    res, rest = split_outputs(d, len(sets), 9, 256, (1, 1, 1, 1))
    pairs = rest.reshape(15, 256, 2)
    np.savez_compressed(os.path.join(OUT, "f90.npz"), nq=8, init_idx=[170], init_re=[1.0], ops_1b=ops,
                        order_1b=order, scale=np.ones(15), ham_i_1b=hi, ham_j_1b=hj, ham_v=hv,
                        angles=np.array(sets), E=res["E"], G=res["G"], H=res["H"], S=res["S"],
                        pair_partner=pairs[..., 0].astype(np.uint32), pair_sign=pairs[..., 1].astype(np.int8),
                        known_E=np.array(expected["E0"]), known_gnorm=np.array(expected["G0"]))
    print("f90", res["E"], np.linalg.norm(res["G"], axis=1))


def read_order(path):
    param, scale = [], []
    for line in open(path):
        line = line.strip()
        if not line:
            continue
        parts = line.split(",")
        param.append(int(parts[0]))
        scale.append(float(parts[1]) if len(parts) > 1 else 1.0)
    return np.array(param, dtype=np.int32), np.array(scale)


def read_params(path):
    toks = open(path).read().split("\n")
    sets, k = [], 0
    while k < len(toks):
        t = toks[k].strip()
        if not t:
            k += 1
            continue
        n = int(t)
        vals = [float(toks[k + 2 + i]) for i in range(n)]
        sets.append(vals)
        k += 2 + n
    return np.array(sets)


def read_initial(path, nq_hint=None):
    init = []
    for line in open(path):
        line = line.strip()
        if not line:
            continue
        parts = line.split(",")
        bits = parts[0].strip()
        re_ = float(parts[1]) if len(parts) > 1 and parts[1].strip() else 1.0
        im_ = float(parts[2]) if len(parts) > 2 and parts[2].strip() else 0.0
        init.append((int(bits, 2), re_, im_, len(bits)))
    return init


def hams_case(name, sub, cplx=False, optimise=False, tag=None):
    base = os.path.join(REF, "Hams", name, sub, name.split("_")[0]) if sub else os.path.join(REF, "Hams", name, name)
    init = read_initial(base + "_Initial.dat")
    nq = init[0][3]
    ops = np.loadtxt(base + "_Operators.dat", dtype=np.int32).reshape(-1, 4)
    param, scale = read_order(base + "_Order.dat")
    params = read_params(base + "_Parameters.dat")
    nuclear = float(open(base + "_Nuclear_Energy.dat").read()) if os.path.exists(base + "_Nuclear_Energy.dat") else 0.0
    P = int(param.max())
    rng = np.random.default_rng(5)
    sets = [params[-1][:P], rng.uniform(-0.5, 0.5, P), params[0][:P]]  # optimise() starts from the last set
    fx = dict(nq=nq, init_idx=[i[0] for i in init], init_re=[i[1] for i in init], init_im=[i[2] for i in init],
              ops_1b=ops, order_1b=param, scale=scale, nuclear=nuclear, angles=np.array(sets))
    if os.path.exists(base + "_oneEInts.bin"):
        N = nq // 2
        fx["h1"] = np.fromfile(base + "_oneEInts.bin").reshape(N, N)
        fx["g2"] = np.fromfile(base + "_twoEInts.bin").reshape(N, N, N, N)
        ham = [f"ham ints {base}"]
    else:
        cv = np.loadtxt(base + "_Ham_Coeff.dat", delimiter=",", ndmin=2)[:, 0]
        ij = np.loadtxt(base + "_Ham_Index.dat", dtype=np.int64, ndmin=2)
        fx.update(ham_i_1b=ij[:, 0].astype(np.int32), ham_j_1b=ij[:, 1].astype(np.int32), ham_v=cv)
        ham = [f"ham triplets {len(cv)}"] + [f"{a - 1} {b - 1} {float(c)!r}" for (a, b), c in zip(ij, cv)]
    s = spec(nq, [(i[0], i[1], i[2]) for i in init], ops - 1, param - 1, scale, ham, sets,
             optimise=int(optimise), nuclear=nuclear)
    d = run(s, cplx)
    res, rest = split_outputs(d, len(sets), P, 1 << nq, (1, 1, 1, 1), cplx)
    fx.update(E=res["E"], G=res["G"], H=res["H"], S=res["S"])
    if optimise:
        fx["opt_E"] = rest[0]
        fx["opt_angles"] = rest[3:3 + int(rest[2])]
    np.savez_compressed(os.path.join(OUT, (tag or name.lower()) + ".npz"), **fx)
    print(tag or name, res["E"], fx.get("opt_E"))


def synthetic_case(tag, N, na, nb, layers, seed, pairs=False, hess=True):
    h, g = synthetic_integrals(N, seed)
    ops, param, scale = tups_operators(N, layers)
    P = int(param.max())
    rng = np.random.default_rng(seed + 100)
    sets = [rng.uniform(-0.1, 0.1, P), rng.uniform(-0.3, 0.3, P)]
    with tempfile.TemporaryDirectory() as td:
        prefix = os.path.join(td, "syn")
        write_integrals(prefix, h, g)
        hf = hartree_fock_index(N, na, nb)
        s = spec(2 * N, [(hf, 1.0, 0.0)], ops - 1, param - 1, scale, [f"ham ints {prefix}"], sets,
                 want=(1, 1, int(hess), 1), pairs=int(pairs))
        d = run(s)
    res, rest = split_outputs(d, len(sets), P, 1 << (2 * N), (1, 1, int(hess), 1))
    # keep the final states compressed to the sector to keep the fixture small
    sect = [s_ for s_ in range(1 << (2 * N)) if bin(s_ >> N).count("1") == na and bin(s_ & ((1 << N) - 1)).count("1") == nb]
    fx = dict(N=N, na=na, nb=nb, layers=layers, seed=seed, hf=hf, ops_1b=ops, order_1b=param, scale=scale,
              angles=np.array(sets), E=res["E"], G=res["G"], S_sector=res["S"][:, sect], sector=np.array(sect, dtype=np.uint32))
    if hess:
        fx["H"] = res["H"]
    if pairs:
        pr = rest.reshape(len(ops), 1 << (2 * N), 2)
        fx["pair_partner"] = pr[..., 0].astype(np.uint32)
        fx["pair_sign"] = pr[..., 1].astype(np.int8)
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), **fx)
    print(tag, res["E"])


PROPERTY_ROWS = ("Elec. Energy", "Real Elec. Energy", "Elec. + Nuc. Energy",
                 "NumberOfNegativeHessianEValues", "NumberOfNearZeroHessianEValues",
                 "NumberOfPositiveHessianEValues", "NumberOfNegativeHessianDiagValues",
                 "NumberOfNearZeroHessianDiagValues", "NumberOfPositiveHessianDiagValues",
                 "NumberOfPositiveMetricEValues", "NumberOfZeroMetricEValues", "NumberOfZeroMetricDiagonalValues",
                 "NormOfGradVector", "OverlapWithState_0", "MagOfOverlapWithState_0")


def batched_case(tag):
    """Configuration 4's batched instances against the reference: instance 0 of each size
    class of the benchmark's 512-instance launch -- 8 orbitals (4a+4b, 2 layers, integral
    seed 0), 10 (5a+5b, 3 layers, seed 256), 12 (6a+6b, 3 layers, seed 448) -- with the
    bench's own TUPS angles (default_rng(0).uniform(-0.3, 0.3) drawn class by class,
    [instances, parameters], each operator taking scale * x[param]): energy and
    compressed gradient.  x{N} holds the operators' angles, xc{N} the parameters."""
    classes = [(8, 4, 2, 256, 0), (10, 5, 3, 192, 256), (12, 6, 3, 64, 448)]
    rng = np.random.default_rng(0)
    fx = {}
    for N, na, L, nb, s0 in classes:
        ops, param, scale = tups_operators(N, L)
        P = int(param.max())
        xc = rng.uniform(-0.3, 0.3, (nb, P))[0]
        ang = np.asarray(scale, dtype=float) * xc[param - 1]
        h, g = synthetic_integrals(N, s0)
        with tempfile.TemporaryDirectory() as td:
            prefix = os.path.join(td, "syn")
            write_integrals(prefix, h, g)
            hf = hartree_fock_index(N, na, na)
            d = run(spec(2 * N, [(hf, 1.0, 0.0)], ops - 1, param - 1, scale, [f"ham ints {prefix}"], [ang],
                         want=(1, 1, 0, 0)), threads=8)
        fx[f"E{N}"] = d[0]
        fx[f"G{N}"] = d[1:1 + P]
        fx[f"x{N}"] = ang
        fx[f"xc{N}"] = xc
        fx[f"seed{N}"] = s0
        print(tag, N, d[0])
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), **fx)


def table_floats(text):
    """The numbers of one printed table row.  The complex rows print "%-20.16g, %-20.16g"
    per path, which runs two numbers together when the first fills its width
    ("4.1e-161.2e-15"): such a token is split after the first number's exponent (%g
    writes at least two exponent digits)."""
    out = []
    for t in text.replace(",", " ").split():
        try:
            out.append(float(t))
            continue
        except ValueError:
            pass
        m = re.match(r"^([-+]?[0-9.]+e[-+][0-9]{2})([-+]?[0-9.].*)$", t)
        if not m:
            raise ValueError("cannot read %r" % t)
        out += [float(m.group(1)), float(m.group(2))]
    return out


def overlaps_case(tag, base, k, cplx=False):
    """The reference's writeProperties with numberOfOverlapsToCompute = k over the zero
    path and the angle sets of fixture `base` (below 5,000 rows: overlaps with the k
    lowest eigenvectors of the dense H): OverlapWithState_i and MagOfOverlapWithState_i
    for i < k per path (eigenvector signs are the reference eigensolver's own)."""
    fx = dict(np.load(os.path.join(OUT, base + ".npz")))
    if base.startswith("syn"):
        N = int(fx["N"])
        h1, g2 = synthetic_integrals(N, int(fx["seed"]))
        nq, init, nuclear = 2 * N, [(int(fx["hf"]), 1.0, 0.0)], 0.0
    else:
        h1, g2 = fx["h1"], fx["g2"]
        nq, nuclear = int(fx["nq"]), float(fx["nuclear"])
        init = [(int(i), float(r), float(m)) for i, r, m in
                zip(fx["init_idx"], fx["init_re"], fx.get("init_im", np.zeros(len(fx["init_idx"]))))]
    sets = [np.asarray(a) for a in fx["angles"]]
    with tempfile.TemporaryDirectory() as td:
        prefix = os.path.join(td, "p")
        write_integrals(prefix, h1, g2)
        sp = spec(nq, init, np.asarray(fx["ops_1b"]) - 1, np.asarray(fx["order_1b"]) - 1, fx["scale"],
                  [f"ham ints {prefix}"], sets, want=(1, 0, 0, 0), nuclear=nuclear)
        sp += [f"properties {prefix}", f"overlaps {k}"]
        sf, of = os.path.join(td, "spec"), os.path.join(td, "out")
        open(sf, "w").write("\n".join(sp) + "\nend\n")
        subprocess.run([DRV + ("_cplx" if cplx else ""), sf, of], check=True, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="4"))
        npath = len(sets) + 1
        ov = np.zeros((k, npath), dtype=complex)
        mag = np.zeros((k, npath))
        for ln in open(prefix + "_table.txt").read().splitlines():
            name = ln[:40].strip()
            for i in range(k):
                vals = None
                if name == f"OverlapWithState_{i}":
                    vals = table_floats(ln[40:])
                    ov[i] = np.array(vals[0::2]) + 1j * np.array(vals[1::2]) if cplx else np.array(vals)
                elif name == f"MagOfOverlapWithState_{i}":
                    mag[i] = table_floats(ln[40:])
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), base=base, k=k, sets=np.array(sets), overlap=ov, mag=mag)
    print(tag, np.round(mag, 6))


def properties_case(tag, base, cplx=False):
    """writeProperties + doSubspaceDiagonalisation of the reference over the zero path,
    the angle sets of fixture `base` and a repeat of its first set (a rank-deficient
    overlap matrix for the subspace step)."""
    fx = dict(np.load(os.path.join(OUT, base + ".npz")))
    if base.startswith("syn"):
        N = int(fx["N"])
        h1, g2 = synthetic_integrals(N, int(fx["seed"]))
        nq, init, nuclear = 2 * N, [(int(fx["hf"]), 1.0, 0.0)], 0.0
    else:
        h1, g2 = fx["h1"], fx["g2"]
        nq, nuclear = int(fx["nq"]), float(fx["nuclear"])
        init = [(int(i), float(r), float(m)) for i, r, m in
                zip(fx["init_idx"], fx["init_re"], fx.get("init_im", np.zeros(len(fx["init_idx"]))))]
    sets = [np.asarray(a) for a in fx["angles"]] + [np.asarray(fx["angles"][0])]
    P = int(np.asarray(fx["order_1b"]).max())
    with tempfile.TemporaryDirectory() as td:
        prefix = os.path.join(td, "p")
        write_integrals(prefix, h1, g2)
        sp = spec(nq, init, np.asarray(fx["ops_1b"]) - 1, np.asarray(fx["order_1b"]) - 1, fx["scale"],
                  [f"ham ints {prefix}"], sets, want=(1, 0, 0, 0), nuclear=nuclear)
        sp += [f"properties {prefix}", f"subspace {len(sets)}"]
        sf, of = os.path.join(td, "spec"), os.path.join(td, "out")
        open(sf, "w").write("\n".join(sp) + "\nend\n")
        r = subprocess.run([DRV + ("_cplx" if cplx else ""), sf, of], check=True, capture_output=True, text=True,
                           env=dict(os.environ, OMP_NUM_THREADS="4"))
        npath = len(sets) + 1
        rows = np.full((len(PROPERTY_ROWS), npath), np.nan)
        ov = np.zeros(npath, dtype=complex)
        for ln in open(prefix + "_table.txt").read().splitlines():
            name = ln[:40].strip()
            if name not in PROPERTY_ROWS:
                continue
            vals = [float(t) for t in ln[40:].replace(",", " ").split()]
            if name == "OverlapWithState_0":
                ov = np.array(vals[0::2]) + 1j * np.array(vals[1::2]) if cplx else np.array(vals, dtype=complex)
                rows[PROPERTY_ROWS.index(name)] = ov.real
            else:
                rows[PROPERTY_ROWS.index(name)] = vals
        hess = np.stack([np.fromfile(f"{prefix}_Path_{k}_Hessian.Matbin").reshape(P, P) for k in range(npath)])
        met = []
        for k in range(npath):
            if cplx:
                m = np.fromfile(f"{prefix}_Path_{k}_Metric.CMatbin").reshape(P, P, 2)
                met.append(m[..., 0])
            else:
                met.append(np.fromfile(f"{prefix}_Path_{k}_Metric.Matbin").reshape(P, P))
        lines = r.stderr.splitlines()
        k = next(i for i, ln in enumerate(lines) if "Rank of Null space of overlap matrix" in ln)
        null_rank = int(lines[k].split(":")[-1])
        sub = np.array([float(t) for t in lines[k + 1].split()])
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), base=base, sets=np.array(sets), rows=rows,
                        row_names=np.array(PROPERTY_ROWS), overlap=ov, hess=hess, metric=np.stack(met),
                        subspace_eigs=sub, subspace_null_rank=null_rank)
    print(tag, rows[0], ov, sub, null_rank)


def sector_list(N, na, nb):
    """Ascending bitstrings of the (na alpha, nb beta) sector (alpha = high N bits)."""
    pc = np.array([bin(v).count("1") for v in range(1 << N)], dtype=np.int64)
    a = np.flatnonzero(pc == na).astype(np.uint32)
    b = np.flatnonzero(pc == nb).astype(np.uint32)
    return ((a[:, None] << np.uint32(N)) | b[None, :]).ravel()


def large_case(tag, N, na, nb, layers, seed, hess, nsample=256):
    """The benchmark's own inputs at 10 / 12 / 14 orbitals (integrals of `seed`, angles
    default_rng(seed + 1).uniform(-0.1, 0.1)): energy, gradient, (Hessian), and a seeded
    sample of the final state's sector amplitudes with the state's norm."""
    h, g = synthetic_integrals(N, seed)
    ops, param, scale = tups_operators(N, layers)
    P = int(param.max())
    x = np.random.default_rng(seed + 1).uniform(-0.1, 0.1, P)
    with tempfile.TemporaryDirectory(dir=os.environ.get("AE_GOLDEN_TMP")) as td:
        prefix = os.path.join(td, "syn")
        write_integrals(prefix, h, g)
        hf = hartree_fock_index(N, na, nb)
        want = (1, 1, int(hess), 1)
        d = run(spec(2 * N, [(hf, 1.0, 0.0)], ops - 1, param - 1, scale, [f"ham ints {prefix}"], [x], want=want),
                threads=8)
    res, _ = split_outputs(d, 1, P, 1 << (2 * N), want)
    state = res["S"][0]
    del d
    sect = sector_list(N, na, nb)
    pick = np.sort(np.random.default_rng(seed + 7).choice(len(sect), nsample, replace=False))
    fx = dict(N=N, na=na, nb=nb, layers=layers, seed=seed, hf=hf, ops_1b=ops, order_1b=param, scale=scale,
              x=x, E=res["E"][0], G=res["G"][0], sample_rank=pick.astype(np.int64), sample_bits=sect[pick],
              sample_amp=state[sect[pick]], norm=float(np.dot(state, state)))
    if hess:
        fx["H"] = res["H"][0]
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), **fx)
    print(tag, fx["E"])


def lucj_case(tag, N, na, lucj_seed, ham_seed, nsample=256):
    """The complex LUCJ circuit of ansatzevolve_gb300.lucj (every operator its own
    parameter, scale 1) on the Hartree-Fock determinant, with the synthetic integrals
    of `ham_seed`: energy, gradient per operator, sampled final-state amplitudes."""
    from ansatzevolve_gb300.lucj import lucj_operators, random_lucj
    K, J = random_lucj(N, lucj_seed)
    ops, ang = lucj_operators(K, J)
    h, g = synthetic_integrals(N, ham_seed)
    P = len(ops)
    with tempfile.TemporaryDirectory(dir=os.environ.get("AE_GOLDEN_TMP")) as td:
        prefix = os.path.join(td, "lucj")
        write_integrals(prefix, h, g)
        hf = hartree_fock_index(N, na, na)
        want = (1, 1, 0, 1)
        d = run(spec(2 * N, [(hf, 1.0, 0.0)], ops, np.arange(P), np.ones(P), [f"ham ints {prefix}"], [ang],
                     want=want), cplx=True, threads=8)
    res, _ = split_outputs(d, 1, P, 1 << (2 * N), want, cplx=True)
    state = res["S"][0]
    del d
    sect = sector_list(N, na, na)
    pick = np.sort(np.random.default_rng(lucj_seed + 7).choice(len(sect), nsample, replace=False))
    amp = state[2 * sect[pick].astype(np.int64)] + 1j * state[2 * sect[pick].astype(np.int64) + 1]
    fx = dict(N=N, na=na, nb=na, lucj_seed=lucj_seed, ham_seed=ham_seed, hf=hf, ops=ops, x=ang, E=res["E"][0],
              G=res["G"][0], sample_rank=pick.astype(np.int64), sample_bits=sect[pick], sample_amp=amp,
              norm=float(np.dot(state, state)))
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), **fx)
    print(tag, fx["E"])


def pairs_case(tag, N, na, nb, layers, nsample=4096):
    """The reference's excitation rule (applyExcToBasisState_, fusedevolve.cpp:27-145)
    for every operator of the N-orbital TUPS circuit over every sector determinant in
    ascending order: per operator the SHA-256 of the partner bitstrings (uint32 LE) and
    of the signs (int8, +1 / -1; an inactive determinant is its own partner with sign
    -1, as the reference returns it), the number of active determinants, and a seeded
    sample of raw entries; plus the SHA-256 of the sector list itself."""
    import hashlib
    ops, param, scale = tups_operators(N, layers)
    hf = hartree_fock_index(N, na, nb)
    sect = sector_list(N, na, nb)
    n = len(sect)
    with tempfile.TemporaryDirectory(dir=os.environ.get("AE_GOLDEN_TMP")) as td:
        pf = os.path.join(td, "pairs")
        s = spec(2 * N, [(hf, 1.0, 0.0)], ops - 1, param - 1, scale, ["ham triplets 1", f"{hf} {hf} 1.0"],
                 [np.zeros(int(param.max()))], want=(0, 0, 0, 0))
        s.append(f"pairsfile {pf}")
        run(s)
        raw = np.fromfile(pf, dtype=np.uint8)
    assert raw.size == len(ops) * n * 5
    pick = np.sort(np.random.default_rng(17).choice(n, nsample, replace=False))
    dig_p, dig_s, active, sp, ss = [], [], [], [], []
    for k in range(len(ops)):
        blk = raw[k * n * 5:(k + 1) * n * 5]
        partner = blk[:4 * n].view("<u4")
        sign = blk[4 * n:].view(np.int8)
        dig_p.append(hashlib.sha256(partner.tobytes()).hexdigest())
        dig_s.append(hashlib.sha256(sign.tobytes()).hexdigest())
        active.append(int(np.count_nonzero(partner != sect)))
        sp.append(partner[pick])
        ss.append(sign[pick])
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), N=N, na=na, nb=nb, layers=layers, ops_1b=ops,
                        sector_sha256=hashlib.sha256(sect.astype("<u4").tobytes()).hexdigest(),
                        partner_sha256=np.array(dig_p), sign_sha256=np.array(dig_s), active=np.array(active),
                        sample_rank=pick.astype(np.int64), sample_partner=np.array(sp), sample_sign=np.array(ss))
    print(tag, len(ops), "operators over", n, "determinants; active", min(active), "..", max(active))


if __name__ == "__main__":
    single = {
        "ref10": lambda: large_case("ref10", 10, 5, 5, 3, 0, hess=True),
        "ref12": lambda: large_case("ref12", 12, 6, 6, 3, 0, hess=True),
        "ref14": lambda: large_case("ref14", 14, 7, 7, 4, 0, hess=False),
        "lucj14": lambda: lucj_case("lucj14", 14, 7, 3, 7),
        "pairs12": lambda: pairs_case("pairs12", 12, 6, 6, 3),
        "batched4": lambda: batched_case("batched4"),
        "overlaps_syn6": lambda: overlaps_case("overlaps_syn6", "syn6", 4),
        "overlaps_h4c": lambda: overlaps_case("overlaps_h4c", "h4c", 3, cplx=True),
    }
    if len(sys.argv) > 1:
        for t in sys.argv[1:]:
            if t.startswith("props_"):
                properties_case(t, t[6:], cplx=t.endswith("c"))
            else:
                single[t]()
        sys.exit(0)
    fortran_case()
    hams_case("TestFermionic", None, tag="ferm")
    hams_case("H4", "L1", optimise=True, tag="h4")
    hams_case("H4_Complex", "L1", cplx=True, tag="h4c")
    synthetic_case("syn6", 6, 3, 3, 2, 3, pairs=True)
    synthetic_case("syn8", 8, 4, 4, 2, 0)
    for t in ("ref10", "ref12", "ref14", "lucj14", "pairs12"):
        single[t]()
    for t in ("overlaps_syn6", "overlaps_h4c", "batched4"):
        single[t]()
    properties_case("props_h4", "h4")
    properties_case("props_h4c", "h4c", cplx=True)
    properties_case("props_syn6", "syn6")
