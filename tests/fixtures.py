"""Shared problem builders for the tests: turn a golden fixture (or a synthetic
configuration) into the inputs of the oracle and of the product API."""
import numpy as np

from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals, tups_operators


def sector_of(nq, init_idx, ops0):
    """(kind, ne, na, nb) the way stateAnsatzManager::construct picks its compressor
    (AnsatzManager.cpp:90-101, storeInitial :271-374, setOperatorSymmetry :202-237)."""
    N = nq // 2
    init_idx = [int(i) for i in init_idx]
    ne = bin(init_idx[0]).count("1")
    same_n = all(bin(i).count("1") == ne for i in init_idx)
    na = bin(init_idx[0] >> N).count("1")
    nb = bin(init_idx[0] & ((1 << N) - 1)).count("1")
    sz = nq % 2 == 0 and all(bin(i >> N).count("1") == na and bin(i & ((1 << N) - 1)).count("1") == nb for i in init_idx)
    dn = (1 << N) - 1
    up = ((1 << nq) - 1) ^ dn
    for e in ops0:
        a, b, c, d = [int(x) for x in e]
        if c < 0:
            cr, de = 1 << a, 1 << b
        else:
            cr, de = (1 << a) | (1 << b), (1 << c) | (1 << d)
        if bin(cr & up).count("1") != bin(de & up).count("1") or bin(cr & dn).count("1") != bin(de & dn).count("1"):
            sz = False
    if not same_n:
        return 0, 0, 0, 0
    return (2 if sz else 1), ne, na, nb


def oracle_from_golden(fx, cplx=False):
    from oracle.oracle import Oracle
    nq = int(fx["nq"])
    ops0 = np.asarray(fx["ops_1b"]) - 1
    kind, ne, na, nb = sector_of(nq, fx["init_idx"], ops0)
    o = Oracle(nq, kind, ne, na, nb, cplx)
    o.set_initial(fx["init_idx"], fx["init_re"], fx.get("init_im"))
    o.set_ops(ops0, np.asarray(fx["order_1b"]) - 1, fx["scale"])
    if "h1" in fx:
        o.set_ham_integrals(fx["h1"], fx["g2"], csr=True)
    else:
        o.set_ham_triplets(np.asarray(fx["ham_i_1b"]) - 1, np.asarray(fx["ham_j_1b"]) - 1, fx["ham_v"])
    return o


def synthetic_problem(N, na, nb, layers, seed):
    h, g = synthetic_integrals(N, seed)
    ops, param, scale = tups_operators(N, layers)
    return dict(N=N, nq=2 * N, na=na, nb=nb, h1=h, g2=g, ops_1b=ops, order_1b=param, scale=scale,
                hf=hartree_fock_index(N, na, nb))


def oracle_synthetic(pb, csr=True):
    from oracle.oracle import Oracle
    o = Oracle(pb["nq"], 2, pb["na"] + pb["nb"], pb["na"], pb["nb"])
    o.set_initial([pb["hf"]], [1.0])
    o.set_ops(np.asarray(pb["ops_1b"]) - 1, np.asarray(pb["order_1b"]) - 1, pb["scale"])
    o.set_ham_integrals(pb["h1"], pb["g2"], csr=csr)
    return o
