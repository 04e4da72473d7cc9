"""Seeded synthetic inputs for the TUPS workloads (no external data set is used).

* ``synthetic_integrals``: random molecular-orbital integrals with the shapes and
  value distributions of the benchmark configurations: h_pq symmetric N(0,1) damped
  by exp(-|p-q|/2); g_pqrs = sum_k L^k_pq L^k_rs with symmetric L^k ~ N(0, 0.3),
  which is 8-fold symmetric.  Arrays are in the layout the reference reads from
  ``<prefix>_oneEInts.bin`` / ``<prefix>_twoEInts.bin``
  (hamiltonianmatrix.cpp:423-453): h[p, q] and g[p, q, r, s] = (pq|rs), C order.
* ``tups_operators``: the tUPS circuit of python/makeOperators.py (non-U3 branch,
  ``buildAnsatzToPython`` :318-383) without the first-layer angle sharing: per
  layer the pairs (1,2),(3,4),... then (2,3),(4,5),...; per pair an alpha+beta
  single sharing one angle, a paired double, and another alpha+beta single.
* ``hartree_fock_index``: the determinant with the lowest Nalpha / Nbeta orbitals
  occupied; qubit k < N is beta, k >= N is alpha (operatorpool.cpp:221-230).
"""
import numpy as np


def synthetic_integrals(n_orb, seed=0, n_factors=None):
    rng = np.random.default_rng(seed)
    k = n_orb if n_factors is None else n_factors
    a = rng.normal(0.0, 1.0, (n_orb, n_orb))
    p = np.arange(n_orb)
    h = 0.5 * (a + a.T) * np.exp(-np.abs(p[:, None] - p[None, :]) / 2.0)
    g = np.zeros((n_orb,) * 4)
    for _ in range(k):
        l = rng.normal(0.0, 0.3, (n_orb, n_orb))
        l = 0.5 * (l + l.T)
        g += np.einsum("pq,rs->pqrs", l, l)
    return np.ascontiguousarray(h), np.ascontiguousarray(g)


def family_tensors(n_orb, seed=0, n_factors=None, pert=1.0):
    """The seeded base and perturbation tensors of family_integrals: (damp, a0, a1,
    [(l0, l1)] * n_factors), drawn in a fixed order."""
    rng = np.random.default_rng(seed)
    k = n_orb if n_factors is None else n_factors
    p = np.arange(n_orb)
    damp = np.exp(-np.abs(p[:, None] - p[None, :]) / 2.0)
    a0 = rng.normal(0.0, 1.0, (n_orb, n_orb))
    a1 = rng.normal(0.0, pert, (n_orb, n_orb))
    ls = []
    for _ in range(k):
        l0 = rng.normal(0.0, 0.3, (n_orb, n_orb))
        l1 = rng.normal(0.0, 0.3 * pert, (n_orb, n_orb))
        ls.append((l0, l1))
    return damp, a0, a1, ls


def family_integrals_from(tensors, s):
    """family_integrals at s from tensors drawn once by family_tensors."""
    damp, a0, a1, ls = tensors
    h = 0.5 * ((a0 + s * a1) + (a0 + s * a1).T) * damp
    g = np.zeros((a0.shape[0],) * 4)
    for l0, l1 in ls:
        l = l0 + s * l1
        l = 0.5 * (l + l.T)
        g += np.multiply.outer(l, l)  # g_pqrs += l_pq l_rs
    return np.ascontiguousarray(h), np.ascontiguousarray(g)


def family_integrals_batch(tensors, svals):
    """family_integrals_from at every s in svals at once: (h [S, N, N], g [S, N, N, N, N]).
    Each element goes through the same operations in the same order as the one-at-a-time
    form, so the two agree bit for bit."""
    damp, a0, a1, ls = tensors
    s = np.asarray(svals, dtype=np.float64).reshape(-1, 1, 1)
    a = a0 + s * a1
    h = 0.5 * (a + a.transpose(0, 2, 1)) * damp
    N = a0.shape[0]
    g = np.zeros((s.shape[0],) + (N,) * 4)
    lk = []
    for l0, l1 in ls:
        l = l0 + s * l1
        lk.append(0.5 * (l + l.transpose(0, 2, 1)))
    # a few instances at a time, so that the outer-product temporary stays in cache
    chunk = 8
    tmp = np.empty((chunk,) + (N,) * 4)
    for c in range(0, s.shape[0], chunk):
        gc = g[c:c + chunk]
        t = tmp[:gc.shape[0]]
        for l in lk:
            lc = l[c:c + chunk]
            np.multiply(lc[:, :, :, None, None], lc[:, None, None, :, :], out=t)
            gc += t
    return np.ascontiguousarray(h), g


def family_h_and_coulomb_batch(tensors, svals):
    """h(s) [S, N, N] and the Coulomb diagonal g_ppqq(s) [S, N, N] of family_integrals_from
    at every s in svals, without forming g (bit-identical to slicing it)."""
    damp, a0, a1, ls = tensors
    s = np.asarray(svals, dtype=np.float64).reshape(-1, 1, 1)
    a = a0 + s * a1
    h = 0.5 * (a + a.transpose(0, 2, 1)) * damp
    N = a0.shape[0]
    d = np.zeros((s.shape[0], N, N))
    for l0, l1 in ls:
        l = l0 + s * l1
        l = 0.5 * (l + l.transpose(0, 2, 1))
        dg = np.diagonal(l, axis1=1, axis2=2)
        d += dg[:, :, None] * dg[:, None, :]
    return np.ascontiguousarray(h), d


def family_integrals(n_orb, s, seed=0, n_factors=None, pert=1.0):
    """h(s) = h0 + s*h1 and L^k(s) = L^k0 + s*L^k1 for a Hamiltonian family scan; the
    perturbation tensors h1, L^k1 are drawn at `pert` times the base tensors' scale."""
    return family_integrals_from(family_tensors(n_orb, seed, n_factors, pert), s)


def tups_operators(n_orb, layers):
    """Operators (1-based, 0 = absent, file convention) and order (1-based param, scale)."""
    ops, order = [], []
    param = 1

    def pair(p, q):
        nonlocal param
        ops.extend([[p, q, 0, 0], [p + n_orb, q + n_orb, 0, 0]])
        order.extend([(param, 1.0), (param, 1.0)])
        param += 1
        ops.append([p, p + n_orb, q, q + n_orb])
        order.append((param, 1.0))
        param += 1
        ops.extend([[p, q, 0, 0], [p + n_orb, q + n_orb, 0, 0]])
        order.extend([(param, 1.0), (param, 1.0)])
        param += 1

    for _ in range(layers):
        for p in range(1, n_orb, 2):
            if p + 1 <= n_orb:
                pair(p, p + 1)
        for p in range(2, n_orb, 2):
            if p + 1 <= n_orb:
                pair(p, p + 1)
    return np.array(ops, dtype=np.int32), np.array([o[0] for o in order], dtype=np.int32), \
        np.array([o[1] for o in order], dtype=np.float64)


def hartree_fock_index(n_orb, n_alpha, n_beta):
    beta = (1 << n_beta) - 1
    alpha = ((1 << n_alpha) - 1) << n_orb
    return alpha | beta


def write_integrals(prefix, h, g):
    np.asarray(h, dtype="<f8").tofile(prefix + "_oneEInts.bin")
    np.asarray(g, dtype="<f8").tofile(prefix + "_twoEInts.bin")
