"""LUCJ decomposition (host set-up): exp(K) as the reference's Givens + phase operator
forms, checked against dense numpy exponentials; the reference-rule oracle runs the
operator list in complex mode."""
import numpy as np
import pytest
from scipy.sparse import csr_matrix
from scipy.sparse.linalg import expm_multiply

from ansatzevolve_gb300.lucj import _expm_antihermitian, lucj_operators, orbital_rotation_ops, random_lucj


def orbital_matrix(seq, N):
    """Product of the orbital matrices of an operator sequence (application order)."""
    U = np.eye(N, dtype=complex)
    for op in seq:
        M = np.eye(N, dtype=complex)
        if op[0] == "rot":
            p, q, t = op[1], op[2], op[3]
            M[p, p] = M[q, q] = np.cos(t)
            M[p, q] = np.sin(t)
            M[q, p] = -np.sin(t)
        else:
            M[op[1], op[1]] = np.exp(1j * op[2])
        U = M @ U
    return U


@pytest.mark.parametrize("N,seed", [(4, 0), (6, 1), (9, 2), (14, 3)])
def test_orbital_rotation_decomposition(N, seed):
    K, _ = random_lucj(N, seed)
    U = _expm_antihermitian(K)
    assert np.allclose(U @ U.conj().T, np.eye(N), atol=1e-13)
    seq = orbital_rotation_ops(U)
    assert np.max(np.abs(orbital_matrix(seq, N) - U)) < 1e-12
    assert sum(op[0] == "rot" for op in seq) <= N * (N - 1) // 2


def sector_states(N, na, nb):
    return np.array(sorted(z for z in range(1 << (2 * N))
                           if bin(z >> N).count("1") == na and bin(z & ((1 << N) - 1)).count("1") == nb), dtype=np.int64)


def hop_matrix(states, p, q):
    """a+_p a_q over the sector basis with Jordan-Wigner signs in qubit order."""
    pos = {int(z): i for i, z in enumerate(states)}
    rows, cols, vals = [], [], []
    lo, hi = min(p, q), max(p, q)
    between = ((1 << hi) - 1) ^ ((1 << (lo + 1)) - 1) if hi > lo else 0
    for j, z in enumerate(states):
        z = int(z)
        if not (z >> q) & 1:
            continue
        if p != q and (z >> p) & 1:
            continue
        z2 = z ^ (1 << q) ^ (1 << p)
        rows.append(pos[z2])
        cols.append(j)
        vals.append(-1.0 if bin(z & between).count("1") & 1 else 1.0)
    return csr_matrix((vals, (rows, cols)), shape=(len(states), len(states)))


def dense_lucj_state(N, na, K, J, states):
    D = len(states)
    Kh = csr_matrix((D, D), dtype=complex)
    for p in range(N):
        for q in range(N):
            if K[p, q] != 0:
                for off in (0, N):
                    Kh = Kh + K[p, q] * hop_matrix(states, p + off, q + off)
    occ = lambda o: ((states >> o) & 1).astype(float)
    jd = np.zeros(D)
    for p in range(N):
        for q in range(p, N):
            if J[p, q] == 0:
                continue
            if p == q:
                jd += J[p, p] * occ(p) * occ(p + N)
            else:
                jd += J[p, q] * (occ(p) + occ(p + N)) * (occ(q) + occ(q + N))
    hf = sum(1 << o for o in range(na)) | sum(1 << (o + N) for o in range(na))
    v = np.zeros(D, dtype=complex)
    v[np.searchsorted(states, hf)] = 1.0
    v = expm_multiply(Kh, v)
    v = np.exp(1j * jd) * v
    return expm_multiply(-Kh, v), hf


@pytest.mark.parametrize("N,na,seed", [(4, 2, 0), (6, 3, 5)])
def test_lucj_operator_list_matches_dense_exponentials(N, na, seed):
    from oracle.oracle import Oracle
    K, J = random_lucj(N, seed)
    states = sector_states(N, na, na)
    want, hf = dense_lucj_state(N, na, K, J, states)
    ops, ang = lucj_operators(K, J)
    o = Oracle(2 * N, 2, 2 * na, na, na, cplx=True)
    assert np.array_equal(o.states(), states)
    o.set_initial([hf], [1.0])
    o.set_ops(ops, np.arange(len(ops)), np.ones(len(ops)))
    got = o.evolve_ops(ang)
    got = got[0::2] + 1j * got[1::2]
    assert np.max(np.abs(got - want)) < 1e-12
