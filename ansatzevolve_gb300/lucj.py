"""LUCJ-type ansatz on the engine: exp(-K) exp(i J) exp(K) applied to a determinant.

K is an anti-Hermitian one-body matrix (the same for both spins), J a real
density-density matrix.  The reference has no exp(K) primitive, so the orbital
rotation is written in the reference's own operator forms, which the engine runs in
complex mode:

* "a b -1 -1" (0-based spin orbitals): exp(theta (a+_b a_a - a+_a a_b)) in the
  reference's sign rule (fusedevolve.cpp:27-145), a real Givens rotation whose
  orbital matrix is [[cos, sin], [-sin, cos]] on (b, a);
* "p p -1 -1": exp(i theta n_p), a phase on orbital p;
* "p q p q": exp(i theta n_p n_q), the density-density (Jastrow) phase.

A one-body exponential exp(sum K_pq a+_p a_q) maps a+_q to sum_p U_pq a+_p with
U = expm(K), and products of such operators multiply their orbital matrices.  U is
reduced to a diagonal by unitary rotations of neighbouring rows (Q_k ... Q_1 U = D,
a QR factorisation by Givens rotations), so U = Q_1^H ... Q_k^H D; each 2x2 factor
M = diag(e^{i f1}, e^{i f2}) R(theta) diag(e^{i f3}, 1) becomes one real Givens
operator between two phase operators.  Phases on one orbital are merged until a
rotation touches it.  Spin orbitals: beta p -> p, alpha p -> p + N.
No counterpart in the reference (it is host set-up code; every amplitude update runs
in the engine's kernels).
"""
import numpy as np


def _expm_antihermitian(K):
    """expm of an anti-Hermitian matrix through the eigen-decomposition of -iK."""
    w, V = np.linalg.eigh(-1j * np.asarray(K))
    return (V * np.exp(1j * w)) @ V.conj().T


def _split_2x2(M):
    """(f1, f2, theta, f3) with M = diag(e^{i f1}, e^{i f2}) R(theta) diag(e^{i f3}, 1),
    R(theta) = [[cos, sin], [-sin, cos]], for a 2x2 unitary M."""
    c, s = abs(M[0, 0]), abs(M[0, 1])
    theta = np.arctan2(s, c)
    if s < 1e-15:
        f1 = 0.0
        f3 = np.angle(M[0, 0])
        f2 = np.angle(M[1, 1])
    elif c < 1e-15:
        f3 = 0.0
        f1 = np.angle(M[0, 1])
        f2 = np.angle(-M[1, 0])
    else:
        f1 = np.angle(M[0, 1])
        f3 = np.angle(M[0, 0]) - f1
        f2 = np.angle(M[1, 1])
    return f1, f2, theta, f3


def orbital_rotation_ops(U):
    """Spatial-orbital operator sequence (application order) whose product is the
    orbital rotation U: list of ("rot", p, q, theta) and ("phase", p, phi)."""
    U = np.array(U, dtype=complex)
    N = U.shape[0]
    W = U.copy()
    Qs = []
    for j in range(N - 1):
        for i in range(N - 1, j, -1):
            x, y = W[i - 1, j], W[i, j]
            r = np.hypot(abs(x), abs(y))
            if abs(y) < 1e-15:
                continue
            # Q [x, y]^T = [r', 0]^T with Q unitary on rows (i-1, i)
            Q = np.array([[np.conj(x), np.conj(y)], [-y, x]]) / r
            W[[i - 1, i], :] = Q @ W[[i - 1, i], :]
            Qs.append((i - 1, Q))
    d = np.diag(W)
    # U = Q_1^H ... Q_k^H D: applied to a state, D acts first, then Q_k^H, ..., Q_1^H
    seq = [("phase", p, float(np.angle(d[p]))) for p in range(N)]
    for p, Q in reversed(Qs):
        f1, f2, theta, f3 = _split_2x2(Q.conj().T)
        seq += [("phase", p, f3), ("rot", p, p + 1, theta), ("phase", p, f1), ("phase", p + 1, f2)]
    # merge phases on an orbital until a rotation touches it
    out, pending = [], {}
    for op in seq:
        if op[0] == "phase":
            pending[op[1]] = pending.get(op[1], 0.0) + op[2]
            continue
        for o in (op[1], op[2]):
            ph = pending.pop(o, 0.0)
            if abs(ph) > 1e-15:
                out.append(("phase", o, ph))
        out.append(op)
    for o in sorted(pending):
        if abs(pending[o]) > 1e-15:
            out.append(("phase", o, pending[o]))
    return out


def lucj_operators(K, J):
    """Engine operators (0-based spin orbitals, -1 = absent) and their angles for
    exp(-K) exp(i J) exp(K) in application order.  J: symmetric real N x N; every
    nonzero J_pq (p <= q) gives the density-density phases of n_p n_q over the spin
    pairs (on site p = q: n_p,alpha n_p,beta)."""
    K = np.asarray(K)
    N = K.shape[0]
    ops, ang = [], []

    def emit_rotation(U):
        for op in orbital_rotation_ops(U):
            for off in (0, N):  # beta, alpha
                if op[0] == "rot":
                    ops.append((op[2] + off, op[1] + off, -1, -1))
                    ang.append(op[3])
                else:
                    ops.append((op[1] + off, op[1] + off, -1, -1))
                    ang.append(op[2])

    U = _expm_antihermitian(K)
    emit_rotation(U)
    for p in range(N):
        for q in range(p, N):
            if J[p, q] == 0:
                continue
            if p == q:
                ops.append((p + N, p, p + N, p))
                ang.append(J[p, p])
                continue
            for a in (p, p + N):
                for b in (q, q + N):
                    ops.append((a, b, a, b))
                    ang.append(J[p, q])
    emit_rotation(U.conj().T)
    return np.array(ops, dtype=np.int32), np.array(ang, dtype=np.float64)


def random_lucj(n_orb, seed, sigma=0.1):
    """K anti-Hermitian with N(0, sigma) real and imaginary parts, nearest-neighbour
    and on-site J ~ N(0, sigma) (symmetric)."""
    rng = np.random.default_rng(seed)
    A = rng.normal(0, sigma, (n_orb, n_orb)) + 1j * rng.normal(0, sigma, (n_orb, n_orb))
    K = np.triu(A, 1)
    K = K - K.conj().T + np.diag(1j * rng.normal(0, sigma, n_orb))
    J = np.zeros((n_orb, n_orb))
    for p in range(n_orb):
        J[p, p] = rng.normal(0, sigma)
        if p + 1 < n_orb:
            J[p, p + 1] = J[p + 1, p] = rng.normal(0, sigma)
    return K, J
