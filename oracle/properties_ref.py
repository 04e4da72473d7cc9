"""numpy restatement of the reference's per-path properties and subspace
diagonalisation (TUPSQuantities::writeProperties, tupsquantities.cpp:185-568;
doSubspaceDiagonalisation, :1600-1700), on top of the oracle (oracle.Oracle).

Test infrastructure only: used by tests/ to check the product's properties entry points
and pinned against the reference's own output (tests/golden/props_*.npz).  The metric
here comes from central differences of the oracle's final states, independently of the
analytic tangents the product uses.
"""
import numpy as np

ZERO = 1e-10        # tupsquantities.cpp:468
SUBSPACE_EPS = 1e-14  # :1660


def decompress(x, param0, scale):
    return np.asarray(scale) * np.asarray(x)[np.asarray(param0)]


def _cvec(o, v):
    return v if not o.cplx else v[0::2] + 1j * v[1::2]


def dense_h(o):
    """The oracle's sector Hamiltonian as a dense matrix (small cases)."""
    rp, col, val = o.csr()
    H = np.zeros((o.D, o.D))
    for i in range(o.D):
        H[i, col[rp[i]:rp[i + 1]]] += val[rp[i]:rp[i + 1]]
    return H


def lowest_eigenpair(o):
    w, V = np.linalg.eigh(dense_h(o))
    return w[0], V[:, 0]


def metric_fd(o, x, param0, scale, h=1e-5):
    """Re(J^dagger J) with J_mu = d psi / d x_mu by central differences."""
    x = np.asarray(x, dtype=float)
    cols = []
    for mu in range(len(x)):
        xp, xm = x.copy(), x.copy()
        xp[mu] += h
        xm[mu] -= h
        d = (o.evolve_ops(decompress(xp, param0, scale)) - o.evolve_ops(decompress(xm, param0, scale))) / (2 * h)
        cols.append(d)
    J = np.array(cols).T  # real view: re / im interleaved, so J^T J = Re(J^dagger J)
    return J.T @ J


def _counts(values):
    v = np.asarray(values)
    return (v < -ZERO).sum(), ((v >= -ZERO) & (v <= ZERO)).sum(), (v > ZERO).sum()


def path_row(o, x, param0, scale, nuclear=0.0, ground=None):
    """The table's rows for one path, in the reference's print order (NaN for the
    overlap rows without a ground state); plus the Hessian and metric."""
    th = decompress(x, param0, scale)
    E, g = o.gradient_comp(x)
    H = o.hessian_comp(x)
    M = metric_fd(o, x, param0, scale)
    psi = _cvec(o, o.evolve_ops(th))
    if o.cplx:
        r = psi.real
        hr = o.apply_h(np.column_stack([r, np.zeros_like(r)]).ravel())[0::2]
        realE = hr @ r / (r @ r)
    else:
        realE = E
    hneg, hzero, hpos = _counts(np.linalg.eigvalsh(H))
    dneg, dzero, dpos = _counts(np.diag(H))
    mw = np.linalg.eigvalsh(M)
    row = [E, realE, E + nuclear, hneg, hzero, hpos, dneg, dzero, dpos,
           (mw > ZERO).sum(), ((mw >= -ZERO) & (mw <= ZERO)).sum(), (np.abs(np.diag(M)) <= ZERO).sum(),
           np.linalg.norm(g)]
    if ground is not None:
        ov = np.vdot(psi, ground)
        row += [ov.real, ov.imag, abs(ov)]
    else:
        row += [np.nan] * 3
    return np.array(row, dtype=float), H, M


def subspace_eigenvalues(o, sets_ops):
    """Eigenvalues of S^-1/2 H S^-1/2 over the states of the angle sets, S's eigenvalues
    below 1e-14 dropped to 0 (their directions give eigenvalue 0), and the null rank."""
    states = np.array([_cvec(o, o.evolve_ops(a)) for a in sets_ops])
    hstates = []
    for a in sets_ops:
        hv = o.apply_h(o.evolve_ops(a))
        hstates.append(_cvec(o, hv))
    hstates = np.array(hstates)
    S = states.conj() @ states.T
    Hm = states.conj() @ hstates.T
    ws, Vs = np.linalg.eigh(S)
    null = int((ws < SUBSPACE_EPS).sum())
    f = np.where(ws < SUBSPACE_EPS, 0.0, 1.0 / np.sqrt(np.maximum(ws, SUBSPACE_EPS)))
    X = (Vs * f) @ Vs.conj().T
    Y = X @ Hm @ X
    return np.linalg.eigvalsh(0.5 * (Y + Y.conj().T)), null
