"""numpy restatement of the reference's DIIS coefficient step (diis.h:16-209 with
simpleNewtonRaphson, diis.cpp:11-66).  Test infrastructure only."""
import numpy as np


def pulay(B):
    """c = B^+ 1 normalised to sum 1 (minimum-norm solve), or the last unit vector when
    the sum vanishes."""
    c = np.linalg.lstsq(B, np.ones(len(B)), rcond=None)[0]
    s = c.sum()
    if s == 0:
        c = np.zeros(len(B))
        c[-1] = 1.0
        return c
    return c / s


def ediis(B):
    """c_i = t_i^2 at the stationary point of t^2.B t^2 - lam (sum t^2 - 1) that Newton
    with eigenvalue-filtered steps and gradient-norm backtracking reaches from
    t = sqrt(n), lam = 1."""
    n = len(B)
    pt = np.full(n + 1, np.sqrt(n))
    pt[n] = 1.0

    def grad(p):
        t, lam = p[:n], p[n]
        g = np.empty(n + 1)
        g[:n] = 4 * (B @ t**2) * t - 2 * lam * t
        g[n] = 1 - (t**2).sum()
        return g

    def hess(p):
        t, lam = p[:n], p[n]
        H = np.zeros((n + 1, n + 1))
        H[:n, :n] = 8 * np.outer(t, t) * B + np.diag(4 * (B @ t**2) - 2 * lam)
        H[n, :n] = H[:n, n] = -2 * t
        return H

    for _ in range(200):
        g = grad(pt)
        gn = np.linalg.norm(g)
        if gn < 1e-12:
            break
        w, V = np.linalg.eigh(hess(pt))
        inv = np.where(np.abs(w) < 1e-6, 0.0, 1 / np.where(np.abs(w) < 1e-6, 1.0, w))
        step = -(V @ (inv * (V.T @ g)))
        pt = pt + step
        while np.linalg.norm(grad(pt)) > gn and np.abs(step).max() > 1e-15:
            step = step / 2
            pt = pt - step
        if not np.abs(step).max() > 1e-15:
            break
    return pt[:n] ** 2
