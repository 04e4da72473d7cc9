"""Learned warm start for the TUPS optimiser.

A small MLP maps a Hamiltonian's integrals to starting angles.  Features are the
flattened one-electron integrals h_pq and the Coulomb-like diagonal g_ppqq; targets
are converged compressed angles produced by the engine itself.  The network is
trained and run by the project's CUDA kernels (aegpu_mlp_*: BF16 weights, FP32
accumulation, Adam, MSE).  Every proposal is screened by the engine: an instance starts
from the proposal only if its energy there is below the energy at the plain start,
so the optimiser's converged answer is decided by the engine, not by the network.
No counterpart in the reference.
"""
import ctypes

import numpy as np

from . import AegpuError, _FP, _P, lib


def features(h1, g2):
    """[h_pq flattened, g_ppqq flattened] for one Hamiltonian (N*N + N*N values)."""
    h1 = np.asarray(h1, dtype=np.float64)
    g2 = np.asarray(g2, dtype=np.float64)
    N = h1.shape[0]
    g = g2.reshape(N, N, N, N)
    diag = g[np.arange(N)[:, None], np.arange(N)[:, None], np.arange(N)[None, :], np.arange(N)[None, :]]
    return np.concatenate([h1.reshape(-1), diag.reshape(-1)])


def _fp(a):
    return a.ctypes.data_as(_FP)


class Mlp:
    """The aegpu_mlp C ABI: n_in -> hidden -> hidden -> n_out, GELU."""

    def __init__(self, n_in, n_out, hidden=512, seed=0):
        self.L = lib()
        h = _P()
        rc = self.L.aegpu_mlp_create(ctypes.byref(h), int(n_in), int(hidden), int(n_out), int(seed))
        if rc:
            raise AegpuError("aegpu_mlp_create failed (%d)" % rc)
        self.h = h
        self.n_in, self.n_out, self.hidden = int(n_in), int(n_out), int(hidden)

    def _check(self, rc):
        if rc:
            raise AegpuError("aegpu mlp error %d: %s" % (rc, self.L.aegpu_mlp_last_error(self.h).decode()))

    def close(self):
        if getattr(self, "h", None):
            self.L.aegpu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def num_params(self):
        return int(self.L.aegpu_mlp_num_params(self.h))

    def set_scaling(self, in_mean, in_scale, out_mean, out_scale):
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (in_mean, in_scale, out_mean, out_scale)]
        self._check(self.L.aegpu_mlp_set_scaling(self.h, *[_fp(a) for a in arrs]))

    def fit_scaling(self, X, T):
        """Standardise inputs and targets by their training-set mean and spread."""
        X = np.asarray(X, dtype=np.float64)
        T = np.asarray(T, dtype=np.float64)
        xs = X.std(axis=0)
        ts = T.std(axis=0)
        self.set_scaling(X.mean(axis=0), np.where(xs > 1e-8, xs, 1.0), T.mean(axis=0), np.where(ts > 1e-8, ts, 1.0))

    def get_params(self):
        p = np.zeros(self.num_params(), dtype=np.float32)
        self._check(self.L.aegpu_mlp_get_params(self.h, _fp(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params()
        self._check(self.L.aegpu_mlp_set_params(self.h, _fp(p)))

    def train(self, X, T, epochs, batch=128, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        n = X.shape[0]
        assert X.shape == (n, self.n_in) and T.shape == (n, self.n_out)
        loss = np.zeros(max(1, epochs), dtype=np.float32)
        self._check(self.L.aegpu_mlp_train(self.h, _fp(X), _fp(T), n, int(epochs), int(batch), float(lr), int(seed),
                                           _fp(loss)))
        return loss[:epochs]

    def loss_grad(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        g = np.zeros(self.num_params(), dtype=np.float32)
        self._check(self.L.aegpu_mlp_loss_grad(self.h, _fp(X), _fp(T), X.shape[0], _fp(loss), _fp(g)))
        return float(loss[0]), g

    def predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], self.n_out), dtype=np.float32)
        self._check(self.L.aegpu_mlp_predict(self.h, _fp(X), X.shape[0], _fp(Y)))
        return Y


def screened_starts(engine, proposals, param0, scale, plain=None):
    """Per instance of a batched engine, the start to optimise from: the network's
    proposal where the engine finds a lower energy there than at the plain start
    (zeros unless given), else the plain start.  Returns (starts, used_proposal)."""
    proposals = np.asarray(proposals, dtype=np.float64)
    nb, P = proposals.shape
    plain = np.zeros((nb, P)) if plain is None else np.asarray(plain, dtype=np.float64)
    p0 = np.asarray(param0)
    sc = np.asarray(scale, dtype=np.float64)
    Ep = engine.energy(sc * proposals[:, p0])
    Ez = engine.energy(sc * plain[:, p0])
    Ep, Ez = np.atleast_1d(Ep), np.atleast_1d(Ez)
    use = Ep < Ez
    return np.where(use[:, None], proposals, plain), use


# ------------------------------------------------------------------ pipeline --
def family_engine(n_orb, n_alpha, layers, nb, integrals=None, mode=None):
    """A batched engine for the TUPS ansatz on a Hamiltonian family: nb instances with
    their own integrals (list of (h1, g2)), Hartree-Fock start, compressed
    parameters (param0, scale).  Returns (engine, param0, scale)."""
    from . import BASIS_SZ, HAM_ON_THE_FLY, Engine
    from .synthetic import hartree_fock_index, tups_operators
    ops, param, scale = tups_operators(n_orb, layers)
    e = Engine(2 * n_orb, BASIS_SZ, 2 * n_alpha, n_alpha, n_alpha, np.asarray(ops) - 1)
    init = np.zeros(e.D)
    init[np.searchsorted(e.states(), hartree_fock_index(n_orb, n_alpha, n_alpha))] = 1.0
    e.set_initial(init)
    if nb > 1:
        e.set_batch(nb)
    if integrals is not None:
        e.set_ham_integrals_batch(np.stack([h for h, _ in integrals]), np.stack([g for _, g in integrals]),
                                  HAM_ON_THE_FLY if mode is None else mode)
    return e, np.asarray(param) - 1, np.asarray(scale, dtype=np.float64)


def converge_batch(n_orb, n_alpha, layers, integrals, starts=None, gtol=1e-6, chunk=256, mode=None):
    """Converged compressed angles for every Hamiltonian in `integrals`, optimised in
    batches of `chunk` instances by the lockstep BFGS (zero start unless given).
    Returns (x [n, P], E [n], |g| [n])."""
    xs, Es, gs = [], [], []
    for c0 in range(0, len(integrals), chunk):
        part = integrals[c0:c0 + chunk]
        e, p0, sc = family_engine(n_orb, n_alpha, layers, len(part), part, mode)
        P = int(p0.max()) + 1
        x0 = np.zeros((len(part), P)) if starts is None else np.asarray(starts[c0:c0 + chunk], dtype=np.float64)
        x, E, gn, _, _ = e.optimise_batch(x0.reshape(len(part), P), p0, sc, gtol=gtol)
        xs.append(x.reshape(len(part), P))
        Es.append(np.atleast_1d(E))
        gs.append(np.atleast_1d(gn))
        e.close()
    return np.concatenate(xs), np.concatenate(Es), np.concatenate(gs)


def train_warmstart(feats, targets, hidden=512, epochs=400, batch=128, lr=1e-3, seed=0):
    """Train the MLP features -> converged angles on the GPU; returns (model, loss history)."""
    feats = np.asarray(feats, dtype=np.float64)
    targets = np.asarray(targets, dtype=np.float64)
    m = Mlp(feats.shape[1], targets.shape[1], hidden=hidden, seed=seed)
    m.fit_scaling(feats, targets)
    hist = m.train(feats, targets, epochs=epochs, batch=batch, lr=lr, seed=seed + 1)
    return m, hist


# ------------------------------------------------------------- family scans --
class FamilySpec:
    """A TUPS ansatz over a Hamiltonian family h(s) = h0 + s h1, L^k(s) = L^k0 + s L^k1
    (synthetic.family_integrals with a fixed seed).  pert: scale of the perturbation
    tensors relative to the base ones (0.25 keeps s in [0, 1] a smooth scan; at 1.0 the
    continuation branch changes every few hundredths of s)."""

    def __init__(self, n_orb=10, n_alpha=5, layers=3, seed=0, pert=0.25):
        from .synthetic import tups_operators
        self.n_orb, self.n_alpha, self.layers, self.seed, self.pert = n_orb, n_alpha, layers, seed, pert
        ops, param, scale = tups_operators(n_orb, layers)
        self.param0 = np.asarray(param) - 1
        self.scale = np.asarray(scale, dtype=np.float64)
        self.P = int(self.param0.max()) + 1

    def tensors(self):
        from .synthetic import family_tensors
        if getattr(self, "_tensors", None) is None:
            self._tensors = family_tensors(self.n_orb, seed=self.seed, pert=self.pert)
        return self._tensors

    def integrals(self, s):
        from .synthetic import family_integrals_from
        return family_integrals_from(self.tensors(), float(s))

    def integrals_batch(self, svals):
        """(h [S, N, N], g [S, N, N, N, N]) at every s, bit-identical to integrals(s)."""
        from .synthetic import family_integrals_batch
        return family_integrals_batch(self.tensors(), svals)

    def features(self, svals):
        """features(*integrals(s)) for every s (bit-identical), without forming g."""
        from .synthetic import family_h_and_coulomb_batch
        h, d = family_h_and_coulomb_batch(self.tensors(), svals)
        return np.concatenate([h.reshape(len(h), -1), d.reshape(len(d), -1)], axis=1)

    def engine(self, nb=1, integrals=None, mode=None):
        e, _, _ = family_engine(self.n_orb, self.n_alpha, self.layers, nb, integrals, mode)
        return e


def scan_origin(spec, n_starts=64, seed=5, s0=0.0, gtol=1e-6):
    """The scan's starting member: the lowest minimum at s = s0 among a batched BFGS
    multi-start (zero angles plus n_starts - 1 seeded U(-1, 1) starts), polished by the
    reference's Newton method.  Following the lowest branch makes the scan smooth where
    a single Newton run from zero angles lands on a higher branch with jumps.
    Returns (x0, E0)."""
    from . import HAM_STORED
    P = spec.P
    ints = spec.integrals(s0)
    e = spec.engine(n_starts, [ints] * n_starts, HAM_STORED)
    starts = np.vstack([np.zeros(P), np.random.default_rng(seed).uniform(-1.0, 1.0, (n_starts - 1, P))])
    xs, Es, _, _, _ = e.optimise_batch(starts, spec.param0, spec.scale, gtol=gtol, max_rounds=5000)
    e.close()
    best = int(np.argmin(Es))
    e1 = spec.engine(1)
    e1.set_ham_integrals(*ints, HAM_STORED)
    x0, E0, _, _, _ = e1.optimise_newton(xs[best], spec.param0, spec.scale, gtol=gtol)
    e1.close()
    return x0, E0


def scan_newton(spec, svals, x_start, gtol=1e-6, mode=None):
    """The plain path of a family scan: one instance at a time in the given order,
    each optimised by the reference's Newton method from the previous instance's
    converged angles (x_start for the first).  Returns (x [M, P], E [M], seconds of
    optimisation, Hessian evaluations, energy evaluations)."""
    import time
    from . import HAM_STORED
    e = spec.engine(1)
    x = np.asarray(x_start, dtype=np.float64).copy()
    xs, Es, t, nh, ne = [], [], 0.0, 0, 0
    for s in svals:
        e.set_ham_integrals(*spec.integrals(s), HAM_STORED if mode is None else mode)
        t0 = time.perf_counter()
        x, E, gn, h, n = e.optimise_newton(x, spec.param0, spec.scale, gtol=gtol)
        t += time.perf_counter() - t0
        xs.append(x.copy())
        Es.append(E)
        nh += h
        ne += n
    e.close()
    return np.array(xs), np.array(Es), t, nh, ne


def scan_bfgs_chain(spec, svals, x_start, gtol=1e-8, mode=None):
    """Training targets: a continuation chain over the given order, each instance
    optimised by BFGS from the previous converged angles and inverse Hessian (the
    first from x_start with the inverse of the analytic Hessian there)."""
    from . import HAM_STORED
    e = spec.engine(1)
    x = np.asarray(x_start, dtype=np.float64).reshape(1, -1).copy()
    hinv = None
    xs, Es, gs, its = [], [], [], []
    for s in svals:
        e.set_ham_integrals(*spec.integrals(s), HAM_STORED if mode is None else mode)
        if hinv is None:
            hinv = np.ascontiguousarray(inverse_hessian(e, x[0], spec)[None])
        x, E, gn, it, r = e.optimise_batch(x, spec.param0, spec.scale, gtol=gtol, max_rounds=5000, hinv=hinv)
        xs.append(x[0].copy())
        Es.append(float(np.atleast_1d(E)[0]))
        gs.append(float(np.atleast_1d(gn)[0]))
        its.append(int(it[0]))
    e.close()
    return np.array(xs), np.array(Es), np.array(gs), np.array(its)


def scan_segmented_chain(spec, svals, x_start, n_seg=32, gtol=1e-8, mode=None, predict=True):
    """Training targets as a two-level continuation over the given (sorted) s values:
    a sequential BFGS chain over n_seg segment heads (every L-th value, L = ceil(M /
    n_seg)), then every segment walked at once -- step t optimises the t-th member of
    all segments in one lockstep batch, each instance from its predecessor's converged
    angles and final inverse Hessian (on-the-fly H per instance).  The same
    continuation as scan_bfgs_chain, with n_seg + L sequential solves instead of M.
    predict: start each solve from the secant predictor through the two previous
    converged points of its chain, x1 + (x1 - x2) (s - s1) / (s1 - s2) (the
    predictor-corrector continuation of Allgower & Georg, Introduction to Numerical
    Continuation Methods, ch. 2), instead of the previous point; the minima reached are
    the same (to the tolerance), the solves shorter.
    Returns (x [M, P], E [M], |g| [M], iterations [M])."""
    from . import HAM_ON_THE_FLY, HAM_STORED
    svals = np.asarray(svals, dtype=np.float64)
    M = len(svals)
    L = -(-M // n_seg)
    heads = np.arange(0, M, L)
    ends = np.append(heads[1:], M)  # one past each segment's last member
    S = len(heads)
    P = spec.P
    xs, Es, gs, its = np.zeros((M, P)), np.zeros(M), np.zeros(M), np.zeros(M, dtype=np.int64)
    # level 1: the heads, one after the other
    e1 = spec.engine(1)
    x = np.asarray(x_start, dtype=np.float64).reshape(1, -1).copy()
    hinv = None
    hinv_heads = np.zeros((S, P, P))
    for k, h in enumerate(heads):
        e1.set_ham_integrals(*spec.integrals(svals[h]), HAM_STORED if mode is None else mode)
        if hinv is None:
            hinv = np.ascontiguousarray(inverse_hessian(e1, x[0], spec)[None])
        if predict and k >= 2:
            h1, h2 = heads[k - 1], heads[k - 2]
            x = (xs[h1] + (xs[h1] - xs[h2]) * (svals[h] - svals[h1]) / (svals[h1] - svals[h2])).reshape(1, -1)
        x, E, gn, it, _ = e1.optimise_batch(x, spec.param0, spec.scale, gtol=gtol, max_rounds=5000, hinv=hinv)
        xs[h], Es[h], gs[h], its[h] = x[0], np.atleast_1d(E)[0], np.atleast_1d(gn)[0], it[0]
        hinv_heads[k] = hinv[0]
    e1.close()
    # level 2: all segments in lockstep; a finished segment repeats its last member,
    # which is already converged and drops out of the launches at once
    eb = spec.engine(S)
    X = xs[heads].copy()
    H = np.ascontiguousarray(hinv_heads)
    s_cur = svals[heads].copy()
    X_prev = s_prev = None
    for t in range(1, L):
        idx = np.minimum(heads + t, ends - 1)
        live = heads + t < ends
        eb.set_ham_integrals_batch(*spec.integrals_batch(svals[idx]), HAM_ON_THE_FLY if mode is None else mode)
        start = X
        if predict and X_prev is not None:
            ds = s_cur - s_prev
            ratio = np.where(live & (ds != 0), (svals[idx] - s_cur) / np.where(ds != 0, ds, 1.0), 0.0)
            start = X + (X - X_prev) * ratio[:, None]
        Xn, E, gn, it, _ = eb.optimise_batch(start, spec.param0, spec.scale, gtol=gtol, max_rounds=5000, hinv=H)
        X_prev, s_prev = X, s_cur
        X, s_cur = Xn, np.where(live, svals[idx], s_cur)
        E, gn = np.atleast_1d(E), np.atleast_1d(gn)
        xs[idx[live]], Es[idx[live]], gs[idx[live]], its[idx[live]] = X[live], E[live], gn[live], it[live]
    eb.close()
    return xs, Es, gs, its


def inverse_hessian(engine, x, spec, floor=1e-3):
    """|H|^-1 over the eigenpairs of the analytic Hessian at x (eigenvalues below
    floor * max |lambda| raised to it): the initial inverse Hessian of warm BFGS."""
    _, _, H = engine.hessian(spec.scale * np.asarray(x)[spec.param0], spec.param0, spec.scale)
    H = 0.5 * (H + H.T)
    w, V = np.linalg.eigh(H)
    a = np.maximum(np.abs(w), floor * np.abs(w).max())
    return (V / a) @ V.T


def scan_batched_warm(spec, svals, model, x_fallback, gtol=1e-6, n_anchor=4, mode=None, max_rounds=2000):
    """The batched, warm-started path: every instance at once, each starting from the
    network's proposal where the engine finds it lower in energy than the fallback
    start, then lockstep BFGS from an inverse Hessian taken at the nearest of n_anchor
    anchor instances (converged instances drop out of the launches).  Instances still
    above gtol after max_rounds finish with the reference's Newton method one at a time
    (their Hamiltonian set-up included in the time).  Returns a dict with x, E, |g|,
    rounds, used proposal flags, the number finished by Newton and the seconds spent
    (batched set-up excluded)."""
    import time
    from . import HAM_ON_THE_FLY, HAM_STORED
    svals = np.asarray(svals, dtype=np.float64)
    M = len(svals)
    h1s, g2s = spec.integrals_batch(svals)
    ints = list(zip(h1s, g2s))
    feats = spec.features(svals)
    e = spec.engine(M)
    e.set_ham_integrals_batch(h1s, g2s, HAM_ON_THE_FLY if mode is None else mode)
    anchors = np.argsort(svals)[(np.arange(n_anchor) * M + M // 2) // n_anchor] if n_anchor else []
    ea = spec.engine(1)
    t0 = time.perf_counter()
    prop = model.predict(feats).astype(np.float64)
    starts, used = screened_starts(e, prop, spec.param0, spec.scale, np.tile(np.asarray(x_fallback, float), (M, 1)))
    hinv = None
    t_anchor = t_setup = 0.0
    if n_anchor:
        hs = []
        for a in anchors:
            t1 = time.perf_counter()
            ea.set_ham_integrals(*ints[a], HAM_STORED)  # set-up of the anchor engine, not timed
            t2 = time.perf_counter()
            hs.append(inverse_hessian(ea, starts[a], spec))
            t_anchor += time.perf_counter() - t2
            t_setup += t2 - t1
        near = np.abs(svals[:, None] - svals[anchors][None, :]).argmin(axis=1)
        hinv = np.ascontiguousarray(np.stack([hs[k] for k in near]))
    t_pre = time.perf_counter() - t0
    t1 = time.perf_counter()
    x, E, gn, it, rounds = e.optimise_batch(starts, spec.param0, spec.scale, gtol=gtol, max_rounds=max_rounds, hinv=hinv)
    E, gn = np.array(np.atleast_1d(E), dtype=float), np.array(np.atleast_1d(gn), dtype=float)
    t_opt = time.perf_counter() - t1
    e.close()
    # stragglers: the plain method from where the batch left them
    t2 = time.perf_counter()
    late = np.flatnonzero(gn >= gtol)
    for b in late:
        ea.set_ham_integrals(*ints[b], HAM_STORED)
        xb, Eb, gb, _, _ = ea.optimise_newton(x[b], spec.param0, spec.scale, gtol=gtol)
        x[b], E[b], gn[b] = xb, Eb, gb
    t_late = time.perf_counter() - t2
    ea.close()
    return dict(x=x, E=E, gnorm=gn, iters=it, rounds=rounds, used=used, newton_finished=len(late),
                seconds=t_opt + t_late + t_pre - t_setup, t_opt=t_opt, t_late=t_late, t_pre=t_pre - t_setup,
                t_anchor=t_anchor)
