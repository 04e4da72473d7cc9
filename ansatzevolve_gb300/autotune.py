"""Autotuner for the engine's launch shapes.

For one problem class (orbitals, electrons, layers, batch size, Hamiltonian kind) it
times the captured energy + gradient graph under candidate settings of the engine's
knobs and keeps the fastest:

* TUNE_PASS_OPS: excitations fused into one pass of the statevector (1..6; more per
  pass means fewer sweeps over HBM, but fewer commuting excitations to fill a pass);
* TUNE_CTAS_PER_SM: CTAs per SM of the pass kernels (occupancy against tail effects);
* TUNE_OTF_THREADS: threads per CTA of the on-the-fly H*psi kernel (one CTA per alpha
  string and chunk of beta strings);
* TUNE_SPMV_TPR: threads per row of the stored-H product (0 = chosen by size).

The search is greedy, one knob at a time in that order.  Results are cached in a JSON
file (AEGPU_TUNE_CACHE, default ~/.cache/ansatzevolve_gb300/autotune.json) under a key
that names the problem class, so later engines of the class start tuned.  No
counterpart in the reference, whose fuse size is fixed at 12.
"""
import json
import os
import time

import numpy as np

from . import HAM_ON_THE_FLY, TUNE_CTAS_PER_SM, TUNE_OTF_THREADS, TUNE_PASS_OPS, TUNE_SPMV_TPR

CANDIDATES = {
    TUNE_CTAS_PER_SM: (2, 4, 8, 16),
    TUNE_PASS_OPS: (4, 5, 6),
    TUNE_OTF_THREADS: (128, 256, 512, 1024),
    TUNE_SPMV_TPR: (1, 2, 4, 8),
}
DEFAULT = {TUNE_PASS_OPS: 6, TUNE_CTAS_PER_SM: 4, TUNE_OTF_THREADS: 512, TUNE_SPMV_TPR: 0}


def cache_path():
    return os.environ.get("AEGPU_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "ansatzevolve_gb300",
                                                           "autotune.json"))


def problem_key(n_orb, n_alpha, n_beta, layers, nb, ham_mode, per_instance):
    return "tups_N%d_a%d_b%d_L%d_nb%d_%s%s" % (n_orb, n_alpha, n_beta, layers, nb,
                                               "otf" if ham_mode == HAM_ON_THE_FLY else "stored",
                                               "_own" if per_instance else "_shared")


def load_cache(path=None):
    path = path or cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(cache, path=None):
    path = path or cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def lookup(key, path=None):
    """The cached knob settings of a problem class ({} when not tuned)."""
    ent = load_cache(path).get(key)
    return {int(k): int(v) for k, v in ent["best"].items()} if ent else {}


def time_config(build, tuning, reps=5):
    """Seconds per evaluation graph replay of build(tuning) (after two warm-ups)."""
    e = build(tuning)
    try:
        e.launch_io()
        e.launch_io()
        e.io_get_results()
        t = time.perf_counter()
        for _ in range(reps):
            e.launch_io()
        e.io_get_results()
        return (time.perf_counter() - t) / reps
    finally:
        e.close()


def tune(key, build, knobs=(TUNE_CTAS_PER_SM, TUNE_PASS_OPS, TUNE_OTF_THREADS), reps=5, path=None, log=None):
    """Greedy search over `knobs` in order (add TUNE_SPMV_TPR for stored Hamiltonians);
    build(tuning) -> an engine with its Hamiltonian and angles in its io buffer.
    Stores and returns the best settings."""
    best = dict(DEFAULT)
    trials = []
    t_best = time_config(build, best, reps)
    trials.append((dict(best), t_best))
    tried = {tuple(sorted(best.items()))}
    for knob in knobs:
        for v in CANDIDATES[knob]:
            cand = dict(best)
            cand[knob] = v
            if tuple(sorted(cand.items())) in tried:
                continue
            tried.add(tuple(sorted(cand.items())))
            t = time_config(build, cand, reps)
            trials.append((dict(cand), t))
            if log:
                log("%s %s: %.3f ms" % (key, cand, t * 1e3))
            if t < t_best:
                best, t_best = cand, t
    cache = load_cache(path)
    cache[key] = {"best": {str(k): v for k, v in best.items()}, "seconds": t_best,
                  "default_seconds": trials[0][1],
                  "trials": [[{str(k): v for k, v in c.items()}, t] for c, t in trials]}
    save_cache(cache, path)
    return best, t_best, trials


def tups_builder(n_orb, n_alpha, layers, nb, integrals, ham_mode, angles, per_instance=True):
    """build(tuning) for a TUPS batch with the given integrals ([(h1, g2)] per
    instance, or one pair shared) and angles [nb, nops]."""

    def build(tuning):
        from . import BASIS_SZ, Engine
        from .synthetic import hartree_fock_index, tups_operators
        ops, _, _ = tups_operators(n_orb, layers)
        e = Engine(2 * n_orb, BASIS_SZ, 2 * n_alpha, n_alpha, n_alpha, np.asarray(ops) - 1, tuning=tuning)
        init = np.zeros(e.D)
        init[np.searchsorted(e.states(), hartree_fock_index(n_orb, n_alpha, n_alpha))] = 1.0
        e.set_initial(init)
        if nb > 1:
            e.set_batch(nb)
        if per_instance:
            e.set_ham_integrals_batch(np.stack([h for h, _ in integrals]), np.stack([g for _, g in integrals]), ham_mode)
        else:
            e.set_ham_integrals(integrals[0][0], integrals[0][1], ham_mode)
        e.io_put_angles(angles)
        e.io_get_results()
        return e

    return build
