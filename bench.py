"""Benchmark: TUPS energy+gradient evaluations per second on GB300 (FP64).

Workload (the configuration the metric is quoted on): tUPS, 12 spatial orbitals,
6 alpha + 6 beta electrons (853,776 determinants), 3 layers (99 parameters, 165
excitations), seeded synthetic random integrals, H stored as fixed-width rows in
HBM.  One step = one energy+gradient evaluation: forward evolution of the fused
blocks, H*psi fused with <psi|H psi>, and the adjoint sweep that yields every
operator's gradient (the reference's FusedEvolve::evolve + evolveDerivative(&E)).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`value` is measured with the inputs resident in HBM (CUDA events on the engine's
stream); `e2e` is the same metric through the reference-compatible C ABI
(getEnergy + getGradient_COMP with host buffers, copies inside the timed region).
Under torchrun every rank runs an independent replica (the path does not shard),
timing is the max over ranks and `value` sums all ranks' evaluations.
`--impl reference` times the reference's own CPU implementation (built natively on
this host from its sources by oracle/build_ref.sh --timing, all host threads) on the
same workload; without that build, the oracle's C restatement of it.

Two more objects on the same line: `batched` (512 instances of 8, 10 and 12 orbitals
with their own integrals, one graph launch per step) and `time_to_converge` (a
10-orbital Hamiltonian family scan: the reference's Newton method one instance at a
time against the batched, network-warm-started path).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TUPS energy+gradient evals/s (12 orb, FP64) and time-to-converge vs plain"
N_ORB, N_A, N_B, LAYERS, SEED = 12, 6, 6, 3, 0


def set_orbitals(n):
    """Smaller or larger cases of the same workload for profiling (default 12)."""
    global N_ORB, N_A, N_B, LAYERS
    N_ORB, N_A, N_B, LAYERS = n, n // 2, n // 2, 2 if n <= 8 else (4 if n >= 14 else 3)


def workload_desc(D, P, nops, ham):
    if LUCJ:
        return {"workload": "LUCJ exp(-K) exp(iJ) exp(K), complex128, %d orbitals, %da+%db electrons (D=%d), %d "
                            "operators (K, J seed %d), synthetic random integrals seed %d, H %s"
                            % (N_ORB, N_A, N_B, D, nops, LUCJ_SEED, LUCJ_HAM_SEED, ham),
                "global_batch": 1, "parallelism": "replicas", "l2": "state vectors larger than L2"}
    return {"workload": "tUPS %d orbitals, %da+%db electrons (D=%d), %d layers (%d parameters, %d excitations), "
                        "synthetic random integrals seed 0, H %s" % (N_ORB, N_A, N_B, D, LAYERS, P, nops, ham),
            "global_batch": 1, "parallelism": "replicas", "l2": "inputs larger than L2 (H rows stream from HBM every step)"}


LUCJ = False
# DRAM traffic / algorithmic bytes of k_spmv_sell (uncoded rows) measured by ncu on the
# 10-orbital launch (669.27 MB read + 3.68 MB written for 668.57 MB algorithmic)
SELL_TRAFFIC_RATIO = (669.273856 + 3.678720) / 668.570112
# DRAM traffic / streamed bytes of k_spmv_vell (coded rows) measured by ncu on the
# 10-orbital launch (355.99 MB read + 4.28 MB written for 356.13 MB of coded rows,
# x and y); profiles/k_spmv_vell_tups10_stored.md
VELL_TRAFFIC_RATIO = (355.988992 + 4.284160) / 356.130432
# the same for the spin-flip half product (profiles/k_spmv_vell_tups10_half.md): DRAM
# bytes of one launch over the coded rows with a <= b (31,878 of 63,504) plus x and y
VELL_HALF_TRAFFIC_RATIO = (189.438720 + 3.268096) / (31878 * 5592 / 1e6 + 16 * 63504 / 1e6)


def coded_row_bytes(D, W, width):
    """Bytes one coded-row product streams: explicit entries (diagonal + singles) at
    12 B, coded doubles at 6 B (4-byte column + 2-byte code), each part padded to a
    multiple of 4 entries, plus x and y; None where the engine keeps uncoded rows
    (value table over 2^15 entries, N > 12, or AEGPU_CODED_ROWS=0)."""
    NP = N_ORB * (N_ORB - 1) // 2
    if 1 + NP * NP + N_ORB ** 4 > (1 << 15) or os.environ.get("AEGPU_CODED_ROWS") == "0":
        return None
    we = 1 + N_A * (N_ORB - N_A) + N_B * (N_ORB - N_B)
    se, sd = (we + 3) // 4 * 4, (width - we + 3) // 4 * 4
    return D * (se * 12 + sd * 6) + 16 * D * W


# the LUCJ circuit's seeds (K, J and the integrals), those of the reference-pinned
# fixture tests/golden/lucj14.npz
LUCJ_SEED, LUCJ_HAM_SEED = 3, 7
# profiling case: only the first LUCJ_OPS operators of the LUCJ circuit (0 = all), so
# that the checkpoints of a 14-orbital run stay within a few GB under ncu
LUCJ_OPS = 0


def problem():
    from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals, tups_operators
    h1, g2 = synthetic_integrals(N_ORB, LUCJ_HAM_SEED if LUCJ else SEED)
    hf = hartree_fock_index(N_ORB, N_A, N_B)
    if LUCJ:
        # exp(-K) exp(iJ) exp(K), K anti-Hermitian N(0, 0.1), nearest-neighbour J ~ N(0, 0.1)
        from ansatzevolve_gb300.lucj import lucj_operators, random_lucj
        K, J = random_lucj(N_ORB, LUCJ_SEED)
        ops0, ang = lucj_operators(K, J)
        # at the size of the reference-pinned fixture, its own operators and angles (the
        # decomposition of exp(K) may pick angles 2 pi apart on another machine's LAPACK)
        fxp = os.path.join(ROOT, "tests", "golden", "lucj%d.npz" % N_ORB)
        if os.path.exists(fxp):
            fx = np.load(fxp)
            if int(fx["lucj_seed"]) == LUCJ_SEED and int(fx["ham_seed"]) == LUCJ_HAM_SEED:
                ops0, ang = np.asarray(fx["ops"]), np.asarray(fx["x"])
        if LUCJ_OPS:
            ops0, ang = ops0[:LUCJ_OPS], ang[:LUCJ_OPS]
        n = len(ops0)
        return dict(h1=h1, g2=g2, ops0=ops0, ops1=None, p0=np.arange(n), scale=np.ones(n), P=n, x=ang, hf=hf,
                    cplx=True)
    ops, param, scale = tups_operators(N_ORB, LAYERS)
    P = int(param.max())
    x = np.random.default_rng(SEED + 1).uniform(-0.1, 0.1, P)
    return dict(h1=h1, g2=g2, ops0=ops - 1, ops1=ops, p0=param - 1, scale=scale, P=P, x=x, hf=hf, cplx=False)


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, max clock, throttle reasons)."""

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for k, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(k)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_baseline(pb, max_seconds=30.0):
    """The reference itself on the host cores (oracle/_ref/ref_driver_native) on a bounded
    sample, with the oracle's energy and gradient for the parity check; without the
    reference build, the oracle (C restatement of the reference algorithm, OpenMP)."""
    from oracle.oracle import Oracle, lib as olib
    if reference_available() is None and not LUCJ:
        r = reference_timing(pb, 3, 0, max_seconds)
        t = float(np.median(r["times"][1:])) if len(r["times"]) > 1 else float(r["times"][0])
        return {"value": 1.0 / t, "unit": "evals/s", "cores": r["cores"], "kind": "reference",
                "cpu_model": r["cpu_model"],
                "sample": "%d FusedEvolve::evolve + evolveDerivative(&E) units of the same %d-orbital workload "
                          "(median of all but the first), the reference built natively on this host "
                          "(oracle/_ref/ref_driver_native); set-up %.1f s not timed"
                          % (len(r["times"]), N_ORB, r["setup_s"])}, r["E"], r["g"]
    o = Oracle(2 * N_ORB, 2, N_A + N_B, N_A, N_B, cplx=pb["cplx"])
    o.set_initial([pb["hf"]], [1.0])
    o.set_ops(pb["ops0"], pb["p0"], pb["scale"])
    o.set_ham_integrals(pb["h1"], pb["g2"], csr=False)
    times = []
    t_end = time.perf_counter() + max_seconds
    for k in range(3):
        t0 = time.perf_counter()
        Ek, gk = o.gradient_comp(pb["x"] + 1e-3 * k)
        times.append(time.perf_counter() - t0)
        if k == 0:
            E, g = Ek, gk
        if time.perf_counter() > t_end:
            break
    t = float(np.median(times[1:])) if len(times) > 1 else times[0]
    return {"value": 1.0 / t, "unit": "evals/s", "cores": int(olib().or_num_threads()), "kind": "port",
            "sample": "%d energy+gradient evaluations of the same %d-orbital workload (%s), operator-list H*psi "
                      "as the reference picks for this size" % (len(times), N_ORB, "median of all but the first"
                                                                  if len(times) > 1 else "single evaluation")}, E, g


# the reference itself, built natively on this host from its own sources by
# oracle/build_ref.sh --timing (build() does it when the sources are there)
REF_DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver_native")


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return None


def reference_timing(pb, steps, warmup, budget):
    """The reference's own FusedEvolve::evolve + evolveDerivative(&E) -- the unit of the
    metric, as its CLI benchmark times it (main.cpp:415-425) -- on all host threads:
    oracle/_ref/ref_driver_native builds the reference's HamiltonianMatrix from the
    integral files (at 12 orbitals the reference picks its on-the-fly operator list by
    itself), then times `steps` units after `warmup` untimed ones, within `budget` s."""
    import tempfile
    from ansatzevolve_gb300.synthetic import write_integrals
    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as td:
        prefix = os.path.join(td, "ints")
        write_integrals(prefix, pb["h1"], pb["g2"])
        spec = ["nqubits %d" % (2 * N_ORB), "initial 1", "%d 1.0 0.0" % pb["hf"], "ops %d" % len(pb["ops0"])]
        spec += [" ".join(str(int(v)) for v in o) for o in pb["ops0"]]
        spec += ["order %d" % len(pb["p0"])] + ["%d %r" % (int(p), float(c)) for p, c in zip(pb["p0"], pb["scale"])]
        spec += ["ham ints %s" % prefix, "nuclear 0.0", "anglesets 1 %d" % pb["P"], " ".join(repr(float(v)) for v in pb["x"]),
                 "want 0 0 0 0", "time %d" % max(1, steps), "timewarmup %d" % max(0, warmup), "timebudget %r" % budget,
                 "end"]
        sp, op = os.path.join(td, "spec"), os.path.join(td, "out")
        with open(sp, "w") as f:
            f.write("\n".join(spec) + "\n")
        t0 = time.perf_counter()
        subprocess.run([REF_DRIVER, sp, op], check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL,
                       env=dict(os.environ, OMP_NUM_THREADS=str(threads)))
        wall = time.perf_counter() - t0
        d = np.fromfile(op, dtype="<f8")
    n = int(d[2])
    times = d[3:3 + n]
    E = float(d[3 + n])
    P = int(d[4 + n])
    g = d[5 + n:5 + n + P]
    return {"setup_s": float(d[0]), "cores": int(d[1]), "times": times, "E": E, "g": g, "wall_s": wall,
            "cpu_model": cpu_model()}


def reference_available():
    if not os.path.exists(REF_DRIVER):
        return "oracle/_ref/ref_driver_native not built (no reference sources on this host)"
    return None


def run_reference(args, rank, world):
    if rank != 0:
        return
    pb = problem()
    budget = float(os.environ.get("AE_REFERENCE_BUDGET_S", "150"))
    why = reference_available()
    D = math.comb(N_ORB, N_A) * math.comb(N_ORB, N_B)
    if why is None and not LUCJ:
        r = reference_timing(pb, args.steps, args.warmup, budget)
        done, dt = len(r["times"]), float(np.sum(r["times"]))
        v = done / dt
        cb = {"value": v, "unit": "evals/s", "cores": r["cores"], "kind": "reference", "cpu_model": r["cpu_model"],
              "binary": "oracle/_ref/ref_driver_native (the reference's sources, g++ -O3 native, OpenMP)",
              "sample": "%d of %d requested FusedEvolve::evolve + evolveDerivative(&E) units (main.cpp:415-425) "
                        "within the %.0f s budget, after %d untimed; reference set-up %.1f s not timed"
                        % (done, args.steps, budget, args.warmup, r["setup_s"])}
        line = {"metric": METRIC, "value": v, "unit": "evals/s", "n_gpus": world, "steps": done,
                "warmup": args.warmup, "ms_per_step": 1e3 * dt / done, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random integrals)", "impl": "reference",
                "config": workload_desc(D, pb["P"], len(pb["ops0"]),
                                        "applied from the reference's operator list on the fly (its own choice at "
                                        "this size)"),
                "cpu_baseline": cb,
                "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        ref = os.path.join(ROOT, "tests", "golden", "ref%d.npz" % N_ORB)
        if os.path.exists(ref):
            fx = np.load(ref)
            line["parity_reference"] = {"dE": abs(r["E"] - float(fx["E"])), "max_dg": float(np.max(np.abs(r["g"] - fx["G"]))),
                                        "source": "tests/golden/ref%d.npz" % N_ORB}
        print(json.dumps(line), flush=True)
        return
    # fallback: the oracle's C restatement of the reference algorithm
    from oracle.oracle import Oracle, lib as olib
    o = Oracle(2 * N_ORB, 2, N_A + N_B, N_A, N_B, cplx=pb["cplx"])
    o.set_initial([pb["hf"]], [1.0])
    o.set_ops(pb["ops0"], pb["p0"], pb["scale"])
    o.set_ham_integrals(pb["h1"], pb["g2"], csr=False)
    for w in range(min(args.warmup, 1)):
        o.gradient_comp(pb["x"])
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        o.gradient_comp(pb["x"] + 1e-4 * done)
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    dt = time.perf_counter() - t0
    v = done / dt
    line = {"metric": METRIC, "value": v, "unit": "evals/s", "n_gpus": world, "steps": done, "warmup": min(args.warmup, 1),
            "ms_per_step": 1e3 * dt / done, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": workload_desc(int(o.D), pb["P"], len(pb["ops0"]), "applied from the operator list on the fly"),
            "cpu_baseline": {"value": v, "unit": "evals/s", "cores": int(olib().or_num_threads()), "kind": "port",
                             "cpu_model": cpu_model(), "why_port": why or "LUCJ circuit: complex build not timed",
                             "sample": "%d of %d requested steps within the %.0f s budget" % (done, args.steps, budget)},
            "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def e2e_c_abi(pb, steps, warmup, reuse_hpsi=True):
    """getEnergy + getGradient_COMP through the reference-compatible C ABI, host buffers.
    reuse_hpsi=False: getGradient_COMP recomputes H psi, as the reference's
    evolveDerivative does (fusedevolve.cpp:2292), i.e. two H products per pair."""
    import ansatzevolve_gb300 as ae
    saved = os.environ.get("AEGPU_REUSE_HPSI")
    os.environ["AEGPU_REUSE_HPSI"] = "1" if reuse_hpsi else "0"
    m = ae.stateAnsatzManager()
    assert m.storeInitial(2 * N_ORB, [pb["hf"]], [1.0])
    assert m.storeOperators(pb["ops1"].tolist())
    assert m.storeParameterDependencies(list(zip(pb["p0"], pb["scale"])))
    assert m.storeIntegrals(pb["h1"], pb["g2"], ae.HAM_STORED)
    xs = [pb["x"], pb["x"] + 1e-3]
    for k in range(warmup):
        m.getExpectationValue(xs[k % 2])
        m.getGradientComp(xs[k % 2])
    t0 = time.perf_counter()
    for k in range(steps):
        E = m.getExpectationValue(xs[k % 2])
        g = m.getGradientComp(xs[k % 2])
    dt = time.perf_counter() - t0
    P = pb["P"]
    m.close()
    if saved is None:
        os.environ.pop("AEGPU_REUSE_HPSI", None)
    else:
        os.environ["AEGPU_REUSE_HPSI"] = saved
    return {"value": steps / dt, "unit": "evals/s", "h2d_bytes_per_step": 2 * 8 * P, "d2h_bytes_per_step": 8 + 8 * P,
            "ms_per_step": 1e3 * dt / steps,
            "api": "getEnergy + getGradient_COMP (%s)" % ("H*psi cached between the pair" if reuse_hpsi else
                                                          "H*psi recomputed by getGradient_COMP, as the reference does")}


def max_over_ranks(ms, dist):
    """The slowest rank's timed-region length (every rank runs an independent replica)."""
    if not dist:
        return ms
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def tuned(key):
    """Knob settings for a problem class: the local autotuner cache, else the table
    tuned on GB300 that ships with the package, else the defaults."""
    from ansatzevolve_gb300 import autotune
    t = autotune.lookup(key)
    if not t:
        t = autotune.lookup(key, os.path.join(ROOT, "ansatzevolve_gb300", "tuned_gb300.json"))
    return t


def batched_bench(stream, steps=10, warmup=3):
    """512 instances with their own seeded integrals and U(-0.3, 0.3) TUPS angles (one per
    parameter, drawn [instances, parameters] class by class), evaluated
    by ONE graph launch: 256 x 8 orbitals (4a+4b, 2 layers), 192 x 10 orbitals (5a+5b,
    3 layers), 64 x 12 orbitals (6a+6b, 3 layers); instance i uses integral seed i."""
    import torch
    import ansatzevolve_gb300 as ae
    from ansatzevolve_gb300 import autotune
    from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals, tups_operators
    classes = [(8, 4, 2, 256, 0, ae.HAM_STORED), (10, 5, 3, 192, 256, ae.HAM_ON_THE_FLY),
               (12, 6, 3, 64, 448, ae.HAM_ON_THE_FLY)]
    rng = np.random.default_rng(SEED)
    engines, per_class = [], []
    t0 = time.perf_counter()
    for N, na, L, nb, s0, mode in classes:
        key = autotune.problem_key(N, na, na, L, nb, mode, True)
        tuning = tuned(key)
        ops, param, scale = tups_operators(N, L)
        e = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops - 1, tuning=tuning or None)
        init = np.zeros(e.D)
        init[np.searchsorted(e.states(), hartree_fock_index(N, na, na))] = 1.0
        e.set_initial(init)
        e.set_batch(nb)
        ints = [synthetic_integrals(N, s) for s in range(s0, s0 + nb)]
        e.set_ham_integrals_batch(np.stack([i[0] for i in ints]), np.stack([i[1] for i in ints]), mode)
        # TUPS angles: one per parameter (an alpha-beta pair of singles shares it)
        X = rng.uniform(-0.3, 0.3, (nb, int(param.max())))
        e.io_put_angles(np.asarray(scale, dtype=float)[None, :] * X[:, param - 1])
        e.io_get_results()
        engines.append(e)
        per_class.append({"orbitals": N, "instances": nb, "D": e.D, "ham": "stored" if mode == ae.HAM_STORED else
                          "on the fly", "tuning": {str(k): v for k, v in e.tuning().items()},
                          "tuned": bool(tuning)})
    setup_s = time.perf_counter() - t0
    grp = ae.Group(engines)
    sp = stream.cuda_stream
    peak_t = ae.fp64_peak() / 2.0  # T DFMA/s
    for _ in range(warmup):
        grp.launch(sp)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        grp.launch(sp)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    # each class alone, for the breakdown
    for e, pc in zip(engines, per_class):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e.launch_io(sp)
        a.record(stream)
        for _ in range(3):
            e.launch_io(sp)
        b.record(stream)
        torch.cuda.synchronize()
        pc["ms_per_batch"] = a.elapsed_time(b) / 3
        pc["evals_per_s"] = pc["instances"] / (pc["ms_per_batch"] / 1e3)
        # the class against the FP64 pipe: FP64 instructions of its evaluations (one DFMA
        # per matrix element, per amplitude-layer forward, two adjoint) over the measured
        # DFMA rate
        fw = sum(e.fp64_work())
        pc["fp64_instr_per_batch"] = int(fw * pc["instances"])
        pc["fp64_frac"] = fw * pc["instances"] / (pc["ms_per_batch"] / 1e3) / 1e12 / peak_t
    E, g = engines[0].io_get_results()
    fp64_all = sum(pc["fp64_instr_per_batch"] for pc in per_class)
    # instance 0 of every class against the reference's own output for the same integrals
    # and angles (tests/golden/batched4.npz)
    ref = os.path.join(ROOT, "tests", "golden", "batched4.npz")
    if os.path.exists(ref):
        fx = np.load(ref)
        for (N, na, L, nb, s0, mode), e, pc in zip(classes, engines, per_class):
            Ei, gi = e.io_get_results()
            _, param, scale = tups_operators(N, L)
            gc = np.zeros(int(param.max()))
            np.add.at(gc, param - 1, scale * gi[0])
            pc["parity_reference"] = {"dE": abs(float(Ei[0]) - float(fx["E%d" % N])),
                                      "max_dg": float(np.max(np.abs(gc - fx["G%d" % N]))),
                                      "source": "tests/golden/batched4.npz (instance 0)"}
    out = {"value": 512 / (ms / 1e3), "unit": "instance energy+gradient evals/s", "instances": 512,
           "fp64_frac": fp64_all / (ms / 1e3) / 1e12 / peak_t, "fp64_peak_T_per_s": peak_t,
           "ms_per_step": ms, "steps": steps, "warmup": warmup, "graph_launches_per_step": 1,
           "gpu_launches_per_step": grp.launch_count(), "classes": per_class, "setup_s": setup_s,
           "finite": bool(np.all(np.isfinite(E)) and np.all(np.isfinite(g)))}
    grp.close()
    for e in engines:
        e.close()
    return out


def aux_case_bench(n_orb, lucj, stream, steps=5, warmup=2):
    """Configuration 3: 14 orbitals, 7a+7b (11,778,624 determinants), 4 tUPS layers or the
    complex128 LUCJ circuit, H regenerated on the fly from the integrals.  Energy +
    gradient evaluations by graph replay (CUDA events), per-phase times on the stream
    path, the FP64-pipe fraction of the H product, the HBM fraction of the forward and
    adjoint sweeps (algorithmic bytes: 16 B per amplitude per pass forward, 32 B adjoint;
    complex amplitudes count twice), and parity against the reference's own output
    (tests/golden/ref14.npz, lucj14.npz)."""
    global LUCJ
    import torch
    import ansatzevolve_gb300 as ae
    from ansatzevolve_gb300 import autotune
    saved = (N_ORB, LUCJ)
    set_orbitals(n_orb)
    LUCJ = lucj
    try:
        pb = problem()
        mode = ae.HAM_ON_THE_FLY
        tuning = tuned(autotune.problem_key(N_ORB, N_A, N_B, LAYERS, 1, mode, lucj))
        t0 = time.perf_counter()
        eng = ae.Engine(2 * N_ORB, ae.BASIS_SZ, N_A + N_B, N_A, N_B, pb["ops0"], complex_mode=pb["cplx"],
                        tuning=tuning or None)
        W = 2 if pb["cplx"] else 1
        init = np.zeros(eng.D * W)
        init[W * np.searchsorted(eng.states(), pb["hf"])] = 1.0
        eng.set_initial(init)
        eng.set_ham_integrals(pb["h1"], pb["g2"], mode)
        setup_s = time.perf_counter() - t0
        info = eng.info()
        D = info["D"]
        ang = torch.tensor(pb["scale"] * pb["x"][pb["p0"]], dtype=torch.float64, device="cuda")
        E_d = torch.zeros(1, dtype=torch.float64, device="cuda")
        g_d = torch.zeros(len(pb["ops0"]), dtype=torch.float64, device="cuda")
        sp = stream.cuda_stream
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                eng.gradient_dev(ang.data_ptr(), E_d.data_ptr(), g_d.data_ptr(), sp)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            eng.gradient_dev(ang.data_ptr(), E_d.data_ptr(), g_d.data_ptr(), sp)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / steps
        eng.phase_timing(True)
        eng.phase_times()
        with torch.cuda.stream(stream):
            for _ in range(3):
                eng.gradient_dev(ang.data_ptr(), E_d.data_ptr(), g_d.data_ptr(), sp)
        torch.cuda.synchronize()
        phase_ms, nph = eng.phase_times()
        eng.phase_timing(False)
        ph = [phase_ms[k] / max(nph, 1) for k in range(3)]
        fw = eng.fp64_work()
        peak_t = ae.fp64_peak() / 2.0
        peak, peak_kind = measured_peak()
        passes = info["blocks"]
        touched = info["active"]  # amplitudes touched per sweep (a diagonal pass touches all D)
        half_passes = bool(eng.half_status()[0])
        if half_passes:  # one orbit of every mirror pair; a diagonal half pass every a <= b
            touched = eng.half_info()["active"]
        fwd_bytes, adj_bytes = 16 * touched * W, 32 * touched * W
        out = {"value": 1e3 / ms, "unit": "evals/s", "ms_per_step": ms, "steps": steps, "warmup": warmup,
               "config": workload_desc(D, pb["P"], len(pb["ops0"]), "regenerated on the fly"),
               "setup_s": setup_s, "passes": passes, "half_passes": half_passes,
               "phase_ms": {"evolve": ph[0], "hpsi_energy": ph[1], "adjoint": ph[2]},
               "hpsi_fp64": {"instructions": int(fw[0]), "achieved_T_per_s": fw[0] / (ph[1] / 1e3) / 1e12,
                             "peak_T_per_s": peak_t, "frac": fw[0] / (ph[1] / 1e3) / 1e12 / peak_t,
                             "peak_source": "measured (aegpu_fp64_peak)"},
               "sweeps_hbm": {"algorithmic_bytes": {"evolve": fwd_bytes, "adjoint": adj_bytes},
                              "achieved_gbs": {"evolve": fwd_bytes / (ph[0] / 1e3) / 1e9,
                                               "adjoint": adj_bytes / (ph[2] / 1e3) / 1e9},
                              "frac": {"evolve": fwd_bytes / (ph[0] / 1e3) / 1e9 / peak,
                                       "adjoint": adj_bytes / (ph[2] / 1e3) / 1e9 / peak},
                              "peak_gbs": peak, "peak_source": peak_kind},
               # the sweeps' own bound: their FP64 instructions (complex multiplies of the
               # phase passes, Givens updates and gradient sums) against the measured rate
               "sweeps_fp64": {"instructions": {"evolve": int(fw[1]), "adjoint": int(fw[2])},
                               "frac": {"evolve": fw[1] / (ph[0] / 1e3) / 1e12 / peak_t if ph[0] else None,
                                        "adjoint": fw[2] / (ph[2] / 1e3) / 1e12 / peak_t if ph[2] else None},
                               "peak_T_per_s": peak_t, "peak_source": "measured (aegpu_fp64_peak)"},
               "tuning": {"settings": {str(k): v for k, v in eng.tuning().items()}, "tuned": bool(tuning)}}
        ref = os.path.join(ROOT, "tests", "golden", ("lucj%d.npz" if lucj else "ref%d.npz") % N_ORB)
        if os.path.exists(ref):
            fx = np.load(ref)
            g_ops = g_d.cpu().numpy()
            g = np.zeros(pb["P"])
            np.add.at(g, pb["p0"], pb["scale"] * g_ops)
            if fx["x"].shape == pb["x"].shape and np.allclose(fx["x"], pb["x"]):
                out["parity_reference"] = {"dE": abs(float(E_d.item()) - float(fx["E"])),
                                           "max_dg": float(np.max(np.abs(g - fx["G"]))),
                                           "source": os.path.relpath(ref, ROOT)}
        eng.close()
        return out
    finally:
        set_orbitals(saved[0])
        LUCJ = saved[1]


def plain_mode(spec, s0, x0):
    """The faster H representation for the plain path's single 10-orbital instances:
    the reference's Newton method from x0 at s0, timed with each (after one untimed run)."""
    import ansatzevolve_gb300 as ae
    from ansatzevolve_gb300 import warmstart as ws
    t = {}
    for mode in (ae.HAM_STORED, ae.HAM_ON_THE_FLY):
        ws.scan_newton(spec, [s0], x0, gtol=1e-6, mode=mode)
        t[mode] = ws.scan_newton(spec, [s0], x0, gtol=1e-6, mode=mode)[2]
    best = min(t, key=t.get)
    return best, {"stored_s": t[ae.HAM_STORED], "on_the_fly_s": t[ae.HAM_ON_THE_FLY],
                  "chosen": "stored" if best == ae.HAM_STORED else "on the fly"}


def batched_columns_bench(stream, h=1e-4, n_line=8):
    """Configuration 4's other use of a batch: for one instance of each size class
    (8, 10, 12 orbitals; integral seed 0; angles U(-0.3, 0.3)), its line-search points
    x + t d (d = -g, n_line values of t in (0, 1.5]) and all its Hessian columns by central
    differences of the analytic gradient, (g(x + h e_i) - g(x - h e_i)) / 2h, evaluated
    as ONE batched energy + gradient launch of 2P + n_line + 1 instances, checked against
    the analytic Hessian of the same instance."""
    import torch
    import ansatzevolve_gb300 as ae
    from ansatzevolve_gb300.synthetic import hartree_fock_index, synthetic_integrals, tups_operators
    out = []
    for N, na, L, mode in [(8, 4, 2, ae.HAM_STORED), (10, 5, 3, ae.HAM_ON_THE_FLY), (12, 6, 3, ae.HAM_ON_THE_FLY)]:
        ops, param, scale = tups_operators(N, L)
        p0, P = param - 1, int(param.max())
        h1, g2 = synthetic_integrals(N, 0)
        x = np.random.default_rng(N).uniform(-0.3, 0.3, P)
        e1 = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops - 1)
        init = np.zeros(e1.D)
        init[np.searchsorted(e1.states(), hartree_fock_index(N, na, na))] = 1.0
        e1.set_initial(init)
        e1.set_ham_integrals(h1, g2, ae.HAM_STORED)
        t0 = time.perf_counter()
        _, g0, Hx = e1.hessian(scale * x[p0], p0, scale)
        t_hess = time.perf_counter() - t0
        e1.close()
        ts = np.linspace(1.5 / n_line, 1.5, n_line)
        X = np.vstack([x + h * np.eye(P), x - h * np.eye(P), x[None, :] + ts[:, None] * (-g0)[None, :], x[None, :]])
        nb = len(X)
        e = ae.Engine(2 * N, ae.BASIS_SZ, 2 * na, na, na, ops - 1)
        e.set_initial(init)
        e.set_batch(nb)
        e.set_ham_integrals(h1, g2, mode)
        e.io_put_angles(scale[None, :] * X[:, p0])
        e.io_get_results()
        sp = stream.cuda_stream
        for _ in range(2):
            e.launch_io(sp)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(3):
            e.launch_io(sp)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / 3
        E, gops = e.io_get_results()
        e.close()
        G = np.zeros((nb, P))
        for k in range(nb):
            np.add.at(G[k], p0, scale * gops[k])
        Hfd = (G[:P] - G[P:2 * P]) / (2 * h)
        out.append({"orbitals": N, "parameters": P, "instances": nb, "ham": "stored" if mode == ae.HAM_STORED else
                    "on the fly", "ms_per_batch": ms, "evals_per_s": nb / (ms / 1e3),
                    "hessian_columns_max_dev": float(np.max(np.abs(Hfd - Hx))), "analytic_hessian_ms": 1e3 * t_hess,
                    "line_search_E": [float(v) for v in E[2 * P:2 * P + n_line]], "E_at_x": float(E[-1])})
    return {"classes": out, "fd_step": h,
            "api": "aegpu_launch_io: one captured graph of the batched energy + gradient evaluation per class"}


def ttc_bench(n_train=2000, n_heldout=200, n_plain=200, epochs=400, n_seg=64, batch=256, chain_gtol=1e-6):
    """Time to converge over a 10-orbital Hamiltonian family scan (5a+5b, 3 layers,
    81 parameters): h(s) = h0 + s h1, L^k(s) = L^k0 + s L^k1.  Both paths start the scan
    from the s = 0 member's lowest minimum found by a 64-start batched search (shared,
    not timed).
    Plain: one instance at a time in increasing s, the reference's Newton method from
    the previous converged angles, with the faster of the stored and on-the-fly H for a
    single instance (measured first), timed on the first n_plain held-out values (all
    of them by default; mean per instance).  Batched + warm-started: all n_heldout
    instances in one batch, network proposals screened by the engine against the s = 0
    angles, then lockstep BFGS from the inverse Hessians at 8 anchors (converged
    instances drop out of the launches; any still unconverged after 2000 rounds would
    finish with the plain method, timed).  The network is trained once per family on
    n_train converged angle sets from a two-level continuation chain (n_seg heads in
    sequence, then the segments in lockstep batches, each solve to |g| < chain_gtol:
    the targets only seed proposals, which the batched path converges to 1e-6 itself),
    its cost reported separately and charged in speedup_including_training.  GB300,
    (chain_gtol, n_seg): (1e-8, 125) 4.5x with the training charged, (1e-7, 125) 4.8x,
    (1e-6, 32) 5.3x, (1e-6, 64) 5.4x, 200/200 energies matched in every case."""
    from ansatzevolve_gb300 import warmstart as ws
    spec = ws.FamilySpec(10, 5, 3, seed=0)
    t0 = time.perf_counter()
    x0, E0 = ws.scan_origin(spec)
    t_origin = time.perf_counter() - t0
    s_tr = np.sort(np.random.default_rng(2024).uniform(0, 1, n_train))
    s_ho = np.sort(np.random.default_rng(77).uniform(0, 1, n_heldout))
    t0 = time.perf_counter()
    xtr, Etr, gtr, its = ws.scan_segmented_chain(spec, s_tr, x0, n_seg=n_seg, gtol=chain_gtol)
    t_chain = time.perf_counter() - t0
    t0 = time.perf_counter()
    model, hist = ws.train_warmstart(spec.features(s_tr), xtr, epochs=epochs, batch=batch, lr=1e-3)
    t_train = time.perf_counter() - t0
    r = ws.scan_batched_warm(spec, s_ho, model, x0, gtol=1e-6, n_anchor=8)
    mode, mode_info = plain_mode(spec, s_ho[0], x0)
    xp, Ep, tp, nh, ne = ws.scan_newton(spec, s_ho[:n_plain], x0, gtol=1e-6, mode=mode)
    plain_per = tp / n_plain
    batched_per = r["seconds"] / n_heldout
    dE = r["E"][:n_plain] - Ep
    model.close()
    train_s = t_chain + t_train
    return {"speedup": plain_per / batched_per, "unit": "x (plain seconds per instance / batched seconds per instance)",
            # the one-off training cost charged to this one scan of n_heldout instances
            "speedup_including_training": plain_per * n_heldout / (r["seconds"] + train_s),
            "plain_s_per_instance": plain_per, "plain_instances_timed": n_plain, "plain_ham": mode_info,
            "plain_hessians": nh, "plain_energy_evals": ne,
            "batched_s_total": r["seconds"], "batched_instances": n_heldout, "batched_s_per_instance": batched_per,
            "batched_rounds": int(r["rounds"]), "batched_iters_median": float(np.median(r["iters"])),
            "batched_iters_max": int(r["iters"].max()), "proposals_used": int(r["used"].sum()),
            "finished_by_newton": int(r["newton_finished"]), "newton_finish_s": r["t_late"],
            "anchor_hessian_s": r["t_anchor"], "max_gnorm": float(r["gnorm"].max()), "gtol": 1e-6,
            "energy_match_1e-8": int(np.sum(np.abs(dE) < 1e-8)), "energy_compared": n_plain,
            "max_abs_dE": float(np.abs(dE).max()),
            "training": {"instances": n_train, "chain_s": t_chain, "chain_iters_median": float(np.median(its)),
                         "chain": "%d heads in sequence, then the %d segments walked in lockstep batches; each solve "
                                  "starts from the secant predictor of its chain" % (n_seg, n_seg),
                         "chain_max_gnorm": float(np.max(gtr)), "chain_gtol": chain_gtol,
                         "mlp_train_s": t_train, "epochs": epochs, "minibatch": batch, "loss_first": float(hist[0]),
                         "loss_last": float(hist[-1]), "origin_s": t_origin, "origin_energy": float(E0)},
            "workload": "10 orbitals 5a+5b, 3 layers (81 parameters), family h(s)=h0+s h1, L(s)=L0+s L1, seed 0, "
                        "h1 and L1 at %.2f of the base scale; %d training / %d held-out s ~ U(0,1)"
                        % (spec.pert, n_train, n_heldout)}


def gram_kernel_bench(args, n=853776, V=100):
    """The Hessian's Gram contraction 2 T_C^T (H T_C) on its own at the 12-orbital shape
    (upper triangle, V = 100 columns of n doubles, random columns): CUDA-event time per
    call and the DFMA rate of the 5,200 x n DFMAs it issues (325 micro-tiles of 4 x 4)."""
    import torch
    import ansatzevolve_gb300 as ae
    L = ae.lib()
    g = torch.Generator(device="cuda").manual_seed(0)
    TC = torch.randn(V, n, dtype=torch.float64, device="cuda", generator=g)
    HTC = torch.randn(V, n, dtype=torch.float64, device="cuda", generator=g)
    C = torch.zeros(V, V, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()

    def call():
        rc = L.aegpu_gram_upper_dev(TC.data_ptr(), n, HTC.data_ptr(), n, n, 1, V, 2.0, C.data_ptr(), 0, V, s.cuda_stream)
        assert rc == 0

    for _ in range(max(args.warmup, 3)):
        call()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(args.steps):
        call()
    b.record(s)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / args.steps
    nb = (V + 3) // 4
    dfma = nb * (nb + 1) // 2 * 16 * n
    print(json.dumps({"kernel": "k_gram (aegpu_gram_upper_dev)", "n": n, "V": V, "ms": ms, "dfma": dfma,
                      "T_dfma_per_s": dfma / (ms / 1e3) / 1e12, "peak_T_dfma_per_s": ae.fp64_peak() / 2.0}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--ham", default=None, choices=["stored", "otf"],
                    help="stored (default up to 12 orbitals) or on the fly (default at 14: the stored "
                         "operator of D = 11.8M does not fit in HBM)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--orbitals", type=int, default=12, choices=[8, 10, 12, 14],
                    help="workload size (the metric is quoted at 12; others are profiling cases)")
    ap.add_argument("--lucj", action="store_true", help="complex LUCJ ansatz instead of tUPS (no C-ABI e2e)")
    ap.add_argument("--lucj-ops", type=int, default=0,
                    help="profiling case: only the first N operators of the LUCJ circuit (no reference parity)")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-hessian", action="store_true")
    ap.add_argument("--no-ground", action="store_true", help="skip the lowest-eigenpair (Lanczos) timing")
    ap.add_argument("--no-ttc", action="store_true")
    ap.add_argument("--no-config3", action="store_true", help="skip the 14-orbital tUPS and LUCJ objects")
    ap.add_argument("--kernel", default=None, choices=["gram"],
                    help="time one kernel on its own instead (gram: the Hessian's Gram contraction at the "
                         "12-orbital shape, 100 columns of 853,776 doubles)")
    ap.add_argument("--ttc-train", type=int, default=2000)
    ap.add_argument("--ttc-heldout", type=int, default=200)
    ap.add_argument("--ttc-plain", type=int, default=200)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gpu" else args.warmup
    set_orbitals(args.orbitals)
    global LUCJ, LUCJ_OPS
    LUCJ = args.lucj
    LUCJ_OPS = args.lucj_ops
    if LUCJ:
        args.no_e2e = True
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.kernel == "gram":
        return gram_kernel_bench(args)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import ansatzevolve_gb300 as ae
    pb = problem()
    if args.ham is None:
        args.ham = "otf" if args.orbitals >= 14 else "stored"
    mode = ae.HAM_STORED if args.ham == "stored" else ae.HAM_ON_THE_FLY

    e2e = e2e_uncached = None
    if not args.no_e2e:
        e2e = e2e_c_abi(pb, max(10, args.steps // 10), 2)
        e2e_uncached = e2e_c_abi(pb, max(10, args.steps // 10), 2, reuse_hpsi=False)

    from ansatzevolve_gb300 import autotune
    tuning = tuned(autotune.problem_key(N_ORB, N_A, N_B, LAYERS, 1, mode, False))
    eng = ae.Engine(2 * N_ORB, ae.BASIS_SZ, N_A + N_B, N_A, N_B, pb["ops0"], complex_mode=pb["cplx"],
                    tuning=tuning or None)
    W = 2 if pb["cplx"] else 1
    init = np.zeros(eng.D * W)
    init[W * np.searchsorted(eng.states(), pb["hf"])] = 1.0
    eng.set_initial(init)
    t0 = time.perf_counter()
    eng.set_ham_integrals(pb["h1"], pb["g2"], mode)
    setup_s = time.perf_counter() - t0
    info = eng.info()
    D = info["D"]
    ang = torch.tensor(pb["scale"] * pb["x"][pb["p0"]], dtype=torch.float64, device="cuda")
    E_d = torch.zeros(1, dtype=torch.float64, device="cuda")
    g_d = torch.zeros(len(pb["ops0"]), dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            eng.gradient_dev(ang.data_ptr(), E_d.data_ptr(), g_d.data_ptr(), sp)
    torch.cuda.synchronize()
    launches0 = eng.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            eng.gradient_dev(ang.data_ptr(), E_d.data_ptr(), g_d.data_ptr(), sp)
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = eng.launch_count() - launches0
    # per-phase CUDA-event times of the same evaluation on the stream path (the timed
    # loop above replays one captured graph, which has no events between kernels)
    eng.phase_timing(True)
    eng.phase_times()
    with torch.cuda.stream(stream):
        for _ in range(min(args.steps, 20)):
            eng.gradient_dev(ang.data_ptr(), E_d.data_ptr(), g_d.data_ptr(), sp)
    torch.cuda.synchronize()
    phase_ms, nph = eng.phase_times()
    eng.phase_timing(False)
    half = bool(eng.flip_status()[0])
    half_passes = bool(eng.half_status()[0])

    def timed_without(knobs, note):
        """The same timed loop with the given symmetry knobs switched off (then back on):
        evals/s, per-phase ms and the energy's distance from the headline run's."""
        E_sym = float(E_d.item())
        for k in knobs:
            eng.set_tuning(k, 0)
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                eng.gradient_dev(ang.data_ptr(), E_d.data_ptr(), g_d.data_ptr(), sp)
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            eng.gradient_dev(ang.data_ptr(), E_d.data_ptr(), g_d.data_ptr(), sp)
        f1.record(stream)
        torch.cuda.synchronize()
        fms = f0.elapsed_time(f1) / args.steps
        E_off = float(E_d.item())
        eng.phase_timing(True)
        eng.phase_times()
        with torch.cuda.stream(stream):
            for _ in range(min(args.steps, 20)):
                eng.gradient_dev(ang.data_ptr(), E_d.data_ptr(), g_d.data_ptr(), sp)
        torch.cuda.synchronize()
        fph, fn = eng.phase_times()
        eng.phase_timing(False)
        for k in knobs:
            eng.set_tuning(k, 1)
        with torch.cuda.stream(stream):
            eng.gradient_dev(ang.data_ptr(), E_d.data_ptr(), g_d.data_ptr(), sp)
        torch.cuda.synchronize()
        return {"value": 1e3 / fms, "unit": "evals/s", "ms_per_step": fms,
                "phase_ms": {"evolve": fph[0] / max(fn, 1), "hpsi_energy": fph[1] / max(fn, 1),
                             "adjoint": fph[2] / max(fn, 1)},
                "dE_vs_headline": abs(E_off - E_sym), "note": note}

    # the same timed loop with the spin-flip symmetry switched off, reported beside the
    # headline: the half product alone (every row of H psi computed), and everything
    # (every row and every orbit of every pass, as the reference computes them)
    full_product = full_evaluation = None
    if half:
        full_product = timed_without([ae.TUNE_FLIP], "the same loop with AEGPU_TUNE_FLIP = 0: every row of H psi "
                                                     "computed")
    if half or half_passes:
        full_evaluation = timed_without([ae.TUNE_FLIP, ae.TUNE_HALF],
                                        "the same loop with AEGPU_TUNE_FLIP = 0 and AEGPU_TUNE_HALF = 0: every row "
                                        "of H psi and every orbit of every pass computed, as the reference does")
    # one full analytic Hessian (evolveHessian), median of three, host buffers
    hess_ms = None
    if not args.no_hessian:
        ang_h = pb["scale"] * pb["x"][pb["p0"]]
        th = []
        for k in range(3):
            t0 = time.perf_counter()
            eng.hessian(ang_h + 1e-4 * k, pb["p0"], pb["scale"])
            th.append(time.perf_counter() - t0)
        hess_ms = 1e3 * float(np.median(th))
    # the properties pass's ground state: Lanczos on the same H product to 1e-8
    ground = None
    if not args.no_ground:
        runs = []
        for _ in range(3):
            t0 = time.perf_counter()
            lam, res, nprod = eng.lowest_eigenpair(tol=1e-8, basis=100, max_products=5000)
            runs.append(time.perf_counter() - t0)
        dt = float(np.median(runs))
        ground = {"ms": 1e3 * dt, "runs_ms": [round(1e3 * t, 1) for t in runs], "products": nprod,
                  "ms_per_product": 1e3 * dt / nprod, "residual": res, "eigenvalue": lam,
                  "api": "aegpu_lowest_eigenpair (Lanczos, full reorthogonalisation), median of 3, host wall time"}
    t_max = max_over_ranks(ms, dist)
    if rank != 0:
        dist.destroy_process_group()
        return
    ms_step = t_max / args.steps
    value = world * args.steps / (t_max / 1e3)

    # roofline of the dominant kernel (H*psi): algorithmic bytes per launch
    peak, peak_kind = measured_peak()
    nnz = info["nnz"]
    # the spin-flip half product needs the rows with a <= b only (nA (nA + 1) / 2 of
    # nA^2), the input x and the whole of y
    nA = int(round(D ** 0.5))
    row_frac = (nA * (nA + 1) // 2) / D if half else 1.0
    hpsi_bytes = int(nnz * row_frac) * 12 + 16 * D * W if mode == ae.HAM_STORED else 16 * D * W
    full_hpsi_bytes = nnz * 12 + 16 * D * W if mode == ae.HAM_STORED else 16 * D * W
    t_hpsi = phase_ms[1] / max(nph, 1) / 1e3
    achieved = hpsi_bytes / t_hpsi / 1e9
    coded_bytes = coded_row_bytes(D, W, nnz // D) if mode == ae.HAM_STORED else None
    if coded_bytes and half:
        # the half product streams the coded rows with a <= b (the other rows of the
        # listed 32-row slabs are skipped without loads)
        coded_bytes = int((coded_bytes - 16 * D * W) * row_frac) + 16 * D * W
    # whole-step algorithmic bytes (forward 16 B/amp/pass, H*psi, backward 32 B/amp/pass);
    # the spin-flip half passes keep the nA (nA + 1) / 2 amplitudes with a <= b
    passes = info["blocks"]
    amp_frac = (nA * (nA + 1) // 2) / D if half_passes else 1.0
    step_bytes = int(passes * 48 * D * W * amp_frac) + hpsi_bytes
    # FP64-pipe roofline of the same step: FP64 instructions per evaluation against the
    # DFMA throughput measured on this device right now
    fw = eng.fp64_work()
    fw_h = fw[0]
    peak_t = ae.fp64_peak() / 2.0  # T DFMA/s
    ph = [phase_ms[k] / max(nph, 1) / 1e3 for k in range(3)]
    fp64 = {"unit": "T FP64 instr/s", "peak": peak_t, "peak_source": "measured (aegpu_fp64_peak)",
            "instructions_per_step": int(sum(fw)),
            "achieved": sum(fw) / (ms_step / 1e3) / 1e12, "frac": sum(fw) / (ms_step / 1e3) / 1e12 / peak_t,
            "phase_frac": {"evolve": fw[1] / ph[0] / 1e12 / peak_t if ph[0] else None,
                           "hpsi_energy": fw[0] / ph[1] / 1e12 / peak_t if ph[1] else None,
                           "adjoint": fw[2] / ph[2] / 1e12 / peak_t if ph[2] else None}}
    line = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random integrals)",
        "config": workload_desc(D, pb["P"], len(pb["ops0"]),
                                ("stored in HBM as coded rows (%.1f GB: diagonal and singles explicit, doubles as "
                                 "2-byte codes into a value table)" % ((coded_bytes - 16 * D * W) / 1e9) if coded_bytes else
                                 "stored as %d-wide rows in HBM (%.1f GB)" % (info["ell_width"], nnz * 12 / 1e9))
                                if mode == ae.HAM_STORED else "regenerated on the fly"),
        "roofline": {"bound": "hbm",
                     "kernel": ("k_spmv_vell (H*psi, coded rows)" if coded_bytes else "k_spmv_sell (H*psi)")
                     if mode == ae.HAM_STORED else "k_otf_strings (H*psi)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind,
                     # algorithmic bytes: 12 B per nonzero (FP64 value + int32 column) of the rows
                     # the product computes + x, y
                     "algorithmic_bytes": hpsi_bytes,
                     "product": ("spin-flip half: rows with alpha string <= beta string, mirrored (the state "
                                 "passed the device invariance test)" if half else "full: every row"),
                     "full_product_algorithmic_bytes": full_hpsi_bytes,
                     # DRAM bytes per launch: the ncu count of the 10-orbital launch of this kernel
                     # (traffic / streamed bytes) scaled to this launch
                     "traffic": (coded_bytes * (VELL_HALF_TRAFFIC_RATIO if half else VELL_TRAFFIC_RATIO) if coded_bytes
                                 else hpsi_bytes * SELL_TRAFFIC_RATIO) if mode == ae.HAM_STORED else None,
                     "traffic_source": (("profiles/k_spmv_vell_tups10_half.md" if half else
                                         "profiles/k_spmv_vell_tups10_stored.md") + " (scaled by streamed bytes)"
                                        if coded_bytes else "profiles/k_spmv_sell_tups10_stored.md (scaled by nonzeros)")
                     if mode == ae.HAM_STORED else None,
                     "stream_bytes": coded_bytes, "stream_frac": coded_bytes / t_hpsi / 1e9 / peak if coded_bytes else None,
                     "fp64_frac": fw_h / t_hpsi / 1e12 / peak_t if fw_h else None,
                     "note": "coded rows stream 6 B per double excitation (column + 2-byte code into a value table "
                             "in shared memory) instead of 12 B, so the kernel moves about half the algorithmic "
                             "bytes and is bound by the FP64 pipe (fp64_frac); achieved counts the algorithmic "
                             "bytes" if coded_bytes else None,
                     "launch_ms": t_hpsi * 1e3},
        "step_roofline": {"algorithmic_bytes": step_bytes, "achieved_gbs": step_bytes / (ms_step / 1e3) / 1e9,
                          "frac": step_bytes / (ms_step / 1e3) / 1e9 / peak,
                          "phase_ms": {"evolve": phase_ms[0] / max(nph, 1), "hpsi_energy": phase_ms[1] / max(nph, 1),
                                       "adjoint": phase_ms[2] / max(nph, 1)}},
        "fp64_roofline": fp64,
        "gpu_launches": int(launches),
        "tuning": {"settings": {str(k): v for k, v in eng.tuning().items()}, "tuned": bool(tuning)},
        "clocks": clk.summary(),
        "setup_s": setup_s,
    }
    line["passes"] = {"count": passes,
                      "kind": ("spin-flip half passes: one orbit of every mirror pair, the amplitudes with alpha "
                               "string <= beta string kept current (every excitation's angle equals its "
                               "mirror's and the start state is symmetric)" if half_passes else "full passes")}
    if full_product:
        line["full_product"] = full_product
    if full_evaluation:
        line["full_evaluation"] = full_evaluation
    if e2e:
        line["e2e"] = e2e
        line["e2e_uncached"] = e2e_uncached
    if hess_ms is not None:
        line["hessian"] = {"ms": hess_ms, "parameters": pb["P"], "api": "aegpu_hessian (host buffers), median of 3"}
    if ground is not None:
        line["ground_state"] = ground
    eng.close()
    if not args.no_batched:
        line["batched"] = batched_bench(stream)
    if not args.no_batched:
        line["batched_columns"] = batched_columns_bench(stream)
    if not args.no_config3 and N_ORB == 12 and not LUCJ:
        line["config3"] = aux_case_bench(14, False, stream)
        line["lucj14"] = aux_case_bench(14, True, stream, steps=3)
    if not args.no_ttc:
        line["time_to_converge"] = ttc_bench(args.ttc_train, args.ttc_heldout, args.ttc_plain)
    # parity of this very run against the reference's own output for the same inputs
    # (tests/golden/ref<N>.npz, produced by the reference build)
    ref = os.path.join(ROOT, "tests", "golden", "ref%d.npz" % N_ORB)
    if os.path.exists(ref) and not LUCJ:
        fx = np.load(ref)
        if fx["x"].shape == pb["x"].shape and np.allclose(fx["x"], pb["x"]):
            g_ops = g_d.cpu().numpy()
            g = np.zeros(pb["P"])
            np.add.at(g, pb["p0"], pb["scale"] * g_ops)
            line["parity_reference"] = {"dE": abs(float(E_d.item()) - float(fx["E"])),
                                        "max_dg": float(np.max(np.abs(g - fx["G"]))),
                                        "source": "tests/golden/ref%d.npz" % N_ORB}
    if not args.no_cpu:
        cb, Eo, go = cpu_baseline(pb)
        line["cpu_baseline"] = cb
        # parity of this very run against the oracle
        g_ops = g_d.cpu().numpy()
        g = np.zeros(pb["P"])
        np.add.at(g, pb["p0"], pb["scale"] * g_ops)
        line["parity"] = {"dE": abs(float(E_d.item()) - Eo), "max_dg": float(np.max(np.abs(g - go)))}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
