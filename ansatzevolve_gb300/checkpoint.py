"""Checkpoints of optimisation state: angle sets in the reference's Parameters file
format (XX_Parameters.dat; read by loadParameters, TUPSLoadingUtils.cpp:176-290, and
described in Manual.md "The Paramter file") so a run can be resumed by the reference or
by this package, plus a compact .npz of a batched scan (angles, energies, seeds)."""
import numpy as np


def write_parameters(path, angle_sets, energies=None):
    """One block per angle set: the count, an 'Energy of minimum k= E' line (the
    reference reads the number after '='), then one angle per line, each number with
    17 significant digits so that it reads back exactly."""
    sets = [np.asarray(a, dtype=np.float64).ravel() for a in np.atleast_2d(angle_sets)]
    with open(path, "w") as f:
        for k, a in enumerate(sets):
            E = 0.0 if energies is None else float(np.atleast_1d(energies)[k])
            f.write("%d\n" % a.size)
            f.write("Energy of minimum %6d=  %.17g written by ansatzevolve_gb300\n" % (k + 1, E))
            for v in a:
                f.write("%.17g\n" % v)


def read_parameters(path):
    """(angle sets, energies) with the reference parser's rules: a count, a line whose
    number after '=' is the energy, then that many angles; repeated to the end."""
    sets, energies = [], []
    with open(path) as f:
        lines = [ln.strip() for ln in f]
    k = 0
    while k < len(lines):
        if not lines[k]:
            k += 1
            continue
        n = int(lines[k])
        head = lines[k + 1]
        energies.append(float(head.split("=", 1)[1].split()[0]) if "=" in head else 0.0)
        sets.append(np.array([float(lines[k + 2 + i]) for i in range(n)]))
        k += 2 + n
    return sets, np.array(energies)


def save_scan(path, svals, x, energies, seeds):
    """A batched scan's state: family parameters s, converged angles, energies and the
    seeds that regenerate the inputs."""
    np.savez_compressed(path, s=np.asarray(svals), x=np.asarray(x), E=np.asarray(energies),
                        seeds=np.asarray(seeds, dtype=np.int64))


def load_scan(path):
    d = np.load(path)
    return d["s"], d["x"], d["E"], d["seeds"]
