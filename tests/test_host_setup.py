"""CPU tests of the host-side setup logic and of the library boundary (no GPU).

* fused-block grouping reproduces the reference's regenCache layout
  (fusedevolve.cpp:1797-1967) for the TUPS circuits of the benchmark configurations;
* orbit tables, interpreted step by step in numpy, evolve a vector exactly like the
  oracle applying the same excitations one at a time;
* the spin-flip half tables of a pass cover the canonical amplitudes (alpha string <=
  beta string) of the full pass once each, and a pass without mirrors is refused;
* the engine's passes merge runs of diagonal blocks and, for the half passes, keep
  every operator's mirror in its pass;
* the shared library exports every symbol declared in include/*.h.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from ansatzevolve_gb300 import host_block_layout, host_orbits, LIB_PATH, lib
from ansatzevolve_gb300.synthetic import tups_operators
from oracle.oracle import Oracle, exc_apply
from tests.conftest import ROOT


@pytest.mark.parametrize("N,layers,expected", [
    (8, 2, [8, 4, 8, 6, 3, 6] * 2),
    (10, 3, [10, 5, 10, 8, 4, 8] * 3),
    (12, 3, [12, 6, 12, 10, 5, 10] * 3),
    (14, 4, [7, 7, 7, 7, 7, 12, 6, 12] * 4),
])
def test_block_layout_matches_reference_grouping(N, layers, expected):
    ops, _, _ = tups_operators(N, layers)
    perm, sizes = host_block_layout(2 * N, ops - 1)
    assert list(sizes) == expected
    assert sorted(perm) == list(range(len(ops)))


def _interpret_orbits(st, ops0, idx, groups, ang, v):
    """Apply one block through its orbit tables the way the GPU kernel does."""
    v = v.copy()
    for off, norb, k, mask in groups:
        slots = [i for i in range(len(ops0)) if mask & (1 << i)]
        assert len(slots) == k
        n = 1 << k
        for o in range(norb):
            mem = idx[off + o * n: off + (o + 1) * n].astype(np.int64)
            x = v[mem]
            for layer, sl in enumerate(slots):
                S, C = np.sin(ang[sl]), np.cos(ang[sl])
                for p in range(n // 2):
                    lo = ((p >> layer) << (layer + 1)) | (p & ((1 << layer) - 1))
                    hi = lo | (1 << layer)
                    kind, partner, s = exc_apply(int(st[mem[lo]]), ops0[sl])
                    assert kind == 1 and partner == st[mem[hi]]
                    a, b = x[lo], x[hi]
                    x[lo] = s * S * b + C * a
                    x[hi] = -s * S * a + C * b
            v[mem] = x
    return v


@pytest.mark.parametrize("N,na,nb", [(4, 2, 2), (5, 3, 2)])
def test_orbit_tables_reproduce_sequential_rotations(N, na, nb):
    ops, _, _ = tups_operators(N, 1)
    ops0 = ops - 1
    perm, sizes = host_block_layout(2 * N, ops0)
    rng = np.random.default_rng(7)
    o = Oracle(2 * N, 2, na + nb, na, nb)
    st = o.states()
    start = 0
    for bs in sizes:
        blk = ops0[perm[start:start + bs]]
        start += bs
        idx, groups, tiles = host_orbits(2 * N, 2, na + nb, na, nb, blk)
        # every determinant appears at most once, tiles cover the rank list in order
        assert len(np.unique(idx)) == len(idx)
        assert tiles[0, 3] == 0 and tiles[-1, 3] + (tiles[-1, 2] << groups[tiles[-1, 0], 2]) == len(idx)
        ang = rng.uniform(-1, 1, bs)
        v = rng.normal(size=len(st))
        got = _interpret_orbits(st, blk, idx, groups, ang, v)
        o.set_initial(st, v)
        o.set_ops(blk, np.arange(bs), np.ones(bs))
        want = o.evolve_ops(ang)
        np.testing.assert_allclose(got, want, atol=1e-14, rtol=0)


def _declared_symbols():
    names = set()
    for h in sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(\w+)\s*\(", src, flags=re.M):
            if m.group(1) not in ("if", "defined", "extern"):
                names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    lib()
    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    declared = _declared_symbols()
    assert len(declared) >= 40
    missing = sorted(declared - exported)
    assert not missing, missing


@pytest.mark.parametrize("block", [0, 1])
def test_half_tables_cover_the_canonical_amplitudes_once(block):
    """Spin-flip half tables of a tUPS pass (8 orbitals: three alpha/beta single pairs,
    then the paired doubles): the amplitudes that write are the canonical (a <= b)
    images of every amplitude the full pass touches, each exactly once; an entry's rank
    is the canonical rank of its bitstring; members that do not write sit only in
    self-mirror tasks; the tables hold about half the full pass."""
    from ansatzevolve_gb300 import host_half_orbits
    N, na = 8, 4
    ops, _, _ = tups_operators(N, 2)
    ops0 = np.asarray(ops) - 1
    perm, sizes = host_block_layout(2 * N, ops0)
    first = int(np.sum(np.abs(sizes[:block])))
    sel = ops0[perm[first:first + min(6, abs(int(sizes[block])))]]
    full, _, _ = host_orbits(2 * N, 2, 2 * na, na, na, sel)
    idx, bits, tasks = host_half_orbits(2 * N, na, sel)
    strs = np.array([s for s in range(1 << N) if bin(s).count("1") == na])
    nB = len(strs)
    rank = {int(s): i for i, s in enumerate(strs)}

    def canon(r):
        a, b = divmod(int(r), nB)
        return min(a, b) * nB + max(a, b)

    write = (bits & (1 << 31)) == 0
    got = [int(r) for r in idx[write]]
    want = sorted({canon(r) for r in full})
    assert sorted(got) == want  # every canonical amplitude once
    lo = (1 << N) - 1
    for r, s in zip(idx, bits & 0x7FFFFFFF):
        a, b = rank[int(s) >> N], rank[int(s) & lo]
        assert int(r) == min(a, b) * nB + max(a, b)
    for g, off, n, m in tasks:
        if not (g >> 31):
            assert np.all(write[off:off + n])
    assert len(idx) < 0.6 * len(full)


def test_half_tables_refuse_a_pass_without_mirrors():
    """Alpha singles alone have no beta mirrors: no half tables."""
    from ansatzevolve_gb300 import AegpuError, host_half_orbits
    N = 8
    sel = np.array([[N + 1, N + 0, -1, -1], [N + 3, N + 2, -1, -1]])
    with pytest.raises(AegpuError):
        host_half_orbits(2 * N, 4, sel)


def test_pass_layout_merges_diagonal_runs_and_cuts_between_mirrors():
    """The engine's passes: the 14-orbital LUCJ circuit's runs of diagonal blocks merged
    into passes of at most 12 operators (the grouping alone leaves 254 diagonal blocks,
    177 of them single); with the mirror cut every pass holds the mirror of each of its
    operators, and the 14-orbital tUPS blocks that the divisor rule cut in two (14 -> 7
    + 7) are whole again; every operator appears once in grouping order within a run."""
    from ansatzevolve_gb300 import host_pass_layout
    from ansatzevolve_gb300.lucj import lucj_operators, random_lucj
    N = 14
    K, J = random_lucj(N, 3)
    ops, _ = lucj_operators(K, J)
    passes, diag, mirrored = host_pass_layout(2 * N, ops, 6, False)
    assert not mirrored
    assert sum(diag) == 90 and len(passes) == 170
    assert all(len(p) <= (12 if d else 6) for p, d in zip(passes, diag))
    assert sorted(np.concatenate(passes)) == list(range(len(ops)))
    passes, diag, mirrored = host_pass_layout(2 * N, ops, 6, True)
    assert mirrored
    assert sum(diag) == 92 and len(passes) == 170  # the engine's layout (78 rotation passes)

    def mirror(o):
        f = lambda i: -1 if i < 0 else (i + N if i < N else i - N)
        return tuple(f(int(i)) for i in o)

    def masks(o):
        a, b, c, d = (int(i) for i in o)
        return (frozenset([a]), frozenset([b])) if c < 0 else (frozenset([a, b]), frozenset([c, d]))

    for p in passes:
        ms = [masks(ops[o]) for o in p]
        for o in p:
            assert masks(mirror(ops[o])) in ms
    tops, _, _ = tups_operators(N, 4)
    tp, td, tm = host_pass_layout(2 * N, tops - 1, 6, True)
    assert tm and not any(td)
    assert len(tp) == 52  # 13 passes per layer: 14 -> 4+4+6, 7 -> 3+4, 14 -> 4+4+6, 12 -> 6+6, 6, 12 -> 6+6
