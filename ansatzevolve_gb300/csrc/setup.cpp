// Host-side setup: basis enumeration, commuting-block grouping, orbit tables.
#include "setup.h"

#include <algorithm>
#include <numeric>
#include <thread>

namespace ae {

static int popc(uint32_t x) { return __builtin_popcount(x); }

bool Basis::init(int nq_, int kind_, int ne_, int na_, int nb_, std::string &err)
{
    nq = nq_; kind = kind_; ne = ne_; na = na_; nb = nb_; N = nq / 2;
    if (nq < 1 || nq > 30) { err = "number of qubits out of range (1..30)"; return false; }
    if (kind == BASIS_SZ) {
        if (nq % 2) { err = "Sz sector needs an even number of qubits"; return false; }
        rankA.assign(1u << N, -1);
        rankB.assign(1u << N, -1);
        strA.clear(); strB.clear();
        for (uint32_t s = 0; s < (1u << N); ++s) {
            if (popc(s) == na) { rankA[s] = (int32_t)strA.size(); strA.push_back(s); }
            if (popc(s) == nb) { rankB[s] = (int32_t)strB.size(); strB.push_back(s); }
        }
        nA = (uint32_t)strA.size();
        nB = (uint32_t)strB.size();
        D = (uint64_t)nA * nB;
    } else {
        if (nq > 28) { err = "sectors without Sz symmetry are limited to 28 qubits"; return false; }
        rank.assign(1ull << nq, -1);
        states.clear();
        for (uint64_t s = 0; s < (1ull << nq); ++s)
            if (kind == BASIS_FULL || popc((uint32_t)s) == ne) {
                rank[s] = (int32_t)states.size();
                states.push_back((uint32_t)s);
            }
        D = states.size();
    }
    if (D == 0) { err = "empty determinant sector"; return false; }
    if (D >= (1ull << 31)) { err = "determinant sector too large"; return false; }
    return true;
}

// stateRotate::exc helpers, operatorpool.h:140-197.
bool exc_is_diagonal(const Exc &e)
{
    if (e.v[2] == -1) return e.v[0] == e.v[1];
    uint32_t c = (1u << e.v[0]) | (1u << e.v[1]), a = (1u << e.v[2]) | (1u << e.v[3]);
    return (c ^ a) == 0;
}

bool exc_has_diagonal(const Exc &e)
{
    if (e.v[2] == -1 && e.v[3] == -1) return e.v[0] == e.v[1];
    for (int i = 0; i < 4; ++i)
        for (int j = i + 1; j < 4; ++j)
            if (e.v[i] == e.v[j]) return true;
    return false;
}

bool exc_commutes(const Exc &x, const Exc &y)
{
    uint32_t f = 0, s = 0;
    for (int i = 0; i < 4; ++i) {
        if (x.v[i] != -1) f |= 1u << x.v[i];
        if (y.v[i] != -1) s |= 1u << y.v[i];
    }
    return !(f & s) || (exc_is_diagonal(x) && exc_is_diagonal(y));
}

std::vector<Block> group_blocks(const std::vector<Exc> &excs, int max_fuse, std::vector<int> &perm)
{
    const size_t n = excs.size();
    perm.resize(n);
    std::iota(perm.begin(), perm.end(), 0);
    auto diag = [&](size_t i) { return exc_is_diagonal(excs[perm[i]]); };
    if (n > 1) {
        size_t start = 0, end = 1;
        while (end < n) {
            bool all = true;
            while (all && end < n) {
                for (size_t k = start; k < end; ++k) {
                    bool ok = exc_commutes(excs[perm[k]], excs[perm[end]]) && diag(k) == diag(end);
                    if (!ok) { all = false; break; }
                }
                if (all) end++;
            }
            for (size_t trial = end; trial < n; ++trial) {
                bool all2 = true;
                for (size_t k = start; k < trial; ++k) {
                    if (diag(start) != diag(trial)) { all2 = false; break; }
                    if (!exc_commutes(excs[perm[k]], excs[perm[trial]])) { all2 = false; break; }
                }
                if (all2) {
                    for (size_t k = trial; k > end; --k) std::swap(perm[k], perm[k - 1]);
                    end++;
                }
            }
            start = end;
            end = start + 1;
        }
    }
    std::vector<size_t> bounds{0};
    for (size_t i = 0; i < n; ++i)
        for (size_t j = bounds.back(); j < i; ++j) {
            bool ext = exc_commutes(excs[perm[i]], excs[perm[j]]) && diag(i) == diag(j);
            if (!ext) { bounds.push_back(i); break; }
        }
    bounds.push_back(n);
    std::vector<Block> out;
    for (size_t b = 0; b + 1 < bounds.size(); ++b) {
        size_t len = bounds[b + 1] - bounds[b];
        size_t fuse = len;
        if ((int)len > max_fuse)
            for (int f = max_fuse; f > 0; --f)
                if (len % f == 0) { fuse = f; break; }
        for (size_t c = bounds[b]; c < bounds[b + 1]; c += fuse) {
            Block blk;
            blk.diagonal = diag(c);
            for (size_t k = c; k < c + fuse; ++k) blk.ops.push_back(perm[k]);
            out.push_back(std::move(blk));
        }
    }
    return out;
}

std::vector<Block> merge_commuting(const std::vector<Block> &blocks, const std::vector<Exc> &excs)
{
    std::vector<Block> out;
    for (const auto &b : blocks) {
        if (!out.empty() && !b.diagonal && !out.back().diagonal) {
            bool all = true;
            for (int x : out.back().ops) {
                for (int y : b.ops)
                    if (!exc_commutes(excs[x], excs[y])) { all = false; break; }
                if (!all) break;
            }
            if (all) {
                out.back().ops.insert(out.back().ops.end(), b.ops.begin(), b.ops.end());
                continue;
            }
        }
        out.push_back(b);
    }
    return out;
}

std::vector<int> mirror_ops(const std::vector<ExcCode> &codes, const std::vector<Block> &blocks, int N)
{
    // search domains: every paired block, and every run of consecutive diagonal blocks
    // (split_passes merges such a run before cutting it into passes)
    std::vector<std::vector<int>> domains;
    bool run = false;
    for (const auto &b : blocks) {
        if (!(b.diagonal && run)) domains.emplace_back();
        domains.back().insert(domains.back().end(), b.ops.begin(), b.ops.end());
        run = b.diagonal;
    }
    std::vector<int> mir(codes.size(), -1);
    for (const auto &dom : domains)
        for (int o : dom) {
            if (mir[o] >= 0) continue;
            const uint32_t fc = flip_bits(codes[o].create, N), fa = flip_bits(codes[o].annihilate, N);
            for (int p : dom)
                if (mir[p] < 0 && codes[p].create == fc && codes[p].annihilate == fa && (p != o || fc == codes[o].create)) {
                    mir[o] = p;
                    mir[p] = o;
                    break;
                }
        }
    return mir;
}

// A paired block cut between mirror units: the units in order of first appearance,
// packed greedily into the fewest passes of <= max_pass operators with near-equal
// operator counts.  Empty result: the block is not closed under the mirror.
static std::vector<Block> split_by_mirror(const Block &b, int max_pass, const std::vector<int> &mir)
{
    std::vector<std::vector<int>> units;
    std::vector<char> seen(mir.size(), 0);
    for (int o : b.ops) {
        if (seen[o]) continue;
        const int m = mir[o];
        if (m < 0 || std::find(b.ops.begin(), b.ops.end(), m) == b.ops.end()) return {};
        seen[o] = 1;
        if (m == o) {
            units.push_back({o});
        } else {
            seen[m] = 1;
            units.push_back({o, m});
        }
    }
    const int n = (int)b.ops.size();
    for (auto &u : units)
        if ((int)u.size() > max_pass) return {};
    int parts = (n + max_pass - 1) / max_pass;
    for (;; ++parts) {  // the fewest passes the units fit in, near-equal by count
        std::vector<Block> out;
        Block cur;
        int done = 0, k = 0;
        bool fits = true;
        for (auto &u : units) {
            const int bound = (int)((int64_t)n * (k + 1) / parts);
            if (!cur.ops.empty() && (done + (int)u.size() > bound || (int)(cur.ops.size() + u.size()) > max_pass)) {
                out.push_back(cur);
                cur = Block{};
                ++k;
            }
            cur.ops.insert(cur.ops.end(), u.begin(), u.end());
            done += (int)u.size();
            if ((int)cur.ops.size() > max_pass) fits = false;
        }
        if (!cur.ops.empty()) out.push_back(cur);
        if (fits && (int)out.size() <= parts) return out;
    }
}

std::vector<Block> split_passes(const std::vector<Block> &blocks, int max_pass, const std::vector<int> *mirror)
{
    std::vector<Block> out;
    // Consecutive diagonal blocks form one run (any two diagonal operators commute):
    // the divisor rule of the grouping cuts a run of prime length into single-operator
    // blocks, each of which would be a full sweep over the statevector.  The run is
    // cut into the fewest near-equal passes of <= kMaxDiagSlots operators instead, in
    // the same operator order.
    std::vector<int> run;
    auto flush = [&]() {
        const int n = (int)run.size();
        if (!n) return;
        if (mirror && n > kMaxDiagSlots) {
            Block r;
            r.diagonal = true;
            r.ops = run;
            std::vector<Block> cut = split_by_mirror(r, kMaxDiagSlots, *mirror);
            if (!cut.empty()) {
                for (auto &c : cut) c.diagonal = true;
                out.insert(out.end(), cut.begin(), cut.end());
                run.clear();
                return;
            }
        }
        const int parts = (n + kMaxDiagSlots - 1) / kMaxDiagSlots;
        int start = 0;
        for (int p = 0; p < parts; ++p) {
            const int len = n / parts + (p < n % parts ? 1 : 0);
            Block c;
            c.diagonal = true;
            c.ops.assign(run.begin() + start, run.begin() + start + len);
            start += len;
            out.push_back(std::move(c));
        }
        run.clear();
    };
    for (const auto &b : blocks) {
        const int n = (int)b.ops.size();
        if (b.diagonal) {
            run.insert(run.end(), b.ops.begin(), b.ops.end());
            continue;
        }
        flush();
        if (n <= max_pass) {
            out.push_back(b);
            continue;
        }
        if (mirror) {
            std::vector<Block> cut = split_by_mirror(b, max_pass, *mirror);
            if (!cut.empty()) {
                out.insert(out.end(), cut.begin(), cut.end());
                continue;
            }
        }
        const int parts = (n + max_pass - 1) / max_pass;
        int start = 0;
        for (int p = 0; p < parts; ++p) {
            const int len = n / parts + (p < n % parts ? 1 : 0);
            Block c;
            c.diagonal = false;
            c.ops.assign(b.ops.begin() + start, b.ops.begin() + start + len);
            start += len;
            out.push_back(std::move(c));
        }
    }
    flush();
    return out;
}

OrbitTables build_orbits(const Basis &B, const std::vector<ExcCode> &codes, int nthreads)
{
    const int nb = (int)codes.size();
    const uint32_t nmask = 1u << nb;
    const uint64_t D = B.D;
    if (nthreads < 1) nthreads = 1;
    // pass 1 (parallel over rank ranges): per chunk, the roots of every mask in ascending order
    struct Chunk { std::vector<std::vector<uint32_t>> roots; };
    std::vector<Chunk> chunks(nthreads);
    auto work = [&](int t) {
        uint64_t lo = D * t / nthreads, hi = D * (t + 1) / nthreads;
        auto &roots = chunks[t].roots;
        roots.assign(nmask, {});
        for (uint64_t z = lo; z < hi; ++z) {
            uint32_t s = B.bits(z), m = 0;
            bool root = true;
            for (int i = 0; i < nb; ++i) {
                uint32_t p; int sg;
                if (apply_exc(codes[i], s, p, sg) == 1) {
                    if (p < s) { root = false; break; }
                    m |= 1u << i;
                }
            }
            if (root && m) roots[m].push_back((uint32_t)z);
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();

    OrbitTables T;
    for (uint32_t m = 1; m < nmask; ++m) {
        uint64_t nroots = 0;
        for (auto &c : chunks) nroots += c.roots[m].size();
        if (!nroots) continue;
        OrbitGroup g{};
        g.idx_off = (uint32_t)T.idx.size();
        g.n_orbits = (uint32_t)nroots;
        g.mask = m;
        g.k = 0;
        for (int i = 0; i < nb; ++i)
            if (m & (1u << i)) g.slot[g.k++] = (int8_t)i;
        const uint32_t osz = 1u << g.k;
        T.idx.reserve(T.idx.size() + nroots * osz);
        T.bits.reserve(T.bits.size() + nroots * osz);
        std::vector<uint32_t> orb(osz);
        for (auto &c : chunks)
            for (uint32_t root : c.roots[m]) {
                orb[0] = B.bits(root);
                for (uint32_t i = 0; i < g.k; ++i) {
                    const uint32_t stride = 1u << i;
                    for (uint32_t q = 0; q < stride; ++q) {
                        uint32_t p; int sg;
                        apply_exc(codes[g.slot[i]], orb[q], p, sg);
                        orb[q + stride] = p;
                    }
                }
                for (uint32_t q = 0; q < osz; ++q) {
                    int64_t r = B.rank_of(orb[q]);
                    if (r < 0) T.ok = false;
                    T.idx.push_back((uint32_t)(r < 0 ? 0 : r));
                    T.bits.push_back(orb[q]);
                }
            }
        const uint32_t per_tile = osz >= (uint32_t)kTileElems ? 1u : (uint32_t)kTileElems / osz;
        for (uint32_t o = 0; o < g.n_orbits; o += per_tile) {
            OrbitTile t{};
            t.group = (uint32_t)T.groups.size();
            t.orbit0 = o;
            t.n_orbits = std::min(per_tile, g.n_orbits - o);
            t.elem_off = g.idx_off + o * osz;
            T.tiles.push_back(t);
        }
        if (g.k <= (uint32_t)kMaxWarpLayers) {
            const uint32_t per_task = (uint32_t)kWarpElems / osz;
            for (uint32_t o = 0; o < g.n_orbits; o += per_task) {
                WarpTask w{};
                w.group = (uint32_t)T.groups.size();
                w.elem_off = g.idx_off + o * osz;
                w.n = std::min(per_task, g.n_orbits - o) * osz;
                w.mask = m;
                T.wtasks.push_back(w);
            }
        }
        T.groups.push_back(g);
        T.active += nroots * osz;
        T.amp_layers += nroots * osz * g.k;
    }
    return T;
}

bool make_passes(const std::vector<Exc> &excs, const std::vector<ExcCode> &codes, int N, int max_pass,
                 bool mirror_split, std::vector<Block> &passes, std::vector<int> &perm, std::vector<int> &mirror)
{
    std::vector<Block> grouped = group_blocks(excs, kMaxDiagSlots, perm);
    mirror.clear();
    bool half = mirror_split;
    if (half) {
        grouped = merge_commuting(grouped, excs);
        mirror = mirror_ops(codes, grouped, N);
        for (int m : mirror) half = half && m >= 0;
        if (!half) mirror.clear();
    }
    passes = split_passes(grouped, max_pass, half ? &mirror : nullptr);
    // the application order is the passes' order (a cut between mirror units may
    // reorder operators inside a commuting run)
    perm.clear();
    for (const Block &b : passes) perm.insert(perm.end(), b.ops.begin(), b.ops.end());
    return half;
}

HalfTables build_half_orbits(const Basis &B, const OrbitTables &T, const std::vector<ExcCode> &codes,
                             const std::vector<int> &mslot, int nthreads)
{
    HalfTables H;
    const int N = B.N;
    const uint32_t lo = (1u << N) - 1u;
    if (B.kind != BASIS_SZ || B.nA != B.nB) {
        H.ok = false;
        return H;
    }
    if (nthreads < 1) nthreads = 1;
    for (size_t gi = 0; gi < T.groups.size(); ++gi) {
        const OrbitGroup &g = T.groups[gi];
        if (g.k > (uint32_t)kMaxWarpLayers) {
            H.ok = false;
            return H;
        }
        const uint32_t osz = 1u << g.k;
        // per orbit: 0 its mirror is kept, 1 kept (one of a mirror pair), 2 kept (its own
        // mirror), 3 a rank or sign check failed; classified in parallel over orbit ranges
        std::vector<uint8_t> cls(g.n_orbits, 0);
        int nt = 1;
        auto work = [&](int t) {
            const uint32_t o0 = (uint32_t)((uint64_t)g.n_orbits * t / nt);
            const uint32_t o1 = (uint32_t)((uint64_t)g.n_orbits * (t + 1) / nt);
            for (uint32_t o = o0; o < o1; ++o) {
                const size_t off = g.idx_off + (size_t)o * osz;
                uint32_t key = UINT32_MAX, mkey = UINT32_MAX;
                bool bad = false;
                for (uint32_t q = 0; q < osz && !bad; ++q) {
                    const uint32_t s = T.bits[off + q], fs = flip_bits(s, N);
                    const int64_t r = B.rank_of(fs);
                    if (r < 0) {
                        bad = true;
                        break;
                    }
                    key = std::min(key, T.idx[off + q]);
                    mkey = std::min(mkey, (uint32_t)r);
                    for (uint32_t l = 0; l < g.k; ++l) {
                        const int sl = g.slot[l];
                        if (mslot[sl] < 0 || exc_sign(codes[sl], s) != exc_sign(codes[mslot[sl]], fs)) {
                            bad = true;
                            break;
                        }
                    }
                }
                cls[o] = bad ? 3 : key < mkey ? 1 : key == mkey ? 2 : 0;
            }
        };
        // threads only for large groups (spawning them costs more than small groups' work)
        nt = (int)std::min<uint64_t>((uint64_t)nthreads, std::max<uint64_t>(1, (uint64_t)g.n_orbits * osz >> 16));
        std::vector<std::thread> th;
        for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
        work(0);
        for (auto &x : th) x.join();
        std::vector<uint32_t> keep[2];  // [0] one of a mirror pair, [1] self-mirror
        for (uint32_t o = 0; o < g.n_orbits; ++o) {
            if (cls[o] == 3) {
                H.ok = false;
                return H;
            }
            if (cls[o]) keep[cls[o] - 1].push_back(o);
        }
        for (int self = 0; self < 2; ++self) {
            const uint32_t first = (uint32_t)H.idx.size();
            for (uint32_t o : keep[self]) {
                const size_t off = g.idx_off + (size_t)o * osz;
                for (uint32_t q = 0; q < osz; ++q) {
                    const uint32_t s = T.bits[off + q];
                    const uint32_t x = (uint32_t)B.rankA[s >> N], y = (uint32_t)B.rankB[s & lo];
                    H.idx.push_back(std::min(x, y) * B.nB + std::max(x, y));
                    H.bits.push_back(s | ((self && x > y) ? kNoWriteBit : 0u));
                }
            }
            const uint32_t per_task = (uint32_t)kWarpElems / osz, nk = (uint32_t)keep[self].size();
            for (uint32_t o = 0; o < nk; o += per_task) {
                WarpTask w{};
                w.group = (uint32_t)gi | (self ? kSelfMirrorTask : 0u);
                w.elem_off = first + o * osz;
                w.n = std::min(per_task, nk - o) * osz;
                w.mask = g.mask;
                H.wtasks.push_back(w);
            }
            H.active += (uint64_t)nk * osz;
            H.amp_layers += (uint64_t)nk * osz * g.k;
        }
    }
    return H;
}

}  // namespace ae

// ------------------------------------------------------------ host inspection --
#include "../../include/aegpu.h"

extern "C" int aegpu_host_block_layout(int nq, int nops, const int *ops, int *perm, int *block_sizes, int *n_blocks)
{
    if (nops < 1 || !ops || !n_blocks) return AEGPU_ERR_ARG;
    std::vector<ae::Exc> excs(nops);
    for (int i = 0; i < nops; ++i)
        for (int j = 0; j < 4; ++j) {
            if (ops[4 * i + j] < -1 || ops[4 * i + j] >= nq) return AEGPU_ERR_ARG;
            excs[i].v[j] = (int8_t)ops[4 * i + j];
        }
    std::vector<int> p;
    auto blocks = ae::group_blocks(excs, 12, p);
    if (perm) std::copy(p.begin(), p.end(), perm);
    if (block_sizes)
        for (size_t b = 0; b < blocks.size() && (int)b < *n_blocks; ++b)
            block_sizes[b] = (int)blocks[b].ops.size() * (blocks[b].diagonal ? -1 : 1);
    *n_blocks = (int)blocks.size();
    return AEGPU_OK;
}

extern "C" int aegpu_host_orbits(int nq, int kind, int ne, int na, int nb, int nops, const int *ops, uint32_t *idx,
                                 int64_t *n_idx, uint32_t *groups, int64_t *n_groups, uint32_t *tiles, int64_t *n_tiles)
{
    if (nops < 1 || nops > 12 || !ops || !n_idx || !n_groups || !n_tiles) return AEGPU_ERR_ARG;
    ae::Basis B;
    std::string err;
    if (!B.init(nq, kind, ne, na, nb, err)) return AEGPU_ERR_ARG;
    std::vector<ae::ExcCode> codes;
    for (int i = 0; i < nops; ++i) codes.push_back(ae::make_exc_code(ops[4 * i], ops[4 * i + 1], ops[4 * i + 2], ops[4 * i + 3]));
    ae::OrbitTables T = ae::build_orbits(B, codes, 2);
    if (!T.ok) return AEGPU_ERR_UNSUPPORTED;
    const int64_t ci = *n_idx, cg = *n_groups, ct = *n_tiles;
    *n_idx = (int64_t)T.idx.size();
    *n_groups = (int64_t)T.groups.size();
    *n_tiles = (int64_t)T.tiles.size();
    if (idx && ci >= *n_idx) std::copy(T.idx.begin(), T.idx.end(), idx);
    if (groups && cg >= *n_groups)
        for (size_t g = 0; g < T.groups.size(); ++g) {
            groups[4 * g] = T.groups[g].idx_off;
            groups[4 * g + 1] = T.groups[g].n_orbits;
            groups[4 * g + 2] = T.groups[g].k;
            groups[4 * g + 3] = T.groups[g].mask;
        }
    if (tiles && ct >= *n_tiles)
        for (size_t t = 0; t < T.tiles.size(); ++t) {
            tiles[4 * t] = T.tiles[t].group;
            tiles[4 * t + 1] = T.tiles[t].orbit0;
            tiles[4 * t + 2] = T.tiles[t].n_orbits;
            tiles[4 * t + 3] = T.tiles[t].elem_off;
        }
    return AEGPU_OK;
}

extern "C" int aegpu_host_half_orbits(int nq, int nA_elec, int nops, const int *ops, uint32_t *idx, uint32_t *bits,
                                      int64_t *n_idx, uint32_t *tasks, int64_t *n_tasks)
{
    if (nops < 1 || nops > 12 || !ops || !n_idx || !n_tasks || nq % 2) return AEGPU_ERR_ARG;
    ae::Basis B;
    std::string err;
    if (!B.init(nq, ae::BASIS_SZ, 2 * nA_elec, nA_elec, nA_elec, err)) return AEGPU_ERR_ARG;
    std::vector<ae::ExcCode> codes;
    ae::Block blk;
    for (int i = 0; i < nops; ++i) {
        for (int j = 0; j < 4; ++j)
            if (ops[4 * i + j] < -1 || ops[4 * i + j] >= nq) return AEGPU_ERR_ARG;
        codes.push_back(ae::make_exc_code(ops[4 * i], ops[4 * i + 1], ops[4 * i + 2], ops[4 * i + 3]));
        blk.ops.push_back(i);
    }
    const std::vector<int> mir = ae::mirror_ops(codes, {blk}, B.N);
    for (int m : mir)
        if (m < 0) return AEGPU_ERR_UNSUPPORTED;
    ae::OrbitTables T = ae::build_orbits(B, codes, 2);
    if (!T.ok) return AEGPU_ERR_UNSUPPORTED;
    ae::HalfTables H = ae::build_half_orbits(B, T, codes, mir, 2);
    if (!H.ok) return AEGPU_ERR_UNSUPPORTED;
    const int64_t ci = *n_idx, ct = *n_tasks;
    *n_idx = (int64_t)H.idx.size();
    *n_tasks = (int64_t)H.wtasks.size();
    if (idx && bits && ci >= *n_idx) {
        std::copy(H.idx.begin(), H.idx.end(), idx);
        std::copy(H.bits.begin(), H.bits.end(), bits);
    }
    if (tasks && ct >= *n_tasks)
        for (size_t t = 0; t < H.wtasks.size(); ++t) {
            tasks[4 * t] = H.wtasks[t].group;
            tasks[4 * t + 1] = H.wtasks[t].elem_off;
            tasks[4 * t + 2] = H.wtasks[t].n;
            tasks[4 * t + 3] = H.wtasks[t].mask;
        }
    return AEGPU_OK;
}

extern "C" int aegpu_host_pass_layout(int nq, int nops, const int *ops, int max_pass, int mirror_split, int *pass_ops,
                                      int *pass_sizes, int *n_passes)
{
    if (nops < 1 || !ops || !n_passes || max_pass < 1 || max_pass > ae::kMaxWarpLayers || nq % 2) return AEGPU_ERR_ARG;
    std::vector<ae::Exc> excs(nops);
    std::vector<ae::ExcCode> codes(nops);
    for (int i = 0; i < nops; ++i) {
        for (int j = 0; j < 4; ++j) {
            if (ops[4 * i + j] < -1 || ops[4 * i + j] >= nq) return AEGPU_ERR_ARG;
            excs[i].v[j] = (int8_t)ops[4 * i + j];
        }
        codes[i] = ae::make_exc_code(ops[4 * i], ops[4 * i + 1], ops[4 * i + 2], ops[4 * i + 3]);
    }
    std::vector<int> perm, mir;
    std::vector<ae::Block> passes;
    const bool half = ae::make_passes(excs, codes, nq / 2, max_pass, mirror_split != 0, passes, perm, mir);
    const int cap = *n_passes;
    *n_passes = (int)passes.size();
    if (pass_sizes && pass_ops && cap >= *n_passes) {
        int k = 0;
        for (size_t p = 0; p < passes.size(); ++p) {
            pass_sizes[p] = (int)passes[p].ops.size() * (passes[p].diagonal ? -1 : 1);
            for (int o : passes[p].ops) pass_ops[k++] = o;
        }
    }
    return half || !mirror_split ? AEGPU_OK : AEGPU_ERR_UNSUPPORTED;
}
