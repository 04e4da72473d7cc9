// Host-side setup for the GPU engine: determinant basis, commuting-block grouping
// and per-block orbit tables.  Runs once per problem shape; the tables are then
// uploaded to HBM and consumed by the block-rotation kernels in engine.cu.
#pragma once
#include "exc_rule.h"
#include <cstdint>
#include <string>
#include <vector>

namespace ae {

enum BasisKind { BASIS_FULL = 0, BASIS_NUMBER = 1, BASIS_SZ = 2 };

// Sector basis in ascending bitstring order (the reference's decompressPerm,
// operatorpool.cpp:207-242 / operatorpool.h:49-77).  In the Sz sector a
// determinant is (alpha string << N) | beta string, so its rank is
// rankA[alpha] * nB + rankB[beta]: alpha strings select rows of a nA x nB matrix.
struct Basis {
    int nq = 0, N = 0, kind = BASIS_FULL;
    int ne = 0, na = 0, nb = 0;
    uint64_t D = 0;
    uint32_t nA = 0, nB = 0;
    std::vector<uint32_t> strA, strB;    // Sz: alpha / beta strings, ascending
    std::vector<int32_t> rankA, rankB;   // Sz: 2^N tables, -1 outside the sector
    std::vector<uint32_t> states;        // FULL / NUMBER: rank -> bitstring
    std::vector<int32_t> rank;           // FULL / NUMBER: 2^nq table, -1 outside

    bool init(int nq, int kind, int ne, int na, int nb, std::string &err);
    uint32_t bits(uint64_t z) const
    {
        if (kind == BASIS_SZ) return (strA[z / nB] << N) | strB[z % nB];
        return states[z];
    }
    int64_t rank_of(uint32_t s) const
    {
        if (kind == BASIS_SZ) {
            int32_t a = rankA[s >> N], b = rankB[s & ((1u << N) - 1u)];
            return (a < 0 || b < 0) ? -1 : (int64_t)a * nB + b;
        }
        if (s >= (1ull << nq)) return -1;
        return rank[s];
    }
};

struct Exc {
    int8_t v[4];
};

// One fused pass: a run of mutually commuting excitations (all diagonal or all
// paired) applied as a single sweep over the statevector.
struct Block {
    bool diagonal = false;
    std::vector<int> ops;   // operator indices (original order) in application order
};

// Operators per diagonal pass: the phase table of a pass has 2^kMaxDiagSlots entries.
constexpr int kMaxDiagSlots = 12;

// Cut every paired block into passes of at most max_pass excitations (commuting, so
// any cut gives the same product); orbits of a pass then have at most 2^max_pass
// members.  Runs of consecutive diagonal blocks are merged and cut into the fewest
// near-equal passes of at most kMaxDiagSlots operators.  The operator order (the
// grouping's permutation) is unchanged.
// mirror (nullable): operator -> its spin-flip mirror (mirror_ops); a paired block in
// which every operator's mirror lies is cut between mirror units (a pair, or one
// operator that is its own mirror), so that every pass holds the mirrors of its
// operators.
std::vector<Block> split_passes(const std::vector<Block> &blocks, int max_pass,
                                const std::vector<int> *mirror = nullptr);

// Consecutive paired blocks whose operators all commute (the grouping's divisor rule
// cuts a commuting run of, e.g., 14 operators into two blocks of 7) merged into one,
// in the same operator order, so that split_passes can cut the run between mirror
// units.
std::vector<Block> merge_commuting(const std::vector<Block> &blocks, const std::vector<Exc> &excs);

// Spin-flip mirror of every operator (Sz basis, N spatial orbitals): the operator of
// the same block (for a diagonal operator: of the same run of consecutive diagonal
// blocks) whose created and annihilated orbitals are this one's with alpha and beta
// exchanged (itself for a paired double or a density-density operator of one
// alpha-beta pair), -1 if there is none.  Operators with equal masks are paired in
// order.
std::vector<int> mirror_ops(const std::vector<ExcCode> &codes, const std::vector<Block> &blocks, int N);

// The engine's passes for an operator list: the grouping (group_blocks), then with
// mirror_split (Sz basis, as many alpha as beta strings) commuting blocks merged
// (merge_commuting), mirrors found (mirror_ops) and the blocks cut between mirror units;
// split_passes in either case.  perm receives the application order (the passes'
// operators in order), mirror the operator -> mirror map where every operator has one
// (empty otherwise), and the result tells whether the mirror cut was applied.
bool make_passes(const std::vector<Exc> &excs, const std::vector<ExcCode> &codes, int N, int max_pass,
                 bool mirror_split, std::vector<Block> &passes, std::vector<int> &perm, std::vector<int> &mirror);

// Bitstring with the alpha (high N bits) and beta (low N bits) strings exchanged.
inline uint32_t flip_bits(uint32_t s, int N)
{
    const uint32_t lo = (1u << N) - 1u;
    return ((s & lo) << N) | ((s >> N) & lo);
}

// Greedy commuting-block grouping with forward moves, restating
// FusedEvolve::regenCache (fusedevolve.cpp:1797-1967): a block grows while the next
// operator commutes with all members (diagonal only with diagonal); later operators
// that commute with the block and with everything they jump over are moved
// forward into it; blocks longer than max_fuse are cut into equal chunks of the
// largest divisor <= max_fuse (fusedevolve.cpp:1915-1926).
std::vector<Block> group_blocks(const std::vector<Exc> &excs, int max_fuse, std::vector<int> &perm);

bool exc_is_diagonal(const Exc &e);
bool exc_has_diagonal(const Exc &e);
bool exc_commutes(const Exc &x, const Exc &y);

// Orbit tables of one paired block (fusedevolve.cpp:718-915 restated for the GPU).
// Every determinant on which at least one block excitation acts lies on exactly one
// orbit: the hypercube {apply(T, root) : T subset of its active excitations}; the
// root is the member that every active excitation maps to a larger bitstring.
// Orbits are grouped by active mask; inside a group they are listed by ascending
// root, each as 2^k ranks in hypercube order (bit i of the position = i-th active
// excitation applied).  A tile is a run of whole orbits of one group with at most
// kTileElems members: one CTA stages a tile in shared memory and applies all k
// butterfly layers there, so the statevector crosses HBM once per block.
constexpr int kTileElems = 4096;

struct OrbitGroup {
    uint32_t idx_off;    // first entry in the block's rank list
    uint32_t n_orbits;
    uint32_t k;          // active excitations per orbit
    uint32_t mask;       // block-local active mask
    int8_t slot[16];     // block-local excitation slot of layer i
};

struct OrbitTile {
    uint32_t group;
    uint32_t orbit0;
    uint32_t n_orbits;
    uint32_t elem_off;   // first entry in the block's rank list
};

// A warp task is a run of whole orbits of one group with at most 64 members (the
// orbits of a pass of <= 6 excitations): one warp holds it in registers, two
// amplitudes per lane, and runs every butterfly layer with shuffles.
constexpr int kWarpElems = 64;
constexpr int kMaxWarpLayers = 6;

struct WarpTask {
    uint32_t group;
    uint32_t elem_off;   // first entry in the block's rank list
    uint32_t n;          // members (<= 64)
    uint32_t mask;       // the group's active-excitation mask
};

struct OrbitTables {
    std::vector<uint32_t> idx;        // ranks, grouped / ordered as described
    std::vector<uint32_t> bits;       // the determinants' bitstrings, parallel to idx
    std::vector<OrbitGroup> groups;
    std::vector<OrbitTile> tiles;
    std::vector<WarpTask> wtasks;     // only when every orbit has <= 64 members
    uint64_t active = 0;              // number of determinants touched by the block
    uint64_t amp_layers = 0;          // sum over touched determinants of their active layers
    bool ok = true;                   // false if an excitation leaves the sector
};

OrbitTables build_orbits(const Basis &B, const std::vector<ExcCode> &codes, int nthreads);

// Spin-flip half tables of a pass (Sz basis with as many alpha as beta strings).  When
// the pass holds the mirror of each of its operators and each operator's sign on a
// determinant equals its mirror's sign on the mirrored determinant, the pass commutes
// with the exchange of the alpha and beta strings, so a state with psi(a,b) =
// psi(b,a) keeps that symmetry and only the amplitudes with a <= b need to be stored.
// Orbits then come in mirror pairs (kept: the one whose smallest rank is below its
// mirror's) or are their own mirror (kept, weight 1/2 in the gradient sums).  Entries
// hold the rank of the stored (canonical) amplitude (min(a,b), max(a,b)); bit 31 of
// an entry's bitstring marks the member of a self-mirror orbit that must not write
// (its mirror, also in the orbit, writes the same canonical amplitude).  Warp tasks
// of self-mirror orbits carry bit 31 in their group field.  mslot: slot -> slot of
// its mirror operator.
struct HalfTables {
    std::vector<uint32_t> idx, bits;
    std::vector<WarpTask> wtasks;
    uint64_t active = 0, amp_layers = 0;
    bool ok = true;   // false: a sign or rank check failed (no half passes)
};
constexpr uint32_t kNoWriteBit = 1u << 31;
constexpr uint32_t kSelfMirrorTask = 1u << 31;
HalfTables build_half_orbits(const Basis &B, const OrbitTables &T, const std::vector<ExcCode> &codes,
                             const std::vector<int> &mslot, int nthreads);

}  // namespace ae
