// GB300 statevector engine: the CUDA side of the aegpu C ABI (include/aegpu.h).
//
// Data layout in HBM (one problem per engine, nb instances of it per evaluation):
//   psi, hpsi          FP64[nb][D*W]  W = 1 (real) or 2 (complex, re/im interleaved)
//   checkpoints        per pass, the amplitudes after it in orbit order, per instance
//   basis tables       Sz sector: alpha/beta strings + 2^N rank tables (a few KB);
//                      other sectors: D bitstrings + 2^nq rank table
//   orbit tables       per pass: uint32 ranks and bitstrings of every touched
//                      determinant, grouped into orbits (hypercubes of the active
//                      excitations), plus group/tile/warp-task descriptors (setup.cpp)
//   Hamiltonian        CSR (general), coded sliced rows built from integrals (the
//                      doubles as 2-byte codes into a value table; uncoded sliced rows
//                      above 12 orbitals), or the string tables of the on-the-fly
//                      product (one set per instance for a Hamiltonian family)
//   Hessian scratch    per-operator tangents FP64[nops][D*W], compressed tangents
//                      and H*tangents column-major [P+1][D*W]
//
// Kernels (all FP64; bandwidth- or FP64-pipe-bound, no tensor cores):
//   k_warp_rot       a pass of <= 6 commuting excitations with the orbits in warp
//                    registers (shuffles, one FMA per amplitude per layer; reference
//                    RunFuseN, fusedevolve.cpp:917-1774); writes the pass's output
//                    amplitudes as the adjoint sweep's checkpoint; the instance
//                    dimension also carries the Hessian's tangents through a pass
//   k_warp_adj       checkpointed adjoint pass: gradient of every excitation from the
//                    checkpoint and H psi, then H psi rotated back (fusedevolve.cpp:461-485)
//   k_block_tangent  forward block + tangents T_op = G_op psi, a CTA staging whole
//                    orbits (<= 4096 amplitudes) in shared memory (fusedevolve.cpp:492-518)
//   k_warp_hess      second-derivative sweep of the Hessian: every tangent against the
//                    back-propagated H psi through a pass (fusedevolve.cpp:2670-2761)
//   k_diag_*         the same four for diagonal (number / density-density) blocks,
//                    complex mode (fusedevolve.cpp:625-717)
//   k_pass_prep      per evaluation: sin/cos and the scaled-Givens constants of every
//                    pass and direction, the scale products of every active mask, and
//                    the phase table of every diagonal pass
//   k_spmv           warp-per-row CSR y = H x fused with the <x|y> partial sums
//   k_spmv_vell      y = H x over coded rows (value table in shared memory, 1-8
//                    threads per row, equal row shares per CTA) fused with <x|y>; with
//                    several right-hand sides per thread for the Hessian's tangents
//   k_spmv_sell      the same over uncoded sliced rows
//   k_vtab_build, k_vell_build, k_ell_build
//                    value table and rows of H generated from h_pq/(pq|rs): diagonal,
//                    alpha/beta singles, alpha-alpha/beta-beta/alpha-beta doubles
//   k_otf_strings    y = H x with no stored matrix: CTA per alpha string, thread per
//                    determinant, one FP64 FMA per matrix element (otf_tables.cpp)
//   k_lanczos_update the three-term step of the Lanczos recurrence (alpha and beta stay
//                    in device memory; the dot products, norms and the basis products
//                    of the reorthogonalisation are the kernels of dense.cu)
// All reductions are two-stage and in a fixed order, so results are bit-identical
// from run to run.
#include "../../include/aegpu.h"
#include "exc_rule.h"
#include "newton.h"
#include "otf_tables.h"
#include "setup.h"
#include "dense.h"

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <vector>

using namespace ae;

namespace {
// Host-side fault injection for tests: after this many further engine allocations,
// every allocation fails as if the device were out of memory (-1: off).
std::atomic<int64_t> g_fail_alloc_after{-1};

// NVTX range over a host-side phase (visible in Nsight timelines; no cost without a tool)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};
}  // namespace

namespace {

constexpr int kMaxSlots = 12;          // excitations per fused block (the reference's maxFuse)
static_assert(kMaxDiagSlots <= kMaxSlots, "a diagonal pass's phase table and partial sums hold kMaxSlots slots");
constexpr int kRotThreads = 256;
constexpr int kSpmvThreads = 256;
constexpr int kDiagGrid = 152 * 4;

struct DevBasis {
    int kind, N, nq;
    uint32_t nA, nB;
    uint32_t div_m, div_l;  // z / nB = (hi + ((z - hi) >> 1)) >> (l - 1), hi = umulhi(m, z)
    uint64_t D;
    const uint32_t *strA, *strB;
    const int32_t *rankA, *rankB;
    const uint32_t *states;
    const int32_t *rank;

    __device__ __forceinline__ uint32_t div_nB(uint32_t z) const
    {
        if (div_l == 0) return z;
        const uint32_t hi = __umulhi(div_m, z);
        return (hi + ((z - hi) >> 1)) >> (div_l - 1);
    }
    __device__ __forceinline__ uint32_t bits(uint32_t z) const
    {
        if (kind == BASIS_SZ) {
            const uint32_t a = div_nB(z);
            return (strA[a] << N) | strB[z - a * nB];
        }
        return states[z];
    }
    __device__ __forceinline__ int64_t rank_of(uint32_t s) const
    {
        if (kind == BASIS_SZ) {
            int32_t a = rankA[s >> N], b = rankB[s & ((1u << N) - 1u)];
            return (a < 0 || b < 0) ? -1 : (int64_t)a * nB + b;
        }
        return rank[s];
    }
};

struct PassConst {
    ExcCode code;
    double f;      // layer scale (C or dir*S)
    double m;      // S/C (tan form) or C/S (cot form), with dir applied to S
    int tan_form;
    int pad;
};

struct BlockArgs {
    const uint32_t *idx;
    const uint32_t *obits;   // bitstrings parallel to idx (warp kernels)
    const OrbitGroup *groups;
    const OrbitTile *tiles;
    const int *ops;          // slot -> operator
    int nslots;
    const ExcCode *codes;    // per operator
    const double *sc;        // per operator: sin, cos
    double dir;              // +1 forward, -1 backward
    DevBasis basis;
    const PassConst *pc;     // this pass's layer constants for this direction (instance 0)
    const double *sigma;     // this pass's scale products per active mask (instance 0)
    int64_t pc_stride, sig_stride;  // per-instance strides of pc / sigma
    const int *active;       // instance mask of the warp kernels (nullable)
    // spin-flip half passes (warp kernels): where half[b] is set, instance b runs the
    // pass's half tables (canonical ranks, no-write bits, self-mirror tasks) instead
    const int *half;         // per instance (nullable: full tables)
    const uint32_t *idx_h, *obits_h;
    const WarpTask *tasks_h;
    int ntasks_h;
    // the Hessian's tangent kernels: grid row v works on vector vmap[v] (nullable: v)
    const int *vmap;
    int task_order;          // warp kernels' first task: 0 CTA-major, 1 warp-major (task_first)
};

// First task of this warp in the warp kernels' grid-stride loop (stride: the grid's
// warps).  CTA-major hands a CTA consecutive tasks; warp-major hands warp w of CTA c
// task w * gridDim.x + c, so that, in a launch whose CTAs are all resident at once, the
// tasks left over once every warp has one spread over every CTA (and so every SM)
// instead of filling the first CTAs.  Both orders visit each task once.
__device__ __forceinline__ int task_first(const BlockArgs &a)
{
    return a.task_order ? (int)((threadIdx.x >> 5) * gridDim.x + blockIdx.x)
                        : (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
}

// The tables instance b runs: the half tables where its half flag is set.
struct PassTables {
    const uint32_t *idx, *obits;
    const WarpTask *tasks;
    int ntasks;
    bool half;
};
__device__ __forceinline__ PassTables pass_tables(const BlockArgs &a, const WarpTask *tasks, int ntasks, int b)
{
    if (a.half && a.half[b]) return PassTables{a.idx_h, a.obits_h, a.tasks_h, a.ntasks_h, true};
    return PassTables{a.idx, a.obits, tasks, ntasks, false};
}

__device__ __forceinline__ uint32_t insert_zero_bit(uint32_t p, int i)
{
    return ((p >> i) << (i + 1)) | (p & ((1u << i) - 1u));
}

// Stored Hamiltonian rows ("sliced ELL"): rows are grouped in slabs of 32; inside a
// slab, entry group g (4 consecutive entries of a row) of the 32 rows is contiguous,
// so thread r of a warp reads its row with 16-byte column loads and 32-byte value
// loads that coalesce across the warp.  q = entries per row / 4.
__device__ __forceinline__ size_t ell_pos(int64_t r, int64_t e, int64_t q)
{
    return ((((size_t)(r >> 5) * q + (size_t)(e >> 2)) << 5) + (size_t)(r & 31)) * 4 + (size_t)(e & 3);
}

// ---------------------------------------------------------------- utilities --
// Instance b of a batched launch is skipped when the engine's mask says so (the mask
// pointer is null for launches that are not per instance, e.g. the Hessian's columns).
__device__ __forceinline__ bool skip_instance(const int *active, int b) { return active && !active[b]; }

// dst[b * n + i] = src[i] for every instance b = blockIdx.y (the shared start vector)
__global__ void k_broadcast(const double *__restrict__ src, double *__restrict__ dst, int64_t n,
                            const int *__restrict__ active)
{
    if (skip_instance(active, blockIdx.y)) return;
    dst += (size_t)blockIdx.y * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-order block sum; result valid in thread 0.  red needs blockDim/32 doubles.
__device__ __forceinline__ double block_sum(double v, double *red)
{
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    return s;
}

// One CTA per instance: out[b] = scale * sum of parts[b * n .. b * n + n).
__global__ void k_reduce_sum(const double *__restrict__ parts, int n, double *__restrict__ out, double scale,
                             const int *__restrict__ active)
{
    __shared__ double red[32];
    if (skip_instance(active, blockIdx.x)) return;
    parts += (size_t)blockIdx.x * n;
    double s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += parts[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) out[blockIdx.x] = s * scale;
}

// Per-CTA partial sums of <a|b> over instance blockIdx.y (vectors at stride n):
// parts[blockIdx.y * gridDim.x + blockIdx.x].
__global__ void k_dot(const double *__restrict__ a, const double *__restrict__ b, int64_t n, double *__restrict__ parts,
                      const int *__restrict__ active)
{
    __shared__ double red[32];
    if (skip_instance(active, blockIdx.y)) return;
    a += (size_t)blockIdx.y * n;
    b += (size_t)blockIdx.y * n;
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(a[i], b[i], s);
    s = block_sum(s, red);
    if (threadIdx.x == 0) parts[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
}

// -------------------------------------------------------- block rotations --
// Stage the tile's ranks' bitstrings and load the layer constants.
struct TileCtx {
    uint32_t n;       // amplitudes in the tile
    int k;            // layers
    const uint32_t *idx;
};

__device__ __forceinline__ TileCtx load_tile(const BlockArgs &a, uint32_t *bits, ExcCode *code, double *C,
                                             double *S, int *slot)
{
    const OrbitTile t = a.tiles[blockIdx.x];
    const OrbitGroup &g = a.groups[t.group];
    TileCtx c;
    c.k = (int)g.k;
    c.n = t.n_orbits << g.k;
    c.idx = a.idx + t.elem_off;
    if (threadIdx.x < (unsigned)c.k) {
        int s = g.slot[threadIdx.x];
        int op = a.ops[s];
        slot[threadIdx.x] = s;
        code[threadIdx.x] = a.codes[op];
        S[threadIdx.x] = a.dir * a.sc[2 * op];
        C[threadIdx.x] = a.sc[2 * op + 1];
    }
    for (uint32_t e = threadIdx.x; e < c.n; e += blockDim.x) bits[e] = a.basis.bits(c.idx[e]);
    __syncthreads();
    return c;
}

template <int W>
__device__ __forceinline__ void gather(double *v, const double *__restrict__ src, const TileCtx &c)
{
    for (uint32_t e = threadIdx.x; e < c.n; e += blockDim.x) {
        const size_t z = c.idx[e];
#pragma unroll
        for (int w = 0; w < W; ++w) v[e * W + w] = src[z * W + w];
    }
}

template <int W>
__device__ __forceinline__ void scatter(const double *v, double *__restrict__ dst, const TileCtx &c)
{
    for (uint32_t e = threadIdx.x; e < c.n; e += blockDim.x) {
        const size_t z = c.idx[e];
#pragma unroll
        for (int w = 0; w < W; ++w) dst[z * W + w] = v[e * W + w];
    }
}

// One butterfly layer: x' = C x + s S y, y' = C y - s S x (fusedevolve.cpp:461-468).
template <int W>
__device__ __forceinline__ void layer(double *v, const uint32_t *bits, const TileCtx &c, int i, const ExcCode &code,
                                      double Ci, double Si)
{
    const uint32_t half = c.n >> 1;
    for (uint32_t p = threadIdx.x; p < half; p += blockDim.x) {
        const uint32_t lo = insert_zero_bit(p, i), hi = lo | (1u << i);
        const double sS = exc_sign(code, bits[lo]) * Si;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const double x = v[lo * W + w], y = v[hi * W + w];
            v[lo * W + w] = fma(sS, y, Ci * x);
            v[hi * W + w] = fma(-sS, x, Ci * y);
        }
    }
}


// Forward block that also writes the tangents T_slot = G_slot psi (after the block,
// which equals G psi before it because the block's excitations commute).
template <int W>
__global__ void __launch_bounds__(kRotThreads) k_block_tangent(BlockArgs a, double *psi, double *T, size_t tstride,
                                                               const int *tpos)
{
    extern __shared__ double sm[];
    double *v = sm;
    uint32_t *bits = (uint32_t *)(sm + kTileElems * W);
    __shared__ ExcCode code[kMaxSlots];
    __shared__ double C[kMaxSlots], S[kMaxSlots];
    __shared__ int slot[kMaxSlots];
    const TileCtx c = load_tile(a, bits, code, C, S, slot);
    gather<W>(v, psi, c);
    __syncthreads();
    for (int i = 0; i < c.k; ++i) {
        layer<W>(v, bits, c, i, code[i], C[i], S[i]);
        __syncthreads();
    }
    scatter<W>(v, psi, c);
    for (int i = 0; i < c.k; ++i) {
        double *Ti = T + (size_t)tpos[a.ops[slot[i]]] * tstride;
        for (uint32_t e = threadIdx.x; e < c.n; e += blockDim.x) {
            const uint32_t pe = e ^ (1u << i);
            const double s = exc_sign(code[i], bits[e]);
            const size_t z = c.idx[e];
#pragma unroll
            for (int w = 0; w < W; ++w) Ti[z * W + w] = s * v[pe * W + w];
        }
    }
}


// ------------------------------------------------ warp-register passes --
// A pass holds <= 6 commuting excitations, so every orbit has <= 64 members and a
// warp keeps a whole task (one or more orbits) in registers: two amplitudes per
// lane, positions p = lane and lane + 32.  Layer i pairs p with p ^ (1 << i): a
// shuffle for i < 5, the lane's other register for i = 5.  No shared-memory
// staging and no block barriers.  Each layer is applied in a scaled ("fast
// Givens") form with one FP64 FMA per amplitude:
//   |C| >= |S|:  v'' = v + (S/C) s v_p,   true value = C v''
//   |C| <  |S|:  v'' = (C/S) v + s v_p,   true value = S v''
// and the product of the per-layer scales is applied once when the task is
// written back.  The adjoint sweep accumulates <h|G_j psi> = sum_z h_z s_z psi_p(z)
// in the scaled frame (stored = true / product of the scales applied so far) and
// multiplies it by the squared product of those scales.  (Per-element form of
// fusedevolve.cpp:461-483.)
constexpr int kWarpThreads = 256;

__device__ __forceinline__ double flip(double x, int s)
{
    return __longlong_as_double(__double_as_longlong(x) ^ ((unsigned long long)(s < 0) << 63));
}

// The warp sums of six per-lane values at once, by recursive halving: at each step a
// lane keeps half of its values and adds its partner's copies of them, so the six sums
// take 9 double shuffles instead of 6 x 5.  Lane l with (l & 3) == 0 returns the sum of
// value l >> 2 (l >> 2 = 6, 7: padding).  The order of the additions is fixed.
static_assert(kMaxWarpLayers == 6, "warp_sum6 reduces six values");
__device__ __forceinline__ double warp_sum6(const double (&x)[kMaxWarpLayers], int lane)
{
    double v8[8];
#pragma unroll
    for (int i = 0; i < 6; ++i) v8[i] = x[i];
    v8[6] = v8[7] = 0.0;
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
    double v4[4], v2[2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        v4[i] = (b4 ? v8[i + 4] : v8[i]) + __shfl_xor_sync(0xffffffffu, b4 ? v8[i] : v8[i + 4], 16);
#pragma unroll
    for (int i = 0; i < 2; ++i)
        v2[i] = (b3 ? v4[i + 2] : v4[i]) + __shfl_xor_sync(0xffffffffu, b3 ? v4[i] : v4[i + 2], 8);
    double v = (b2 ? v2[1] : v2[0]) + __shfl_xor_sync(0xffffffffu, b2 ? v2[0] : v2[1], 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v;
}

// One DFMA whatever the form: the operands are chosen with integer selects, so the
// compiler cannot evaluate both forms on the FP64 pipe.
__device__ __forceinline__ double rot_scaled(const PassConst &q, double v, double vp, int s)
{
    const double a = q.tan_form ? flip(q.m, s) : q.m;
    const double b = q.tan_form ? vp : v;
    const double c = q.tan_form ? v : flip(vp, s);
    return fma(a, b, c);
}

// Per-evaluation preparation, one CTA per (pass, instance): sin / cos of the pass's
// angles (kept for the Hessian and diagonal kernels), the scaled-Givens constants of
// every layer for both directions, and for every active mask the product of its
// layer scales.  The pass kernels then only read these (no FP64 division, no
// per-CTA set-up barrier on the hot path).
struct PrepArgs {
    const int *pass_ops;    // operators of all passes, concatenated
    const int *pass_off;    // first operator of each pass
    const int *pass_n;      // operators per pass
    const int *pass_diag;   // 1 for diagonal passes (no scaled-Givens constants)
    const int64_t *pass_tab; // diagonal passes: offset of the pass's phase table
    int64_t tab_stride;     // phase-table doubles per instance
    const ExcCode *codes;
    int nops, npass;
    const int *active;      // instance mask (nullable)
    // spin-flip half passes (nullable: none): operator -> mirror operator, the gate
    // (one int: tables built, symmetric start state, knob on) and the per-instance flag
    const int *mirror;
    const int *half_gate;
    int *half;
};

// A diagonal pass's phase table: tab[2m], tab[2m + 1] = cos, sin of the sum of the
// angles of the slots in m (the adjoint direction negates the sine where it reads it).
__device__ void diag_phase_table(const int *ops, int ns, const double *__restrict__ ang, double *__restrict__ tab)
{
    for (int m = threadIdx.x; m < (1 << ns); m += blockDim.x) {
        double th = 0;
        for (int i = 0; i < ns; ++i)
            if (m & (1 << i)) th += ang[ops[i]];
        double s, c;
        sincos(th, &s, &c);
        tab[2 * m] = c;
        tab[2 * m + 1] = s;
    }
}

__global__ void k_pass_prep(PrepArgs a, const double *__restrict__ ang, double *__restrict__ sc,
                            PassConst *__restrict__ pc, double *__restrict__ sig, double *__restrict__ tab)
{
    const int pass = blockIdx.x, b = blockIdx.y;
    if (skip_instance(a.active, b)) return;
    if (pass == 0 && a.half) {
        // instance b takes the half passes when the gate is open and every operator's
        // angle equals its mirror's (the evolution then commutes with the exchange of
        // the alpha and beta strings)
        __shared__ int ok;
        if (threadIdx.x == 0) ok = *a.half_gate;
        __syncthreads();
        const double *ab = ang + (size_t)b * a.nops;
        for (int o = threadIdx.x; o < a.nops; o += blockDim.x)
            if (ab[o] != ab[a.mirror[o]]) ok = 0;  // every writer stores 0
        __syncthreads();
        if (threadIdx.x == 0) a.half[b] = ok;
    }
    const int ns = a.pass_n[pass];
    const int *ops = a.pass_ops + a.pass_off[pass];
    if (a.pass_diag[pass])
        diag_phase_table(ops, ns, ang + (size_t)b * a.nops, tab + (size_t)b * a.tab_stride + a.pass_tab[pass]);
    __shared__ double f[2][kMaxWarpLayers];
    const bool paired = !a.pass_diag[pass] && ns <= kMaxWarpLayers;
    if (threadIdx.x < (unsigned)ns) {
        const int op = ops[threadIdx.x];
        double S0, C;
        sincos(ang[(size_t)b * a.nops + op], &S0, &C);
        sc[(size_t)b * 2 * a.nops + 2 * op] = S0;
        sc[(size_t)b * 2 * a.nops + 2 * op + 1] = C;
        if (paired)
            for (int d = 0; d < 2; ++d) {
                const double S = d == 0 ? S0 : -S0;
                PassConst q;
                q.code = a.codes[op];
                q.pad = 0;
                if (fabs(C) >= fabs(S)) {
                    q.tan_form = 1;
                    q.f = C;
                    q.m = S / C;
                } else {
                    q.tan_form = 0;
                    q.f = S;
                    q.m = C / S;
                }
                f[d][threadIdx.x] = q.f;
                pc[(((size_t)b * a.npass + pass) * 2 + d) * kMaxWarpLayers + threadIdx.x] = q;
            }
    }
    __syncthreads();
    if (!paired) return;
    for (int m = threadIdx.x; m < (1 << ns); m += blockDim.x)
        for (int d = 0; d < 2; ++d) {
            double prod = 1.0;
            for (int j = 0; j < ns; ++j)
                if (m & (1 << j)) prod *= f[d][j];
            sig[(((size_t)b * a.npass + pass) * 2 + d) * (1 << kMaxWarpLayers) + m] = prod;
        }
}

// Instance b = blockIdx.y.  ckpt (nullable): the pass's amplitudes after rotation,
// stored in the pass's orbit order (same index as the rank list), for the adjoint.
// Programmatic dependent launch: a pass kernel launched with the programmatic-
// serialisation attribute may start while the previous kernel drains.  Before the
// wait it touches only set-up data (task lists and orbit rank / bitstring tables,
// written before any evaluation); after it, everything the previous kernels wrote is
// visible.  It then lets its own successor start, which in turn can only pass its
// wait once this grid has completed.  Without the attribute both are no-ops.
__device__ __forceinline__ void pdl_prologue(const BlockArgs &a, const WarpTask *__restrict__ tasks, int ntasks)
{
    const int t = task_first(a), lane = threadIdx.x & 31;
    if (t < ntasks) {
        const WarpTask task = tasks[t];
        if (2 * lane < (int)task.n) {  // inside this task's entries
            asm volatile("prefetch.global.L2 [%0];" ::"l"(a.idx + task.elem_off + 2 * lane));
            asm volatile("prefetch.global.L2 [%0];" ::"l"(a.obits + task.elem_off + 2 * lane));
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <int W>
__global__ void __launch_bounds__(kWarpThreads) k_warp_rot(BlockArgs a, const WarpTask *__restrict__ tasks, int ntasks,
                                                           double *vecs, int64_t inst_stride, double *__restrict__ ckpt,
                                                           int64_t ckpt_stride)
{
    pdl_prologue(a, tasks, ntasks);
    const int lane = threadIdx.x & 31, b = blockIdx.y;
    if (skip_instance(a.active, b)) return;
    const PassConst *pc = a.pc + (size_t)b * a.pc_stride;
    const double *sig = a.sigma + (size_t)b * a.sig_stride;
    double *psi = vecs + (size_t)(a.vmap ? a.vmap[b] : b) * inst_stride;
    if (ckpt) ckpt += (size_t)b * ckpt_stride;
    const PassTables pt = pass_tables(a, tasks, ntasks, b);
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int t = task_first(a); t < pt.ntasks; t += nw) {
        const WarpTask task = pt.tasks[t];
        const uint32_t mask = task.mask;
        const uint32_t *idx = pt.idx + task.elem_off, *obits = pt.obits + task.elem_off;
        const bool ok0 = lane < (int)task.n, ok1 = lane + 32 < (int)task.n;
        const uint32_t z0 = ok0 ? idx[lane] : 0u, z1 = ok1 ? idx[lane + 32] : 0u;
        const uint32_t b0 = ok0 ? obits[lane] : 0u, b1 = ok1 ? obits[lane + 32] : 0u;
        // half tables: the mirror member of a self-mirror orbit writes this amplitude
        const bool w0 = ok0 && !(b0 & kNoWriteBit), w1 = ok1 && !(b1 & kNoWriteBit);
        double v0[W], v1[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            v0[w] = ok0 ? psi[(size_t)z0 * W + w] : 0.0;
            v1[w] = ok1 ? psi[(size_t)z1 * W + w] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < kMaxWarpLayers; ++j) {
            if (!(mask & (1u << j))) continue;
            const int i = __popc(mask & ((1u << j) - 1u));
            const PassConst q = pc[j];
            const int s0 = exc_sign(q.code, b0), s1 = exc_sign(q.code, b1);
#pragma unroll
            for (int w = 0; w < W; ++w) {
                double p0, p1;
                if (i < 5) {
                    p0 = __shfl_xor_sync(0xffffffffu, v0[w], 1 << i);
                    p1 = __shfl_xor_sync(0xffffffffu, v1[w], 1 << i);
                } else {
                    p0 = v1[w];
                    p1 = v0[w];
                }
                v0[w] = rot_scaled(q, v0[w], p0, s0);
                v1[w] = rot_scaled(q, v1[w], p1, s1);
            }
        }
        const double sigma = sig[mask];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const double t0 = sigma * v0[w], t1 = sigma * v1[w];
            if (w0) psi[(size_t)z0 * W + w] = t0;
            if (w1) psi[(size_t)z1 * W + w] = t1;
            if (ckpt) {
                if (ok0) ckpt[((size_t)task.elem_off + lane) * W + w] = t0;
                if (ok1) ckpt[((size_t)task.elem_off + lane + 32) * W + w] = t1;
            }
        }
    }
}

// Checkpointed adjoint pass (instance b = blockIdx.y).  psi after this pass comes
// from the forward sweep's checkpoint (orbit order, coalesced), h = H psi
// back-propagated to the same point is gathered; since the pass's excitations
// commute, the gradient of excitation j is <h|G_j psi> evaluated right there:
// sum_z h_z s_j(z) psi_p(z), one FP64 FMA per amplitude and layer.  Only h is then
// rotated back (-theta) through the pass, one FMA per amplitude and layer.
template <int W>
__global__ void __launch_bounds__(kWarpThreads) k_warp_adj(BlockArgs a, const WarpTask *__restrict__ tasks, int ntasks,
                                                           const double *__restrict__ ckpt, int64_t ckpt_stride,
                                                           double *hv, int64_t inst_stride, double *partials,
                                                           int64_t part_stride)
{
    __shared__ double red[kMaxWarpLayers][kWarpThreads / 32];
    pdl_prologue(a, tasks, ntasks);
    const int lane = threadIdx.x & 31, b = blockIdx.y;
    if (skip_instance(a.active, b)) return;
    const PassConst *pc = a.pc + (size_t)b * a.pc_stride;
    const double *sig = a.sigma + (size_t)b * a.sig_stride;
    double *h = hv + (size_t)b * inst_stride;
    ckpt += (size_t)b * ckpt_stride;
    const PassTables pt = pass_tables(a, tasks, ntasks, b);
    const int nw = (gridDim.x * blockDim.x) >> 5;
    double accS[kMaxWarpLayers];
#pragma unroll
    for (int j = 0; j < kMaxWarpLayers; ++j) accS[j] = 0.0;
    for (int t = task_first(a); t < pt.ntasks; t += nw) {
        const WarpTask task = pt.tasks[t];
        const uint32_t mask = task.mask;
        const uint32_t *idx = pt.idx + task.elem_off, *obits = pt.obits + task.elem_off;
        const bool ok0 = lane < (int)task.n, ok1 = lane + 32 < (int)task.n;
        const uint32_t z0 = ok0 ? idx[lane] : 0u, z1 = ok1 ? idx[lane + 32] : 0u;
        const uint32_t b0 = ok0 ? obits[lane] : 0u, b1 = ok1 ? obits[lane + 32] : 0u;
        const bool w0 = ok0 && !(b0 & kNoWriteBit), w1 = ok1 && !(b1 & kNoWriteBit);
        // a self-mirror orbit of the half tables is its own mirror: half weight, so that
        // the operator's sum plus its mirror's counts it once
        const double wt = (task.group & kSelfMirrorTask) ? 0.5 : 1.0;
        const double *cp = ckpt + (size_t)task.elem_off * W;
        double v0[W], v1[W], h0[W], h1[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            v0[w] = ok0 ? cp[lane * W + w] : 0.0;
            v1[w] = ok1 ? cp[(lane + 32) * W + w] : 0.0;
            h0[w] = ok0 ? h[(size_t)z0 * W + w] : 0.0;
            h1[w] = ok1 ? h[(size_t)z1 * W + w] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < kMaxWarpLayers; ++j) {
            if (!(mask & (1u << j))) continue;
            const int i = __popc(mask & ((1u << j) - 1u));
            const PassConst q = pc[j];
            const int s0 = exc_sign(q.code, b0), s1 = exc_sign(q.code, b1);
            double g = 0.0;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                double p0, p1;
                if (i < 5) {
                    p0 = __shfl_xor_sync(0xffffffffu, v0[w], 1 << i);
                    p1 = __shfl_xor_sync(0xffffffffu, v1[w], 1 << i);
                } else {
                    p0 = v1[w];
                    p1 = v0[w];
                }
                g = fma(h0[w], flip(p0, s0), g);
                g = fma(h1[w], flip(p1, s1), g);
            }
            accS[j] = fma(wt, g, accS[j]);
        }
#pragma unroll
        for (int j = 0; j < kMaxWarpLayers; ++j) {
            if (!(mask & (1u << j))) continue;
            const int i = __popc(mask & ((1u << j) - 1u));
            const PassConst q = pc[j];
            const int s0 = exc_sign(q.code, b0), s1 = exc_sign(q.code, b1);
#pragma unroll
            for (int w = 0; w < W; ++w) {
                double p0, p1;
                if (i < 5) {
                    p0 = __shfl_xor_sync(0xffffffffu, h0[w], 1 << i);
                    p1 = __shfl_xor_sync(0xffffffffu, h1[w], 1 << i);
                } else {
                    p0 = h1[w];
                    p1 = h0[w];
                }
                h0[w] = rot_scaled(q, h0[w], p0, s0);
                h1[w] = rot_scaled(q, h1[w], p1, s1);
            }
        }
        const double sigma = sig[mask];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            if (w0) h[(size_t)z0 * W + w] = sigma * h0[w];
            if (w1) h[(size_t)z1 * W + w] = sigma * h1[w];
        }
    }
    // fixed-order CTA sum: the warp's six sums by recursive halving, then the warps in order
    const int warp = threadIdx.x >> 5;
    const double wsum = warp_sum6(accS, lane);
    if ((lane & 3) == 0 && (lane >> 2) < kMaxWarpLayers) red[lane >> 2][warp] = wsum;
    __syncthreads();
    if (threadIdx.x < kMaxSlots) {
        double sum = 0.0;
        if (threadIdx.x < kMaxWarpLayers)
            for (int w = 0; w < kWarpThreads / 32; ++w) sum += red[threadIdx.x][w];
        partials[(size_t)b * part_stride + (size_t)blockIdx.x * kMaxSlots + threadIdx.x] = sum;
    }
}

// Second-derivative sweep of the Hessian through one pass (evolveHessian,
// fusedevolve.cpp:2670-2761), vector v = blockIdx.y of the tangents T: with the bra h
// (H psi back-propagated to this pass's output, read only) every excitation j of the
// pass at application position >= v contributes <h|G_j T_v>, taken at the pass output
// (the pass's excitations commute), then T_v is rotated back through the pass.
// partials[(blockIdx.x * nvec + v) * kMaxSlots + slot] (fixed-order CTA sums).
template <int W>
__global__ void __launch_bounds__(kWarpThreads) k_warp_hess(BlockArgs a, const WarpTask *__restrict__ tasks, int ntasks,
                                                            const double *__restrict__ h, double *T, int64_t tstride,
                                                            int nvec, int block_pos0, double *__restrict__ partials)
{
    __shared__ double red[kMaxWarpLayers][kWarpThreads / 32];
    const int lane = threadIdx.x & 31, vec = blockIdx.y;
    const int vpos = a.vmap ? a.vmap[vec] : vec;  // the tangent's application position
    const PassConst *pc = a.pc;
    const double *sig = a.sigma;
    double *t = T + (size_t)vpos * tstride;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    double accS[kMaxWarpLayers];
#pragma unroll
    for (int j = 0; j < kMaxWarpLayers; ++j) accS[j] = 0.0;
    for (int k = task_first(a); k < ntasks; k += nw) {
        const WarpTask task = tasks[k];
        const uint32_t mask = task.mask;
        const uint32_t *idx = a.idx + task.elem_off, *obits = a.obits + task.elem_off;
        const bool ok0 = lane < (int)task.n, ok1 = lane + 32 < (int)task.n;
        const uint32_t z0 = ok0 ? idx[lane] : 0u, z1 = ok1 ? idx[lane + 32] : 0u;
        const uint32_t b0 = ok0 ? obits[lane] : 0u, b1 = ok1 ? obits[lane + 32] : 0u;
        double v0[W], v1[W], h0[W], h1[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            v0[w] = ok0 ? t[(size_t)z0 * W + w] : 0.0;
            v1[w] = ok1 ? t[(size_t)z1 * W + w] : 0.0;
            h0[w] = ok0 ? h[(size_t)z0 * W + w] : 0.0;
            h1[w] = ok1 ? h[(size_t)z1 * W + w] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < kMaxWarpLayers; ++j) {
            if (!(mask & (1u << j)) || block_pos0 + j < vpos) continue;
            const int i = __popc(mask & ((1u << j) - 1u));
            const PassConst q = pc[j];
            const int s0 = exc_sign(q.code, b0), s1 = exc_sign(q.code, b1);
            double g = 0.0;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                double p0, p1;
                if (i < 5) {
                    p0 = __shfl_xor_sync(0xffffffffu, v0[w], 1 << i);
                    p1 = __shfl_xor_sync(0xffffffffu, v1[w], 1 << i);
                } else {
                    p0 = v1[w];
                    p1 = v0[w];
                }
                g = fma(h0[w], flip(p0, s0), g);
                g = fma(h1[w], flip(p1, s1), g);
            }
            accS[j] += g;
        }
#pragma unroll
        for (int j = 0; j < kMaxWarpLayers; ++j) {
            if (!(mask & (1u << j))) continue;
            const int i = __popc(mask & ((1u << j) - 1u));
            const PassConst q = pc[j];
            const int s0 = exc_sign(q.code, b0), s1 = exc_sign(q.code, b1);
#pragma unroll
            for (int w = 0; w < W; ++w) {
                double p0, p1;
                if (i < 5) {
                    p0 = __shfl_xor_sync(0xffffffffu, v0[w], 1 << i);
                    p1 = __shfl_xor_sync(0xffffffffu, v1[w], 1 << i);
                } else {
                    p0 = v1[w];
                    p1 = v0[w];
                }
                v0[w] = rot_scaled(q, v0[w], p0, s0);
                v1[w] = rot_scaled(q, v1[w], p1, s1);
            }
        }
        const double sigma = sig[mask];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            if (ok0) t[(size_t)z0 * W + w] = sigma * v0[w];
            if (ok1) t[(size_t)z1 * W + w] = sigma * v1[w];
        }
    }
    const int warp = threadIdx.x >> 5;
    const double wsum = warp_sum6(accS, lane);
    if ((lane & 3) == 0 && (lane >> 2) < kMaxWarpLayers) red[lane >> 2][warp] = wsum;
    __syncthreads();
    if (threadIdx.x < kMaxSlots) {
        double sum = 0.0;
        if (threadIdx.x < kMaxWarpLayers)
            for (int w = 0; w < kWarpThreads / 32; ++w) sum += red[threadIdx.x][w];
        partials[((size_t)blockIdx.x * nvec + vec) * kMaxSlots + threadIdx.x] = sum;
    }
}

// ------------------------------------------------------- diagonal blocks --
// Complex mode only: number / density-density operators multiply every active
// amplitude by exp(+i * sum of the active angles) (RunFuseNDiagonal,
// fusedevolve.cpp:625-717), exp(-i * ...) in the adjoint direction.  The pass's table
// (k_pass_prep) holds (cos, sin) of the angle sum of every slot subset m.
struct DiagArgs {
    const int *ops;
    int nslots;
    const ExcCode *codes;
    const double *table;  // this pass's phase table, instance 0; instance b at + b * tab_stride
    int64_t tab_stride;
    uint64_t sin_flip;    // 0 forward; sign bit (adjoint direction: the conjugate phase)
    // Sz basis: slot mask of determinant (a, b) = smA[a] & smB[b] (the slots whose
    // alpha / beta annihilation bits the string holds); null: from the bitstring
    const uint16_t *smA, *smB;
    DevBasis basis;
    const int *active;    // instance mask (nullable)
    // spin-flip half passes (nullable): where half[b] is set, instance b keeps only the
    // amplitudes (a, b) with a <= b current (the others are skipped), and the adjoint
    // counts a = b at half weight (the gradient adds the mirror operator's sum)
    const int *half;
};

__device__ __forceinline__ uint32_t diag_mask(const DiagArgs &a, uint32_t bits)
{
    uint32_t m = 0;
    for (int i = 0; i < a.nslots; ++i) {
        const uint32_t ann = a.codes[a.ops[i]].annihilate;
        if ((bits & ann) == ann) m |= 1u << i;
    }
    return m;
}

// (cos, sin) of the phase of slot subset m in this pass's direction
__device__ __forceinline__ double2 diag_phase(const DiagArgs &a, uint32_t m)
{
    const double2 t = __ldg(reinterpret_cast<const double2 *>(a.table) + m);
    return make_double2(t.x, __longlong_as_double(__double_as_longlong(t.y) ^ a.sin_flip));
}

// The streaming diagonal kernels take kDiagUnroll amplitudes z, z + S, ... (S = grid
// threads) per iteration: their masks first, then all their loads, then the arithmetic,
// so that each thread keeps several HBM loads in flight (one amplitude per iteration left
// the kernels latency-bound).  A thread still visits its amplitudes in ascending order,
// so every per-thread sum keeps its order.
constexpr int kDiagUnroll = 4;

// The slots' annihilation masks in shared memory (read once per CTA, not per amplitude).
__device__ __forceinline__ void diag_load_masks(const DiagArgs &a, uint32_t *ann)
{
    if (threadIdx.x < a.nslots) ann[threadIdx.x] = a.codes[a.ops[threadIdx.x]].annihilate;
    __syncthreads();
}

__device__ __forceinline__ uint32_t diag_mask_s(const uint32_t *ann, int nslots, uint32_t bits)
{
    uint32_t m = 0;
    for (int i = 0; i < nslots; ++i)
        if ((bits & ann[i]) == ann[i]) m |= 1u << i;
    return m;
}

// slot mask of amplitude z (< D): two string-table loads in the Sz basis, else the
// slots' annihilation masks (ann, shared memory) against the bitstring.  hm (half
// passes, Sz basis only): 0 for the amplitudes (a, b) with a > b; *same: a == b.
__device__ __forceinline__ uint32_t diag_mask_z(const DiagArgs &a, const uint32_t *ann, uint32_t z, bool hm = false,
                                                bool *same = nullptr)
{
    if (a.smA) {
        const uint32_t r = a.basis.div_nB(z), c = z - r * a.basis.nB;
        if (same) *same = r == c;
        if (hm && r > c) return 0u;
        return (uint32_t)__ldg(a.smA + r) & (uint32_t)__ldg(a.smB + c);
    }
    if (same) *same = false;
    return diag_mask_s(ann, a.nslots, a.basis.bits(z));
}

// ckpt (nullable, single vector): the amplitudes after the pass, for the adjoint sweep.
__global__ void __launch_bounds__(256, 4) k_diag_rot(DiagArgs a, double *vecs, size_t vstride, int nvec,
                                                     double *__restrict__ ckpt, int64_t inst_stride, int64_t ckpt_stride)
{
    __shared__ uint32_t ann[kMaxSlots];
    const uint64_t D = a.basis.D;
    if (skip_instance(a.active, blockIdx.y)) return;
    diag_load_masks(a, ann);
    a.table += (size_t)blockIdx.y * a.tab_stride;
    vecs += (size_t)blockIdx.y * inst_stride;
    if (ckpt) ckpt += (size_t)blockIdx.y * ckpt_stride;
    const bool hm = a.half && a.half[blockIdx.y];
    const uint64_t S = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t z0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; z0 < D; z0 += kDiagUnroll * S) {
        uint32_t m[kDiagUnroll];
#pragma unroll
        for (int u = 0; u < kDiagUnroll; ++u) {
            const uint64_t z = z0 + u * S;
            m[u] = z < D ? diag_mask_z(a, ann, (uint32_t)z, hm) : 0u;
        }
        for (int vec = 0; vec < nvec; ++vec) {
            double *p = vecs + vec * vstride;
            double2 v[kDiagUnroll];
#pragma unroll
            for (int u = 0; u < kDiagUnroll; ++u)
                if (m[u]) v[u] = *reinterpret_cast<const double2 *>(p + 2 * (z0 + u * S));
#pragma unroll
            for (int u = 0; u < kDiagUnroll; ++u) {
                if (!m[u]) continue;
                const uint64_t z = z0 + u * S;
                const double2 t = diag_phase(a, m[u]);
                const double2 r = make_double2(t.x * v[u].x - t.y * v[u].y, t.y * v[u].x + t.x * v[u].y);
                *reinterpret_cast<double2 *>(p + 2 * z) = r;
                if (ckpt) *reinterpret_cast<double2 *>(ckpt + 2 * z) = r;
            }
        }
    }
}

// Checkpointed adjoint of a diagonal pass: gradient <h|i n psi> at the pass output
// (psi from the checkpoint), then h rotated back; psi untouched.  ONE: a pass with a
// single operator (most LUCJ phase passes), whose one gradient sum needs one register;
// otherwise kMaxSlots sums in registers and half the loads in flight, so that four
// 256-thread CTAs per SM (the fixed grid kDiagGrid) stay resident.
template <bool ONE>
__global__ void __launch_bounds__(256, 4) k_diag_adj(DiagArgs a, const double *__restrict__ ckpt, int64_t ckpt_stride,
                                                     double *h, int64_t inst_stride, double *partials,
                                                     int64_t part_stride)
{
    constexpr int NS = ONE ? 1 : kMaxSlots;
    constexpr int U = ONE ? kDiagUnroll : kDiagUnroll / 2;
    __shared__ double red[8];
    __shared__ uint32_t ann[kMaxSlots];
    if (skip_instance(a.active, blockIdx.y)) return;
    diag_load_masks(a, ann);
    a.table += (size_t)blockIdx.y * a.tab_stride;
    ckpt += (size_t)blockIdx.y * ckpt_stride;
    h += (size_t)blockIdx.y * inst_stride;
    partials += (size_t)blockIdx.y * part_stride;
    double acc[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) acc[i] = 0;
    const uint64_t D = a.basis.D;
    const uint64_t S = (uint64_t)gridDim.x * blockDim.x;
    const bool hm = a.half && a.half[blockIdx.y];
    for (uint64_t z0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; z0 < D; z0 += U * S) {
        uint32_t m[U];
        bool same[U];
        double2 x[U], y[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t z = z0 + u * S;
            same[u] = false;
            m[u] = z < D ? diag_mask_z(a, ann, (uint32_t)z, hm, &same[u]) : 0u;
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (m[u]) {
                const uint64_t z = z0 + u * S;
                x[u] = __ldg(reinterpret_cast<const double2 *>(ckpt + 2 * z));
                y[u] = *reinterpret_cast<const double2 *>(h + 2 * z);
            }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (!m[u]) continue;
            const double q = y[u].y * x[u].x - y[u].x * x[u].y;
            // half passes: a = b at half weight (an FMA costs what the add did)
            const double wt = (hm && same[u]) ? 0.5 : 1.0;
            // FP64 adds past the pass's own slots would still take FP64 issue slots when
            // predicated off: leave the unrolled loop at the (uniform) slot count
#pragma unroll
            for (int i = 0; i < NS; ++i) {
                if (i == a.nslots) break;
                if (ONE || (m[u] & (1u << i))) acc[i] = fma(wt, q, acc[i]);
            }
            const double2 t = diag_phase(a, m[u]);
            *reinterpret_cast<double2 *>(h + 2 * (z0 + u * S)) =
                make_double2(t.x * y[u].x - t.y * y[u].y, t.y * y[u].x + t.x * y[u].y);
        }
    }
#pragma unroll
    for (int i = 0; i < NS; ++i) {  // the block's own slots only (uniform bound: block_sum syncs)
        if (i == a.nslots) break;
        const double g = block_sum(acc[i], red);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kMaxSlots + i] = g;
    }
}

// Adjoint of a diagonal pass in the Sz basis, psi viewed as the nA x nB matrix of
// (alpha string, beta string) amplitudes.  A CTA owns sp.cols columns (beta strings;
// the smallest power of two >= nB between 32 and 256) and a run of rows; thread t keeps
// column b and walks its rows a, so a warp always works on one row and the row's alpha
// slot mask smA[a] is the same on all its lanes.
// With q = Im(h psi*) at (a, b) (psi from the checkpoint), the gradient of slot i is the
// sum of q over the amplitudes where i is active, which the kernel splits three ways:
//   beta-only slots (no alpha bits in the annihilation mask): active on every row of a
//     column in which they are active at all: one running column sum per thread,
//     added to those slots once at the end;
//   alpha-only and mixed slots: the bits of smA[a] & (alpha-only | mixed), the same on
//     the whole warp, so that only the slots active on this row issue an FP64 add
//     (mixed ones add q where the column's beta bits also hold, else 0), into
//     per-thread sums in shared memory.
// So an amplitude costs the phase product (2 FP64), one add for the column, one per
// slot active on its row and the back-rotation (4), in place of one predicated add per
// slot of the pass.  The sums are fixed-order (per thread, then block_sum per slot).
constexpr int kDiagAdjThreads = 256;
// Passes with fewer slots keep k_diag_adj: the predicated adds it saves are few, and
// on GB300 (14-orbital LUCJ, ncu) a 2-slot pass took 149 us there against 211 us here,
// a 6-slot pass 292 us against 262 us.
constexpr int kDiagAdjSzMinSlots = 5;

constexpr int kDiagMaxColBlocks = 32;
struct DiagSplit {
    int cols;         // columns per CTA (power of two, <= kDiagAdjThreads)
    int col_blocks;   // CTAs across the columns
    int row_chunks;   // CTAs down the rows
    uint32_t b_only;  // slots with no alpha bits
    uint32_t a_rows;  // alpha-only and mixed slots
    uint32_t mixed;   // slots with both alpha and beta bits
    // half passes: the same col_blocks * row_chunks CTAs over the triangle a <= b, so
    // that every CTA has a near-equal share: column block c gets the CTAs
    // [half_first[c], half_first[c + 1]) for its rows 0 .. (c + 1) * cols - 1, cut at
    // equal work (tri_row) (half_first[0] = -1: more column blocks than
    // kDiagMaxColBlocks, no such split)
    int half_first[kDiagMaxColBlocks + 1];
};

// Rows of column block [lo, lo + L) in the half passes: row r < lo meets all L
// columns, row lo + j the L - j columns b >= r.  The first row at which the work of the
// rows before it reaches x (W(r) = r L for r <= lo, lo L + j L - j (j - 1) / 2 past it);
// the root of the quadratic in float, then exact integer steps.
__device__ __forceinline__ uint32_t tri_row(uint64_t x, uint32_t lo, uint32_t L)
{
    if (x <= (uint64_t)lo * L) return (uint32_t)((x + L - 1) / L);
    const uint64_t xp = x - (uint64_t)lo * L;
    auto C = [L](int64_t j) { return (uint64_t)(j * (int64_t)L - j * (j - 1) / 2); };
    const float t = 2.0f * L + 1.0f;
    int64_t j = (int64_t)((t - sqrtf(fmaxf(0.0f, t * t - 8.0f * (float)xp))) * 0.5f);
    if (j < 0) j = 0;
    while (j > 0 && C(j - 1) >= xp) --j;
    while (C(j) < xp) ++j;
    return lo + (uint32_t)j;
}

__global__ void __launch_bounds__(kDiagAdjThreads, 4) k_diag_adj_sz(DiagArgs a, DiagSplit sp,
                                                                    const double *__restrict__ ckpt,
                                                                    int64_t ckpt_stride, double *h,
                                                                    int64_t inst_stride, double *partials,
                                                                    int64_t part_stride)
{
    constexpr int U = 4;  // rows in flight per thread
    __shared__ double sacc[kMaxSlots][kDiagAdjThreads];
    __shared__ double red[kDiagAdjThreads / 32];
    if (skip_instance(a.active, blockIdx.y)) return;
    a.table += (size_t)blockIdx.y * a.tab_stride;
    ckpt += (size_t)blockIdx.y * ckpt_stride;
    h += (size_t)blockIdx.y * inst_stride;
    partials += (size_t)blockIdx.y * part_stride;
    const int tid = threadIdx.x;
    for (int i = 0; i < a.nslots; ++i) sacc[i][tid] = 0.0;
    const uint32_t nA = a.basis.nA, nB = a.basis.nB;
    // half passes: only the rows a <= b of this column, a = b at half weight; the warp
    // stops after the last row that any of its 32 columns needs
    const bool hm = a.half && a.half[blockIdx.y];
    int cb = blockIdx.x % sp.col_blocks, rc = blockIdx.x / sp.col_blocks;
    uint32_t r0 = (uint32_t)((uint64_t)nA * rc / sp.row_chunks);
    uint32_t r1 = (uint32_t)((uint64_t)nA * (rc + 1) / sp.row_chunks);
    if (hm && sp.half_first[0] >= 0) {
        // this column block's share of the CTAs, cut into rows of equal work
        cb = 0;
        while (cb + 1 < sp.col_blocks && (int)blockIdx.x >= sp.half_first[cb + 1]) ++cb;
        rc = (int)blockIdx.x - sp.half_first[cb];
        const int nch = sp.half_first[cb + 1] - sp.half_first[cb];
        const uint32_t lo = (uint32_t)(cb * sp.cols), L = min(nB, lo + (uint32_t)sp.cols) - lo;
        const uint64_t Wb = (uint64_t)lo * L + (uint64_t)L * (L + 1) / 2;
        r0 = tri_row(Wb * rc / nch, lo, L);
        r1 = tri_row(Wb * (rc + 1) / nch, lo, L);
    }
    const uint32_t b = (uint32_t)(cb * sp.cols + (tid & (sp.cols - 1)));
    const bool col_ok = b < nB;
    const uint32_t mb = col_ok ? (uint32_t)__ldg(a.smB + b) : 0u;
    const int lanes = kDiagAdjThreads / sp.cols;  // row lanes per CTA
    double col = 0.0;
    const uint32_t warp_b_end = (uint32_t)(cb * sp.cols + ((tid & (sp.cols - 1)) & ~31)) + 32u;
    const uint32_t r_end = hm ? min(r1, warp_b_end) : r1;
    for (uint32_t a0 = r0 + (uint32_t)(tid / sp.cols); a0 < r_end; a0 += U * lanes) {
        uint32_t ma[U], m[U];
        double2 x[U], y[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t ar = a0 + u * lanes;
            ma[u] = ar < r_end ? (uint32_t)__ldg(a.smA + ar) : 0u;
            m[u] = col_ok && !(hm && ar > b) ? ma[u] & mb : 0u;
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (m[u]) {
                const size_t z = (size_t)(a0 + u * lanes) * nB + b;
                x[u] = __ldg(reinterpret_cast<const double2 *>(ckpt + 2 * z));
                y[u] = *reinterpret_cast<const double2 *>(h + 2 * z);
            }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const double q = m[u] ? y[u].y * x[u].x - y[u].x * x[u].y : 0.0;
            const double wt = (hm && a0 + u * lanes == b) ? 0.5 : 1.0;
            if (sp.b_only) col = fma(wt, q, col);
            for (uint32_t r = ma[u] & sp.a_rows; r; r &= r - 1u) {  // uniform over the warp
                const int i = __ffs(r) - 1;
                const bool on = !((sp.mixed >> i) & 1u) || ((mb >> i) & 1u);
                sacc[i][tid] = fma(wt, on ? q : 0.0, sacc[i][tid]);
            }
            if (m[u]) {
                const size_t z = (size_t)(a0 + u * lanes) * nB + b;
                const double2 t = diag_phase(a, m[u]);
                *reinterpret_cast<double2 *>(h + 2 * z) =
                    make_double2(t.x * y[u].x - t.y * y[u].y, t.y * y[u].x + t.x * y[u].y);
            }
        }
    }
    for (int i = 0; i < a.nslots; ++i) {  // uniform bound: block_sum synchronises
        const double v = sacc[i][tid] + ((((sp.b_only & mb) >> i) & 1u) ? col : 0.0);
        const double g = block_sum(v, red);
        if (tid == 0) partials[(size_t)blockIdx.x * kMaxSlots + i] = g;
    }
}

__global__ void k_diag_tangent(DiagArgs a, double *psi, double *T, size_t tstride, const int *tpos)
{
    const uint64_t D = a.basis.D;
    for (uint64_t z = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; z < D; z += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t m = a.smA ? diag_mask_z(a, nullptr, (uint32_t)z) : diag_mask(a, a.basis.bits((uint32_t)z));
        if (!m) continue;
        const double2 ph = diag_phase(a, m);
        const double c = ph.x, s = ph.y;
        double *p = psi + 2 * z;
        const double re = c * p[0] - s * p[1], im = s * p[0] + c * p[1];
        p[0] = re;
        p[1] = im;
        for (int i = 0; i < a.nslots; ++i)
            if (m & (1u << i)) {
                double *t = T + (size_t)tpos[a.ops[i]] * tstride + 2 * z;
                t[0] = -im;
                t[1] = re;
            }
    }
}

__global__ void __launch_bounds__(256) k_diag_hess(DiagArgs a, const double *h, double *T, size_t tstride, int nvec,
                                                   int block_pos0, double *partials)
{
    __shared__ double red[8];
    const int vec = blockIdx.y;
    double acc[kMaxSlots];
#pragma unroll
    for (int i = 0; i < kMaxSlots; ++i) acc[i] = 0;
    const uint64_t D = a.basis.D;
    double *t = T + (size_t)vec * tstride;
    for (uint64_t z = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; z < D; z += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t m = a.smA ? diag_mask_z(a, nullptr, (uint32_t)z) : diag_mask(a, a.basis.bits((uint32_t)z));
        if (!m) continue;
        double *x = t + 2 * z;
        const double xr = x[0], xi = x[1], hr = h[2 * z], hi = h[2 * z + 1];
        const double q = hi * xr - hr * xi;
#pragma unroll
        for (int i = 0; i < kMaxSlots; ++i) {
            if (i == a.nslots) break;  // uniform bound, as in k_diag_adj
            if ((m & (1u << i)) && block_pos0 + i >= vec) acc[i] += q;
        }
        const double2 ph = diag_phase(a, m);
        x[0] = ph.x * xr - ph.y * xi;
        x[1] = ph.y * xr + ph.x * xi;
    }
#pragma unroll
    for (int i = 0; i < kMaxSlots; ++i) {  // compile-time indices keep acc in registers
        if (i == a.nslots) break;
        const double g = block_sum(acc[i], red);
        if (threadIdx.x == 0) partials[((size_t)blockIdx.x * nvec + vec) * kMaxSlots + i] = g;
    }
}

// After a sweep of spin-flip half passes only the amplitudes (a, b) with a <= b are
// current: each is copied to its mirror (b, a), for the instances that took them.
template <int W>
__global__ void k_flip_fill(DevBasis B, double *psi, int64_t inst_stride, const int *__restrict__ half,
                            const int *__restrict__ active)
{
    const int inst = blockIdx.y;
    if (!half[inst] || skip_instance(active, inst)) return;
    psi += (size_t)inst * inst_stride;
    for (uint64_t z = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; z < B.D; z += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = B.div_nB((uint32_t)z), c = (uint32_t)z - a * B.nB;
        if (a <= c) continue;
        const size_t src = (size_t)c * B.nB + a;
#pragma unroll
        for (int w = 0; w < W; ++w) psi[z * W + w] = psi[src * W + w];
    }
}

__global__ void k_set_int(int *p, int v) { *p = v; }

// ------------------------------------------------------------ reductions --
// grad[op] = scale * sum over the tiles of op's block of partials[tile][slot].
// warp per (instance, operator); instance b's partial sums start at b * part_stride.
// Spin-flip half passes (half[b] set; mirror: operator -> mirror operator): the
// sweep visited one orbit of every mirror pair, so the gradient of an operator is its
// own sum plus its mirror's (the two results are the same sum, bit for bit).
__global__ void k_grad_reduce(const double *__restrict__ partials, const int64_t *__restrict__ op_part_off,
                              const int *__restrict__ op_ntiles, const int *__restrict__ op_slot, int nops, double scale,
                              double *__restrict__ grad, int nb, int64_t part_stride, const int *__restrict__ active,
                              const int *__restrict__ mirror, const int *__restrict__ half)
{
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (gw >= nops * nb) return;
    const int b = gw / nops, warp = gw - b * nops;
    if (skip_instance(active, b)) return;
    grad += (size_t)b * nops;
    auto op_sum = [&](int op) {
        const double *p = partials + (size_t)b * part_stride + op_part_off[op];
        const int nt = op_ntiles[op], sl = op_slot[op];
        double s = 0;
        for (int t = lane; t < nt; t += 32) s += p[(size_t)t * kMaxSlots + sl];
        return warp_sum(s);
    };
    double s = op_sum(warp);
    if (mirror && half && half[b]) s += op_sum(mirror[warp]);
    if (lane == 0) grad[warp] = scale * s;
}

// Hessian second-derivative partials of one block -> Hops (nops x nops, row-major).
// Half tangents (vmap, mirror, tpos set): grid row vec carried the tangent at position
// vmap[vec]; the pair of operators it yields also stands for its mirror pair, whose
// value is the same (the circuit commutes with the exchange of the alpha and beta
// strings), where the mirror pair's earlier operator is one whose tangent was not
// carried (so that no pair is counted twice).
__global__ void k_hess_reduce(const double *__restrict__ partials, int ntiles, int nvec, int nslots,
                              const int *__restrict__ pos_op, const int *__restrict__ block_ops, int block_pos0,
                              double *__restrict__ Hops, int nops, double factor, const int *__restrict__ vmap,
                              const int *__restrict__ mirror, const int *__restrict__ tpos)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= nvec * nslots) return;
    const int vec = warp / nslots, sl = warp % nslots;
    const int vpos = vmap ? vmap[vec] : vec;
    if (block_pos0 + sl < vpos) return;
    double s = 0;
    for (int t = lane; t < ntiles; t += 32) s += partials[((size_t)t * nvec + vec) * kMaxSlots + sl];
    s = warp_sum(s);
    if (lane == 0) {
        const int i = pos_op[vpos], j = block_ops[sl];
        Hops[(size_t)i * nops + j] += factor * s;
        if (i != j) Hops[(size_t)j * nops + i] += factor * s;
        if (vmap) {
            const int mi = mirror[i], mj = mirror[j];
            const bool same = (mi == i && mj == j) || (mi == j && mj == i);
            const int first = tpos[mi] <= tpos[mj] ? mi : mj;        // the mirror pair's earlier operator
            const bool carried = tpos[first] <= tpos[mirror[first]];  // its tangent was carried
            if (!same && !carried) {
                Hops[(size_t)mi * nops + mj] += factor * s;
                if (mi != mj) Hops[(size_t)mj * nops + mi] += factor * s;
            }
        }
    }
}

// -------------------------------------------------------------- H * psi --
// Warp per row, y_j = sum_k val[k] x[col[k]], fused with partial sums of <x|y>.
template <int W, bool ELL>
__global__ void __launch_bounds__(kSpmvThreads) k_spmv(const int64_t *__restrict__ rowptr, int ell_width,
                                                       const int32_t *__restrict__ col, const double *__restrict__ val,
                                                       const double *__restrict__ x, double *__restrict__ y, int64_t D,
                                                       double *__restrict__ epart, const int *__restrict__ active)
{
    __shared__ double red[kSpmvThreads / 32];
    if (skip_instance(active, blockIdx.y)) return;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    x += (size_t)blockIdx.y * D * W;  // instance blockIdx.y, same matrix
    y += (size_t)blockIdx.y * D * W;
    if (epart) epart += (size_t)blockIdx.y * gridDim.x;
    double e = 0;
    for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < D; r += warps) {
        const int64_t b = ELL ? r * ell_width : rowptr[r], end = ELL ? b + ell_width : rowptr[r + 1];
        double acc[W];
#pragma unroll
        for (int w = 0; w < W; ++w) acc[w] = 0;
        for (int64_t k = b + lane; k < end; k += 32) {
            const double h = __ldg(val + k);
            const size_t c = (size_t)__ldg(col + k);
#pragma unroll
            for (int w = 0; w < W; ++w) acc[w] = fma(h, __ldg(x + c * W + w), acc[w]);
        }
#pragma unroll
        for (int w = 0; w < W; ++w) acc[w] = warp_sum(acc[w]);
        if (lane == 0) {
#pragma unroll
            for (int w = 0; w < W; ++w) {
                y[r * W + w] = acc[w];
                e = fma(acc[w], x[r * W + w], e);
            }
        }
    }
    e = block_sum(e, red);
    if (threadIdx.x == 0 && epart) epart[blockIdx.x] = e;
}

// Sliced-ELL product, one thread per row: 4 independent FP64 accumulators, no
// cross-lane reduction (its shuffles and adds would cost FP64 issue slots, the
// binding pipe of this kernel on GB300), fused with the partial sums of <x|y>.
template <int W, int T>
__global__ void __launch_bounds__(kSpmvThreads) k_spmv_sell(int64_t q, const int32_t *__restrict__ col,
                                                            const double *__restrict__ val,
                                                            const double *__restrict__ x, double *__restrict__ y,
                                                            int64_t D, double *__restrict__ epart, int64_t mat_stride,
                                                            const int *__restrict__ active)
{
    if (skip_instance(active, blockIdx.y)) return;
    // T threads per row: a warp covers 32/T consecutive rows of one 32-row slab; lane
    // (sub, k) takes row k's groups sub, sub+T, ... (each group read by 32/T lanes is
    // one contiguous run), and the T partial sums meet in a fixed butterfly.
    constexpr int RPW = 32 / T;
    __shared__ double red[kSpmvThreads / 32];
    const int lane = threadIdx.x & 31, sub = lane / RPW;
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane) / T + lane % RPW;
    // instance blockIdx.y: its vectors, and its matrix (mat_stride = 0 when shared)
    col += (size_t)blockIdx.y * mat_stride;
    val += (size_t)blockIdx.y * mat_stride;
    x += (size_t)blockIdx.y * D * W;
    y += (size_t)blockIdx.y * D * W;
    if (epart) epart += (size_t)blockIdx.y * gridDim.x;
    double e = 0;
    double a0[W], a1[W], a2[W], a3[W];
#pragma unroll
    for (int w = 0; w < W; ++w) a0[w] = a1[w] = a2[w] = a3[w] = 0.0;
    if (r < D) {
        const size_t base = ell_pos(r, 0, q);  // group g of this row starts at base + 128 g
        const int4 *c4 = reinterpret_cast<const int4 *>(col + base);
        const double2 *v2 = reinterpret_cast<const double2 *>(val + base);
        for (int64_t g = sub; g < q; g += T) {
            const int4 c = __ldg(c4 + 32 * g);
            const double2 h01 = __ldg(v2 + 64 * g), h23 = __ldg(v2 + 64 * g + 1);
#pragma unroll
            for (int w = 0; w < W; ++w) {
                a0[w] = fma(h01.x, __ldg(x + (size_t)c.x * W + w), a0[w]);
                a1[w] = fma(h01.y, __ldg(x + (size_t)c.y * W + w), a1[w]);
                a2[w] = fma(h23.x, __ldg(x + (size_t)c.z * W + w), a2[w]);
                a3[w] = fma(h23.y, __ldg(x + (size_t)c.w * W + w), a3[w]);
            }
        }
    }
#pragma unroll
    for (int w = 0; w < W; ++w) {
        double acc = (a0[w] + a1[w]) + (a2[w] + a3[w]);
#pragma unroll
        for (int o = RPW; o < 32; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (r < D && sub == 0) {
            y[r * W + w] = acc;
            e = fma(acc, x[r * W + w], e);
        }
    }
    e = block_sum(e, red);
    if (threadIdx.x == 0 && epart) epart[blockIdx.x] = e;
}


// Compressed tangents T_C[j][w][mu] = sum_{op: param(op)=mu} scale_op T[pos(op)][j][w];
// column P holds psi (fusedevolve.cpp:2609-2612, m_compressMatrixPsi).
// mpos (nullable; the Hessian's half tangents): for entry k, -1, or the position of the
// mirror tangent that was carried in its place; the tangent is then that one with the
// alpha and beta strings exchanged, read at the mirrored amplitude (rows and columns of
// the nA x nA string matrix swapped; B gives nB and the division).
__global__ void k_tc_build(const double *__restrict__ T, size_t tstride, const double *__restrict__ psi,
                           const int *__restrict__ prm_ptr, const int *__restrict__ prm_pos,
                           const double *__restrict__ prm_scale, int P, int W, int64_t D, double *__restrict__ TC,
                           const int *__restrict__ mpos, DevBasis B)
{
    const int V = P + 1;
    const int64_t total = D * W * V;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int mu = (int)(t % V);
        const int64_t jw = t / V;
        double s;
        if (mu == P) {
            s = psi[jw];
        } else {
            s = 0;
            for (int k = prm_ptr[mu]; k < prm_ptr[mu + 1]; ++k) {
                if (mpos && mpos[k] >= 0) {
                    const uint32_t z = (uint32_t)(jw / W), w = (uint32_t)(jw - (int64_t)z * W);
                    const uint32_t ra = B.div_nB(z), rb = z - ra * B.nB;
                    const size_t jm = ((size_t)rb * B.nB + ra) * W + w;
                    s += prm_scale[k] * T[(size_t)mpos[k] * tstride + jm];
                } else {
                    s += prm_scale[k] * T[(size_t)prm_pos[k] * tstride + jw];
                }
            }
        }
        TC[(size_t)mu * D * W + jw] = s;  // column-major: column mu is a contiguous vector
    }
}

// --------------------------------------------- Hamiltonian from integrals --
struct IntArgs {
    int N, nq;
    const double *h1, *g2;
    DevBasis basis;
    int nOa, nVa, nOb, nVb;
    int64_t width;    // entries per row
    int64_t stride;   // stored entries per row (width rounded up to a multiple of 4; padding is col = row, val = 0)
    // coded rows (see k_vell_build): explicit entries (diagonal + singles) and coded
    // entries (doubles), each rounded up to a multiple of 4
    int64_t width_e, stride_e, width_d, stride_d;
    int NP;           // spatial orbital pairs N (N - 1) / 2
};

__device__ __forceinline__ double two_e(const IntArgs &a, int p, int q, int r, int s)
{
    // op a^+_p a^+_q a_r a_s, p<q, r<s (hamiltonianmatrix.cpp:456-470, 479-505)
    const int N = a.N;
    const int sp = p >= N, sq = q >= N, sr = r >= N, ss = s >= N;
    const int P = p - sp * N, Q = q - sq * N, R = r - sr * N, S = s - ss * N;
    double E = 0;
    if (sp == sr && sq == ss) E += a.g2[(((size_t)Q * N + S) * N + P) * N + R];
    if (sp == ss && sq == sr) E -= a.g2[(((size_t)Q * N + R) * N + P) * N + S];
    return fabs(E) > 1e-13 ? E : 0.0;
}

__device__ __forceinline__ uint32_t below(int x) { return (1u << x) - 1u; }

__device__ __forceinline__ double op_sign(uint32_t J, uint32_t mask) { return (__popc(J & mask) & 1) ? -1.0 : 1.0; }

__device__ __forceinline__ double double_val(const IntArgs &a, uint32_t J, int p, int q, int r, int s)
{
    // created p<q (in J), destroyed r<s
    uint32_t m = below(p) ^ below(q) ^ below(r) ^ below(s);
    m &= ~((1u << p) | (1u << q) | (1u << r) | (1u << s));
    return op_sign(J, m) * two_e(a, p, q, r, s);
}

// Single p <- r (J holds p, the input determinant holds r): one-electron op plus the
// two-electron ops a^+_p a^+_t a_r a_t over the other occupied orbitals t of J.
__device__ double single_val(const IntArgs &a, uint32_t J, int p, int r)
{
    const int N = a.N;
    uint32_t m = (below(p) ^ below(r)) & ~((1u << p) | (1u << r));
    double h = a.h1[(p % N) * N + (r % N)];
    double v = 0;
    uint32_t occ = J & ~(1u << p);
    while (occ) {
        const int t = __ffs(occ) - 1;
        occ &= occ - 1;
        const int c0 = min(p, t), c1 = max(p, t), d0 = min(r, t), d1 = max(r, t);
        v += double_val(a, J, c0, c1, d0, d1);
    }
    return v + (fabs(h) > 1e-13 ? op_sign(J, m) * h : 0.0);
}

__device__ double diag_val(const IntArgs &a, uint32_t J)
{
    const int N = a.N;
    double v = 0;
    uint32_t o1 = J;
    while (o1) {
        const int p = __ffs(o1) - 1;
        o1 &= o1 - 1;
        uint32_t o2 = o1;
        while (o2) {
            const int q = __ffs(o2) - 1;
            o2 &= o2 - 1;
            v += two_e(a, p, q, p, q);
        }
    }
    uint32_t o = J;
    while (o) {
        const int p = __ffs(o) - 1;
        o &= o - 1;
        const double h = a.h1[(p % N) * N + (p % N)];
        if (fabs(h) > 1e-13) v += h;
    }
    return v;
}

// k-th set bit of x (0-based)
__device__ __forceinline__ int nth_bit(uint32_t x, int k)
{
    for (int i = 0; i < k; ++i) x &= x - 1;
    return __ffs(x) - 1;
}

// pair index -> (i < j) in lexicographic order over n items
__device__ __forceinline__ void pair_of(int k, int n, int &i, int &j)
{
    i = 0;
    while (k >= n - 1 - i) {
        k -= n - 1 - i;
        ++i;
    }
    j = i + 1 + k;
}

// Entry e of row J: returns the input determinant and the matrix element.
// Order: diagonal; alpha singles; beta singles; aa doubles; bb doubles; ab doubles.
__device__ void row_entry(const IntArgs &a, uint32_t J, int64_t e, uint32_t &I, double &v)
{
    const int N = a.N;
    const uint32_t full = below(N);
    const uint32_t Ja = J >> N, Jb = J & full;
    const uint32_t Va = ~Ja & full, Vb = ~Jb & full;
    const int64_t Sa = (int64_t)a.nOa * a.nVa, Sb = (int64_t)a.nOb * a.nVb;
    const int64_t Daa = (int64_t)(a.nOa * (a.nOa - 1) / 2) * (a.nVa * (a.nVa - 1) / 2);
    const int64_t Dbb = (int64_t)(a.nOb * (a.nOb - 1) / 2) * (a.nVb * (a.nVb - 1) / 2);
    if (e == 0) {
        I = J;
        v = diag_val(a, J);
        return;
    }
    e -= 1;
    if (e < Sa) {
        const int p = nth_bit(Ja, (int)(e / a.nVa)) + N, r = nth_bit(Va, (int)(e % a.nVa)) + N;
        I = J ^ (1u << p) ^ (1u << r);
        v = single_val(a, J, p, r);
        return;
    }
    e -= Sa;
    if (e < Sb) {
        const int p = nth_bit(Jb, (int)(e / a.nVb)), r = nth_bit(Vb, (int)(e % a.nVb));
        I = J ^ (1u << p) ^ (1u << r);
        v = single_val(a, J, p, r);
        return;
    }
    e -= Sb;
    if (e < Daa + Dbb) {
        const bool alpha = e < Daa;
        if (!alpha) e -= Daa;
        const uint32_t O = alpha ? Ja : Jb, Vv = alpha ? Va : Vb;
        const int nO = alpha ? a.nOa : a.nOb, nV = alpha ? a.nVa : a.nVb, off = alpha ? N : 0;
        const int nvp = nV * (nV - 1) / 2;
        int i0, i1, j0, j1;
        pair_of((int)(e / nvp), nO, i0, i1);
        pair_of((int)(e % nvp), nV, j0, j1);
        const int p = nth_bit(O, i0) + off, q = nth_bit(O, i1) + off;
        const int r = nth_bit(Vv, j0) + off, s = nth_bit(Vv, j1) + off;
        I = J ^ (1u << p) ^ (1u << q) ^ (1u << r) ^ (1u << s);
        v = double_val(a, J, p, q, r, s);
        return;
    }
    e -= Daa + Dbb;
    {
        const int64_t ea = e / Sb, eb = e % Sb;
        const int pa = nth_bit(Ja, (int)(ea / a.nVa)) + N, ra = nth_bit(Va, (int)(ea % a.nVa)) + N;
        const int pb = nth_bit(Jb, (int)(eb / a.nVb)), rb = nth_bit(Vb, (int)(eb % a.nVb));
        I = J ^ (1u << pa) ^ (1u << ra) ^ (1u << pb) ^ (1u << rb);
        v = double_val(a, J, pb, pa, rb, ra);
    }
}

__global__ void k_ell_build(IntArgs a, int32_t *__restrict__ col, double *__restrict__ val, int64_t r0, int64_t r1)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t q = a.stride >> 2, D = (int64_t)a.basis.D;
    for (int64_t r = r0 + (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < r1; r += warps) {
        // rows past D pad the last slab: column 0, value 0
        const uint32_t J = r < D ? a.basis.bits((uint32_t)r) : 0u;
        for (int64_t e = lane; e < a.stride; e += 32) {
            uint32_t I = J;
            double v = 0.0;
            int32_t c = 0;
            if (r < D) {
                if (e < a.width) row_entry(a, J, e, I, v);
                c = (int32_t)a.basis.rank_of(I);
            }
            const size_t p = ell_pos(r, e, q);
            col[p] = c;
            val[p] = v;
        }
    }
}

// ------------------------------------------------------ coded stored rows --
// 96 % of a row's entries are double excitations, whose value is a fermionic sign times
// an integral combination that depends only on the four orbitals (two_e).  Coded rows
// keep those as a 2-byte code -- sign << 15 | index into a value table of every distinct
// two_e -- next to the 4-byte column, and keep the diagonal and the singles (whose values
// depend on the determinant) explicit.  Table: [0] = 0 (padding), then the same-spin
// values two_e(P, Q, R, S) for spatial pairs P < Q, R < S (alpha and beta share them),
// then the alpha-beta values two_e(pb, pa, rb, ra) at ((pa N + ra) N + pb) N + rb.  The
// product sign * table[index] is exactly the value row_entry builds.
constexpr int kVtabMax = 1 << 15;
constexpr int kVellThreads = 1024;
constexpr int kVellNV1 = 4, kVellNV2 = 2;  // right-hand sides per thread (real, complex) of the multi-vector product

__host__ __device__ __forceinline__ int64_t vtab_len(int N)
{
    const int64_t NP = (int64_t)N * (N - 1) / 2;
    return 1 + NP * NP + (int64_t)N * N * N * N;
}

__device__ __forceinline__ int pair_index(int i, int j, int n)  // i < j, lexicographic (pair_of's order)
{
    return i * n - i * (i + 1) / 2 + (j - i - 1);
}

__global__ void k_vtab_build(IntArgs a, double *__restrict__ vtab)
{
    const int N = a.N, NP = a.NP;
    const int64_t n = vtab_len(N), ss = (int64_t)NP * NP;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        double v = 0.0;
        if (k >= 1 && k <= ss) {
            int P, Q, R, S;
            pair_of((int)((k - 1) / NP), N, P, Q);
            pair_of((int)((k - 1) % NP), N, R, S);
            v = two_e(a, P + N, Q + N, R + N, S + N);
        } else if (k > ss) {
            const int64_t t = k - 1 - ss;
            const int rb = (int)(t % N), pb = (int)((t / N) % N), ra = (int)((t / N / N) % N), pa = (int)(t / N / N / N);
            v = two_e(a, pb, pa + N, rb, ra + N);
        }
        vtab[k] = v;
    }
}

// Coded double d of row J (d counts the row's aa, bb, ab doubles in row_entry's order):
// the input determinant and the code.
__device__ void row_code(const IntArgs &a, uint32_t J, int64_t d, uint32_t &I, uint16_t &code)
{
    const int N = a.N;
    const uint32_t full = below(N);
    const uint32_t Ja = J >> N, Jb = J & full;
    const uint32_t Va = ~Ja & full, Vb = ~Jb & full;
    const int64_t Sb = (int64_t)a.nOb * a.nVb;
    const int64_t Daa = (int64_t)(a.nOa * (a.nOa - 1) / 2) * (a.nVa * (a.nVa - 1) / 2);
    const int64_t Dbb = (int64_t)(a.nOb * (a.nOb - 1) / 2) * (a.nVb * (a.nVb - 1) / 2);
    int p, q, r, t;
    int64_t idx;
    if (d < Daa + Dbb) {
        const bool alpha = d < Daa;
        if (!alpha) d -= Daa;
        const uint32_t O = alpha ? Ja : Jb, Vv = alpha ? Va : Vb;
        const int nO = alpha ? a.nOa : a.nOb, nV = alpha ? a.nVa : a.nVb, off = alpha ? N : 0;
        const int nvp = nV * (nV - 1) / 2;
        int i0, i1, j0, j1;
        pair_of((int)(d / nvp), nO, i0, i1);
        pair_of((int)(d % nvp), nV, j0, j1);
        const int P = nth_bit(O, i0), Q = nth_bit(O, i1), R = nth_bit(Vv, j0), S = nth_bit(Vv, j1);
        p = P + off, q = Q + off, r = R + off, t = S + off;
        idx = 1 + (int64_t)pair_index(P, Q, N) * a.NP + pair_index(R, S, N);
    } else {
        d -= Daa + Dbb;
        const int64_t ea = d / Sb, eb = d % Sb;
        const int pa = nth_bit(Ja, (int)(ea / a.nVa)), ra = nth_bit(Va, (int)(ea % a.nVa));
        const int pb = nth_bit(Jb, (int)(eb / a.nVb)), rb = nth_bit(Vb, (int)(eb % a.nVb));
        p = pb, q = pa + N, r = rb, t = ra + N;
        idx = 1 + (int64_t)a.NP * a.NP + (((int64_t)pa * N + ra) * N + pb) * N + rb;
    }
    I = J ^ (1u << p) ^ (1u << q) ^ (1u << r) ^ (1u << t);
    uint32_t m = below(p) ^ below(q) ^ below(r) ^ below(t);
    m &= ~((1u << p) | (1u << q) | (1u << r) | (1u << t));
    code = (uint16_t)((uint32_t)idx | ((__popc(J & m) & 1u) << 15));
}

// Coded rows of rows [r0, r1): both parts in the sliced layout of ell_pos (slabs of 32
// rows, inside a slab the 4-entry groups of the 32 rows contiguous).  values_only: new
// integrals for rows already built -- columns and codes depend on the determinants
// alone, so only the explicit values are rewritten (the table is rebuilt apart).
__global__ void k_vell_build(IntArgs a, int32_t *__restrict__ colE, double *__restrict__ valE, int32_t *__restrict__ colD,
                             uint16_t *__restrict__ codeD, int64_t r0, int64_t r1, bool values_only)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t qe = a.stride_e >> 2, qd = a.stride_d >> 2, D = (int64_t)a.basis.D;
    for (int64_t r = r0 + (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < r1; r += warps) {
        // padding: rows past D and entries past the row's width point at the row itself
        // (row 0 past D) with value / code 0
        const uint32_t J = r < D ? a.basis.bits((uint32_t)r) : 0u;
        const int32_t self = r < D ? (int32_t)r : 0;
        for (int64_t e = lane; e < a.stride_e; e += 32) {
            uint32_t I = J;
            double v = 0.0;
            int32_t c = self;
            if (r < D && e < a.width_e) {
                row_entry(a, J, e, I, v);
                if (!values_only) c = (int32_t)a.basis.rank_of(I);
            }
            const size_t p = ell_pos(r, e, qe);
            if (!values_only) colE[p] = c;
            valE[p] = v;
        }
        if (values_only) continue;
        for (int64_t e = lane; e < a.stride_d; e += 32) {
            uint32_t I = J;
            uint16_t code = 0;
            int32_t c = self;
            if (r < D && e < a.width_d) {
                row_code(a, J, e, I, code);
                c = (int32_t)a.basis.rank_of(I);
            }
            const size_t p = ell_pos(r, e, qd);
            colD[p] = c;
            codeD[p] = code;
        }
    }
}

struct VellArgs {
    const int32_t *colE, *colD;
    const double *valE, *vtab;
    const uint16_t *codeD;
    int64_t qe, qd;               // groups of 4 per row
    int64_t inst_e, inst_d;       // entries between instances' explicit / coded parts (0 = shared)
    int64_t vtab_len, vtab_inst;  // table entries, entries between instances' tables (0 = shared)
};

__device__ __forceinline__ double signed_value(const double *tab, uint32_t code)
{
    const double t = tab[code & 0x7fffu];
    return __longlong_as_double(__double_as_longlong(t) ^ ((long long)(code >> 15) << 63));
}

// ------------------------------------------------ spin-flip half product --
// With as many alpha as beta electrons, the Sz basis pairs determinant (a, b) (alpha
// string a, beta string b; row a * nB + b) with its spin-flipped partner (b, a).  A
// Hamiltonian built from spin-free integrals takes the same value on both members of
// every pair of pairs (H[(b,a),(b',a')] = H[(a,b),(a',b')], the sign of the flip being
// the same for every determinant), so when x(b, a) = x(a, b) for every pair -- true, up
// to rounding, of every state a spin-adapted ansatz with one angle per spatial
// excitation makes from a closed-shell start (tUPS through its compressed parameters,
// LUCJ) -- (H x)(b, a) = (H x)(a, b) as well: the product computes the rows with
// a <= b and writes each result to its mirror row too, half the matrix elements (the
// symmetry the direct-CI literature uses for Ms = 0: Knowles & Handy, Chem. Phys. Lett.
// 111, 315 (1984); Olsen et al., J. Chem. Phys. 89, 2185 (1988)).  Every product that
// may take this path first measures the invariance of its input on the device
// (k_flip_check); the product kernels read the partial sums in a fixed order and take
// the half product only when ||x - flip x|| <= kFlipTol ||x||, the full one otherwise.
constexpr double kFlipTol = 1e-12;

struct FlipArgs {
    const double *part;     // per instance, G pairs (sum |x|^2, sum over a < b of |x(a,b) - x(b,a)|^2); null: full product
    const int32_t *slabs;   // stored rows: the 32-row slabs that hold a row with a <= b, ascending
    int64_t nslabs;
    int *used;              // per instance: 1 where the product took the half path (nullable)
    int G;
    uint32_t nB, div_m, div_l;  // z / nB as in DevBasis
    __device__ __forceinline__ uint32_t alpha_of(uint32_t z) const
    {
        if (div_l == 0) return z;
        const uint32_t hi = __umulhi(div_m, z);
        return (hi + ((z - hi) >> 1)) >> (div_l - 1);
    }
};

// Partial sums of the invariance test for instance blockIdx.y: sum |x|^2 and the sum
// over a < b of |x(a,b) - x(b,a)|^2, one pair per CTA, in a fixed order.
template <int W>
__global__ void k_flip_check(FlipArgs f, const double *__restrict__ x, int64_t D, double *__restrict__ part,
                             const int *__restrict__ active)
{
    __shared__ double red[32];
    if (skip_instance(active, blockIdx.y)) return;
    x += (size_t)blockIdx.y * D * W;
    double s0 = 0.0, s1 = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < D; r += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t a = f.alpha_of((uint32_t)r), b = (uint32_t)r - a * f.nB;
        const int64_t rf = (int64_t)b * f.nB + a;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const double v = x[r * W + w];
            s0 = fma(v, v, s0);
            if (a < b) {
                const double d = v - x[rf * W + w];
                s1 = fma(d, d, s1);
            }
        }
    }
    s0 = block_sum(s0, red);
    s1 = block_sum(s1, red);
    if (threadIdx.x == 0) {
        double *p = part + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 2;
        p[0] = s0;
        p[1] = s1;
    }
}

// The half-product decision for instance b, by warp 0 of the calling CTA (every lane
// returns it): the G partial pairs summed lane-strided, then a fixed butterfly.
__device__ __forceinline__ bool flip_half(const FlipArgs &f, int b)
{
    if (!f.part) return false;
    const double *p = f.part + (size_t)b * f.G * 2;
    const int lane = threadIdx.x & 31;
    double s0 = 0.0, s1 = 0.0;
    for (int i = lane; i < f.G; i += 32) {
        s0 += p[2 * i];
        s1 += p[2 * i + 1];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    return s1 <= kFlipTol * kFlipTol * s0;  // a zero vector passes (s1 = s0 = 0)
}

// y = H x with coded rows.  T threads per row as in k_spmv_sell.  Each CTA owns an
// equal contiguous share of the rows (a multiple of 32), walked 1024 / T rows at a
// time, so that every SM ends with the same work (the FP64 pipe is the limit, and a
// grid of whole row blocks left some SMs one block behind the rest); the value table is
// staged once per CTA, in shared memory.  NV > 1: one thread carries NV right-hand sides (instances
// blockIdx.y * NV + v, shared matrix, no energy and no mask), so each matrix entry read
// serves NV products.  Energy partial per CTA: sum over its rows of y_r x_r.
// Half product (flip.part set and every right-hand side of the CTA flip-invariant):
// the CTAs share the slabs of flip.slabs instead of all rows, rows with a > b are left
// to their mirror, and each row's result also goes to its mirror row (energy: both rows).
template <int W, int T, int NV>
__global__ void __launch_bounds__(kVellThreads, 1) k_spmv_vell(VellArgs m, const double *__restrict__ x,
                                                               double *__restrict__ y, int64_t D, int ninst,
                                                               double *__restrict__ epart, const int *__restrict__ active,
                                                               FlipArgs flip)
{
    extern __shared__ double tab[];
    __shared__ double red[kVellThreads / 32];
    __shared__ int s_half;
    const int b0 = blockIdx.y * NV;
    if (NV == 1 && skip_instance(active, b0)) return;
    if (threadIdx.x < 32) {
        // half product only when every right-hand side of the CTA passed the test
        bool h = flip.part != nullptr;
        for (int v = 0; v < NV && h; ++v)
            if (b0 + v < ninst) h = flip_half(flip, b0 + v);
        if (threadIdx.x == 0) {
            s_half = h;
            if (NV == 1 && flip.used && blockIdx.x == 0) flip.used[b0] = h;
        }
    }
    const double *vt = m.vtab + (size_t)b0 * m.vtab_inst;
    for (int64_t i = threadIdx.x; i < m.vtab_len; i += blockDim.x) tab[i] = vt[i];
    __syncthreads();
    const bool half = s_half;
    const int32_t *colE = m.colE + (size_t)b0 * m.inst_e, *colD = m.colD + (size_t)b0 * m.inst_d;
    const double *valE = m.valE + (size_t)b0 * m.inst_e;
    const uint16_t *codeD = m.codeD + (size_t)b0 * m.inst_d;
    constexpr int RPW = 32 / T;
    const int lane = threadIdx.x & 31, sub = lane / RPW;
    const int64_t rows_per_iter = kVellThreads / T;
    // units: rows (full product) or the rows of the listed slabs (half product)
    const int64_t nunits = half ? flip.nslabs * 32 : D;
    const int64_t share = ((nunits + gridDim.x - 1) / gridDim.x + 31) & ~(int64_t)31;
    const int64_t u_lo = (int64_t)blockIdx.x * share, u_hi = u_lo + share < nunits ? u_lo + share : nunits;
    double e = 0.0;
    for (int64_t ub = u_lo; ub < u_hi; ub += rows_per_iter) {
        const int64_t uu = ub + (threadIdx.x - lane) / T + lane % RPW;
        int64_t r = D, rf = -1;  // r = D: no row; rf >= 0: the mirror row also gets the result
        if (uu < u_hi) {
            if (!half) {
                r = uu;
            } else {
                const int64_t rr = (int64_t)flip.slabs[uu >> 5] * 32 + (uu & 31);
                if (rr < D) {
                    const uint32_t a = flip.alpha_of((uint32_t)rr), b = (uint32_t)rr - a * flip.nB;
                    if (a <= b) r = rr;
                    if (a < b) rf = (int64_t)b * flip.nB + a;
                }
            }
        }
        double acc[NV][W][2];
#pragma unroll
        for (int v = 0; v < NV; ++v)
#pragma unroll
            for (int w = 0; w < W; ++w) acc[v][w][0] = acc[v][w][1] = 0.0;
        if (r < D) {
            {
                const size_t base = ell_pos(r, 0, m.qe);
                const int4 *c4 = reinterpret_cast<const int4 *>(colE + base);
                const double2 *v2 = reinterpret_cast<const double2 *>(valE + base);
                for (int64_t g = sub; g < m.qe; g += T) {
                    const int4 c = __ldg(c4 + 32 * g);
                    const double2 h01 = __ldg(v2 + 64 * g), h23 = __ldg(v2 + 64 * g + 1);
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        const double *xv = x + (size_t)(b0 + v < ninst ? b0 + v : b0) * D * W;
#pragma unroll
                        for (int w = 0; w < W; ++w) {
                            acc[v][w][0] = fma(h01.x, __ldg(xv + (size_t)c.x * W + w), acc[v][w][0]);
                            acc[v][w][1] = fma(h01.y, __ldg(xv + (size_t)c.y * W + w), acc[v][w][1]);
                            acc[v][w][0] = fma(h23.x, __ldg(xv + (size_t)c.z * W + w), acc[v][w][0]);
                            acc[v][w][1] = fma(h23.y, __ldg(xv + (size_t)c.w * W + w), acc[v][w][1]);
                        }
                    }
                }
            }
            {
                const size_t base = ell_pos(r, 0, m.qd);
                const int4 *c4 = reinterpret_cast<const int4 *>(colD + base);
                const uint2 *k2 = reinterpret_cast<const uint2 *>(codeD + base);
#pragma unroll 2
                for (int64_t g = sub; g < m.qd; g += T) {
                    const int4 c = __ldg(c4 + 32 * g);
                    const uint2 k = __ldg(k2 + 32 * g);
                    const double h0 = signed_value(tab, k.x & 0xffffu), h1 = signed_value(tab, k.x >> 16);
                    const double h2 = signed_value(tab, k.y & 0xffffu), h3 = signed_value(tab, k.y >> 16);
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        const double *xv = x + (size_t)(b0 + v < ninst ? b0 + v : b0) * D * W;
#pragma unroll
                        for (int w = 0; w < W; ++w) {
                            acc[v][w][0] = fma(h0, __ldg(xv + (size_t)c.x * W + w), acc[v][w][0]);
                            acc[v][w][1] = fma(h1, __ldg(xv + (size_t)c.y * W + w), acc[v][w][1]);
                            acc[v][w][0] = fma(h2, __ldg(xv + (size_t)c.z * W + w), acc[v][w][0]);
                            acc[v][w][1] = fma(h3, __ldg(xv + (size_t)c.w * W + w), acc[v][w][1]);
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            if (b0 + v >= ninst) continue;
            double *yv = y + (size_t)(b0 + v) * D * W;
            const double *xv = x + (size_t)(b0 + v) * D * W;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                double s = acc[v][w][0] + acc[v][w][1];
#pragma unroll
                for (int o = RPW; o < 32; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (r < D && sub == 0) {
                    yv[r * W + w] = s;
                    if (NV == 1) e = fma(s, xv[r * W + w], e);
                    if (rf >= 0) {
                        yv[rf * W + w] = s;
                        if (NV == 1) e = fma(s, xv[rf * W + w], e);
                    }
                }
            }
        }
    }
    if (NV == 1 && epart) {
        e = block_sum(e, red);
        if (threadIdx.x == 0) epart[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = e;
    }
}

// Diagonal of H, one thread per determinant (setup of the on-the-fly path).
__global__ void k_diag_build(IntArgs a, double *__restrict__ diag)
{
    const int64_t D = (int64_t)a.basis.D;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < D; r += (int64_t)gridDim.x * blockDim.x)
        diag[r] = diag_val(a, a.basis.bits((uint32_t)r));
}

// ------------------------------------------------- H * psi on the fly (strings) --
// One CTA per (alpha string, chunk of beta strings), one thread per determinant.
// Every matrix element costs one FP64 FMA: the alpha string's excitation lists,
// their values and the alpha-beta integral slices of its singles sit in shared
// memory; the beta string's lists come from the precomputed tables (otf_tables.cpp).
// x reads: alpha excitations hit contiguous rows of x across the CTA (coalesced),
// beta excitations stay inside the CTA's own row of x.  Fused with <x|y>.
struct OtfArgs {
    int N, P2, nA, nB;
    int nsa, nda, nsb, ndb;
    const int32_t *sa_rank, *sa_code, *da_rank, *da_code;
    const int32_t *sb_rank, *sb_code, *db_rank, *db_code;
    // integral-dependent tables of instance 0; instance b at + b * (its size), or
    // shared by every instance when `shared` is set
    const double *vss, *vab, *a_alpha, *b_alpha, *a_beta, *b_beta, *diag;
    int shared;
    const int *active;  // instance mask (nullable)
};

__host__ __device__ inline size_t otf_smem_bytes(int N, int P2, int nsa, int nda)
{
    return sizeof(double) * ((size_t)P2 * P2 + (size_t)nsa * N * N + nsa + nda) + sizeof(int32_t) * (2 * (size_t)nsa + nda);
}

__device__ __forceinline__ double flipc(double v, int32_t code)
{
    return __longlong_as_double(__double_as_longlong(v) ^ ((unsigned long long)((uint32_t)code >> 31) << 63));
}

// Half product (flip.part set and the instance's input flip-invariant): only the
// determinants with beta string rb >= ra, each result also written to its mirror
// (rb, ra); a CTA whose beta strings all lie below ra writes a zero energy partial.
template <int W>
__global__ void __launch_bounds__(1024) k_otf_strings(OtfArgs a, const double *__restrict__ x, double *__restrict__ y,
                                                      double *__restrict__ epart, FlipArgs flip)
{
    extern __shared__ double sm[];
    __shared__ double red[32];
    __shared__ int s_half;
    const int N = a.N, NN = a.N * a.N, nsa = a.nsa, nda = a.nda;
    const int ra = blockIdx.x;
    if (skip_instance(a.active, blockIdx.z)) return;
    if (threadIdx.x < 32) {
        const bool h = flip_half(flip, blockIdx.z);
        if (threadIdx.x == 0) {
            s_half = h;
            if (flip.used && blockIdx.x == 0 && blockIdx.y == 0) flip.used[blockIdx.z] = h;
        }
    }
    __syncthreads();
    const bool half = s_half;
    if (half && (int64_t)(blockIdx.y + 1) * blockDim.x <= ra) {
        if (threadIdx.x == 0 && epart)
            epart[(size_t)blockIdx.z * gridDim.x * gridDim.y + (size_t)blockIdx.y * gridDim.x + blockIdx.x] = 0.0;
        return;
    }
    {
        // instance blockIdx.z: its vectors and (unless shared) its integral tables
        const size_t b = blockIdx.z, D = (size_t)a.nA * a.nB, bt = a.shared ? 0 : b;
        x += b * D * W;
        y += b * D * W;
        if (epart) epart += b * gridDim.x * gridDim.y;
        a.vss += bt * a.P2 * a.P2;
        a.vab += bt * NN * NN;
        a.a_alpha += bt * a.nA * NN;
        a.b_alpha += bt * a.nB * NN;
        a.a_beta += bt * a.nB * NN;
        a.b_beta += bt * a.nA * NN;
        a.diag += bt * D;
    }
    double *vss = sm;
    double *vsl = vss + (size_t)a.P2 * a.P2;
    double *sa_val = vsl + (size_t)nsa * NN;
    double *da_val = sa_val + nsa;
    int32_t *sa_rank = (int32_t *)(da_val + nda);
    int32_t *sa_code = sa_rank + nsa;
    int32_t *da_rank = sa_code + nsa;
    for (int i = threadIdx.x; i < a.P2 * a.P2; i += blockDim.x) vss[i] = a.vss[i];
    for (int i = threadIdx.x; i < nsa; i += blockDim.x) {
        const int32_t code = a.sa_code[(size_t)ra * nsa + i];
        sa_rank[i] = a.sa_rank[(size_t)ra * nsa + i];
        sa_code[i] = code;
        sa_val[i] = a.a_alpha[(size_t)ra * NN + (code & 31) * N + ((code >> 5) & 31)];
    }
    for (int i = threadIdx.x; i < nsa * NN; i += blockDim.x) {
        const int sidx = i / NN, k = i - sidx * NN;
        const int32_t code = a.sa_code[(size_t)ra * nsa + sidx];
        vsl[i] = a.vab[((size_t)((code & 31) * N + ((code >> 5) & 31))) * NN + k];
    }
    for (int i = threadIdx.x; i < nda; i += blockDim.x) {
        const int32_t code = a.da_code[(size_t)ra * nda + i];
        da_rank[i] = a.da_rank[(size_t)ra * nda + i];
        da_val[i] = flipc(a.vss[code & 0x7fffffff], code);
    }
    __syncthreads();
    const int nB = a.nB;
    const int rb = blockIdx.y * blockDim.x + threadIdx.x;
    double en = 0;
    if (rb < nB && (!half || rb >= ra)) {
        const size_t row = (size_t)ra * nB + rb;
        const double dg = a.diag[row];
        double acc[W];
#pragma unroll
        for (int w = 0; w < W; ++w) acc[w] = dg * x[row * W + w];
        // alpha singles: sign * (A_alpha[ra] + B_alpha[rb])
        const double *bal = a.b_alpha + (size_t)rb * NN;
        for (int s = 0; s < nsa; ++s) {
            const int32_t code = sa_code[s];
            const double v = flipc(sa_val[s] + bal[(code & 31) * N + ((code >> 5) & 31)], code);
            const size_t c = (size_t)sa_rank[s] * nB + rb;
#pragma unroll
            for (int w = 0; w < W; ++w) acc[w] = fma(v, x[c * W + w], acc[w]);
        }
        // alpha-alpha doubles
        for (int d = 0; d < nda; ++d) {
            const size_t c = (size_t)da_rank[d] * nB + rb;
#pragma unroll
            for (int w = 0; w < W; ++w) acc[w] = fma(da_val[d], x[c * W + w], acc[w]);
        }
        const size_t rowA = (size_t)ra * nB;
        const int32_t *sbr = a.sb_rank + (size_t)rb * a.nsb, *sbc = a.sb_code + (size_t)rb * a.nsb;
        const double *abe = a.a_beta + (size_t)rb * NN, *bbe = a.b_beta + (size_t)ra * NN;
        // beta singles: sign * (A_beta[rb] + B_beta[ra])
        for (int t = 0; t < a.nsb; ++t) {
            const int32_t code = sbc[t];
            const int k = (code & 31) * N + ((code >> 5) & 31);
            const double v = flipc(abe[k] + bbe[k], code);
            const size_t c = rowA + sbr[t];
#pragma unroll
            for (int w = 0; w < W; ++w) acc[w] = fma(v, x[c * W + w], acc[w]);
        }
        // beta-beta doubles
        const int32_t *dbr = a.db_rank + (size_t)rb * a.ndb, *dbc = a.db_code + (size_t)rb * a.ndb;
        for (int d = 0; d < a.ndb; ++d) {
            const int32_t code = dbc[d];
            const double v = flipc(vss[code & 0x7fffffff], code);
            const size_t c = rowA + dbr[d];
#pragma unroll
            for (int w = 0; w < W; ++w) acc[w] = fma(v, x[c * W + w], acc[w]);
        }
        // alpha-beta doubles: (pa ra|pb rb), sign = product of the two single signs
        for (int t = 0; t < a.nsb; ++t) {
            const int32_t tc = sbc[t];
            const int kb = (tc & 31) * N + ((tc >> 5) & 31);
            const size_t ct = (size_t)sbr[t];
#pragma unroll 4
            for (int s = 0; s < nsa; ++s) {
                const double v = flipc(vsl[s * NN + kb], sa_code[s] ^ tc);
                const size_t c = (size_t)sa_rank[s] * nB + ct;
#pragma unroll
                for (int w = 0; w < W; ++w) acc[w] = fma(v, x[c * W + w], acc[w]);
            }
        }
        const size_t mir = (size_t)rb * nB + ra;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            y[row * W + w] = acc[w];
            en = fma(acc[w], x[row * W + w], en);
            if (half && rb > ra) {
                y[mir * W + w] = acc[w];
                en = fma(acc[w], x[mir * W + w], en);
            }
        }
    }
    en = block_sum(en, red);
    if (threadIdx.x == 0 && epart) epart[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = en;
}

// ------------------------------------------------------------------ host --
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    ~DevBuf() { reset(); }
    void reset()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

}  // namespace

struct aegpu_engine {
    std::string err;
    int64_t dev_bytes = 0;
    bool alloc_failed = false;  // a set-up allocation failed (checked at the end of set-up)
    int64_t launches = 0;
    cudaStream_t stream = nullptr;
    int sm_count = 152;
    int smem_per_sm = 228 * 1024;

    Basis B;
    bool cplx = false;
    int W = 1;
    std::vector<Exc> excs;
    std::vector<ExcCode> codes;
    std::vector<Block> blocks;
    std::vector<int> perm;        // application order of the operators
    std::vector<int> pos_of_op;   // inverse of perm
    std::vector<int> block_pos0;  // first application position of every block
    std::vector<int> op_block, op_slot;

    struct DevBlock {
        bool diagonal = false;
        int nslots = 0;
        int ntiles = 0;           // shared-memory tiles (multi-vector Hessian kernels)
        int nwtasks = 0;          // warp tasks (evolve / adjoint kernels)
        int wgrid = 0;            // CTAs of the warp kernels; also partial-sum rows
        int rgrid = 0;            // CTAs of the forward warp kernel (as many as stay resident)
        WarpTask *wtasks = nullptr;
        int64_t part_off = 0;     // offset of this block's gradient partials
        int64_t ckpt_off = 0;     // offset (doubles) of this pass's checkpoint
        uint32_t *idx = nullptr, *bits = nullptr;
        OrbitGroup *groups = nullptr;
        OrbitTile *tiles = nullptr;
        int *ops = nullptr;
        uint64_t active = 0;
        uint64_t amp_layers = 0;  // touched amplitudes x their active layers
        // diagonal passes: phase-table offset (doubles, per instance), Sz-basis slot
        // masks of the alpha / beta strings (null in other bases), and the slot
        // activations summed over the determinants (FP64 work accounting)
        int64_t tab_off = 0;
        uint16_t *smA = nullptr, *smB = nullptr;
        uint64_t slot_acts = 0;
        DiagSplit split{};        // Sz basis: launch shape and slot classes of k_diag_adj_sz
        // spin-flip half tables (paired passes; build_half_orbits)
        uint32_t *idx_h = nullptr, *bits_h = nullptr;
        WarpTask *wtasks_h = nullptr;
        int nwtasks_h = 0;
        uint64_t active_h = 0, amp_layers_h = 0;
        // diagonal passes as half passes: the amplitudes (a, b) with a <= b that hold an
        // active slot, and their slot activations (FP64 work accounting)
        uint64_t slot_acts_h = 0;
    };
    std::vector<DevBlock> dblocks;
    std::vector<void *> allocs;

    // device basis
    DevBasis db{};
    // device arrays
    ExcCode *d_codes = nullptr;
    int *d_tpos = nullptr;          // op -> tangent slot (application position)
    int *d_pos_op = nullptr;        // application position -> op
    int64_t *d_op_part_off = nullptr;
    int *d_op_ntiles = nullptr, *d_op_slot = nullptr;
    PrepArgs prep{};                // pass lists for k_pass_prep
    double *d_start = nullptr;      // start vector, shared by every instance
    int64_t n_partials = 0;         // gradient partial sums per instance
    int64_t n_ckpt = 0;             // checkpoint doubles per instance
    int64_t n_diag_tab = 0;         // phase-table doubles of the diagonal passes per instance
    // spin-flip half passes: possible for this problem (Sz basis, as many alpha as beta
    // strings, no diagonal passes, every pass closed under the mirror with matching
    // signs), the start state symmetric, the knob (AEGPU_TUNE_HALF; AEGPU_HALF=0 in the
    // environment switches it off); the device gate is their conjunction, the
    // per-instance flag adds the angle test of each evaluation
    bool half_static = false, start_sym = true, tune_half = true;
    int task_order = 1;  // warp-major where a launch fits one wave (order_for; AEGPU_TASK_ORDER=0: never)
    int rot_occ = 0, adj_occ = 0;  // resident CTAs per SM of k_warp_rot / k_warp_adj
    std::vector<int> mirror;        // operator -> mirror operator (half passes only)
    int *d_mirror = nullptr, *d_half_gate = nullptr;
    int *d_half = nullptr;          // per instance (alloc_instances)
    int64_t n_epart = 0;            // H psi partial sums per instance
    int spmv_grid = 0;

    // Per-instance buffers, instance b at b * (per-instance size).  An engine evaluates
    // nb instances per call: nb angle vectors over one problem, with one shared
    // Hamiltonian or one Hamiltonian per instance.
    int nb = 1;
    double *d_ang = nullptr, *d_sc = nullptr, *d_diag_table = nullptr, *d_sig = nullptr;
    PassConst *d_pc = nullptr;
    double *d_psi = nullptr, *d_h = nullptr, *d_tmp = nullptr;
    double *d_partials = nullptr, *d_epart = nullptr, *d_scalar = nullptr, *d_grad = nullptr;
    double *d_flip_part = nullptr;  // per instance, sm_count pairs of the invariance test
    int *d_flip_used = nullptr;     // per instance, the last energy product's choice
    bool flip_tried = false;        // the last energy product ran the invariance test
    double *d_ckpt = nullptr;  // per pass: amplitudes after the pass (adjoint sweep input)
    int *d_active = nullptr;   // per instance: 0 = skip it in batched launches
    std::vector<std::pair<void *, size_t>> inst_allocs;

    // Hamiltonian (its device arrays, released when it is replaced)
    std::vector<void *> ham_allocs;
    std::unordered_map<void *, size_t> ham_alloc_bytes;
    int ham_kind = 0;  // 1 CSR, 2 ELL, 3 on the fly
    bool ham_per_instance = false;
    int64_t ham_entries = 0;
    int64_t ell_stride_inst = 0;  // doubles between instances' stored matrices (0 = shared)
    int64_t *d_rowptr = nullptr;
    int32_t *d_col = nullptr;
    double *d_val = nullptr;
    // coded stored rows (k_vell_build; used when the value table fits, N <= 12)
    bool ell_coded = false;
    VellArgs vell{};
    IntArgs ints{};
    double *d_h1 = nullptr, *d_g2 = nullptr;
    int ell_width = 0;
    OtfArgs otf{};
    int otf_threads = 0, otf_chunks = 0;

    // launch-shape knobs (aegpu_set_tuning): excitations per pass (<= kMaxWarpLayers),
    // CTAs per SM of the pass kernels, threads per CTA of the on-the-fly H kernel
    int tune_pass_ops = kMaxWarpLayers;
    int tune_ctas_per_sm = 4;  // best single-instance shape at 10-12 orbitals on GB300
    int tune_otf_threads = 512;
    bool otf_threads_set = false;  // set through the knob: no automatic CTA size
    int tune_spmv_tpr = 0;  // threads per stored-H row: 0 = by size (>= 4 CTAs per SM)
    // programmatic dependent launch of the pass kernels: -1 = by size (on up to 2^19
    // amplitudes per launch, where launch latency is a visible share of a pass; off
    // above, where early-resident dependents slow the FP64-bound passes: GB300,
    // 8 / 10 orbitals -6 %, 12 orbitals (853,776 amplitudes) +1.7 %)
    int tune_pdl = -1;
    // keep H psi between an energy and a gradient at the same angles (AEGPU_REUSE_HPSI=0
    // in the environment, or the knob, makes the gradient recompute it)
    bool reuse_hpsi = true;
    // spin-flip half product of the energy's H psi (knob AEGPU_TUNE_FLIP, environment
    // AEGPU_FLIP=0 to switch it off); possible for integral Hamiltonians in the Sz
    // basis with as many alpha as beta electrons (flip_ok), taken per evaluation when
    // the state passes the device test
    bool tune_flip = true;
    bool flip_ok = false;
    int32_t *d_flip_slabs = nullptr;  // coded rows: slabs holding a row with a <= b
    int64_t n_flip_slabs = 0;
    bool pdl_on() const { return tune_pdl >= 0 ? tune_pdl != 0 : (int64_t)B.D * W * nb <= (int64_t)1 << 19; }
    int spmv_tpr() const
    {
        if (tune_spmv_tpr) return tune_spmv_tpr;
        int t = 1;
        while (t < 8 && (int64_t)B.D * t < (int64_t)sm_count * 4 * kSpmvThreads) t *= 2;
        return t;
    }

    // optional CUDA-event timing of the phases of *_dev evaluations
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::array<cudaEvent_t, 4>> ev_marks;
    double phase_ms[3] = {0, 0, 0};
    int64_t phase_n = 0;
    cudaEvent_t next_event()
    {
        cudaEvent_t ev;
        if (!ev_pool.empty()) {
            ev = ev_pool.back();
            ev_pool.pop_back();
        } else {
            cudaEventCreate(&ev);
        }
        return ev;
    }

    // CUDA graph of one energy + gradient evaluation (angles from d_ang, results in
    // d_scalar / d_grad), captured on first use of aegpu_gradient_dev
    cudaGraphExec_t grad_graph = nullptr;
    cudaGraph_t grad_graph_def = nullptr;  // its definition (child node of group graphs)
    // the same evaluation split in two (host-buffer calls): pass constants + evolve +
    // H psi + energy, and the adjoint sweep + gradient reduction
    cudaGraphExec_t energy_graph = nullptr, back_graph = nullptr;
    int64_t energy_graph_launches = 0, back_graph_launches = 0;
    int64_t graph_launches = 0;  // kernels inside the graph
    int64_t generation = 0;      // bumped whenever device buffers or the Hamiltonian's buffers change
    int ints_ntab = 0, ints_mode_asked = -1;  // shape of the current integral Hamiltonian
    bool use_graph = true;

    // Hessian scratch, kept between calls with the same parameter count
    struct HessScratch {
        int V = 0;
        double *T = nullptr, *TC = nullptr, *HTC = nullptr, *THT = nullptr, *Hops = nullptr, *hpart = nullptr;
        double *MET = nullptr;  // metric of the compressed tangents
        double *gram = nullptr; // partial sums of the Gram / projection contractions
        int *pptr = nullptr, *ppos = nullptr;
        double *pscale = nullptr;
        double *flip = nullptr;  // invariance-test partials of the V columns
        int *vmap = nullptr, *mpos = nullptr;  // half tangents: carried positions, mirror reads
        std::vector<std::pair<void *, size_t>> allocs;
    } hess;

    // lowest eigenpair of H (aegpu_lowest_eigenpair), valid until H is replaced
    double *d_ground = nullptr;
    int n_ground = 0;       // columns allocated in d_ground
    int ground_states = 0;  // eigenpairs held there
    // scalar results and dot-product partial sums of the properties pass
    double *d_small = nullptr;
    size_t small_len() const { return 8 + 16 * (size_t)sm_count; }
    double ground_value = 0.0;
    bool ground_valid = false;

    // state caching: psi / hpsi valid for these angles
    std::vector<double> cached_angles;
    bool psi_valid = false, h_valid = false;

    ~aegpu_engine()
    {
        for (void *p : allocs) cudaFree(p);
        for (auto &m : ev_marks)
            for (auto ev : m) cudaEventDestroy(ev);
        for (auto ev : ev_pool) cudaEventDestroy(ev);
        drop_graph();
        if (stream) cudaStreamDestroy(stream);
    }

    template <typename T>
    T *alloc(size_t n)
    {
        void *p = nullptr;
        if (n == 0) n = 1;
        if (g_fail_alloc_after.load() >= 0 && g_fail_alloc_after.fetch_sub(1) <= 0) {
            g_fail_alloc_after.store(0);
            alloc_failed = true;
            return nullptr;
        }
        cudaError_t rc = cudaMalloc(&p, n * sizeof(T));
        if (rc != cudaSuccess) {
            cudaGetLastError();
            alloc_failed = true;
            return nullptr;
        }
        allocs.push_back(p);
        dev_bytes += (int64_t)(n * sizeof(T));
        return (T *)p;
    }
    void release(void *p, size_t bytes)
    {
        if (!p) return;
        auto it = std::find(allocs.begin(), allocs.end(), p);
        if (it != allocs.end()) allocs.erase(it);
        cudaFree(p);
        dev_bytes -= (int64_t)bytes;
    }
    int fail(int code, const std::string &m)
    {
        err = m;
        return code;
    }
    int cuda_check(const char *where)
    {
        cudaError_t rc = cudaGetLastError();
        if (rc != cudaSuccess) return fail(AEGPU_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(rc));
        return AEGPU_OK;
    }
    template <typename T>
    T *upload(const std::vector<T> &v)
    {
        T *p = alloc<T>(v.size());
        if (p && !v.empty()) cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
        return p;
    }

    // Arguments of pass bi in direction dir (+1 forward, -1 adjoint); half: the
    // instances may take the spin-flip half tables (evolution and energy gradient).
    BlockArgs block_args(int bi, double dir, bool half = false) const
    {
        const DevBlock &b = dblocks[bi];
        const int d = dir > 0 ? 0 : 1;
        const int npass = (int)dblocks.size();
        BlockArgs a;
        a.idx = b.idx;
        a.obits = b.bits;
        a.groups = b.groups;
        a.tiles = b.tiles;
        a.ops = b.ops;
        a.nslots = b.nslots;
        a.codes = d_codes;
        a.sc = d_sc;
        a.dir = dir;
        a.basis = db;
        a.pc = d_pc + ((size_t)bi * 2 + d) * kMaxWarpLayers;
        a.sigma = d_sig + ((size_t)bi * 2 + d) * (1 << kMaxWarpLayers);
        a.pc_stride = (int64_t)npass * 2 * kMaxWarpLayers;
        a.sig_stride = (int64_t)npass * 2 * (1 << kMaxWarpLayers);
        a.active = d_active;
        a.half = half && half_static ? d_half : nullptr;
        a.idx_h = b.idx_h;
        a.obits_h = b.bits_h;
        a.tasks_h = b.wtasks_h;
        a.ntasks_h = b.nwtasks_h;
        a.vmap = nullptr;
        a.task_order = 0;
        return a;
    }
    // Task order of a warp-kernel launch of grid g with occ resident CTAs per SM:
    // warp-major when every CTA is resident at once (one wave; the single-instance
    // sweeps), else CTA-major -- with several waves the CTA scheduler balances the SMs
    // itself, and consecutive tasks in one CTA share cached table and amplitude lines.
    int order_for(dim3 g, int occ) const
    {
        return task_order && (int64_t)g.x * g.y * g.z <= (int64_t)sm_count * occ ? 1 : 0;
    }
    // Device gate of the half passes: the tables are built, the start state is
    // symmetric and the knob is on.
    void write_half_gate();  // in order on the engine's stream (k_set_int)
    size_t vec_elems() const { return (size_t)B.D * W; }

    template <typename T>
    T *ham_alloc(size_t n)
    {
        T *p = alloc<T>(n);
        if (p) {
            ham_allocs.push_back((void *)p);
            ham_alloc_bytes[(void *)p] = std::max<size_t>(n, 1) * sizeof(T);
        }
        return p;
    }
    // Release the current Hamiltonian (and the graph that reads it).
    void drop_ham()
    {
        for (void *p : ham_allocs) release(p, ham_alloc_bytes[p]);
        ham_allocs.clear();
        ham_alloc_bytes.clear();
        ham_kind = 0;
        ints_ntab = 0;
        ints_mode_asked = -1;
        ham_per_instance = false;
        ell_stride_inst = 0;
        d_rowptr = nullptr;
        d_col = nullptr;
        d_val = nullptr;
        ell_coded = false;
        vell = VellArgs{};
        d_h1 = d_g2 = nullptr;
        flip_ok = false;
        d_flip_slabs = nullptr;
        n_flip_slabs = 0;
        drop_graph();
        h_valid = false;
        ground_valid = false;
    }
    void drop_graph()
    {
        ++generation;
        if (grad_graph) cudaGraphExecDestroy(grad_graph);
        if (grad_graph_def) cudaGraphDestroy(grad_graph_def);
        if (energy_graph) cudaGraphExecDestroy(energy_graph);
        if (back_graph) cudaGraphExecDestroy(back_graph);
        grad_graph = nullptr;
        grad_graph_def = nullptr;
        energy_graph = back_graph = nullptr;
    }

    // (Re)allocate the per-instance buffers for nb instances.
    int alloc_instances(int n_inst)
    {
        for (auto &pa : inst_allocs) release(pa.first, pa.second);
        inst_allocs.clear();
        nb = n_inst;
        const size_t nops = excs.size(), npass = dblocks.size(), n = vec_elems(), B_ = (size_t)nb;
        bool ok = true;
        auto get = [&](auto *&ptr, size_t count) {
            using T = std::remove_reference_t<decltype(*ptr)>;
            ptr = alloc<T>(count);
            ok = ok && ptr;
            inst_allocs.push_back({(void *)ptr, std::max<size_t>(count, 1) * sizeof(T)});
        };
        get(d_ang, B_ * nops);
        get(d_sc, B_ * 2 * nops);
        get(d_pc, B_ * npass * 2 * kMaxWarpLayers);
        get(d_sig, B_ * npass * 2 * (1 << kMaxWarpLayers));
        get(d_diag_table, B_ * std::max<int64_t>(n_diag_tab, 1));
        get(d_psi, B_ * n);
        get(d_h, B_ * n);
        get(d_tmp, B_ * n);
        get(d_partials, B_ * std::max<int64_t>(n_partials, 1));
        get(d_epart, B_ * std::max<int64_t>(n_epart, 1));
        get(d_flip_part, B_ * 2 * (size_t)sm_count);
        get(d_flip_used, B_);
        get(d_half, B_);
        if (d_half) cudaMemset(d_half, 0, B_ * sizeof(int));
        flip_tried = false;
        get(d_scalar, std::max<size_t>(B_, 4));
        get(d_grad, B_ * nops);
        get(d_ckpt, B_ * std::max<int64_t>(n_ckpt, 1));
        get(d_active, B_);
        if (d_active) {
            const std::vector<int> ones(B_, 1);
            cudaMemcpy(d_active, ones.data(), B_ * sizeof(int), cudaMemcpyHostToDevice);
        }
        prep.active = d_active;
        prep.half = half_static ? d_half : nullptr;
        drop_graph();
        cached_angles.clear();
        psi_valid = h_valid = false;
        if (!ok) return fail(AEGPU_ERR_NOMEM, "device allocation of the instance buffers failed");
        return AEGPU_OK;
    }
    // Arguments of diagonal pass b in direction dir (+1 forward, -1 adjoint).
    DiagArgs diag_args(const DevBlock &b, double dir, bool masked = true, bool half = false) const
    {
        DiagArgs a;
        a.active = masked ? d_active : nullptr;
        a.half = half && half_static ? d_half : nullptr;
        a.ops = b.ops;
        a.nslots = b.nslots;
        a.codes = d_codes;
        a.table = d_diag_table + b.tab_off;
        a.tab_stride = n_diag_tab;
        a.sin_flip = dir > 0 ? 0ull : 1ull << 63;
        a.smA = b.smA;
        a.smB = b.smB;
        a.basis = db;
        return a;
    }
    size_t rot_smem(int nvec_tiles) const { return (size_t)kTileElems * (nvec_tiles * W * 8 + 4); }
};

namespace {

template <typename K>
int set_smem(K kernel, size_t need, int optin)
{
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    if (need + fa.sharedSizeBytes > (size_t)optin) return 1;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return 0;
}

// Opt the tile kernels into the shared memory they use (1, 2 or 3 staged vectors of
// kTileElems amplitudes plus the bitstrings), within the device's per-block limit.
int set_smem_limits(int dev)
{
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    auto need = [](int nv, int W) { return (size_t)kTileElems * (nv * W * 8 + 4); };
    int bad = 0;
    bad += set_smem(k_block_tangent<1>, need(1, 1), optin);
    bad += set_smem(k_block_tangent<2>, need(1, 2), optin);
    // the coded-row product stages its value table (<= 196 KB at 12 orbitals): allow the most
    {
        const void *kerns[] = {(const void *)k_spmv_vell<1, 1, 1>, (const void *)k_spmv_vell<1, 2, 1>,
                               (const void *)k_spmv_vell<1, 4, 1>, (const void *)k_spmv_vell<1, 8, 1>,
                               (const void *)k_spmv_vell<2, 1, 1>, (const void *)k_spmv_vell<2, 2, 1>,
                               (const void *)k_spmv_vell<2, 4, 1>, (const void *)k_spmv_vell<2, 8, 1>,
                               (const void *)k_spmv_vell<1, 1, kVellNV1>, (const void *)k_spmv_vell<1, 2, kVellNV1>,
                               (const void *)k_spmv_vell<1, 4, kVellNV1>, (const void *)k_spmv_vell<1, 8, kVellNV1>,
                               (const void *)k_spmv_vell<2, 1, kVellNV2>, (const void *)k_spmv_vell<2, 2, kVellNV2>,
                               (const void *)k_spmv_vell<2, 4, kVellNV2>, (const void *)k_spmv_vell<2, 8, kVellNV2>};
        for (const void *kern : kerns) {
            cudaFuncAttributes fa{};
            if (cudaFuncGetAttributes(&fa, kern) == cudaSuccess)
                cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
        }
    }
    // the on-the-fly kernel's need depends on N (<= 150 KB at 14 orbitals): allow the most
    for (int W = 1; W <= 2; ++W) {
        cudaFuncAttributes fa{};
        auto kern = W == 1 ? (const void *)k_otf_strings<1> : (const void *)k_otf_strings<2>;
        if (cudaFuncGetAttributes(&fa, kern) == cudaSuccess)
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    }
    cudaGetLastError();
    return bad;
}

// Forward evolution of the first ninst instances from the start vector (pass
// constants already prepared from d_ang).
// Launch of a pass kernel, with the programmatic-serialisation attribute when the PDL
// knob is on (captured graphs keep it as a programmatic edge).
template <typename... KArgs, typename... Args>
void launch_pass(const aegpu_engine *e, void (*kernel)(KArgs...), dim3 grid, Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(kWarpThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = e->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = e->pdl_on() ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

int run_evolve(aegpu_engine *e, int ninst)
{
    NvtxRange r("aegpu evolve");
    const int64_t n = (int64_t)e->vec_elems();
    k_broadcast<<<dim3((unsigned)std::min<int64_t>((n + 255) / 256, e->sm_count * 4), ninst), 256, 0, e->stream>>>(
        e->d_start, e->d_psi, n, e->d_active);
    e->launches += 1;
    for (int bi = 0; bi < (int)e->dblocks.size(); ++bi) {
        auto &b = e->dblocks[bi];
        double *ck = e->d_ckpt + b.ckpt_off;
        if (b.diagonal) {
            k_diag_rot<<<dim3(kDiagGrid, ninst), 256, 0, e->stream>>>(e->diag_args(b, 1.0, true, true), e->d_psi, 0,
                                                                       1, ck, n, e->n_ckpt);
            e->launches += 1;
        } else if (b.nwtasks) {
            BlockArgs a = e->block_args(bi, 1.0, true);
            const dim3 g(b.rgrid, ninst);
            a.task_order = e->order_for(g, e->rot_occ);
            if (e->W == 1)
                launch_pass(e, k_warp_rot<1>, g, a, (const WarpTask *)b.wtasks, b.nwtasks, e->d_psi, n, ck, e->n_ckpt);
            else
                launch_pass(e, k_warp_rot<2>, g, a, (const WarpTask *)b.wtasks, b.nwtasks, e->d_psi, n, ck, e->n_ckpt);
            e->launches += 1;
        }
    }
    if (e->half_static) {
        // instances that took the half passes: complete psi from its a <= b amplitudes
        const dim3 g((unsigned)std::min<int64_t>(((int64_t)e->B.D + 255) / 256, e->sm_count * 4), ninst);
        if (e->W == 1)
            k_flip_fill<1><<<g, 256, 0, e->stream>>>(e->db, e->d_psi, n, e->d_half, e->d_active);
        else
            k_flip_fill<2><<<g, 256, 0, e->stream>>>(e->db, e->d_psi, n, e->d_half, e->d_active);
        e->launches += 1;
    }
    return e->cuda_check("evolve");
}

// Pass constants of the first ninst instances from their angles in d_ang.
int run_prep(aegpu_engine *e, int ninst, bool masked = true)
{
    PrepArgs pa = e->prep;
    pa.active = masked ? e->d_active : nullptr;
    k_pass_prep<<<dim3((unsigned)e->dblocks.size(), ninst), 64, 0, e->stream>>>(pa, e->d_ang, e->d_sc, e->d_pc,
                                                                             e->d_sig, e->d_diag_table);
    e->launches += 1;
    return e->cuda_check("pass constants");
}

int upload_angles(aegpu_engine *e, const double *angles, bool host, int ninst, bool masked = true)
{
    const size_t n = e->excs.size() * (size_t)ninst;
    cudaMemcpyAsync(e->d_ang, angles, n * sizeof(double), host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                    e->stream);
    return run_prep(e, ninst, masked);
}

// y = H x for the first ninst instances (vectors at stride D*W), with <x|y> partial
// sums into epart (nullable; *nparts partial sums per instance).
// flip: try the spin-flip half product, with the invariance test's partials in
// flip_part (2 * sm_count doubles per instance) and the per-instance choice recorded in
// flip_used (nullable; the energy evaluation's record for aegpu_flip_status).
int run_apply(aegpu_engine *e, const double *x, double *y, double *epart, int ninst, int *nparts = nullptr,
              bool masked = true, bool flip = false, double *flip_part = nullptr, int *flip_used = nullptr)
{
    const int *act = masked ? e->d_active : nullptr;
    if (nparts) *nparts = e->spmv_grid;
    const int64_t D = (int64_t)e->B.D;
    // spin-flip half product: test every instance's input first (one launch); the
    // product kernels read the test's partials and pick the half or the full product
    FlipArgs fa{};
    const bool coded = e->ham_kind == 2 && e->ell_coded;
    if (flip_used) e->flip_tried = false;
    if (flip && flip_part && e->tune_flip && e->flip_ok && (coded || e->ham_kind == 3)) {
        if (flip_used) e->flip_tried = true;
        fa.part = flip_part;
        fa.used = flip_used;
        fa.slabs = e->d_flip_slabs;
        fa.nslabs = e->n_flip_slabs;
        fa.G = e->sm_count;
        fa.nB = e->db.nB;
        fa.div_m = e->db.div_m;
        fa.div_l = e->db.div_l;
        const dim3 g(e->sm_count, ninst);
        if (e->W == 1)
            k_flip_check<1><<<g, 256, 0, e->stream>>>(fa, x, D, flip_part, act);
        else
            k_flip_check<2><<<g, 256, 0, e->stream>>>(fa, x, D, flip_part, act);
        e->launches += 1;
    }
    if (e->ham_kind == 1) {
        const dim3 g(e->spmv_grid, ninst);
        if (e->W == 1)
            k_spmv<1, false><<<g, kSpmvThreads, 0, e->stream>>>(e->d_rowptr, 0, e->d_col, e->d_val, x, y, D, epart,
                                                                act);
        else
            k_spmv<2, false><<<g, kSpmvThreads, 0, e->stream>>>(e->d_rowptr, 0, e->d_col, e->d_val, x, y, D, epart,
                                                                act);
    } else if (e->ham_kind == 2 && e->ell_coded) {
        const int T = e->spmv_tpr();
        const int64_t rows_per_cta = kVellThreads / T;
        const int64_t nblk = (D + rows_per_cta - 1) / rows_per_cta;
        const size_t smem = (size_t)e->vell.vtab_len * sizeof(double);
        // one 1024-thread CTA per SM (its 64 registers per thread fill the register file)
        const int gx = (int)std::min<int64_t>(nblk, (int64_t)e->sm_count);
        // several right-hand sides per thread when the instances share the matrix and
        // need neither energies nor the instance mask (the Hessian's tangents, Lanczos)
        const bool multi = ninst > 1 && !epart && !act && e->vell.inst_e == 0;
        const int nv = multi ? (e->W == 1 ? kVellNV1 : kVellNV2) : 1;
        const dim3 g(gx, (ninst + nv - 1) / nv);
#define AE_VELL(WW, TT, NN) \
    k_spmv_vell<WW, TT, NN><<<g, kVellThreads, smem, e->stream>>>(e->vell, x, y, D, ninst, epart, act, fa)
        if (e->W == 1) {
            if (multi) {
                if (T == 1) AE_VELL(1, 1, kVellNV1); else if (T == 2) AE_VELL(1, 2, kVellNV1);
                else if (T == 4) AE_VELL(1, 4, kVellNV1); else AE_VELL(1, 8, kVellNV1);
            } else {
                if (T == 1) AE_VELL(1, 1, 1); else if (T == 2) AE_VELL(1, 2, 1); else if (T == 4) AE_VELL(1, 4, 1);
                else AE_VELL(1, 8, 1);
            }
        } else {
            if (multi) {
                if (T == 1) AE_VELL(2, 1, kVellNV2); else if (T == 2) AE_VELL(2, 2, kVellNV2);
                else if (T == 4) AE_VELL(2, 4, kVellNV2); else AE_VELL(2, 8, kVellNV2);
            } else {
                if (T == 1) AE_VELL(2, 1, 1); else if (T == 2) AE_VELL(2, 2, 1); else if (T == 4) AE_VELL(2, 4, 1);
                else AE_VELL(2, 8, 1);
            }
        }
#undef AE_VELL
        if (nparts) *nparts = gx;
    } else if (e->ham_kind == 2) {
        const int T = e->spmv_tpr();
        const int64_t rows_per_cta = kSpmvThreads / T;
        const int sg = (int)((D + rows_per_cta - 1) / rows_per_cta);
        const dim3 g(sg, ninst);
        const int64_t q = e->ell_width >> 2, ms = e->ell_stride_inst;
#define AE_SELL(WW, TT) \
    k_spmv_sell<WW, TT><<<g, kSpmvThreads, 0, e->stream>>>(q, e->d_col, e->d_val, x, y, D, epart, ms, act)
        if (e->W == 1) {
            if (T == 1) AE_SELL(1, 1); else if (T == 2) AE_SELL(1, 2); else if (T == 4) AE_SELL(1, 4); else AE_SELL(1, 8);
        } else {
            if (T == 1) AE_SELL(2, 1); else if (T == 2) AE_SELL(2, 2); else if (T == 4) AE_SELL(2, 4); else AE_SELL(2, 8);
        }
#undef AE_SELL
        if (nparts) *nparts = sg;
    } else if (e->ham_kind == 3) {
        const dim3 g(e->otf.nA, e->otf_chunks, ninst);
        const size_t smem = otf_smem_bytes(e->otf.N, e->otf.P2, e->otf.nsa, e->otf.nda);
        OtfArgs o = e->otf;
        o.active = act;
        if (e->W == 1)
            k_otf_strings<1><<<g, e->otf_threads, smem, e->stream>>>(o, x, y, epart, fa);
        else
            k_otf_strings<2><<<g, e->otf_threads, smem, e->stream>>>(o, x, y, epart, fa);
        if (nparts) *nparts = e->otf.nA * e->otf_chunks;
    } else {
        return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    }
    e->launches += 1;
    return e->cuda_check("apply H");
}

// E_dev[b] = <psi_b|H psi_b> for the first ninst instances (H psi left in d_h).
int run_energy(aegpu_engine *e, double *E_dev, int ninst)
{
    NvtxRange r("aegpu H*psi + energy");
    int np = 0;
    int rc = run_apply(e, e->d_psi, e->d_h, e->d_epart, ninst, &np, true, true, e->d_flip_part, e->d_flip_used);
    if (rc) return rc;
    k_reduce_sum<<<ninst, 256, 0, e->stream>>>(e->d_epart, np, E_dev, 1.0, e->d_active);
    e->launches += 1;
    return e->cuda_check("energy");
}

// Adjoint sweep over all passes for the first ninst instances (h updated in place,
// psi taken from the checkpoints), per-op gradients scale * <h|G_op psi> in
// grad_dev[b * nops + op] (scale 2 for the energy gradient, 1 for a projection).
// half: the instances that took the spin-flip half passes in the forward sweep take
// them here too (h = H psi has the symmetry); false only after a full forward sweep.
int run_backward(aegpu_engine *e, double *grad_dev, int ninst, double scale = 2.0, bool half = true)
{
    NvtxRange r("aegpu adjoint sweep");
    const int64_t n = (int64_t)e->vec_elems();
    const int nops = (int)e->excs.size();
    for (int bi = (int)e->dblocks.size() - 1; bi >= 0; --bi) {
        auto &b = e->dblocks[bi];
        double *part = e->d_partials + b.part_off;
        const double *ck = e->d_ckpt + b.ckpt_off;
        if (b.diagonal) {
            const DiagArgs da = e->diag_args(b, -1.0, true, half);
            if (b.smA && b.nslots >= kDiagAdjSzMinSlots)
                k_diag_adj_sz<<<dim3(b.wgrid, ninst), kDiagAdjThreads, 0, e->stream>>>(da, b.split, ck, e->n_ckpt,
                                                                                      e->d_h, n, part, e->n_partials);
            else if (b.nslots == 1)
                k_diag_adj<true><<<dim3(kDiagGrid, ninst), 256, 0, e->stream>>>(da, ck, e->n_ckpt, e->d_h, n, part,
                                                                               e->n_partials);
            else
                k_diag_adj<false><<<dim3(kDiagGrid, ninst), 256, 0, e->stream>>>(da, ck, e->n_ckpt, e->d_h, n, part,
                                                                                e->n_partials);
            e->launches += 1;
        } else if (b.nwtasks) {
            BlockArgs a = e->block_args(bi, -1.0, half);
            const dim3 g(b.wgrid, ninst);
            a.task_order = e->order_for(g, e->adj_occ);
            if (e->W == 1)
                launch_pass(e, k_warp_adj<1>, g, a, (const WarpTask *)b.wtasks, b.nwtasks, ck, e->n_ckpt, e->d_h, n,
                            part, e->n_partials);
            else
                launch_pass(e, k_warp_adj<2>, g, a, (const WarpTask *)b.wtasks, b.nwtasks, ck, e->n_ckpt, e->d_h, n,
                            part, e->n_partials);
            e->launches += 1;
        } else {
            cudaMemset2DAsync(part, e->n_partials * sizeof(double), 0, (size_t)b.wgrid * kMaxSlots * sizeof(double),
                              ninst, e->stream);
        }
    }
    const int warps = nops * ninst;
    const bool hm = half && e->half_static;
    k_grad_reduce<<<(warps * 32 + 255) / 256, 256, 0, e->stream>>>(e->d_partials, e->d_op_part_off, e->d_op_ntiles,
                                                                   e->d_op_slot, nops, scale, grad_dev, ninst,
                                                                   e->n_partials, e->d_active,
                                                                   hm ? e->d_mirror : nullptr,
                                                                   hm ? e->d_half : nullptr);
    e->launches += 1;
    return e->cuda_check("backward");
}

// Capture pass constants + evolve + H psi + adjoint sweep of all nb instances
// (reading d_ang, writing d_scalar / d_grad) into one CUDA graph.
// Capture one evaluation phase set of all nb instances into a graph: kind 0 = pass
// constants + evolve + H psi + energy + adjoint sweep (reading d_ang, writing d_scalar
// / d_grad), 1 = the first four only, 2 = the adjoint sweep only.  def (nullable)
// receives the graph's definition.
int capture_phases(aegpu_engine *e, int kind, cudaGraphExec_t *exec, cudaGraph_t *def, int64_t *nlaunch)
{
    NvtxRange r("aegpu capture evaluation graph");
    cudaStream_t cap = nullptr, saved = e->stream;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return e->cuda_check("graph stream");
    const int64_t l0 = e->launches;
    e->stream = cap;
    cudaGraph_t g = nullptr;
    int rc = AEGPU_OK;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = e->cuda_check("begin capture");
    if (!rc) {
        if (kind != 2) {
            rc = run_prep(e, e->nb);
            if (!rc) rc = run_evolve(e, e->nb);
            if (!rc) rc = run_energy(e, e->d_scalar, e->nb);
        }
        if (!rc && kind != 1) rc = run_backward(e, e->d_grad, e->nb);
        cudaError_t ce = cudaStreamEndCapture(cap, &g);
        if (!rc && ce != cudaSuccess) rc = e->fail(AEGPU_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(ce));
    }
    if (!rc && cudaGraphInstantiate(exec, g, 0) != cudaSuccess) rc = e->cuda_check("graph instantiate");
    if (!rc && def) {
        *def = g;
    } else if (g) {
        cudaGraphDestroy(g);
    }
    cudaStreamDestroy(cap);
    e->stream = saved;
    *nlaunch = e->launches - l0;
    e->launches = l0;
    cudaGetLastError();
    return rc;
}

int capture_grad_graph(aegpu_engine *e)
{
    return capture_phases(e, 0, &e->grad_graph, &e->grad_graph_def, &e->graph_launches);
}

// Replay the energy-phase (1) or adjoint-phase (2) graph on the engine's stream.
int launch_phases(aegpu_engine *e, int kind)
{
    cudaGraphExec_t &g = kind == 1 ? e->energy_graph : e->back_graph;
    int64_t &nl = kind == 1 ? e->energy_graph_launches : e->back_graph_launches;
    if (!g) {
        int rc = capture_phases(e, kind, &g, nullptr, &nl);
        if (rc) return rc;
    }
    if (cudaGraphLaunch(g, e->stream) != cudaSuccess) return e->cuda_check("graph launch");
    e->launches += nl;
    return AEGPU_OK;
}

bool same_angles(const aegpu_engine *e, const double *angles)
{
    return e->psi_valid && e->cached_angles.size() == e->excs.size() * (size_t)e->nb &&
           std::equal(e->cached_angles.begin(), e->cached_angles.end(), angles);
}

// psi of every instance evolved to these host angles ([nb][nops]), unless it already is.
int ensure_state(aegpu_engine *e, const double *angles)
{
    if (same_angles(e, angles)) return AEGPU_OK;
    int rc = upload_angles(e, angles, true, e->nb);
    if (!rc) rc = run_evolve(e, e->nb);
    if (rc) return rc;
    e->cached_angles.assign(angles, angles + e->excs.size() * (size_t)e->nb);
    e->psi_valid = true;
    e->h_valid = false;
    return AEGPU_OK;
}

int stream_sync(aegpu_engine *e, const char *where)
{
    cudaError_t rc = cudaStreamSynchronize(e->stream);
    if (rc != cudaSuccess) return e->fail(AEGPU_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(rc));
    return e->cuda_check(where);
}

}  // namespace

// ------------------------------------------------- allocation-free H * x --
// For callers that cannot allocate device memory: the entry point
// aegpu_csr_energy_noalloc keeps the per-block partial sums of <x|H x> in this
// fixed device array instead of engine-owned scratch.  Every device that loads the
// library holds it until the process exits.  One partial sum per 256-row block:
// at most kNoAllocMaxPartials blocks, i.e. kNoAllocMaxRows rows.
constexpr int kNoAllocMaxPartials = 16384;
constexpr int64_t kNoAllocRowsPerPartial = 256;
constexpr int64_t kNoAllocMaxRows = kNoAllocMaxPartials * kNoAllocRowsPerPartial;  // 4,194,304
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxPartials];

namespace {
std::mutex g_noalloc_mu;
constexpr int kNoAllocMaxDevices = 64;
double *g_noalloc_addr[kNoAllocMaxDevices] = {};  // device address of g_noalloc_scratch, per device
}  // namespace

// FP64 pipe probe: every thread runs 8 independent DFMA chains (enough independent
// work to hide the pipe latency); out receives a value that depends on every chain.
__global__ void k_fp64_probe(double *out, int iters, double a, double b)
{
    double r[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) r[k] = threadIdx.x * 1e-3 + k;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) r[k] = fma(r[k], a, b);
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += r[k];
    if (s == 12345.678) out[0] = s;  // keeps the chains live; practically never taken
}

// Excitation rule over a list of determinants, on the device: what the pass kernels and
// the orbit-table builder apply (exc_rule.h), in the reference's output convention
// (applyExcToBasisState_, fusedevolve.cpp:27-145): a paired determinant gives its
// partner and sign, an inactive one itself and -1, an active phase operator itself and
// +1.  The sign of a paired determinant is also recomputed with exc_sign (the pass
// kernels' form); a disagreement is reported as sign 0.
__global__ void k_exc_rule(ExcCode code, const uint32_t *__restrict__ states, int64_t n, uint32_t *__restrict__ partner,
                           int8_t *__restrict__ sign)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t p;
        int sg;
        const int st = apply_exc(code, states[i], p, sg);
        if (st == 1 && exc_sign(code, states[i]) != sg) sg = 0;
        partner[i] = p;
        sign[i] = (int8_t)(st == 0 ? -1 : sg);
    }
}

// ==================================================================== C ABI ==
extern "C" {

int aegpu_exc_rule_dev(int nops, const int *ops, const uint32_t *states_dev, int64_t n, uint32_t *partner_dev,
                       int8_t *sign_dev, void *stream)
{
    if (nops < 0 || (nops && !ops) || n < 0 || (n && (!states_dev || !partner_dev || !sign_dev))) return AEGPU_ERR_ARG;
    for (int o = 0; o < nops; ++o)
        for (int k = 0; k < 4; ++k)
            if (ops[4 * o + k] < -1 || ops[4 * o + k] > 31) return AEGPU_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8));
    for (int o = 0; o < nops && n > 0; ++o) {
        const int *q = ops + 4 * o;
        k_exc_rule<<<grid, 256, 0, s>>>(make_exc_code(q[0], q[1], q[2], q[3]), states_dev, n, partner_dev + (size_t)o * n,
                                        sign_dev + (size_t)o * n);
    }
    const cudaError_t rc = cudaGetLastError();
    return rc == cudaSuccess ? AEGPU_OK : AEGPU_ERR_CUDA;
}

int aegpu_host_exc_rule(int nops, const int *ops, const uint32_t *states, int64_t n, uint32_t *partner, int8_t *sign)
{
    if (nops < 0 || (nops && !ops) || n < 0 || (n && (!states || !partner || !sign))) return AEGPU_ERR_ARG;
    for (int o = 0; o < nops; ++o) {
        const int *q = ops + 4 * o;
        for (int k = 0; k < 4; ++k)
            if (q[k] < -1 || q[k] > 31) return AEGPU_ERR_ARG;
        const ExcCode code = make_exc_code(q[0], q[1], q[2], q[3]);
        for (int64_t i = 0; i < n; ++i) {
            uint32_t p;
            int sg;
            const int st = apply_exc(code, states[i], p, sg);
            if (st == 1 && exc_sign(code, states[i]) != sg) sg = 0;
            partner[(size_t)o * n + i] = p;
            sign[(size_t)o * n + i] = (int8_t)(st == 0 ? -1 : sg);
        }
    }
    return AEGPU_OK;
}

int aegpu_create(aegpu_engine **out)
{
    if (!out) return AEGPU_ERR_ARG;
    *out = nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return AEGPU_ERR_CUDA;
    }
    auto *e = new aegpu_engine();
    cudaDeviceGetAttribute(&e->sm_count, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&e->smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (const char *v = std::getenv("AEGPU_REUSE_HPSI")) e->reuse_hpsi = std::strcmp(v, "0") != 0;
    if (const char *v = std::getenv("AEGPU_FLIP")) e->tune_flip = std::strcmp(v, "0") != 0;
    if (const char *v = std::getenv("AEGPU_HALF")) e->tune_half = std::strcmp(v, "0") != 0;
    if (const char *v = std::getenv("AEGPU_TASK_ORDER")) e->task_order = std::strcmp(v, "0") != 0;
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete e;
        return AEGPU_ERR_CUDA;
    }
    if (set_smem_limits(dev)) {
        delete e;
        return AEGPU_ERR_CUDA;
    }
    e->spmv_grid = e->sm_count * 8;
    *out = e;
    return AEGPU_OK;
}

void aegpu_destroy(aegpu_engine *e) { delete e; }

const char *aegpu_last_error(const aegpu_engine *e) { return e ? e->err.c_str() : "null engine"; }

// Slot masks of a diagonal pass by string (Sz basis): slot i is active on determinant
// (a, b) when the alpha string a holds the alpha bits of its annihilation mask and the
// beta string b the beta bits, so the mask is smA[a] & smB[b] (two table loads in place
// of a loop over the slots).  Also the slot activations summed over all determinants.
static void diag_string_masks(aegpu_engine *e, const Block &b, aegpu_engine::DevBlock &d)
{
    const Basis &B = e->B;
    const int ns = (int)b.ops.size();
    if (B.kind != BASIS_SZ) {
        // counted for the work accounting only; above 2^22 determinants the counts are
        // left as estimates (half the determinants per slot)
        d.slot_acts = (uint64_t)ns * B.D / 2;
        d.active = B.D;
        if (B.D > (1u << 22)) return;
        d.slot_acts = d.active = 0;
        for (uint64_t z = 0; z < B.D; ++z) {
            const uint32_t bits = B.bits(z);
            bool any = false;
            for (int op : b.ops)
                if ((bits & e->codes[op].annihilate) == e->codes[op].annihilate) {
                    d.slot_acts++;
                    any = true;
                }
            d.active += any;
        }
        return;
    }
    const uint32_t lo = (1u << B.N) - 1u;
    std::vector<uint16_t> mA(B.nA), mB(B.nB);
    std::vector<uint64_t> cA(ns, 0), cB(ns, 0);
    for (uint32_t r = 0; r < B.nA; ++r) {
        uint32_t m = 0;
        for (int i = 0; i < ns; ++i) {
            const uint32_t ann = e->codes[b.ops[i]].annihilate >> B.N;
            if ((B.strA[r] & ann) == ann) { m |= 1u << i; cA[i]++; }
        }
        mA[r] = (uint16_t)m;
    }
    for (uint32_t r = 0; r < B.nB; ++r) {
        uint32_t m = 0;
        for (int i = 0; i < ns; ++i) {
            const uint32_t ann = e->codes[b.ops[i]].annihilate & lo;
            if ((B.strB[r] & ann) == ann) { m |= 1u << i; cB[i]++; }
        }
        mB[r] = (uint16_t)m;
    }
    d.slot_acts = 0;
    for (int i = 0; i < ns; ++i) d.slot_acts += cA[i] * cB[i];
    // launch shape and slot classes of the adjoint kernel k_diag_adj_sz
    DiagSplit &sp = d.split;
    sp.cols = 32;
    while (sp.cols < kDiagAdjThreads && (uint32_t)sp.cols < B.nB) sp.cols *= 2;
    sp.col_blocks = (int)((B.nB + sp.cols - 1) / sp.cols);
    sp.row_chunks = (int)std::max<int64_t>(1, std::min<int64_t>(B.nA, kDiagGrid / sp.col_blocks));
    sp.b_only = sp.a_rows = sp.mixed = 0;
    for (int i = 0; i < ns; ++i) {
        const uint32_t ann = e->codes[b.ops[i]].annihilate;
        const bool ha = (ann >> B.N) != 0, hb = (ann & lo) != 0;
        if (!ha) sp.b_only |= 1u << i;
        else sp.a_rows |= 1u << i;
        if (ha && hb) sp.mixed |= 1u << i;
    }
    if (ns >= kDiagAdjSzMinSlots) d.wgrid = sp.col_blocks * sp.row_chunks;
    // the half passes' split of the same CTAs over the triangle, by each column block's
    // share of its amplitudes, every block at least one CTA
    sp.half_first[0] = -1;
    const int G = sp.col_blocks * sp.row_chunks;
    if (sp.col_blocks <= kDiagMaxColBlocks && G >= sp.col_blocks) {
        std::vector<double> w(sp.col_blocks);
        double W = 0;
        for (int c = 0; c < sp.col_blocks; ++c) {
            // amplitudes (a, b) with a <= b in the block's columns (tri_row's total)
            const double lo = (double)c * sp.cols, L = std::min<double>(B.nB, (double)(c + 1) * sp.cols) - lo;
            w[c] = lo * L + L * (L + 1) / 2.0;
            W += w[c];
        }
        std::vector<int> n(sp.col_blocks, 1);
        int used = sp.col_blocks;
        for (int c = 0; c < sp.col_blocks; ++c) {
            const int extra = (int)std::floor((G - sp.col_blocks) * w[c] / W);
            n[c] += extra;
            used += extra;
        }
        for (int c = sp.col_blocks - 1; used < G; c = (c + sp.col_blocks - 1) % sp.col_blocks) {
            n[c]++;
            used++;
        }
        sp.half_first[0] = 0;
        for (int c = 0; c < sp.col_blocks; ++c) sp.half_first[c + 1] = sp.half_first[c] + n[c];
    }
    // determinants with at least one active slot, from the histograms of the two masks
    std::vector<uint64_t> hA((size_t)1 << ns, 0), hB((size_t)1 << ns, 0);
    for (uint16_t m : mA) hA[m]++;
    for (uint16_t m : mB) hB[m]++;
    std::vector<uint32_t> uA, uB;
    for (uint32_t m = 1; m < hA.size(); ++m)
        if (hA[m]) uA.push_back(m);
    for (uint32_t m = 1; m < hB.size(); ++m)
        if (hB[m]) uB.push_back(m);
    d.active = 0;
    for (uint32_t u : uA)
        for (uint32_t v : uB)
            if (u & v) d.active += hA[u] * hB[v];
    // the same counts over a <= b: a pass that holds the mirror of every slot is active on
    // (a, b) exactly where it is active on (b, a), slot for mirror slot, so each count over
    // a <= b is half of the full count plus half of its count on the diagonal a = b
    if (B.nA == B.nB) {
        uint64_t same_act = 0, same_slots = 0;
        for (uint32_t r = 0; r < B.nA; ++r) {
            const uint32_t m = (uint32_t)mA[r] & (uint32_t)mB[r];
            same_act += m != 0;
            same_slots += (uint64_t)__builtin_popcount(m);
        }
        d.active_h = (d.active + same_act) / 2;
        d.slot_acts_h = (d.slot_acts + same_slots) / 2;
    }
    d.smA = e->upload(mA);
    d.smB = e->upload(mB);
}

int aegpu_set_problem(aegpu_engine *e, int nq, int basis_kind, int n_elec, int n_alpha, int n_beta, int complex_mode,
                      int nops, const int *ops)
{
    if (!e) return AEGPU_ERR_ARG;
    if (e->d_start) return e->fail(AEGPU_ERR_STATE, "the problem is already set (create a new engine)");
    NvtxRange r("aegpu set problem");
    if (nops < 1 || !ops) return e->fail(AEGPU_ERR_ARG, "no excitations");
    if (!e->B.init(nq, basis_kind, n_elec, n_alpha, n_beta, e->err)) return AEGPU_ERR_ARG;
    e->cplx = complex_mode != 0;
    e->W = e->cplx ? 2 : 1;
    e->excs.resize(nops);
    e->codes.resize(nops);
    for (int i = 0; i < nops; ++i) {
        for (int j = 0; j < 4; ++j) {
            int v = ops[4 * i + j];
            if (v < -1 || v >= nq) return e->fail(AEGPU_ERR_ARG, "excitation index out of range");
            e->excs[i].v[j] = (int8_t)v;
        }
        const Exc &x = e->excs[i];
        bool single = x.v[0] >= 0 && x.v[1] >= 0 && x.v[2] < 0 && x.v[3] < 0;
        bool dbl = x.v[0] >= 0 && x.v[1] >= 0 && x.v[2] >= 0 && x.v[3] >= 0;
        if (!single && !dbl) return e->fail(AEGPU_ERR_ARG, "excitation is neither a single nor a double");
        if (exc_is_diagonal(x) != exc_has_diagonal(x))
            return e->fail(AEGPU_ERR_UNSUPPORTED, "excitation with a repeated orbital that is not diagonal");
        if (dbl && (x.v[0] == x.v[1] || x.v[2] == x.v[3]) && !exc_is_diagonal(x))
            return e->fail(AEGPU_ERR_ARG, "double excitation creates or destroys one orbital twice");
        if (exc_is_diagonal(x) && !e->cplx)
            return e->fail(AEGPU_ERR_UNSUPPORTED, "diagonal (number) operators need complex mode");
        e->codes[i] = make_exc_code(x.v[0], x.v[1], x.v[2], x.v[3]);
    }
    // the reference's commuting blocks, cut into passes of <= 6 excitations so that
    // every orbit fits one warp's registers
    // spin-flip half passes need the Sz basis with as many alpha as beta strings and every
    // operator's mirror in its block or diagonal run (then in its pass); the application
    // order (the Hessian's positions) is the passes' order
    e->half_static = make_passes(e->excs, e->codes, e->B.N, e->tune_pass_ops,
                                 e->B.kind == BASIS_SZ && e->B.nA == e->B.nB, e->blocks, e->perm, e->mirror);
    e->pos_of_op.assign(nops, 0);
    for (int p = 0; p < nops; ++p) e->pos_of_op[e->perm[p]] = p;

    // device basis
    DevBasis db{};
    db.kind = e->B.kind;
    db.N = e->B.N;
    db.nq = nq;
    db.nA = e->B.nA;
    db.nB = e->B.nB;
    db.D = e->B.D;
    // unsigned division by the constant nB with a multiply-high (round-up method)
    if (db.nB > 1) {
        uint32_t l = 0;
        while ((1ull << l) < db.nB) ++l;
        db.div_l = l;
        db.div_m = (uint32_t)(((1ull << 32) * ((1ull << l) - db.nB)) / db.nB + 1);
    } else {
        db.div_l = 0;
        db.div_m = 0;
    }
    if (e->B.kind == BASIS_SZ) {
        db.strA = e->upload(e->B.strA);
        db.strB = e->upload(e->B.strB);
        db.rankA = e->upload(e->B.rankA);
        db.rankB = e->upload(e->B.rankB);
    } else {
        db.states = e->upload(e->B.states);
        db.rank = e->upload(e->B.rank);
    }
    e->db = db;
    e->d_codes = e->upload(e->codes);

    // resident CTAs per SM of the forward and adjoint warp kernels (their register counts)
    int rot_occ = 0, adj_occ = 0;
    if (e->cplx) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rot_occ, k_warp_rot<2>, kWarpThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&adj_occ, k_warp_adj<2>, kWarpThreads, 0);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rot_occ, k_warp_rot<1>, kWarpThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&adj_occ, k_warp_adj<1>, kWarpThreads, 0);
    }
    cudaGetLastError();
    e->rot_occ = rot_occ;
    e->adj_occ = adj_occ;
    // orbit tables per block
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    e->dblocks.clear();
    e->n_diag_tab = 0;
    e->block_pos0.clear();
    e->op_block.assign(nops, 0);
    e->op_slot.assign(nops, 0);
    int64_t part_off = 0, ckpt_off = 0;
    int pos = 0;
    for (size_t bi = 0; bi < e->blocks.size(); ++bi) {
        const Block &b = e->blocks[bi];
        aegpu_engine::DevBlock d;
        d.diagonal = b.diagonal;
        d.nslots = (int)b.ops.size();
        d.ops = e->upload(b.ops);
        e->block_pos0.push_back(pos);
        for (int s = 0; s < d.nslots; ++s) {
            e->op_block[b.ops[s]] = (int)bi;
            e->op_slot[b.ops[s]] = s;
        }
        pos += d.nslots;
        if (!b.diagonal) {
            std::vector<ExcCode> bc;
            for (int op : b.ops) bc.push_back(e->codes[op]);
            OrbitTables T = build_orbits(e->B, bc, (int)hw);
            if (!T.ok) return e->fail(AEGPU_ERR_UNSUPPORTED, "an excitation leaves the determinant sector");
            d.idx = e->upload(T.idx);
            d.bits = e->upload(T.bits);
            d.groups = e->upload(T.groups);
            d.tiles = e->upload(T.tiles);
            d.ntiles = (int)T.tiles.size();
            d.wtasks = e->upload(T.wtasks);
            d.nwtasks = (int)T.wtasks.size();
            d.wgrid = std::max(1, std::min(e->sm_count * e->tune_ctas_per_sm, (d.nwtasks + 7) / 8));
            // the forward kernel needs fewer registers than the adjoint: as many CTAs as stay
            // resident, so that a warp takes at most one task where the tasks allow
            d.rgrid = std::max(1, std::min(e->sm_count * std::max(e->tune_ctas_per_sm, rot_occ), (d.nwtasks + 7) / 8));
            d.active = T.active;
            d.amp_layers = T.amp_layers;
            if (e->half_static) {
                std::vector<int> mslot(b.ops.size(), -1);
                for (size_t i = 0; i < b.ops.size(); ++i)
                    for (size_t j = 0; j < b.ops.size(); ++j)
                        if (b.ops[j] == e->mirror[b.ops[i]]) mslot[i] = (int)j;
                HalfTables H = build_half_orbits(e->B, T, bc, mslot, (int)hw);
                if (!H.ok) {
                    e->half_static = false;
                } else {
                    d.idx_h = e->upload(H.idx);
                    d.bits_h = e->upload(H.bits);
                    d.wtasks_h = e->upload(H.wtasks);
                    d.nwtasks_h = (int)H.wtasks.size();
                    d.active_h = H.active;
                    d.amp_layers_h = H.amp_layers;
                }
            }
        } else {
            d.ntiles = kDiagGrid;
            d.wgrid = kDiagGrid;
            d.tab_off = e->n_diag_tab;
            e->n_diag_tab += (int64_t)2 << d.nslots;
            diag_string_masks(e, b, d);
        }
        d.part_off = part_off;
        part_off += (int64_t)d.wgrid * kMaxSlots;
        d.ckpt_off = ckpt_off;
        ckpt_off += (int64_t)(d.diagonal ? e->B.D : d.active) * (e->cplx ? 2 : 1);
        e->dblocks.push_back(d);
    }
    e->n_partials = part_off;
    std::vector<int64_t> opo(nops);
    std::vector<int> opn(nops), ops_slot(nops);
    for (int o = 0; o < nops; ++o) {
        const auto &d = e->dblocks[e->op_block[o]];
        opo[o] = d.part_off;
        opn[o] = d.wgrid;
        ops_slot[o] = e->op_slot[o];
    }
    e->d_op_part_off = e->upload(opo);
    e->d_op_ntiles = e->upload(opn);
    e->d_op_slot = e->upload(ops_slot);
    e->d_tpos = e->upload(e->pos_of_op);
    e->d_pos_op = e->upload(e->perm);

    // pass lists for the per-evaluation constant preparation
    std::vector<int> pops, poff, pn, pdiag;
    std::vector<int64_t> ptab;
    for (size_t bi = 0; bi < e->blocks.size(); ++bi) {
        const Block &b = e->blocks[bi];
        poff.push_back((int)pops.size());
        pn.push_back((int)b.ops.size());
        pdiag.push_back(b.diagonal ? 1 : 0);
        ptab.push_back(b.diagonal ? e->dblocks[bi].tab_off : 0);
        pops.insert(pops.end(), b.ops.begin(), b.ops.end());
    }
    PrepArgs pa{};
    pa.pass_ops = e->upload(pops);
    pa.pass_off = e->upload(poff);
    pa.pass_n = e->upload(pn);
    pa.pass_diag = e->upload(pdiag);
    pa.pass_tab = e->upload(ptab);
    pa.tab_stride = e->n_diag_tab;
    pa.codes = e->d_codes;
    pa.nops = nops;
    pa.npass = (int)e->blocks.size();
    if (e->half_static) {
        e->d_mirror = e->upload(e->mirror);
        e->d_half_gate = e->alloc<int>(1);
        pa.mirror = e->d_mirror;
        pa.half_gate = e->d_half_gate;
    }
    e->prep = pa;

    if (e->alloc_failed) return e->fail(AEGPU_ERR_NOMEM, "device allocation failed while building the passes");
    const size_t n = e->vec_elems();
    e->n_ckpt = ckpt_off;
    // partial sums per instance: the CSR grid, or one per CTA of the stored-H product at
    // up to 8 threads per row
    e->n_epart = std::max<int64_t>(e->spmv_grid, ((int64_t)e->B.D * 8 + kSpmvThreads - 1) / kSpmvThreads);
    e->d_start = e->alloc<double>(n);
    if (!e->d_start || !pa.pass_ops || !pa.pass_diag) return e->fail(AEGPU_ERR_NOMEM, "device allocation failed");
    int rc = e->alloc_instances(e->nb);
    if (rc) return rc;
    if (e->alloc_failed) return e->fail(AEGPU_ERR_NOMEM, "device allocation failed");
    cudaMemset(e->d_start, 0, n * sizeof(double));
    e->start_sym = true;
    e->write_half_gate();
    // setup copies ran on the legacy stream: finish them before any engine-stream work
    if (cudaDeviceSynchronize() != cudaSuccess) return e->cuda_check("set_problem");
    return e->cuda_check("set_problem");
}

int64_t aegpu_dim(const aegpu_engine *e) { return e ? (int64_t)e->B.D : -1; }

int aegpu_amplitude_width(const aegpu_engine *e) { return e ? e->W : -1; }

int aegpu_basis_states(const aegpu_engine *e, uint32_t *out)
{
    if (!e || !out) return AEGPU_ERR_ARG;
    for (uint64_t z = 0; z < e->B.D; ++z) out[z] = e->B.bits(z);
    return AEGPU_OK;
}

int aegpu_num_blocks(const aegpu_engine *e) { return e ? (int)e->blocks.size() : -1; }

int aegpu_block_layout(const aegpu_engine *e, int *perm, int *block_sizes)
{
    if (!e) return AEGPU_ERR_ARG;
    if (perm) std::copy(e->perm.begin(), e->perm.end(), perm);
    if (block_sizes)
        for (size_t b = 0; b < e->blocks.size(); ++b) block_sizes[b] = (int)e->blocks[b].ops.size() * (e->blocks[b].diagonal ? -1 : 1);
    return AEGPU_OK;
}

int aegpu_set_initial(aegpu_engine *e, const double *amps)
{
    if (!e || !amps) return AEGPU_ERR_ARG;
    if (!e->d_start) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    cudaMemcpy(e->d_start, amps, (size_t)e->B.D * e->W * sizeof(double), cudaMemcpyHostToDevice);
    e->psi_valid = e->h_valid = false;
    if (e->half_static) {
        // the half passes need a start state with psi(a,b) = psi(b,a)
        bool sym = true;
        const uint64_t nB = e->B.nB;
        for (uint64_t x = 0; x < nB && sym; ++x)
            for (uint64_t y = x + 1; y < nB && sym; ++y)
                for (int w = 0; w < e->W; ++w)
                    if (amps[(x * nB + y) * e->W + w] != amps[(y * nB + x) * e->W + w]) sym = false;
        e->start_sym = sym;
        e->write_half_gate();
    }
    cudaDeviceSynchronize();
    return e->cuda_check("set_initial");
}

int aegpu_set_ham_csr(aegpu_engine *e, int64_t nnz, const int64_t *rowptr, const int32_t *col, const double *val)
{
    if (!e || !rowptr || (nnz > 0 && (!col || !val))) return AEGPU_ERR_ARG;
    if (!e->d_start) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    const int64_t D = (int64_t)e->B.D;
    if (rowptr[0] != 0 || rowptr[D] != nnz) return e->fail(AEGPU_ERR_ARG, "inconsistent CSR row pointers");
    for (int64_t k = 0; k < nnz; ++k)
        if (col[k] < 0 || col[k] >= D) return e->fail(AEGPU_ERR_ARG, "CSR column out of range");
    e->drop_ham();
    e->d_rowptr = e->ham_alloc<int64_t>(D + 1);
    e->d_col = e->ham_alloc<int32_t>(nnz);
    e->d_val = e->ham_alloc<double>(nnz);
    if (!e->d_rowptr || !e->d_col || !e->d_val) return e->fail(AEGPU_ERR_NOMEM, "CSR allocation failed");
    cudaMemcpy(e->d_rowptr, rowptr, (D + 1) * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (nnz) {
        cudaMemcpy(e->d_col, col, nnz * sizeof(int32_t), cudaMemcpyHostToDevice);
        cudaMemcpy(e->d_val, val, nnz * sizeof(double), cudaMemcpyHostToDevice);
    }
    e->ham_kind = 1;
    e->ham_per_instance = false;
    e->ell_stride_inst = 0;
    e->ham_entries = nnz;
    e->h_valid = false;
    cudaDeviceSynchronize();
    return e->cuda_check("set_ham_csr");
}

}  // extern "C"

namespace {

// Hamiltonian from integrals for ntab table sets: ntab = 1 shares one Hamiltonian
// between all instances, ntab = nb gives instance b the integrals h1s[b], g2s[b].
// Value tables and coded rows of every instance (the engine's integrals already on the
// device; e->vell and e->ints set).
static void build_coded_rows(aegpu_engine *e, int ntab, bool values_only)
{
    const IntArgs a = e->ints;
    const int N = a.N;
    const size_t NN = (size_t)N * N, N4 = NN * NN;
    const int64_t D = (int64_t)e->B.D, Dpad = (D + 31) & ~(int64_t)31;
    const size_t per_e = (size_t)Dpad * a.stride_e, per_d = (size_t)Dpad * a.stride_d;
    const VellArgs &v = e->vell;
    const int64_t chunk = 1 << 16;
    for (int t = 0; t < ntab; ++t) {
        IntArgs ai = a;
        ai.h1 = e->d_h1 + NN * t;
        ai.g2 = e->d_g2 + N4 * t;
        k_vtab_build<<<(int)((v.vtab_len + 255) / 256), 256, 0, e->stream>>>(ai, (double *)v.vtab + (size_t)v.vtab_len * t);
        e->launches += 1;
        for (int64_t r0 = 0; r0 < Dpad; r0 += chunk) {
            k_vell_build<<<e->sm_count * 8, 256, 0, e->stream>>>(ai, (int32_t *)v.colE + per_e * t,
                                                                (double *)v.valE + per_e * t,
                                                                (int32_t *)v.colD + per_d * t,
                                                                (uint16_t *)v.codeD + per_d * t, r0,
                                                                std::min(Dpad, r0 + chunk), values_only);
            e->launches += 1;
        }
    }
}

// New integral values for an integral Hamiltonian of the same shape (same instances
// and representation): the values are written into the existing buffers -- stored rows
// rebuilt, on-the-fly integral tables and diagonal rebuilt; the string tables do not
// depend on the integrals -- so every device pointer, and the captured evaluation
// graphs that hold them, stay valid.  A family scan changes only the values.
static int refresh_integrals(aegpu_engine *e, const double *h1s, const double *g2s, int ntab)
{
    NvtxRange r("aegpu refresh Hamiltonian");
    const int N = e->B.N;
    const size_t NN = (size_t)N * N, N4 = NN * NN;
    cudaStream_t s = e->stream;
    if (stream_sync(e, "refresh integrals")) return AEGPU_ERR_CUDA;  // nothing in flight reads the old values
    cudaMemcpy(e->d_h1, h1s, sizeof(double) * NN * ntab, cudaMemcpyHostToDevice);
    cudaMemcpy(e->d_g2, g2s, sizeof(double) * N4 * ntab, cudaMemcpyHostToDevice);
    const int64_t D = (int64_t)e->B.D;
    IntArgs a = e->ints;
    if (e->ham_kind == 2 && e->ell_coded) {
        build_coded_rows(e, ntab, true);
    } else if (e->ham_kind == 2) {
        const int64_t Dpad = (D + 31) & ~(int64_t)31;
        const size_t per = (size_t)Dpad * a.stride;
        const int64_t chunk = 1 << 16;
        for (int t = 0; t < ntab; ++t) {
            IntArgs ai = a;
            ai.h1 = e->d_h1 + NN * t;
            ai.g2 = e->d_g2 + N4 * t;
            for (int64_t r0 = 0; r0 < Dpad; r0 += chunk) {
                k_ell_build<<<e->sm_count * 8, 256, 0, s>>>(ai, e->d_col + per * t, e->d_val + per * t, r0,
                                                            std::min(Dpad, r0 + chunk));
                e->launches += 1;
            }
        }
    } else {
        std::vector<OtfTables> T(ntab);
        const int hw = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        std::atomic<int> next{0};
        for (int w = 0; w < std::min(hw, ntab); ++w)
            pool.emplace_back([&]() {
                for (int t; (t = next.fetch_add(1)) < ntab;) {
                    std::vector<double> hv(h1s + NN * t, h1s + NN * (t + 1)), gv(g2s + N4 * t, g2s + N4 * (t + 1));
                    build_otf_tables(e->B, hv, gv, T[t], false);
                }
            });
        for (auto &th : pool) th.join();
        auto put = [&](const double *dst, std::vector<double> OtfTables::*m) {
            const size_t per = (T[0].*m).size();
            std::vector<double> all;
            all.reserve(per * ntab);
            for (auto &x : T) all.insert(all.end(), (x.*m).begin(), (x.*m).end());
            cudaMemcpy((void *)dst, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice);
        };
        put(e->otf.vss, &OtfTables::vss);
        put(e->otf.vab, &OtfTables::vab);
        put(e->otf.a_alpha, &OtfTables::a_alpha);
        put(e->otf.b_alpha, &OtfTables::b_alpha);
        put(e->otf.a_beta, &OtfTables::a_beta);
        put(e->otf.b_beta, &OtfTables::b_beta);
        for (int t = 0; t < ntab; ++t) {
            IntArgs ai = a;
            ai.h1 = e->d_h1 + NN * t;
            ai.g2 = e->d_g2 + N4 * t;
            k_diag_build<<<e->sm_count * 8, 256, 0, s>>>(ai, (double *)e->otf.diag + (size_t)D * t);
            e->launches += 1;
        }
    }
    e->h_valid = false;
    e->ground_valid = false;
    return stream_sync(e, "refresh integrals");
}

int set_integrals(aegpu_engine *e, const double *h1s, const double *g2s, int ntab, int mode)
{
    NvtxRange r("aegpu set Hamiltonian");
    if (!e->d_start) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    if (e->B.kind != BASIS_SZ) return e->fail(AEGPU_ERR_UNSUPPORTED, "integral Hamiltonians need the Sz sector");
    if ((e->ham_kind == 2 || e->ham_kind == 3) && e->d_h1 && e->ints_ntab == ntab && e->ints_mode_asked == mode)
        return refresh_integrals(e, h1s, g2s, ntab);
    const int N = e->B.N;
    const size_t NN = (size_t)N * N, N4 = NN * NN;
    IntArgs a{};
    a.N = N;
    a.nq = e->B.nq;
    a.basis = e->db;
    a.nOa = e->B.na;
    a.nVa = N - e->B.na;
    a.nOb = e->B.nb;
    a.nVb = N - e->B.nb;
    auto c2 = [](int64_t n) { return n * (n - 1) / 2; };
    a.width = 1 + (int64_t)a.nOa * a.nVa + (int64_t)a.nOb * a.nVb + c2(a.nOa) * c2(a.nVa) + c2(a.nOb) * c2(a.nVb) +
              (int64_t)a.nOa * a.nVa * a.nOb * a.nVb;
    a.stride = (a.width + 3) & ~(int64_t)3;
    a.NP = N * (N - 1) / 2;
    a.width_e = 1 + (int64_t)a.nOa * a.nVa + (int64_t)a.nOb * a.nVb;
    a.stride_e = (a.width_e + 3) & ~(int64_t)3;
    a.width_d = a.width - a.width_e;
    a.stride_d = (a.width_d + 3) & ~(int64_t)3;
    // coded rows when the value table has at most 2^15 entries (N <= 12), unless the
    // environment says AEGPU_CODED_ROWS=0
    const char *cenv = std::getenv("AEGPU_CODED_ROWS");
    const bool coded = vtab_len(N) <= kVtabMax && !(cenv && std::strcmp(cenv, "0") == 0);
    e->drop_ham();
    auto ham_alloc = [&](auto *&ptr, size_t count) {
        using T = std::remove_reference_t<decltype(*ptr)>;
        ptr = e->ham_alloc<T>(count);
        return ptr != nullptr;
    };
    auto ham_upload = [&](auto *&ptr, const auto &v) {
        using T = std::remove_const_t<std::remove_reference_t<decltype(*ptr)>>;
        T *p = e->ham_alloc<T>(v.size());
        ptr = p;
        if (!p) return false;
        if (!v.empty()) cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
        return true;
    };
    if (!ham_alloc(e->d_h1, NN * ntab) || !ham_alloc(e->d_g2, N4 * ntab))
        return e->fail(AEGPU_ERR_NOMEM, "integral allocation failed");
    cudaMemcpy(e->d_h1, h1s, sizeof(double) * NN * ntab, cudaMemcpyHostToDevice);
    cudaMemcpy(e->d_g2, g2s, sizeof(double) * N4 * ntab, cudaMemcpyHostToDevice);
    cudaDeviceSynchronize();
    a.h1 = e->d_h1;
    a.g2 = e->d_g2;
    e->ints = a;
    e->ell_width = (int)a.stride;
    const int64_t D = (int64_t)e->B.D;
    const int64_t Dpad = (D + 31) & ~(int64_t)31;
    const double ell_bytes = coded ? ((double)Dpad * (a.stride_e * 12.0 + a.stride_d * 6.0) + vtab_len(N) * 8.0) * ntab
                                   : (double)Dpad * a.stride * 12.0 * ntab;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const int mode_asked = mode;
    if (mode == AEGPU_HAM_AUTO) mode = ell_bytes < 0.6 * (double)free_b ? AEGPU_HAM_STORED : AEGPU_HAM_ON_THE_FLY;
    e->ham_per_instance = ntab > 1;
    if (mode == AEGPU_HAM_STORED && coded) {
        const size_t per_e = (size_t)Dpad * a.stride_e, per_d = (size_t)Dpad * a.stride_d;
        const int64_t L = vtab_len(N);
        VellArgs v{};
        int32_t *colE = nullptr, *colD = nullptr;
        double *valE = nullptr, *vtab = nullptr;
        uint16_t *codeD = nullptr;
        if (!ham_alloc(colE, per_e * ntab) || !ham_alloc(valE, per_e * ntab) || !ham_alloc(colD, per_d * ntab) ||
            !ham_alloc(codeD, per_d * ntab) || !ham_alloc(vtab, (size_t)L * ntab))
            return e->fail(AEGPU_ERR_NOMEM, "coded row allocation failed");
        v.colE = colE;
        v.valE = valE;
        v.colD = colD;
        v.codeD = codeD;
        v.vtab = vtab;
        v.qe = a.stride_e >> 2;
        v.qd = a.stride_d >> 2;
        v.inst_e = ntab > 1 ? (int64_t)per_e : 0;
        v.inst_d = ntab > 1 ? (int64_t)per_d : 0;
        v.vtab_len = L;
        v.vtab_inst = ntab > 1 ? L : 0;
        e->vell = v;
        e->ell_coded = true;
        e->ints = a;
        build_coded_rows(e, ntab, false);
        e->ham_kind = 2;
        e->ham_entries = D * (a.stride_e + a.stride_d);
        e->ell_width = (int)(a.stride_e + a.stride_d);
        e->ell_stride_inst = 0;
        if (e->B.na == e->B.nb) {
            // the 32-row slabs that hold a row (a, b) with a <= b, for the half product
            std::vector<int32_t> slabs;
            const uint32_t nB = e->B.nB;
            for (int64_t sl = 0; sl * 32 < D; ++sl) {
                const int64_t r0 = sl * 32, r1 = std::min<int64_t>(D, r0 + 32);
                // rows r0..r1-1 cover alpha strings r0 / nB .. (r1 - 1) / nB; a row with
                // a <= b exists unless every row of the slab lies below the diagonal
                bool any = false;
                for (int64_t r = r0; r < r1 && !any; ++r) any = (uint64_t)r / nB <= (uint64_t)r % nB;
                if (any) slabs.push_back((int32_t)sl);
            }
            if (!ham_upload(e->d_flip_slabs, slabs)) return e->fail(AEGPU_ERR_NOMEM, "slab list allocation failed");
            e->n_flip_slabs = (int64_t)slabs.size();
            e->flip_ok = true;
        }
    } else if (mode == AEGPU_HAM_STORED) {
        const size_t per = (size_t)Dpad * a.stride;
        if (!ham_alloc(e->d_col, per * ntab) || !ham_alloc(e->d_val, per * ntab))
            return e->fail(AEGPU_ERR_NOMEM, "ELL allocation failed");
        const int64_t chunk = 1 << 16;
        for (int t = 0; t < ntab; ++t) {
            IntArgs ai = a;
            ai.h1 = e->d_h1 + NN * t;
            ai.g2 = e->d_g2 + N4 * t;
            for (int64_t r0 = 0; r0 < Dpad; r0 += chunk) {
                k_ell_build<<<e->sm_count * 8, 256, 0, e->stream>>>(ai, e->d_col + per * t, e->d_val + per * t, r0,
                                                                    std::min(Dpad, r0 + chunk));
                e->launches += 1;
            }
        }
        e->ham_kind = 2;
        e->ham_entries = D * a.stride;
        e->ell_stride_inst = ntab > 1 ? (int64_t)per : 0;
    } else {
        // on the fly: host-built string tables (the string lists do not depend on the
        // integrals; the integral tables are one set per instance), diagonal on the GPU
        std::vector<OtfTables> T(ntab);
        {
            const int hw = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
            std::vector<std::thread> pool;
            std::atomic<int> next{0};
            for (int w = 0; w < std::min(hw, ntab); ++w)
                pool.emplace_back([&]() {
                    for (int t; (t = next.fetch_add(1)) < ntab;) {
                        std::vector<double> hv(h1s + NN * t, h1s + NN * (t + 1)), gv(g2s + N4 * t, g2s + N4 * (t + 1));
                        build_otf_tables(e->B, hv, gv, T[t], t == 0);
                    }
                });
            for (auto &th : pool) th.join();
        }
        auto cat = [&](std::vector<double> OtfTables::*m) {
            std::vector<double> all;
            all.reserve((T[0].*m).size() * ntab);
            for (auto &x : T) all.insert(all.end(), (x.*m).begin(), (x.*m).end());
            return all;
        };
        const OtfTables &T0 = T[0];
        OtfArgs o{};
        o.N = N;
        o.P2 = T0.P2;
        o.nA = (int)e->B.nA;
        o.nB = (int)e->B.nB;
        o.nsa = T0.nsa;
        o.nda = T0.nda;
        o.nsb = T0.nsb;
        o.ndb = T0.ndb;
        bool ok = ham_upload(o.sa_rank, T0.sa_rank) && ham_upload(o.sa_code, T0.sa_code) &&
                  ham_upload(o.da_rank, T0.da_rank) && ham_upload(o.da_code, T0.da_code) &&
                  ham_upload(o.sb_rank, T0.sb_rank) && ham_upload(o.sb_code, T0.sb_code) &&
                  ham_upload(o.db_rank, T0.db_rank) && ham_upload(o.db_code, T0.db_code) &&
                  ham_upload(o.vss, cat(&OtfTables::vss)) && ham_upload(o.vab, cat(&OtfTables::vab)) &&
                  ham_upload(o.a_alpha, cat(&OtfTables::a_alpha)) && ham_upload(o.b_alpha, cat(&OtfTables::b_alpha)) &&
                  ham_upload(o.a_beta, cat(&OtfTables::a_beta)) && ham_upload(o.b_beta, cat(&OtfTables::b_beta));
        double *diag = nullptr;
        ok = ok && ham_alloc(diag, (size_t)D * ntab);
        if (!ok) return e->fail(AEGPU_ERR_NOMEM, "on-the-fly table allocation failed");
        o.diag = diag;
        o.shared = ntab == 1;
        cudaDeviceSynchronize();
        for (int t = 0; t < ntab; ++t) {
            IntArgs ai = a;
            ai.h1 = e->d_h1 + NN * t;
            ai.g2 = e->d_g2 + N4 * t;
            k_diag_build<<<e->sm_count * 8, 256, 0, e->stream>>>(ai, diag + (size_t)D * t);
            e->launches += 1;
        }
        const size_t smem = otf_smem_bytes(N, T0.P2, T0.nsa, T0.nda);
        int optin = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (smem + 1024 > (size_t)optin) return e->fail(AEGPU_ERR_UNSUPPORTED, "too many orbitals for the on-the-fly kernel");
        e->otf = o;
        e->otf_threads = (int)std::min<int64_t>(e->tune_otf_threads, ((int64_t)o.nB + 31) / 32 * 32);
        int smem_sm = 0;
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        if (!e->otf_threads_set && smem_sm > 0 && (size_t)smem_sm < 2 * (smem + 1024)) {
            // the string tables leave room for one CTA per SM (14 orbitals: ~150 KB): make
            // it as large as the registers allow (1024 threads), in equal beta chunks
            const int chunks = (o.nB + 1023) / 1024;
            e->otf_threads = ((o.nB + chunks - 1) / chunks + 31) / 32 * 32;
        }
        e->otf_chunks = (o.nB + e->otf_threads - 1) / e->otf_threads;
        const int64_t nparts = (int64_t)o.nA * e->otf_chunks;
        if (nparts > e->n_epart) {
            e->n_epart = nparts;
            int rc = e->alloc_instances(e->nb);
            if (rc) return rc;
        }
        e->ham_kind = 3;
        e->ham_entries = 0;
        e->ell_stride_inst = 0;
        e->flip_ok = e->B.na == e->B.nb;
    }
    e->ints_ntab = ntab;
    e->ints_mode_asked = mode_asked;
    e->h_valid = false;
    return stream_sync(e, "set_ham_integrals");
}

}  // namespace

extern "C" {

int aegpu_set_ham_integrals(aegpu_engine *e, const double *h1, const double *g2, int mode)
{
    if (!e || !h1 || !g2) return AEGPU_ERR_ARG;
    return set_integrals(e, h1, g2, 1, mode);
}

int aegpu_set_ham_integrals_batch(aegpu_engine *e, const double *h1s, const double *g2s, int mode)
{
    if (!e || !h1s || !g2s) return AEGPU_ERR_ARG;
    return set_integrals(e, h1s, g2s, e->nb, mode);
}

int aegpu_set_batch(aegpu_engine *e, int nb)
{
    if (!e) return AEGPU_ERR_ARG;
    if (nb < 1 || nb > 65535) return e->fail(AEGPU_ERR_ARG, "batch size must be in 1..65535");
    if (!e->d_start) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    if (nb == e->nb) return AEGPU_OK;
    // per-instance Hamiltonians were built for the old batch: they must be set again
    if (e->ham_per_instance) e->drop_ham();
    int rc = e->alloc_instances(nb);
    if (rc) return rc;
    return e->cuda_check("set_batch");
}

int aegpu_batch_size(const aegpu_engine *e) { return e ? e->nb : -1; }

int aegpu_set_active(aegpu_engine *e, const int *active)
{
    if (!e) return AEGPU_ERR_ARG;
    if (!e->d_active) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    std::vector<int> m(e->nb, 1);
    if (active)
        for (int b = 0; b < e->nb; ++b) m[b] = active[b] != 0;
    cudaMemcpyAsync(e->d_active, m.data(), m.size() * sizeof(int), cudaMemcpyHostToDevice, e->stream);
    e->psi_valid = e->h_valid = false;
    return stream_sync(e, "set_active");
}

int aegpu_set_tuning(aegpu_engine *e, int knob, int value)
{
    if (!e) return AEGPU_ERR_ARG;
    switch (knob) {
    case AEGPU_TUNE_PASS_OPS:
        if (value < 1 || value > kMaxWarpLayers) return e->fail(AEGPU_ERR_ARG, "pass size must be 1..6");
        if (e->d_start) return e->fail(AEGPU_ERR_STATE, "set the pass size before the problem");
        e->tune_pass_ops = value;
        return AEGPU_OK;
    case AEGPU_TUNE_CTAS_PER_SM:
        if (value < 1 || value > 64) return e->fail(AEGPU_ERR_ARG, "CTAs per SM must be 1..64");
        if (e->d_start) return e->fail(AEGPU_ERR_STATE, "set the CTAs per SM before the problem");
        e->tune_ctas_per_sm = value;
        return AEGPU_OK;
    case AEGPU_TUNE_OTF_THREADS:
        if (value < 64 || value > 1024 || value % 32) return e->fail(AEGPU_ERR_ARG, "threads must be 64..1024, x32");
        if (e->ham_kind) return e->fail(AEGPU_ERR_STATE, "set the thread count before the Hamiltonian");
        e->tune_otf_threads = value;
        e->otf_threads_set = true;
        return AEGPU_OK;
    case AEGPU_TUNE_PDL:
        if (value < -1 || value > 1) return e->fail(AEGPU_ERR_ARG, "programmatic dependent launch must be -1, 0 or 1");
        e->tune_pdl = value;
        e->drop_graph();
        return AEGPU_OK;
    case AEGPU_TUNE_REUSE_HPSI:
        if (value != 0 && value != 1) return e->fail(AEGPU_ERR_ARG, "H psi reuse must be 0 or 1");
        e->reuse_hpsi = value != 0;
        return AEGPU_OK;
    case AEGPU_TUNE_FLIP:
        if (value != 0 && value != 1) return e->fail(AEGPU_ERR_ARG, "the spin-flip half product must be 0 or 1");
        e->tune_flip = value != 0;
        e->drop_graph();
        e->h_valid = false;
        return AEGPU_OK;
    case AEGPU_TUNE_HALF:
        if (value != 0 && value != 1) return e->fail(AEGPU_ERR_ARG, "the spin-flip half passes must be 0 or 1");
        e->tune_half = value != 0;
        e->write_half_gate();
        e->psi_valid = e->h_valid = false;
        return AEGPU_OK;
    case AEGPU_TUNE_SPMV_TPR:
        if (value != 0 && value != 1 && value != 2 && value != 4 && value != 8)
            return e->fail(AEGPU_ERR_ARG, "threads per row must be 0 (by size), 1, 2, 4 or 8");
        if (e->grad_graph) return e->fail(AEGPU_ERR_STATE, "set the threads per row before the first evaluation");
        e->tune_spmv_tpr = value;
        return AEGPU_OK;
    default:
        return e->fail(AEGPU_ERR_ARG, "unknown tuning knob");
    }
}

int aegpu_flip_status(aegpu_engine *e, int *used)
{
    if (!e || !used) return AEGPU_ERR_ARG;
    if (!e->d_flip_used) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    if (!e->flip_tried) {
        std::fill(used, used + e->nb, 0);
        return AEGPU_OK;
    }
    if (stream_sync(e, "flip status")) return AEGPU_ERR_CUDA;
    cudaMemcpy(used, e->d_flip_used, sizeof(int) * e->nb, cudaMemcpyDeviceToHost);
    return e->cuda_check("flip status");
}

void aegpu_engine::write_half_gate()
{
    if (!d_half_gate) return;
    k_set_int<<<1, 1, 0, stream>>>(d_half_gate, half_static && start_sym && tune_half ? 1 : 0);
}

int aegpu_half_status(aegpu_engine *e, int *used)
{
    if (!e || !used) return AEGPU_ERR_ARG;
    if (!e->d_half) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    if (!e->half_static) {
        std::fill(used, used + e->nb, 0);
        return AEGPU_OK;
    }
    if (stream_sync(e, "half status")) return AEGPU_ERR_CUDA;
    cudaMemcpy(used, e->d_half, sizeof(int) * e->nb, cudaMemcpyDeviceToHost);
    return e->cuda_check("half status");
}

int aegpu_half_info(const aegpu_engine *e, int64_t *info)
{
    if (!e || !info) return AEGPU_ERR_ARG;
    // paired passes: their orbits' amplitudes and amplitude-layers; diagonal passes (as in
    // aegpu_fp64_work, over a <= b): the amplitudes with an active slot and the slot
    // activations, and as touched amplitudes every (a, b) with a <= b
    int64_t act = 0, al = 0, dact = 0, dslots = 0, ndiag = 0;
    for (auto &b : e->dblocks) {
        if (b.diagonal) {
            dact += (int64_t)b.active_h;
            dslots += (int64_t)b.slot_acts_h;
            ndiag++;
            continue;
        }
        act += (int64_t)b.active_h;
        al += (int64_t)b.amp_layers_h;
    }
    const int64_t W = e->W, nA = e->B.nA, Dh = nA * (nA + 1) / 2;
    info[0] = e->half_static ? 1 : 0;
    info[1] = e->half_static ? act + ndiag * Dh : 0;
    info[2] = e->half_static ? (al + act) * W + 4 * dact : 0;
    info[3] = e->half_static ? (2 * al + act) * W + al / 2 + 6 * dact + dslots : 0;
    return AEGPU_OK;
}

int aegpu_get_tuning(const aegpu_engine *e, int knob)
{
    if (!e) return -1;
    switch (knob) {
    case AEGPU_TUNE_PASS_OPS: return e->tune_pass_ops;
    case AEGPU_TUNE_CTAS_PER_SM: return e->tune_ctas_per_sm;
    case AEGPU_TUNE_OTF_THREADS: return e->tune_otf_threads;
    case AEGPU_TUNE_SPMV_TPR: return e->spmv_tpr();
    case AEGPU_TUNE_PDL: return e->pdl_on() ? 1 : 0;
    case AEGPU_TUNE_REUSE_HPSI: return e->reuse_hpsi ? 1 : 0;
    case AEGPU_TUNE_FLIP: return e->tune_flip ? 1 : 0;
    case AEGPU_TUNE_HALF: return e->tune_half ? 1 : 0;
    default: return -1;
    }
}

int aegpu_ham_info(const aegpu_engine *e, int *kind, int64_t *stored)
{
    if (!e) return AEGPU_ERR_ARG;
    if (kind) *kind = e->ham_kind;
    if (stored) *stored = e->ham_entries;
    return AEGPU_OK;
}

int aegpu_evolve(aegpu_engine *e, const double *angles, double *state)
{
    if (!e || !angles) return AEGPU_ERR_ARG;
    if (!e->d_psi) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    int rc = ensure_state(e, angles);
    if (rc) return rc;
    if (state)
        cudaMemcpyAsync(state, e->d_psi, e->vec_elems() * e->nb * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
    return stream_sync(e, "evolve");
}

int aegpu_energy(aegpu_engine *e, const double *angles, double *energy)
{
    if (!e || !angles || !energy) return AEGPU_ERR_ARG;
    if (!e->ham_kind) return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    int rc = AEGPU_OK;
    if (e->use_graph && !e->timing && !same_angles(e, angles)) {
        // pass constants + evolve + H psi + energy as one graph replay
        const size_t nang = e->excs.size() * (size_t)e->nb;
        cudaMemcpyAsync(e->d_ang, angles, nang * sizeof(double), cudaMemcpyHostToDevice, e->stream);
        if ((rc = launch_phases(e, 1))) return rc;
        e->cached_angles.assign(angles, angles + nang);
        e->psi_valid = e->h_valid = true;
    } else {
        rc = ensure_state(e, angles);
        if (rc) return rc;
        if (!e->h_valid) {
            rc = run_energy(e, e->d_scalar, e->nb);
            if (rc) return rc;
            e->h_valid = true;
        }
    }
    cudaMemcpyAsync(energy, e->d_scalar, e->nb * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
    return stream_sync(e, "energy");
}

int aegpu_gradient(aegpu_engine *e, const double *angles, double *energy, double *grad_ops)
{
    if (!e || !angles || !grad_ops) return AEGPU_ERR_ARG;
    if (!e->ham_kind) return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    const size_t nang = e->excs.size() * (size_t)e->nb;
    if (!e->reuse_hpsi) e->h_valid = false;  // recompute H psi, as the reference does (fusedevolve.cpp:2292)
    if (e->use_graph && !e->timing && !(same_angles(e, angles) && e->h_valid)) {
        // the whole evaluation as one graph replay (H psi is not cached for these angles)
        if (!e->grad_graph) {
            int rc = capture_grad_graph(e);
            if (rc) return rc;
        }
        cudaMemcpyAsync(e->d_ang, angles, nang * sizeof(double), cudaMemcpyHostToDevice, e->stream);
        if (cudaGraphLaunch(e->grad_graph, e->stream) != cudaSuccess) return e->cuda_check("graph launch");
        e->launches += e->graph_launches;
        if (energy) cudaMemcpyAsync(energy, e->d_scalar, e->nb * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
        cudaMemcpyAsync(grad_ops, e->d_grad, nang * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
        int rc = stream_sync(e, "gradient");
        if (rc) return rc;
        // psi is left evolved to these angles (the adjoint sweep reads checkpoints only)
        e->cached_angles.assign(angles, angles + nang);
        e->psi_valid = true;
        e->h_valid = false;
        return AEGPU_OK;
    }
    int rc = ensure_state(e, angles);
    if (rc) return rc;
    if (!e->h_valid) {
        rc = run_energy(e, e->d_scalar, e->nb);
        if (rc) return rc;
    }
    // the checkpointed sweep consumes H psi and leaves psi as it is
    rc = e->use_graph && !e->timing ? launch_phases(e, 2) : run_backward(e, e->d_grad, e->nb);
    if (rc) return rc;
    e->h_valid = false;
    if (energy) cudaMemcpyAsync(energy, e->d_scalar, e->nb * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
    cudaMemcpyAsync(grad_ops, e->d_grad, e->excs.size() * e->nb * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
    return stream_sync(e, "gradient");
}

// Projected sweep (FusedEvolve::evolveDerivativeProj, fusedevolve.cpp:2814-2880):
// overlap[b] = <proj_b|psi_b(theta_b)>, grad[b][op] = d overlap / d theta_op.
int aegpu_gradient_proj(aegpu_engine *e, const double *angles, const double *proj, double *overlap, double *grad_ops)
{
    if (!e || !angles || !proj || !grad_ops) return AEGPU_ERR_ARG;
    if (!e->d_psi) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    // the fixed bra has no mirror symmetry: a full forward sweep (its checkpoints) for
    // the full adjoint sweep
    const bool gate = e->half_static && e->start_sym && e->tune_half;
    if (gate) {
        e->tune_half = false;
        e->write_half_gate();
        e->psi_valid = false;
    }
    int rc = ensure_state(e, angles);
    if (gate) {
        e->tune_half = true;
        e->write_half_gate();
    }
    if (rc) return rc;
    const int64_t n = (int64_t)e->vec_elems();
    cudaMemcpyAsync(e->d_h, proj, (size_t)n * e->nb * sizeof(double), cudaMemcpyHostToDevice, e->stream);
    e->h_valid = false;
    const int grid = (int)std::min<int64_t>(std::max<int64_t>(1, (n + 255) / 256), e->n_epart);
    k_dot<<<dim3(grid, e->nb), 256, 0, e->stream>>>(e->d_h, e->d_psi, n, e->d_epart, e->d_active);
    k_reduce_sum<<<e->nb, 256, 0, e->stream>>>(e->d_epart, grid, e->d_scalar, 1.0, e->d_active);
    e->launches += 2;
    rc = run_backward(e, e->d_grad, e->nb, 1.0, false);
    if (rc) return rc;
    if (overlap) cudaMemcpyAsync(overlap, e->d_scalar, e->nb * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
    cudaMemcpyAsync(grad_ops, e->d_grad, e->excs.size() * e->nb * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
    return stream_sync(e, "gradient_proj");
}

int aegpu_gradient_dev(aegpu_engine *e, const double *angles_dev, double *energy_dev, double *grad_dev, void *stream)
{
    if (!e || !angles_dev || !grad_dev) return AEGPU_ERR_ARG;
    if (!e->ham_kind) return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    const size_t nang = e->excs.size() * (size_t)e->nb;
    if (e->use_graph && !e->timing) {
        if (!e->grad_graph) {
            int rc = capture_grad_graph(e);
            if (rc) return rc;
        }
        cudaStream_t st = stream ? (cudaStream_t)stream : e->stream;
        cudaMemcpyAsync(e->d_ang, angles_dev, nang * sizeof(double), cudaMemcpyDeviceToDevice, st);
        if (cudaGraphLaunch(e->grad_graph, st) != cudaSuccess) return e->cuda_check("graph launch");
        e->launches += e->graph_launches;
        if (energy_dev) cudaMemcpyAsync(energy_dev, e->d_scalar, e->nb * sizeof(double), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(grad_dev, e->d_grad, nang * sizeof(double), cudaMemcpyDeviceToDevice, st);
        e->psi_valid = e->h_valid = false;
        return e->cuda_check("gradient_dev");
    }
    cudaStream_t saved = e->stream;
    if (stream) e->stream = (cudaStream_t)stream;
    std::array<cudaEvent_t, 4> ev{};
    if (e->timing)
        for (auto &x : ev) x = e->next_event();
    if (e->timing) cudaEventRecord(ev[0], e->stream);
    int rc = upload_angles(e, angles_dev, false, e->nb);
    if (!rc) rc = run_evolve(e, e->nb);
    if (e->timing) cudaEventRecord(ev[1], e->stream);
    if (!rc) rc = run_energy(e, energy_dev ? energy_dev : e->d_scalar, e->nb);
    if (e->timing) cudaEventRecord(ev[2], e->stream);
    if (!rc) rc = run_backward(e, grad_dev, e->nb);
    if (e->timing) {
        cudaEventRecord(ev[3], e->stream);
        e->ev_marks.push_back(ev);
    }
    e->stream = saved;
    e->psi_valid = e->h_valid = false;
    return rc;
}

int aegpu_io_dev(aegpu_engine *e, double **angles_dev, double **energy_dev, double **grad_dev)
{
    if (!e) return AEGPU_ERR_ARG;
    if (!e->d_ang) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    if (angles_dev) *angles_dev = e->d_ang;
    if (energy_dev) *energy_dev = e->d_scalar;
    if (grad_dev) *grad_dev = e->d_grad;
    return AEGPU_OK;
}

// Evaluate every instance at the angles already in the io buffer (graph replay).
int aegpu_launch_io(aegpu_engine *e, void *stream)
{
    if (!e) return AEGPU_ERR_ARG;
    if (!e->ham_kind) return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    if (!e->grad_graph) {
        int rc = capture_grad_graph(e);
        if (rc) return rc;
    }
    cudaStream_t st = stream ? (cudaStream_t)stream : e->stream;
    if (cudaGraphLaunch(e->grad_graph, st) != cudaSuccess) return e->cuda_check("graph launch");
    e->launches += e->graph_launches;
    e->psi_valid = e->h_valid = false;
    return e->cuda_check("launch_io");
}

// Host <-> io buffer copies on `stream` (NULL: the engine's stream); the get
// synchronises that stream.
int aegpu_io_put_angles(aegpu_engine *e, const double *angles, void *stream)
{
    if (!e || !angles) return AEGPU_ERR_ARG;
    if (!e->d_ang) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    cudaStream_t st = stream ? (cudaStream_t)stream : e->stream;
    cudaMemcpyAsync(e->d_ang, angles, e->excs.size() * e->nb * sizeof(double), cudaMemcpyHostToDevice, st);
    return e->cuda_check("io_put_angles");
}

int aegpu_io_get_results(aegpu_engine *e, double *energy, double *grad, void *stream)
{
    if (!e) return AEGPU_ERR_ARG;
    if (!e->d_ang) return e->fail(AEGPU_ERR_STATE, "set the problem first");
    cudaStream_t st = stream ? (cudaStream_t)stream : e->stream;
    if (energy) cudaMemcpyAsync(energy, e->d_scalar, e->nb * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (grad) cudaMemcpyAsync(grad, e->d_grad, e->excs.size() * e->nb * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaError_t rc = cudaStreamSynchronize(st);
    if (rc != cudaSuccess) return e->fail(AEGPU_ERR_CUDA, std::string("io_get_results: ") + cudaGetErrorString(rc));
    return e->cuda_check("io_get_results");
}

}  // extern "C"

struct aegpu_group {
    std::vector<aegpu_engine *> engines;
    std::vector<int64_t> generations;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t stream = nullptr;  // used when the caller passes none
    cudaStream_t last = nullptr;    // stream of the latest launch
    int64_t launches = 0;
    ~aegpu_group()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (stream) cudaStreamDestroy(stream);
    }
};

extern "C" {

int aegpu_group_create(aegpu_group **out, aegpu_engine *const *engines, int n)
{
    if (!out || !engines || n < 1) return AEGPU_ERR_ARG;
    *out = nullptr;
    auto *g = new aegpu_group();
    cudaGraph_t parent = nullptr;
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaGraphCreate(&parent, 0) != cudaSuccess) {
        cudaGetLastError();
        delete g;
        return AEGPU_ERR_CUDA;
    }
    int rc = AEGPU_OK;
    for (int i = 0; i < n && !rc; ++i) {
        aegpu_engine *e = engines[i];
        if (!e || !e->ham_kind) {
            rc = e ? e->fail(AEGPU_ERR_STATE, "no Hamiltonian set") : AEGPU_ERR_ARG;
            break;
        }
        if (!e->grad_graph_def) rc = capture_grad_graph(e);
        if (rc) break;
        // independent child graphs: the engines' evaluations may run concurrently
        cudaGraphNode_t node;
        if (cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, e->grad_graph_def) != cudaSuccess) {
            cudaGetLastError();
            rc = AEGPU_ERR_CUDA;
            break;
        }
        g->engines.push_back(e);
        g->generations.push_back(e->generation);
        g->launches += e->graph_launches;
    }
    if (!rc && cudaGraphInstantiate(&g->exec, parent, 0) != cudaSuccess) {
        cudaGetLastError();
        rc = AEGPU_ERR_CUDA;
    }
    cudaGraphDestroy(parent);
    if (rc) {
        delete g;
        return rc;
    }
    *out = g;
    return AEGPU_OK;
}

int aegpu_group_launch(aegpu_group *g, void *stream)
{
    if (!g) return AEGPU_ERR_ARG;
    for (size_t i = 0; i < g->engines.size(); ++i)
        if (g->engines[i]->generation != g->generations[i])
            return g->engines[i]->fail(AEGPU_ERR_STATE, "engine changed since the group was created");
    g->last = stream ? (cudaStream_t)stream : g->stream;
    if (cudaGraphLaunch(g->exec, g->last) != cudaSuccess) {
        cudaGetLastError();
        return AEGPU_ERR_CUDA;
    }
    for (auto *e : g->engines) {
        e->launches += e->graph_launches;
        e->psi_valid = e->h_valid = false;
    }
    return AEGPU_OK;
}

int aegpu_group_sync(aegpu_group *g)
{
    if (!g) return AEGPU_ERR_ARG;
    if (g->last && cudaStreamSynchronize(g->last) != cudaSuccess) {
        cudaGetLastError();
        return AEGPU_ERR_CUDA;
    }
    return AEGPU_OK;
}

int64_t aegpu_group_launch_count(const aegpu_group *g) { return g ? g->launches : -1; }

void aegpu_group_destroy(aegpu_group *g) { delete g; }

int aegpu_use_graphs(aegpu_engine *e, int enable)
{
    if (!e) return AEGPU_ERR_ARG;
    e->use_graph = enable != 0;
    return AEGPU_OK;
}

int aegpu_energy_dev(aegpu_engine *e, const double *angles_dev, double *energy_dev, void *stream)
{
    if (!e || !angles_dev || !energy_dev) return AEGPU_ERR_ARG;
    if (!e->ham_kind) return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    cudaStream_t saved = e->stream;
    if (stream) e->stream = (cudaStream_t)stream;
    int rc = upload_angles(e, angles_dev, false, e->nb);
    if (!rc) rc = run_evolve(e, e->nb);
    if (!rc) rc = run_energy(e, energy_dev, e->nb);
    e->stream = saved;
    e->psi_valid = e->h_valid = false;
    return rc;
}

int aegpu_state_dev(aegpu_engine *e, const double **psi, const double **hpsi)
{
    if (!e) return AEGPU_ERR_ARG;
    if (psi) *psi = e->d_psi;
    if (hpsi) *hpsi = e->d_h;
    return AEGPU_OK;
}

int aegpu_apply_h(aegpu_engine *e, const double *x, double *y)
{
    if (!e || !x || !y) return AEGPU_ERR_ARG;
    if (!e->ham_kind) return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    // the engine's own scratch vectors (the cached H psi is given up)
    const size_t n = e->vec_elems() * e->nb;
    e->h_valid = false;
    cudaMemcpyAsync(e->d_tmp, x, n * sizeof(double), cudaMemcpyHostToDevice, e->stream);
    int rc = run_apply(e, e->d_tmp, e->d_h, nullptr, e->nb, nullptr, false);
    if (!rc) {
        cudaMemcpyAsync(y, e->d_h, n * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
        rc = stream_sync(e, "apply_h");
    }
    return rc;
}

}  // extern "C"

// Energy Hessian (proj = nullptr; FusedEvolve::evolveHessian, fusedevolve.cpp:2437-2780)
// or projected Hessian of <proj|psi(theta)> (FusedEvolve::evolveHessianProj,
// fusedevolve.cpp:2882-3183: no T^T H T term, second-derivative sweeps against the
// fixed bra, factor 1); energy receives <psi|H psi> or <proj|psi>.

static int hessian_impl(aegpu_engine *e, const double *angles, const int *param, const double *scale, int nparams,
                        const double *proj, double *energy, double *grad_comp, double *hess_comp,
                        double *metric = nullptr)
{
    NvtxRange r(proj ? "aegpu projected Hessian" : "aegpu Hessian");
    if (!e || !angles || !param || !scale || nparams < 1 || !hess_comp) return AEGPU_ERR_ARG;
    if (!proj && !e->ham_kind) return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    if (e->nb != 1) return e->fail(AEGPU_ERR_UNSUPPORTED, "the Hessian needs a batch size of 1");
    if (e->excs.size() > 65535) return e->fail(AEGPU_ERR_UNSUPPORTED, "the Hessian supports at most 65535 operators");
    const int nops = (int)e->excs.size();
    const int W = e->W;
    const int64_t D = (int64_t)e->B.D;
    const size_t n = (size_t)D * W;
    for (int o = 0; o < nops; ++o)
        if (param[o] < 0 || param[o] >= nparams) return e->fail(AEGPU_ERR_ARG, "parameter index out of range");
    const int V = nparams + 1;
    // parameter -> (application position, scale) lists
    std::vector<int> pptr(nparams + 1, 0), ppos, pcnt(nparams, 0);
    std::vector<double> pscale;
    for (int o = 0; o < nops; ++o) pcnt[param[o]]++;
    for (int m = 0; m < nparams; ++m) pptr[m + 1] = pptr[m] + pcnt[m];
    ppos.assign(nops, 0);
    pscale.assign(nops, 0);
    std::vector<int> fill(pptr.begin(), pptr.end() - 1);
    for (int o = 0; o < nops; ++o) {
        ppos[fill[param[o]]] = e->pos_of_op[o];
        pscale[fill[param[o]]++] = scale[o];
    }
    // scratch (kept between calls for the same parameter count): tangents by
    // application position, compressed tangents and H * them, Gram matrices
    auto &hs = e->hess;
    if (hs.V != V) {
        for (auto &pa : hs.allocs) e->release(pa.first, pa.second);
        hs = aegpu_engine::HessScratch{};
        int64_t maxpart = 0;
        for (auto &b : e->dblocks)
            maxpart = std::max<int64_t>(maxpart, (int64_t)std::max(b.ntiles, b.wgrid) * nops * kMaxSlots);
        auto get = [&](auto *&ptr, size_t count) {
            using T = std::remove_reference_t<decltype(*ptr)>;
            ptr = e->alloc<T>(count);
            hs.allocs.push_back({(void *)ptr, std::max<size_t>(count, 1) * sizeof(T)});
            return ptr != nullptr;
        };
        const int64_t ngram = std::max(gram_scratch_doubles(V, 1, (int64_t)n, e->sm_count),
                                       gemv_scratch_doubles(V, e->sm_count));
        bool ok = get(hs.T, n * nops) && get(hs.TC, n * V) && get(hs.HTC, n * V) && get(hs.THT, (size_t)V * V) &&
                  get(hs.MET, (size_t)V * V) && get(hs.gram, (size_t)ngram) &&
                  get(hs.Hops, (size_t)nops * nops) && get(hs.hpart, maxpart) && get(hs.pptr, (size_t)nparams + 1) &&
                  get(hs.ppos, (size_t)nops) && get(hs.pscale, (size_t)nops) &&
                  get(hs.flip, (size_t)V * 2 * e->sm_count) && get(hs.vmap, (size_t)nops) && get(hs.mpos, (size_t)nops);
        if (!ok) {
            for (auto &pa : hs.allocs) e->release(pa.first, pa.second);
            hs = aegpu_engine::HessScratch{};
            return e->fail(AEGPU_ERR_NOMEM, "Hessian scratch allocation failed");
        }
        hs.V = V;
    }
    double *T = hs.T, *TC = hs.TC, *HTC = hs.HTC, *THT = hs.THT, *Hops = hs.Hops, *hpart = hs.hpart;
    int *d_pptr = hs.pptr, *d_ppos = hs.ppos;
    double *d_pscale = hs.pscale;
    cudaStream_t s = e->stream;
    cudaMemcpyAsync(d_pptr, pptr.data(), pptr.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_ppos, ppos.data(), ppos.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_pscale, pscale.data(), pscale.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    int rc = upload_angles(e, angles, true, 1, false);
    if (rc) return rc;
    // Half tangents: where the angles pass the half passes' test (the circuit commutes
    // with the exchange of the alpha and beta strings), the tangent of an operator's
    // mirror is the mirror image of its own, so only one of each pair (the earlier by
    // position) is carried through the passes and swept; the compressed tangents read
    // the other as a mirror image, and every second-derivative pair also stands for its
    // mirror pair.  Not for the projected Hessian (its bra has no such symmetry) nor for
    // circuits with diagonal passes.
    bool hm = false;
    bool all_paired = true;
    for (auto &b : e->dblocks) all_paired = all_paired && !b.diagonal;
    if (e->half_static && !proj && all_paired) {
        int h = 0;
        cudaMemcpyAsync(&h, e->d_half, sizeof(int), cudaMemcpyDeviceToHost, s);
        if ((rc = stream_sync(e, "hessian"))) return rc;
        hm = h != 0;
    }
    const int nbl = (int)e->dblocks.size();
    std::vector<int> nrep_before(nbl, 0), nrep_upto(nbl, 0);
    if (hm) {
        std::vector<char> rep(nops);
        std::vector<int> vmap, mpos(nops, -1);
        for (int v = 0; v < nops; ++v) {
            rep[v] = v <= e->pos_of_op[e->mirror[e->perm[v]]];
            if (rep[v]) vmap.push_back(v);
        }
        for (int bi = 0; bi < nbl; ++bi) {
            const int p0 = e->block_pos0[bi], p1 = p0 + e->dblocks[bi].nslots;
            for (int v = 0; v < p1; ++v)
                if (rep[v]) {
                    nrep_upto[bi]++;
                    if (v < p0) nrep_before[bi]++;
                }
        }
        for (int k = 0; k < nops; ++k)
            if (!rep[ppos[k]]) mpos[k] = e->pos_of_op[e->mirror[e->perm[ppos[k]]]];
        cudaMemcpyAsync(hs.vmap, vmap.data(), vmap.size() * sizeof(int), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(hs.mpos, mpos.data(), mpos.size() * sizeof(int), cudaMemcpyHostToDevice, s);
        if ((rc = stream_sync(e, "hessian"))) return rc;  // the host vectors go out of scope
    }
    cudaMemsetAsync(T, 0, n * nops * sizeof(double), s);
    cudaMemsetAsync(Hops, 0, (size_t)nops * nops * sizeof(double), s);
    cudaMemcpyAsync(e->d_psi, e->d_start, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    // 1. forward: tangents of every block, earlier tangents carried along
    for (size_t bi = 0; bi < e->dblocks.size(); ++bi) {
        auto &b = e->dblocks[bi];
        const int p0 = e->block_pos0[bi];
        if (b.diagonal) {
            if (p0 > 0) k_diag_rot<<<kDiagGrid, 256, 0, s>>>(e->diag_args(b, 1.0, false), T, n, p0, nullptr, 0, 0);
            k_diag_tangent<<<kDiagGrid, 256, 0, s>>>(e->diag_args(b, 1.0, false), e->d_psi, T, n, e->d_tpos);
            e->launches += p0 > 0 ? 2 : 1;
        } else if (b.ntiles) {
            BlockArgs a = e->block_args((int)bi, 1.0);
            // earlier tangents carried through the pass by the warp-register pass kernel:
            // the p0 tangents are its "instances" (same angles: strides 0, no mask)
            BlockArgs av = a;
            av.pc_stride = av.sig_stride = 0;
            av.active = nullptr;
            if (hm) av.vmap = hs.vmap;
            const int ncarry = hm ? nrep_before[bi] : p0;
            const dim3 gv(b.wgrid, std::min(ncarry, 65535));
            if (W == 1) {
                if (ncarry > 0 && b.nwtasks) k_warp_rot<1><<<gv, kWarpThreads, 0, s>>>(av, b.wtasks, b.nwtasks, T, n, nullptr, 0);
                k_block_tangent<1><<<b.ntiles, kRotThreads, e->rot_smem(1), s>>>(a, e->d_psi, T, n, e->d_tpos);
            } else {
                if (ncarry > 0 && b.nwtasks) k_warp_rot<2><<<gv, kWarpThreads, 0, s>>>(av, b.wtasks, b.nwtasks, T, n, nullptr, 0);
                k_block_tangent<2><<<b.ntiles, kRotThreads, e->rot_smem(1), s>>>(a, e->d_psi, T, n, e->d_tpos);
            }
            e->launches += 2;
        }
    }
    // 2. compressed tangents (column-major: column v is T_C v, column P is psi), H on all
    //    of them as one batched product, Gram matrix 2 T_C^T H T_C
    k_tc_build<<<e->sm_count * 8, 256, 0, s>>>(T, n, e->d_psi, d_pptr, d_ppos, d_pscale, nparams, W, D, TC,
                                               hm ? hs.mpos : nullptr, e->db);
    e->launches += 1;
    // With re / im interleaved, the real dot product over the D*W doubles of two columns
    // is Re(a^dagger b), so every contraction below runs on real columns of n doubles.
    if (metric) {
        // g = Re(T_C^dagger T_C) over the P tangent columns (tupsquantities.cpp:386-389),
        // upper triangle
        e->launches += gram_upper(TC, (int64_t)n, TC, (int64_t)n, (int64_t)n, 1, nparams, 1.0, hs.MET, nullptr, nparams,
                                  hs.gram, e->sm_count, s);
    }
    if (proj) {
        // projected: Re <proj|T_C v> for every column (the last is <proj|psi>;
        // fusedevolve.cpp:3053-3062), bra for the sweeps
        cudaMemcpyAsync(e->d_h, proj, n * sizeof(double), cudaMemcpyHostToDevice, s);
        e->launches += gemv_t(TC, (int64_t)n, (int64_t)n, V, e->d_h, 1.0, THT, hs.gram, e->sm_count, s);
    } else {
        // the V columns as V instances of the H product (the matrix or tables are shared)
        // (every compressed tangent of a spin-adapted ansatz is flip-invariant when psi is:
        // the half product where all columns of a CTA pass the test)
        rc = run_apply(e, TC, HTC, nullptr, V, nullptr, false, true, hs.flip, nullptr);
        if (rc) return rc;
        // 2 Re(T_C^dagger H T_C) (fusedevolve.cpp:2633-2650) is symmetric (H is): only its
        // upper triangle is computed; column P holds the gradient and twice the energy
        e->launches += gram_upper(TC, (int64_t)n, HTC, (int64_t)n, (int64_t)n, 1, V, 2.0, THT, nullptr, V, hs.gram,
                                  e->sm_count, s);
        // H psi for the backward sweeps: the last column
        cudaMemcpyAsync(e->d_h, HTC + (size_t)nparams * n, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    }
    // 3. second-derivative sweeps
    for (int bi = (int)e->dblocks.size() - 1; bi >= 0; --bi) {
        auto &b = e->dblocks[bi];
        const int p0 = e->block_pos0[bi];
        const int nvec = hm ? nrep_upto[bi] : p0 + b.nslots;
        if (b.diagonal) {
            dim3 g(kDiagGrid, nvec);
            k_diag_hess<<<g, 256, 0, s>>>(e->diag_args(b, -1.0, false), e->d_h, T, n, nvec, p0, hpart);
            k_hess_reduce<<<(nvec * b.nslots * 32 + 255) / 256, 256, 0, s>>>(hpart, kDiagGrid, nvec, b.nslots, e->d_pos_op,
                                                                            b.ops, p0, Hops, nops, proj ? 1.0 : 2.0,
                                                                            nullptr, nullptr, nullptr);
            k_diag_rot<<<kDiagGrid, 256, 0, s>>>(e->diag_args(b, -1.0, false), e->d_h, 0, 1, nullptr, 0, 0);
            e->launches += 3;
        } else if (b.nwtasks) {
            // warp-register pass kernels, adjoint direction, one vector per grid.y row
            BlockArgs a = e->block_args(bi, -1.0);
            a.pc_stride = a.sig_stride = 0;
            a.active = nullptr;
            BlockArgs at = a;  // the tangents: the carried ones only with the half tangents
            if (hm) at.vmap = hs.vmap;
            const dim3 g(b.wgrid, std::min(nvec, 65535));
            if (nvec > 0) {
                if (W == 1)
                    k_warp_hess<1><<<g, kWarpThreads, 0, s>>>(at, b.wtasks, b.nwtasks, e->d_h, T, n, nvec, p0, hpart);
                else
                    k_warp_hess<2><<<g, kWarpThreads, 0, s>>>(at, b.wtasks, b.nwtasks, e->d_h, T, n, nvec, p0, hpart);
                k_hess_reduce<<<(nvec * b.nslots * 32 + 255) / 256, 256, 0, s>>>(
                    hpart, b.wgrid, nvec, b.nslots, e->d_pos_op, b.ops, p0, Hops, nops, proj ? 1.0 : 2.0,
                    hm ? hs.vmap : nullptr, hm ? e->d_mirror : nullptr, hm ? e->d_tpos : nullptr);
            }
            // the bra back through the pass
            if (W == 1)
                k_warp_rot<1><<<b.wgrid, kWarpThreads, 0, s>>>(a, b.wtasks, b.nwtasks, e->d_h, 0, nullptr, 0);
            else
                k_warp_rot<2><<<b.wgrid, kWarpThreads, 0, s>>>(a, b.wtasks, b.nwtasks, e->d_h, 0, nullptr, 0);
            e->launches += 3;
        }
    }
    std::vector<double> hops((size_t)nops * nops), tht((size_t)V * V);
    cudaMemcpyAsync(hops.data(), Hops, hops.size() * 8, cudaMemcpyDeviceToHost, s);
    if (metric) cudaMemcpyAsync(metric, hs.MET, (size_t)nparams * nparams * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(tht.data(), THT, (proj ? (size_t)V : tht.size()) * 8, cudaMemcpyDeviceToHost, s);
    rc = stream_sync(e, "hessian");
    e->psi_valid = e->h_valid = false;
    if (rc) return rc;
    if (metric)  // upper triangle (column-major) to the full symmetric matrix
        for (int j = 0; j < nparams; ++j)
            for (int i = j + 1; i < nparams; ++i) metric[(size_t)j * nparams + i] = metric[(size_t)i * nparams + j];
    if (proj) {
        // Hessian = C Hops C^T (fusedevolve.cpp:3171); gradient and overlap from <proj|T_C>
        for (size_t k = 0; k < (size_t)nparams * nparams; ++k) hess_comp[k] = 0.0;
        for (int a = 0; a < nops; ++a)
            for (int b = 0; b < nops; ++b)
                hess_comp[(size_t)param[a] * nparams + param[b]] += scale[a] * scale[b] * hops[(size_t)a * nops + b];
        if (grad_comp)
            for (int i = 0; i < nparams; ++i) grad_comp[i] = tht[i];
        if (energy) *energy = tht[nparams];
        return AEGPU_OK;
    }
    // Hessian = C Hops C^T + THT (fusedevolve.cpp:2762-2763); THT column-major V x V,
    // upper triangle (i <= j at tht[j * V + i])
    for (int i = 0; i < nparams; ++i)
        for (int j = 0; j < nparams; ++j)
            hess_comp[(size_t)i * nparams + j] = i <= j ? tht[(size_t)j * V + i] : tht[(size_t)i * V + j];
    for (int a = 0; a < nops; ++a)
        for (int b = 0; b < nops; ++b)
            hess_comp[(size_t)param[a] * nparams + param[b]] += scale[a] * scale[b] * hops[(size_t)a * nops + b];
    if (grad_comp)
        for (int i = 0; i < nparams; ++i) grad_comp[i] = tht[(size_t)nparams * V + i];
    if (energy) *energy = tht[(size_t)nparams * V + nparams] / 2.0;
    return AEGPU_OK;
}

extern "C" {

int aegpu_hessian(aegpu_engine *e, const double *angles, const int *param, const double *scale, int nparams,
                  double *energy, double *grad_comp, double *hess_comp)
{
    return hessian_impl(e, angles, param, scale, nparams, nullptr, energy, grad_comp, hess_comp);
}

int aegpu_hessian_proj(aegpu_engine *e, const double *angles, const int *param, const double *scale, int nparams,
                       const double *proj, double *overlap, double *grad_comp, double *hess_comp)
{
    if (!proj) return AEGPU_ERR_ARG;
    return hessian_impl(e, angles, param, scale, nparams, proj, overlap, grad_comp, hess_comp);
}

int aegpu_hessian_metric(aegpu_engine *e, const double *angles, const int *param, const double *scale, int nparams,
                         double *energy, double *grad_comp, double *hess_comp, double *metric)
{
    if (!metric) return AEGPU_ERR_ARG;
    return hessian_impl(e, angles, param, scale, nparams, nullptr, energy, grad_comp, hess_comp, metric);
}

}  // extern "C"

// ------------------------------------------------------------------ properties --
// The quantities TUPSQuantities::writeProperties and doSubspaceDiagonalisation report
// (tupsquantities.cpp:185-568, 1600-1769): the lowest eigenpair of H, overlaps of
// evolved states with it, and the Hamiltonian / overlap matrices of a set of states.

// Lanczos three-term step on the device: w -= alpha v + beta v_prev (beta, v_prev
// absent on the first step), with alpha and beta read from device memory.
__global__ void k_lanczos_update(double *__restrict__ w, const double *__restrict__ v, const double *__restrict__ vp,
                                 const double *alpha, const double *beta, int64_t n)
{
    const double a = *alpha, b = vp ? *beta : 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        w[i] = vp ? w[i] - a * v[i] - b * vp[i] : w[i] - a * v[i];
}

// Small device scratch of the properties pass: scalar results and the partial sums of
// the dot products (dense.cu), allocated once per engine.
static double *small_scratch(aegpu_engine *e)
{
    if (!e->d_small) e->d_small = e->alloc<double>(e->small_len());
    return e->d_small;
}

extern "C" {

}  // extern "C"

// Lanczos with full reorthogonalisation for the nst lowest eigenpairs of H in the sector,
// restarted after `basis` products.  nst = 1 starts from the initial state and restarts
// from the Ritz vector; nst > 1 starts from a seeded pseudo-random real vector (so that
// eigenstates of every spin symmetry of the sector are present, as in a dense
// eigensolver) and restarts from the sum of the nst Ritz vectors.  The vectors stay in
// e->d_ground (nst columns).  Signs: <start|v> > 0, or, where that overlap vanishes, the
// largest-magnitude entry positive.
static int lanczos_lowest(aegpu_engine *e, int nst, double tol, int basis, int max_products, double *eigenvalues,
                          double *residuals, int *products)
{
    NvtxRange r("aegpu lowest eigenpairs");
    if (!e->ham_kind) return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    if (e->nb != 1) return e->fail(AEGPU_ERR_UNSUPPORTED, "the ground state needs a batch size of 1");
    const size_t n = e->vec_elems();
    if ((size_t)nst > n) return e->fail(AEGPU_ERR_ARG, "more eigenstates than determinants");
    const int m = (int)std::min<size_t>((size_t)std::max(basis, nst + 1), n);
    if (m + 1 > 4096) return e->fail(AEGPU_ERR_UNSUPPORTED, "Lanczos basis larger than 4095 vectors");
    e->ground_valid = false;
    if (e->n_ground < nst) {
        if (e->d_ground) e->release(e->d_ground, (size_t)e->n_ground * n * sizeof(double));
        e->d_ground = e->alloc<double>(n * (size_t)nst);
        e->n_ground = e->d_ground ? nst : 0;
        if (!e->d_ground) return e->fail(AEGPU_ERR_NOMEM, "ground state allocation failed");
    }
    double *sm = small_scratch(e);
    if (!sm) return e->fail(AEGPU_ERR_NOMEM, "scratch allocation failed");
    // basis vectors; reorthogonalisation coefficients, alpha / beta of the recurrence, a
    // spare slot, a repeat flag and the partial sums of gemv_t
    const size_t nscal = (size_t)(m + 1) + 2 * (size_t)m + 2 + (size_t)gemv_scratch_doubles(m + 1, e->sm_count);
    double *Vb = e->alloc<double>((size_t)(m + 1) * n);
    double *scal = e->alloc<double>(nscal);
    auto release = [&] {
        e->release(Vb, (size_t)(m + 1) * n * sizeof(double));
        e->release(scal, nscal * sizeof(double));
    };
    if (!Vb || !scal) {
        release();
        return e->fail(AEGPU_ERR_NOMEM, "Lanczos basis allocation failed");
    }
    double *d_c = scal, *d_alpha = scal + (m + 1), *d_beta = d_alpha + m, *d_wn = d_beta + m, *d_part = d_wn + 2;
    int *d_again = (int *)(d_wn + 1);
    double *d_res = sm, *d_dpart = sm + 4;
    cudaStream_t s = e->stream;
    const int64_t ni = (int64_t)n;
    const int vgrid = (int)std::min<int64_t>((ni + 255) / 256, (int64_t)e->sm_count * 8);
    auto host_scalars = [&](int k, double *out) {
        cudaMemcpyAsync(out, d_res, k * sizeof(double), cudaMemcpyDeviceToHost, s);
        return stream_sync(e, "Lanczos");
    };
    // Lanczos with full reorthogonalisation, restarted when the basis is full.  The
    // recurrence runs on the device (alpha and beta stay in device memory); the host reads
    // them and checks the Ritz pairs every kCheck products.
    constexpr int kCheck = 8;
    if (nst == 1) {
        cudaMemcpyAsync(e->d_ground, e->d_start, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    } else {
        std::vector<double> r0(n);
        uint64_t st = 0x9e3779b97f4a7c15ull;
        for (size_t i = 0; i < n; ++i) {
            st += 0x9e3779b97f4a7c15ull;
            uint64_t z = st;
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
            z ^= z >> 31;
            // complex mode: imaginary parts zero (H is real, so the eigenvectors stay real)
            r0[i] = (e->W == 2 && (i & 1)) ? 0.0 : (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
        }
        cudaMemcpyAsync(e->d_ground, r0.data(), n * sizeof(double), cudaMemcpyHostToDevice, s);
        if (int rc = stream_sync(e, "Lanczos start")) {
            release();
            return rc;
        }
    }
    int prod = 0, rc = 0;
    bool done = false;
    std::vector<double> al, be, sv, th;
    // nst = 1: from a start with psi(a,b) = psi(b,a) every Krylov vector keeps that
    // symmetry exactly (H preserves it, and the recurrence, the reorthogonalisation and
    // the restarts update mirrored amplitudes by the same arithmetic), so the products
    // may take the spin-flip half product; each tests its input first (run_apply)
    const bool flip = nst == 1;
    while (!done) {
        double nx = 0.0;
        e->launches += ae::dot(e->d_ground, e->d_ground, ni, 1, d_res, 1, d_dpart, e->sm_count, s);
        if ((rc = host_scalars(1, &nx))) {
            release();
            return rc;
        }
        if (!(nx > 0.0)) {
            release();
            return e->fail(AEGPU_ERR_STATE, "the start vector is zero");
        }
        e->launches += ae::axpby(Vb, e->d_ground, ni, 0.0, 1.0 / nx, nullptr, s);
        int k = 0, checked = 0;
        for (int j = 0; j < m && !done; ++j) {
            double *v = Vb + (size_t)j * n, *w = Vb + (size_t)(j + 1) * n;
            if ((rc = run_apply(e, v, w, nullptr, 1, nullptr, false, flip, flip ? e->d_flip_part : nullptr))) {
                release();
                return rc;
            }
            ++prod;
            e->launches += ae::dot(v, w, ni, 1, d_alpha + j, 0, d_dpart, e->sm_count, s);
            k_lanczos_update<<<vgrid, 256, 0, s>>>(w, v, j ? Vb + (size_t)(j - 1) * n : nullptr, d_alpha + j,
                                                   j ? d_beta + (j - 1) : nullptr, ni);
            ++e->launches;
            // classical Gram-Schmidt against the whole basis.  The three-term update above
            // already removed the v_j and v_{j-1} components (where the cancellation
            // happens), so one pass is normally the second orthogonalisation for them
            // ("twice is enough", Giraud, Langou and Rozloznik 2005).  A second pass runs
            // only when the first removed a large part of w: ||w|| after it below 0.7 of
            // ||w|| before it (the Daniel-Gragg-Kaufman-Stewart criterion; with an
            // orthonormal basis the norm before is sqrt(||w||^2 + ||c||^2)).  The decision
            // is taken on the device, and the second pass's kernels return at once when
            // it is not needed.
            e->launches += gemv_t(Vb, ni, ni, j + 1, w, 1.0, d_c, d_part, e->sm_count, s);
            e->launches += gemv_n(Vb, ni, ni, j + 1, d_c, -1.0, 1.0, w, s);
            e->launches += ae::dot(w, w, ni, 1, d_beta + j, 1, d_dpart, e->sm_count, s, d_c, j + 1, 0.7, d_again);
            e->launches += gemv_t(Vb, ni, ni, j + 1, w, 1.0, d_c, d_part, e->sm_count, s, d_again);
            e->launches += gemv_n(Vb, ni, ni, j + 1, d_c, -1.0, 1.0, w, s, d_again);
            e->launches += ae::dot(w, w, ni, 1, d_beta + j, 1, d_dpart, e->sm_count, s, nullptr, 0, 0.0, nullptr, d_again);
            e->launches += ae::axpby(w, w, ni, 1.0, 0.0, d_beta + j, s);
            const int jn = j + 1;
            if (jn - checked < kCheck && jn < m && prod < max_products && jn < ni) continue;
            // read alpha / beta so far; the first k at which the Ritz pairs converged, or the
            // basis is exhausted (beta ~ 0), ends the run
            al.resize(jn);
            be.resize(jn);
            cudaMemcpyAsync(al.data(), d_alpha, jn * sizeof(double), cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(be.data(), d_beta, jn * sizeof(double), cudaMemcpyDeviceToHost, s);
            if ((rc = stream_sync(e, "Lanczos"))) {
                release();
                return rc;
            }
            for (int kk = checked + 1; kk <= jn; ++kk) {
                std::vector<double> a(al.begin(), al.begin() + kk), b(be.begin(), be.begin() + kk);
                k = kk;
                if (nst == 1) {
                    ae::tridiag_lowest(a, b, kk, sv);
                    if (std::abs(be[kk - 1] * sv[kk - 1]) <= 0.5 * tol || !(be[kk - 1] > 1e-300)) {
                        done = true;
                        break;
                    }
                } else {
                    ae::tridiag_lowest_k(a, b, kk, nst, th, sv);
                    bool conv = kk >= nst;
                    for (int i = 0; conv && i < nst; ++i)
                        conv = std::abs(be[kk - 1] * sv[(size_t)i * kk + kk - 1]) <= 0.5 * tol;
                    if (conv || (kk >= nst && !(be[kk - 1] > 1e-300))) {
                        done = true;
                        break;
                    }
                }
            }
            checked = jn;
            if (prod >= max_products || jn == ni) done = true;
        }
        // Ritz vectors x_i = V s_i over the first k basis vectors (the result, or the
        // restart vector: x_0, or the sum of the x_i)
        if (nst == 1) {
            cudaMemcpyAsync(d_c, sv.data(), (size_t)k * sizeof(double), cudaMemcpyHostToDevice, s);
            e->launches += gemv_n(Vb, ni, ni, k, d_c, 1.0, 0.0, e->d_ground, s);
        } else {
            const int kk = k;
            std::vector<double> a(al.begin(), al.begin() + kk), b(be.begin(), be.begin() + kk);
            ae::tridiag_lowest_k(a, b, kk, nst, th, sv);
            const int got = std::min(nst, kk);
            for (int i = 0; i < got; ++i) {
                cudaMemcpyAsync(d_c, sv.data() + (size_t)i * kk, (size_t)kk * sizeof(double), cudaMemcpyHostToDevice, s);
                e->launches += gemv_n(Vb, ni, ni, kk, d_c, 1.0, 0.0, e->d_ground + (size_t)i * n, s);
                if ((rc = stream_sync(e, "Lanczos"))) {  // d_c is reused by the next vector
                    release();
                    return rc;
                }
            }
            if (got < nst) {
                release();
                return e->fail(AEGPU_ERR_STATE, "the Krylov space holds fewer eigenvectors than requested");
            }
            if (!done)
                for (int i = 1; i < nst; ++i)
                    e->launches += ae::axpby(e->d_ground, e->d_ground + (size_t)i * n, ni, 1.0, 1.0, nullptr, s);
        }
        if ((rc = stream_sync(e, "Lanczos"))) {
            release();
            return rc;
        }
    }
    // unit norm, the sign convention, and the Rayleigh quotient and true residual
    for (int i = 0; i < nst; ++i) {
        double *x = e->d_ground + (size_t)i * n;
        double sc[2] = {0.0, 0.0};
        e->launches += ae::dot(x, x, ni, 1, d_res, 1, d_dpart, e->sm_count, s);
        e->launches += ae::dot(e->d_start, x, ni, 1, d_res + 1, 0, d_dpart, e->sm_count, s);
        if ((rc = host_scalars(2, sc))) {
            release();
            return rc;
        }
        double sign = sc[1] < 0 ? -1.0 : 1.0;
        if (nst > 1 && std::abs(sc[1]) < 1e-12 * sc[0]) {
            std::vector<double> hx(n);
            cudaMemcpyAsync(hx.data(), x, n * sizeof(double), cudaMemcpyDeviceToHost, s);
            if ((rc = stream_sync(e, "Lanczos"))) {
                release();
                return rc;
            }
            size_t best = 0;
            for (size_t q = 1; q < n; ++q)
                if (std::abs(hx[q]) > std::abs(hx[best]) * (1.0 + 1e-12)) best = q;
            sign = hx[best] < 0 ? -1.0 : 1.0;
        }
        e->launches += ae::axpby(x, x, ni, sign / sc[0], 0.0, nullptr, s);
        double *w = Vb;
        if ((rc = run_apply(e, x, w, nullptr, 1, nullptr, false, flip, flip ? e->d_flip_part : nullptr))) {
            release();
            return rc;
        }
        ++prod;
        double lam = 0.0, res = 0.0;
        e->launches += ae::dot(x, w, ni, 1, d_res, 0, d_dpart, e->sm_count, s);
        if ((rc = host_scalars(1, &lam))) {
            release();
            return rc;
        }
        e->launches += ae::axpby(w, x, ni, 1.0, -lam, nullptr, s);
        e->launches += ae::dot(w, w, ni, 1, d_res, 1, d_dpart, e->sm_count, s);
        if ((rc = host_scalars(1, &res))) {
            release();
            return rc;
        }
        eigenvalues[i] = lam;
        if (residuals) residuals[i] = res;
        if (i == 0) e->ground_value = lam;
    }
    release();
    e->ground_states = nst;
    e->ground_valid = true;
    if (products) *products = prod;
    return AEGPU_OK;
}

extern "C" {

int aegpu_lowest_eigenpair(aegpu_engine *e, double tol, int basis, int max_products, double *eigenvalue,
                           double *residual, int *products)
{
    if (!e || !eigenvalue || !(tol > 0) || basis < 2 || max_products < 2) return AEGPU_ERR_ARG;
    return lanczos_lowest(e, 1, tol, basis, max_products, eigenvalue, residual, products);
}

int aegpu_lowest_eigenpairs(aegpu_engine *e, int nstates, double tol, int basis, int max_products, double *eigenvalues,
                            double *residuals, int *products)
{
    if (!e || nstates < 1 || !eigenvalues || !(tol > 0) || basis < 2 || max_products < 2) return AEGPU_ERR_ARG;
    return lanczos_lowest(e, nstates, tol, basis, max_products, eigenvalues, residuals, products);
}

int aegpu_ground_overlaps(aegpu_engine *e, const double *angles, int nstates, double *overlaps)
{
    NvtxRange r("aegpu ground overlaps");
    if (!e || !angles || !overlaps || nstates < 1) return AEGPU_ERR_ARG;
    if (e->nb != 1) return e->fail(AEGPU_ERR_UNSUPPORTED, "overlaps need a batch size of 1");
    if (!e->ground_valid) return e->fail(AEGPU_ERR_STATE, "no ground state: call aegpu_lowest_eigenpairs first");
    if (nstates > e->ground_states) return e->fail(AEGPU_ERR_ARG, "fewer eigenstates computed than requested");
    int rc = ensure_state(e, angles);
    if (rc) return rc;
    double *sm = small_scratch(e);
    if (!sm) return e->fail(AEGPU_ERR_NOMEM, "scratch allocation failed");
    const int64_t D = (int64_t)e->B.D;
    const size_t n = e->vec_elems();
    for (int i = 0; i < nstates; ++i) {
        const double *v = e->d_ground + (size_t)i * n;
        if (e->W == 1) {
            e->launches += ae::dot(e->d_psi, v, D, 1, sm, 0, sm + 4, e->sm_count, e->stream);
            cudaMemsetAsync(sm + 1, 0, sizeof(double), e->stream);
        } else {
            // <psi|v> = sum conj(psi) v
            e->launches += ae::dotc(e->d_psi, v, D, sm, sm + 4, e->sm_count, e->stream);
        }
        cudaMemcpyAsync(overlaps + 2 * i, sm, 2 * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
        if ((rc = stream_sync(e, "ground overlaps"))) return rc;
    }
    return AEGPU_OK;
}

int aegpu_ground_state(aegpu_engine *e, double *state)
{
    if (!e || !state) return AEGPU_ERR_ARG;
    if (!e->ground_valid) return e->fail(AEGPU_ERR_STATE, "no ground state: call aegpu_lowest_eigenpair first");
    cudaMemcpyAsync(state, e->d_ground, e->vec_elems() * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
    return stream_sync(e, "ground state");
}

int aegpu_ground_overlap(aegpu_engine *e, const double *angles, double *overlap)
{
    NvtxRange r("aegpu ground overlap");
    if (!e || !angles || !overlap) return AEGPU_ERR_ARG;
    if (e->nb != 1) return e->fail(AEGPU_ERR_UNSUPPORTED, "overlaps need a batch size of 1");
    if (!e->ground_valid) return e->fail(AEGPU_ERR_STATE, "no ground state: call aegpu_lowest_eigenpair first");
    int rc = ensure_state(e, angles);
    if (rc) return rc;
    double *sm = small_scratch(e);
    if (!sm) return e->fail(AEGPU_ERR_NOMEM, "scratch allocation failed");
    const int64_t D = (int64_t)e->B.D;
    if (e->W == 1) {
        e->launches += ae::dot(e->d_psi, e->d_ground, D, 1, sm, 0, sm + 4, e->sm_count, e->stream);
        cudaMemsetAsync(sm + 1, 0, sizeof(double), e->stream);
    } else {
        // <psi|v> = sum conj(psi) v
        e->launches += ae::dotc(e->d_psi, e->d_ground, D, sm, sm + 4, e->sm_count, e->stream);
    }
    cudaMemcpyAsync(overlap, sm, 2 * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
    return stream_sync(e, "ground overlap");
}

int aegpu_real_energy(aegpu_engine *e, const double *angles, double *real_energy)
{
    if (!e || !angles || !real_energy) return AEGPU_ERR_ARG;
    if (!e->ham_kind) return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    if (e->nb != 1) return e->fail(AEGPU_ERR_UNSUPPORTED, "the real-part energy needs a batch size of 1");
    int rc = ensure_state(e, angles);
    if (!rc && !e->h_valid) {
        rc = run_energy(e, e->d_scalar, 1);
        if (!rc) e->h_valid = true;
    }
    if (rc) return rc;
    double *sm = small_scratch(e);
    if (!sm) return e->fail(AEGPU_ERR_NOMEM, "scratch allocation failed");
    const int64_t n = (int64_t)e->B.D, inc = e->W;
    // H is real, so Re(H psi) = H Re(psi): <r|H r> / <r|r> from the even (real) entries
    double v[2] = {0.0, 0.0};
    e->launches += ae::dot(e->d_psi, e->d_h, n, inc, sm, 0, sm + 4, e->sm_count, e->stream);
    e->launches += ae::dot(e->d_psi, e->d_psi, n, inc, sm + 1, 0, sm + 4, e->sm_count, e->stream);
    cudaMemcpyAsync(v, sm, 2 * sizeof(double), cudaMemcpyDeviceToHost, e->stream);
    if ((rc = stream_sync(e, "real-part energy"))) return rc;
    *real_energy = v[0] / v[1];
    return AEGPU_OK;
}

int aegpu_subspace_matrices(aegpu_engine *e, int nsets, const double *angles, double *h_re, double *h_im, double *s_re,
                            double *s_im)
{
    NvtxRange r("aegpu subspace matrices");
    if (!e || nsets < 1 || nsets > 65535 || !angles || !h_re || !s_re) return AEGPU_ERR_ARG;
    if (!e->ham_kind) return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    if (e->nb != 1) return e->fail(AEGPU_ERR_UNSUPPORTED, "subspace matrices need a batch size of 1");
    const size_t n = e->vec_elems(), nops = e->excs.size();
    const int W = e->W;
    const int64_t D = (int64_t)e->B.D;
    const size_t nn = (size_t)nsets * nsets;
    const int64_t ngram = gram_scratch_doubles(nsets, W, D, e->sm_count);
    double *Psi = e->alloc<double>(n * nsets), *HPsi = e->alloc<double>(n * nsets), *M = e->alloc<double>(4 * nn),
           *G = e->alloc<double>((size_t)ngram);
    auto release = [&] {
        e->release(Psi, n * nsets * sizeof(double));
        e->release(HPsi, n * nsets * sizeof(double));
        e->release(M, 4 * nn * sizeof(double));
        e->release(G, (size_t)ngram * sizeof(double));
    };
    if (!Psi || !HPsi || !M || !G) {
        release();
        return e->fail(AEGPU_ERR_NOMEM, "subspace buffers allocation failed");
    }
    cudaStream_t s = e->stream;
    int rc = 0;
    // the evolved states as columns, then H on all of them as one batched product
    for (int k = 0; k < nsets; ++k) {
        if ((rc = upload_angles(e, angles + (size_t)k * nops, true, 1, false)) || (rc = run_evolve(e, 1))) {
            release();
            return rc;
        }
        cudaMemcpyAsync(Psi + (size_t)k * n, e->d_psi, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    }
    e->psi_valid = e->h_valid = false;
    e->cached_angles.clear();
    if ((rc = run_apply(e, Psi, HPsi, nullptr, nsets, nullptr, false))) {
        release();
        return rc;
    }
    // upper triangles of <psi_i|H psi_j> and <psi_i|psi_j> (complex: conjugate-linear in
    // the first argument; real and imaginary parts), column-major nsets x nsets
    e->launches += gram_upper(Psi, (int64_t)n, HPsi, (int64_t)n, D, W, nsets, 1.0, M, W == 2 ? M + nn : nullptr, nsets, G,
                              e->sm_count, s);
    e->launches += gram_upper(Psi, (int64_t)n, Psi, (int64_t)n, D, W, nsets, 1.0, M + 2 * nn, W == 2 ? M + 3 * nn : nullptr,
                              nsets, G, e->sm_count, s);
    std::vector<double> hm(4 * nn, 0.0);
    cudaMemcpyAsync(hm.data(), M, (W == 2 ? 4 : 3) * nn * sizeof(double), cudaMemcpyDeviceToHost, s);
    rc = stream_sync(e, "subspace matrices");
    release();
    if (rc) return rc;
    // both matrices are Hermitian: (i, j) for i <= j from the upper triangle (column-major
    // at j * nsets + i), the rest by conjugate symmetry; out[i * nsets + j] row-major
    for (int i = 0; i < nsets; ++i)
        for (int j = 0; j < nsets; ++j) {
            const size_t cm = i <= j ? (size_t)j * nsets + i : (size_t)i * nsets + j, rm = (size_t)i * nsets + j;
            const double sg = i <= j ? 1.0 : -1.0;
            h_re[rm] = hm[cm];
            s_re[rm] = hm[2 * nn + cm];
            if (h_im) h_im[rm] = W == 2 ? sg * hm[nn + cm] : 0.0;
            if (s_im) s_im[rm] = W == 2 ? sg * hm[3 * nn + cm] : 0.0;
        }
    return AEGPU_OK;
}

int aegpu_apply_dev(aegpu_engine *e, const double *x_dev, double *y_dev, double *energy_dev, void *stream)
{
    if (!e || !x_dev || !y_dev) return AEGPU_ERR_ARG;
    if (!e->ham_kind) return e->fail(AEGPU_ERR_STATE, "no Hamiltonian set");
    cudaStream_t saved = e->stream;
    if (stream) e->stream = (cudaStream_t)stream;
    int np = 0;
    int rc = run_apply(e, x_dev, y_dev, energy_dev ? e->d_epart : nullptr, e->nb, &np, false, true, e->d_flip_part,
                       nullptr);
    if (!rc && energy_dev) {
        k_reduce_sum<<<e->nb, 256, 0, e->stream>>>(e->d_epart, np, energy_dev, 1.0, nullptr);
        e->launches += 1;
        rc = e->cuda_check("apply_dev");
    }
    e->stream = saved;
    return rc;
}

int aegpu_phase_timing(aegpu_engine *e, int enable)
{
    if (!e) return AEGPU_ERR_ARG;
    e->timing = enable != 0;
    return AEGPU_OK;
}

int aegpu_phase_times(aegpu_engine *e, double *ms, int64_t *count)
{
    if (!e || !ms) return AEGPU_ERR_ARG;
    for (auto &m : e->ev_marks) {
        cudaEventSynchronize(m[3]);
        for (int p = 0; p < 3; ++p) {
            float t = 0;
            cudaEventElapsedTime(&t, m[p], m[p + 1]);
            e->phase_ms[p] += t;
        }
        e->phase_n += 1;
        for (auto ev : m) e->ev_pool.push_back(ev);
    }
    e->ev_marks.clear();
    for (int p = 0; p < 3; ++p) ms[p] = e->phase_ms[p];
    if (count) *count = e->phase_n;
    e->phase_ms[0] = e->phase_ms[1] = e->phase_ms[2] = 0;
    e->phase_n = 0;
    return e->cuda_check("phase_times");
}

int aegpu_problem_info(const aegpu_engine *e, int64_t *info)
{
    // D, nops, blocks, ham kind, stored H entries, stored row width, amplitudes touched per
    // sweep over all blocks, nonzeros of H (without row padding)
    if (!e || !info) return AEGPU_ERR_ARG;
    info[0] = (int64_t)e->B.D;
    info[1] = (int64_t)e->excs.size();
    info[2] = (int64_t)e->blocks.size();
    info[3] = e->ham_kind;
    info[4] = e->ham_entries;
    info[5] = e->ell_width;
    int64_t act = 0;
    for (auto &b : e->dblocks) act += b.diagonal ? (int64_t)e->B.D : (int64_t)b.active;
    info[6] = act;
    info[7] = e->ham_kind == 1 ? e->ham_entries : (e->ham_kind ? (int64_t)e->B.D * e->ints.width : 0);
    return AEGPU_OK;
}

int aegpu_fp64_work(const aegpu_engine *e, int64_t *work)
{
    // FP64 instructions of one energy + gradient evaluation per instance:
    // [0] H psi (one DFMA per stored / regenerated matrix element + the energy FMA),
    // [1] forward passes (one DFMA per amplitude-layer + one DMUL per amplitude),
    // [2] adjoint passes (two DFMA per amplitude-layer + one DMUL per amplitude + one
    //     DADD per lane-layer for the gradient sums);
    if (!e || !work) return AEGPU_ERR_ARG;
    // diagonal passes (complex): a complex multiply (4) per amplitude with an active slot
    // forward; adjoint the phase product (2), the back-rotation (4) and one DADD per
    // active slot
    int64_t al = 0, act = 0, dact = 0, dslots = 0;
    for (auto &b : e->dblocks) {
        if (b.diagonal) {
            dact += (int64_t)b.active;
            dslots += (int64_t)b.slot_acts;
            continue;
        }
        al += (int64_t)b.amp_layers;
        act += (int64_t)b.active;
    }
    const int64_t D = (int64_t)e->B.D, W = e->W;
    const int64_t elems = e->ham_kind == 1 ? e->ham_entries : (e->ham_kind ? D * e->ints.width : 0);
    work[0] = (elems + D) * W;
    work[1] = (al + act) * W + 4 * dact;
    work[2] = (2 * al + act) * W + al / 2 + 6 * dact + dslots;
    // [3] H psi by the spin-flip half product: the rows with a <= b, the energy FMAs of
    // every row, and the invariance test (one FMA per amplitude, one per pair a < b)
    work[3] = 0;
    const bool coded = e->ham_kind == 2 && e->ell_coded;
    if (e->flip_ok && (coded || e->ham_kind == 3)) {
        const int64_t nA = e->B.nA, Dh = nA * (nA + 1) / 2;
        work[3] = (Dh * e->ints.width + D + D + (D - nA) / 2) * W;
    }
    return AEGPU_OK;
}

// Measured DFMA throughput of this device (TFLOP/s, an FMA counted as 2 flops): a
// ~50 ms probe over every SM.
int aegpu_fp64_peak(double *tflops)
{
    if (!tflops) return AEGPU_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AEGPU_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return AEGPU_ERR_NOMEM;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    k_fp64_probe<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);  // warm-up
    cudaEventRecord(e0);
    k_fp64_probe<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess || ms <= 0) return AEGPU_ERR_CUDA;
    *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    return AEGPU_OK;
}

int64_t aegpu_device_bytes(const aegpu_engine *e) { return e ? e->dev_bytes : -1; }

// Test hook (no counterpart in the reference): the next n engine allocations succeed,
// all later ones fail as out of memory, until called again with n < 0.
void aegpu_debug_fail_alloc_after(int64_t n) { g_fail_alloc_after.store(n < 0 ? -1 : n); }
int64_t aegpu_launch_count(const aegpu_engine *e) { return e ? e->launches : -1; }

// No counterpart in the reference (see include/aegpu.h for the contract).
int aegpu_csr_energy_noalloc(int64_t D, const int64_t *rowptr_dev, const int32_t *col_dev, const double *val_dev,
                             const double *x_dev, double *y_dev, double *energy_dev, void *stream)
{
    if (D < 1 || !rowptr_dev || !col_dev || !val_dev || !x_dev || !y_dev || !energy_dev) return AEGPU_ERR_ARG;
    // y is written while other rows still read x, and the energy while y is read: the
    // three must be distinct (an in-place call would race and return wrong results)
    if ((const void *)x_dev == (const void *)y_dev || (const void *)energy_dev == (const void *)x_dev ||
        energy_dev == y_dev)
        return AEGPU_ERR_ARG;
    if (D > kNoAllocMaxRows) {
        fprintf(stderr, "aegpu_csr_energy_noalloc: %lld rows exceed the fixed scratch limit of %lld rows\n",
                (long long)D, (long long)kNoAllocMaxRows);
        return AEGPU_ERR_TOO_LARGE;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
        cudaGetLastError();
        return AEGPU_ERR_CUDA;
    }
    double *scratch = nullptr;
    {
        // first call on this device: resolve the array's device address (host code may
        // not use the symbol itself); this set-up must happen outside any stream capture
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return AEGPU_ERR_CUDA;
            }
            g_noalloc_addr[dev] = (double *)p;
        }
        scratch = g_noalloc_addr[dev];
    }
    // every partial sum the reduction reads is written by this call first, so the
    // array needs no clearing between calls
    const int grid = (int)((D + kNoAllocRowsPerPartial - 1) / kNoAllocRowsPerPartial);
    cudaStream_t s = (cudaStream_t)stream;
    k_spmv<1, false><<<grid, kSpmvThreads, 0, s>>>(rowptr_dev, 0, col_dev, val_dev, x_dev, y_dev, D, scratch, nullptr);
    k_reduce_sum<<<1, 256, 0, s>>>(scratch, grid, energy_dev, 1.0, nullptr);
    const cudaError_t rc = cudaGetLastError();
    return rc == cudaSuccess ? AEGPU_OK : AEGPU_ERR_CUDA;
}

}  // extern "C"
