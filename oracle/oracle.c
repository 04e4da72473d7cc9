/*
 * oracle.c -- CPU restatement of AnsatzEvolve's statevector hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity reference for the CUDA product
 * path and the timed CPU baseline ("port") of bench.py; nothing in the product
 * library links, loads or calls it.  It restates the reference algorithm in plain
 * C (+ OpenMP for the row loops the reference runs on its thread pool), and it is
 * itself pinned against the reference built from source (oracle/build_ref.sh) and
 * the reference's known answers (tests/golden/, tests/test_oracle_pin.py).
 *
 * Reference anchors (paths inside the AnsatzEvolve project):
 *   basis / compressors          src/operatorpool.cpp:207-242, src/operatorpool.h:49-77
 *   excitation partner + sign    src/fusedevolve.cpp:27-145 (same rule as operatorpool.cpp:24-156)
 *   Hamiltonian from integrals   src/hamiltonianmatrix.cpp:402-554 (+ filter :603-626, Sz rule operatorpool.cpp:244-253)
 *   Hamiltonian from triplets    src/hamiltonianmatrix.cpp:628-659
 *   CSR assembly from op list    src/hamiltonianmatrix.cpp:556-601
 *   H*psi on the fly             src/hamiltonianmatrix.cpp:915-1009
 *   evolve                       src/fusedevolve.cpp:2105-2159 (rotation :431-491, diagonal :625-717)
 *   gradient (adjoint sweep)     src/fusedevolve.cpp:2263-2346
 *   Hessian                      src/fusedevolve.cpp:2437-2780
 *   parameter compression        src/tupsquantities.cpp:643-667
 *
 * The fused-block ordering of the reference (regenCache, fusedevolve.cpp:1797-1967)
 * only regroups commuting excitations; the product of exponentials it evaluates is
 * the same, so this restatement applies the excitations one at a time in operator
 * order.  Results agree with the reference to rounding (pinned in the tests).
 *
 * Complex mode follows the reference's complex build: amplitudes are interleaved
 * (re, im); real excitations rotate re and im alike; diagonal (number / density-
 * density) operators multiply the active amplitudes by exp(+i*theta).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { OR_FULL = 0, OR_NUMBER = 1, OR_SZ = 2 };

static int popc32(uint32_t x) { return __builtin_popcount(x); }

/* ---------------------------------------------------------------- basis ---- */
/* Ascending enumeration of the sector, operatorpool.cpp:224-241 / operatorpool.h:57-73. */
static int in_sector(uint32_t s, int nq, int kind, int ne, int na, int nb)
{
    if (kind == OR_FULL) return 1;
    if (kind == OR_NUMBER) return popc32(s) == ne;
    uint32_t lo = s & ((1u << (nq / 2)) - 1u);
    return popc32(s >> (nq / 2)) == na && popc32(lo) == nb;
}

int64_t or_basis_size(int nq, int kind, int ne, int na, int nb)
{
    int64_t n = 0;
    for (uint64_t s = 0; s < (1ull << nq); ++s) n += in_sector((uint32_t)s, nq, kind, ne, na, nb);
    return n;
}

void or_basis_states(int nq, int kind, int ne, int na, int nb, uint32_t *out)
{
    int64_t n = 0;
    for (uint64_t s = 0; s < (1ull << nq); ++s)
        if (in_sector((uint32_t)s, nq, kind, ne, na, nb)) out[n++] = (uint32_t)s;
}

/* ------------------------------------------------------ excitation rule ---- */
/* fusedevolve.cpp:27-145.  Returns 0 inactive, 1 active (partner, sign), 2 active
 * diagonal (phase i, complex only).  sign is +1 / -1 as the reference's bool. */
int or_exc_apply(uint32_t state, int a, int b, int c, int d, uint32_t *partner, int *sign)
{
    uint32_t create, annihilate, mask;
    int phase = 1;
    *partner = state;
    *sign = 1;
    if (a < 0 && b < 0) return 0;
    if (c > -1 && d > -1) {
        if (a == b || c == d) return 0;
        create = (1u << a) | (1u << b);
        annihilate = (1u << c) | (1u << d);
        mask = ((1u << a) - 1u) ^ ((1u << b) - 1u) ^ ((1u << c) - 1u) ^ ((1u << d) - 1u);
        mask &= ~(create | annihilate);
        if (a > b) phase = -phase;
        if (c > d) phase = -phase;
    } else {
        create = 1u << a;
        annihilate = 1u << b;
        mask = ((1u << a) - 1u) ^ ((1u << b) - 1u);
        mask &= ~(create | annihilate);
    }
    if (popc32(state & mask) & 1) phase = -phase;
    uint32_t m = state & (create | annihilate);
    if (create == annihilate) {
        if ((m & annihilate) == annihilate) { *sign = 1; return 2; }
        return 0;
    }
    if ((m & annihilate) == annihilate && ((m ^ annihilate) & create) == 0) {
        *partner = state ^ annihilate ^ create;
        *sign = phase;
        return 1;
    }
    if ((m & create) == create && ((m ^ create) & annihilate) == 0) {
        *partner = state ^ create ^ annihilate;
        *sign = -phase;
        return 1;
    }
    return 0;
}

/* -------------------------------------------------------------- context ---- */
typedef struct {
    uint32_t create, destroy, signmask;
} or_hop;

typedef struct {
    int nq, kind, cplx;
    int64_t D;
    uint32_t *states;   /* rank -> bitstring */
    int32_t *rank;      /* bitstring -> rank or -1 (2^nq entries), compressPerm */
    /* excitations */
    int nops, nparams;
    int8_t *ops;        /* 4 per op, 0-based, -1 absent */
    int *param;
    double *scale;
    /* Hamiltonian: CSR (row-major, y = H x) or operator list */
    int ham_kind;       /* 0 none, 1 csr, 2 op list */
    int64_t *rowptr;
    int32_t *col;
    double *val;
    int nhops;
    or_hop *hops;
    double *hvals;
    /* initial state (compressed, 1 or 2 doubles per element) */
    double *start;
} or_ctx;

void *or_create(int nq, int kind, int ne, int na, int nb, int cplx)
{
    or_ctx *c = (or_ctx *)calloc(1, sizeof(or_ctx));
    c->nq = nq;
    c->kind = kind;
    c->cplx = cplx;
    c->D = or_basis_size(nq, kind, ne, na, nb);
    c->states = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)c->D);
    or_basis_states(nq, kind, ne, na, nb, c->states);
    c->rank = (int32_t *)malloc(sizeof(int32_t) * ((size_t)1 << nq));
    for (uint64_t s = 0; s < (1ull << nq); ++s) c->rank[s] = -1;
    for (int64_t i = 0; i < c->D; ++i) c->rank[c->states[i]] = (int32_t)i;
    c->start = (double *)calloc((size_t)c->D * (cplx ? 2 : 1), sizeof(double));
    return c;
}

void or_destroy(void *p)
{
    or_ctx *c = (or_ctx *)p;
    if (!c) return;
    free(c->states); free(c->rank); free(c->ops); free(c->param); free(c->scale);
    free(c->rowptr); free(c->col); free(c->val); free(c->hops); free(c->hvals); free(c->start);
    free(c);
}

int64_t or_dim(void *p) { return ((or_ctx *)p)->D; }
void or_states(void *p, uint32_t *out) { or_ctx *c = (or_ctx *)p; memcpy(out, c->states, sizeof(uint32_t) * (size_t)c->D); }

/* Initial state, 0-based full-space indices, compressed as compressVector does. */
int or_set_initial(void *p, int n, const int *idx, const double *re, const double *im)
{
    or_ctx *c = (or_ctx *)p;
    int w = c->cplx ? 2 : 1;
    memset(c->start, 0, sizeof(double) * (size_t)c->D * w);
    for (int k = 0; k < n; ++k) {
        if (idx[k] < 0 || (uint64_t)idx[k] >= (1ull << c->nq)) return 1;
        int32_t r = c->rank[idx[k]];
        if (r < 0) continue;
        c->start[(size_t)r * w] = re[k];
        if (c->cplx) c->start[(size_t)r * w + 1] = im ? im[k] : 0.0;
    }
    return 0;
}

int or_set_ops(void *p, int nops, const int *ops4, const int *param, const double *scale, int nparams)
{
    or_ctx *c = (or_ctx *)p;
    free(c->ops); free(c->param); free(c->scale);
    c->nops = nops;
    c->nparams = nparams;
    c->ops = (int8_t *)malloc(4 * (size_t)nops);
    c->param = (int *)malloc(sizeof(int) * (size_t)nops);
    c->scale = (double *)malloc(sizeof(double) * (size_t)nops);
    for (int i = 0; i < nops; ++i) {
        for (int j = 0; j < 4; ++j) c->ops[4 * i + j] = (int8_t)ops4[4 * i + j];
        c->param[i] = param[i];
        c->scale[i] = scale ? scale[i] : 1.0;
    }
    return 0;
}

/* --------------------------------------------------------- Hamiltonian ---- */
static int cmp_i64(const void *a, const void *b)
{
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

/* Sort (row, col, val) triplets and sum duplicates into CSR: setFromTriplets. */
static void build_csr(or_ctx *c, int64_t n, int64_t *keys, double *vals)
{
    int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * 2 * (size_t)(n ? n : 1));
    for (int64_t k = 0; k < n; ++k) { perm[2 * k] = keys[k]; perm[2 * k + 1] = k; }
    qsort(perm, (size_t)n, 2 * sizeof(int64_t), cmp_i64);
    free(c->rowptr); free(c->col); free(c->val);
    c->rowptr = (int64_t *)calloc((size_t)c->D + 1, sizeof(int64_t));
    c->col = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
    c->val = (double *)malloc(sizeof(double) * (size_t)(n ? n : 1));
    int64_t nnz = 0, last = -1;
    /* duplicates are summed in insertion order, as Eigen's setFromTriplets does */
    for (int64_t k = 0; k < n;) {
        int64_t key = perm[2 * k];
        int64_t j = k;
        while (j < n && perm[2 * j] == key) ++j;
        /* stable: indices among equal keys ascending */
        int64_t cnt = j - k;
        int64_t *ids = (int64_t *)malloc(sizeof(int64_t) * (size_t)cnt);
        for (int64_t t = 0; t < cnt; ++t) ids[t] = perm[2 * (k + t) + 1];
        qsort(ids, (size_t)cnt, sizeof(int64_t), cmp_i64);
        double s = 0;
        for (int64_t t = 0; t < cnt; ++t) s += vals[ids[t]];
        free(ids);
        int64_t row = key / c->D, colv = key % c->D;
        (void)last;
        c->col[nnz] = (int32_t)colv;
        c->val[nnz] = s;
        c->rowptr[row + 1]++;
        nnz++;
        k = j;
    }
    for (int64_t r = 0; r < c->D; ++r) c->rowptr[r + 1] += c->rowptr[r];
    free(perm);
    c->ham_kind = 1;
}

/* hamiltonianmatrix.cpp:628-659: 0-based full-space triplets, out-of-sector dropped.
 * The reference stores them as (i,j) and computes y = x H; we store the transpose
 * (row j, col i) so that y_j = sum_i H(i,j) x_i is a row-major CSR product. */
int or_set_ham_triplets(void *p, int n, const int *ii, const int *jj, const double *v)
{
    or_ctx *c = (or_ctx *)p;
    int64_t *keys = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
    double *vals = (double *)malloc(sizeof(double) * (size_t)(n ? n : 1));
    int64_t m = 0;
    for (int k = 0; k < n; ++k) {
        if (ii[k] < 0 || jj[k] < 0 || (uint64_t)ii[k] >= (1ull << c->nq) || (uint64_t)jj[k] >= (1ull << c->nq)) continue;
        int32_t ri = c->rank[ii[k]], rj = c->rank[jj[k]];
        if (ri < 0 || rj < 0) continue;
        keys[m] = (int64_t)rj * c->D + ri;
        vals[m] = v[k];
        m++;
    }
    build_csr(c, m, keys, vals);
    free(keys);
    free(vals);
    return 0;
}

/* hamiltonianmatrix.cpp:402-554 with the Sz filter of operatorpool.cpp:244-253.
 * h1: N*N row-major; g2: N^4 in the file layout g2[((i*N+l)*N+j)*N+k] = (il|jk).
 * mode 1 assembles CSR (constructFromSecQuant, :556-601), mode 2 keeps the op list. */
int or_set_ham_integrals(void *p, const double *h1, const double *g2, int mode)
{
    or_ctx *c = (or_ctx *)p;
    int nq = c->nq, N = nq / 2;
    size_t cap = (size_t)nq * nq * nq * nq + (size_t)nq * nq;
    or_hop *hops = (or_hop *)malloc(sizeof(or_hop) * cap);
    double *hv = (double *)malloc(sizeof(double) * cap);
    int n = 0;
#define TWOE(i, j, k, l) g2[((((size_t)(i) * N) + (l)) * N + (j)) * N + (k)]
    for (int a = 0; a < nq; ++a)
        for (int b = a + 1; b < nq; ++b)
            for (int cc = 0; cc < nq; ++cc)
                for (int d = cc + 1; d < nq; ++d) {
                    int sa = a >= N, sb = b >= N, sc = cc >= N, sd = d >= N;
                    int pa = a % N, pb = b % N, pc = cc % N, pd = d % N;
                    double E = 0;
                    if (sa == sc && sb == sd) E += TWOE(pb, pa, pc, pd);
                    if (sa == sd && sb == sc) E -= TWOE(pb, pa, pd, pc);
                    if (fabs(E) > 1e-13) {
                        uint32_t cr = (1u << a) | (1u << b), de = (1u << cc) | (1u << d);
                        uint32_t m = ((1u << a) - 1u) ^ ((1u << b) - 1u) ^ ((1u << cc) - 1u) ^ ((1u << d) - 1u);
                        m &= ~(cr | de);
                        hops[n].create = cr; hops[n].destroy = de; hops[n].signmask = m;
                        hv[n++] = E;
                    }
                }
    for (int a = 0; a < nq; ++a)
        for (int cc = 0; cc < nq; ++cc) {
            double E = h1[(a % N) * N + (cc % N)];
            if (fabs(E) > 1e-13) {
                uint32_t m = ((1u << a) - 1u) ^ ((1u << cc) - 1u);
                m &= ~((1u << a) | (1u << cc));
                hops[n].create = 1u << a; hops[n].destroy = 1u << cc; hops[n].signmask = m;
                hv[n++] = E;
            }
        }
#undef TWOE
    if (mode == 2 && c->kind == OR_SZ) {
        /* postProcessOperators: keep operators whose spin counts balance */
        uint32_t dn = (1u << N) - 1u, up = ((1u << nq) - 1u) ^ dn;
        int m = 0;
        for (int k = 0; k < n; ++k) {
            or_hop h = hops[k];
            if (popc32(h.create & up) == popc32(h.destroy & up) && popc32(h.create & dn) == popc32(h.destroy & dn)) {
                hops[m] = h;
                hv[m++] = hv[k];
            }
        }
        n = m;
    }
    free(c->hops); free(c->hvals);
    c->hops = hops;
    c->hvals = hv;
    c->nhops = n;
    if (mode == 1) {
        /* triplets (k, j) for op applied to basis state k giving j; stored transposed */
        int64_t cap2 = 1024, m = 0;
        int64_t *keys = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap2);
        double *vals = (double *)malloc(sizeof(double) * (size_t)cap2);
        for (int64_t k = 0; k < c->D; ++k) {
            uint32_t s = c->states[k];
            for (int o = 0; o < n; ++o) {
                uint32_t de = s ^ hops[o].destroy;
                if (de & hops[o].destroy) continue;
                if (de & hops[o].create) continue;
                uint32_t j = de | hops[o].create;
                int sg = popc32(s & hops[o].signmask) & 1;
                int32_t rj = c->rank[j];
                if (rj < 0) continue;
                if (m == cap2) {
                    cap2 *= 2;
                    keys = (int64_t *)realloc(keys, sizeof(int64_t) * (size_t)cap2);
                    vals = (double *)realloc(vals, sizeof(double) * (size_t)cap2);
                }
                keys[m] = (int64_t)rj * c->D + k;
                vals[m++] = sg ? -hv[o] : hv[o];
            }
        }
        build_csr(c, m, keys, vals);
        free(keys);
        free(vals);
    } else {
        c->ham_kind = 2;
    }
    return 0;
}

int64_t or_ham_nnz(void *p) { or_ctx *c = (or_ctx *)p; return c->ham_kind == 1 ? c->rowptr[c->D] : -1; }
int or_ham_nops(void *p) { return ((or_ctx *)p)->nhops; }

void or_ham_csr(void *p, int64_t *rowptr, int32_t *col, double *val)
{
    or_ctx *c = (or_ctx *)p;
    memcpy(rowptr, c->rowptr, sizeof(int64_t) * ((size_t)c->D + 1));
    memcpy(col, c->col, sizeof(int32_t) * (size_t)c->rowptr[c->D]);
    memcpy(val, c->val, sizeof(double) * (size_t)c->rowptr[c->D]);
}

/* y = H x for nv interleaved components per element (1 real, 2 complex). */
static void ham_apply(const or_ctx *c, const double *x, double *y, int w)
{
    int64_t D = c->D;
    if (c->ham_kind == 1) {
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t r = 0; r < D; ++r) {
            double a0 = 0, a1 = 0;
            for (int64_t k = c->rowptr[r]; k < c->rowptr[r + 1]; ++k) {
                a0 += c->val[k] * x[(size_t)c->col[k] * w];
                if (w == 2) a1 += c->val[k] * x[(size_t)c->col[k] * w + 1];
            }
            y[(size_t)r * w] = a0;
            if (w == 2) y[(size_t)r * w + 1] = a1;
        }
        return;
    }
    /* operator-list loop of hamiltonianmatrix.cpp:915-1009, run over output indices */
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t j = 0; j < D; ++j) {
        uint32_t js = c->states[j];
        double a0 = 0, a1 = 0;
        uint32_t bad = 0, good = 0, de = 0;
        int n = c->nhops;
        if (n > 0) {
            good = c->hops[0].create;
            de = js ^ good;
            if (de & good) bad = good;
        }
        for (int o = 0; o < n; ++o) {
            const or_hop *h = &c->hops[o];
            if (h->create == bad) continue;
            bad = 0;
            if (h->create != good) {
                good = h->create;
                de = js ^ good;
                if (de & good) { bad = good; continue; }
            }
            if (de & h->destroy) continue;
            uint32_t i = de | h->destroy;
            int sg = popc32(js & h->signmask) & 1;
            int32_t ri = c->rank[i];
            if (ri < 0) continue;
            double v = sg ? -c->hvals[o] : c->hvals[o];
            a0 += x[(size_t)ri * w] * v;
            if (w == 2) a1 += x[(size_t)ri * w + 1] * v;
        }
        y[(size_t)j * w] = a0;
        if (w == 2) y[(size_t)j * w + 1] = a1;
    }
}

/* (H x) on a subset of rows only -- a spot check that stays cheap at sizes where a
 * full operator-list apply (hamiltonianmatrix.cpp:915-1009) would take minutes. */
int or_apply_h_rows(void *p, const double *x, const int64_t *rows, int n, double *y)
{
    or_ctx *c = (or_ctx *)p;
    if (c->ham_kind != 2) return 1;
    int w = c->cplx ? 2 : 1;
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < n; ++k) {
        int64_t j = rows[k];
        uint32_t js = c->states[j];
        double a0 = 0, a1 = 0;
        for (int o = 0; o < c->nhops; ++o) {
            const or_hop *h = &c->hops[o];
            uint32_t de = js ^ h->create;
            if (de & h->create) continue;
            if (de & h->destroy) continue;
            uint32_t i = de | h->destroy;
            int sg = popc32(js & h->signmask) & 1;
            int32_t ri = c->rank[i];
            if (ri < 0) continue;
            double v = sg ? -c->hvals[o] : c->hvals[o];
            a0 += x[(size_t)ri * w] * v;
            if (w == 2) a1 += x[(size_t)ri * w + 1] * v;
        }
        y[(size_t)k * w] = a0;
        if (w == 2) y[(size_t)k * w + 1] = a1;
    }
    return 0;
}

int or_apply_h(void *p, const double *x, double *y)
{
    or_ctx *c = (or_ctx *)p;
    if (!c->ham_kind) return 1;
    ham_apply(c, x, y, c->cplx ? 2 : 1);
    return 0;
}

static double rdot(const double *a, const double *b, int64_t n)
{
    double s = 0;
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* --------------------------------------------------------- evolution ---- */
/* One excitation exp(theta G) on vector v (w doubles per element).  For every
 * active determinant z with partner p(z) and sign s(z): (G v)_z = s(z) v_{p(z)};
 * pairs are visited once from their lower rank.  fusedevolve.cpp:461-468, 625-717. */
static void rotate_op(const or_ctx *c, const int8_t *e, double th, double *v, int w)
{
    double S = sin(th), C = cos(th);
    int64_t D = c->D;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < D; ++z) {
        uint32_t pbits; int s;
        int act = or_exc_apply(c->states[z], e[0], e[1], e[2], e[3], &pbits, &s);
        if (act == 2) { /* diagonal: v_z *= exp(i th) */
            double re = v[(size_t)z * 2], im = v[(size_t)z * 2 + 1];
            v[(size_t)z * 2] = C * re - S * im;
            v[(size_t)z * 2 + 1] = S * re + C * im;
            continue;
        }
        if (act != 1) continue;
        int32_t pz = c->rank[pbits];
        if (pz < 0 || pz < z) continue;
        for (int k = 0; k < w; ++k) {
            double x = v[(size_t)z * w + k], y = v[(size_t)pz * w + k];
            v[(size_t)z * w + k] = s * y * S + x * C;
            v[(size_t)pz * w + k] = -s * x * S + y * C;
        }
    }
}

/* out = G v (the tangent direction of one excitation), fusedevolve.cpp:492-518. */
static void apply_gen(const or_ctx *c, const int8_t *e, const double *v, double *out, int w)
{
    int64_t D = c->D;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < D; ++z) {
        uint32_t pbits; int s;
        int act = or_exc_apply(c->states[z], e[0], e[1], e[2], e[3], &pbits, &s);
        if (act == 2) {
            out[(size_t)z * 2] = -v[(size_t)z * 2 + 1];
            out[(size_t)z * 2 + 1] = v[(size_t)z * 2];
            continue;
        }
        int32_t pz = act == 1 ? c->rank[pbits] : -1;
        for (int k = 0; k < w; ++k) out[(size_t)z * w + k] = pz >= 0 ? s * v[(size_t)pz * w + k] : 0.0;
    }
}

/* Re <h | G v> for one excitation. */
static double braket_gen(const or_ctx *c, const int8_t *e, const double *h, const double *v, int w)
{
    int64_t D = c->D;
    double acc = 0;
#pragma omp parallel for schedule(static) reduction(+ : acc)
    for (int64_t z = 0; z < D; ++z) {
        uint32_t pbits; int s;
        int act = or_exc_apply(c->states[z], e[0], e[1], e[2], e[3], &pbits, &s);
        if (act == 2) {
            acc += h[(size_t)z * 2 + 1] * v[(size_t)z * 2] - h[(size_t)z * 2] * v[(size_t)z * 2 + 1];
            continue;
        }
        if (act != 1) continue;
        int32_t pz = c->rank[pbits];
        if (pz < 0) continue;
        for (int k = 0; k < w; ++k) acc += h[(size_t)z * w + k] * s * v[(size_t)pz * w + k];
    }
    return acc;
}

/* psi = prod_ops exp(theta_op G_op) psi0, operators applied in list order. */
int or_evolve(void *p, const double *angles, double *out)
{
    or_ctx *c = (or_ctx *)p;
    int w = c->cplx ? 2 : 1;
    memcpy(out, c->start, sizeof(double) * (size_t)c->D * w);
    for (int o = 0; o < c->nops; ++o) rotate_op(c, c->ops + 4 * o, angles[o], out, w);
    return 0;
}

/* E (without nuclear energy) and per-operator gradient dE/dtheta_op:
 * Hpsi, then a backward sweep with -theta, fusedevolve.cpp:2263-2346.
 * grad_op may be NULL. */
int or_energy_gradient(void *p, const double *angles, double *E, double *grad_op)
{
    or_ctx *c = (or_ctx *)p;
    int w = c->cplx ? 2 : 1;
    size_t n = (size_t)c->D * w;
    double *psi = (double *)malloc(sizeof(double) * n), *h = (double *)malloc(sizeof(double) * n);
    or_evolve(p, angles, psi);
    ham_apply(c, psi, h, w);
    if (E) *E = rdot(h, psi, (int64_t)n);
    if (grad_op) {
        for (int o = c->nops - 1; o >= 0; --o) {
            const int8_t *e = c->ops + 4 * o;
            grad_op[o] = 2.0 * braket_gen(c, e, h, psi, w);
            rotate_op(c, e, -angles[o], psi, w);
            rotate_op(c, e, -angles[o], h, w);
        }
    }
    free(psi);
    free(h);
    return 0;
}

/* Projected variant (FusedEvolve::evolveDerivativeProj, fusedevolve.cpp:2814-2880):
 * overlap = <proj|psi(theta)> and grad_op = d<proj|psi>/dtheta_op (no factor 2), the
 * same backward sweep with the fixed bra proj in place of H psi. */
int or_gradient_proj(void *p, const double *angles, const double *proj, double *overlap, double *grad_op)
{
    or_ctx *c = (or_ctx *)p;
    int w = c->cplx ? 2 : 1;
    size_t n = (size_t)c->D * w;
    double *psi = (double *)malloc(sizeof(double) * n), *h = (double *)malloc(sizeof(double) * n);
    or_evolve(p, angles, psi);
    memcpy(h, proj, sizeof(double) * n);
    if (overlap) *overlap = rdot(h, psi, (int64_t)n);
    if (grad_op) {
        for (int o = c->nops - 1; o >= 0; --o) {
            const int8_t *e = c->ops + 4 * o;
            grad_op[o] = braket_gen(c, e, h, psi, w);
            rotate_op(c, e, -angles[o], psi, w);
            rotate_op(c, e, -angles[o], h, w);
        }
    }
    free(psi);
    free(h);
    return 0;
}

/* Full second derivative d^2E/dtheta_i dtheta_j over operator angles:
 * 2 Re<T_i|H|T_j> + 2 Re<Hpsi| d_i d_j psi>, fusedevolve.cpp:2437-2780. */
int or_hessian_ops(void *p, const double *angles, double *Hops)
{
    or_ctx *c = (or_ctx *)p;
    int w = c->cplx ? 2 : 1, P = c->nops;
    size_t n = (size_t)c->D * w;
    double *T = (double *)calloc(n * (size_t)P, sizeof(double));
    double *HT = (double *)malloc(sizeof(double) * n * (size_t)P);
    double *psi = (double *)malloc(sizeof(double) * n), *h = (double *)malloc(sizeof(double) * n);
    double *t = (double *)malloc(sizeof(double) * n), *hb = (double *)malloc(sizeof(double) * n);
    memcpy(psi, c->start, sizeof(double) * n);
    /* tangents: T_k = G_k psi_k, then evolved through the rest of the circuit */
    for (int o = 0; o < P; ++o) {
        const int8_t *e = c->ops + 4 * o;
        rotate_op(c, e, angles[o], psi, w);
        apply_gen(c, e, psi, T + n * o, w);
        for (int k = 0; k < o; ++k) rotate_op(c, e, angles[o], T + n * k, w);
    }
    ham_apply(c, psi, h, w);
    for (int i = 0; i < P; ++i) ham_apply(c, T + n * i, HT + n * i, w);
    for (int i = 0; i < P; ++i)
        for (int j = 0; j < P; ++j) Hops[(size_t)i * P + j] = 2.0 * rdot(T + n * i, HT + n * j, (int64_t)n);
    /* second-derivative term: backward sweeps of (T_i, Hpsi) */
    for (int i = 0; i < P; ++i) {
        memcpy(t, T + n * i, sizeof(double) * n);
        memcpy(hb, h, sizeof(double) * n);
        for (int j = P - 1; j >= i; --j) {
            const int8_t *e = c->ops + 4 * j;
            double v = 2.0 * braket_gen(c, e, hb, t, w);
            Hops[(size_t)i * P + j] += v;
            if (j != i) Hops[(size_t)j * P + i] += v;
            rotate_op(c, e, -angles[j], t, w);
            rotate_op(c, e, -angles[j], hb, w);
        }
    }
    free(T); free(HT); free(psi); free(h); free(t); free(hb);
    return 0;
}

/* Compressed (per-parameter) quantities, tupsquantities.cpp:643-667:
 * theta_op = scale_op * x_param(op); g_mu = sum_op scale_op g_op [param(op)=mu]. */
void or_decompress_angles(void *p, const double *x, double *ang)
{
    or_ctx *c = (or_ctx *)p;
    for (int o = 0; o < c->nops; ++o) ang[o] = c->scale[o] * x[c->param[o]];
}

int or_gradient_comp(void *p, const double *x, double *E, double *g)
{
    or_ctx *c = (or_ctx *)p;
    double *ang = (double *)malloc(sizeof(double) * c->nops), *go = (double *)malloc(sizeof(double) * c->nops);
    or_decompress_angles(p, x, ang);
    or_energy_gradient(p, ang, E, go);
    for (int m = 0; m < c->nparams; ++m) g[m] = 0;
    for (int o = 0; o < c->nops; ++o) g[c->param[o]] += c->scale[o] * go[o];
    free(ang);
    free(go);
    return 0;
}

int or_hessian_comp(void *p, const double *x, double *H)
{
    or_ctx *c = (or_ctx *)p;
    int P = c->nops, M = c->nparams;
    double *ang = (double *)malloc(sizeof(double) * P), *Ho = (double *)malloc(sizeof(double) * P * P);
    or_decompress_angles(p, x, ang);
    or_hessian_ops(p, ang, Ho);
    for (int a = 0; a < M * M; ++a) H[a] = 0;
    for (int i = 0; i < P; ++i)
        for (int j = 0; j < P; ++j)
            H[(size_t)c->param[i] * M + c->param[j]] += c->scale[i] * c->scale[j] * Ho[(size_t)i * P + j];
    free(ang);
    free(Ho);
    return 0;
}

int or_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
