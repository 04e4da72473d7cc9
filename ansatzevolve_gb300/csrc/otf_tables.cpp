// Host-built tables for the string-driven on-the-fly H*psi kernel (k_otf_strings).
//
// In the Sz sector a determinant is an (alpha string, beta string) pair and every
// matrix element of the reference's Hamiltonian (operator list of
// hamiltonianmatrix.cpp:402-554, applied as in :915-1009) factorises over the two
// strings:
//  * excitation lists per string: single (p<-r) and same-spin double excitations with
//    the rank of the excited string and the fermionic sign, which is the parity of the
//    string's occupied orbitals strictly between the moved ones (the other string's
//    bits cancel out of the reference's sign mask);
//  * same-spin doubles: V[(p1<p2),(r1<r2)] = (p2 r2|p1 r1) - (p2 r1|p1 r2)
//    (two_e below, the reference's getTwoElectronEnergy with its 1e-13 cut);
//  * alpha-beta doubles: V = (pa ra|pb rb), with sign = product of the two strings'
//    single-excitation signs;
//  * a single p<-r of spin s equals sign * (A_s[own string][p][r] + B_s[other string][p][r])
//    with A_s = h_pr + sum over the other occupied orbitals t of the same spin of
//    (-1)^[t strictly between p and r] V(sort(p,t), sort(r,t)) and B_s = sum over the
//    occupied orbitals of the other spin of V(sort(p,t), sort(r,t)).
// Everything here is setup (once per Hamiltonian); all H*psi work runs on the GPU.
#include "otf_tables.h"

#include <algorithm>
#include <cmath>

namespace ae {

namespace {

inline uint32_t below(int x) { return (1u << x) - 1u; }
inline int parity(uint32_t x) { return __builtin_popcount(x) & 1; }

struct TwoE {
    int N;
    const double *g;  // g[((p*N+q)*N+r)*N+s] = (pq|rs)
    // op a^+_p a^+_q a_r a_s with spin orbitals p<q, r<s (hamiltonianmatrix.cpp:456-470, 479-505)
    double operator()(int p, int q, int r, int s) const
    {
        const int sp = p >= N, sq = q >= N, sr = r >= N, ss = s >= N;
        const int P = p - sp * N, Q = q - sq * N, R = r - sr * N, S = s - ss * N;
        double E = 0;
        if (sp == sr && sq == ss) E += g[(((size_t)Q * N + S) * N + P) * N + R];
        if (sp == ss && sq == sr) E -= g[(((size_t)Q * N + R) * N + P) * N + S];
        return std::abs(E) > 1e-13 ? E : 0.0;
    }
};

int pair_index(int i, int j, int n)  // i < j < n, lexicographic
{
    return i * n - i * (i + 1) / 2 + (j - i - 1);
}

void string_lists(const std::vector<uint32_t> &strs, const std::vector<int32_t> &rank, int N, int nO,
                  std::vector<int32_t> &s_rank, std::vector<int32_t> &s_code, std::vector<int32_t> &d_rank,
                  std::vector<int32_t> &d_code, int &ns, int &nd)
{
    const int nV = N - nO;
    const int P2 = N * (N - 1) / 2;
    ns = nO * nV;
    nd = (nO * (nO - 1) / 2) * (nV * (nV - 1) / 2);
    s_rank.assign(strs.size() * (size_t)ns, 0);
    s_code.assign(strs.size() * (size_t)ns, 0);
    d_rank.assign(strs.size() * (size_t)std::max(nd, 0), 0);
    d_code.assign(strs.size() * (size_t)std::max(nd, 0), 0);
    for (size_t k = 0; k < strs.size(); ++k) {
        const uint32_t s = strs[k];
        std::vector<int> occ, vir;
        for (int i = 0; i < N; ++i) ((s >> i) & 1 ? occ : vir).push_back(i);
        int t = 0;
        for (int p : occ)
            for (int r : vir) {
                const uint32_t m = (below(p) ^ below(r)) & ~((1u << p) | (1u << r));
                s_rank[k * ns + t] = rank[s ^ (1u << p) ^ (1u << r)];
                s_code[k * ns + t] = (p | (r << 5)) | (parity(s & m) ? (int32_t)0x80000000 : 0);
                ++t;
            }
        int d = 0;
        for (size_t a = 0; a < occ.size(); ++a)
            for (size_t b = a + 1; b < occ.size(); ++b)
                for (size_t c = 0; c < vir.size(); ++c)
                    for (size_t e = c + 1; e < vir.size(); ++e) {
                        const int p1 = occ[a], p2 = occ[b], r1 = vir[c], r2 = vir[e];
                        uint32_t m = below(p1) ^ below(p2) ^ below(r1) ^ below(r2);
                        m &= ~((1u << p1) | (1u << p2) | (1u << r1) | (1u << r2));
                        d_rank[k * nd + d] = rank[s ^ (1u << p1) ^ (1u << p2) ^ (1u << r1) ^ (1u << r2)];
                        const int code = pair_index(p1, p2, N) * P2 + pair_index(r1, r2, N);
                        d_code[k * nd + d] = code | (parity(s & m) ? (int32_t)0x80000000 : 0);
                        ++d;
                    }
    }
}

// A_s[string][p*N+r] (same-spin part + h) and B_s[other string][p*N+r] (cross-spin part).
void single_tables(const TwoE &V, const std::vector<double> &h1, int N, int off_self, int off_other,
                   const std::vector<uint32_t> &self, const std::vector<uint32_t> &other, std::vector<double> &A,
                   std::vector<double> &B)
{
    A.assign(self.size() * (size_t)N * N, 0.0);
    B.assign(other.size() * (size_t)N * N, 0.0);
    for (size_t k = 0; k < self.size(); ++k) {
        const uint32_t s = self[k];
        for (int p = 0; p < N; ++p)
            for (int r = 0; r < N; ++r) {
                if (p == r) continue;
                const double h = h1[(size_t)p * N + r];
                double v = std::abs(h) > 1e-13 ? h : 0.0;
                const int P = p + off_self, R = r + off_self;
                for (int t = 0; t < N; ++t) {
                    if (!((s >> t) & 1) || t == p || t == r) continue;
                    const int T = t + off_self;
                    const double term = V(std::min(P, T), std::max(P, T), std::min(R, T), std::max(R, T));
                    const bool between = t > std::min(p, r) && t < std::max(p, r);
                    v += between ? -term : term;
                }
                A[k * N * N + (size_t)p * N + r] = v;
            }
    }
    for (size_t k = 0; k < other.size(); ++k) {
        const uint32_t s = other[k];
        for (int p = 0; p < N; ++p)
            for (int r = 0; r < N; ++r) {
                if (p == r) continue;
                const int P = p + off_self, R = r + off_self;
                double v = 0;
                for (int t = 0; t < N; ++t) {
                    if (!((s >> t) & 1)) continue;
                    const int T = t + off_other;
                    v += V(std::min(P, T), std::max(P, T), std::min(R, T), std::max(R, T));
                }
                B[k * N * N + (size_t)p * N + r] = v;
            }
    }
}

}  // namespace

void build_otf_tables(const Basis &B, const std::vector<double> &h1, const std::vector<double> &g2, OtfTables &T,
                      bool with_strings)
{
    const int N = B.N;
    T.N = N;
    T.P2 = N * (N - 1) / 2;
    TwoE V{N, g2.data()};
    if (with_strings) {
        string_lists(B.strA, B.rankA, N, B.na, T.sa_rank, T.sa_code, T.da_rank, T.da_code, T.nsa, T.nda);
        string_lists(B.strB, B.rankB, N, B.nb, T.sb_rank, T.sb_code, T.db_rank, T.db_code, T.nsb, T.ndb);
    }
    // same-spin doubles (pairs of orbitals inside one spin block; identical for both spins)
    T.vss.assign((size_t)T.P2 * T.P2, 0.0);
    for (int p1 = 0; p1 < N; ++p1)
        for (int p2 = p1 + 1; p2 < N; ++p2)
            for (int r1 = 0; r1 < N; ++r1)
                for (int r2 = r1 + 1; r2 < N; ++r2)
                    T.vss[(size_t)pair_index(p1, p2, N) * T.P2 + pair_index(r1, r2, N)] = V(p1, p2, r1, r2);
    // alpha-beta doubles: created {pb, pa+N}, destroyed {rb, ra+N}
    T.vab.assign((size_t)N * N * N * N, 0.0);
    for (int pa = 0; pa < N; ++pa)
        for (int ra = 0; ra < N; ++ra)
            for (int pb = 0; pb < N; ++pb)
                for (int rb = 0; rb < N; ++rb)
                    T.vab[(((size_t)pa * N + ra) * N + pb) * N + rb] = V(pb, pa + N, rb, ra + N);
    // singles: alpha (block N..2N-1), beta (block 0..N-1)
    single_tables(V, h1, N, N, 0, B.strA, B.strB, T.a_alpha, T.b_alpha);
    single_tables(V, h1, N, 0, N, B.strB, B.strA, T.a_beta, T.b_beta);
}

}  // namespace ae
