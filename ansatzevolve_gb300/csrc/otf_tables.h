// Host-built tables of the string-driven on-the-fly Hamiltonian (otf_tables.cpp).
#pragma once
#include "setup.h"

#include <cstdint>
#include <vector>

namespace ae {

struct OtfTables {
    int N = 0, P2 = 0;
    int nsa = 0, nda = 0, nsb = 0, ndb = 0;  // singles / doubles per alpha / beta string
    // per string (rank-major): excited-string rank and code.  Single code: p | r<<5 |
    // sign<<31 (p occupied, r empty); double code: pair(p1,p2)*P2 + pair(r1,r2) | sign<<31
    std::vector<int32_t> sa_rank, sa_code, da_rank, da_code;
    std::vector<int32_t> sb_rank, sb_code, db_rank, db_code;
    std::vector<double> vss;                 // [P2][P2] same-spin doubles
    std::vector<double> vab;                 // [pa][ra][pb][rb] alpha-beta doubles
    std::vector<double> a_alpha, b_alpha;    // [alpha string][p*N+r], [beta string][p*N+r]
    std::vector<double> a_beta, b_beta;      // [beta string][p*N+r],  [alpha string][p*N+r]
};

// with_strings = false skips the per-string excitation lists (they depend only on the
// basis), for the second and later instances of a batch that share them.
void build_otf_tables(const Basis &B, const std::vector<double> &h1, const std::vector<double> &g2, OtfTables &T,
                      bool with_strings = true);

}  // namespace ae
