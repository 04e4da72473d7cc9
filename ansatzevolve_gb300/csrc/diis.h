// DIIS extrapolation of the projected iteration (the reference's DIIS class, diis.h:16-209,
// used by TUPSQuantities::iterativeTups, tupsquantities.cpp:2072-2128): a history of
// (quantity, error vector) pairs; the next quantity is sum_i c_i q_i with sum_i c_i = 1 and
// the c minimising c^T B c, B_ij = <e_i|e_j> (the real part of the inner product).
//   Pulay DIIS: c = B^+ 1 / (1^T B^+ 1), B^+ the minimum-norm pseudo-inverse.
//   EDIIS: c_i = t_i^2 (so c >= 0), with (t, lambda) a stationary point of
//     t^2 . B t^2 - lambda (sum t^2 - 1), found by Newton-Raphson from t_i = sqrt(n),
//     lambda = 1 (simpleNewtonRaphson, diis.cpp:11-66).
#pragma once
#include <cstddef>
#include <deque>
#include <vector>

namespace ae {

// The coefficient step alone on a given n x n matrix B (row-major); c has n entries.
void diis_coefficients(int n, const std::vector<double> &B, bool ediis, std::vector<double> &c);

class Diis {
public:
    Diis(size_t maxSize, bool ediis) : m_max(maxSize), m_ediis(ediis) {}
    void reset()
    {
        m_q.clear();
        m_e.clear();
        m_B.clear();
    }
    size_t size() const { return m_q.size(); }
    void addNew(const std::vector<double> &quantity, const std::vector<double> &error);
    // next quantity and (optional) the extrapolated error sum_i c_i e_i
    bool getNext(std::vector<double> &quantity, std::vector<double> *extrapolatedError = nullptr);

private:
    size_t m_max;
    bool m_ediis;
    std::deque<std::vector<double>> m_q, m_e;
    std::deque<std::deque<double>> m_B;  // inner products of the stored error vectors
};

}  // namespace ae
