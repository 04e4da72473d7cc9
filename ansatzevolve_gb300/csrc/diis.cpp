// DIIS extrapolation (see diis.h).  Host-only and small: the history holds at most
// maxSize vectors, and B is kept incrementally (one row of inner products per new error
// vector).
#include "diis.h"

#include "newton.h"

#include <algorithm>
#include <cmath>
#include <limits>

namespace ae {

namespace {

double dot(const std::vector<double> &a, const std::vector<double> &b)
{
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
}

double norm(const std::vector<double> &v) { return std::sqrt(dot(v, v)); }

// minimum-norm solution of the symmetric system A x = r (pseudo-inverse over the
// eigenvalues above n * eps * max |eigenvalue|, or above an absolute floor)
std::vector<double> sym_pinv_solve(int n, const std::vector<double> &A, const std::vector<double> &r, double floor_abs,
                                   bool relative)
{
    std::vector<double> w, V;
    sym_eig(n, A, w, V);
    double wmax = 0.0;
    for (double x : w) wmax = std::max(wmax, std::abs(x));
    const double cut = relative ? n * std::numeric_limits<double>::epsilon() * wmax : floor_abs;
    std::vector<double> x(n, 0.0);
    for (int k = 0; k < n; ++k) {
        if (!(std::abs(w[k]) > cut)) continue;
        double p = 0.0;
        for (int i = 0; i < n; ++i) p += V[(size_t)i * n + k] * r[i];
        p /= w[k];
        for (int i = 0; i < n; ++i) x[i] += V[(size_t)i * n + k] * p;
    }
    return x;
}

// simpleNewtonRaphson (diis.cpp:11-66) on the EDIIS Lagrangian in (t, lambda)
std::vector<double> ediis_coefficients(int n, const std::vector<double> &B)
{
    const int m = n + 1;
    std::vector<double> pt(m, std::sqrt((double)n));
    pt[n] = 1.0;
    auto grad = [&](const std::vector<double> &p) {
        std::vector<double> g(m), t2(n);
        for (int i = 0; i < n; ++i) t2[i] = p[i] * p[i];
        double s = 0.0;
        for (int i = 0; i < n; ++i) {
            double bt = 0.0;
            for (int j = 0; j < n; ++j) bt += B[(size_t)i * n + j] * t2[j];
            g[i] = 4.0 * bt * p[i] - 2.0 * p[n] * p[i];
            s += t2[i];
        }
        g[n] = 1.0 - s;
        return g;
    };
    auto hess = [&](const std::vector<double> &p) {
        std::vector<double> H((size_t)m * m, 0.0), t2(n);
        for (int i = 0; i < n; ++i) t2[i] = p[i] * p[i];
        for (int i = 0; i < n; ++i) {
            double bt = 0.0;
            for (int j = 0; j < n; ++j) bt += B[(size_t)i * n + j] * t2[j];
            for (int j = 0; j < n; ++j) H[(size_t)i * m + j] = 8.0 * p[i] * B[(size_t)i * n + j] * p[j];
            H[(size_t)i * m + i] += 4.0 * bt - 2.0 * p[n];
            H[(size_t)i * m + n] = H[(size_t)n * m + i] = -2.0 * p[i];
        }
        return H;
    };
    for (int left = 200; left-- > 0;) {
        const std::vector<double> g = grad(pt), H = hess(pt);
        const double gn = norm(g);
        if (gn < 1e-12) break;
        std::vector<double> w, V;
        sym_eig(m, H, w, V);
        std::vector<double> step(m, 0.0);
        for (int k = 0; k < m; ++k) {
            if (std::abs(w[k]) < 1e-6) continue;
            double p = 0.0;
            for (int i = 0; i < m; ++i) p += V[(size_t)i * m + k] * g[i];
            p /= w[k];
            for (int i = 0; i < m; ++i) step[i] -= V[(size_t)i * m + k] * p;
        }
        for (int i = 0; i < m; ++i) pt[i] += step[i];
        auto infn = [&] {
            double x = 0.0;
            for (double s : step) x = std::max(x, std::abs(s));
            return x;
        };
        while (norm(grad(pt)) > gn && infn() > 1e-15) {
            for (int i = 0; i < m; ++i) {
                step[i] *= 0.5;
                pt[i] -= step[i];
            }
        }
        if (!(infn() > 1e-15)) break;
    }
    std::vector<double> c(n);
    for (int i = 0; i < n; ++i) c[i] = pt[i] * pt[i];
    return c;
}

}  // namespace

void diis_coefficients(int n, const std::vector<double> &B, bool ediis, std::vector<double> &c)
{
    if (ediis) {
        c = ediis_coefficients(n, B);
        return;
    }
    c = sym_pinv_solve(n, B, std::vector<double>(n, 1.0), 0.0, true);
    double s = 0.0;
    for (double x : c) s += x;
    if (s == 0.0) {
        std::fill(c.begin(), c.end(), 0.0);
        c[n - 1] = 1.0;
    } else {
        for (double &x : c) x /= s;
    }
}

void Diis::addNew(const std::vector<double> &quantity, const std::vector<double> &error)
{
    std::deque<double> row;
    for (size_t i = 0; i < m_e.size(); ++i) {
        const double b = dot(m_e[i], error);
        m_B[i].push_back(b);
        row.push_back(b);
    }
    row.push_back(dot(error, error));
    m_B.push_back(row);
    m_q.push_back(quantity);
    m_e.push_back(error);
    if (m_q.size() > m_max) {
        m_q.pop_front();
        m_e.pop_front();
        m_B.pop_front();
        for (auto &r : m_B) r.pop_front();
    }
}

bool Diis::getNext(std::vector<double> &quantity, std::vector<double> *extrapolatedError)
{
    const int n = (int)m_q.size();
    if (n == 0) return false;
    std::vector<double> B((size_t)n * n), c;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) B[(size_t)i * n + j] = m_B[i][j];
    diis_coefficients(n, B, m_ediis, c);
    quantity.assign(m_q[0].size(), 0.0);
    for (int i = 0; i < n; ++i)
        for (size_t k = 0; k < quantity.size(); ++k) quantity[k] += c[i] * m_q[i][k];
    if (extrapolatedError) {
        extrapolatedError->assign(m_e[0].size(), 0.0);
        for (int i = 0; i < n; ++i)
            for (size_t k = 0; k < extrapolatedError->size(); ++k) (*extrapolatedError)[k] += c[i] * m_e[i][k];
    }
    return true;
}

}  // namespace ae
