// Per-path properties and subspace diagonalisation (TUPSQuantities::writeProperties,
// tupsquantities.cpp:185-568, and doSubspaceDiagonalisation, :1600-1700).  Host
// analysis only: energies, gradients, Hessians, metrics, overlaps and subspace matrices
// all come from the GPU engine through include/aegpu.h; what runs here is the small
// dense eigen-analysis the reference does with Eigen.
#include "../../include/aegpu.h"
#include "newton.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

namespace {

constexpr double kZeroThreshold = 1e-10;      // tupsquantities.cpp:468
constexpr double kSubspacePrecision = 1e-14;  // :1660

int num_ops(const aegpu_engine *e)
{
    int64_t info[8] = {0};
    if (aegpu_problem_info(e, info)) return -1;
    return (int)info[1];
}

// Eigenvalues of a Hermitian n x n matrix (row-major real and imaginary parts) from
// its real symmetric 2n x 2n embedding [[Re, -Im], [Im, Re]], whose spectrum is every
// eigenvalue twice; vecs (optional) are the embedding's eigenvectors.
void herm_eig(int n, const std::vector<double> &re, const std::vector<double> &im, std::vector<double> &w,
              std::vector<double> *vecs = nullptr)
{
    const int m = 2 * n;
    std::vector<double> A((size_t)m * m);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const double r = re[(size_t)i * n + j], c = im.empty() ? 0.0 : im[(size_t)i * n + j];
            A[(size_t)i * m + j] = r;
            A[(size_t)(i + n) * m + (j + n)] = r;
            A[(size_t)(i + n) * m + j] = c;
            A[(size_t)i * m + (j + n)] = -c;
        }
    std::vector<double> V;
    ae::sym_eig(m, A, w, V);
    if (vecs) vecs->swap(V);
}

}  // namespace

extern "C" {

int aegpu_path_properties(aegpu_engine *e, const double *angles, const int *param, const double *scale, int nparams,
                          double nuclear_energy, int flags, double *row, double *hessian, double *metric)
{
    if (!e || !angles || !param || !scale || nparams < 1 || !row) return AEGPU_ERR_ARG;
    const int nops = num_ops(e);
    if (nops < 0) return AEGPU_ERR_ARG;
    const double nan = std::numeric_limits<double>::quiet_NaN();
    for (int k = 0; k < AEGPU_PROPERTY_ROWS; ++k) row[k] = nan;
    const size_t P = (size_t)nparams;
    std::vector<double> g(P, 0.0), H, M;
    double E = 0.0;
    int rc;
    const bool withHessian = (flags & AEGPU_PROP_HESSIAN) != 0;
    if (withHessian) {
        H.resize(P * P);
        M.resize(P * P);
        rc = aegpu_hessian_metric(e, angles, param, scale, nparams, &E, g.data(), H.data(), M.data());
    } else {
        std::vector<double> gops((size_t)nops);
        rc = aegpu_gradient(e, angles, &E, gops.data());
        for (int o = 0; !rc && o < nops; ++o) {
            if (param[o] < 0 || param[o] >= nparams) return AEGPU_ERR_ARG;
            g[(size_t)param[o]] += scale[o] * gops[(size_t)o];
        }
    }
    if (rc) return rc;
    double realE = 0.0;
    if ((rc = aegpu_real_energy(e, angles, &realE))) return rc;
    row[AEGPU_PROP_ELEC_ENERGY] = E;
    row[AEGPU_PROP_REAL_ELEC_ENERGY] = realE;
    row[AEGPU_PROP_ELEC_NUC_ENERGY] = E + nuclear_energy;
    if (withHessian) {
        // eigenvalue and diagonal counts of the Hessian and the metric (:471-533)
        std::vector<double> w, V;
        ae::sym_eig(nparams, H, w, V);
        double neg = 0, zero = 0, pos = 0;
        for (double x : w) (x > kZeroThreshold ? pos : x < -kZeroThreshold ? neg : zero) += 1;
        row[AEGPU_PROP_NEG_HESSIAN_EVALUES] = neg;
        row[AEGPU_PROP_NEAR_ZERO_HESSIAN_EVALUES] = zero;
        row[AEGPU_PROP_POS_HESSIAN_EVALUES] = pos;
        neg = zero = pos = 0;
        for (size_t i = 0; i < P; ++i) {
            const double x = H[i * P + i];
            (x > kZeroThreshold ? pos : x < -kZeroThreshold ? neg : zero) += 1;
        }
        row[AEGPU_PROP_NEG_HESSIAN_DIAG] = neg;
        row[AEGPU_PROP_NEAR_ZERO_HESSIAN_DIAG] = zero;
        row[AEGPU_PROP_POS_HESSIAN_DIAG] = pos;
        ae::sym_eig(nparams, M, w, V);
        pos = zero = 0;
        for (double x : w) {
            if (x > kZeroThreshold) pos += 1;
            else if (x >= -kZeroThreshold) zero += 1;  // below -threshold: reported as a problem, not counted
        }
        row[AEGPU_PROP_POS_METRIC_EVALUES] = pos;
        row[AEGPU_PROP_ZERO_METRIC_EVALUES] = zero;
        zero = 0;
        for (size_t i = 0; i < P; ++i) zero += std::abs(M[i * P + i]) <= kZeroThreshold ? 1 : 0;
        row[AEGPU_PROP_ZERO_METRIC_DIAG] = zero;
        if (hessian) std::copy(H.begin(), H.end(), hessian);
        if (metric) std::copy(M.begin(), M.end(), metric);
    }
    double gn = 0.0;
    for (double x : g) gn += x * x;
    row[AEGPU_PROP_NORM_OF_GRAD] = std::sqrt(gn);
    if (flags & AEGPU_PROP_OVERLAP) {
        double ov[2];
        if ((rc = aegpu_ground_overlap(e, angles, ov))) return rc;
        row[AEGPU_PROP_OVERLAP_RE] = ov[0];
        row[AEGPU_PROP_OVERLAP_IM] = ov[1];
        row[AEGPU_PROP_OVERLAP_MAG] = std::hypot(ov[0], ov[1]);
    }
    return AEGPU_OK;
}

int aegpu_host_tridiag_lowest(int k, const double *a, const double *b, double *v, double *theta)
{
    if (k < 1 || !a || (k > 1 && !b) || !v || !theta) return AEGPU_ERR_ARG;
    std::vector<double> av(a, a + k), bv(b ? b : a, b ? b + (k - 1) : a), vv;
    *theta = ae::tridiag_lowest(av, bv, k, vv);
    std::copy(vv.begin(), vv.end(), v);
    return AEGPU_OK;
}

int aegpu_host_tridiag_lowest_k(int k, int nev, const double *a, const double *b, double *theta, double *V)
{
    if (k < 1 || nev < 1 || nev > k || !a || (k > 1 && !b) || !theta || !V) return AEGPU_ERR_ARG;
    std::vector<double> av(a, a + k), bv(b ? b : a, b ? b + (k - 1) : a), th, vv;
    ae::tridiag_lowest_k(av, bv, k, nev, th, vv);
    std::copy(th.begin(), th.end(), theta);
    std::copy(vv.begin(), vv.end(), V);
    return AEGPU_OK;
}

int aegpu_subspace_eigenvalues(aegpu_engine *e, int nsets, const double *angles, double *eigenvalues, int *null_rank)
{
    if (!e || nsets < 1 || !angles || !eigenvalues) return AEGPU_ERR_ARG;
    const size_t n = (size_t)nsets;
    std::vector<double> hr(n * n), hi(n * n), sr(n * n), si(n * n);
    int rc = aegpu_subspace_matrices(e, nsets, angles, hr.data(), hi.data(), sr.data(), si.data());
    if (rc) return rc;
    return aegpu_host_subspace_eigenvalues(nsets, hr.data(), hi.data(), sr.data(), si.data(), eigenvalues, null_rank);
}

int aegpu_host_subspace_eigenvalues(int nsets, const double *h_re, const double *h_im, const double *s_re,
                                    const double *s_im, double *eigenvalues, int *null_rank)
{
    if (nsets < 1 || !h_re || !s_re || !eigenvalues) return AEGPU_ERR_ARG;
    const size_t n = (size_t)nsets;
    std::vector<double> hr(h_re, h_re + n * n), sr(s_re, s_re + n * n);
    std::vector<double> hi = h_im ? std::vector<double>(h_im, h_im + n * n) : std::vector<double>(n * n, 0.0);
    std::vector<double> si = s_im ? std::vector<double>(s_im, s_im + n * n) : std::vector<double>(n * n, 0.0);
    // S^-1/2 over the range of S (eigenvalues below the precision are the null space),
    // then the eigenvalues of S^-1/2 H S^-1/2 (:1656-1684).  In the real embedding every
    // eigenvalue appears twice: take every second one.
    std::vector<double> ws, Vs;
    herm_eig(nsets, sr, si, ws, &Vs);
    const int m = 2 * nsets;
    int nullr = 0;
    std::vector<double> f((size_t)m);
    for (int k = 0; k < m; ++k) {
        if (ws[(size_t)k] < kSubspacePrecision) {
            f[(size_t)k] = 0.0;
            ++nullr;
        } else {
            f[(size_t)k] = 1.0 / std::sqrt(ws[(size_t)k]);
        }
    }
    std::vector<double> X((size_t)m * m, 0.0);  // embedded S^-1/2 = V diag(f) V^T
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) {
            double acc = 0.0;
            for (int k = 0; k < m; ++k) acc += Vs[(size_t)i * m + k] * f[(size_t)k] * Vs[(size_t)j * m + k];
            X[(size_t)i * m + j] = acc;
        }
    std::vector<double> He((size_t)m * m);  // embedded H
    for (int i = 0; i < nsets; ++i)
        for (int j = 0; j < nsets; ++j) {
            const double r = hr[(size_t)i * n + j], c = hi[(size_t)i * n + j];
            He[(size_t)i * m + j] = r;
            He[(size_t)(i + nsets) * m + (j + nsets)] = r;
            He[(size_t)(i + nsets) * m + j] = c;
            He[(size_t)i * m + (j + nsets)] = -c;
        }
    std::vector<double> T((size_t)m * m, 0.0), Y((size_t)m * m, 0.0);
    for (int i = 0; i < m; ++i)
        for (int k = 0; k < m; ++k) {
            const double x = X[(size_t)i * m + k];
            for (int j = 0; j < m; ++j) T[(size_t)i * m + j] += x * He[(size_t)k * m + j];
        }
    for (int i = 0; i < m; ++i)
        for (int k = 0; k < m; ++k) {
            const double t = T[(size_t)i * m + k];
            for (int j = 0; j < m; ++j) Y[(size_t)i * m + j] += t * X[(size_t)k * m + j];
        }
    for (int i = 0; i < m; ++i)  // symmetrise against rounding
        for (int j = 0; j < i; ++j) {
            const double a = 0.5 * (Y[(size_t)i * m + j] + Y[(size_t)j * m + i]);
            Y[(size_t)i * m + j] = Y[(size_t)j * m + i] = a;
        }
    std::vector<double> wy, Vy;
    ae::sym_eig(m, Y, wy, Vy);
    for (int k = 0; k < nsets; ++k) eigenvalues[k] = wy[(size_t)2 * k];
    if (null_rank) *null_rank = nullr / 2;
    return AEGPU_OK;
}

}  // extern "C"
