// Newton-Raphson optimiser of the TUPS angles (restates TUPSQuantities::OptimiseTups).
#pragma once
#include <cstdint>
#include <functional>
#include <vector>

namespace ae {

struct NewtonProblem {
    int nparams = 0;
    std::vector<int> param;       // per operator: compressed parameter
    std::vector<double> scale;    // per operator: scale factor
    double gtol = 1e-12;          // stop when |g| < gtol (tupsquantities.cpp:1233, 1982)
    // theta: per-operator angles.  E, g (compressed), H (compressed, row-major)
    std::function<bool(const std::vector<double> &theta, double &E, std::vector<double> &g)> energy_grad;
    std::function<bool(const std::vector<double> &theta, double &E, std::vector<double> &g, std::vector<double> &H)> hessian;
};

struct NewtonStats {
    int64_t hessian_evals = 0, energy_evals = 0;
    double energy = 0, gnorm = 0;
};

void sym_eig(int n, const std::vector<double> &A, std::vector<double> &w, std::vector<double> &V);
// Lowest eigenvalue (returned) and unit eigenvector v of the symmetric tridiagonal
// matrix with diagonal a[0..k-1] and off-diagonal b[0..k-2].
double tridiag_lowest(const std::vector<double> &a, const std::vector<double> &b, int k, std::vector<double> &v);
// The nev lowest eigenvalues (ascending) and unit eigenvectors V[j * k + i] of the same
// matrix.
void tridiag_lowest_k(const std::vector<double> &a, const std::vector<double> &b, int k, int nev,
                      std::vector<double> &theta, std::vector<double> &V);
bool optimise_newton(NewtonProblem &p, std::vector<double> &theta, NewtonStats &st, bool verbose);

// The projected iteration (TUPSQuantities::iterativeTups, tupsquantities.cpp:2044-2145,
// with runNewtonMethodProjected, :1238-1465): the bra psiH = H psi(theta_prev) is frozen,
// <psiH|psi(theta)> is minimised by Newton steps with the projected Hessian, then psiH is
// renewed; stops when the projected gradient at the renewed bra is below gtol.
struct ProjectedProblem {
    int nparams = 0;
    std::vector<int> param;
    std::vector<double> scale;
    double gtol = 1e-5;             // tupsquantities.cpp:2096
    int max_outer = 3000;           // :2076
    // DIIS over the outer iterations (:2101-2122, off in the reference: doDIIS = false):
    // history length (0 = off; the reference's is 15) and EDIIS (true) or Pulay DIIS
    int diis_size = 0;
    bool ediis = true;
    // psi = psi(theta) and psiH = H psi (device-size vectors on the host)
    std::function<bool(const std::vector<double> &theta, std::vector<double> &psiH, std::vector<double> &psi)> bra;
    // overlap <psiH|psi(theta)> and its compressed gradient
    std::function<bool(const std::vector<double> &theta, const std::vector<double> &psiH, double &ov,
                       std::vector<double> &g)> proj_grad;
    // overlap, compressed gradient and compressed Hessian (row-major)
    std::function<bool(const std::vector<double> &theta, const std::vector<double> &psiH, double &ov,
                       std::vector<double> &g, std::vector<double> &H)> proj_hess;
};

bool optimise_projected(ProjectedProblem &p, std::vector<double> &theta, NewtonStats &st, int &outer_iters);

}  // namespace ae
