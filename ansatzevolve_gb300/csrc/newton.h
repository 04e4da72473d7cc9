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
bool optimise_newton(NewtonProblem &p, std::vector<double> &theta, NewtonStats &st, bool verbose);

}  // namespace ae
