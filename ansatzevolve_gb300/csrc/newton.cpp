// Newton-Raphson optimiser of the TUPS angles (TUPSQuantities::OptimiseTups,
// tupsquantities.cpp:1940-2011; runNewtonMethod :704-1236; the negative-curvature
// escape doStepsUntilHessianIsPositiveDefinite :1467-1598).  Host-side control
// only: every energy, gradient and Hessian comes from the GPU engine through the
// callbacks.  The step is -V |Lambda|^-1 V^T g over the eigenpairs of the
// compressed Hessian (|lambda| >= 1e-10), followed by the reference's cubic
// model line search on t in (0, 1.5].
#include "newton.h"

#include "diis.h"

#include <algorithm>
#include <cmath>
#include <cstdio>

namespace ae {

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major).
// Eigenvalues ascending; V column k is the eigenvector of w[k].
void sym_eig(int n, const std::vector<double> &A_in, std::vector<double> &w, std::vector<double> &V)
{
    std::vector<double> A = A_in;
    V.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0, tot = 0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double a = A[(size_t)i * n + j] * A[(size_t)i * n + j];
                tot += a;
                if (i != j) off += a;
            }
        if (off <= 1e-30 * std::max(tot, 1e-300)) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[(size_t)p * n + q];
                if (std::abs(apq) < 1e-300) continue;
                const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
                const double theta = (aqq - app) / (2 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::abs(theta) + std::sqrt(theta * theta + 1));
                const double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
                    A[(size_t)k * n + p] = c * akp - s * akq;
                    A[(size_t)k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
                    A[(size_t)p * n + k] = c * apk - s * aqk;
                    A[(size_t)q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
                    V[(size_t)k * n + p] = c * vkp - s * vkq;
                    V[(size_t)k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return A[(size_t)a * n + a] < A[(size_t)b * n + b]; });
    w.resize(n);
    std::vector<double> V2((size_t)n * n);
    for (int k = 0; k < n; ++k) {
        w[k] = A[(size_t)order[k] * n + order[k]];
        for (int i = 0; i < n; ++i) V2[(size_t)i * n + k] = V[(size_t)i * n + order[k]];
    }
    V.swap(V2);
}

// Lowest eigenpair of the symmetric tridiagonal matrix with diagonal a[0..k-1] and
// off-diagonal b[0..k-2]: the eigenvalue by Sturm-sequence bisection, the unit
// eigenvector by inverse iteration with the LDL^T factors of the shifted matrix, which
// the shift just below the eigenvalue keeps positive definite.
void tridiag_lowest_k(const std::vector<double> &a, const std::vector<double> &b, int k, int nev,
                      std::vector<double> &theta, std::vector<double> &V)
{
    // eigenvalue j by bisection on the Sturm count (below(x) = eigenvalues below x),
    // its vector by shifted inverse iteration, orthogonalised against the earlier ones
    // (close eigenvalues give nearly parallel iterates otherwise)
    nev = std::min(nev, k);
    double lo0 = a[0], hi0 = a[0], scale = 0.0;
    for (int i = 0; i < k; ++i) {
        const double r = (i > 0 ? std::abs(b[i - 1]) : 0.0) + (i + 1 < k ? std::abs(b[i]) : 0.0);
        lo0 = std::min(lo0, a[i] - r);
        hi0 = std::max(hi0, a[i] + r);
        scale = std::max(scale, std::abs(a[i]) + r);
    }
    const double tiny = std::max(scale, 1e-300) * 1e-300;
    auto below = [&](double x) {
        int c = 0;
        double q = a[0] - x;
        for (int i = 0;; ++i) {
            if (q < 0) ++c;
            if (i + 1 == k) break;
            if (std::abs(q) < tiny) q = -tiny;
            q = a[i + 1] - x - b[i] * b[i] / q;
        }
        return c;
    };
    theta.assign(nev, 0.0);
    V.assign((size_t)nev * k, 0.0);
    for (int j = 0; j < nev; ++j) {
        double lo = lo0, hi = hi0;
        for (int it = 0; it < 2100 && hi - lo > 4e-16 * std::max(std::abs(lo), std::abs(hi)); ++it) {
            const double mid = 0.5 * (lo + hi);
            if (mid <= lo || mid >= hi) break;
            if (below(mid) >= j + 1) hi = mid; else lo = mid;
        }
        theta[j] = 0.5 * (lo + hi);
        const double sigma = theta[j] - std::max(scale, 1e-300) * 1e-13;
        std::vector<double> d(k), l(k, 0.0);
        d[0] = a[0] - sigma;
        for (int i = 1; i < k; ++i) {
            l[i] = b[i - 1] / (std::abs(d[i - 1]) < tiny ? tiny : d[i - 1]);
            d[i] = a[i] - sigma - l[i] * b[i - 1];
        }
        for (int i = 0; i < k; ++i)
            if (std::abs(d[i]) < tiny) d[i] = tiny;
        double *v = &V[(size_t)j * k];
        for (int i = 0; i < k; ++i) v[i] = 1.0 / std::sqrt((double)k) * ((i + j) % 2 ? -1.0 : 1.0);
        for (int it = 0; it < 4; ++it) {
            for (int i = 1; i < k; ++i) v[i] -= l[i] * v[i - 1];
            for (int i = 0; i < k; ++i) v[i] /= d[i];
            for (int i = k - 2; i >= 0; --i) v[i] -= l[i + 1] * v[i + 1];
            for (int q = 0; q < j; ++q) {
                const double *u = &V[(size_t)q * k];
                double c = 0.0;
                for (int i = 0; i < k; ++i) c += u[i] * v[i];
                for (int i = 0; i < k; ++i) v[i] -= c * u[i];
            }
            double nv = 0.0;
            for (int i = 0; i < k; ++i) nv += v[i] * v[i];
            nv = std::sqrt(nv);
            for (int i = 0; i < k; ++i) v[i] /= nv;
        }
    }
}

double tridiag_lowest(const std::vector<double> &a, const std::vector<double> &b, int k, std::vector<double> &v)
{
    double lo = a[0], hi = a[0], scale = 0.0;
    for (int i = 0; i < k; ++i) {
        const double r = (i > 0 ? std::abs(b[i - 1]) : 0.0) + (i + 1 < k ? std::abs(b[i]) : 0.0);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
        scale = std::max(scale, std::abs(a[i]) + r);
    }
    const double tiny = std::max(scale, 1e-300) * 1e-300;
    auto below = [&](double x) {  // number of eigenvalues below x
        int c = 0;
        double q = a[0] - x;
        for (int i = 0;; ++i) {
            if (q < 0) ++c;
            if (i + 1 == k) break;
            if (std::abs(q) < tiny) q = -tiny;
            q = a[i + 1] - x - b[i] * b[i] / q;
        }
        return c;
    };
    for (int it = 0; it < 2100 && hi - lo > 4e-16 * std::max(std::abs(lo), std::abs(hi)); ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (below(mid) >= 1) hi = mid; else lo = mid;
    }
    const double theta = 0.5 * (lo + hi);
    const double sigma = theta - std::max(scale, 1e-300) * 1e-13;
    std::vector<double> d(k), l(k, 0.0);
    d[0] = a[0] - sigma;
    for (int i = 1; i < k; ++i) {
        l[i] = b[i - 1] / d[i - 1];
        d[i] = a[i] - sigma - l[i] * b[i - 1];
    }
    v.assign(k, 1.0 / std::sqrt((double)k));
    for (int it = 0; it < 3; ++it) {
        for (int i = 1; i < k; ++i) v[i] -= l[i] * v[i - 1];
        for (int i = 0; i < k; ++i) v[i] /= d[i];
        for (int i = k - 2; i >= 0; --i) v[i] -= l[i + 1] * v[i + 1];
        double nv = 0.0;
        for (double x : v) nv += x * x;
        nv = std::sqrt(nv);
        for (double &x : v) x /= nv;
    }
    return theta;
}

static double norm2(const std::vector<double> &v)
{
    double s = 0;
    for (double x : v) s += x * x;
    return std::sqrt(s);
}

// theta (per operator) += t * D dx (D_{i mu} = scale_i [param_i = mu])
static void step(std::vector<double> &th, const std::vector<double> &base, const NewtonProblem &p, const std::vector<double> &dx,
                 long double t)
{
    th = base;
    for (size_t i = 0; i < th.size(); ++i) th[i] += (double)(t * (long double)(p.scale[i] * dx[p.param[i]]));
}

// runNewtonMethod, tupsquantities.cpp:704-1236 (the "else" branch that is active).
static bool run_newton(NewtonProblem &p, std::vector<double> &th, NewtonStats &st, bool verbose)
{
    const int P = p.nparams;
    const double zeroThreshold = 1e-10;
    std::vector<double> g, H, w, V, gt;
    for (int count = 0; count < 500; ++count) {
        double E;
        if (!p.hessian(th, E, g, H)) return false;
        st.hessian_evals++;
        st.energy_evals++;
        sym_eig(P, H, w, V);
        // dx = -V |1/lambda| V^T g
        std::vector<double> vg(P, 0.0), dx(P, 0.0);
        for (int k = 0; k < P; ++k) {
            double s = 0;
            for (int i = 0; i < P; ++i) s += V[(size_t)i * P + k] * g[i];
            vg[k] = std::abs(w[k]) >= zeroThreshold ? s * std::abs(1.0 / w[k]) : 0.0;
        }
        for (int i = 0; i < P; ++i) {
            double s = 0;
            for (int k = 0; k < P; ++k) s += V[(size_t)i * P + k] * vg[k];
            dx[i] = -s;
        }
        const std::vector<double> base = th;
        long double tMax = 1.5, t = 1, newT = 1;
        step(th, base, p, dx, t);
        long double Hdd = 0, gd = 0;
        for (int i = 0; i < P; ++i) {
            double s = 0;
            for (int j = 0; j < P; ++j) s += H[(size_t)i * P + j] * dx[j];
            Hdd += (long double)dx[i] * s;
            gd += (long double)dx[i] * g[i];
        }
        double gnorm = norm2(g);
        int searchCount = 0;
        while (true) {
            searchCount++;
            double Et;
            if (!p.energy_grad(th, Et, gt)) return false;
            st.energy_evals++;
            long double b = Hdd, c = gd, fd = 0;
            for (int i = 0; i < P; ++i) fd += (long double)gt[i] * dx[i];
            long double a = (fd - (b + c)) / (t * t);
            b /= t;
            const long double disc = b * b - 4 * a * c;
            if (a >= 0) {
                newT = (-b + std::sqrt(disc)) / (2 * a);
            } else if (disc >= 0) {
                const long double t1 = (-b + std::sqrt(disc)) / (2 * a);
                const long double E1 = a * t1 * t1 * t1 / 3 + b * t1 * t1 / 2 + c * t1 + E;
                const long double E2 = a * tMax * tMax * tMax / 3 + b * tMax * tMax / 2 + c * tMax + E;
                newT = E2 < E1 ? tMax : t1;
            } else {
                newT = tMax;
            }
            double stepNorm = 0;
            for (size_t i = 0; i < th.size(); ++i) {
                const double d = (double)(newT * (long double)(p.scale[i] * dx[p.param[i]]));
                stepNorm += d * d;
            }
            stepNorm = std::sqrt(stepNorm);
            if (Et - E > 1e-10 && gnorm > 1e-8 && stepNorm > 1e-8) {
                t = t / 2;
                tMax = tMax / 2;
                step(th, base, p, dx, t);
                if (searchCount > 20) break;
            } else {
                if (newT > tMax) newT = tMax;
                step(th, base, p, dx, newT);
                break;
            }
        }
        if (verbose) fprintf(stderr, "Energy: %.10lg GradNorm: %lg Energy Evals: %ld, Hess Evals: %ld\n", E, gnorm,
                             (long)st.energy_evals, (long)st.hessian_evals);
        if (gnorm < p.gtol) break;
    }
    return true;
}

// doStepsUntilHessianIsPositiveDefinite(..., doDerivativeSteps = false), :1467-1598
static bool escape_negative(NewtonProblem &p, std::vector<double> &th, NewtonStats &st, bool &solved)
{
    const int P = p.nparams;
    solved = false;
    std::vector<double> g, H, w, V;
    for (int count = 0; count < 10; ++count) {
        double E;
        if (!p.hessian(th, E, g, H)) return false;
        st.hessian_evals++;
        sym_eig(P, H, w, V);
        bool found = false;
        std::vector<double> dx(P, 0.0);
        for (int k = 0; k < P; ++k)
            if (w[k] < -1e-7) {
                found = solved = true;
                for (int i = 0; i < P; ++i) dx[i] += V[(size_t)i * P + k] * 0.01;
            }
        const std::vector<double> base = th;
        step(th, base, p, dx, 1);
        if (!found) break;
    }
    return true;
}

bool optimise_newton(NewtonProblem &p, std::vector<double> &th, NewtonStats &st, bool verbose)
{
    bool amStuck = false;
    std::vector<double> g;
    for (int outer = 0; outer < 100; ++outer) {
        if (!run_newton(p, th, st, verbose)) return false;
        bool found = false;
        if (!escape_negative(p, th, st, found)) return false;
        double E;
        if (!p.energy_grad(th, E, g)) return false;
        st.energy_evals++;
        st.energy = E;
        st.gnorm = norm2(g);
        if (verbose) fprintf(stderr, "Energy: %.15lg GradNorm: %lg\n", E, st.gnorm);
        if (st.gnorm < p.gtol) break;
        if (!found && amStuck) break;
        amStuck = !found;
    }
    return true;
}

// runNewtonMethodProjected (tupsquantities.cpp:1238-1465, the active branch: no
// overlap normalisation, |1/lambda| steps, cubic line search with forward steps, at
// most 6 trial points, stop at |g| < 1e-10 or after 500 Hessians).
static bool run_newton_projected(ProjectedProblem &p, std::vector<double> &th, const std::vector<double> &psiH,
                                 NewtonStats &st)
{
    const int P = p.nparams;
    const double zeroThreshold = 1e-10;
    std::vector<double> g, H, w, V, gt;
    NewtonProblem np;  // for step()
    np.param = p.param;
    np.scale = p.scale;
    for (int count = 0; count < 500; ++count) {
        double E;
        if (!p.proj_hess(th, psiH, E, g, H)) return false;
        st.hessian_evals++;
        st.energy_evals++;
        sym_eig(P, H, w, V);
        std::vector<double> vg(P, 0.0), dx(P, 0.0);
        for (int k = 0; k < P; ++k) {
            double s = 0;
            for (int i = 0; i < P; ++i) s += V[(size_t)i * P + k] * g[i];
            vg[k] = std::abs(w[k]) >= zeroThreshold ? s * std::abs(1.0 / w[k]) : 0.0;
        }
        for (int i = 0; i < P; ++i) {
            double s = 0;
            for (int k = 0; k < P; ++k) s += V[(size_t)i * P + k] * vg[k];
            dx[i] = -s;
        }
        const double gnorm = norm2(g);
        long double bH = 0, cg = 0;
        for (int i = 0; i < P; ++i) {
            double s = 0;
            for (int j = 0; j < P; ++j) s += H[(size_t)i * P + j] * dx[j];
            bH += (long double)dx[i] * s;
            cg += (long double)dx[i] * g[i];
        }
        const std::vector<double> base = th;
        const size_t maxSearch = 5;
        size_t searchCount = 0;
        long double tMax = 1.5, t = 1, newT = 1, lastGood = newT;
        bool forward = false;
        step(th, base, np, dx, t);
        while (true) {
            searchCount++;
            double Et;
            if (!p.proj_grad(th, psiH, Et, gt)) return false;
            st.energy_evals++;
            long double b = bH, c = cg, found = 0;
            for (int i = 0; i < P; ++i) found += (long double)gt[i] * dx[i];
            long double a = (found - (b + c)) / (t * t);
            b /= t;
            if (Et < E && gnorm > 1e-5) forward = true;
            const long double disc = b * b - 4 * a * c;
            if (a >= 0) {
                newT = (-b + std::sqrt(disc)) / (2 * a);
            } else if (disc >= 0) {
                const long double t1 = (-b + std::sqrt(disc)) / (2 * a);
                const long double E1 = a * t1 * t1 * t1 / 3 + b * t1 * t1 / 2 + c * t1 + E;
                const long double E2 = a * tMax * tMax * tMax / 3 + b * tMax * tMax / 2 + c * tMax + E;
                newT = E2 < E1 ? tMax : t1;
            } else {
                newT = tMax;
            }
            if (newT > tMax) newT = tMax;
            step(th, base, np, dx, newT);
            if (searchCount > maxSearch) break;
            if (Et > E && gnorm > 1e-5) {
                if (forward) {
                    if (lastGood > tMax / 2) lastGood = tMax / 2;
                    t = t / 2;
                    tMax = tMax / 2;
                    newT = lastGood;
                    step(th, base, np, dx, newT);
                    break;
                }
                forward = false;
                t = t / 2;
                tMax = tMax / 2;
                step(th, base, np, dx, t);
            } else {
                if (forward) {
                    t = 2 * t;
                    tMax = 2 * tMax;
                    step(th, base, np, dx, t);
                    lastGood = newT;
                } else {
                    if (newT > tMax) newT = tMax;
                    step(th, base, np, dx, newT);
                    break;
                }
            }
        }
        if (gnorm < 1e-10) break;
    }
    return true;
}

bool optimise_projected(ProjectedProblem &p, std::vector<double> &th, NewtonStats &st, int &outer_iters)
{
    std::vector<double> psiH, g, psi, prevPsi;
    if (!p.bra(th, psiH, prevPsi)) return false;
    outer_iters = 0;
    double E = 0, gnorm = 0;
    Diis diis((size_t)std::max(p.diis_size, 1), p.ediis);
    const size_t nops = th.size();
    while (outer_iters++ < p.max_outer) {
        if (!run_newton_projected(p, th, psiH, st)) return false;
        if (!p.bra(th, psiH, psi)) return false;
        if (!p.proj_grad(th, psiH, E, g)) return false;
        st.energy_evals++;
        gnorm = norm2(g);
        if (gnorm < p.gtol) break;
        if (p.diis_size > 0 && outer_iters < p.max_outer) {  // the returned angles keep their energy
            // compressed angles (first operator of each parameter) and the change of
            // the state as the error vector; the extrapolated angles start the next
            // Newton run, with the bra of the unextrapolated state (:2101-2122)
            std::vector<double> x(p.nparams, 0.0), err(psi.size());
            std::vector<bool> seen(p.nparams, false);
            for (size_t o = 0; o < nops; ++o)
                if (!seen[p.param[o]] && p.scale[o] != 0) {
                    x[p.param[o]] = th[o] / p.scale[o];
                    seen[p.param[o]] = true;
                }
            for (size_t i = 0; i < psi.size(); ++i) err[i] = psi[i] - prevPsi[i];
            diis.addNew(x, err);
            diis.getNext(x);
            for (size_t o = 0; o < nops; ++o) th[o] = p.scale[o] * x[p.param[o]];
        }
        prevPsi.swap(psi);
    }
    st.energy = E;
    st.gnorm = gnorm;
    return true;
}

}  // namespace ae
