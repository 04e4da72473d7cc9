// Optimisers over the engine ABI (host-side control only; every energy and gradient
// comes from the GPU engine).
//
// * aegpu_optimise_newton: the reference's optimiser (TUPSQuantities::OptimiseTups,
//   tupsquantities.cpp:1940-2011) for one instance, with the engine's analytic
//   Hessian (newton.cpp restates it).  This is the plain one-instance-at-a-time path.
// * aegpu_optimise_batch: all nb instances of a batched engine optimised in lockstep
//   by BFGS (inverse-Hessian update, Nocedal & Wright, Numerical Optimization, 2nd
//   ed., Alg. 6.1 with the initial scaling of eq. 6.20) with a backtracking Armijo
//   line search.  Every round is ONE batched energy + gradient evaluation: each
//   instance contributes its current trial point, so line-search points of some
//   instances and new iterates of others share the launch, and converged instances
//   are masked out of it (aegpu_set_active).  No counterpart in the reference, which
//   optimises one angle vector at a time.
#include "../../include/aegpu.h"
#include "diis.h"
#include "newton.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

namespace {

struct BfgsInstance {
    enum Phase { kFirst, kTrial, kDone } phase = kFirst;
    std::vector<double> x, g, xt, p, Hinv;
    double f = 0, alpha = 1, gp = 0;
    bool scaled = false;
    int iters = 0, resets = 0;
};

double dot(const double *a, const double *b, int n)
{
    double s = 0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

void set_identity(std::vector<double> &H, int P, double d)
{
    H.assign((size_t)P * P, 0.0);
    for (int i = 0; i < P; ++i) H[(size_t)i * P + i] = d;
}

// p = -Hinv g; falls back to steepest descent when that is not a descent direction.
void direction(BfgsInstance &s, int P)
{
    s.p.assign(P, 0.0);
    for (int i = 0; i < P; ++i) s.p[i] = -dot(&s.Hinv[(size_t)i * P], s.g.data(), P);
    s.gp = dot(s.g.data(), s.p.data(), P);
    if (!(s.gp < 0)) {
        set_identity(s.Hinv, P, 1.0);
        s.scaled = false;
        s.resets++;
        for (int i = 0; i < P; ++i) s.p[i] = -s.g[i];
        s.gp = dot(s.g.data(), s.p.data(), P);
    }
}

void start_trial(BfgsInstance &s, int P, double max_step)
{
    const double pn = std::sqrt(dot(s.p.data(), s.p.data(), P));
    s.alpha = pn > max_step ? max_step / pn : 1.0;
    s.xt.resize(P);
    for (int i = 0; i < P; ++i) s.xt[i] = s.x[i] + s.alpha * s.p[i];
    s.phase = BfgsInstance::kTrial;
}

}  // namespace

extern "C" {

int aegpu_optimise_batch(aegpu_engine *e, int nparams, const int *param, const double *scale, double *x, double gtol,
                         int max_rounds, double max_step, double *hinv, double *energy, double *gnorm, int *iters,
                         int64_t *rounds)
{
    if (!e || nparams < 1 || !param || !scale || !x || !(gtol > 0) || max_rounds < 1) return AEGPU_ERR_ARG;
    const int nb = aegpu_batch_size(e);
    int64_t info[8];
    int rc = aegpu_problem_info(e, info);
    if (rc) return rc;
    const int nops = (int)info[1], P = nparams;
    for (int o = 0; o < nops; ++o)
        if (param[o] < 0 || param[o] >= P) return AEGPU_ERR_ARG;
    if (!(max_step > 0)) max_step = 1.0;
    std::vector<BfgsInstance> st(nb);
    for (int b = 0; b < nb; ++b) {
        st[b].x.assign(x + (size_t)b * P, x + (size_t)(b + 1) * P);
        st[b].xt = st[b].x;
        if (hinv) {
            // caller's initial inverse Hessian (e.g. from a nearby instance): no rescaling
            st[b].Hinv.assign(hinv + (size_t)b * P * P, hinv + (size_t)(b + 1) * P * P);
            st[b].scaled = true;
        } else {
            set_identity(st[b].Hinv, P, 1.0);
        }
    }
    std::vector<double> ang((size_t)nb * nops), E(nb), gops((size_t)nb * nops), gc(P), s(P), y(P), Hy(P);
    std::vector<int> active(nb, 1), last(nb, 1);
    int64_t round = 0;
    for (; round < max_rounds; ++round) {
        bool any = false;
        for (int b = 0; b < nb; ++b) {
            active[b] = st[b].phase != BfgsInstance::kDone;
            any = any || active[b];
        }
        if (!any) break;
        // converged instances drop out of the batched launches
        if (active != last) {
            if ((rc = aegpu_set_active(e, active.data()))) return rc;
            last = active;
        }
        // theta_op = scale[op] * x[param[op]] for every instance's trial point
        for (int b = 0; b < nb; ++b)
            for (int o = 0; o < nops; ++o) ang[(size_t)b * nops + o] = scale[o] * st[b].xt[param[o]];
        if ((rc = aegpu_io_put_angles(e, ang.data(), nullptr)) || (rc = aegpu_launch_io(e, nullptr)) ||
            (rc = aegpu_io_get_results(e, E.data(), gops.data(), nullptr)))
            return rc;
        for (int b = 0; b < nb; ++b) {
            BfgsInstance &I = st[b];
            if (I.phase == BfgsInstance::kDone) continue;
            std::fill(gc.begin(), gc.end(), 0.0);
            for (int o = 0; o < nops; ++o) gc[param[o]] += scale[o] * gops[(size_t)b * nops + o];
            const double ft = E[b];
            if (I.phase == BfgsInstance::kFirst) {
                I.f = ft;
                I.g = gc;
                if (std::sqrt(dot(gc.data(), gc.data(), P)) < gtol) {
                    I.phase = BfgsInstance::kDone;
                    continue;
                }
                direction(I, P);
                start_trial(I, P, max_step);
                continue;
            }
            // Armijo sufficient decrease; below the evaluation's rounding level the
            // energy cannot resolve the decrease, so a smaller gradient accepts too
            const double gnt = std::sqrt(dot(gc.data(), gc.data(), P)), gn = std::sqrt(dot(I.g.data(), I.g.data(), P));
            const double noise = 1e-13 * std::max(1.0, std::abs(I.f));
            const bool armijo = ft <= I.f + 1e-4 * I.alpha * I.gp;
            const bool flat = std::abs(ft - I.f) <= noise && gnt < gn;
            if (armijo || flat) {
                for (int i = 0; i < P; ++i) {
                    s[i] = I.xt[i] - I.x[i];
                    y[i] = gc[i] - I.g[i];
                }
                const double sy = dot(s.data(), y.data(), P);
                const double ss = dot(s.data(), s.data(), P), yy = dot(y.data(), y.data(), P);
                if (sy > 1e-12 * std::sqrt(ss * yy) && sy > 0) {
                    if (!I.scaled) {
                        set_identity(I.Hinv, P, sy / yy);  // eq. 6.20
                        I.scaled = true;
                    }
                    // Hinv += rho((1 + rho y'Hy) s s' - Hy s' - s Hy')
                    const double rho = 1.0 / sy;
                    for (int i = 0; i < P; ++i) Hy[i] = dot(&I.Hinv[(size_t)i * P], y.data(), P);
                    const double c = rho * (1.0 + rho * dot(y.data(), Hy.data(), P));
                    for (int i = 0; i < P; ++i)
                        for (int j = 0; j < P; ++j)
                            I.Hinv[(size_t)i * P + j] += c * s[i] * s[j] - rho * (Hy[i] * s[j] + s[i] * Hy[j]);
                }
                I.x = I.xt;
                I.f = ft;
                I.g = gc;
                I.iters++;
                if (gnt < gtol) {
                    I.phase = BfgsInstance::kDone;
                    continue;
                }
                direction(I, P);
                start_trial(I, P, max_step);
            } else {
                // backtrack: minimiser of the quadratic through f, g'p and f(alpha),
                // kept within [0.1, 0.5] alpha
                const double denom = 2.0 * (ft - I.f - I.alpha * I.gp);
                double a = denom > 0 ? -I.gp * I.alpha * I.alpha / denom : 0.5 * I.alpha;
                a = std::min(0.5 * I.alpha, std::max(0.1 * I.alpha, a));
                const double pn = std::sqrt(dot(I.p.data(), I.p.data(), P));
                if (a * pn < 1e-14) {
                    // the line search failed: restart from steepest descent
                    set_identity(I.Hinv, P, 1.0);
                    I.scaled = false;
                    I.resets++;
                    if (I.resets > 50) {
                        I.phase = BfgsInstance::kDone;
                        I.xt = I.x;
                        continue;
                    }
                    direction(I, P);
                    start_trial(I, P, max_step);
                    continue;
                }
                I.alpha = a;
                for (int i = 0; i < P; ++i) I.xt[i] = I.x[i] + a * I.p[i];
            }
        }
    }
    if ((rc = aegpu_set_active(e, nullptr))) return rc;
    for (int b = 0; b < nb; ++b) {
        std::copy(st[b].x.begin(), st[b].x.end(), x + (size_t)b * P);
        if (energy) energy[b] = st[b].f;
        if (gnorm) gnorm[b] = st[b].g.empty() ? -1.0 : std::sqrt(dot(st[b].g.data(), st[b].g.data(), P));
        if (iters) iters[b] = st[b].iters;
        if (hinv) std::copy(st[b].Hinv.begin(), st[b].Hinv.end(), hinv + (size_t)b * P * P);
    }
    if (rounds) *rounds = round;
    return AEGPU_OK;
}

int aegpu_optimise_newton(aegpu_engine *e, int nparams, const int *param, const double *scale, double *x, double gtol,
                          double *energy, double *gnorm, int64_t *hessian_evals, int64_t *energy_evals)
{
    if (!e || nparams < 1 || !param || !scale || !x || !(gtol > 0)) return AEGPU_ERR_ARG;
    if (aegpu_batch_size(e) != 1) return AEGPU_ERR_UNSUPPORTED;
    int64_t info[8];
    int rc = aegpu_problem_info(e, info);
    if (rc) return rc;
    const int nops = (int)info[1], P = nparams;
    for (int o = 0; o < nops; ++o)
        if (param[o] < 0 || param[o] >= P) return AEGPU_ERR_ARG;
    ae::NewtonProblem p;
    p.nparams = P;
    p.param.assign(param, param + nops);
    p.scale.assign(scale, scale + nops);
    p.gtol = gtol;
    int err = AEGPU_OK;
    p.energy_grad = [&](const std::vector<double> &th, double &E, std::vector<double> &g) {
        std::vector<double> gops(nops);
        if ((err = aegpu_gradient(e, th.data(), &E, gops.data()))) return false;
        g.assign(P, 0.0);
        for (int i = 0; i < nops; ++i) g[param[i]] += scale[i] * gops[i];
        return true;
    };
    p.hessian = [&](const std::vector<double> &th, double &E, std::vector<double> &g, std::vector<double> &H) {
        g.assign(P, 0.0);
        H.assign((size_t)P * P, 0.0);
        return (err = aegpu_hessian(e, th.data(), param, scale, P, &E, g.data(), H.data())) == AEGPU_OK;
    };
    std::vector<double> th(nops);
    for (int o = 0; o < nops; ++o) th[o] = scale[o] * x[param[o]];
    ae::NewtonStats st;
    if (!ae::optimise_newton(p, th, st, false)) return err ? err : AEGPU_ERR_CUDA;
    // back to the compressed parameters (each parameter's first operator)
    std::vector<bool> seen(P, false);
    for (int o = 0; o < nops; ++o)
        if (!seen[param[o]] && scale[o] != 0) {
            x[param[o]] = th[o] / scale[o];
            seen[param[o]] = true;
        }
    if (energy) *energy = st.energy;
    if (gnorm) *gnorm = st.gnorm;
    if (hessian_evals) *hessian_evals = st.hessian_evals;
    if (energy_evals) *energy_evals = st.energy_evals;
    return AEGPU_OK;
}

int aegpu_optimise_projected(aegpu_engine *e, int nparams, const int *param, const double *scale, double *x,
                             double gtol, int max_outer, double *energy, double *gnorm, int64_t *hessian_evals,
                             int64_t *energy_evals, int *outer_iters)
{
    return aegpu_optimise_projected_diis(e, nparams, param, scale, x, gtol, max_outer, 0, 1, energy, gnorm,
                                         hessian_evals, energy_evals, outer_iters);
}

int aegpu_optimise_projected_diis(aegpu_engine *e, int nparams, const int *param, const double *scale, double *x,
                                  double gtol, int max_outer, int diis_size, int ediis, double *energy, double *gnorm,
                                  int64_t *hessian_evals, int64_t *energy_evals, int *outer_iters)
{
    if (!e || nparams < 1 || !param || !scale || !x || !(gtol > 0) || max_outer < 1 || diis_size < 0)
        return AEGPU_ERR_ARG;
    if (aegpu_batch_size(e) != 1) return AEGPU_ERR_UNSUPPORTED;
    int64_t info[8];
    int rc = aegpu_problem_info(e, info);
    if (rc) return rc;
    const int nops = (int)info[1], P = nparams;
    const size_t n = (size_t)aegpu_dim(e) * (size_t)aegpu_amplitude_width(e);
    for (int o = 0; o < nops; ++o)
        if (param[o] < 0 || param[o] >= P) return AEGPU_ERR_ARG;
    ae::ProjectedProblem p;
    p.nparams = P;
    p.param.assign(param, param + nops);
    p.scale.assign(scale, scale + nops);
    p.gtol = gtol;
    p.max_outer = max_outer;
    p.diis_size = diis_size;
    p.ediis = ediis != 0;
    int err = AEGPU_OK;
    p.bra = [&](const std::vector<double> &th, std::vector<double> &psiH, std::vector<double> &psi) {
        psiH.assign(n, 0.0);
        psi.assign(n, 0.0);
        return (err = aegpu_evolve(e, th.data(), psi.data())) == AEGPU_OK &&
               (err = aegpu_apply_h(e, psi.data(), psiH.data())) == AEGPU_OK;
    };
    p.proj_grad = [&](const std::vector<double> &th, const std::vector<double> &psiH, double &ov,
                      std::vector<double> &g) {
        std::vector<double> gops(nops);
        if ((err = aegpu_gradient_proj(e, th.data(), psiH.data(), &ov, gops.data()))) return false;
        g.assign(P, 0.0);
        for (int i = 0; i < nops; ++i) g[param[i]] += scale[i] * gops[i];
        return true;
    };
    p.proj_hess = [&](const std::vector<double> &th, const std::vector<double> &psiH, double &ov,
                      std::vector<double> &g, std::vector<double> &H) {
        g.assign(P, 0.0);
        H.assign((size_t)P * P, 0.0);
        return (err = aegpu_hessian_proj(e, th.data(), param, scale, P, psiH.data(), &ov, g.data(), H.data())) ==
               AEGPU_OK;
    };
    std::vector<double> th(nops);
    for (int o = 0; o < nops; ++o) th[o] = scale[o] * x[param[o]];
    ae::NewtonStats st;
    int outer = 0;
    if (!ae::optimise_projected(p, th, st, outer)) return err ? err : AEGPU_ERR_CUDA;
    std::vector<bool> seen(P, false);
    for (int o = 0; o < nops; ++o)
        if (!seen[param[o]] && scale[o] != 0) {
            x[param[o]] = th[o] / scale[o];
            seen[param[o]] = true;
        }
    if (energy) *energy = st.energy;
    if (gnorm) *gnorm = st.gnorm;
    if (hessian_evals) *hessian_evals = st.hessian_evals;
    if (energy_evals) *energy_evals = st.energy_evals;
    if (outer_iters) *outer_iters = outer;
    return AEGPU_OK;
}

int aegpu_host_diis_coefficients(int n, const double *B, int ediis, double *c)
{
    if (n < 1 || !B || !c) return AEGPU_ERR_ARG;
    std::vector<double> b(B, B + (size_t)n * n), cv;
    ae::diis_coefficients(n, b, ediis != 0, cv);
    std::copy(cv.begin(), cv.end(), c);
    return AEGPU_OK;
}

}  // extern "C"
