// The reference's C / Fortran ABI (AnsatzSynthInterface.cpp:18-629) over the GPU
// stateAnsatzManager: same argument checks, index conventions and return codes.
#include "../../include/AnsatzSynthInterface.h"
#include "manager.h"
#include "runfiles.h"

#include <cstdio>
#include <cstring>
#include <limits>
#include <sstream>

using ae::log_line;
using ae::stateAnsatzManager;
using ae::RunFiles;
using ae::loadRunFiles;
using ae::storeRunFiles;

static bool traceInterfaceCalls = false;

template <typename T>
static std::string list(const T *p, int n)
{
    std::ostringstream s;
    s.precision(17);
    for (int i = 0; i < n && p; ++i) s << (i ? ", " : "") << p[i];
    return s.str();
}

extern "C" {

void setTraceInterfaceCalls(int val) { traceInterfaceCalls = val != 0; }

void *init(void)
{
    try {
        auto *p = new stateAnsatzManager;
        if (traceInterfaceCalls) log_line("Constructed object");
        return p;
    } catch (...) {
        return nullptr;
    }
}

int cleanup(void *ctx)
{
    if (traceInterfaceCalls) log_line("cleanup called");
    if (ctx == nullptr) {
        log_line("(void**) ctx is nullptr, something has gone wrong. Potential Leak");
        return 1;
    }
    void **my = (void **)ctx;
    if (*my == nullptr) return 0;
    delete static_cast<stateAnsatzManager *>(*my);
    *my = nullptr;
    return 0;
}

int setExcitation(int nparams, const int *operators, const int *orderfile, void *ctx)
{
    return setExcitationScale(nparams, operators, orderfile, nullptr, ctx);
}

int setExcitationScale(int nparams, const int *operators, const int *orderfile, const double *scale, void *ctx)
{
    if (ctx == nullptr) { log_line("nullptr ctx passed"); return 1; }
    if (nparams < 1) { log_line("nparams < 1"); return 2; }
    if (!operators || !orderfile) { log_line("nullptr operators or orderfile passed"); return 2; }
    if (traceInterfaceCalls) {
        log_line("setExcitationScale called with: nParams " + std::to_string(nparams));
        log_line("operators " + list(operators, nparams * 4));
        log_line("orderfile " + list(orderfile, nparams));
        if (scale) log_line("scale " + list(scale, nparams));
    }
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<ae::Exc4> excs(nparams);
    for (int i = 0; i < nparams; ++i) {
        int v[4];
        for (int j = 0; j < 4; ++j) {
            v[j] = operators[nparams * j + i] - 1;  // Fortran order, 1-based
            if (v[j] > std::numeric_limits<int8_t>::max() || v[j] < -1) {
                log_line("Excitation out of bounds, max is 128 " + std::to_string(operators[nparams * j + i]));
                return 3;
            }
        }
        excs[i] = {(int8_t)v[0], (int8_t)v[1], (int8_t)v[2], (int8_t)v[3]};
    }
    if (!m->storeOperators(excs)) return 4;
    std::vector<std::pair<int, double>> dep;
    for (int i = 0; i < nparams; ++i) {
        if (orderfile[i] > nparams) { log_line("orderfile out of bounds " + std::to_string(orderfile[i])); return 5; }
        dep.push_back({orderfile[i] - 1, scale ? scale[i] : 1.0});
    }
    if (!m->storeParameterDependencies(dep)) return 6;
    return 0;
}

int setHamiltonian(int N, const int *iIndexes, const int *jIndexes, const double *coeffs, void *ctx)
{
    if (ctx == nullptr) { log_line("nullptr ctx passed"); return 1; }
    if (traceInterfaceCalls) {
        log_line("setHamiltonian called with: N " + std::to_string(N));
        log_line("iIndexes " + list(iIndexes, N));
        log_line("jIndexes " + list(jIndexes, N));
        log_line("coeffs " + list(coeffs, N));
    }
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    if (N < 1) { log_line("N < 1"); return 2; }
    if (!iIndexes || !jIndexes || !coeffs) { log_line("nullptr Hamiltonian arrays"); return 2; }
    std::vector<int> i(iIndexes, iIndexes + N), j(jIndexes, jIndexes + N);
    for (int &x : i) x--;
    for (int &x : j) x--;
    std::vector<double> c(coeffs, coeffs + N);
    if (!m->storeHamiltonian(std::move(i), std::move(j), std::move(c))) return 3;
    return 0;
}

int setInitialState(int numQubits, int N, const int *iIndexes, const double *coeffs, void *ctx)
{
    if (ctx == nullptr) { log_line("nullptr ctx passed"); return 1; }
    if (traceInterfaceCalls) {
        log_line("setInitialState called with: numQubits " + std::to_string(numQubits) + " N " + std::to_string(N));
        log_line("iIndexes " + list(iIndexes, N));
        log_line("coeffs " + list(coeffs, N));
    }
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    if (N < 1) { log_line("N < 1"); return 2; }
    if (numQubits < 1) { log_line("numQubits < 1"); return 2; }
    if (!iIndexes || !coeffs) { log_line("nullptr initial-state arrays"); return 2; }
    std::vector<int> i(iIndexes, iIndexes + N);
    for (int &x : i) x--;
    std::vector<double> c(coeffs, coeffs + N);
    if (!m->storeInitial(numQubits, i, c)) return 3;
    return 0;
}

int setInitialStateComplex(int numQubits, int N, const int *iIndexes, const std::complex<double> *coeffs, void *ctx)
{
    if (ctx == nullptr) { log_line("nullptr ctx passed"); return 1; }
    if (traceInterfaceCalls)
        log_line("setInitialStateComplex called with: numQubits " + std::to_string(numQubits) + " N " + std::to_string(N));
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    if (N < 1) { log_line("N < 1"); return 2; }
    if (numQubits < 1) { log_line("numQubits < 1"); return 2; }
    if (!iIndexes || !coeffs) { log_line("nullptr initial-state arrays"); return 2; }
    std::vector<int> i(iIndexes, iIndexes + N);
    for (int &x : i) x--;
    std::vector<std::complex<double>> c(coeffs, coeffs + N);
    if (!m->storeInitial(numQubits, i, c)) return 3;
    return 0;
}

int getEnergy(int NAngles, const double *angles, double *energy, void *ctx)
{
    if (ctx == nullptr) { log_line("nullptr ctx passed"); return 1; }
    if (angles == nullptr) { log_line("nullptr angles passed"); return 2; }
    if (NAngles < 1) { log_line("NAngles < 1"); return 3; }
    if (energy == nullptr) { log_line("nullptr energy passed"); return 3; }
    if (traceInterfaceCalls) log_line("getEnergy called with: NAngles " + std::to_string(NAngles) + " angles " + list(angles, NAngles));
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    if (!m->getExpectationValue(std::vector<double>(angles, angles + NAngles), *energy)) return 3;
    return 0;
}

int getFinalState(int NAngles, const double *angles, int NBasisVectors, double *finalState, void *ctx)
{
    if (ctx == nullptr) { log_line("nullptr ctx passed"); return 1; }
    if (angles == nullptr) { log_line("nullptr angles passed"); return 2; }
    if (finalState == nullptr) { log_line("nullptr finalState passed"); return 3; }
    if (NBasisVectors < 1) { log_line("NBasisVectors < 1"); return 4; }
    if (NAngles < 1) { log_line("NAngles < 1"); return 5; }
    if (traceInterfaceCalls) log_line("getFinalState called with: NAngles " + std::to_string(NAngles) + " NBasisVectors " + std::to_string(NBasisVectors));
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<double> s;
    if (!m->getFinalState(std::vector<double>(angles, angles + NAngles), s)) return 6;
    if (s.size() != (size_t)NBasisVectors) {
        log_line("Final state does not have the write number allocated, NBasisVectors should be " + std::to_string(s.size()));
        return 7;
    }
    memcpy(finalState, s.data(), s.size() * sizeof(double));
    return 0;
}

int getFinalStateComplex(int NAngles, const double *angles, int NBasisVectors, std::complex<double> *finalState, void *ctx)
{
    if (ctx == nullptr) { log_line("nullptr ctx passed"); return 1; }
    if (angles == nullptr) { log_line("nullptr angles passed"); return 2; }
    if (finalState == nullptr) { log_line("nullptr finalState passed"); return 3; }
    if (NBasisVectors < 1) { log_line("NBasisVectors < 1"); return 4; }
    if (NAngles < 1) { log_line("NAngles < 1"); return 5; }
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<std::complex<double>> s;
    if (!m->getFinalState(std::vector<double>(angles, angles + NAngles), s)) return 6;
    if (s.size() != (size_t)NBasisVectors) {
        log_line("Final state does not have the right number allocated, NBasisVectors should be " + std::to_string(s.size()));
        return 7;
    }
    memcpy((void *)finalState, s.data(), s.size() * sizeof(std::complex<double>));
    return 0;
}

int getGradient_COMP(int NAngles, const double *angles, double *gradient, void *ctx)
{
    if (ctx == nullptr) { log_line("nullptr ctx passed"); return 1; }
    if (angles == nullptr) { log_line("nullptr angles passed"); return 2; }
    if (gradient == nullptr) { log_line("nullptr gradient passed"); return 3; }
    if (NAngles < 1) { log_line("NAngles < 1"); return 4; }
    if (traceInterfaceCalls) log_line("getGradient_COMP called with: NAngles " + std::to_string(NAngles) + " angles " + list(angles, NAngles));
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<double> g;
    if (!m->getGradientComp(std::vector<double>(angles, angles + NAngles), g)) return 5;
    if ((size_t)NAngles != g.size()) {
        log_line("Gradient is the wrong size, This is a Bug on the implementation side");
        return -6;
    }
    memcpy(gradient, g.data(), g.size() * sizeof(double));
    return 0;
}

int getHessian_COMP(int NAngles, const double *angles, double *hessian, void *ctx)
{
    if (ctx == nullptr) { log_line("nullptr ctx passed"); return 1; }
    if (angles == nullptr) { log_line("nullptr angles passed"); return 2; }
    if (hessian == nullptr) { log_line("nullptr hessian passed"); return 3; }
    if (NAngles < 1) { log_line("NAngles < 1"); return 4; }
    if (traceInterfaceCalls) log_line("getHessian_COMP called with: NAngles " + std::to_string(NAngles) + " angles " + list(angles, NAngles));
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<double> H;
    if (!m->getHessianComp(std::vector<double>(angles, angles + NAngles), H)) return 5;
    const int P = m->numberOfParameters();
    if (NAngles != P || H.size() != (size_t)P * P) {
        log_line("Hessian has wront dimensions, This is a bug on the implementation side");
        return -6;
    }
    for (int i = 0; i < P; ++i)
        for (int j = 0; j < P; ++j) hessian[NAngles * j + i] = H[(size_t)i * P + j];
    return 0;
}

int setRunPath(const char *path, void *ctx)
{
    if (ctx == nullptr) return 1;
    if (!path) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    return m->storeRunPath(path) ? 0 : 3;
}

int setIntegrals(int norb, const double *h1, const double *g2, int mode, void *ctx)
{
    if (ctx == nullptr) return 1;
    if (norb < 1 || norb > 15 || !h1 || !g2 || mode < 0 || mode > 2) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<double> a(h1, h1 + (size_t)norb * norb), b(g2, g2 + (size_t)norb * norb * norb * norb);
    return m->storeIntegrals(norb, a, b, mode) ? 0 : 3;
}

int setNuclearEnergy(double e, void *ctx)
{
    if (ctx == nullptr) return 1;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    return m->storeNuclearEnergy(e) ? 0 : 3;
}

int optimise(int NAngles, double *angles, double *energy, void *ctx)
{
    if (ctx == nullptr) return 1;
    if (!angles || NAngles < 1) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    if (!m->setAngles(std::vector<double>(angles, angles + NAngles))) return 3;
    if (!m->optimise()) return 3;
    std::vector<double> x = m->getAngles();
    if ((int)x.size() != NAngles && NAngles != m->numberOfOperators()) return 3;
    if (NAngles == m->numberOfParameters())
        memcpy(angles, x.data(), x.size() * sizeof(double));
    if (energy && !m->getExpectationValue(*energy)) return 3;
    return 0;
}

static bool angle_rows(int npaths, int nangles, const double *angles, std::vector<std::vector<double>> &rows)
{
    if (npaths < 1 || nangles < 1 || !angles) return false;
    rows.clear();
    for (int k = 0; k < npaths; ++k) rows.emplace_back(angles + (size_t)k * nangles, angles + (size_t)(k + 1) * nangles);
    return true;
}

int getProperties(int npaths, int nangles, const double *angles, int flags, double *table, void *ctx)
{
    if (ctx == nullptr) return 1;
    std::vector<std::vector<double>> rows;
    if (!table || !angle_rows(npaths, nangles, angles, rows)) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<double> t;
    if (!m->getProperties(rows, flags, t)) return 3;
    std::copy(t.begin(), t.end(), table);
    return 0;
}

int iterativeOptimise(int NAngles, double *angles, double *energy, void *ctx)
{
    if (ctx == nullptr) return 1;
    if (!angles || NAngles < 1) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    if (!m->setAngles(std::vector<double>(angles, angles + NAngles))) return 3;
    if (!m->iterativeOptimise()) return 3;
    std::vector<double> x = m->getAngles();
    if (NAngles == m->numberOfParameters()) memcpy(angles, x.data(), x.size() * sizeof(double));
    if (energy && !m->getExpectationValue(*energy)) return 3;
    return 0;
}

int generatePathsForSubspace(int numberOfPaths, double *eigenvalues, int *nullRank, double *energies, void *ctx)
{
    if (ctx == nullptr) return 1;
    if (numberOfPaths < 1) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<double> w, E;
    int nr = 0;
    if (!m->generatePathsForSubspace((size_t)numberOfPaths, &w, &nr, nullptr, &E)) return 3;
    if (eigenvalues) std::copy(w.begin(), w.end(), eigenvalues);
    if (energies) std::copy(E.begin(), E.end(), energies);
    if (nullRank) *nullRank = nr;
    return 0;
}

int getGradient(int NAngles, const double *angles, double *gradient, void *ctx)
{
    if (ctx == nullptr) return 1;
    if (NAngles < 1 || !angles || !gradient) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<double> g;
    if (!m->getGradient(std::vector<double>(angles, angles + NAngles), g)) return 3;
    std::copy(g.begin(), g.end(), gradient);
    return 0;
}

int getHessian(int NAngles, const double *angles, double *hessian, void *ctx)
{
    if (ctx == nullptr) return 1;
    if (NAngles < 1 || !angles || !hessian) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<double> H;
    if (!m->getHessian(std::vector<double>(angles, angles + NAngles), H)) return 3;
    std::copy(H.begin(), H.end(), hessian);  // symmetric: row- and column-major agree
    return 0;
}

int getExpectationValues(int nrows, int nangles, const double *angles, double *energies, void *ctx)
{
    if (ctx == nullptr) return 1;
    if (nrows < 1 || nangles < 1 || !angles || !energies) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<double> E;
    if (!m->getExpectationValues(std::vector<double>(angles, angles + (size_t)nrows * nangles), nrows, nangles, E))
        return 3;
    std::copy(E.begin(), E.end(), energies);
    return 0;
}

int writeProperties(int npaths, int nangles, const double *angles, int flags, const char *runPath, void *ctx)
{
    if (ctx == nullptr) return 1;
    std::vector<std::vector<double>> rows;
    if (!angle_rows(npaths, nangles, angles, rows)) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    return m->writeProperties(rows, !(flags & AEGPU_PROP_HESSIAN), (flags & AEGPU_PROP_OVERLAP) != 0,
                              (flags & AEGPU_PROP_HF_PATH) != 0, runPath ? runPath : "")
               ? 0
               : 3;
}

int setNumberOfOverlapsToCompute(int n, void *ctx)
{
    if (ctx == nullptr) return 1;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    if (n <= 0) return 2;
    m->setNumberOfOverlapsToCompute(n);
    return 0;
}

int getLowestEigenvalue(double *eigenvalue, double *residual, void *ctx)
{
    if (ctx == nullptr) return 1;
    if (!eigenvalue) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    double res = 0;
    if (!m->getLowestEigenvalue(*eigenvalue, res)) return 3;
    if (residual) *residual = res;
    return 0;
}

int getSubspaceEigenvalues(int npaths, int nangles, const double *angles, double *eigenvalues, int *nullRank, void *ctx)
{
    if (ctx == nullptr) return 1;
    std::vector<std::vector<double>> rows;
    if (!eigenvalues || !angle_rows(npaths, nangles, angles, rows)) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    std::vector<double> w;
    int nr = 0;
    if (!m->getSubspaceEigenvalues(rows, w, nr)) return 3;
    std::copy(w.begin(), w.end(), eigenvalues);
    if (nullRank) *nullRank = nr;
    return 0;
}

int setRunFiles(const char *prefix, void *ctx)
{
    if (ctx == nullptr) return 1;
    if (!prefix || !*prefix) return 2;
    auto *m = static_cast<stateAnsatzManager *>(ctx);
    std::lock_guard<std::mutex> lock(m->m_interfaceLock);
    RunFiles rf;
    std::string err;
    if (!loadRunFiles(prefix, false, rf, err) || !storeRunFiles(*m, rf, prefix, err)) {
        log_line("setRunFiles: " + err);
        return 3;
    }
    return 0;
}

}  // extern "C"
