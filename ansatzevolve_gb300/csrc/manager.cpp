// stateAnsatzManager (drop-in for AnsatzManager.cpp:12-829).  Host-side setup and
// bookkeeping only; every statevector operation is an aegpu_* call on the GPU.
#include "manager.h"

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <numeric>
#include <unistd.h>

namespace ae {

void log_line(const std::string &s)
{
    fprintf(stderr, "%s\n", s.c_str());
}

static int popc(uint32_t x) { return __builtin_popcount(x); }

stateAnsatzManager::stateAnsatzManager()
{
    char buf[4096];
    if (getcwd(buf, sizeof(buf))) m_runPath = buf;
}

stateAnsatzManager::~stateAnsatzManager()
{
    if (m_engine) aegpu_destroy(m_engine);
}

bool stateAnsatzManager::storeOperators(const std::vector<Exc4> &excs)
{
    if (m_isConstructed) { log_line("Already constructed, setup cant be modified now"); return false; }
    if (excs.empty()) { log_line("Excitations given has zero size"); return false; }
    m_excitations = excs;
    return true;
}

bool stateAnsatzManager::storeInitial(int nq, const std::vector<int> &idx, const std::vector<double> &c)
{
    std::vector<std::complex<double>> cc(c.begin(), c.end());
    bool ok = storeInitial(nq, idx, cc);
    if (ok) m_initComplex = false;
    return ok;
}

// AnsatzManager.cpp:271-374: records the state and detects particle-number and Sz symmetry.
bool stateAnsatzManager::storeInitial(int nq, const std::vector<int> &idx, const std::vector<std::complex<double>> &c)
{
    bool ok = true;
    if (m_isConstructed) { log_line("Already constructed, setup cant be modified now"); ok = false; }
    if (nq < 1) { log_line("Number of qubits < 1"); ok = false; }
    if (idx.empty() || c.empty()) { log_line("Initial state has no elements"); ok = false; }
    if (idx.size() != c.size()) { log_line("Initial state indexes and coeffs are a different size"); ok = false; }
    if (nq > 30) { log_line("Number of qubits > 30 is not supported"); ok = false; }
    for (int i : idx)
        if (ok && (i < 0 || (int64_t)i >= (1ll << nq))) { log_line("Initial state index out of range"); ok = false; }
    if (!ok) return false;
    m_initIdx = idx;
    m_initCoeff = c;
    m_initComplex = true;
    double mag = 0;
    std::vector<std::pair<int, std::complex<double>>> dense;
    for (size_t k = 0; k < idx.size(); ++k) mag += std::norm(c[k]);
    mag = std::sqrt(mag);
    if (std::abs(mag - 1) > 1e-14) log_line("Warning: Initial vector is not normalised, the error is " + std::to_string(std::abs(mag - 1)));
    m_numberOfQubits = nq;
    int np = -1, su = -1, sd = -1;
    bool sameN = true, sz = nq % 2 == 0;
    for (size_t k = 0; k < idx.size(); ++k) {
        if (c[k] == std::complex<double>(0, 0)) continue;
        int n = popc((uint32_t)idx[k]);
        if (np == -1) np = n;
        if (n != np) { sameN = false; break; }
        int u = popc((uint32_t)idx[k] >> (nq / 2)), d = popc((uint32_t)idx[k] & ((1u << (nq / 2)) - 1u));
        if (su == -1) su = u;
        if (sd == -1) sd = d;
        if (u != su || d != sd) sz = false;
    }
    if (np == -1) log_line("Warning: Could not determine particle number");
    else if (!sameN) log_line("Warning: not all the same particle number");
    m_numberOfParticles = m_spinUp = m_spinDown = -1;
    m_InitialSZSym = m_particleSym = false;
    if (sameN && np != -1) {
        m_numberOfParticles = np;
        m_particleSym = true;
        if (sz && su != -1 && sd != -1) {
            m_InitialSZSym = true;
            m_spinUp = su;
            m_spinDown = sd;
        }
    }
    return true;
}

bool stateAnsatzManager::storeHamiltonian(std::vector<int> &&i, std::vector<int> &&j, std::vector<double> &&c)
{
    bool ok = true;
    if (m_isConstructed) { log_line("Already constructed, setup cant be modified now"); ok = false; }
    if (i.empty() || j.empty() || c.empty()) { log_line("Hamiltonian Matrix has no elements"); ok = false; }
    if (i.size() != j.size() || i.size() != c.size()) { log_line("Hamiltonian Matrix indexes and coeffs are a different size"); ok = false; }
    m_iIndexes = std::move(i);
    m_jIndexes = std::move(j);
    m_coeffs = std::move(c);
    return ok;
}

bool stateAnsatzManager::storeNuclearEnergy(double e)
{
    if (m_isConstructed) { log_line("Already constructed, setup cant be modified now"); return false; }
    m_nuclearEnergy = e;
    return true;
}

// AnsatzManager.cpp:411-445
bool stateAnsatzManager::storeParameterDependencies(const std::vector<std::pair<int, double>> &pd)
{
    if (m_isConstructed) { log_line("Already constructed, setup cant be modified now"); return false; }
    if (pd.empty()) { log_line("Parameter Dependencies, (order file) has zero size"); return false; }
    m_parameterDependency = pd;
    m_numberOfUniqueParameters = -1;
    for (auto &p : pd) {
        if (p.first < 0) { log_line("Order cannot be negative"); m_parameterDependency.clear(); return false; }
        m_numberOfUniqueParameters = std::max(p.first + 1, m_numberOfUniqueParameters);
    }
    if ((size_t)m_numberOfUniqueParameters > pd.size()) {
        m_numberOfUniqueParameters = -1;
        m_parameterDependency.clear();
        return false;
    }
    return true;
}

bool stateAnsatzManager::storeRunPath(const std::string &p)
{
    if (m_isConstructed) { log_line("Already constructed, setup cant be modified now"); return false; }
    if (p.empty()) { log_line("Run path has zero size"); return false; }
    m_runPath = p;
    return true;
}

bool stateAnsatzManager::storeIntegrals(int n, const std::vector<double> &h1, const std::vector<double> &g2, int mode)
{
    if (m_isConstructed) { log_line("Already constructed, setup cant be modified now"); return false; }
    if (n < 1 || h1.size() != (size_t)n * n || g2.size() != (size_t)n * n * n * n) {
        log_line("Integral arrays have the wrong size");
        return false;
    }
    m_intsN = n;
    m_h1 = h1;
    m_g2 = g2;
    m_intsMode = mode;
    return true;
}

// AnsatzManager.cpp:202-237
void stateAnsatzManager::setOperatorSymmetry()
{
    m_OperatorSZSym = !m_excitations.empty();
    const int nq = m_numberOfQubits;
    uint32_t dn = (1u << (nq / 2)) - 1u, up = ((nq >= 32 ? 0u : (1u << nq)) - 1u) ^ dn;
    for (const auto &e : m_excitations) {
        uint32_t cr, de;
        if (e.third < 0 && e.fourth < 0) {
            cr = 1u << e.first;
            de = 1u << e.second;
        } else {
            cr = (1u << e.first) | (1u << e.second);
            de = (1u << e.third) | (1u << e.fourth);
        }
        m_OperatorSZSym = m_OperatorSZSym && popc(cr & up) == popc(de & up) && popc(cr & dn) == popc(de & dn);
    }
}

bool stateAnsatzManager::validateToRun()
{
    if (!m_isConstructed && !construct()) {
        log_line("Not yet Constructed, something is missing");
        return false;
    }
    return m_engine != nullptr;
}

static bool read_file(const std::string &path, std::vector<char> &out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    return true;
}

// AnsatzManager.cpp:51-153
bool stateAnsatzManager::construct()
{
    if (m_isConstructed) return true;
    bool ok = true;
    if (m_numberOfQubits == -1) { log_line("Number of Qubits is not set. Make sure the initial state has been provided and has elements"); ok = false; }
    if (m_initIdx.empty()) { log_line("Make sure the initial state has been provided"); ok = false; }
    if (m_excitations.empty()) { log_line("No excitations have been set"); ok = false; }
    if (m_parameterDependency.empty() || m_numberOfUniqueParameters == -1) { log_line("Parameter Dependencies, (order file) has zero size"); ok = false; }
    if (m_parameterDependency.size() != m_excitations.size()) { log_line("More operators than parameters dependencies given"); ok = false; }
    if (!ok) return false;
    for (const auto &e : m_excitations) {
        const int8_t v[4] = {e.first, e.second, e.third, e.fourth};
        bool single = v[0] >= 0 && v[1] >= 0 && v[2] < 0 && v[3] < 0, dbl = v[0] >= 0 && v[1] >= 0 && v[2] >= 0 && v[3] >= 0;
        if (!single && !dbl) { log_line("exc is neither single nor double excitation"); return false; }
        for (int k = 0; k < 4; ++k)
            if (v[k] >= m_numberOfQubits) { log_line("Excitation index exceeds the number of qubits"); return false; }
    }
    setOperatorSymmetry();
    int kind = AEGPU_BASIS_FULL;
    if (m_particleSym) kind = (m_InitialSZSym && m_OperatorSZSym) ? AEGPU_BASIS_SZ : AEGPU_BASIS_NUMBER;
    m_basisKind = kind;
    // complex amplitudes when the state is complex or a diagonal (phase) operator is present
    bool hasDiag = false;
    for (const auto &e : m_excitations) {
        if (e.third < 0) hasDiag |= e.first == e.second;
        else hasDiag |= (((1u << e.first) | (1u << e.second)) ^ ((1u << e.third) | (1u << e.fourth))) == 0;
    }
    bool cplxCoeff = false;
    for (auto &c : m_initCoeff) cplxCoeff |= c.imag() != 0;
    m_complex = hasDiag || cplxCoeff;

    m_param.resize(m_parameterDependency.size());
    m_scale.resize(m_parameterDependency.size());
    for (size_t i = 0; i < m_parameterDependency.size(); ++i) {
        m_param[i] = m_parameterDependency[i].first;
        m_scale[i] = m_parameterDependency[i].second;
    }
    if (aegpu_create(&m_engine) != AEGPU_OK) { log_line("Could not create the GPU engine (no CUDA device?)"); m_engine = nullptr; return false; }
    std::vector<int> ops;
    for (const auto &e : m_excitations) {
        ops.push_back(e.first); ops.push_back(e.second); ops.push_back(e.third); ops.push_back(e.fourth);
    }
    int rc = aegpu_set_problem(m_engine, m_numberOfQubits, kind, std::max(0, m_numberOfParticles), std::max(0, m_spinUp),
                               std::max(0, m_spinDown), m_complex ? 1 : 0, (int)m_excitations.size(), ops.data());
    if (rc) { log_line(std::string("GPU setup failed: ") + aegpu_last_error(m_engine)); aegpu_destroy(m_engine); m_engine = nullptr; return false; }
    // compressed initial state
    const int64_t D = aegpu_dim(m_engine);
    std::vector<uint32_t> states(D);
    aegpu_basis_states(m_engine, states.data());
    std::vector<double> start((size_t)D * (m_complex ? 2 : 1), 0.0);
    for (size_t k = 0; k < m_initIdx.size(); ++k) {
        auto it = std::lower_bound(states.begin(), states.end(), (uint32_t)m_initIdx[k]);
        if (it == states.end() || *it != (uint32_t)m_initIdx[k]) continue;
        size_t r = it - states.begin();
        if (m_complex) {
            start[2 * r] = m_initCoeff[k].real();
            start[2 * r + 1] = m_initCoeff[k].imag();
        } else {
            start[r] = m_initCoeff[k].real();
        }
    }
    aegpu_set_initial(m_engine, start.data());
    if (!setHamiltonian()) { aegpu_destroy(m_engine); m_engine = nullptr; return false; }
    m_angles.assign(m_excitations.size(), 0.0);
    m_isConstructed = true;
    m_haveEvolved = false;
    return evolveIfNeeded();
}

// Sector CSR (row = output) from (row i, column j) entries of the full 2^nq matrix:
// the reference stores H(i, j) and computes y = x H, so y_j = sum_i x_i H(i, j).
static void triplets_to_csr(const std::vector<uint32_t> &states, const std::vector<int> &ii, const std::vector<int> &jj,
                            const std::vector<double> &vv, std::vector<int64_t> &rowptr, std::vector<int32_t> &col,
                            std::vector<double> &val)
{
    const int64_t D = (int64_t)states.size();
    auto rank = [&](int s) -> int64_t {
        auto it = std::lower_bound(states.begin(), states.end(), (uint32_t)s);
        return (it != states.end() && *it == (uint32_t)s) ? it - states.begin() : -1;
    };
    struct T { int64_t row, col; double v; size_t order; };
    std::vector<T> t;
    t.reserve(vv.size());
    for (size_t k = 0; k < vv.size(); ++k) {
        if (ii[k] < 0 || jj[k] < 0) continue;
        int64_t ri = rank(ii[k]), rj = rank(jj[k]);
        if (ri < 0 || rj < 0) continue;
        t.push_back({rj, ri, vv[k], k});
    }
    std::sort(t.begin(), t.end(), [](const T &a, const T &b) {
        return a.row != b.row ? a.row < b.row : (a.col != b.col ? a.col < b.col : a.order < b.order);
    });
    rowptr.assign(D + 1, 0);
    col.clear();
    val.clear();
    for (size_t k = 0; k < t.size();) {
        size_t m = k;
        double s = 0;
        while (m < t.size() && t[m].row == t[k].row && t[m].col == t[k].col) s += t[m++].v;
        col.push_back((int32_t)t[k].col);
        val.push_back(s);
        rowptr[t[k].row + 1]++;
        k = m;
    }
    for (int64_t r = 0; r < D; ++r) rowptr[r + 1] += rowptr[r];
}

// Operator list of hamiltonianmatrix.cpp:402-554 and its CSR assembly (:556-601),
// for integral Hamiltonians outside the Sz sector (small systems; setup only).
static void integrals_to_csr(int nq, const std::vector<double> &h1, const std::vector<double> &g2,
                             const std::vector<uint32_t> &states, std::vector<int64_t> &rowptr, std::vector<int32_t> &col,
                             std::vector<double> &val)
{
    const int N = nq / 2;
    struct Op { uint32_t cr, de, mask; double v; };
    std::vector<Op> ops;
    auto G = [&](int i, int j, int k, int l) { return g2[(((size_t)i * N + l) * N + j) * N + k]; };
    for (int a = 0; a < nq; ++a)
        for (int b = a + 1; b < nq; ++b)
            for (int c = 0; c < nq; ++c)
                for (int d = c + 1; d < nq; ++d) {
                    int sa = a >= N, sb = b >= N, sc = c >= N, sd = d >= N;
                    double E = 0;
                    if (sa == sc && sb == sd) E += G(b % N, a % N, c % N, d % N);
                    if (sa == sd && sb == sc) E -= G(b % N, a % N, d % N, c % N);
                    if (std::abs(E) > 1e-13) {
                        uint32_t cr = (1u << a) | (1u << b), de = (1u << c) | (1u << d);
                        uint32_t m = ((1u << a) - 1u) ^ ((1u << b) - 1u) ^ ((1u << c) - 1u) ^ ((1u << d) - 1u);
                        ops.push_back({cr, de, m & ~(cr | de), E});
                    }
                }
    for (int a = 0; a < nq; ++a)
        for (int c = 0; c < nq; ++c) {
            double E = h1[(a % N) * N + (c % N)];
            if (std::abs(E) > 1e-13) {
                uint32_t m = ((1u << a) - 1u) ^ ((1u << c) - 1u);
                ops.push_back({1u << a, 1u << c, m & ~((1u << a) | (1u << c)), E});
            }
        }
    std::vector<int> ii, jj;
    std::vector<double> vv;
    for (uint32_t s : states)
        for (auto &o : ops) {
            uint32_t d = s ^ o.de;
            if (d & o.de) continue;
            if (d & o.cr) continue;
            uint32_t j = d | o.cr;
            bool neg = popc(s & o.mask) & 1;
            ii.push_back((int)s);
            jj.push_back((int)j);
            vv.push_back(neg ? -o.v : o.v);
        }
    triplets_to_csr(states, ii, jj, vv, rowptr, col, val);
}

// AnsatzManager.cpp:185-200 + HamiltonianMatrix constructors (hamiltonianmatrix.cpp:628-706)
bool stateAnsatzManager::setHamiltonian()
{
    const int64_t D = aegpu_dim(m_engine);
    std::vector<uint32_t> states(D);
    aegpu_basis_states(m_engine, states.data());
    std::vector<int64_t> rowptr;
    std::vector<int32_t> col;
    std::vector<double> val;
    int rc;
    if (!m_iIndexes.empty()) {
        triplets_to_csr(states, m_iIndexes, m_jIndexes, m_coeffs, rowptr, col, val);
        rc = aegpu_set_ham_csr(m_engine, (int64_t)col.size(), rowptr.data(), col.data(), val.data());
        m_coeffs.clear(); m_iIndexes.clear(); m_jIndexes.clear();
    } else {
        std::vector<double> h1 = m_h1, g2 = m_g2;
        const int N = m_numberOfQubits / 2;
        if (h1.empty()) {
            // <runPath>_Ham_Coeff.dat / _Ham_Index.dat first (s_loadMatrix), then integrals
            FILE *fc = fopen((m_runPath + "_Ham_Coeff.dat").c_str(), "r");
            FILE *fi = fopen((m_runPath + "_Ham_Index.dat").c_str(), "r");
            if (fc && fi) {
                std::vector<int> ii, jj;
                std::vector<double> vv;
                double re, im;
                unsigned a, b;
                while (fscanf(fc, "%lg, %lg \n", &re, &im) >= 1 && fscanf(fi, "%u %u\n", &a, &b) == 2) {
                    ii.push_back((int)a - 1);
                    jj.push_back((int)b - 1);
                    vv.push_back(re);
                    im = 0;
                }
                fclose(fc);
                fclose(fi);
                triplets_to_csr(states, ii, jj, vv, rowptr, col, val);
                rc = aegpu_set_ham_csr(m_engine, (int64_t)col.size(), rowptr.data(), col.data(), val.data());
                if (rc) log_line(std::string("Hamiltonian upload failed: ") + aegpu_last_error(m_engine));
                return rc == AEGPU_OK;
            }
            if (fc) fclose(fc);
            if (fi) fclose(fi);
            std::vector<char> b1, b2;
            if (!read_file(m_runPath + "_oneEInts.bin", b1) || !read_file(m_runPath + "_twoEInts.bin", b2)) {
                log_line("Could not construct Hamiltonian: no triplets, integrals or matrix files at " + m_runPath);
                return false;
            }
            if (b1.size() != (size_t)N * N * 8 || b2.size() != (size_t)N * N * N * N * 8) {
                log_line("Integral files have the wrong amount of data. Hamiltonians should be in Molecular orbital format");
                return false;
            }
            h1.resize((size_t)N * N);
            g2.resize((size_t)N * N * N * N);
            memcpy(h1.data(), b1.data(), b1.size());
            memcpy(g2.data(), b2.data(), b2.size());
        } else if (m_intsN != N) {
            log_line("Integrals do not match the number of qubits");
            return false;
        }
        if (m_basisKind == AEGPU_BASIS_SZ) {
            rc = aegpu_set_ham_integrals(m_engine, h1.data(), g2.data(), m_intsMode);
        } else {
            integrals_to_csr(m_numberOfQubits, h1, g2, states, rowptr, col, val);
            rc = aegpu_set_ham_csr(m_engine, (int64_t)col.size(), rowptr.data(), col.data(), val.data());
        }
    }
    if (rc) log_line(std::string("Hamiltonian setup failed: ") + aegpu_last_error(m_engine));
    return rc == AEGPU_OK;
}

bool stateAnsatzManager::evolveIfNeeded()
{
    if (m_haveEvolved) return true;
    int rc = aegpu_evolve(m_engine, m_angles.data(), nullptr);
    if (rc) { log_line(std::string("evolve failed: ") + aegpu_last_error(m_engine)); return false; }
    m_haveEvolved = true;
    return true;
}

bool stateAnsatzManager::decompress(const std::vector<double> &in, std::vector<double> &out)
{
    const size_t nops = m_excitations.size();
    if (in.size() == nops) { out = in; return true; }
    if ((int)in.size() == m_numberOfUniqueParameters) {
        out.resize(nops);
        for (size_t i = 0; i < nops; ++i) out[i] = m_scale[i] * in[m_param[i]];
        return true;
    }
    log_line("Incorrect number of angles given " + std::to_string(in.size()));
    return false;
}

// AnsatzManager.cpp:467-506
bool stateAnsatzManager::setAngles(std::vector<double> angles)
{
    if (!validateToRun()) return false;
    std::vector<double> a;
    if (!decompress(angles, a)) return false;
    if (a != m_angles) {
        m_angles = a;
        m_haveEvolved = false;
        return evolveIfNeeded();
    }
    return true;
}

std::vector<double> stateAnsatzManager::getAngles()
{
    if (!validateToRun()) return {};
    std::vector<double> x(m_numberOfUniqueParameters, 0.0);
    std::vector<bool> seen(m_numberOfUniqueParameters, false);
    for (size_t i = 0; i < m_angles.size(); ++i)
        if (!seen[m_param[i]] && m_scale[i] != 0) {
            x[m_param[i]] = m_angles[i] / m_scale[i];
            seen[m_param[i]] = true;
        }
    return x;
}

bool stateAnsatzManager::getExpectationValue(double &E)
{
    if (!validateToRun()) return false;
    int rc = aegpu_energy(m_engine, m_angles.data(), &E);
    if (rc) { log_line(std::string("energy failed: ") + aegpu_last_error(m_engine)); return false; }
    E += m_nuclearEnergy;
    return true;
}

bool stateAnsatzManager::getFinalState(std::vector<std::complex<double>> &out)
{
    if (!validateToRun()) return false;
    const int64_t D = aegpu_dim(m_engine);
    const int w = m_complex ? 2 : 1;
    std::vector<double> comp((size_t)D * w);
    if (aegpu_evolve(m_engine, m_angles.data(), comp.data())) {
        log_line(std::string("evolve failed: ") + aegpu_last_error(m_engine));
        return false;
    }
    std::vector<uint32_t> states(D);
    aegpu_basis_states(m_engine, states.data());
    out.assign((size_t)1 << m_numberOfQubits, {0.0, 0.0});
    for (int64_t z = 0; z < D; ++z) out[states[z]] = {comp[(size_t)z * w], w == 2 ? comp[(size_t)z * w + 1] : 0.0};
    return true;
}

bool stateAnsatzManager::getFinalState(std::vector<double> &out)
{
    std::vector<std::complex<double>> c;
    if (!getFinalState(c)) return false;
    if (m_complex) log_line("Warning casting complex values to real discards imaginary part, GetFinalState");
    out.resize(c.size());
    for (size_t i = 0; i < c.size(); ++i) out[i] = c[i].real();
    return true;
}

// AnsatzManager.cpp:581-606 -> FusedEvolve::evolveDerivative, then C * g
bool stateAnsatzManager::getGradientComp(std::vector<double> &g)
{
    if (!validateToRun()) return false;
    std::vector<double> gops(m_excitations.size());
    double E;
    int rc = aegpu_gradient(m_engine, m_angles.data(), &E, gops.data());
    if (rc) { log_line(std::string("gradient failed: ") + aegpu_last_error(m_engine)); return false; }
    g.assign(m_numberOfUniqueParameters, 0.0);
    for (size_t i = 0; i < gops.size(); ++i) g[m_param[i]] += m_scale[i] * gops[i];
    return true;
}

bool stateAnsatzManager::getHessianComp(std::vector<double> &H)
{
    if (!validateToRun()) return false;
    const int P = m_numberOfUniqueParameters;
    H.assign((size_t)P * P, 0.0);
    std::vector<double> g(P);
    double E;
    int rc = aegpu_hessian(m_engine, m_angles.data(), m_param.data(), m_scale.data(), P, &E, g.data(), H.data());
    if (rc) { log_line(std::string("hessian failed: ") + aegpu_last_error(m_engine)); return false; }
    return true;
}

// Per-operator derivatives (AnsatzManager.cpp:562-579, 608-624).  The reference's fused
// build cannot provide them and traps; here they are the gradient and Hessian with
// every operator its own parameter (identity compression).
bool stateAnsatzManager::getGradient(std::vector<double> &g)
{
    if (!validateToRun()) return false;
    g.assign(m_excitations.size(), 0.0);
    double E;
    int rc = aegpu_gradient(m_engine, m_angles.data(), &E, g.data());
    if (rc) { log_line(std::string("gradient failed: ") + aegpu_last_error(m_engine)); return false; }
    return true;
}

bool stateAnsatzManager::getHessian(std::vector<double> &H)
{
    if (!validateToRun()) return false;
    const int n = (int)m_excitations.size();
    std::vector<int> id(n);
    for (int i = 0; i < n; ++i) id[i] = i;
    std::vector<double> one(n, 1.0), g(n);
    H.assign((size_t)n * n, 0.0);
    double E;
    int rc = aegpu_hessian(m_engine, m_angles.data(), id.data(), one.data(), n, &E, g.data(), H.data());
    if (rc) { log_line(std::string("hessian failed: ") + aegpu_last_error(m_engine)); return false; }
    return true;
}

bool stateAnsatzManager::getGradient(const std::vector<double> &a, std::vector<double> &g)
{
    return setAngles(a) && getGradient(g);
}
bool stateAnsatzManager::getHessian(const std::vector<double> &a, std::vector<double> &H)
{
    return setAngles(a) && getHessian(H);
}

bool stateAnsatzManager::getExpectationValue(const std::vector<double> &a, double &E)
{
    return setAngles(a) && getExpectationValue(E);
}
bool stateAnsatzManager::getFinalState(const std::vector<double> &a, std::vector<double> &s)
{
    return setAngles(a) && getFinalState(s);
}
bool stateAnsatzManager::getFinalState(const std::vector<double> &a, std::vector<std::complex<double>> &s)
{
    return setAngles(a) && getFinalState(s);
}
bool stateAnsatzManager::getGradientComp(const std::vector<double> &a, std::vector<double> &g)
{
    return setAngles(a) && getGradientComp(g);
}
bool stateAnsatzManager::getHessianComp(const std::vector<double> &a, std::vector<double> &H)
{
    return setAngles(a) && getHessianComp(H);
}

// AnsatzManager.cpp:709-754 (evolveMultiple + getEnergies): the rows are evaluated as
// instances of a batched engine (shared Hamiltonian), in chunks whose per-instance
// buffers (state, H*state, pass checkpoints) stay within a few GB; the engine returns to
// a batch of one afterwards.
bool stateAnsatzManager::getExpectationValues(const std::vector<double> &angles, int nrows, int ncols, std::vector<double> &E)
{
    if (!validateToRun()) return false;
    if (nrows < 0 || ncols < 0 || angles.size() != (size_t)nrows * ncols) { log_line("Incorrect angle matrix"); return false; }
    const size_t nops = m_excitations.size();
    std::vector<double> all((size_t)nrows * nops);
    for (int r = 0; r < nrows; ++r) {
        std::vector<double> row(angles.begin() + (size_t)r * ncols, angles.begin() + (size_t)(r + 1) * ncols), a;
        if (!decompress(row, a)) return false;
        std::copy(a.begin(), a.end(), all.begin() + (size_t)r * nops);
    }
    E.assign(nrows, 0.0);
    int64_t info[8] = {0};
    aegpu_problem_info(m_engine, info);
    const double perInstance = (double)(info[2] + 4) * (double)info[0] * (m_complex ? 16.0 : 8.0);
    const int chunk = (int)std::max(1.0, std::min({256.0, (double)nrows, 8e9 / std::max(perInstance, 1.0)}));
    bool ok = true;
    for (int r0 = 0; r0 < nrows && ok; r0 += chunk) {
        const int n = std::min(chunk, nrows - r0);
        // a short last chunk repeats its last row up to the batch size (no reallocation)
        std::vector<double> a((size_t)chunk * nops), e(chunk);
        for (int k = 0; k < chunk; ++k) {
            const int src = r0 + std::min(k, n - 1);
            std::copy(all.begin() + (size_t)src * nops, all.begin() + (size_t)(src + 1) * nops, a.begin() + (size_t)k * nops);
        }
        int rc = aegpu_set_batch(m_engine, chunk);
        if (!rc) rc = aegpu_energy(m_engine, a.data(), e.data());
        if (rc) {
            log_line(std::string("energy failed: ") + aegpu_last_error(m_engine));
            ok = false;
            break;
        }
        for (int k = 0; k < n; ++k) E[r0 + k] = e[k] + m_nuclearEnergy;
    }
    if (aegpu_set_batch(m_engine, 1)) {
        log_line(std::string("restoring a batch of one failed: ") + aegpu_last_error(m_engine));
        return false;
    }
    // leave the manager's current state where it was
    m_haveEvolved = false;
    return ok && evolveIfNeeded();
}

bool stateAnsatzManager::getLowestEigenvalue(double &eigenvalue, double &residual, double tol)
{
    if (!validateToRun()) return false;
    // the Hamiltonian is fixed once constructed: one Lanczos run per tolerance
    if (!m_haveGround || tol < m_groundTol) {
        m_haveStates = 0;  // the single-state run replaces a k-state one on the device
        int products = 0;
        int rc = aegpu_lowest_eigenpair(m_engine, tol, 100, 100000, &m_groundE, &m_groundRes, &products);
        if (rc) { log_line(std::string("lowest eigenpair failed: ") + aegpu_last_error(m_engine)); return false; }
        if (m_groundRes > tol) log_line("lowest eigenpair: residual " + std::to_string(m_groundRes) + " above the tolerance");
        m_haveGround = true;
        m_groundTol = tol;
    }
    eigenvalue = m_groundE;
    residual = m_groundRes;
    return true;
}

bool stateAnsatzManager::setNumberOfOverlapsToCompute(int n)
{
    if (n <= 0) {
        log_line("numberOfOverlapsToCompute must be positive, set to 1");  // main.cpp:182-185
        n = 1;
    }
    m_numberOfOverlaps = n;
    return true;
}

bool stateAnsatzManager::getEigenstateOverlaps(const std::vector<std::vector<double>> &paths, int k,
                                               std::vector<double> &eigenvalues, std::vector<double> &overlaps)
{
    if (!validateToRun()) return false;
    if (m_haveStates < k) {
        // the k-state run replaces the single ground state on the device
        std::vector<double> E(k), res(k);
        int products = 0;
        int rc = aegpu_lowest_eigenpairs(m_engine, k, 1e-10, std::max(100, 20 * k), 100000, E.data(), res.data(),
                                         &products);
        if (rc) { log_line(std::string("lowest eigenpairs failed: ") + aegpu_last_error(m_engine)); return false; }
        for (int i = 0; i < k; ++i)
            if (res[i] > 1e-10) log_line("eigenpair " + std::to_string(i) + ": residual " + std::to_string(res[i]) +
                                         " above the tolerance");
        m_stateE = E;
        m_haveStates = k;
        m_haveGround = false;
    }
    eigenvalues.assign(m_stateE.begin(), m_stateE.begin() + k);
    overlaps.assign(paths.size() * 2 * (size_t)k, 0.0);
    for (size_t p = 0; p < paths.size(); ++p) {
        std::vector<double> a;
        if (!decompress(paths[p], a)) return false;
        int rc = aegpu_ground_overlaps(m_engine, a.data(), k, &overlaps[p * 2 * k]);
        if (rc) { log_line(std::string("overlaps failed: ") + aegpu_last_error(m_engine)); return false; }
    }
    m_haveEvolved = false;
    return evolveIfNeeded();
}

bool stateAnsatzManager::getProperties(const std::vector<std::vector<double>> &paths, int flags, std::vector<double> &table,
                                       std::vector<std::vector<double>> *hessians,
                                       std::vector<std::vector<double>> *metrics)
{
    if (!validateToRun()) return false;
    if (flags & AEGPU_PROP_OVERLAP) {
        double lam = 0, res = 0;
        if (!getLowestEigenvalue(lam, res)) return false;
    }
    const size_t P = (size_t)m_numberOfUniqueParameters;
    table.assign(paths.size() * AEGPU_PROPERTY_ROWS, 0.0);
    if (hessians) hessians->assign(paths.size(), std::vector<double>(P * P));
    if (metrics) metrics->assign(paths.size(), std::vector<double>(P * P));
    for (size_t k = 0; k < paths.size(); ++k) {
        std::vector<double> a;
        if (!decompress(paths[k], a)) return false;
        int rc = aegpu_path_properties(m_engine, a.data(), m_param.data(), m_scale.data(), (int)P, m_nuclearEnergy, flags,
                                       &table[k * AEGPU_PROPERTY_ROWS], hessians ? (*hessians)[k].data() : nullptr,
                                       metrics ? (*metrics)[k].data() : nullptr);
        if (rc) { log_line(std::string("properties failed: ") + aegpu_last_error(m_engine)); return false; }
    }
    m_haveEvolved = false;
    return evolveIfNeeded();
}

namespace {

// writeMatrix / writeVector / writeColumnVector of tupsquantities.cpp:25-164: row-major
// binary and a %.10g CSV for matrices (complex: re, im pairs and "re+imj,"), a row
// binary plus %.16g CSVs for vectors.
void write_matrix(const std::string &name, const std::vector<double> &M, size_t n, bool complexFile)
{
    if (FILE *f = fopen((name + (complexFile ? ".CMatbin" : ".Matbin")).c_str(), "wb")) {
        for (size_t i = 0; i < n * n; ++i) {
            const double z[2] = {M[i], 0.0};
            fwrite(z, sizeof(double), complexFile ? 2 : 1, f);
        }
        fclose(f);
    }
    if (FILE *f = fopen((name + (complexFile ? ".CMatcsv" : ".Matcsv")).c_str(), "w")) {
        for (size_t i = 0; i < n; ++i) {
            for (size_t j = 0; j < n; ++j) {
                if (complexFile) fprintf(f, "%.10g+%.10gj,", M[i * n + j], 0.0);
                else fprintf(f, "%.10g,", M[i * n + j]);
            }
            fprintf(f, "\n");
        }
        fclose(f);
    }
}

void write_vector(const std::string &name, const std::vector<double> &v)
{
    if (FILE *f = fopen((name + ".Vecbin").c_str(), "wb")) {
        fwrite(v.data(), sizeof(double), v.size(), f);
        fclose(f);
    }
    if (FILE *f = fopen((name + ".Veccsv").c_str(), "w")) {
        for (double x : v) fprintf(f, "%.16g,", x);
        fprintf(f, "\n");
        fclose(f);
    }
    if (FILE *f = fopen((name + ".ColVeccsv").c_str(), "w")) {
        for (double x : v) fprintf(f, "%.16g\n", x);
        fclose(f);
    }
}

}  // namespace

// TUPSQuantities::writeProperties (tupsquantities.cpp:185-568) with its printout
// (printOutputHeaders / printOutputLine, :2146-2205) and files: per path the Hessian
// and the metric (<runPath>_Path_<k>_Hessian / _Metric), and the overlap magnitudes
// with the ground state (<runPath>_MagOfOverlapWithGroundState_0).  haveHF: the first
// path is the zero-angle one (the "HF" column).
bool stateAnsatzManager::writeProperties(const std::vector<std::vector<double>> &paths, bool noHess, bool lowestEigenvalue,
                                         bool haveHF, const std::string &runPath, FILE *out)
{
    if (!validateToRun()) return false;
    std::vector<double> table;
    std::vector<std::vector<double>> H, M;
    // overlaps with more than the lowest eigenstate below 5,000 rows (the reference's dense
    // eigensolver regime, tupsquantities.cpp:229-276); computed after the table, which
    // then leaves its own overlap rows out
    const int64_t D = aegpu_dim(m_engine);
    const int nov = lowestEigenvalue ? (D < 5000 ? (int)std::min<int64_t>(m_numberOfOverlaps, D) : 1) : 0;
    const int flags = (noHess ? 0 : AEGPU_PROP_HESSIAN) | (nov == 1 ? AEGPU_PROP_OVERLAP : 0);
    if (!getProperties(paths, flags, table, noHess ? nullptr : &H, noHess ? nullptr : &M)) return false;
    const size_t np = paths.size(), P = (size_t)m_numberOfUniqueParameters;
    std::vector<double> ovl;  // [path][state][re, im]
    if (nov == 1) {
        ovl.assign(np * 2, 0.0);
        for (size_t k = 0; k < np; ++k) {
            ovl[2 * k] = table[k * AEGPU_PROPERTY_ROWS + AEGPU_PROP_OVERLAP_RE];
            ovl[2 * k + 1] = table[k * AEGPU_PROPERTY_ROWS + AEGPU_PROP_OVERLAP_IM];
        }
    } else if (nov > 1) {
        std::vector<double> eigs;
        if (!getEigenstateOverlaps(paths, nov, eigs, ovl)) return false;
    }
    if (!noHess && !runPath.empty())
        for (size_t k = 0; k < np; ++k) {
            write_matrix(runPath + "_Path_" + std::to_string(k) + "_Hessian", H[k], P, false);
            write_matrix(runPath + "_Path_" + std::to_string(k) + "_Metric", M[k], P, m_complex);
        }
    const int col = m_complex ? 42 : 26;
    if (!out) out = stdout;
    fprintf(out, "\n%-40s %40s \n%-40s", "Results:", "Path Number", "");
    if (haveHF) fprintf(out, "%-*s", col, "HF");
    for (size_t i = 1; i <= (haveHF ? np - 1 : np); ++i) fprintf(out, "%-*zu", col, i);
    fprintf(out, "\n");
    static const char *names[] = {"Elec. Energy", "Real Elec. Energy", "Elec. + Nuc. Energy",
                                  "NumberOfNegativeHessianEValues", "NumberOfNearZeroHessianEValues",
                                  "NumberOfPositiveHessianEValues", "NumberOfNegativeHessianDiagValues",
                                  "NumberOfNearZeroHessianDiagValues", "NumberOfPositiveHessianDiagValues",
                                  "NumberOfPositiveMetricEValues", "NumberOfZeroMetricEValues",
                                  "NumberOfZeroMetricDiagonalValues", "NormOfGradVector"};
    for (int r = 0; r <= AEGPU_PROP_NORM_OF_GRAD; ++r) {
        if (noHess && r >= AEGPU_PROP_NEG_HESSIAN_EVALUES && r <= AEGPU_PROP_ZERO_METRIC_DIAG) continue;
        fprintf(out, "%-40s", names[r]);
        for (size_t k = 0; k < np; ++k) fprintf(out, "%-*.16g", col, table[k * AEGPU_PROPERTY_ROWS + r]);
        fprintf(out, "\n");
    }
    for (int st = 0; st < nov; ++st) {
        std::vector<double> mag(np);
        fprintf(out, "%-40s", ("OverlapWithState_" + std::to_string(st)).c_str());
        for (size_t k = 0; k < np; ++k) {
            const double re = ovl[(k * nov + st) * 2], im = ovl[(k * nov + st) * 2 + 1];
            if (m_complex)
                fprintf(out, "%-20.16g, %-20.16g", re, im);
            else
                fprintf(out, "%-*.16g", col, re);
            mag[k] = std::hypot(re, im);
        }
        fprintf(out, "\n%-40s", ("MagOfOverlapWithState_" + std::to_string(st)).c_str());
        for (double v : mag) fprintf(out, "%-*.16g", col, v);
        fprintf(out, "\n");
        if (!runPath.empty()) write_vector(runPath + "_MagOfOverlapWithGroundState_" + std::to_string(st), mag);
    }
    fflush(out);
    return true;
}

bool stateAnsatzManager::getSubspaceEigenvalues(const std::vector<std::vector<double>> &paths, std::vector<double> &eigs,
                                                int &nullRank)
{
    if (!validateToRun()) return false;
    if (paths.empty()) { log_line("no paths given"); return false; }
    const size_t nops = m_excitations.size();
    std::vector<double> all(paths.size() * nops);
    for (size_t k = 0; k < paths.size(); ++k) {
        std::vector<double> a;
        if (!decompress(paths[k], a)) return false;
        std::copy(a.begin(), a.end(), all.begin() + k * nops);
    }
    eigs.assign(paths.size(), 0.0);
    int rc = aegpu_subspace_eigenvalues(m_engine, (int)paths.size(), all.data(), eigs.data(), &nullRank);
    if (rc) { log_line(std::string("subspace diagonalisation failed: ") + aegpu_last_error(m_engine)); return false; }
    m_haveEvolved = false;
    return evolveIfNeeded();
}

}  // namespace ae

#include "newton.h"

namespace ae {

// AnsatzManager.cpp:756-773 -> TUPSQuantities::OptimiseTups
// AnsatzManager.cpp:775-829: minima from random starts (std::srand(100), angles
// 2 pi rand() / RAND_MAX per parameter), each optimised by Newton-Raphson and kept when
// its energy differs from the ones found by more than 1e-10, then the subspace
// diagonalisation over them.  The reference's fused build refuses this (standard ansatz
// only) and otherwise loops until it finds enough minima; here at most 50 starts per
// requested path are tried.
bool stateAnsatzManager::generatePathsForSubspace(size_t numberOfPaths, std::vector<double> *eigenvalues, int *nullRank,
                                                  std::vector<std::vector<double>> *minima,
                                                  std::vector<double> *energies)
{
    if (!validateToRun()) return false;
    if (numberOfPaths == 0) { log_line("numberOfPaths must be positive"); return false; }
    std::srand(100);
    const int P = m_numberOfUniqueParameters;
    std::vector<double> Es;
    std::vector<std::vector<double>> paths;
    const size_t maxTries = 50 * numberOfPaths;
    for (size_t tries = 0; paths.size() < numberOfPaths && tries < maxTries; ++tries) {
        std::vector<double> x((size_t)P);
        for (int i = 0; i < P; ++i) x[(size_t)i] = (2 * M_PI * std::rand()) / RAND_MAX;
        double E = 0;
        if (!setAngles(x) || !optimise() || !getExpectationValue(E)) return false;
        if (std::none_of(Es.begin(), Es.end(), [&](double e) { return std::abs(e - E) < 1e-10; })) {
            Es.push_back(E);
            paths.push_back(m_angles);
        }
    }
    if (paths.size() < numberOfPaths) {
        log_line("generatePathsForSubspace: found " + std::to_string(paths.size()) + " distinct minima of " +
                 std::to_string(numberOfPaths));
        return false;
    }
    log_line("Found following Energies " + [&] {
        std::string t;
        for (double e : Es) t += std::to_string(e) + " ";
        return t;
    }());
    std::vector<double> w;
    int nr = 0;
    if (!getSubspaceEigenvalues(paths, w, nr)) return false;
    if (eigenvalues) *eigenvalues = w;
    if (nullRank) *nullRank = nr;
    if (minima) *minima = paths;
    if (energies) *energies = Es;
    return true;
}

// The driver's iterativeOptimise verb (main.cpp:502-515): TUPSQuantities::iterativeTups
// (the projected iteration, tupsquantities.cpp:2044-2145) from the current angles, then
// Newton-Raphson (OptimiseTups) from where it stopped.
bool stateAnsatzManager::iterativeOptimise()
{
    if (!validateToRun()) return false;
    const int P = m_numberOfUniqueParameters;
    std::vector<double> x((size_t)P, 0.0);
    std::vector<bool> seen((size_t)P, false);
    for (size_t o = 0; o < m_angles.size(); ++o)
        if (!seen[(size_t)m_param[o]] && m_scale[o] != 0) {
            x[(size_t)m_param[o]] = m_angles[o] / m_scale[o];
            seen[(size_t)m_param[o]] = true;
        }
    double E = 0, gn = 0;
    int64_t nh = 0, ne = 0;
    int outer = 0;
    int rc = aegpu_optimise_projected(m_engine, P, m_param.data(), m_scale.data(), x.data(), 1e-5, 3000, &E, &gn, &nh,
                                      &ne, &outer);
    if (rc) { log_line(std::string("iterative optimisation failed: ") + aegpu_last_error(m_engine)); return false; }
    log_line("iterativeTups: energy " + std::to_string(E) + " projected gradient " + std::to_string(gn) + " after " +
             std::to_string(outer) + " renewals");
    return setAngles(x) && optimise();
}

bool stateAnsatzManager::optimise()
{
    if (!validateToRun()) return false;
    NewtonProblem p;
    p.nparams = m_numberOfUniqueParameters;
    p.param = m_param;
    p.scale = m_scale;
    const int P = p.nparams;
    p.energy_grad = [&](const std::vector<double> &th, double &E, std::vector<double> &g) {
        std::vector<double> gops(th.size());
        if (aegpu_gradient(m_engine, th.data(), &E, gops.data())) return false;
        g.assign(P, 0.0);
        for (size_t i = 0; i < gops.size(); ++i) g[m_param[i]] += m_scale[i] * gops[i];
        return true;
    };
    p.hessian = [&](const std::vector<double> &th, double &E, std::vector<double> &g, std::vector<double> &H) {
        g.assign(P, 0.0);
        H.assign((size_t)P * P, 0.0);
        return aegpu_hessian(m_engine, th.data(), m_param.data(), m_scale.data(), P, &E, g.data(), H.data()) == AEGPU_OK;
    };
    NewtonStats st;
    std::vector<double> th = m_angles;
    if (!optimise_newton(p, th, st, true)) {
        log_line(std::string("optimise failed: ") + aegpu_last_error(m_engine));
        return false;
    }
    optimiseHessianEvals = st.hessian_evals;
    optimiseEnergyEvals = st.energy_evals;
    m_angles = th;
    m_haveEvolved = false;
    return evolveIfNeeded();
}

}  // namespace ae
