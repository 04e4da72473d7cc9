// Pinning driver for the reference AnsatzEvolve library (test infrastructure only).
//
// Linked against the reference's own objects by oracle/build_ref.sh.  It drives the
// reference's public C++ API (stateAnsatzManager, AnsatzManager.h:59-295) and, for
// timing, FusedEvolve exactly the way the reference CLI benchmark does
// (main.cpp:404-425), and writes every result as raw little-endian doubles so that
// tests/golden/make_golden.py can turn them into committed fixtures.
//
// Input is a whitespace-separated text spec (see tests/golden/make_golden.py):
//   nqubits Q
//   initial n   {idx re im} x n          (0-based full-space indices)
//   ops n       {a b c d} x n            (0-based, -1 = absent)
//   order n     {param scale} x n        (0-based parameter index)
//   ham triplets n {i j v} x n  |  ham ints <prefix>
//   nuclear E
//   anglesets m len {values}             (compressed or per-operator angles)
//   want e g h s                         (0/1 flags per output)
//   pairs 0|1                            (dump the per-excitation partner/sign rule)
//   pairsfile <path>                     (the same rule over the sector of the initial
//                                         state only, ascending bitstrings: for every
//                                         excitation uint32 partners then int8 signs,
//                                         written raw to <path>)
//   optimise 0|1
//   time k                               (k timed evolve+evolveDerivative units)
//   timewarmup w                         (untimed units before them, default 1)
//   timebudget s                         (stop timing after s seconds, default none)
//   properties <prefix>                  (TUPSQuantities::writeProperties over the zero
//                                         path + the angle sets; its table goes to
//                                         <prefix>_table.txt, its matrices to <prefix>_Path_*)
//   overlaps k                           (with properties: numberOfOverlapsToCompute)
//   subspace n                           (with properties: doSubspaceDiagonalisation of
//                                         the first n angle sets; printed on stderr)
//   end
// Output: for every angle set, E, gradient, Hessian (column-major), final state;
// then the pair table, then the optimised energy + angles, then timings (set-up
// seconds, thread count, n, n unit times, E, P, the compressed gradient).
#include "AnsatzManager.h"
#include "fusedevolve.h"
#include "hamiltonianmatrix.h"
#include "operatorpool.h"
#include "threadpool.h"
#include "tupsquantities.h"
#include <chrono>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

// Free function with external linkage in fusedevolve.cpp:27-145.
std::pair<uint32_t, bool> applyExcToBasisState_(uint32_t state, const stateRotate::exc &a);

template <typename T> T toNum(double re, double) { return re; }
template <> std::complex<double> toNum<std::complex<double>>(double re, double im) { return {re, im}; }

static void put(FILE *f, const double *p, size_t n) { fwrite(p, sizeof(double), n, f); }
static void put1(FILE *f, double v) { put(f, &v, 1); }

int main(int argc, char **argv)
{
    if (argc < 3) { fprintf(stderr, "usage: ref_driver spec out\n"); return 2; }
    std::ifstream in(argv[1]);
    FILE *out = fopen(argv[2], "wb");
    if (!in || !out) { fprintf(stderr, "cannot open files\n"); return 2; }
    constexpr bool isComplex = !std::is_same_v<realNumType, numType>;

    int nq = 0;
    std::vector<int> initIdx;
    std::vector<numType> initCoeff;
    std::vector<stateRotate::exc> excs;
    std::vector<std::pair<int, realNumType>> order;
    std::vector<int> hi, hj;
    std::vector<realNumType> hv;
    std::string intsPrefix;
    double nuclear = 0;
    std::vector<std::vector<double>> angleSets;
    int wantE = 1, wantG = 1, wantH = 0, wantS = 0, wantPairs = 0, wantOpt = 0, timeK = 0, timeWarm = 1;
    double timeBudget = 0.0;
    std::string propsPrefix, pairsPath;
    int subspaceN = 0, overlapsK = 1;

    std::string tok;
    while (in >> tok) {
        if (tok == "nqubits") in >> nq;
        else if (tok == "initial") {
            int n; in >> n;
            for (int k = 0; k < n; ++k) {
                int idx; double re, im; in >> idx >> re >> im;
                initIdx.push_back(idx);
                initCoeff.push_back(toNum<numType>(re, im));
            }
        } else if (tok == "ops") {
            int n; in >> n;
            for (int k = 0; k < n; ++k) {
                int v[4]; in >> v[0] >> v[1] >> v[2] >> v[3];
                int8_t a[4] = {(int8_t)v[0], (int8_t)v[1], (int8_t)v[2], (int8_t)v[3]};
                excs.emplace_back(a);
            }
        } else if (tok == "order") {
            int n; in >> n;
            for (int k = 0; k < n; ++k) { int p; double s; in >> p >> s; order.push_back({p, s}); }
        } else if (tok == "ham") {
            std::string kind; in >> kind;
            if (kind == "triplets") {
                int n; in >> n;
                for (int k = 0; k < n; ++k) { int i, j; double v; in >> i >> j >> v; hi.push_back(i); hj.push_back(j); hv.push_back(v); }
            } else in >> intsPrefix;
        } else if (tok == "nuclear") in >> nuclear;
        else if (tok == "anglesets") {
            int m, len; in >> m >> len;
            for (int k = 0; k < m; ++k) { std::vector<double> a(len); for (auto &x : a) in >> x; angleSets.push_back(a); }
        } else if (tok == "want") in >> wantE >> wantG >> wantH >> wantS;
        else if (tok == "pairs") in >> wantPairs;
        else if (tok == "pairsfile") in >> pairsPath;
        else if (tok == "optimise") in >> wantOpt;
        else if (tok == "time") in >> timeK;
        else if (tok == "timewarmup") in >> timeWarm;
        else if (tok == "timebudget") in >> timeBudget;
        else if (tok == "properties") in >> propsPrefix;
        else if (tok == "subspace") in >> subspaceN;
        else if (tok == "overlaps") in >> overlapsK;
        else if (tok == "end") break;
        else { fprintf(stderr, "bad token %s\n", tok.c_str()); return 2; }
    }
    threadpool::getInstance(NUM_CORES);

    stateAnsatzManager man;
    bool ok = man.storeInitial(nq, initIdx, initCoeff) && man.storeOperators(excs) &&
              man.storeParameterDependencies(order) && man.storeNuclearEnergy(nuclear);
    if (!hv.empty()) ok = ok && man.storeHamiltonian(std::move(hi), std::move(hj), std::move(hv));
    else ok = ok && man.storeRunPath(intsPrefix);
    if (!ok) { fprintf(stderr, "setup failed\n"); return 3; }

    for (auto &ang : angleSets) {
        if (wantE) {
            realNumType E = 0;
            if (!man.getExpectationValue(ang, E)) { fprintf(stderr, "energy failed\n"); return 4; }
            put1(out, E);
        }
        if (wantG) {
            vector<realNumType> g;
            if (!man.getGradientComp(ang, g)) { fprintf(stderr, "gradient failed\n"); return 4; }
            put(out, &g[0], g.size());
        }
        if (wantH) {
            Matrix<realNumType>::EigenMatrix H;
            if (!man.getHessianComp(ang, H)) { fprintf(stderr, "hessian failed\n"); return 4; }
            for (long j = 0; j < H.cols(); ++j)
                for (long i = 0; i < H.rows(); ++i) put1(out, H(i, j));
        }
        if (wantS) {
            vector<numType> s;
            if (!man.getFinalState(ang, s)) { fprintf(stderr, "state failed\n"); return 4; }
            put(out, (const double *)&s[0], s.size() * (isComplex ? 2 : 1));
        }
    }
    if (wantPairs) {
        // partner bitstring and sign of every excitation on every full-space bitstring
        uint32_t n = 1u << nq;
        for (size_t e = 0; e < excs.size(); ++e)
            for (uint32_t s = 0; s < n; ++s) {
                uint32_t in_s = isComplex ? (s << 1) : s;
                auto r = applyExcToBasisState_(in_s, excs[e]);
                uint32_t partner = isComplex ? (r.first >> 1) : r.first;
                double rec[2] = {(double)partner, r.second ? 1.0 : -1.0};
                put(out, rec, 2);
            }
    }
    if (!pairsPath.empty()) {
        // applyExcToBasisState_ (fusedevolve.cpp:27-145) over the ascending sector list
        uint32_t ones = -1;
        int spinUp = bitwiseDot(initIdx[0] >> (nq / 2), ones, 32), spinDown = bitwiseDot(initIdx[0], ones, nq / 2);
        std::vector<uint32_t> sector;
        for (uint32_t s = 0; s < (1u << nq); ++s)
            if (bitwiseDot(s >> (nq / 2), ones, 32) == spinUp && bitwiseDot(s, ones, nq / 2) == spinDown)
                sector.push_back(s);
        FILE *pf = fopen(pairsPath.c_str(), "wb");
        if (!pf) { fprintf(stderr, "cannot open %s\n", pairsPath.c_str()); return 2; }
        std::vector<uint32_t> partner(sector.size());
        std::vector<int8_t> sign(sector.size());
        for (size_t e = 0; e < excs.size(); ++e) {
            for (size_t k = 0; k < sector.size(); ++k) {
                uint32_t in_s = isComplex ? (sector[k] << 1) : sector[k];
                auto r = applyExcToBasisState_(in_s, excs[e]);
                partner[k] = isComplex ? (r.first >> 1) : r.first;
                sign[k] = r.second ? 1 : -1;
            }
            fwrite(partner.data(), sizeof(uint32_t), partner.size(), pf);
            fwrite(sign.data(), 1, sign.size(), pf);
        }
        fclose(pf);
    }
    if (wantOpt) {
        auto t0 = std::chrono::steady_clock::now();
        if (!man.optimise()) { fprintf(stderr, "optimise failed\n"); return 4; }
        auto t1 = std::chrono::steady_clock::now();
        realNumType E = 0;
        man.getExpectationValue(E);
        auto a = man.getAngles();
        put1(out, E);
        put1(out, std::chrono::duration<double>(t1 - t0).count());
        put1(out, (double)a.size());
        put(out, a.data(), a.size());
    }
    if (timeK > 0 && !intsPrefix.empty()) {
        // FusedEvolve::evolve + evolveDerivative(&E): one H*psi per unit, as in main.cpp:415-425
        uint32_t ones = -1;
        int spinUp = bitwiseDot(initIdx[0] >> (nq / 2), ones, 32), spinDown = bitwiseDot(initIdx[0], ones, nq / 2);
        std::shared_ptr<compressor> comp = std::make_shared<SZAndnumberOperatorCompressor>(1u << nq, spinUp, spinDown);
        vector<numType> full;
        full.resize(1u << nq, false, nullptr);
        for (size_t k = 0; k < initIdx.size(); ++k) full[initIdx[k]] = initCoeff[k];
        vector<numType> start;
        compressor::compressVector<numType>(full, start, comp);
        auto t0 = std::chrono::steady_clock::now();
        auto Ham = std::make_shared<HamiltonianMatrix<realNumType, numType>>(intsPrefix, nq, comp);
        int P = 0;
        for (auto &o : order) P = std::max(P, o.first + 1);
        TUPSQuantities q(Ham, order, P, 0, intsPrefix);
        FusedEvolve FE(start, Ham, q.m_compressMatrix, q.m_deCompressMatrix);
        FE.updateExc(excs);
        std::vector<realNumType> ang(excs.size());
        const auto &a0 = angleSets.at(0);
        if (a0.size() == excs.size()) ang = a0;
        else for (size_t i = 0; i < excs.size(); ++i) ang[i] = a0[order[i].first] * order[i].second;
        vector<numType> dest;
        vector<realNumType> deriv;
        realNumType E = 0;
        FE.evolve(dest, ang);
        FE.evolveDerivative(dest, deriv, ang, &E);
        auto t1 = std::chrono::steady_clock::now();
        for (int w = 0; w < timeWarm; ++w) { FE.evolve(dest, ang); FE.evolveDerivative(dest, deriv, ang, &E); }
        std::vector<double> times;
        const auto tstart = std::chrono::steady_clock::now();
        for (int k = 0; k < timeK; ++k) {
            auto a = std::chrono::steady_clock::now();
            FE.evolve(dest, ang);
            FE.evolveDerivative(dest, deriv, ang, &E);
            auto b = std::chrono::steady_clock::now();
            times.push_back(std::chrono::duration<double>(b - a).count());
            if (timeBudget > 0 && std::chrono::duration<double>(b - tstart).count() > timeBudget) break;
        }
        put1(out, std::chrono::duration<double>(t1 - t0).count());
        put1(out, (double)NUM_CORES);
        put1(out, (double)times.size());
        put(out, times.data(), times.size());
        put1(out, E);
        put1(out, (double)deriv.size());
        put(out, &deriv[0], deriv.size());
    }
    if (!propsPrefix.empty() && !intsPrefix.empty()) {
        // the reference's own properties pass (tupsquantities.cpp:185-568) on the
        // integral Hamiltonian, as the CLI's writeproperties verb runs it (main.cpp:520-529)
        uint32_t ones = -1;
        int spinUp = bitwiseDot(initIdx[0] >> (nq / 2), ones, 32), spinDown = bitwiseDot(initIdx[0], ones, nq / 2);
        std::shared_ptr<compressor> comp = std::make_shared<SZAndnumberOperatorCompressor>(1u << nq, spinUp, spinDown);
        vector<numType> full;
        full.resize(1u << nq, false, nullptr);
        for (size_t k = 0; k < initIdx.size(); ++k) full[initIdx[k]] = initCoeff[k];
        vector<numType> start;
        compressor::compressVector<numType>(full, start, comp);
        auto Ham = std::make_shared<HamiltonianMatrix<realNumType, numType>>(intsPrefix, nq, comp);
        int P = 0;
        for (auto &o : order) P = std::max(P, o.first + 1);
        FILE *table = fopen((propsPrefix + "_table.txt").c_str(), "w");
        TUPSQuantities q(Ham, order, P, nuclear, propsPrefix, table);
        auto FE = std::make_shared<FusedEvolve>(start, Ham, q.m_compressMatrix, q.m_deCompressMatrix);
        FE->updateExc(excs);
        std::vector<std::vector<ansatz::rotationElement>> paths(1, std::vector<ansatz::rotationElement>(excs.size(), {0, 0.0}));
        for (auto &a0 : angleSets) {
            paths.emplace_back(excs.size(), ansatz::rotationElement{0, 0.0});
            for (size_t i = 0; i < excs.size(); ++i)
                paths.back()[i].second = a0.size() == excs.size() ? a0[i] : a0[order[i].first] * order[i].second;
        }
        TUPSQuantitiesOptions opts;
        opts.numberOfOverlapsToCompute = overlapsK;
        q.writeProperties(nullptr, FE, paths, opts);
        fclose(table);
        if (subspaceN > 0) q.doSubspaceDiagonalisation(nullptr, FE, (size_t)subspaceN, paths);
    }
    fclose(out);
    return 0;
}
