// stateAnsatzManager: drop-in replacement of the reference's manager class
// (AnsatzManager.h:59-295).  Same lifecycle: store* calls record the setup, the
// first evaluation validates it, picks the determinant sector, builds the
// Hamiltonian and the GPU engine, and later calls only re-evolve when the angles
// change.  All evaluation work runs on the GPU through the aegpu C ABI.
#pragma once
#include "../../include/aegpu.h"

#include <complex>
#include <cstdio>
#include <cstdint>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

namespace ae {

struct Exc4 {
    int8_t first, second, third, fourth;  // 0-based, -1 absent (stateRotate::exc)
};

class stateAnsatzManager {
public:
    // Per-context lock for external interfaces (AnsatzManager.h:115-121); not taken internally.
    std::mutex m_interfaceLock;

    stateAnsatzManager();
    ~stateAnsatzManager();
    stateAnsatzManager(const stateAnsatzManager &) = delete;
    stateAnsatzManager &operator=(const stateAnsatzManager &) = delete;

    bool storeOperators(const std::vector<Exc4> &excs);
    bool storeInitial(int numberOfQubits, const std::vector<int> &indexes, const std::vector<double> &coeffs);
    bool storeInitial(int numberOfQubits, const std::vector<int> &indexes, const std::vector<std::complex<double>> &coeffs);
    bool storeHamiltonian(std::vector<int> &&iIndexes, std::vector<int> &&jIndexes, std::vector<double> &&coeffs);
    bool storeNuclearEnergy(double nuclearEnergy);
    bool storeParameterDependencies(const std::vector<std::pair<int, double>> &parameterDependency);
    bool storeRunPath(const std::string &runPath);
    // Extension: integrals from memory (h[p*N+q], g[((p*N+q)*N+r)*N+s] = (pq|rs)), same
    // meaning as the <runPath>_oneEInts.bin / _twoEInts.bin files.  mode: AEGPU_HAM_*.
    bool storeIntegrals(int nOrbitals, const std::vector<double> &h1, const std::vector<double> &g2, int mode = 0);

    bool setAngles(std::vector<double> angles);
    std::vector<double> getAngles();  // compressed (m_normCompressMatrix)

    bool getExpectationValue(double &exptValue);
    bool getFinalState(std::vector<double> &finalState);                 // real part, 2^nq entries
    bool getFinalState(std::vector<std::complex<double>> &finalState);   // 2^nq entries
    bool getGradientComp(std::vector<double> &gradient);
    bool getHessianComp(std::vector<double> &hessian);                   // P x P, row-major (symmetric)
    // per operator (nOps and nOps x nOps): the reference's fused build traps here
    bool getGradient(std::vector<double> &gradient);
    bool getHessian(std::vector<double> &hessian);

    bool getExpectationValue(const std::vector<double> &angles, double &exptValue);
    bool getFinalState(const std::vector<double> &angles, std::vector<double> &finalState);
    bool getFinalState(const std::vector<double> &angles, std::vector<std::complex<double>> &finalState);
    bool getGradientComp(const std::vector<double> &angles, std::vector<double> &gradient);
    bool getHessianComp(const std::vector<double> &angles, std::vector<double> &hessian);
    bool getGradient(const std::vector<double> &angles, std::vector<double> &gradient);
    bool getHessian(const std::vector<double> &angles, std::vector<double> &hessian);
    // rows of `angles` (row-major, nrows x ncols) are angle sets; ncols = P or nOps
    bool getExpectationValues(const std::vector<double> &angles, int nrows, int ncols, std::vector<double> &exptValues);

    // Newton-Raphson with cubic backtracking (TUPSQuantities::OptimiseTups).
    bool optimise();
    // The projected iteration (TUPSQuantities::iterativeTups) then optimise().
    bool iterativeOptimise();
    // Distinct minima from seeded random starts, then the subspace diagonalisation over
    // them (AnsatzManager.cpp:775-829); the outputs are optional (minima per operator).
    bool generatePathsForSubspace(size_t numberOfPaths, std::vector<double> *eigenvalues = nullptr,
                                  int *nullRank = nullptr, std::vector<std::vector<double>> *minima = nullptr,
                                  std::vector<double> *energies = nullptr);

    // TUPSQuantities::writeProperties (tupsquantities.cpp:185-568): one row of
    // AEGPU_PROPERTY_ROWS values per path (compressed or per-operator angles), flags
    // AEGPU_PROP_HESSIAN / AEGPU_PROP_OVERLAP; the overlap rows use the lowest eigenvector,
    // computed first when needed.  Hessians / metrics (optional) per path, row-major.
    bool getProperties(const std::vector<std::vector<double>> &paths, int flags, std::vector<double> &table,
                       std::vector<std::vector<double>> *hessians = nullptr,
                       std::vector<std::vector<double>> *metrics = nullptr);
    // TUPSQuantities::writeProperties: the table printed to `out` (stdout when null) in
    // the reference's layout and, with a run path, its Hessian / metric / overlap files.
    bool writeProperties(const std::vector<std::vector<double>> &paths, bool noHess, bool lowestEigenvalue,
                         bool haveHF, const std::string &runPath, FILE *out = nullptr);
    // Lowest eigenvalue of H in the sector (electronic, without the nuclear energy).
    bool getLowestEigenvalue(double &eigenvalue, double &residual, double tol = 1e-10);
    // The reference's TUPSQuantitiesOptions::numberOfOverlapsToCompute (tupsquantities.h:22,
    // the CLI's option, main.cpp:181-185): writeProperties reports the overlaps with the
    // n lowest eigenstates when H has fewer than 5,000 rows (at most its row count), else
    // with the lowest one only (tupsquantities.cpp:229-276).
    bool setNumberOfOverlapsToCompute(int n);
    int numberOfOverlapsToCompute() const { return m_numberOfOverlaps; }
    // The k lowest eigenvalues of H in the sector (every spin symmetry of the sector) and
    // the overlaps <psi(path)|v_i> (re, im per state) for each path.
    bool getEigenstateOverlaps(const std::vector<std::vector<double>> &paths, int k, std::vector<double> &eigenvalues,
                               std::vector<double> &overlaps);
    // TUPSQuantities::doSubspaceDiagonalisation (tupsquantities.cpp:1600-1700).
    bool getSubspaceEigenvalues(const std::vector<std::vector<double>> &paths, std::vector<double> &eigenvalues,
                                int &nullRank);

    // introspection (not in the reference API)
    int numberOfQubits() const { return m_numberOfQubits; }
    int numberOfParameters() const { return m_numberOfUniqueParameters; }
    int numberOfOperators() const { return (int)m_excitations.size(); }
    bool isComplex() const { return m_complex; }
    aegpu_engine *engine() { return m_engine; }
    double nuclearEnergy() const { return m_nuclearEnergy; }
    const std::vector<int> &params() const { return m_param; }
    const std::vector<double> &scales() const { return m_scale; }
    int64_t optimiseHessianEvals = 0, optimiseEnergyEvals = 0;

private:
    bool validateToRun();
    bool construct();
    bool setHamiltonian();
    void setOperatorSymmetry();
    bool decompress(const std::vector<double> &in, std::vector<double> &out);
    bool evolveIfNeeded();

    std::vector<Exc4> m_excitations;
    std::vector<int> m_initIdx;
    std::vector<std::complex<double>> m_initCoeff;
    bool m_initComplex = false;
    std::vector<int> m_iIndexes, m_jIndexes;
    std::vector<double> m_coeffs;
    std::vector<double> m_h1, m_g2;
    int m_intsN = 0, m_intsMode = 0;
    std::vector<std::pair<int, double>> m_parameterDependency;
    std::vector<int> m_param;
    std::vector<double> m_scale;
    std::string m_runPath;
    double m_nuclearEnergy = 0;
    int m_numberOfUniqueParameters = -1;
    int m_numberOfQubits = -1;
    int m_numberOfParticles = -1, m_spinUp = -1, m_spinDown = -1;
    bool m_particleSym = false, m_InitialSZSym = false, m_OperatorSZSym = false;
    bool m_complex = false;
    bool m_isConstructed = false;
    int m_basisKind = 0;

    aegpu_engine *m_engine = nullptr;
    std::vector<double> m_angles;          // per operator
    bool m_haveEvolved = false;
    bool m_haveGround = false;             // lowest eigenpair computed (kept on the device)
    double m_groundE = 0, m_groundRes = 0, m_groundTol = 0;
    int m_numberOfOverlaps = 1;
    int m_haveStates = 0;                  // eigenpairs of the k-state run kept on the device
    std::vector<double> m_stateE;
};

void log_line(const std::string &s);

}  // namespace ae
