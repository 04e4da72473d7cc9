/*
 * AnsatzSynthInterface.h -- the reference's C / Fortran entry points, kept verbatim
 * as the drop-in boundary (signatures of src/Generated/AnsatzSynthInterface.h:14-26,
 * behaviour of src/AnsatzSynthInterface.cpp:18-629).  Exported by
 * libansatzevolve_gb300.so; every statevector operation behind them runs on the GPU.
 *
 *   init                 AnsatzSynthInterface.cpp:28   new manager handle
 *   cleanup              :42   takes the ADDRESS of the handle (void**); 0 ok, 1 null
 *   setExcitation        :64   = setExcitationScale(..., scale = NULL)
 *   setExcitationScale   :84   Fortran column-major 1-based operators[n*j+i]; 1-based order
 *   setHamiltonian       :154  1-based (i, j, coeff) triplets of the 2^nq matrix
 *   setInitialState      :201  1-based basis indices, real amplitudes
 *   setInitialStateComplex :252  complex amplitudes (always available here)
 *   getEnergy            :313  angles compressed or per operator; <psi|H|psi> + nuclear
 *   getFinalState        :362  dense 2^nq real state (real part in complex mode)
 *   getFinalStateComplex :440  dense 2^nq complex state
 *   getGradient_COMP     :519  compressed gradient; -6 on an internal size mismatch
 *   getHessian_COMP      :578  compressed Hessian, column-major hessian[n*j+i]
 *   setTraceInterfaceCalls :18 log every call's arguments
 * Return codes are the reference's: 0 ok, small positive per-argument errors, and
 * -6 for implementation faults.  No call traps.
 */
#ifndef ANSATZSYNTHINTERFACE_H
#define ANSATZSYNTHINTERFACE_H
#include <stddef.h>
#ifdef __cplusplus
#include <complex>
#define AE_DOUBLE_COMPLEX std::complex<double>
extern "C" {
#else
#define AE_DOUBLE_COMPLEX double _Complex
#endif

int cleanup(void *ctx);
int getEnergy(int nangles, const double *angles, double *energy, void *ctx);
int getFinalState(int nangles, const double *angles, int nbasisvectors, double *finalstate, void *ctx);
int getFinalStateComplex(int nangles, const double *angles, int nbasisvectors, AE_DOUBLE_COMPLEX *finalstate, void *ctx);
int getGradient_COMP(int nangles, const double *angles, double *gradient, void *ctx);
int getHessian_COMP(int nangles, const double *angles, double *hessian, void *ctx);
void *init(void);
int setExcitation(int nparams, const int *operators, const int *orderfile, void *ctx);
int setExcitationScale(int nparams, const int *operators, const int *orderfile, const double *scalefactor, void *ctx);
int setHamiltonian(int n, const int *iindexes, const int *jindexes, const double *coeffs, void *ctx);
int setInitialState(int numqubits, int n, const int *iindexes, const double *coeffs, void *ctx);
int setInitialStateComplex(int numqubits, int n, const int *iindexes, const AE_DOUBLE_COMPLEX *coeffs, void *ctx);
void setTraceInterfaceCalls(int val);

/* Extensions (no counterpart in the reference's C ABI, which has no way to pass
 * integrals; the reference reaches them only through stateAnsatzManager::storeRunPath):
 * setRunPath       -- prefix of <prefix>_oneEInts.bin / _twoEInts.bin (or _Ham_*.dat)
 * setIntegrals     -- integrals from memory: h[p*N+q], g[((p*N+q)*N+r)*N+s] = (pq|rs);
 *                     mode 0 auto, 1 stored rows, 2 on the fly
 * setNuclearEnergy -- constant added to every energy
 * optimise         -- Newton-Raphson from the current angles; writes the optimised
 *                     compressed angles and energy
 * setRunFiles      -- the whole setup the reference's command-line driver reads from a
 *                     path prefix (src/main.cpp:235-386): <prefix>_Initial.dat,
 *                     _Operators.dat, _Order.dat, _Nuclear_Energy.dat (if present) and
 *                     the Hamiltonian files of setRunPath (formats: aegpu_runfiles.h)
 * All return 0 on success, 1 for a null handle, 2 for bad arguments, 3 on failure. */
int setRunPath(const char *path, void *ctx);
int setIntegrals(int norb, const double *h1, const double *g2, int mode, void *ctx);
int setNuclearEnergy(double e, void *ctx);
int optimise(int nangles, double *angles, double *energy, void *ctx);
int setRunFiles(const char *prefix, void *ctx);
/* Properties (the reference's writeProperties / subspace diagonalisation, which its
 * C ABI does not expose): npaths angle rows of nangles (compressed or per operator).
 * getProperties writes npaths rows of AEGPU_PROPERTY_ROWS values (include/aegpu.h:
 * energies, Hessian / metric counts with AEGPU_PROP_HESSIAN, gradient norm, overlaps
 * with the lowest eigenvector with AEGPU_PROP_OVERLAP; NaN where not computed).
 * getLowestEigenvalue: the lowest eigenvalue of H in the sector (electronic).
 * getSubspaceEigenvalues: the npaths eigenvalues of S^-1/2 H S^-1/2 and S's null rank. */
/* getExpectationValues: energies (with the nuclear energy) of nrows angle rows of
 * nangles (compressed or per operator), evaluated as one batch on the GPU
 * (stateAnsatzManager::getExpectationValues, src/AnsatzManager.cpp:709-754). */
int getExpectationValues(int nrows, int nangles, const double *angles, double *energies, void *ctx);
/* getGradient / getHessian: derivatives with respect to every operator's angle (nOps and
 * nOps x nOps values) at compressed or per-operator angles.  The reference's fused build
 * traps on these (src/AnsatzManager.cpp:570-574, 616-620); here every operator is its
 * own parameter. */
/* generatePathsForSubspace (src/AnsatzManager.cpp:775-829): numberOfPaths distinct
 * minima (energies, with the nuclear energy; NULL to skip) from seeded random starts,
 * then the eigenvalues of the subspace Hamiltonian over them and its overlap matrix's
 * null rank.  3 when fewer distinct minima turn up in 50 starts per path. */
int generatePathsForSubspace(int numberOfPaths, double *eigenvalues, int *nullRank, double *energies, void *ctx);
/* iterativeOptimise: the driver's iterativeOptimise verb (src/main.cpp:502-515), the
 * projected iteration (iterativeTups) then Newton-Raphson; angles and energy as in
 * optimise. */
int iterativeOptimise(int nangles, double *angles, double *energy, void *ctx);
int getGradient(int nangles, const double *angles, double *gradient, void *ctx);
int getHessian(int nangles, const double *angles, double *hessian, void *ctx);
int getProperties(int npaths, int nangles, const double *angles, int flags, double *table, void *ctx);
int getLowestEigenvalue(double *eigenvalue, double *residual, void *ctx);
/* writeProperties: the reference's printed table on stdout and, when runPath is given,
 * its files <runPath>_Path_<k>_Hessian / _Metric (.Matbin / .Matcsv, complex runs write
 * the metric as .CMatbin / .CMatcsv) and <runPath>_MagOfOverlapWithGroundState_0
 * (.Vecbin / .Veccsv / .ColVeccsv); flags as getProperties plus AEGPU_PROP_HF_PATH. */
int writeProperties(int npaths, int nangles, const double *angles, int flags, const char *runPath, void *ctx);
/* setNumberOfOverlapsToCompute: the reference's numberOfOverlapsToCompute option
 * (TUPSQuantitiesOptions, tupsquantities.h:22; CLI main.cpp:181-185): writeProperties then
 * reports OverlapWithState_i / MagOfOverlapWithState_i for the n lowest eigenstates of H
 * when H has fewer than 5,000 rows (at most its row count), else for the lowest only.
 * 1 null context, 2 n < 1. */
int setNumberOfOverlapsToCompute(int n, void *ctx);
int getSubspaceEigenvalues(int npaths, int nangles, const double *angles, double *eigenvalues, int *nullRank,
                           void *ctx);

#ifdef __cplusplus
}
#endif
#endif
