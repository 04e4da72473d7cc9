// Readers for the reference's run files, the inputs its command-line driver takes
// from a path prefix (main.cpp:221-386):
//   <prefix>_Initial.dat         initial state, "bitstring,re[,im]" per line
//   <prefix>_Operators.dat       excitations "a b c d", 1-based, 0 = absent
//   <prefix>_Order.dat           "parameter[,scale]" per operator, 1-based
//   <prefix>_Parameters.dat      angle sets: count, an "...= energy ..." line, angles
//   <prefix>_Nuclear_Energy.dat  one number (optional)
//   <prefix>_extractedmin        bare angle sets (optional, loadExtractedMin)
// The Hamiltonian files (<prefix>_oneEInts.bin / _twoEInts.bin or _Ham_*.dat) are
// read by stateAnsatzManager::storeRunPath when the manager is constructed.
#pragma once
#include "manager.h"

#include <complex>
#include <string>
#include <utility>
#include <vector>

namespace ae {

struct RunFiles {
    int numberOfQubits = 0;
    std::vector<int> initialIndex;  // 0-based, into the full 2^nq space
    std::vector<std::complex<double>> initialCoeff;
    std::vector<Exc4> operators;  // 0-based, -1 absent
    std::vector<std::pair<int, double>> orders;  // 0-based parameter, scale
    // Parameters the operators use: max order + 1 (what the manager works with).
    int numberOfParameters = 0;
    // The reference driver's count, max(max order + 1, angles in the last set of the
    // Parameters file) (TUPSLoadingUtils.cpp:255, 287); it also sizes extractedmin's sets.
    int numberOfUniqueParameters = 0;
    // Angle sets in file order, numberOfParameters each: the angle of parameter p is
    // the file's p-th angle when the file's last set has more than p angles and the
    // set itself has one, else 0 (TUPSLoadingUtils.cpp:275-280).
    std::vector<std::vector<double>> parameterSets;
    std::vector<double> parameterEnergies;  // the number after '=' on each set's line
    double nuclearEnergy = 0.0;
    bool haveNuclearEnergy = false;
};

// TUPSLoadingUtils.cpp:48-97: bit i of an index is the i-th character from the right;
// the qubit count is the longest bitstring; a line with a bitstring alone has
// coefficient 1; a repeated bitstring keeps its last coefficient.
bool readCsvState(const std::string &path, int &numberOfQubits, std::vector<int> &index,
                  std::vector<std::complex<double>> &coeff, std::string &err);
// TUPSLoadingUtils.cpp:10-36 (loadPath): four integers per operator, made 0-based.
bool loadOperators(const std::string &path, std::vector<Exc4> &ops, std::string &err);
// TUPSLoadingUtils.cpp:259-293: "parameter" or "parameter,scale" per operator.
bool loadOrder(const std::string &path, std::vector<std::pair<int, double>> &orders, std::string &err);
// TUPSLoadingUtils.cpp:233-254: repeated {count; text '=' energy text; count angles}.
bool loadParameterFile(const std::string &path, std::vector<std::vector<double>> &sets,
                       std::vector<double> &energies, std::string &err);
// TUPSLoadingUtils.cpp:298-360: whitespace-separated angles, n per set.
bool loadExtractedMin(const std::string &path, int n, std::vector<std::vector<double>> &sets, std::string &err);
// TUPSLoadingUtils.cpp:156-173: false (energy 0) when the file is missing or empty.
bool LoadNuclearEnergy(double &nuclearEnergy, const std::string &prefix);

// TUPSLoadingUtils.cpp:176-296 (loadParameters): the order file (one relation per
// operator, nOps of them) and the Parameters file (optional) into rf's orders, parameter
// counts, angle sets and energies; with extractedMinPath, the sets of that file instead.
bool loadParameters(const std::string &orderPath, const std::string &parameterPath, size_t nOps,
                    const std::string &extractedMinPath, RunFiles &rf, std::string &err);

// All of the above for one prefix, as the driver loads them (main.cpp:235-386).  A
// missing Parameters file leaves no angle sets (the driver carries on with only the
// zero-angle path); extractedMin replaces the Parameters file's sets with those of
// <prefix>_extractedmin.
bool loadRunFiles(const std::string &prefix, bool extractedMin, RunFiles &rf, std::string &err);
// storeInitial / storeOperators / storeParameterDependencies / storeNuclearEnergy /
// storeRunPath(prefix) on a manager that has not been constructed yet.
bool storeRunFiles(stateAnsatzManager &m, const RunFiles &rf, const std::string &prefix, std::string &err);

}  // namespace ae
