// Readers for the reference's run files and their C ABI (include/aegpu_runfiles.h).
// The file formats follow TUPSLoadingUtils.cpp and the reference manual's description
// of the data files; malformed input that the reference reads as garbage (a truncated
// operator line, a short angle set, an unreadable count) is an error here instead.
#include "runfiles.h"

#include "../../include/aegpu_runfiles.h"

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <iterator>
#include <limits>
#include <map>

namespace ae {

namespace {

bool slurp(const std::string &path, std::string &out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    return true;
}

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

// Whitespace-separated numbers, as fscanf's %i / %lg read them.
struct Cursor {
    const std::string &s;
    size_t p = 0;
    explicit Cursor(const std::string &str) : s(str) {}
    void skip_ws() { while (p < s.size() && is_space(s[p])) ++p; }
    bool at_end() { skip_ws(); return p >= s.size(); }
    bool read_long(long &v)
    {
        skip_ws();
        if (p >= s.size()) return false;
        const char *b = s.c_str() + p;
        char *e = nullptr;
        errno = 0;
        v = std::strtol(b, &e, 10);
        if (e == b || errno == ERANGE) return false;
        p += (size_t)(e - b);
        return true;
    }
    bool read_double(double &v)
    {
        skip_ws();
        if (p >= s.size()) return false;
        const char *b = s.c_str() + p;
        char *e = nullptr;
        v = std::strtod(b, &e);
        if (e == b) return false;
        p += (size_t)(e - b);
        return true;
    }
};

std::vector<std::string> lines_of(const std::string &s)
{
    std::vector<std::string> out;
    size_t a = 0;
    while (a <= s.size()) {
        size_t b = s.find('\n', a);
        if (b == std::string::npos) b = s.size();
        std::string l = s.substr(a, b - a);
        if (!l.empty() && l.back() == '\r') l.pop_back();
        out.push_back(l);
        a = b + 1;
    }
    return out;
}

}  // namespace

bool readCsvState(const std::string &path, int &numberOfQubits, std::vector<int> &index,
                  std::vector<std::complex<double>> &coeff, std::string &err)
{
    std::string text;
    if (!slurp(path, text)) { err = "cannot open " + path; return false; }
    numberOfQubits = 0;
    index.clear();
    coeff.clear();
    std::map<int, size_t> where;
    int lineNo = 0;
    for (const std::string &line : lines_of(text)) {
        ++lineNo;
        size_t p = 0;
        while (p < line.size() && is_space(line[p])) ++p;
        if (p == line.size()) continue;
        size_t q = p;
        while (q < line.size() && (line[q] == '0' || line[q] == '1')) ++q;
        const size_t len = q - p;
        if (len == 0) { err = path + ":" + std::to_string(lineNo) + ": missing bitstring"; return false; }
        if (len > 31) { err = path + ":" + std::to_string(lineNo) + ": bitstring longer than 31 qubits"; return false; }
        int bits = 0;
        for (size_t i = 0; i < len; ++i)
            if (line[q - 1 - i] == '1') bits |= 1 << i;
        double re = 1.0, im = 0.0;  // a bitstring alone: magnitude 1 (TUPSLoadingUtils.cpp:73-79)
        if (q < line.size() && line[q] == ',') {
            const char *b = line.c_str() + q + 1;
            char *e = nullptr;
            const double v = std::strtod(b, &e);
            if (e != b) {
                re = v;
                const char *c = e;
                while (*c && is_space(*c)) ++c;
                if (*c == ',') {
                    const double w = std::strtod(c + 1, &e);
                    if (e != c + 1) im = w;
                }
            }
        }
        numberOfQubits = std::max(numberOfQubits, (int)len);
        auto it = where.find(bits);
        if (it != where.end()) {
            coeff[it->second] = {re, im};  // a repeated bitstring overwrites the earlier one
        } else {
            where[bits] = index.size();
            index.push_back(bits);
            coeff.push_back({re, im});
        }
    }
    if (index.empty()) { err = path + ": no basis states"; return false; }
    return true;
}

bool loadOperators(const std::string &path, std::vector<Exc4> &ops, std::string &err)
{
    std::string text;
    if (!slurp(path, text)) { err = "cannot open " + path; return false; }
    ops.clear();
    Cursor c(text);
    while (!c.at_end()) {
        long v[4];
        for (int k = 0; k < 4; ++k) {
            if (!c.read_long(v[k])) {
                err = path + ": operator " + std::to_string(ops.size() + 1) + " does not have four integers";
                return false;
            }
            if (v[k] < 0 || v[k] > 64) {
                err = path + ": operator " + std::to_string(ops.size() + 1) + " has an index outside 0..64";
                return false;
            }
        }
        ops.push_back({(int8_t)(v[0] - 1), (int8_t)(v[1] - 1), (int8_t)(v[2] - 1), (int8_t)(v[3] - 1)});
    }
    return true;
}

bool loadOrder(const std::string &path, std::vector<std::pair<int, double>> &orders, std::string &err)
{
    std::string text;
    if (!slurp(path, text)) { err = "cannot open " + path; return false; }
    orders.clear();
    Cursor c(text);
    while (!c.at_end()) {
        long o = 0;
        if (!c.read_long(o)) { err = path + ": entry " + std::to_string(orders.size() + 1) + " is not an integer"; return false; }
        if (o < 1 || o > std::numeric_limits<int>::max()) {
            err = path + ": entry " + std::to_string(orders.size() + 1) + ": Order cannot be negative";
            return false;
        }
        double scale = 1.0;
        // "%i,%lg": the scale only when a comma follows the integer directly
        if (c.p < text.size() && text[c.p] == ',') {
            ++c.p;
            double v;
            if (c.read_double(v)) scale = v;
        }
        orders.push_back({(int)(o - 1), scale});
    }
    return true;
}

bool loadParameterFile(const std::string &path, std::vector<std::vector<double>> &sets,
                       std::vector<double> &energies, std::string &err)
{
    std::string text;
    if (!slurp(path, text)) { err = "cannot open " + path; return false; }
    sets.clear();
    energies.clear();
    Cursor c(text);
    while (!c.at_end()) {
        long n = 0;
        if (!c.read_long(n) || n < 0) { err = path + ": Format Invalid, Number of Parameters (set " + std::to_string(sets.size() + 1) + ")"; return false; }
        // "%*[^=]= %lg %*[^\n]": skip to '=', read the energy, drop the rest of the line
        const size_t eq = text.find('=', c.p);
        if (eq == std::string::npos) { err = path + ": set " + std::to_string(sets.size() + 1) + " has no '=' energy line"; return false; }
        c.p = eq + 1;
        double e = std::nan("");
        if (!c.read_double(e)) e = std::nan("");
        const size_t nl = text.find('\n', c.p);
        c.p = nl == std::string::npos ? text.size() : nl;
        std::vector<double> a((size_t)n);
        for (long i = 0; i < n; ++i)
            if (!c.read_double(a[(size_t)i])) {
                err = path + ": set " + std::to_string(sets.size() + 1) + " has fewer than " + std::to_string(n) + " angles";
                return false;
            }
        sets.push_back(std::move(a));
        energies.push_back(e);
    }
    return true;
}

bool loadExtractedMin(const std::string &path, int n, std::vector<std::vector<double>> &sets, std::string &err)
{
    std::string text;
    if (!slurp(path, text)) { err = "cannot open " + path; return false; }
    if (n < 1) { err = path + ": no parameters to read"; return false; }
    sets.clear();
    Cursor c(text);
    while (!c.at_end()) {
        std::vector<double> a((size_t)n);
        for (int i = 0; i < n; ++i)
            if (!c.read_double(a[(size_t)i])) {
                err = path + ": Unable to read an angle when I expected an angle (set " + std::to_string(sets.size() + 1) + ")";
                return false;
            }
        sets.push_back(std::move(a));
    }
    return true;
}

bool LoadNuclearEnergy(double &nuclearEnergy, const std::string &prefix)
{
    nuclearEnergy = 0.0;
    std::string text;
    if (!slurp(prefix + "_Nuclear_Energy.dat", text)) return false;
    Cursor c(text);
    double v;
    if (!c.read_double(v)) return false;
    nuclearEnergy = v;
    return true;
}

bool loadParameters(const std::string &orderPath, const std::string &parameterPath, size_t nOps,
                    const std::string &extractedMinPath, RunFiles &rf, std::string &err)
{
    if (!loadOrder(orderPath, rf.orders, err)) return false;
    if (rf.orders.size() != nOps) {
        err = orderPath + ": " + std::to_string(rf.orders.size()) + " relations for " + std::to_string(nOps) +
              " operators (More operators in path than relations given)";
        return false;
    }
    int maxOrder = -1;
    for (const auto &o : rf.orders) maxOrder = std::max(maxOrder, o.first);
    rf.numberOfParameters = maxOrder + 1;

    std::vector<std::vector<double>> raw;
    std::string perr;
    int lastCount = 0;
    rf.parameterEnergies.clear();
    if (loadParameterFile(parameterPath, raw, rf.parameterEnergies, perr)) {
        if (!raw.empty()) lastCount = (int)raw.back().size();
    } else if (perr.rfind("cannot open", 0) != 0) {
        err = perr;  // present but malformed
        return false;
    }
    rf.numberOfUniqueParameters = std::max(rf.numberOfParameters, lastCount);
    if (!extractedMinPath.empty()) {
        if (!loadExtractedMin(extractedMinPath, rf.numberOfUniqueParameters, raw, err)) return false;
        lastCount = rf.numberOfUniqueParameters;
        rf.parameterEnergies.assign(raw.size(), std::nan(""));
    }
    rf.parameterSets.clear();
    for (const auto &set : raw) {
        std::vector<double> x((size_t)rf.numberOfParameters, 0.0);
        for (int p = 0; p < rf.numberOfParameters; ++p)
            if (p < lastCount && (size_t)p < set.size()) x[(size_t)p] = set[(size_t)p];
        rf.parameterSets.push_back(std::move(x));
    }
    return true;
}

bool loadRunFiles(const std::string &prefix, bool extractedMin, RunFiles &rf, std::string &err)
{
    rf = RunFiles();
    if (!readCsvState(prefix + "_Initial.dat", rf.numberOfQubits, rf.initialIndex, rf.initialCoeff, err)) return false;
    if (!loadOperators(prefix + "_Operators.dat", rf.operators, err)) return false;
    if (!loadParameters(prefix + "_Order.dat", prefix + "_Parameters.dat", rf.operators.size(),
                        extractedMin ? prefix + "_extractedmin" : std::string(), rf, err))
        return false;
    rf.haveNuclearEnergy = LoadNuclearEnergy(rf.nuclearEnergy, prefix);
    return true;
}

bool storeRunFiles(stateAnsatzManager &m, const RunFiles &rf, const std::string &prefix, std::string &err)
{
    bool complexState = false;
    for (const auto &c : rf.initialCoeff) complexState = complexState || c.imag() != 0.0;
    bool ok = complexState ? m.storeInitial(rf.numberOfQubits, rf.initialIndex, rf.initialCoeff) : [&] {
        std::vector<double> re;
        for (const auto &c : rf.initialCoeff) re.push_back(c.real());
        return m.storeInitial(rf.numberOfQubits, rf.initialIndex, re);
    }();
    if (!ok) { err = "the initial state was refused"; return false; }
    if (!m.storeOperators(rf.operators)) { err = "the operators were refused"; return false; }
    if (!m.storeParameterDependencies(rf.orders)) { err = "the parameter dependencies were refused"; return false; }
    if (rf.haveNuclearEnergy && !m.storeNuclearEnergy(rf.nuclearEnergy)) { err = "the nuclear energy was refused"; return false; }
    if (!m.storeRunPath(prefix)) { err = "the run path was refused"; return false; }
    return true;
}

}  // namespace ae

struct aegpu_run_files {
    ae::RunFiles rf;
};

static thread_local std::string g_run_files_error;

extern "C" {

int aegpu_run_files_load(const char *prefix, int extracted_min, aegpu_run_files **out)
{
    if (!prefix || !*prefix || !out) { g_run_files_error = "null or empty argument"; return 2; }
    *out = nullptr;
    auto *f = new aegpu_run_files();
    if (!ae::loadRunFiles(prefix, extracted_min != 0, f->rf, g_run_files_error)) {
        delete f;
        return 3;
    }
    g_run_files_error.clear();
    *out = f;
    return 0;
}

int aegpu_run_file_read(const char *path, int kind, aegpu_run_files **out)
{
    if (!path || !*path || !out || kind < AEGPU_RUN_FILE_INITIAL || kind > AEGPU_RUN_FILE_NUCLEAR) {
        g_run_files_error = "null, empty or unknown argument";
        return 2;
    }
    *out = nullptr;
    auto *f = new aegpu_run_files();
    bool ok = true;
    if (kind == AEGPU_RUN_FILE_INITIAL)
        ok = ae::readCsvState(path, f->rf.numberOfQubits, f->rf.initialIndex, f->rf.initialCoeff, g_run_files_error);
    else if (kind == AEGPU_RUN_FILE_OPERATORS)
        ok = ae::loadOperators(path, f->rf.operators, g_run_files_error);
    else
        f->rf.haveNuclearEnergy = ae::LoadNuclearEnergy(f->rf.nuclearEnergy, path);
    if (!ok) {
        delete f;
        return 3;
    }
    g_run_files_error.clear();
    *out = f;
    return 0;
}

int aegpu_run_files_parameters(const char *order_path, const char *parameter_path, int n_ops, aegpu_run_files **out)
{
    if (!order_path || !*order_path || !parameter_path || n_ops < 0 || !out) {
        g_run_files_error = "null or empty argument";
        return 2;
    }
    *out = nullptr;
    auto *f = new aegpu_run_files();
    if (!ae::loadParameters(order_path, parameter_path, (size_t)n_ops, std::string(), f->rf, g_run_files_error)) {
        delete f;
        return 3;
    }
    g_run_files_error.clear();
    *out = f;
    return 0;
}

const char *aegpu_run_files_error(void) { return g_run_files_error.c_str(); }

int aegpu_run_files_sizes(const aegpu_run_files *f, int *nq, int *n_initial, int *n_ops, int *n_params,
                          int *n_unique, int *n_sets)
{
    if (!f) return 2;
    if (nq) *nq = f->rf.numberOfQubits;
    if (n_initial) *n_initial = (int)f->rf.initialIndex.size();
    if (n_ops) *n_ops = (int)std::max(f->rf.operators.size(), f->rf.orders.size());
    if (n_params) *n_params = f->rf.numberOfParameters;
    if (n_unique) *n_unique = f->rf.numberOfUniqueParameters;
    if (n_sets) *n_sets = (int)f->rf.parameterSets.size();
    return 0;
}

int aegpu_run_files_get(const aegpu_run_files *f, int *initial_index, double *initial_coeff, int *operators_1b,
                        int *order_1b, double *scale, double *sets, double *energies, double *nuclear)
{
    if (!f) return 2;
    const ae::RunFiles &rf = f->rf;
    for (size_t i = 0; i < rf.initialIndex.size(); ++i) {
        if (initial_index) initial_index[i] = rf.initialIndex[i];
        if (initial_coeff) {
            initial_coeff[2 * i] = rf.initialCoeff[i].real();
            initial_coeff[2 * i + 1] = rf.initialCoeff[i].imag();
        }
    }
    // a handle holds operators, orders or both (a single file read fills one of them)
    for (size_t i = 0; i < rf.operators.size(); ++i) {
        const ae::Exc4 &e = rf.operators[i];
        if (operators_1b) {
            operators_1b[4 * i] = e.first + 1;
            operators_1b[4 * i + 1] = e.second + 1;
            operators_1b[4 * i + 2] = e.third + 1;
            operators_1b[4 * i + 3] = e.fourth + 1;
        }
    }
    for (size_t i = 0; i < rf.orders.size(); ++i) {
        if (order_1b) order_1b[i] = rf.orders[i].first + 1;
        if (scale) scale[i] = rf.orders[i].second;
    }
    const size_t P = (size_t)rf.numberOfParameters;
    for (size_t s = 0; s < rf.parameterSets.size(); ++s) {
        if (sets) std::copy(rf.parameterSets[s].begin(), rf.parameterSets[s].end(), sets + s * P);
        if (energies) energies[s] = rf.parameterEnergies[s];
    }
    if (nuclear) *nuclear = rf.haveNuclearEnergy ? rf.nuclearEnergy : std::nan("");
    return 0;
}

void aegpu_run_files_free(aegpu_run_files *f) { delete f; }

}  // extern "C"
