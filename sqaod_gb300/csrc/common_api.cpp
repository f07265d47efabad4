// common_api.cpp -- host-side pieces of the sqaod C++ solver API: preference
// strings (sqaodc/common/Preference.cpp:20-78), the solver state machine and
// algorithm defaulting (sqaodc/common/Solver.cpp:32-218), bit-set helpers
// (sqaodc/common/Common.cpp:79-145) and error reporting
// (sqaodc/common/defines.cpp:32-63).
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <strings.h>

#include <string>

#include <sqaodc/common/Common.h>

namespace sqaod {

bool isSQAAlgorithm(Algorithm algo) { return algo == algoNaive || algo == algoColoring; }

const char *algorithmToString(Algorithm algo) {
    switch (algo) {
    case algoNaive: return "naive";
    case algoColoring: return "coloring";
    case algoBruteForceSearch: return "brute_force_search";
    case algoSADefault: return "sa_default";
    case algoSANaive: return "sa_naive";
    case algoSAColoring: return "sa_coloring";
    case algoDefault: return "default";
    default: return "unknown";
    }
}

Algorithm algorithmFromString(const char *s) {
    static const struct { const char *name; Algorithm algo; } table[] = {
        {"naive", algoNaive}, {"coloring", algoColoring}, {"brute_force_search", algoBruteForceSearch},
        {"sa_default", algoSADefault}, {"sa_naive", algoSANaive}, {"sa_coloring", algoSAColoring},
        {"default", algoDefault}};
    for (const auto &e : table)
        if (strcasecmp(e.name, s) == 0) return e.algo;
    return algoUnknown;
}

PreferenceName preferenceNameFromString(const char *s) {
    static const struct { const char *name; PreferenceName pn; } table[] = {
        {"algorithm", pnAlgorithm}, {"n_trotters", pnNumTrotters}, {"tile_size", pnTileSize},
        {"tile_size_0", pnTileSize0}, {"tile_size_1", pnTileSize1}, {"precision", pnPrecision},
        {"device", pnDevice}, {"experiment", pnExperiment}};
    for (const auto &e : table)
        if (strcasecmp(e.name, s) == 0) return e.pn;
    return pnUnknown;
}

const char *preferenceNameToString(PreferenceName pn) {
    switch (pn) {
    case pnAlgorithm: return "algorithm";
    case pnNumTrotters: return "n_trotters";
    case pnTileSize: return "tile_size";
    case pnTileSize0: return "tile_size_0";
    case pnTileSize1: return "tile_size_1";
    case pnPrecision: return "precision";
    case pnDevice: return "device";
    case pnExperiment: return "experiment";
    default: return "unknown";
    }
}

void deleteInstance(NullBase *instance) { delete instance; }

void throwError(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw std::runtime_error(buf);
}

void log(const char *fmt, ...) {
    if (!getenv("SQAOD_VERBOSE")) return;
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
    fputc('\n', stderr);
}

void unpackBitSet(BitSet *unpacked, PackedBitSet packed, int N) {
    unpacked->resize(N);
    for (int pos = 0; pos < N; ++pos) (*unpacked)(pos) = (char)((packed >> (N - 1 - pos)) & 1);
}

BitSet x_from_q(const BitSet &q) {
    BitSet x(q.size);
    // spins are read as signed bytes: plain char is unsigned on some targets
    // (aarch64), where -1 would otherwise read as 255
    for (SizeType i = 0; i < q.size; ++i) x(i) = (char)(((int)(signed char)q(i) + 1) / 2);
    return x;
}

// ---------------------------------------------------------- state machine
// Clearing a state also clears the states that depend on it (Solver.cpp:44-68).
template <class real>
void Solver<real>::clearState(SolverState state) {
    int clear = 0;
    switch (state) {
    case solRandSeedGiven:
        clear = solRandSeedGiven;
        break;
    case solProblemSet:
        clear |= solProblemSet;  // fall through
    case solPrepared:
        clear |= solPrepared;  // fall through
    case solQSet:
        clear |= solQSet;  // fall through
    case solEAvailable:
    case solSolutionAvailable:
        clear |= solEAvailable | solSolutionAvailable;
        break;
    default:
        break;
    }
    solverState_ &= ~clear;
}

template <class real>
void Solver<real>::setState(SolverState state) {
    clearState(state);
    solverState_ |= state;
}

template <class real>
void Solver<real>::throwErrorIfProblemNotSet() const {
    throwErrorIf(!isProblemSet(), "Problem is not set.");
}

template <class real>
void Solver<real>::throwErrorIfNotPrepared() const {
    throwErrorIfProblemNotSet();
    throwErrorIf(!isPrepared(), "not prepared, call prepare() in advance.");
}

template <class real>
void Solver<real>::throwErrorIfQNotSet() const {
    throwErrorIf(!isQSet(), "Bits(x or q) not initialized.  Plase set or randomize in advance.");
}

template <class real>
static const char *typeString();
template <>
const char *typeString<float>() { return "float"; }
template <>
const char *typeString<double>() { return "double"; }

template <class real>
Preferences Annealer<real>::getPreferences() const {
    Preferences prefs;
    prefs.pushBack(Preference(pnAlgorithm, this->getAlgorithm()));
    prefs.pushBack(Preference(pnNumTrotters, m_));
    prefs.pushBack(Preference(pnPrecision, typeString<real>()));
    return prefs;
}

template <class real>
void Annealer<real>::setPreference(const Preference &pref) {
    if (pref.name == pnNumTrotters) {
        throwErrorIf(pref.nTrotters <= 0, "# trotters must be a positive integer.");
        if (m_ != pref.nTrotters) Solver<real>::clearState(Solver<real>::solPrepared);
        m_ = pref.nTrotters;
    } else if (pref.name == pnAlgorithm) {
        this->selectAlgorithm(pref.algo);
    }
}

template <class real>
void Annealer<real>::selectDefaultAlgorithm(Algorithm algoOrg, Algorithm algoDef, Algorithm algoSADef) {
    if (algoOrg == algoDefault) {
        algo_ = algoDef;
    } else if (algoOrg == algoSADefault) {
        algo_ = algoSADef;
    } else {
        algo_ = isSQAAlgorithm(algoOrg) ? algoDef : algoSADef;
        log("%s is not supported, selecting the default algorithm of %s.", algorithmToString(algoOrg),
            algorithmToString(algo_));
    }
}

template <class real>
void Annealer<real>::selectDefaultSAAlgorithm(Algorithm algoOrg, Algorithm algoSADef) {
    if (algoOrg != algoSADef) {
        algo_ = algoSADef;
        log("Selecting %s as the default SA algorithm.", algorithmToString(algo_));
    }
}

template <class real>
Preferences DenseGraphBFSearcher<real>::getPreferences() const {
    Preferences prefs;
    prefs.pushBack(Preference(pnAlgorithm, algoBruteForceSearch));
    prefs.pushBack(Preference(pnTileSize, tileSize_));
    prefs.pushBack(Preference(pnPrecision, typeString<real>()));
    return prefs;
}

template <class real>
void DenseGraphBFSearcher<real>::setPreference(const Preference &pref) {
    if (pref.name == pnTileSize) {
        throwErrorIf(pref.tileSize <= 0, "tileSize must be a positive integer.");
        tileSize_ = roundUp(pref.tileSize, 256);
    }
}

template <class real>
Preferences BipartiteGraphBFSearcher<real>::getPreferences() const {
    Preferences prefs;
    prefs.pushBack(Preference(pnAlgorithm, algoBruteForceSearch));
    prefs.pushBack(Preference(pnTileSize0, tileSize0_));
    prefs.pushBack(Preference(pnTileSize1, tileSize1_));
    prefs.pushBack(Preference(pnPrecision, typeString<real>()));
    return prefs;
}

template <class real>
void BipartiteGraphBFSearcher<real>::setPreference(const Preference &pref) {
    if (pref.name == pnTileSize0) {
        throwErrorIf(pref.tileSize <= 0, "tileSize0 must be a positive integer.");
        tileSize0_ = roundUp(pref.tileSize, 256);
    }
    if (pref.name == pnTileSize1) {
        throwErrorIf(pref.tileSize <= 0, "tileSize1 must be a positive integer.");
        tileSize1_ = roundUp(pref.tileSize, 256);
    }
}

template struct Solver<float>;
template struct Annealer<float>;
template struct DenseGraphBFSearcher<float>;
template struct BipartiteGraphBFSearcher<float>;
template struct Solver<double>;
template struct DenseGraphBFSearcher<double>;
template struct BipartiteGraphBFSearcher<double>;

}  // namespace sqaod
