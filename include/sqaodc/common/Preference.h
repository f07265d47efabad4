// Preference.h -- solver preferences of the sqaod C++ solver API
// (enums and tagged union of sqaodc/common/Preference.h:8-63; string forms
// of sqaodc/common/Preference.cpp:20-78).
#pragma once

#include <sqaodc/common/Array.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

namespace sqaod {

enum Algorithm {
    algoUnknown,
    algoDefault,
    algoNaive,
    algoColoring,
    algoBruteForceSearch,
    algoSADefault,
    algoSANaive,
    algoSAColoring,
};

bool isSQAAlgorithm(Algorithm algo);
const char *algorithmToString(Algorithm algo);
Algorithm algorithmFromString(const char *algoStr);

enum PreferenceName {
    pnUnknown = 0,
    pnAlgorithm = 1,
    pnNumTrotters = 2,
    pnTileSize = 3,
    pnTileSize0 = 4,
    pnTileSize1 = 5,
    pnPrecision = 6,
    pnDevice = 7,
    pnExperiment = 100,
};

PreferenceName preferenceNameFromString(const char *name);
const char *preferenceNameToString(PreferenceName pn);

struct Preference {
    Preference(PreferenceName n, SizeType s) : name(n), size(s) {}
    Preference(PreferenceName n, Algorithm a) : name(n), algo(a) {}
    Preference(PreferenceName n, const char *s) : name(n), str(s) {}
    Preference() : name(pnUnknown), size(0) {}

    PreferenceName name;
    union {
        SizeType size;
        const char *str;
        Algorithm algo;
        SizeType tileSize;
        SizeType nTrotters;
        const char *precision;
        const char *device;
        int experiment;
    };
};

typedef ArrayType<Preference> Preferences;

}  // namespace sqaod

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
