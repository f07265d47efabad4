// Solver.h -- abstract solver interfaces of the sqaod C++ solver API.
//
// Same class hierarchy, virtual methods and solver-state rules as
// sqaodc/common/Solver.h:17-252 / Solver.cpp:32-218 of the reference:
// Solver -> {Annealer, BFSearcher} x {DenseGraphSolver, BipartiteGraphSolver}.
#pragma once

#include <sqaodc/common/Matrix.h>
#include <sqaodc/common/Preference.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

namespace sqaod {

enum OptimizeMethod {
    optNone = -1,
    optMinimize = 0,
    optMaximize = 1,
};

void deleteInstance(NullBase *instance);

template <class real>
struct Solver : NullBase {
    virtual ~Solver() {}

    virtual Algorithm selectAlgorithm(Algorithm algo) = 0;
    virtual Algorithm getAlgorithm() const = 0;
    virtual Preferences getPreferences() const = 0;
    virtual void setPreference(const Preference &pref) = 0;

    template <class V>
    void setPreference(PreferenceName name, const V value) {
        Preference pref(name, value);
        setPreference(pref);
    }
    void setPreferences(const Preferences &prefs) {
        for (SizeType i = 0; i < prefs.size(); ++i) setPreference(prefs[i]);
    }

    virtual const VectorType<real> &get_E() const = 0;
    virtual void prepare() = 0;
    virtual void calculate_E() = 0;
    virtual void makeSolution() = 0;

protected:
    Solver() : solverState_(solNone), om_(optNone) {}

    int solverState_;
    enum SolverState {
        solNone = 0,
        solProblemSet = 1,
        solPrepared = 2,
        solEAvailable = 4,
        solSolutionAvailable = 8,
        solRandSeedGiven = 16,
        solQSet = 32,
    };

    void setState(SolverState state);
    void clearState(SolverState state);
    bool isRandSeedGiven() const { return (solverState_ & solRandSeedGiven) != 0; }
    bool isProblemSet() const { return (solverState_ & solProblemSet) != 0; }
    bool isPrepared() const { return (solverState_ & solPrepared) != 0; }
    bool isQSet() const { return (solverState_ & solQSet) != 0; }
    bool isEAvailable() const { return (solverState_ & solEAvailable) != 0; }
    bool isSolutionAvailable() const { return (solverState_ & solSolutionAvailable) != 0; }
    void throwErrorIfProblemNotSet() const;
    void throwErrorIfNotPrepared() const;
    void throwErrorIfQNotSet() const;

    OptimizeMethod om_;
};

template <class real>
struct BFSearcher : Solver<real> {
    virtual ~BFSearcher() {}
    virtual Algorithm selectAlgorithm(Algorithm) { return algoBruteForceSearch; }
    virtual Algorithm getAlgorithm() const { return algoBruteForceSearch; }
    virtual void search() = 0;

protected:
    BFSearcher() {}
};

template <class real>
struct Annealer : Solver<real> {
    virtual ~Annealer() {}

    virtual Algorithm getAlgorithm() const { return algo_; }
    virtual Preferences getPreferences() const;
    virtual void setPreference(const Preference &pref);
    using Solver<real>::setPreference;

    virtual void seed(unsigned long long seed) = 0;
    virtual void randomizeSpin() = 0;
    virtual void annealOneStep(real G, real beta) = 0;
    virtual real getSystemE(real G, real beta) const = 0;
    // prepare() + randomizeSpin()
    virtual void initAnneal() {
        this->prepare();
        this->randomizeSpin();
    }

protected:
    Annealer() : algo_(algoDefault), m_(0) {}
    Algorithm algo_;
    void selectDefaultAlgorithm(Algorithm algoOrg, Algorithm algoDef, Algorithm algoSADef);
    void selectDefaultSAAlgorithm(Algorithm algoOrg, Algorithm algoSADef);
    SizeType m_;
};

template <class real>
struct DenseGraphSolver {
    virtual ~DenseGraphSolver() {}
    void getProblemSize(SizeType *N) const { *N = N_; }
    virtual void setQUBO(const MatrixType<real> &W, OptimizeMethod om = optMinimize) = 0;
    virtual const BitSetArray &get_x() const = 0;

protected:
    DenseGraphSolver() : N_(0) {}
    SizeType N_;
};

template <class real>
struct BipartiteGraphSolver {
    virtual ~BipartiteGraphSolver() {}
    void getProblemSize(SizeType *N0, SizeType *N1) const {
        *N0 = N0_;
        *N1 = N1_;
    }
    virtual void setQUBO(const VectorType<real> &b0, const VectorType<real> &b1, const MatrixType<real> &W,
                         OptimizeMethod om = optMinimize) = 0;
    virtual const BitSetPairArray &get_x() const = 0;

protected:
    BipartiteGraphSolver() : N0_(0), N1_(0) {}
    SizeType N0_, N1_;
};

template <class real>
struct DenseGraphBFSearcher : BFSearcher<real>, DenseGraphSolver<real> {
    virtual ~DenseGraphBFSearcher() {}
    virtual Preferences getPreferences() const;
    virtual void setPreference(const Preference &pref);
    using Solver<real>::setPreference;
    virtual bool searchRange(PackedBitSet *curXEnd) = 0;
    virtual void search() {
        this->prepare();
        while (!searchRange(nullptr)) {
        }
        this->makeSolution();
    }

protected:
    DenseGraphBFSearcher() : x_(0), xMax_(0), tileSize_(0) {}
    PackedBitSet x_, xMax_;
    SizeType tileSize_;
};

template <class real>
struct DenseGraphAnnealer : Annealer<real>, DenseGraphSolver<real> {
    virtual ~DenseGraphAnnealer() {}
    virtual void setHamiltonian(const VectorType<real> &h, const MatrixType<real> &J, real c = real(0.)) = 0;
    virtual void getHamiltonian(VectorType<real> *h, MatrixType<real> *J, real *c) const = 0;
    virtual void set_q(const BitSet &q) = 0;
    virtual void set_qset(const BitSetArray &q) = 0;
    virtual const BitSetArray &get_q() const = 0;

protected:
    DenseGraphAnnealer() {}
};

template <class real>
struct BipartiteGraphBFSearcher : BFSearcher<real>, BipartiteGraphSolver<real> {
    virtual ~BipartiteGraphBFSearcher() {}
    virtual Preferences getPreferences() const;
    virtual void setPreference(const Preference &pref);
    using Solver<real>::setPreference;
    virtual bool searchRange(PackedBitSet *curX0End, PackedBitSet *curX1End) = 0;
    virtual void search() {
        this->prepare();
        while (!searchRange(nullptr, nullptr)) {
        }
        this->makeSolution();
    }

protected:
    BipartiteGraphBFSearcher() : x0_(0), x1_(0), x0max_(0), x1max_(0), tileSize0_(0), tileSize1_(0) {}
    PackedBitSet x0_, x1_, x0max_, x1max_;
    SizeType tileSize0_, tileSize1_;
};

template <class real>
struct BipartiteGraphAnnealer : Annealer<real>, BipartiteGraphSolver<real> {
    virtual ~BipartiteGraphAnnealer() {}
    virtual void setHamiltonian(const VectorType<real> &h0, const VectorType<real> &h1, const MatrixType<real> &J,
                                real c = real(0.)) = 0;
    virtual void getHamiltonian(VectorType<real> *h0, VectorType<real> *h1, MatrixType<real> *J,
                                real *c) const = 0;
    virtual void set_q(const BitSetPair &qPair) = 0;
    virtual void set_qset(const BitSetPairArray &qPairs) = 0;
    virtual const BitSetPairArray &get_q() const = 0;

protected:
    BipartiteGraphAnnealer() {}
};

}  // namespace sqaod

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
