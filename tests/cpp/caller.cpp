// caller.cpp -- a C++ caller of the reference's solver API, in the shape of
// sqaodc/tests/perf.cpp:87-112: it includes only <sqaodc/sqaodc.h>, links
// libsqaod_gb300.so, creates the solvers through the sqaod::cuda factories,
// anneals / searches, and prints one JSON line per solver with its minimum
// energy and the bits of its best solution (checked against FP64 by
// tests/test_gpu_cpp_caller.py).
//
//   caller <N> <m> <seed>
#include <sqaodc/sqaodc.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>

namespace sq = sqaod;

template <class real>
static sq::MatrixType<real> symmetric_W(int N, unsigned seed) {
    std::mt19937 gen(seed);
    std::uniform_real_distribution<double> U(-1., 1.);
    sq::MatrixType<real> W(N, N);
    for (int i = 0; i < N; ++i)
        for (int j = i; j < N; ++j) W(i, j) = W(j, i) = (real)U(gen);
    return W;
}

template <class real>
static std::string values(const sq::MatrixType<real> &W) {
    std::string s;
    char buf[40];
    for (int i = 0; i < W.rows; ++i)
        for (int j = 0; j < W.cols; ++j) {
            snprintf(buf, sizeof(buf), "%s%.17g", s.empty() ? "" : ", ", (double)W(i, j));
            s += buf;
        }
    return s;
}

template <class real>
static std::string bits(const sq::BitSet &x) {
    std::string s;
    for (int i = 0; i < x.size; ++i) s += x(i) ? '1' : '0';
    return s;
}

template <class real>
static void anneal(const char *name, int N, int m, unsigned seed) {
    sq::MatrixType<real> W = symmetric_W<real>(N, seed);
    sq::cuda::DenseGraphAnnealer<real> *ann = sq::cuda::newDenseGraphAnnealer<real>();
    sq::cuda::Device *dev = sq::cuda::newDevice(0);
    ann->assignDevice(*dev);
    ann->seed(seed);
    ann->setQUBO(W, sq::optMinimize);
    ann->setPreference(sq::Preference(sq::pnNumTrotters, m));
    ann->setPreference(sq::Preference(sq::pnAlgorithm, sq::algoColoring));
    ann->prepare();
    ann->randomizeSpin();
    for (real G = 5.; G > 0.01; G *= (real)0.97) ann->annealOneStep(G, (real)50.);
    ann->makeSolution();
    const sq::VectorType<real> &E = ann->get_E();
    const sq::BitSetArray &x = ann->get_x();
    int best = 0;
    for (int i = 1; i < E.size; ++i)
        if (E(i) < E(best)) best = i;
    sq::Preferences prefs = ann->getPreferences();
    const char *prec = "?";
    for (int i = 0; i < (int)prefs.size(); ++i)
        if (prefs[i].name == sq::pnPrecision) prec = prefs[i].precision;
    printf("{\"solver\": \"%s\", \"precision\": \"%s\", \"N\": %d, \"m\": %d, \"seed\": %u, \"E\": %.17g, "
           "\"x\": \"%s\", \"W\": [%s]}\n",
           name, prec, N, m, seed, (double)E(best), bits<real>(x[best]).c_str(), values(W).c_str());
    sq::deleteInstance(ann);
    delete dev;
}

template <class real>
static void search(const char *name, int N, unsigned seed) {
    std::mt19937 gen(seed);
    std::uniform_int_distribution<int> U(-8, 8);
    sq::MatrixType<real> W(N, N);
    for (int i = 0; i < N; ++i)
        for (int j = i; j < N; ++j) W(i, j) = W(j, i) = (real)U(gen);
    sq::cuda::DenseGraphBFSearcher<real> *bf = sq::cuda::newDenseGraphBFSearcher<real>();
    bf->setQUBO(W, sq::optMinimize);
    bf->search();
    const sq::VectorType<real> &E = bf->get_E();
    const sq::BitSetArray &x = bf->get_x();
    printf("{\"solver\": \"%s\", \"N\": %d, \"seed\": %u, \"E\": %.17g, \"n\": %d, \"x\": \"%s\", \"W\": [%s]}\n", name,
           N, seed, (double)E(0), (int)x.size(), bits<real>(x[0]).c_str(), values(W).c_str());
    sq::deleteInstance(bf);
}

int main(int argc, char **argv) {
    const int N = argc > 1 ? atoi(argv[1]) : 64;
    const int m = argc > 2 ? atoi(argv[2]) : 8;
    const unsigned seed = argc > 3 ? (unsigned)atoi(argv[3]) : 1;
    try {
        anneal<float>("dense_annealer", N, m, seed);
        anneal<double>("dense_annealer", N, m, seed);
        search<float>("dense_bf_searcher", 20, seed);
        search<double>("dense_bf_searcher", 20, seed);
    } catch (const std::exception &e) {
        fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
