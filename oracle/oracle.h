/*
 * oracle.h -- CPU oracle for the sqaod annealing / brute-force-search hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; it is used by tests/, by __graft_entry__.smoke() and by the
 * cpu_baseline / reference legs of bench.py, always as the checker or as the
 * timed CPU baseline, never as the thing that is measured or shipped.
 *
 * Contents (each function cites the reference file:line it restates; paths are
 * relative to the shinmorino/sqaod source tree):
 *   - MT19937 (the generator behind sqaod::Random, sqaodc/common/Random.cpp:70-168)
 *   - Philox4x32-10 (Salmon et al., SC'11), the counter RNG the GPU build uses
 *   - the reference dot product in the AVX2 lane order (sqaodc/cpu/Dot_SIMD.cpp:160-210)
 *   - FP64 formulas: QUBO->Ising (h, J, c) and energies
 *     (sqaodc/cpu/SharedFormulas.cpp:10-202, sqaodpy/sqaod/py/formulas.py)
 *   - the reference CPU annealers (sqaodc/cpu/CPUDenseGraphAnnealer.cpp:251-371,
 *     sqaodc/cpu/CPUBipartiteGraphAnnealer.cpp:288-542) with their MT19937 streams
 *   - the reference CPU brute-force searchers (sqaodc/cpu/CPUDenseGraphBFSearcher.cpp,
 *     CPUDenseGraphBatchSearch.cpp, CPUBipartiteGraphBFSearcher.cpp,
 *     CPUBipartiteGraphBatchSearch.cpp)
 *   - an FP64 replay of the GPU build's own sweeps over the same Philox stream.
 *
 * Parity pins: MT19937 and the AVX2-order dot are checked against the
 * reference's own Random.cpp / Dot_SIMD.cpp compiled from source (oracle/_ref,
 * built by oracle/build.py); formulas and BF results are checked against
 * golden vectors generated from the reference's numpy backend
 * (tests/golden/make_golden.py) and against the reference tests' known answers.
 */
#ifndef SQAOD_GB300_ORACLE_H
#define SQAOD_GB300_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- RNGs */

/* Philox4x32-10: out = philox(ctr, key). */
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

typedef struct orc_mt {
    uint32_t mt[624];
    int mti;
} orc_mt;

void orc_mt_seed(orc_mt *r, unsigned long long s);
uint32_t orc_mt_u32(orc_mt *r);
uint32_t orc_mt_randint(orc_mt *r, int n);
float orc_mt_f32(orc_mt *r);
double orc_mt_f64(orc_mt *r);
/* fill out[n] with the first n words after seeding with s (test helper) */
void orc_mt_stream(unsigned long long s, int n, uint32_t *out);

/* Reference dot product, AVX2 lane order.  Reads roundUp(N, 16) elements of
 * both vectors: the caller zero-pads them, as sqaod's 64-byte-aligned rows are. */
float orc_dot_ref(const float *v0, const float *v1, int N);

/* ------------------------------------------------------------ formulas */

void orc_dg_hamiltonian(const double *W, int N, double *h, double *J, double *c);
void orc_dg_energy_qubo(const double *W, int N, const int8_t *x, int n, double *E);
void orc_dg_energy_ising(const double *h, const double *J, double c, int N,
                         const int8_t *q, int m, double *E);
void orc_bg_hamiltonian(const double *b0, const double *b1, const double *W, int N0, int N1,
                        double *h0, double *h1, double *J, double *c);
void orc_bg_energy_qubo(const double *b0, const double *b1, const double *W, int N0, int N1,
                        const int8_t *x0, const int8_t *x1, int n, double *E);
void orc_bg_energy_ising(const double *h0, const double *h1, const double *J, double c,
                         int N0, int N1, const int8_t *q0, const int8_t *q1, int m, double *E);
void orc_bg_energy_qubo_2d(const double *b0, const double *b1, const double *W, int N0, int N1,
                           const int8_t *x0, int n0, const int8_t *x1, int n1, double *E);

/* ------------------------------------------------------ BF searchers */

/* Dense BF search with the reference CPU semantics: nWorkers OpenMP workers,
 * each sweeping its own tileSize tile per round, ties appended while the
 * worker's list is shorter than tileSize, strict '<' resets; the merge takes
 * strict '<' or unions '==' while shorter than tileSize, sorts ascending and
 * truncates to tileSize.  Energies are evaluated in FP64 and rounded to fp32
 * (exact for integer-valued W).  Returns the number of solutions written to
 * xout (capacity cap); *Emin gets the (sign-corrected) minimum. */
int orc_dg_bf_search_ref(const float *W, int N, int om, int tileSize, int nWorkers,
                         float *Emin, uint64_t *xout, int cap);
/* Dense BF over [xBegin, xEnd) only, first `cap` minimisers in ascending order. */
int orc_dg_bf_search_range(const float *W, int N, int om, uint64_t xBegin, uint64_t xEnd,
                           int cap, float *Emin, uint64_t *xout);
/* Exact dense BF for integer-valued symmetric W (|sum W| < 2^30): every state
 * in Gray-code order with integer local fields, so one state costs N integer
 * adds and N = 32 finishes in seconds on a few cores.  For integer W the
 * reference CPU searcher's fp32 energies are exact, so its result is the
 * smallest min(count, tileSize) minimisers ascending: this returns the first
 * `cap` of all minimisers ascending (Emin sign-corrected), *nMin = how many
 * exist.  Returns the number written, -2 for bad N, -3 for non-integer,
 * asymmetric or too large W, -4 when a worker's list overflowed. */
int orc_dg_bf_search_exact_int(const float *W, int N, int om, int cap, int nWorkers,
                               double *Emin, uint64_t *xout, long long *nMin);
/* Bipartite BF with the reference CPU semantics (tile0 x tile1 tiles, up to
 * N0+N1 solutions, no sort).  xout holds (x0, x1) pairs. */
int orc_bg_bf_search_ref(const float *b0, const float *b1, const float *W, int N0, int N1,
                         int om, int tileSize0, int tileSize1, int nWorkers,
                         float *Emin, uint64_t *xout, int cap);
/* Bipartite BF, all minimising pairs in (x0-major, x1-minor) ascending order, first cap. */
int orc_bg_bf_search_sorted(const float *b0, const float *b1, const float *W, int N0, int N1,
                            int om, int cap, float *Emin, uint64_t *xout);

/* Throughput helper for the CPU baseline: sweeps nTiles tiles of tileSize
 * states starting at xBegin with nWorkers threads using the reference's
 * per-tile formulation (X*W, row-wise dot, scan).  Returns the minimum found. */
float orc_dg_bf_sweep_tiles(const float *W, int N, uint64_t xBegin, int tileSize, int nTiles,
                            int nWorkers);

/* ------------------------------------------- reference CPU annealers */

enum { ORC_ALGO_NAIVE = 0, ORC_ALGO_COLORING = 1, ORC_ALGO_SA_NAIVE = 2, ORC_ALGO_SA_COLORING = 3 };

typedef struct orc_dga orc_dga;
orc_dga *orc_dga_new(int N, int m, int nWorkers);
void orc_dga_free(orc_dga *a);
int orc_dga_workers(const orc_dga *a);
void orc_dga_set_hamiltonian(orc_dga *a, const float *h, const float *J, float c);
void orc_dga_seed(orc_dga *a, unsigned long long seed);
void orc_dga_randomize(orc_dga *a);
void orc_dga_set_q(orc_dga *a, const int8_t *q);
void orc_dga_get_q(const orc_dga *a, int8_t *q);
void orc_dga_step(orc_dga *a, int algo, float G, float beta);
void orc_dga_energy(const orc_dga *a, double *E);

typedef struct orc_bga orc_bga;
orc_bga *orc_bga_new(int N0, int N1, int m, int nWorkers);
void orc_bga_free(orc_bga *a);
int orc_bga_workers(const orc_bga *a);
void orc_bga_set_hamiltonian(orc_bga *a, const float *h0, const float *h1, const float *J, float c);
void orc_bga_seed(orc_bga *a, unsigned long long seed);
void orc_bga_randomize(orc_bga *a);
void orc_bga_set_q(orc_bga *a, const int8_t *q0, const int8_t *q1);
void orc_bga_get_q(const orc_bga *a, int8_t *q0, int8_t *q1);
void orc_bga_step(orc_bga *a, int algo, float G, float beta);
void orc_bga_energy(const orc_bga *a, double *E);

/* ------------------------------ FP64 replay of the GPU build's sweeps */

/* Philox stream tags (counter word 3).  The GPU build draws every random
 * number as philox((c0, c1, step, tag | side << 8), (seed_lo, seed_hi)). */
enum {
    ORC_TAG_DSWEEP = 0x11,   /* dense coloring: c0 = iteration k, c1 = trotter y */
    ORC_TAG_DSA = 0x12,      /* dense SA: c0 = iteration k, c1 = trotter y */
    ORC_TAG_DNAIVE = 0x13,   /* dense naive: c0 = trial t */
    ORC_TAG_RAND = 0x21,     /* randomizeSpin: c0 = 128-spin chunk, c1 = trotter */
    ORC_TAG_BSWEEP = 0x31,   /* bipartite coloring: c0 = spin, c1 = trotter */
    ORC_TAG_BSA = 0x32,      /* bipartite SA coloring */
    ORC_TAG_BNAIVE = 0x33,   /* bipartite naive: c0 = trial */
    ORC_TAG_BSANAIVE = 0x34, /* bipartite SA naive: c0 = trial, c1 = trotter */
};

/* randomizeSpin of the GPU build: q[y][j] from the Philox stream */
void orc_gpu_randomize(uint64_t seed, uint32_t step, int tagSide, int m, int N, int8_t *q);

typedef struct orc_replay_stats {
    long long n_trials;
    long long n_accept;         /* device-accepted flips */
    long long n_mismatch;       /* FP64 decision != device decision */
    long long n_mismatch_small; /* ... of which the FP64 margin is below tol */
    long long n_small_margin;   /* trials with FP64 margin below tol */
    double max_mismatch_margin;
} orc_replay_stats;

/* Replays one annealOneStep of the dense GPU sweep (algo: naive / coloring /
 * sa_naive) in FP64 from q (m x N, in/out), following the device trace
 * (accept bits, see the layout in oracle.c) and comparing every decision. */
void orc_dg_replay(const float *h, const float *J, int N, int m, int algo,
                   uint64_t seed, uint32_t step, float G, float beta,
                   int8_t *q, const uint32_t *trace, double tol, orc_replay_stats *st);
/* nSteps consecutive steps (counters step0 + s, G[s], beta[s], trace of step s
 * at trace + s * ceil(N m / 32)) with resident FP64 fields: the same decisions
 * as orc_dg_replay at a cost that makes N = 4096, m = 256 replayable.  h and J
 * are FP64 (the fp32 couplings of a float problem convert exactly); J must be
 * symmetric with a zero diagonal. */
void orc_dg_replay_steps(const double *h, const double *J, int N, int m, int algo, uint64_t seed,
                         uint32_t step0, int nSteps, const float *G, const float *beta, int8_t *q,
                         const uint32_t *trace, double tol, orc_replay_stats *st);
/* Same for the bipartite sweeps (algo: naive / coloring / sa_naive / sa_coloring),
 * with FP64 h0, h1, J. */
void orc_bg_replay(const double *h0, const double *h1, const double *J, int N0, int N1, int m,
                   int algo, uint64_t seed, uint32_t step, float G, float beta,
                   int8_t *q0, int8_t *q1, const uint32_t *trace, double tol,
                   orc_replay_stats *st);

#ifdef __cplusplus
}
#endif

#endif
