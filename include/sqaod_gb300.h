/*
 * sqaod_gb300.h -- C ABI of the GB300-native sqaod annealing / brute-force
 * search hot path (libsqaod_gb300.so).
 *
 * Two layers, both plain C (pointers, sizes, status codes; no C++ or torch
 * types):
 *
 *  1. Solver-handle layer (sq103_dg_annealer_*, sq103_bg_annealer_*,
 *     sq103_dg_bf_*, sq103_bg_bf_*).  One entry point per method of the
 *     reference's CPython method tables, so a binding (ctypes, cffi, a CPython
 *     extension) maps one-to-one onto them:
 *       annealers:     sqaodc/pyglue/annealer.inc:885-908
 *       BF searchers:  sqaodc/pyglue/bf_searcher.inc:479-494
 *     behind which stand the C++ interfaces sqaod::cuda::DenseGraphAnnealer,
 *     BipartiteGraphAnnealer, DenseGraphBFSearcher, BipartiteGraphBFSearcher
 *     <float> (sqaodc/cuda/api.h:40-67, sqaodc/common/Solver.h:17-252); the
 *     same classes are exported as C++ through include/sqaodc/.
 *
 *  2. Kernel layer (sq103_dense_*, sq103_bipartite_*, sq103_bf_*): device
 *     pointers, a caller-supplied stream (void * = cudaStream_t), no
 *     allocation.  These replace the reference's device math
 *     (sqaodc/cuda/DeviceFormulas.cpp, DeviceMath.cpp, DeviceKernels.cu,
 *     DeviceDenseGraphBatchSearch.cu, DeviceBipartiteGraphBatchSearch.cu) and
 *     the per-step sweeps of CUDADenseGraphAnnealer.cu / CUDABipartiteGraphAnnealer.cu.
 *
 * Every function returns 0 on success.  Handle-layer functions return -1 on a
 * user error (the reference throws std::runtime_error there,
 * sqaodc/common/defines.h:43-46) with the message available from
 * sq103_last_error(); positive values are CUDA error codes or sq103 device
 * status codes (1 = a bounded device wait timed out, 2 = bad shape,
 * 3 = capacity exceeded).
 *
 * Layouts: matrices are row-major and dense (row stride = number of columns
 * unless an ld argument says otherwise); spins q are int8 {-1, +1}; bits x are
 * int8 {0, 1}; packed bit sets put variable i at bit (N - 1 - i) (MSB-first,
 * sqaodc/common/Common.cpp:79-93).  optimize: 0 = minimise, 1 = maximise
 * (sqaodc/common/Solver.h:10-15).
 */
#ifndef SQAOD_GB300_H
#define SQAOD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SQ103_API __attribute__((visibility("default")))
#else
#define SQ103_API
#endif

/* ------------------------------------------------------------ common */

/* message of the last failed handle-layer call on this thread */
SQ103_API const char *sq103_last_error(void);
/* library version (1.0.3 of the reference API: sqaodc/common/defines.h:80) */
SQ103_API int sq103_version(void);
/* makes CUDA device devNo current for the calling thread: the solvers created
 * and called on that thread run there (sqaod::cuda::Device + assignDevice,
 * sqaodc/cuda/api.h:16-37) */
SQ103_API int sq103_device_set(int devNo);

/* ------------------------------------------------ kernel layer: dense */

/* One dense annealing instance for the sweep kernels.  Replaces the state
 * the reference keeps in CUDADenseGraphAnnealer (sqaodc/cuda/CUDADenseGraphAnnealer.h). */
typedef struct sq103_dense_task {
    const float *J;       /* N x N Ising couplings, row stride ldJ, zero diagonal, symmetric */
    const float *h;       /* N */
    int8_t *q;            /* m x N spins, row stride N */
    float *F;             /* m x N local fields F[y][i] = sum_j J[i][j] q[y][j] */
    uint32_t *trace;      /* optional: accept bits, ceil(N m / 32) words per step; coloring and
                             sa_naive set bit k m + y for iteration k of trotter y, naive bit t
                             for trial t */
    unsigned long long *accepted; /* optional: accepted-flip counter (atomically added) */
    const float *G;       /* nSteps transverse fields (kT for SA), device memory; or NULL: use Gs */
    const float *beta;    /* nSteps inverse temperatures (ignored by SA); or NULL: use betas */
    float Gs, betas;      /* G and beta of every step when the arrays are NULL */
    int *status;          /* optional device status word (timeouts) */
    uint64_t seed;        /* Philox key */
    uint32_t step0;       /* Philox step counter of the first step */
    int N, m, ldJ;
    int algo;             /* 0 naive, 1 coloring, 2 sa_naive */
    int nSteps;
    void *ws;             /* optional device workspace for the multi-CTA sweep */
    unsigned long long wsBytes; /* its size; sq103_dense_ws_bytes(N, m, nSteps) */
    int flags;            /* bits 0-1: 0 = choose the kernel, 1 = one CTA per instance, 2 = one CTA per
                             trotter.  Test hooks of the one-CTA-per-trotter sweep: 16 = every bounded
                             wait gives up after 1 ms (not 4 s); 32 = trotter 0 never publishes its accept
                             words, so its neighbours' waits run out and the kernel ends with status 1 */
    const double *J64;    /* optional FP64 couplings of a <double> problem (N x N, row stride N; J is their
                             fp32 rounding): trials the fp32 path flags are decided from these */
    const double *h64;    /* optional FP64 h of a <double> problem */
} sq103_dense_task;

/* workspace the multi-CTA sweep needs for nSteps steps (one 64-bit accept word per trotter and
 * 32 iterations) */
SQ103_API unsigned long long sq103_dense_ws_bytes(int N, int m, int nSteps);
/* 1 if the one-CTA-per-trotter sweep can run this shape on the current device (N >= 64, m >= 2;
 * the launch also needs ldJ % 4 == 0 and a 16-byte aligned J) */
SQ103_API int sq103_dense_multicta_ok(int N, int m, int algo);
/* No counterpart in the reference.  Up to 16 independent instances in one
 * cooperative launch of the one-CTA-per-trotter sweep (their trotter counts
 * summed within sq103_dense_multicta_capacity of the largest N); each task
 * needs its own ws.  Every instance ends exactly as when launched alone. */
SQ103_API int sq103_dense_anneal_pack(const sq103_dense_task *tasks, int n, void *stream);
/* CTAs of the one-CTA-per-trotter sweep that can be resident at once for rows of N spins */
SQ103_API int sq103_dense_multicta_capacity(int N);

/* ------------------------------------------- tensor-core field refresh
 * F[y][r] = sum_k q[y][k] B[r][k] on tcgen05 (operands by TMA, accumulators in
 * TMEM); replaces the J.q contractions DeviceDotJqVec4
 * (sqaodc/cuda/DeviceBatchedDot.cuh:247-262) and the cuBLAS SGEMMs of
 * CUDABipartiteGraphAnnealer.cu:393-401.  B is held as four signed 8-bit digit
 * planes of its 31-bit fixed-point value (exact in bf16); with +-1 spins every
 * partial sum is an integer below 2^24, so the contraction is exact and the
 * result is within the quantisation of B (2^-29 of max |B| per element) of the
 * exact field, rounded once to fp32.  K < 2^17. */
/* bytes of the digit buffer of an R x K matrix B (256-byte aligned allocation) */
SQ103_API unsigned long long sq103_tc_digits_bytes(int R, int K);
/* bytes of the bf16 spin scratch of m rows of K spins (16-byte aligned) */
SQ103_API unsigned long long sq103_tc_spins_bytes(int m, int K);
/* digit planes of B = J (R x K, row stride ldJ; transpose = 0) or B = J^T (J is
 * K x R, row stride ldJ; transpose = 1) */
SQ103_API int sq103_tc_make_digits(const float *J, int ldJ, int R, int K, int transpose, void *digits, void *stream);
/* F (m x R, row stride ldF) from the digits and q (m x K int8, row stride ldq);
 * spinsBf16: sq103_tc_spins_bytes(m, K) of scratch.  status: optional device word
 * set to 1 when a bounded wait gave up.  flags: 0; test hooks 1 = the first K
 * block's copies are never issued, 2 = waits give up after 1 ms. */
SQ103_API int sq103_tc_refresh(const void *digits, int R, int K, const int8_t *q, int ldq, int m, void *spinsBf16,
                               float *F, int ldF, int flags, int *status, void *stream);
/* 1 when the dense annealers refresh N-spin fields on the tensor cores (N >= 1024) */
SQ103_API int sq103_dense_refresh_uses_tc(int N);
/* 1 when the bipartite annealers compute the half-step fields on the tensor cores
 * (N0 N1 >= 2^20 and at least 64 output tiles of 128 trotters x 64 spins per half
 * step); the task then carries the digits of J and J^T */
SQ103_API int sq103_bipartite_refresh_uses_tc(int N0, int N1, int m);
/* the dense refresh of every path: sq103_tc_refresh from `digits` (of J, R = K = N)
 * when given, else sq103_dense_field_refresh */
SQ103_API int sq103_dense_refresh(const float *J, int ldJ, const void *digits, void *spinsBf16, const int8_t *q,
                                  float *F, int N, int m, int *status, void *stream);

/* QUBO -> Ising (h, J, c); replaces DeviceDenseGraphFormulas::calculateHamiltonian
 * (sqaodc/cuda/DeviceFormulas.cpp:24-31).  scratch: N doubles. */
SQ103_API int sq103_dense_hamiltonian(const float *W, int ldW, int N, int maximize, float *h, float *J,
                                      int ldJ, float *c, double *c64, double *scratch, void *stream);
/* F = q J for all trotters (the local-field refresh). */
SQ103_API int sq103_dense_field_refresh(const float *J, int ldJ, const int8_t *q, float *F, int N, int m,
                                        void *stream);
/* One instance of a batched field refresh. */
typedef struct sq103_field_job {
    const float *J;   /* N x N couplings, row stride ldJ */
    const int8_t *q;  /* m x N spins */
    float *F;         /* m x N fields */
    int N, m, ldJ;
    int tile0;        /* its first output tile: the sum over earlier jobs of ceil(N/64) ceil(m/64) */
} sq103_field_job;
/* F = q J of every job in one launch (no counterpart in the reference: the batch
 * refreshes its many small instances together).  jobs and tileJob (the job of
 * each of the nTiles output tiles, in tile order) in device memory.  Each job's
 * fields are bit-identical to sq103_dense_field_refresh of that job. */
SQ103_API int sq103_dense_field_refresh_batch(const sq103_field_job *jobs, const int *tileJob, int nTiles,
                                              void *stream);
/* FP64 Ising energies of all trotters (calculate_E; sqaodc/cuda/DeviceFormulas.cpp:42-49);
 * the row sums q J are accumulated in double-float (about 2^-44 relative).
 * r_scratch: m x N doubles. */
SQ103_API int sq103_dense_energy(const float *J, int ldJ, const float *h, const double *c64,
                                 const int8_t *q, int N, int m, int maximize, double *r_scratch,
                                 double *E64, float *E32, void *stream);
/* sq103_dense_energy without a caller-supplied scratch buffer; it has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory: code inside a framework whose pool owns all device memory,
 * or a service that must not grow its footprint after start-up.  The m x N
 * FP64 row sums live in a static device array of
 * sq103_dense_energy_static_max() = 262144 doubles (2 MiB, held by every GPU
 * that loads the library); m * N above that returns 3 (capacity) with a
 * message in sq103_last_error() and launches nothing.  Nothing is allocated
 * and nothing needs to start at zero (every scratch value is written before
 * it is read).  The first call on each device looks up the array's device
 * address (cudaGetSymbolAddress, with that device current); make that first
 * call before any stream capture.  One scratch array serves all callers of a
 * device: calls that overlap in time (other streams, other threads) race on
 * it and must be serialised by the caller. */
SQ103_API unsigned long long sq103_dense_energy_static_max(void);
SQ103_API int sq103_dense_energy_static(const float *J, int ldJ, const float *h, const double *c64,
                                        const int8_t *q, int N, int m, int maximize, double *E64, float *E32,
                                        void *stream);
/* sum_y q_y . q_{y+1} (DeviceDotSpins, sqaodc/cuda/DeviceBatchedDot.cuh:145-160) */
SQ103_API int sq103_ring_dot(const int8_t *q, int N, int m, long long *out, void *stream);
/* randomizeSpin (sqaodc/cuda/DeviceKernels.cu:550-572) from the Philox stream */
SQ103_API int sq103_randomize_spins(int8_t *q, int N, int m, uint64_t seed, uint32_t step, int tagSide,
                                    void *stream);
/* nSteps annealOneStep sweeps of one instance (CUDADenseGraphAnnealer::annealOneStepSQA/SA,
 * sqaodc/cuda/CUDADenseGraphAnnealer.cu:524-602).  The task is passed by value. */
SQ103_API int sq103_dense_anneal(const sq103_dense_task *task, void *stream);
/* nTasks instances in one launch; d_tasks lives in device memory. */
SQ103_API int sq103_dense_anneal_batch(const sq103_dense_task *d_tasks, int nTasks, int maxN, int maxM,
                                       void *stream);
/* Persistent batch sweep: `grid` CTAs take instances from d_queue (two ints,
 * zero before the first launch; the kernel leaves them zero) in the order
 * d_order (largest first); instance i runs steps [d_pos[i], d_pos[i] +
 * stepsPerLaunch) of its schedule (task.nSteps steps in total, task.G /
 * task.beta indexed by step) and advances d_pos[i].  Replaying the same
 * launch (e.g. from a CUDA graph) therefore advances every instance.
 * smemBytes: shared memory per CTA (instances whose spins and fields fit are
 * staged there).  d_nTasks (optional): the instance count read on the device,
 * so that a captured launch stays valid while instances come and go. */
SQ103_API int sq103_dense_batch_launch(const sq103_dense_task *d_tasks, int nTasks, const int *d_nTasks,
                                       const int *d_order, int *d_pos, int *d_queue, int stepsPerLaunch, int grid,
                                       int smemBytes, void *stream);
SQ103_API int sq103_dense_batch_max_smem(void);
/* Least smemBytes a batch launch needs when its largest instance has maxM
 * trotters (the per-phase flip lists); an instance whose lists do not fit is
 * skipped, its pos unchanged and 3 (capacity) written to its status. */
SQ103_API int sq103_dense_batch_min_smem(int maxM);
SQ103_API int sq103_dense_batch_ctas_per_sm(int smemBytes);

/* -------------------------------------------- kernel layer: bipartite */

typedef struct sq103_bipartite_task {
    const float *J;       /* N1 x N0 */
    const float *h0, *h1; /* N0, N1 */
    int8_t *q0, *q1;      /* m x N0, m x N1 */
    float *F0, *F1;       /* m x N0, m x N1 field scratch */
    uint32_t *trace;
    unsigned long long *accepted;
    const float *G, *beta; /* device arrays of nSteps entries, or NULL: use Gs / betas */
    float Gs, betas;
    uint64_t seed;
    uint32_t step0;
    int N0, N1, m, algo, nSteps;
    const double *J64, *h0_64, *h1_64; /* optional FP64 problem of a <double> annealer (J64 N1 x N0; J, h0,
                                          h1 are its fp32 rounding): trials the fp32 path flags are
                                          decided from these */
    const void *digits1, *digits0;     /* optional: the half-step fields on the tensor cores from the
                                          digits of J (for F1) and of J^T (for F0), sq103_tc_make_digits */
    void *spinsBf16;                   /* their spin scratch, sq103_tc_spins_bytes(m, max(N0, N1)) */
    int *status;                       /* optional status word (a bounded wait of the refresh gave up) */
} sq103_bipartite_task;

/* (sqaodc/cuda/DeviceFormulas.cpp:107-117). scratch: N0 + N1 doubles */
SQ103_API int sq103_bipartite_hamiltonian(const float *b0, const float *b1, const float *W, int N0,
                                          int N1, int maximize, float *h0, float *h1, float *J, float *c,
                                          double *c64, double *scratch, void *stream);
/* side 1: F[y][i] = sum_j J[i][j] qFixed[y][j];  side 0: F[y][j] = sum_i qFixed[y][i] J[i][j]
 * (the per-half-step cuBLAS GEMMs of CUDABipartiteGraphAnnealer.cu:393-401) */
SQ103_API int sq103_bipartite_fields(const float *J, int N0, int N1, const int8_t *qFixed, int side,
                                     float *F, int m, void *stream);
/* FP64 energies (sqaodc/cuda/DeviceFormulas.cpp:120-140); r_scratch: m x N1 doubles */
SQ103_API int sq103_bipartite_energy(const float *J, const float *h0, const float *h1, const double *c64,
                                     const int8_t *q0, const int8_t *q1, int N0, int N1, int m,
                                     int maximize, double *r_scratch, double *E64, float *E32,
                                     void *stream);

/* ------------------------------------- kernel layer: FP64 formula kernels */
/* The formulas with real = double (sqaodc/cuda/DeviceFormulas.cpp:24-140 of
 * the <double> instantiation): FP64 inputs, FP64 sums in a fixed order.
 * Dense: W, J N x N row-major; scratch N doubles.  Energies: E[y] =
 * sign (-c - h q_y^T - q_y J q_y^T), sign -1 when maximize; h may be NULL
 * (zero); a QUBO energy x W x^T is the call with J = W, h = NULL, c = 0,
 * maximize = 1.  Bipartite: W, J N1 x N0; scratch N0 + 2 N1 doubles. */
SQ103_API int sq103_dense_hamiltonian64(const double *W, int N, double *h, double *J, double *c, double *scratch,
                                        void *stream);
SQ103_API int sq103_dense_energy64(const double *J, const double *h, double c, const int8_t *q, int N, int m,
                                   int maximize, double *E, void *stream);
SQ103_API int sq103_bipartite_hamiltonian64(const double *b0, const double *b1, const double *W, int N0, int N1,
                                            double *h0, double *h1, double *J, double *c, double *scratch,
                                            void *stream);
SQ103_API int sq103_bipartite_energy64(const double *J, const double *h0, const double *h1, double c,
                                       const int8_t *q0, const int8_t *q1, int N0, int N1, int m, int maximize,
                                       double *E, void *stream);
/* nSteps annealOneStep of one bipartite instance
 * (CUDABipartiteGraphAnnealer::annealOneStepSQA/SA, :539-625) */
SQ103_API int sq103_bipartite_anneal(const sq103_bipartite_task *task, void *stream);
/* The persistent batch scheme of sq103_dense_batch_launch for bipartite
 * instances (coloring / sa_coloring): one CTA runs both half-step field GEMMs
 * and the colour phases of an instance; bit-identical to sq103_bipartite_anneal. */
SQ103_API int sq103_bipartite_batch_launch(const sq103_bipartite_task *d_tasks, int nTasks, const int *d_nTasks,
                                           const int *d_order, int *d_pos, int *d_queue, int stepsPerLaunch,
                                           int grid, void *stream);

/* ------------------------------------------------- kernel layer: BF */

/* Dense BF over [xBegin, xEnd): fp32 energies of x^T W x (W already signed
 * for the optimisation direction), then every x with E <= Emin + slack is
 * written to cand (up to cap; *count gets the true number).
 * ws: workspace of sq103_bf_workspace_bytes(N) bytes.
 * Replaces DeviceDenseGraphBatchSearch::{calculate_E, partition_xMins, select}
 * (sqaodc/cuda/DeviceDenseGraphBatchSearch.cu:58-187). */
SQ103_API size_t sq103_bf_workspace_bytes(int N);
SQ103_API int sq103_dense_bf_range(const float *W, int N, uint64_t xBegin, uint64_t xEnd, float slack,
                                   void *ws, uint64_t *cand, int cap, int *count, float *Emin32,
                                   void *stream);
/* FP64 energies of packed states (tie-break of the candidates) */
SQ103_API int sq103_dense_bf_refine(const float *W, int N, const uint64_t *x, int n, double *E,
                                    void *stream);
/* Bipartite BF over [x0b, x0e) x [x1b, x1e) (DeviceBipartiteGraphBatchSearch.cu:65-217).
 * cand receives (x0, x1) pairs. ws: sq103_bf_workspace_bytes(N0 + N1) bytes. */
SQ103_API int sq103_bipartite_bf_range(const float *b0, const float *b1, const float *W, int N0, int N1,
                                       uint64_t x0b, uint64_t x0e, uint64_t x1b, uint64_t x1e,
                                       float slack, void *ws, uint64_t *cand, int cap, int *count,
                                       float *Emin32, void *stream);
SQ103_API int sq103_bipartite_bf_refine(const float *b0, const float *b1, const float *W, int N0, int N1,
                                        const uint64_t *pairs, int n, double *E, void *stream);
/* The refines with FP64 couplings (the double-precision searchers screen with
 * the fp32-rounded couplings and re-evaluate the candidates here). */
SQ103_API int sq103_dense_bf_refine64(const double *W, int N, const uint64_t *x, int n, double *E, void *stream);
SQ103_API int sq103_bipartite_bf_refine64(const double *b0, const double *b1, const double *W, int N0, int N1,
                                          const uint64_t *pairs, int n, double *E, void *stream);

/* ------------------------------------------- handle layer: annealers */
/* Mirrors annealer.inc:885-908.  Preferences are passed as strings, as the
 * reference parses them (sqaodc/common/Preference.cpp:61-78):
 * algorithm = naive|coloring|sa_naive|sa_coloring|default|sa_default,
 * n_trotters = <int>.  sq103_*_get_preferences writes
 * "algorithm=...;n_trotters=...;precision=float;device=cuda". */

SQ103_API int sq103_dg_annealer_new(void **handle);
/* <double> annealer (sqaod::cuda::DenseGraphAnnealer<double>,
 * sqaodc/cuda/CUDADenseGraphAnnealer.cu:607-608): every entry point below takes
 * its handle too.  The FP64 problem is set with sq103_dg_annealer_set_qubo64 /
 * set_hamiltonian64; the sweeps run on its fp32 rounding, every trial the fp32
 * test flags is decided from the FP64 couplings, energies are FP64 sums
 * (sq103_dg_annealer_get_E64), and G and beta are taken in fp32. */
SQ103_API int sq103_dg_annealer64_new(void **handle);
SQ103_API int sq103_dg_annealer_set_qubo64(void *handle, const double *W, int N, int optimize);
SQ103_API int sq103_dg_annealer_set_hamiltonian64(void *handle, const double *h, const double *J, double c, int N);
SQ103_API int sq103_dg_annealer_get_hamiltonian64(void *handle, double *h, double *J, double *c);
SQ103_API int sq103_dg_annealer_get_system_E64(void *handle, double G, double beta, double *E);
SQ103_API int sq103_dg_annealer_delete(void *handle);
SQ103_API int sq103_dg_annealer_seed(void *handle, unsigned long long seed);
SQ103_API int sq103_dg_annealer_set_qubo(void *handle, const float *W, int N, int optimize);
SQ103_API int sq103_dg_annealer_set_hamiltonian(void *handle, const float *h, const float *J, float c,
                                                int N);
SQ103_API int sq103_dg_annealer_get_problem_size(void *handle, int *N);
SQ103_API int sq103_dg_annealer_set_preference(void *handle, const char *name, const char *value);
SQ103_API int sq103_dg_annealer_get_preferences(void *handle, char *buf, int buflen);
SQ103_API int sq103_dg_annealer_get_E(void *handle, float *E, int cap, int *n);
SQ103_API int sq103_dg_annealer_get_x(void *handle, int8_t *x, int capRows, int *m);
SQ103_API int sq103_dg_annealer_get_hamiltonian(void *handle, float *h, float *J, float *c);
SQ103_API int sq103_dg_annealer_get_q(void *handle, int8_t *q, int capRows, int *m);
SQ103_API int sq103_dg_annealer_set_q(void *handle, const int8_t *q, int N);
SQ103_API int sq103_dg_annealer_set_qset(void *handle, const int8_t *q, int m, int N);
SQ103_API int sq103_dg_annealer_randomize_spin(void *handle);
SQ103_API int sq103_dg_annealer_calculate_E(void *handle);
SQ103_API int sq103_dg_annealer_prepare(void *handle);
SQ103_API int sq103_dg_annealer_make_solution(void *handle);
SQ103_API int sq103_dg_annealer_get_system_E(void *handle, float G, float beta, float *E);
SQ103_API int sq103_dg_annealer_anneal_one_step(void *handle, float G, float beta);
/* initAnneal: prepare() + randomizeSpin() (named by the target API; the
 * reference has no such method) */
SQ103_API int sq103_dg_annealer_init_anneal(void *handle);
/* extensions: a whole schedule in one call; FP64 energies; counters; trace */
SQ103_API int sq103_dg_annealer_anneal(void *handle, const float *G, const float *beta, int nSteps);
SQ103_API int sq103_dg_annealer_get_E64(void *handle, double *E, int cap, int *n);
SQ103_API int sq103_dg_annealer_get_accepted(void *handle, unsigned long long *accepted);
SQ103_API int sq103_dg_annealer_get_rng_state(void *handle, unsigned long long *seed, uint32_t *step);
/* Checkpoint / resume (no counterpart in the reference): q and F are m x N
 * (spins, resident local fields), sinceRefresh the steps since the last field
 * refresh.  set_checkpoint needs a prepared annealer of the same problem,
 * algorithm and trotter count; the run then continues bit for bit as the one
 * the checkpoint was taken from. */
SQ103_API int sq103_dg_annealer_get_checkpoint(void *handle, int8_t *q, float *F, unsigned long long *seed,
                                               uint32_t *step, int *sinceRefresh);
SQ103_API int sq103_dg_annealer_set_checkpoint(void *handle, const int8_t *q, const float *F, int m, int N,
                                               unsigned long long seed, uint32_t step, int sinceRefresh);
SQ103_API int sq103_dg_annealer_set_trace(void *handle, int enable);
/* kernel selection for the sweep: 0 = automatic, 1 = one CTA per instance, 2 = one CTA per trotter */
SQ103_API int sq103_dg_annealer_set_kernel(void *handle, int flags);
SQ103_API int sq103_dg_annealer_get_trace(void *handle, uint32_t *bits, int nwords);

SQ103_API int sq103_bg_annealer_new(void **handle);
/* <double> bipartite annealer (CUDABipartiteGraphAnnealer.cu:647-648), as above */
SQ103_API int sq103_bg_annealer64_new(void **handle);
SQ103_API int sq103_bg_annealer_set_qubo64(void *handle, const double *b0, const double *b1, const double *W,
                                           int N0, int N1, int optimize);
SQ103_API int sq103_bg_annealer_set_hamiltonian64(void *handle, const double *h0, const double *h1,
                                                  const double *J, double c, int N0, int N1);
SQ103_API int sq103_bg_annealer_get_hamiltonian64(void *handle, double *h0, double *h1, double *J, double *c);
SQ103_API int sq103_bg_annealer_get_system_E64(void *handle, double G, double beta, double *E);
SQ103_API int sq103_bg_annealer_delete(void *handle);
SQ103_API int sq103_bg_annealer_seed(void *handle, unsigned long long seed);
SQ103_API int sq103_bg_annealer_set_qubo(void *handle, const float *b0, const float *b1, const float *W,
                                         int N0, int N1, int optimize);
SQ103_API int sq103_bg_annealer_set_hamiltonian(void *handle, const float *h0, const float *h1,
                                                const float *J, float c, int N0, int N1);
SQ103_API int sq103_bg_annealer_get_problem_size(void *handle, int *N0, int *N1);
SQ103_API int sq103_bg_annealer_set_preference(void *handle, const char *name, const char *value);
SQ103_API int sq103_bg_annealer_get_preferences(void *handle, char *buf, int buflen);
SQ103_API int sq103_bg_annealer_get_E(void *handle, float *E, int cap, int *n);
SQ103_API int sq103_bg_annealer_get_x(void *handle, int8_t *x0, int8_t *x1, int capRows, int *m);
SQ103_API int sq103_bg_annealer_get_hamiltonian(void *handle, float *h0, float *h1, float *J, float *c);
SQ103_API int sq103_bg_annealer_get_q(void *handle, int8_t *q0, int8_t *q1, int capRows, int *m);
SQ103_API int sq103_bg_annealer_set_q(void *handle, const int8_t *q0, const int8_t *q1, int N0, int N1);
SQ103_API int sq103_bg_annealer_set_qset(void *handle, const int8_t *q0, const int8_t *q1, int m, int N0,
                                         int N1);
SQ103_API int sq103_bg_annealer_randomize_spin(void *handle);
SQ103_API int sq103_bg_annealer_calculate_E(void *handle);
SQ103_API int sq103_bg_annealer_prepare(void *handle);
SQ103_API int sq103_bg_annealer_make_solution(void *handle);
SQ103_API int sq103_bg_annealer_get_system_E(void *handle, float G, float beta, float *E);
SQ103_API int sq103_bg_annealer_anneal_one_step(void *handle, float G, float beta);
SQ103_API int sq103_bg_annealer_init_anneal(void *handle);
SQ103_API int sq103_bg_annealer_anneal(void *handle, const float *G, const float *beta, int nSteps);
SQ103_API int sq103_bg_annealer_get_E64(void *handle, double *E, int cap, int *n);
SQ103_API int sq103_bg_annealer_get_accepted(void *handle, unsigned long long *accepted);
SQ103_API int sq103_bg_annealer_get_rng_state(void *handle, unsigned long long *seed, uint32_t *step);
/* Checkpoint / resume: q0 m x N0, q1 m x N1 spins and the Philox state (the
 * fields are recomputed from the spins every half step). */
SQ103_API int sq103_bg_annealer_get_checkpoint(void *handle, int8_t *q0, int8_t *q1, unsigned long long *seed,
                                               uint32_t *step);
SQ103_API int sq103_bg_annealer_set_checkpoint(void *handle, const int8_t *q0, const int8_t *q1, int m, int N0,
                                               int N1, unsigned long long seed, uint32_t step);
SQ103_API int sq103_bg_annealer_set_trace(void *handle, int enable);
SQ103_API int sq103_bg_annealer_get_trace(void *handle, uint32_t *bits, int nwords);

/* ---------------------------------------- handle layer: BF searchers */
/* Mirrors bf_searcher.inc:479-494.  Preferences: tile_size (dense),
 * tile_size_0 / tile_size_1 (bipartite). */

SQ103_API int sq103_dg_bf_new(void **handle);
/* The <double> searcher (the reference's CUDADenseGraphBFSearcher<double>): the
 * other sq103_dg_bf_* functions take either handle.  It screens with the
 * fp32-rounded couplings (the screening slack widened by twice their total
 * rounding) and re-evaluates the candidates with the FP64 couplings, so Emin
 * and the argmin set are those of the FP64 problem.  sq103_dg_bf_set_qubo64
 * sets FP64 couplings on either handle; on a <double> handle sq103_dg_bf_set_qubo
 * takes fp32 couplings as exact doubles. */
SQ103_API int sq103_dg_bf64_new(void **handle);
SQ103_API int sq103_dg_bf_set_qubo64(void *handle, const double *W, int N, int optimize);
SQ103_API int sq103_dg_bf_delete(void *handle);
SQ103_API int sq103_dg_bf_set_qubo(void *handle, const float *W, int N, int optimize);
SQ103_API int sq103_dg_bf_get_problem_size(void *handle, int *N);
SQ103_API int sq103_dg_bf_set_preference(void *handle, const char *name, const char *value);
SQ103_API int sq103_dg_bf_get_preferences(void *handle, char *buf, int buflen);
SQ103_API int sq103_dg_bf_get_x(void *handle, int8_t *x, int capRows, int *n);
SQ103_API int sq103_dg_bf_get_E(void *handle, float *E, int cap, int *n);
SQ103_API int sq103_dg_bf_prepare(void *handle);
SQ103_API int sq103_dg_bf_calculate_E(void *handle);
SQ103_API int sq103_dg_bf_make_solution(void *handle);
/* one tile; *done = 1 when the whole range is searched; curXEnd may be NULL */
SQ103_API int sq103_dg_bf_search_range(void *handle, unsigned long long *curXEnd, int *done);
SQ103_API int sq103_dg_bf_search(void *handle);
/* No counterpart in the reference (multi-GPU sharding): search the packed
 * states [xBegin, xEnd) after prepare(), merged into the searcher's result;
 * the ranges one searcher is given must ascend.  get_E64: the exact FP64
 * minimum found so far (signed for the optimisation direction). */
SQ103_API int sq103_dg_bf_search_subrange(void *handle, unsigned long long xBegin, unsigned long long xEnd);
SQ103_API int sq103_dg_bf_get_E64(void *handle, double *E);
/* No counterpart in the reference: the number of rows sq103_dg_bf_get_x
 * returns (the minimisers kept, at most tile_size), to size its buffer. */
SQ103_API int sq103_dg_bf_solution_count(void *handle, int *n);

SQ103_API int sq103_bg_bf_new(void **handle);
/* The <double> bipartite searcher, as sq103_dg_bf64_new above (W: N1 x N0). */
SQ103_API int sq103_bg_bf64_new(void **handle);
SQ103_API int sq103_bg_bf_set_qubo64(void *handle, const double *b0, const double *b1, const double *W, int N0,
                                     int N1, int optimize);
SQ103_API int sq103_bg_bf_delete(void *handle);
SQ103_API int sq103_bg_bf_set_qubo(void *handle, const float *b0, const float *b1, const float *W, int N0,
                                   int N1, int optimize);
SQ103_API int sq103_bg_bf_get_problem_size(void *handle, int *N0, int *N1);
SQ103_API int sq103_bg_bf_set_preference(void *handle, const char *name, const char *value);
SQ103_API int sq103_bg_bf_get_preferences(void *handle, char *buf, int buflen);
SQ103_API int sq103_bg_bf_get_x(void *handle, int8_t *x0, int8_t *x1, int capRows, int *n);
SQ103_API int sq103_bg_bf_get_E(void *handle, float *E, int cap, int *n);
SQ103_API int sq103_bg_bf_prepare(void *handle);
SQ103_API int sq103_bg_bf_calculate_E(void *handle);
SQ103_API int sq103_bg_bf_make_solution(void *handle);
SQ103_API int sq103_bg_bf_search_range(void *handle, unsigned long long *curX0, unsigned long long *curX1,
                                       int *done);
SQ103_API int sq103_bg_bf_search(void *handle);
/* exact FP64 minimum found so far (negated for maximize) */
SQ103_API int sq103_bg_bf_get_E64(void *handle, double *E);

/* ------------------------------------- handle layer: batched annealer */
/* Many independent dense instances annealed in lock-step: one persistent
 * launch per step for the smaller instances (replayed from a CUDA graph when
 * useGraph != 0), packed one-CTA-per-trotter launches for the larger ones.  No
 * counterpart method table in the reference; each instance follows exactly
 * the rules of sq103_dg_annealer (same seed -> same result).  Coloring
 * algorithm (SA when m == 1). */
SQ103_API int sq103_dense_batch_new(void **handle);
SQ103_API int sq103_dense_batch_delete(void *handle);
SQ103_API int sq103_dense_batch_add(void *handle, const float *W, int N, int m, int optimize,
                                    unsigned long long seed, int *index);
SQ103_API int sq103_dense_batch_set_schedule(void *handle, const float *G, const float *beta, int nSteps);
SQ103_API int sq103_dense_batch_prepare(void *handle);
/* Instances of at least N spins (m >= 2, fitting the device) are stepped by the
 * one-CTA-per-trotter sweep in packed cooperative launches, the rest by the
 * persistent batch kernel; both give the same results.  Default 1024; 0 keeps
 * every instance on the persistent kernel.  Takes effect at the next prepare. */
SQ103_API int sq103_dense_batch_set_multicta_min_n(void *handle, int N);
/* instances on the one-CTA-per-trotter sweep since the last prepare */
SQ103_API int sq103_dense_batch_multicta_count(void *handle, int *n);
SQ103_API int sq103_dense_batch_autotune(void *handle, int trialSteps, int *smemBytes);
/* Trotters per CTA by measurement (no counterpart in the reference): prepares the
 * batch with each candidate size limit of sq103_dense_batch_set_multicta_min_n
 * (one CTA per trotter at or above it, one CTA per instance below), times
 * trialSteps steps from the start of the schedule, keeps the fastest and prepares
 * again (the state is that of a fresh prepare, whatever the choice). */
SQ103_API int sq103_dense_batch_autotune_routing(void *handle, int trialSteps, const int *candidates, int n,
                                                int *chosen);
SQ103_API int sq103_dense_batch_anneal(void *handle, int nSteps, int useGraph);
SQ103_API int sq103_dense_batch_sync(void *handle);
SQ103_API int sq103_dense_batch_info(void *handle, int *nInst, int *pos, int *grid, int *smemBytes);
SQ103_API int sq103_dense_batch_get_E(void *handle, int index, double *E, int cap, int *n);
SQ103_API int sq103_dense_batch_get_q(void *handle, int index, int8_t *q, int capRows, int *m);

/* ------------------------------------------------ handle layer: formula sets */
/* The formulas_methods table of the reference's Python extension
 * (sqaodc/pyglue/formulas.inc:586-605) over the CUDA formula classes
 * (sqaodc/cuda/CUDAFormulas.cpp:8-294): host buffers in and out, one call
 * uploads, computes and copies back.  A batch of m = 1 rows is the reference's
 * single-vector method (dense_graph_calculate_E, ...), m > 1 the batched one.
 * Energies are FP64 (the reference returns them in the solver's real type);
 * bits x must be 0 / 1 and spins q -1 / +1, matrices are dense row-major (row
 * stride = columns) and a dense W or J must be symmetric, or the call fails. */
SQ103_API int sq103_dg_formulas_new(void **handle);
SQ103_API int sq103_dg_formulas_delete(void *handle);
/* E[i] = x_i W x_i^T (dense_graph_calculate_E / dense_graph_batch_calculate_E) */
SQ103_API int sq103_dg_formulas_calculate_E(void *handle, const float *W, int N, const int8_t *x, int m,
                                            double *E);
/* h (N), J (N x N, zero diagonal), c (dense_graph_calculate_hamiltonian) */
SQ103_API int sq103_dg_formulas_calculate_hamiltonian(void *handle, const float *W, int N, float *h, float *J,
                                                      float *c);
/* E[i] = -c - h q_i^T - q_i J q_i^T (dense_graph_[batch_]calculate_E_from_spin) */
SQ103_API int sq103_dg_formulas_calculate_E_from_spin(void *handle, const float *h, const float *J, float c, int N,
                                                      const int8_t *q, int m, double *E);
SQ103_API int sq103_bg_formulas_new(void **handle);
SQ103_API int sq103_bg_formulas_delete(void *handle);
/* E[i] = b0 x0_i^T + b1 x1_i^T + x1_i W x0_i^T, W N1 x N0 (bipartite_graph_[batch_]calculate_E) */
SQ103_API int sq103_bg_formulas_calculate_E(void *handle, const float *b0, const float *b1, const float *W, int N0,
                                            int N1, const int8_t *x0, const int8_t *x1, int m, double *E);
/* E[i1 * m0 + i0] = the energy of (x0_i0, x1_i1), m1 x m0 row-major
 * (bipartite_graph_batch_calculate_E_2d) */
SQ103_API int sq103_bg_formulas_calculate_E_2d(void *handle, const float *b0, const float *b1, const float *W,
                                               int N0, int N1, const int8_t *x0, int m0, const int8_t *x1, int m1,
                                               double *E);
/* h0 (N0), h1 (N1), J (N1 x N0), c (bipartite_graph_calculate_hamiltonian) */
SQ103_API int sq103_bg_formulas_calculate_hamiltonian(void *handle, const float *b0, const float *b1,
                                                      const float *W, int N0, int N1, float *h0, float *h1,
                                                      float *J, float *c);
/* E[i] = -c - h0 q0_i^T - h1 q1_i^T - q1_i J q0_i^T (bipartite_graph_[batch_]calculate_E_from_spin) */
SQ103_API int sq103_bg_formulas_calculate_E_from_spin(void *handle, const float *h0, const float *h1,
                                                      const float *J, float c, int N0, int N1, const int8_t *q0,
                                                      const int8_t *q1, int m, double *E);
/* The same formula sets with real = double (the reference's <double>
 * instantiation of CUDADenseGraphFormulas / CUDABipartiteGraphFormulas):
 * arguments as above with double matrices, vectors and c; FP64 kernels. */
SQ103_API int sq103_dg_formulas64_new(void **handle);
SQ103_API int sq103_dg_formulas64_delete(void *handle);
SQ103_API int sq103_dg_formulas64_calculate_E(void *handle, const double *W, int N, const int8_t *x, int m,
                                              double *E);
SQ103_API int sq103_dg_formulas64_calculate_hamiltonian(void *handle, const double *W, int N, double *h,
                                                        double *J, double *c);
SQ103_API int sq103_dg_formulas64_calculate_E_from_spin(void *handle, const double *h, const double *J, double c,
                                                        int N, const int8_t *q, int m, double *E);
SQ103_API int sq103_bg_formulas64_new(void **handle);
SQ103_API int sq103_bg_formulas64_delete(void *handle);
SQ103_API int sq103_bg_formulas64_calculate_E(void *handle, const double *b0, const double *b1, const double *W,
                                              int N0, int N1, const int8_t *x0, const int8_t *x1, int m, double *E);
SQ103_API int sq103_bg_formulas64_calculate_E_2d(void *handle, const double *b0, const double *b1,
                                                 const double *W, int N0, int N1, const int8_t *x0, int m0,
                                                 const int8_t *x1, int m1, double *E);
SQ103_API int sq103_bg_formulas64_calculate_hamiltonian(void *handle, const double *b0, const double *b1,
                                                        const double *W, int N0, int N1, double *h0, double *h1,
                                                        double *J, double *c);
SQ103_API int sq103_bg_formulas64_calculate_E_from_spin(void *handle, const double *h0, const double *h1,
                                                        const double *J, double c, int N0, int N1,
                                                        const int8_t *q0, const int8_t *q1, int m, double *E);

/* ------------------------------------------- handle layer: request server */
/* Continuous batching of anneal and search requests of mixed size and type (no
 * counterpart in the reference).  Requests are admitted in arrival order while
 * their device-memory footprint fits budgetBytes and a slot is free (one that
 * cannot start yet does not block the ones behind it); every
 * sq103_server_tick advances every active instance by 8 annealOneSteps (one
 * field-refresh period) and completes the finished ones (FP64 energies, spins).  Each request ends
 * exactly as the same seed and schedule would alone (sq103_dg_annealer /
 * sq103_bg_annealer with prepare, randomize_spin and the schedule; the
 * coloring algorithm for m > 1, sa_naive (dense) or sa_coloring (bipartite)
 * for m == 1).  States: 0 queued, 1 active, 2 done. */
SQ103_API int sq103_server_new(void **handle, unsigned long long budgetBytes, int maxSlots);
SQ103_API int sq103_server_delete(void *handle);
SQ103_API int sq103_server_submit_dense(void *handle, const float *W, int N, int m, int optimize,
                                        unsigned long long seed, const float *G, const float *beta, int nSteps,
                                        int *id);
SQ103_API int sq103_server_submit_bipartite(void *handle, const float *b0, const float *b1, const float *W,
                                            int N0, int N1, int m, int optimize, unsigned long long seed,
                                            const float *G, const float *beta, int nSteps, int *id);
SQ103_API int sq103_server_tick(void *handle, int *completed);
SQ103_API int sq103_server_state(void *handle, int id, int *state);
/* A dense brute-force search request (W symmetric N x N, N < 64; the
 * reference's unit of work is CUDADenseGraphBFSearcher::searchRange,
 * sqaodc/cuda/CUDADenseGraphBFSearcher.cpp:155-185).  Each tick searches the
 * next 2^30 states of every active search (at most 4 at a time) on the
 * searcher's own stream while the tick's anneals run; the result is the exact
 * FP64 minimum and the minimisers in ascending packed order, at most tileSize
 * of them, as sq103_dg_bf_search on the same W and tile_size returns them.
 * Its sq103_server_result gives E[0] = the minimum (signed for `optimize`),
 * *m = the number of minimisers and q0 = their bits x (0/1, one row of N each). */
SQ103_API int sq103_server_submit_search(void *handle, const float *W, int N, int optimize, int tileSize, int *id);
/* rows of the request's result: m for an anneal, the minimisers kept for a search */
SQ103_API int sq103_server_result_rows(void *handle, int id, int *rows);
/* E: m FP64 energies; q0 (m x N or m x N0) and q1 (m x N1, bipartite) spins;
 * release != 0 frees the request's host record. */
SQ103_API int sq103_server_result(void *handle, int id, double *E, int capE, int *m, int8_t *q0, int8_t *q1,
                                  long long capBytes, int release);
SQ103_API int sq103_server_stats(void *handle, int *queued, int *active, int *done,
                                 unsigned long long *bytesInUse);
/* at most n large instances admitted at a time (default 64; dense: one CTA per
 * trotter, packed up to 16 per launch; bipartite: per-instance kernels) */
SQ103_API int sq103_server_set_large_limit(void *handle, int n);
/* Fault injection from the host (tests; no counterpart in the reference): writes
 * `value` into the status word of active dense request `id`, in stream order, as a
 * sweep that gave up a bounded device wait does.  Every dense request has its own
 * status word; sq103_server_result of that request then fails (the request is still
 * released when asked), and no other request is affected. */
SQ103_API int sq103_server_inject_status(void *handle, int id, int value);
/* ids of the requests completed since the last call (at most cap, in completion order) */
SQ103_API int sq103_server_completed(void *handle, int *ids, int cap, int *n);

#ifdef __cplusplus
}
#endif

#endif /* SQAOD_GB300_H */
