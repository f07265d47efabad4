// dense.cu -- dense-graph Suzuki-Trotter / SA sweeps and spin randomisation.
//
// Algorithms (one annealOneStep; the FP64 host replay restates the same rules):
//   coloring (SQA): for k in [0, N): phase A = even trotters y < 2*(m/2), phase
//     B = trotter m-1 when m is odd, phase C = odd trotters.  In each phase every
//     trotter makes one trial at x = hi(w0 * N) with u = (w1 >> 8) 2^-24 drawn
//     from philox((k, y, step, 0x11)):
//       dE = (2/m) q_yx (h_x + 2 F_yx) - q_yx (q_{y-1,x} + q_{y+1,x}) coef,
//       coef = log(tanh(G beta / m)) / beta, accept iff dE < 0 or exp(-beta dE) > u.
//     This is the colour order of CPUDenseGraphAnnealer::annealColoredPlaneParallel
//     (sqaodc/cpu/CPUDenseGraphAnnealer.cpp:304-338) and of tryFlipSQAKernel
//     (sqaodc/cuda/CUDADenseGraphAnnealer.cu:430-519).
//   sa_naive: every trotter makes N trials (philox((k, y, step, 0x12))),
//     dE = 2 q (h + 2 F), accept iff exp(-dE / G) > u
//     (CPUDenseGraphAnnealer.cpp:342-371, CUDADenseGraphAnnealer.cu:545-602).
//   naive: N m sequential trials at (y, x) = (hi(w0 m), hi(w1 N)) from
//     philox((t, 0, step, 0x13)) (CPUDenseGraphAnnealer.cpp:268-279).
//
// Instead of the reference's per-trial row dot J[x] . q[y] (4N bytes of J per
// trial), the kernels keep the local fields F[y][i] = sum_j J[i][j] q[y][j]
// resident and apply a rank-1 update F[y][:] += -2 q_yx J[x][:] per accepted
// flip (one J row streamed per accepted flip).  Updates of a row are applied
// in trial order with one rounding each, so every kernel that runs the same
// trials holds bit-identical fields.
#include <cstdio>

#include "sq_common.cuh"
#include "sq_kernels.h"

namespace sq103 {

struct Flip {
    int y, x;
    float d;
};

constexpr int kBlockThreads = 512;

// Applies the flips of one phase, F[y_f][i] += d_f * J[x_f][i], with the nthr
// threads t = 0 .. nthr-1.  The flips of a phase touch distinct rows, and each
// element takes them in list order, so the result does not depend on nthr.
__device__ __forceinline__ void apply_flips(const Flip *flips, int nf, float *F, const float *J, int ldJ, int N, int t,
                                            int nthr) {
    if (N >= nthr || nf == 1) {
        for (int f = 0; f < nf; ++f) {
            Flip fl = flips[f];
            float *Fy = F + (size_t)fl.y * N;
            const float *Jx = J + (size_t)fl.x * ldJ;
            for (int i = t; i < N; i += nthr) Fy[i] = __fmaf_rn(fl.d, __ldg(Jx + i), Fy[i]);
        }
    } else {
        int groups = nthr / N;
        int g = t / N, i = t - g * N;
        if (g < groups)
            for (int f = g; f < nf; f += groups) {
                Flip fl = flips[f];
                F[(size_t)fl.y * N + i] = __fmaf_rn(fl.d, __ldg(J + (size_t)fl.x * ldJ + i), F[(size_t)fl.y * N + i]);
            }
    }
}

// The FP64 decision of a flagged trial at site x of a trotter whose spins are
// qy: from the exact field over the FP64 couplings of a <double> problem when
// the task has them, else over the fp32 couplings.
__device__ __forceinline__ int exact_dense_accept(const sq103_dense_task &T, bool sa, int x, float qyx,
                                                  const int8_t *qy, float qL, float qR, float G, float beta, float u) {
    const double F = T.J64 ? exact_field_thread(T.J64 + (size_t)x * T.N, 1, qy, T.N)
                           : exact_field_thread(T.J + (size_t)x * T.ldJ, 1, qy, T.N);
    const double hx = T.h64 ? T.h64[x] : (double)T.h[x];
    return exact_accept(sa, true, qyx, hx, F, qL, qR, T.m, G, beta, u);
}

// Dynamic shared memory every launch of anneal_instance needs: the flip lists
// of three phases (3 m entries) and their counters, rounded to 16 bytes.
__host__ __device__ constexpr size_t flip_list_bytes(int m) {
    return ((size_t)(3 * m) * sizeof(Flip) + 3 * sizeof(int) + 15) & ~(size_t)15;
}

// The trials of one phase: trotters yb, yb + ys, ... (cnt of them) at spin
// index k, taken by the nthr threads t = 0 .. nthr-1.  Accepted trials flip
// their spin, append (y, x, -2 q) to fl (counter *nfl) and set their trace bit.
// Trials of one phase are independent: the field row of trotter y holds every
// earlier flip of y, so its exact field is the one the trial sees.
__device__ __forceinline__ void decide_phase(const sq103_dense_task &T, bool sa, uint32_t tag, const StepConst &sc,
                                             const DecisionTol &tol, float G, float beta, uint32_t step, int k,
                                             int yb, int ys, int cnt, const float *F, int8_t *q, const float *h,
                                             Flip *fl, int *nfl, uint32_t *trace, int t0, int nthr) {
    const int N = T.N, m = T.m;
    for (int t = t0; t < cnt; t += nthr) {
        int y = yb + t * ys;
        u32x4 r = draw(T.seed, (uint32_t)k, (uint32_t)y, step, tag);
        int x = draw_index(r.x, N);
        float u = draw_unit(r.y);
        size_t o = (size_t)y * N + x;
        float qyx = q[o];
        float dE, qL = 0.f, qR = 0.f;
        if (sa) {
            dE = dense_sa_dE(qyx, h[x], F[o]);
        } else {
            int yl = y == 0 ? m - 1 : y - 1, yr = y == m - 1 ? 0 : y + 1;
            qL = q[(size_t)yl * N + x];
            qR = q[(size_t)yr * N + x];
            dE = dense_sqa_dE(qyx, h[x], F[o], qL, qR, sc.twoDivM, sc.coef);
        }
        int nearT = 0;
        const float L = neg_log_unit(u);
        int acc = metropolis_log(dE, sc.rate, L, trial_xtol(tol, h[x], __fmul_rn(2.f, F[o]), L), nearT);
        if (nearT) acc = exact_dense_accept(T, sa, x, qyx, q + (size_t)y * N, qL, qR, G, beta, u);
        if (acc) {
            q[o] = (int8_t)(-qyx);
            int slot = atomicAdd(nfl, 1);
            fl[slot] = Flip{y, x, -2.f * qyx};
            if (trace) {
                uint32_t bit = (uint32_t)k * (uint32_t)m + (uint32_t)y;
                atomicOr(&trace[bit >> 5], 1u << (bit & 31));
            }
        }
    }
}

// Trotters of colour phase ph (0: even y < 2 (m/2); 1: y = m - 1 when m is odd;
// 2: odd y) of the coloring sweep; cnt = 0 for an empty phase.
__device__ __forceinline__ void color_phase(int m, int ph, int &yb, int &ys, int &cnt) {
    if (ph == 0) {
        yb = 0; ys = 2; cnt = m / 2;
    } else if (ph == 1) {
        yb = m - 1; ys = 1; cnt = m & 1;
    } else {
        yb = 1; ys = 2; cnt = m / 2;
    }
}

// One CTA anneals one instance (all trotters) for steps [s0, s0 + nSteps) of
// its schedule.  Spins, fields and h are staged in shared memory when they
// fit; otherwise the CTA works on global memory.  Returns false, without
// touching the instance, when smemBytes cannot hold the flip lists.
__device__ bool anneal_instance(const sq103_dense_task &T, unsigned char *smem, int smemBytes, int s0, int nSteps) {
    const int N = T.N, m = T.m, tid = threadIdx.x;
    const size_t off = flip_list_bytes(m);
    if (off > (size_t)smemBytes) {
        if (tid == 0 && T.status) atomicExch(T.status, kErrCapacity);
        return false;
    }
    Flip *flips = reinterpret_cast<Flip *>(smem);            // 3 x m
    int *nflip = reinterpret_cast<int *>(flips + 3 * m);      // 3 counters
    size_t stageBytes = (size_t)m * N * 4 + (size_t)N * 4 + (size_t)m * N;
    const bool stage = off + stageBytes <= (size_t)smemBytes;
    float *F;
    const float *h;
    int8_t *q;
    if (stage) {
        F = reinterpret_cast<float *>(smem + off);
        float *hs = F + (size_t)m * N;
        q = reinterpret_cast<int8_t *>(hs + N);
        for (size_t i = tid; i < (size_t)m * N; i += kBlockThreads) {
            F[i] = T.F[i];
            q[i] = T.q[i];
        }
        for (int i = tid; i < N; i += kBlockThreads) hs[i] = T.h[i];
        h = hs;
    } else {
        F = T.F;
        h = T.h;
        q = T.q;
    }
    if (tid < 3) nflip[tid] = 0;
    __syncthreads();

    const uint32_t wordsPerStep = (uint32_t)(((size_t)N * m + 31) / 32);
    const bool pipelined = T.algo == kColoring && m >= 2;
    const int decideThreads = m > 64 ? 64 : 32;
    const int accTid = pipelined ? decideThreads : 0;  // the one thread that counts accepted flips
    unsigned long long accepted = 0;
    int buf = 0;  // flip list of the next phase (sequential order)
    __shared__ Flip naiveFlip;
    __shared__ int naiveAcc;

    if (pipelined) {
        // Coloring with at least two trotters: consecutive phases hold disjoint
        // trotter rows, and a phase reads only its own field rows and its
        // neighbours' spins.  So the first decideThreads threads take the trials
        // of phase p while the others apply the flips of phase p - 1; one barrier
        // per phase.  A phase's rows were last updated two or more phases back,
        // before a barrier.  Flip lists rotate over three buffers: the one being
        // filled, the one being applied, and the next one, whose counter is
        // cleared meanwhile.  Each field row still takes its trotter's flips in
        // trial order, so fields are bit-identical to the sequential order.
        int bc = 0;            // list of the phase being decided
        bool pending = false;  // the previous phase's list waits to be applied
        const int applyThreads = kBlockThreads - decideThreads;
        for (int s = s0; s <= s0 + nSteps; ++s) {
            const bool last = s == s0 + nSteps;  // one more stage applies the final phase
            float G = 0.f, beta = 0.f;
            if (!last) {
                G = T.G ? T.G[s] : T.Gs;
                beta = T.beta ? T.beta[s] : T.betas;
            }
            const StepConst sc = step_const(T.algo, m, G, beta);
            const DecisionTol tol = decision_tol(false, true, sc.twoDivM, sc.coef, sc.rate);
            const uint32_t step = T.step0 + (uint32_t)s;
            uint32_t *trace = T.trace && !last ? T.trace + (size_t)(s - s0) * wordsPerStep : nullptr;
            for (int k = 0; k < (last ? 1 : N); ++k) {
                for (int ph = 0; ph < 3; ++ph) {
                    int yb = 0, ys = 1, cnt = 0;
                    if (!last) {
                        color_phase(m, ph, yb, ys, cnt);
                        if (cnt == 0) continue;
                    } else if (ph) {
                        break;
                    }
                    const int bp = bc == 0 ? 2 : bc - 1, bn = bc == 2 ? 0 : bc + 1;
                    if (tid < decideThreads) {
                        if (!last)
                            decide_phase(T, false, kTagDenseSweep, sc, tol, G, beta, step, k, yb, ys, cnt, F, q, h,
                                         flips + bc * m, nflip + bc, trace, tid, decideThreads);
                    } else {
                        if (pending) {
                            const int nf = nflip[bp];
                            apply_flips(flips + bp * m, nf, F, T.J, T.ldJ, N, tid - decideThreads, applyThreads);
                            if (tid == accTid) accepted += (unsigned long long)nf;
                        }
                        if (tid == accTid) nflip[bn] = 0;
                    }
                    __syncthreads();
                    pending = !last;
                    bc = bn;
                }
            }
        }
    }

    for (int s = s0; s < s0 + nSteps && !pipelined; ++s) {
        const float G = T.G ? T.G[s] : T.Gs, beta = T.beta ? T.beta[s] : T.betas;
        const StepConst sc = step_const(T.algo, m, G, beta);
        const DecisionTol tol = decision_tol(T.algo == kSANaive, true, sc.twoDivM, sc.coef, sc.rate);
        const uint32_t step = T.step0 + (uint32_t)s;
        uint32_t *trace = T.trace ? T.trace + (size_t)(s - s0) * wordsPerStep : nullptr;

        if (T.algo == kNaive) {
            const long long nTrials = (long long)N * m;
            for (long long t = 0; t < nTrials; ++t) {
                if (tid == 0) {
                    u32x4 r = draw(T.seed, (uint32_t)t, 0u, step, kTagDenseNaive);
                    int y = draw_index(r.x, m), x = draw_index(r.y, N);
                    float u = draw_unit(r.z);
                    size_t o = (size_t)y * N + x;
                    float qyx = q[o];
                    int yl = y == 0 ? m - 1 : y - 1, yr = y == m - 1 ? 0 : y + 1;
                    const float qL = q[(size_t)yl * N + x], qR = q[(size_t)yr * N + x];
                    float dE = dense_sqa_dE(qyx, h[x], F[o], qL, qR, sc.twoDivM, sc.coef);
                    int nearT = 0;
                    const float L = neg_log_unit(u);
                    int acc = metropolis_log(dE, sc.rate, L, trial_xtol(tol, h[x], __fmul_rn(2.f, F[o]), L), nearT);
                    if (nearT) acc = exact_dense_accept(T, false, x, qyx, q + (size_t)y * N, qL, qR, G, beta, u);
                    if (acc) {
                        q[o] = (int8_t)(-qyx);
                        naiveFlip = Flip{y, x, -2.f * qyx};
                        if (trace) atomicOr(&trace[t >> 5], 1u << (t & 31));
                        ++accepted;
                    }
                    naiveAcc = acc;
                }
                __syncthreads();
                if (naiveAcc) apply_flips(&naiveFlip, 1, F, T.J, T.ldJ, N, tid, kBlockThreads);
                __syncthreads();
            }
            continue;
        }

        // sa_naive, and coloring with one trotter: each phase's trials need the
        // previous phase's flips applied to the same rows.
        // Two flip lists alternate; the idle one's counter is cleared while the
        // other is applied, so it is zero when the next phase appends to it.
        const bool sa = (T.algo == kSANaive);
        const uint32_t tag = sa ? kTagDenseSA : kTagDenseSweep;
        for (int k = 0; k < N; ++k) {
            for (int ph = 0; ph < 3; ++ph) {
                int yb, ys, cnt;
                if (sa) {
                    if (ph) break;
                    yb = 0; ys = 1; cnt = m;
                } else {
                    color_phase(m, ph, yb, ys, cnt);
                    if (cnt == 0) continue;
                }
                Flip *fl = flips + buf * m;
                decide_phase(T, sa, tag, sc, tol, G, beta, step, k, yb, ys, cnt, F, q, h, fl, nflip + buf, trace,
                             tid, kBlockThreads);
                __syncthreads();
                const int nf = nflip[buf];
                apply_flips(fl, nf, F, T.J, T.ldJ, N, tid, kBlockThreads);
                if (tid == 0) {
                    nflip[buf ^ 1] = 0;
                    accepted += (unsigned long long)nf;
                }
                __syncthreads();
                buf ^= 1;
            }
        }
    }

    if (tid == accTid && T.accepted) atomicAdd(T.accepted, accepted);
    if (stage) {
        for (size_t i = tid; i < (size_t)m * N; i += kBlockThreads) {
            T.F[i] = F[i];
            T.q[i] = q[i];
        }
    }
    __syncthreads();  // shared memory is reused by the CTA's next instance
    return true;
}

__global__ void __launch_bounds__(kBlockThreads) dense_sweep_cta(const sq103_dense_task *tasks,
                                                                 sq103_dense_task single, int smemBytes) {
    extern __shared__ __align__(16) unsigned char smem[];
    const sq103_dense_task T = tasks ? tasks[blockIdx.x] : single;
    anneal_instance(T, smem, smemBytes, 0, T.nSteps);
}

// Persistent batch: CTAs take instances from a queue (order[] lists them
// largest first); instance i runs steps [pos[i], pos[i] + stepsPerLaunch) of
// its own schedule (T.nSteps steps in total) and advances pos[i], so the same
// launch replayed from a CUDA graph moves every instance one step further.
__global__ void __launch_bounds__(kBlockThreads) dense_batch_persistent(const sq103_dense_task *tasks,
                                                                        int nTasksHost, const int *nTasksDev,
                                                                        const int *order, int *pos, int *queue,
                                                                        int stepsPerLaunch, int smemBytes) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int item;
    const int nTasks = nTasksDev ? *nTasksDev : nTasksHost;
    for (;;) {
        if (threadIdx.x == 0) item = atomicAdd(queue, 1);
        __syncthreads();
        const int idx = item;
        __syncthreads();
        if (idx >= nTasks) break;
        const int ti = order ? order[idx] : idx;
        const sq103_dense_task T = tasks[ti];
        const int s0 = pos[ti];
        const int n = min(stepsPerLaunch, T.nSteps - s0);
        if (n > 0 && anneal_instance(T, smem, smemBytes, s0, n) && threadIdx.x == 0) pos[ti] = s0 + n;
    }
    // the last CTA to leave resets the queue for the next replay
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(queue + 1, 1) == (int)gridDim.x - 1) {
            queue[0] = 0;
            queue[1] = 0;
        }
    }
}

__global__ void randomize_kernel(int8_t *q, int N, int m, uint64_t seed, uint32_t step, uint32_t tag) {
    int chunks = (N + 127) / 128;
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)m * chunks) return;
    int y = (int)(idx / chunks), c = (int)(idx - (long long)y * chunks);
    u32x4 r = draw(seed, (uint32_t)c, (uint32_t)y, step, tag);
    uint32_t w[4] = {r.x, r.y, r.z, r.w};
    int8_t *qy = q + (size_t)y * N + (size_t)c * 128;
    int nb = min(128, N - c * 128);
    for (int b = 0; b < nb; ++b) qy[b] = ((w[b >> 5] >> (b & 31)) & 1u) ? 1 : -1;
}

static int g_max_smem = -1;

// largest dynamic shared memory the CTA kernel may use (opt-in limit minus its
// static shared memory); sets the kernel attribute once per process
static int max_dyn_smem() {
    if (g_max_smem < 0) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncAttributes fa;
        cudaFuncGetAttributes(&fa, dense_sweep_cta);
        int dyn = v - (int)fa.sharedSizeBytes;
        if (cudaFuncSetAttribute(dense_sweep_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess) {
            cudaGetLastError();
            dyn = 48 * 1024 - (int)fa.sharedSizeBytes;
        }
        g_max_smem = dyn;
    }
    return g_max_smem;
}

static size_t cta_smem_bytes(int N, int m) {
    size_t base = flip_list_bytes(m);
    size_t stage = (size_t)m * N * 4 + (size_t)N * 4 + (size_t)m * N;
    size_t lim = (size_t)max_dyn_smem();
    if (base + stage <= lim) return base + stage;
    return base;
}

}  // namespace sq103

using namespace sq103;

extern "C" {

SQ103_API int sq103_randomize_spins(int8_t *q, int N, int m, uint64_t seed, uint32_t step, int tagSide,
                                    void *stream) {
    if (N <= 0 || m <= 0) return kErrBadShape;
    long long n = (long long)m * ((N + 127) / 128);
    int blocks = (int)((n + 255) / 256);
    randomize_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(q, N, m, seed, step,
                                                               (uint32_t)kTagRandomize | ((uint32_t)tagSide << 8));
    return (int)cudaGetLastError();
}

int sq103_dense_anneal_multi(const sq103_dense_task *t, void *stream);

SQ103_API int sq103_dense_anneal(const sq103_dense_task *task, void *stream) {
    if (!task || task->N <= 0 || task->m <= 0 || task->nSteps < 0) return kErrBadShape;
    if (task->nSteps == 0) return 0;
    // one CTA per trotter when the shape allows it (or when asked to), else one CTA
    const bool rowsAligned = !(task->ldJ & 3) && !(reinterpret_cast<uintptr_t>(task->J) & 15);
    const int kernel = task->flags & kFlagKernelMask;
    bool multi = kernel == 2 ||
                 (kernel == 0 && task->ws && rowsAligned &&
                  task->wsBytes >= sq103_dense_ws_bytes(task->N, task->m, task->nSteps) &&
                  sq103_dense_multicta_ok(task->N, task->m, task->algo));
    if (multi) {
        if (!sq103_dense_multicta_ok(task->N, task->m, task->algo)) return kErrBadShape;
        return sq103_dense_anneal_multi(task, stream);
    }
    size_t smem = cta_smem_bytes(task->N, task->m);
    if (smem > (size_t)max_dyn_smem()) return kErrBadShape;  // flip lists alone do not fit
    dense_sweep_cta<<<1, kBlockThreads, smem, (cudaStream_t)stream>>>(nullptr, *task, (int)smem);
    return (int)cudaGetLastError();
}

// dynamic shared memory limit of the persistent batch kernel (opt-in limit minus
// its own static shared memory); sets the attribute once per process
static int batch_dyn_smem() {
    static int lim = -1;
    if (lim < 0) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncAttributes fa;
        cudaFuncGetAttributes(&fa, dense_batch_persistent);
        lim = v - (int)fa.sharedSizeBytes;
        if (cudaFuncSetAttribute(dense_batch_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) !=
            cudaSuccess) {
            cudaGetLastError();
            lim = 48 * 1024 - (int)fa.sharedSizeBytes;
        }
    }
    return lim;
}

SQ103_API int sq103_dense_batch_max_smem(void) { return batch_dyn_smem(); }

SQ103_API int sq103_dense_batch_min_smem(int maxM) { return maxM > 0 ? (int)flip_list_bytes(maxM) : 0; }

SQ103_API int sq103_dense_batch_ctas_per_sm(int smemBytes) {
    int perSm = 0;
    if (smemBytes > batch_dyn_smem()) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, dense_batch_persistent, kBlockThreads, smemBytes) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return perSm;
}

SQ103_API int sq103_dense_batch_launch(const sq103_dense_task *d_tasks, int nTasks, const int *d_nTasks,
                                       const int *d_order, int *d_pos, int *d_queue, int stepsPerLaunch, int grid,
                                       int smemBytes, void *stream) {
    if (nTasks <= 0 && !d_nTasks) return 0;
    if (grid <= 0 || smemBytes < 0 || smemBytes > batch_dyn_smem()) return kErrBadShape;
    dense_batch_persistent<<<grid, kBlockThreads, smemBytes, (cudaStream_t)stream>>>(
        d_tasks, nTasks, d_nTasks, d_order, d_pos, d_queue, stepsPerLaunch, smemBytes);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_dense_anneal_batch(const sq103_dense_task *d_tasks, int nTasks, int maxN, int maxM,
                                       void *stream) {
    if (nTasks <= 0) return 0;
    size_t smem = cta_smem_bytes(maxN, maxM);
    if (smem > (size_t)max_dyn_smem()) return kErrBadShape;
    sq103_dense_task dummy = {};
    dense_sweep_cta<<<nTasks, kBlockThreads, smem, (cudaStream_t)stream>>>(d_tasks, dummy, (int)smem);
    return (int)cudaGetLastError();
}

}  // extern "C"
