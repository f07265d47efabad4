// bipartite.cu -- bipartite-graph Suzuki-Trotter / SA sweeps.
//
// One annealOneStep = a half-step on side 1 followed by a half-step on side 0
// (CUDABipartiteGraphAnnealer::annealOneStepSQA, sqaodc/cuda/CUDABipartiteGraphAnnealer.cu:539-560;
// CPUBipartiteGraphAnnealer::annealOneStepColoringParallel, sqaodc/cpu/CPUBipartiteGraphAnnealer.cpp:434-441).
// A half-step computes the fields of the moving side from the fixed side
// (F1 = q0 J^T or F0 = q1 J, spin GEMM), then flips every spin of the moving
// side in colour phases: even trotters, trotter m-1 when m is odd, odd
// trotters.  Spin i of trotter y draws u from philox((i, y, step, 0x31 | side << 8)).w1:
//   dE = (2/m) q (h + F) - q (q_{y-1} + q_{y+1}) coef  (SQA),  2 q (h + F)  (SA, 0x32).
// Unlike the reference GPU kernel (which feeds trotters 2g and 2g+1 the same
// uniform, CUDABipartiteGraphAnnealer.cu:486,499) every trial has its own draw.
//
// naive: (N0+N1) m sequential trials at (x, y) = (hi(w0 (N0+N1)), hi(w1 m)) of
// philox((t, 0, step, 0x33)) (CPUBipartiteGraphAnnealer.cpp:290-328);
// sa_naive: per trotter, (N0+N1) m trials at x = hi(w0 (N0+N1)) of
// philox((t, y, step, 0x34)) (CPUBipartiteGraphAnnealer.cpp:446-480).
// The naive fields are a fixed-order block reduction of one J row or column.
#include "bip_field.cuh"
#include "sq_common.cuh"
#include "sq_kernels.h"

namespace sq103 {

// The fixed side of a half-step, for the exact field of a flagged trial:
// side 1 moves -> F1[y][i] = sum_j J[i][j] q0[y][j] (row i of J); side 0 moves ->
// F0[y][j] = sum_i J[i][j] q1[y][i] (column j, stride N0).
// The FP64 couplings of a <double> problem (J64, and h64 of the moving side) take
// the place of the fp32 ones when present.
struct BipFixed {
    const float *J;
    int N0;
    const int8_t *qB;  // spins of the fixed side, m x NB
    int NB;
    int side;          // the moving side
    float G, beta;
    const double *J64, *h64;
};

__device__ __forceinline__ double bip_exact_field(const BipFixed &B, int y, int i) {
    const int8_t *qb = B.qB + (size_t)y * B.NB;
    if (B.J64)
        return B.side ? exact_field_thread(B.J64 + (size_t)i * B.N0, 1, qb, B.NB)
                      : exact_field_thread(B.J64 + i, (size_t)B.N0, qb, B.NB);
    return B.side ? exact_field_thread(B.J + (size_t)i * B.N0, 1, qb, B.NB)
                  : exact_field_thread(B.J + i, (size_t)B.N0, qb, B.NB);
}

__device__ __forceinline__ double bip_exact_h(const BipFixed &B, const float *h, int i) {
    return B.h64 ? B.h64[i] : (double)h[i];
}

// one colour-phase trial of spin i of trotter y on the moving side; returns 1 if accepted
__device__ __forceinline__ int bip_trial(int8_t *qA, const float *F, const float *h, int Ns, int m, int y, int i,
                                         uint64_t seed, uint32_t step, uint32_t tag, const StepConst &sc, int algo,
                                         uint32_t *trace, unsigned long long bitBase, const BipFixed &B) {
    u32x4 r = draw(seed, (uint32_t)i, (uint32_t)y, step, tag);
    float u = draw_unit(r.y);
    size_t o = (size_t)y * Ns + i;
    float qyx = qA[o];
    float dE, qL = 0.f, qR = 0.f;
    const bool sa = algo == kSAColoring;
    if (sa) {
        dE = bip_sa_dE(qyx, h[i], F[o]);
    } else {
        int yl = y == 0 ? m - 1 : y - 1, yr = y == m - 1 ? 0 : y + 1;
        qL = qA[(size_t)yl * Ns + i];
        qR = qA[(size_t)yr * Ns + i];
        dE = bip_sqa_dE(qyx, h[i], F[o], qL, qR, sc.twoDivM, sc.coef);
    }
    int nearT = 0;
    const float L = neg_log_unit(u);
    const DecisionTol tol = decision_tol(sa, false, sc.twoDivM, sc.coef, sc.rate);
    int acc = metropolis_log(dE, sc.rate, L, trial_xtol(tol, h[i], F[o], L), nearT);
    if (nearT)
        acc = exact_accept(sa, false, qyx, bip_exact_h(B, h, i), bip_exact_field(B, y, i), qL, qR, m, B.G, B.beta, u);
    if (!acc) return 0;
    qA[o] = (int8_t)(-qyx);
    if (trace) {
        unsigned long long bit = bitBase + o;
        atomicOr(&trace[bit >> 5], 1u << (bit & 31));
    }
    return 1;
}

__global__ void __launch_bounds__(256) bip_flip_phase(int8_t *qA, const float *F, const float *h, int Ns, int m,
                                                      int yb, int ys, int cnt, uint64_t seed, uint32_t step,
                                                      uint32_t tag, const float *Gp, const float *bp, float Gsc, float bsc,
                                                      int algo, uint32_t *trace, unsigned long long bitBase,
                                                      unsigned long long *accepted, BipFixed B) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool active = idx < (long long)cnt * Ns;
    int acc = 0;
    if (active) {
        const float G = Gp ? *Gp : Gsc, beta = bp ? *bp : bsc;
        StepConst sc = step_const(algo, m, G, beta);
        int t = (int)(idx / Ns), i = (int)(idx - (long long)t * Ns);
        B.G = G;
        B.beta = beta;
        acc = bip_trial(qA, F, h, Ns, m, yb + t * ys, i, seed, step, tag, sc, algo, trace, bitBase, B);
    }
    if (accepted) {
        unsigned ballot = __ballot_sync(0xffffffffu, acc);
        if ((threadIdx.x & 31) == 0 && ballot) atomicAdd(accepted, (unsigned long long)__popc(ballot));
    }
}

// All colour phases of one SQA half-step in one launch.  A trial's neighbours
// are the same spin index in the adjacent trotters, so a block that owns whole
// columns (spin i of every trotter) orders the phases with __syncthreads:
// even trotters, then trotter m-1 when m is odd, then odd trotters.  Thread t
// of a block takes column i0 + t % C and trotter pairs t / C, t / C + 256 / C,
// ... (C columns per block, chosen so the pairs of a column fill the block);
// the trials, their draws and their arithmetic are those of bip_flip_phase, so
// the spins, trace and accepted count are identical, with one launch per
// half-step in place of two or three.
__global__ void __launch_bounds__(256) bip_flip_half(int8_t *qA, const float *F, const float *h, int Ns, int m, int C,
                                                     uint64_t seed, uint32_t step, uint32_t tag, const float *Gp,
                                                     const float *bp, float Gsc, float bsc, int algo, uint32_t *trace,
                                                     unsigned long long bitBase, unsigned long long *accepted,
                                                     BipFixed B) {
    const int t = (int)threadIdx.x;
    const int i = (int)blockIdx.x * C + t % C, p0 = t / C, pStride = (int)blockDim.x / C;
    const bool col = t < pStride * C && i < Ns;
    const float G = Gp ? *Gp : Gsc, beta = bp ? *bp : bsc;
    const StepConst sc = step_const(algo, m, G, beta);
    B.G = G;
    B.beta = beta;
    const int pairs = m / 2;
    unsigned long long acc = 0;
    for (int ph = 0; ph < 3; ++ph) {
        if (ph == 1 && !(m & 1)) continue;
        if (col) {
            if (ph == 1) {
                if (p0 == 0) acc += bip_trial(qA, F, h, Ns, m, m - 1, i, seed, step, tag, sc, algo, trace, bitBase, B);
            } else {
                for (int p = p0; p < pairs; p += pStride)
                    acc += bip_trial(qA, F, h, Ns, m, 2 * p + (ph == 2 ? 1 : 0), i, seed, step, tag, sc, algo, trace,
                                     bitBase, B);
            }
        }
        __syncthreads();
    }
    if (accepted) {
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0 && acc) atomicAdd(accepted, acc);
    }
}

// columns per block of bip_flip_half: the trotter pairs of a column fill the block
static int flip_half_cols(int m) {
    const int pairs = std::max(1, m / 2);
    return pairs >= 256 ? 1 : 256 / pairs;
}

// fixed-order block sum (256 threads) in fp32
__device__ float block_sum_f32(float v, float *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    float r = 0.f;
    if (warp == 0) {
        r = lane < 8 ? red[lane] : 0.f;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;
}

// field on spin x of `side` in trotter y (fixed-order reduction)
__device__ float bip_field_at(const sq103_bipartite_task &T, int side, int y, int x, float *red) {
    float s = 0.f;
    if (side == 0) {
        for (int i = threadIdx.x; i < T.N1; i += 256)
            s = __fmaf_rn(T.J[(size_t)i * T.N0 + x], (float)T.q1[(size_t)y * T.N1 + i], s);
    } else {
        for (int j = threadIdx.x; j < T.N0; j += 256)
            s = __fmaf_rn(T.J[(size_t)x * T.N0 + j], (float)T.q0[(size_t)y * T.N0 + j], s);
    }
    return block_sum_f32(s, red);
}

// naive (one CTA, grid 1) or sa_naive (one CTA per trotter)
__global__ void __launch_bounds__(256) bip_naive(sq103_bipartite_task T, int s) {
    __shared__ float red[8];
    __shared__ int sx, sy, sside;
    __shared__ float su;
    const bool sa = T.algo == kSANaive;
    const StepConst sc = step_const(T.algo, T.m, T.G ? T.G[s] : T.Gs, T.beta ? T.beta[s] : T.betas);
    const uint32_t step = T.step0 + (uint32_t)s;
    const int Ntot = T.N0 + T.N1;
    const long long perY = (long long)Ntot * T.m;
    const int yFixed = blockIdx.x;
    unsigned long long accepted = 0;
    for (long long t = 0; t < perY; ++t) {
        if (threadIdx.x == 0) {
            u32x4 r = draw(T.seed, (uint32_t)t, sa ? (uint32_t)yFixed : 0u, step, sa ? kTagBipSANaive : kTagBipNaive);
            int x = draw_index(r.x, Ntot);
            sy = sa ? yFixed : draw_index(r.y, T.m);
            su = draw_unit(sa ? r.y : r.z);
            sside = x < T.N0 ? 0 : 1;
            sx = sside ? x - T.N0 : x;
        }
        __syncthreads();
        int x = sx, y = sy, side = sside;
        float F = bip_field_at(T, side, y, x, red);
        if (threadIdx.x == 0) {
            int Ns = side ? T.N1 : T.N0;
            int8_t *qA = side ? T.q1 : T.q0;
            const float *h = side ? T.h1 : T.h0;
            float qyx = qA[(size_t)y * Ns + x];
            float dE;
            if (sa) {
                dE = bip_sa_dE(qyx, h[x], F);
            } else {
                int yl = y == 0 ? T.m - 1 : y - 1, yr = y == T.m - 1 ? 0 : y + 1;
                dE = bip_sqa_dE(qyx, h[x], F, qA[(size_t)yl * Ns + x], qA[(size_t)yr * Ns + x], sc.twoDivM,
                                sc.coef);
            }
            int nearT = 0;
            const float L = neg_log_unit(su);
            const DecisionTol tol = decision_tol(sa, false, sc.twoDivM, sc.coef, sc.rate);
            int acc = metropolis_log(dE, sc.rate, L, trial_xtol(tol, h[x], F, L), nearT);
            if (nearT) {
                const int NB = side ? T.N0 : T.N1;
                const BipFixed B = {T.J, T.N0, side ? T.q0 : T.q1, NB, side, 0.f, 0.f, T.J64,
                                    side ? T.h1_64 : T.h0_64};
                const float qL = sa ? 0.f : qA[(size_t)(y == 0 ? T.m - 1 : y - 1) * Ns + x];
                const float qR = sa ? 0.f : qA[(size_t)(y == T.m - 1 ? 0 : y + 1) * Ns + x];
                acc = exact_accept(sa, false, qyx, bip_exact_h(B, h, x), bip_exact_field(B, y, x), qL, qR, T.m,
                                   T.G ? T.G[s] : T.Gs, T.beta ? T.beta[s] : T.betas, su);
            }
            if (acc) {
                qA[(size_t)y * Ns + x] = (int8_t)(-qyx);
                ++accepted;
                if (T.trace) {
                    unsigned long long bit = (sa ? (unsigned long long)yFixed * perY : 0ull) + (unsigned long long)t;
                    uint32_t *tr = T.trace + (size_t)s * ((perY * (sa ? T.m : 1) + 31) / 32);
                    atomicOr(&tr[bit >> 5], 1u << (bit & 31));
                }
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && T.accepted) atomicAdd(T.accepted, accepted);
}

// Persistent batch of bipartite instances (coloring / sa_coloring): one CTA
// runs a whole annealOneStep of one instance -- both half-step field GEMMs
// (the bip_field tiles, looped by the CTA) and the colour phases -- for steps
// [pos[i], pos[i] + stepsPerLaunch) of its schedule.  Same arithmetic as
// sq103_bipartite_anneal, so results are bit-identical.
__global__ void __launch_bounds__(256) bip_batch_persistent(const sq103_bipartite_task *tasks, const int *nTasksDev,
                                                            int nTasksHost, const int *order, int *pos, int *queue,
                                                            int stepsPerLaunch) {
    extern __shared__ __align__(16) float smem[];  // kBipFieldSmem bytes: field tile staging
    __shared__ int item;
    const int nTasks = nTasksDev ? *nTasksDev : nTasksHost;
    for (;;) {
        if (threadIdx.x == 0) item = atomicAdd(queue, 1);
        __syncthreads();
        const int idx = item;
        __syncthreads();
        if (idx >= nTasks) break;
        const int ti = order ? order[idx] : idx;
        const sq103_bipartite_task T = tasks[ti];
        const int s0 = pos[ti];
        const int n = min(stepsPerLaunch, T.nSteps - s0);
        const int m = T.m, m2 = (m / 2) * 2;
        const bool sa = T.algo == kSAColoring;
        unsigned long long accepted = 0;
        for (int s = s0; s < s0 + n; ++s) {
            const StepConst sc = step_const(T.algo, m, T.G ? T.G[s] : T.Gs, T.beta ? T.beta[s] : T.betas);
            const uint32_t step = T.step0 + (uint32_t)s;
            for (int hs = 0; hs < 2; ++hs) {
                const int side = hs == 0 ? 1 : 0;
                const int Ns = side ? T.N1 : T.N0;
                int8_t *qA = side ? T.q1 : T.q0;
                float *F = side ? T.F1 : T.F0;
                const float *h = side ? T.h1 : T.h0;
                for (int ty = 0; ty < m; ty += kBipTileM)
                    for (int tx = 0; tx < Ns; tx += kBipTileN) {
                        if (side)
                            bip_field_tile<true, false, float>(T.q0, T.N0, T.J, T.N0, F, T.N1, m, T.N1, T.N0, ty,
                                                               tx, smem);
                        else
                            bip_field_tile<false, false, float>(T.q1, T.N1, T.J, T.N0, F, T.N0, m, T.N0, T.N1, ty,
                                                                tx, smem);
                    }
                const uint32_t tag = (uint32_t)(sa ? kTagBipSA : kTagBipSweep) | ((uint32_t)side << 8);
                const BipFixed B = {T.J, T.N0, side ? T.q0 : T.q1, side ? T.N0 : T.N1, side,
                                    T.G ? T.G[s] : T.Gs, T.beta ? T.beta[s] : T.betas, T.J64,
                                    side ? T.h1_64 : T.h0_64};
                for (int ph = 0; ph < 3; ++ph) {
                    int yb, ys, cnt;
                    if (sa) {
                        if (ph) break;
                        yb = 0; ys = 1; cnt = m;
                    } else if (ph == 0) {
                        yb = 0; ys = 2; cnt = m2 / 2;
                    } else if (ph == 1) {
                        if (!(m & 1)) continue;
                        yb = m - 1; ys = 1; cnt = 1;
                    } else {
                        yb = 1; ys = 2; cnt = m2 / 2;
                    }
                    for (long long k = threadIdx.x; k < (long long)cnt * Ns; k += blockDim.x) {
                        int t = (int)(k / Ns), i = (int)(k - (long long)t * Ns);
                        accepted += bip_trial(qA, F, h, Ns, m, yb + t * ys, i, T.seed, step, tag, sc, T.algo, nullptr, 0,
                                              B);
                    }
                    __syncthreads();
                }
            }
        }
        if (n > 0) {
            if (T.accepted) atomicAdd(T.accepted, accepted);
            if (threadIdx.x == 0) pos[ti] = s0 + n;
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(queue + 1, 1) == (int)gridDim.x - 1) {
            queue[0] = 0;
            queue[1] = 0;
        }
    }
}

}  // namespace sq103

using namespace sq103;

extern "C" SQ103_API int sq103_bipartite_batch_launch(const sq103_bipartite_task *d_tasks, int nTasks,
                                                      const int *d_nTasks, const int *d_order, int *d_pos,
                                                      int *d_queue, int stepsPerLaunch, int grid, void *stream) {
    if (grid <= 0) return kErrBadShape;
    // the field tiles' 48 KB plus the kernel's own words exceed the default limit
    cudaError_t e = cudaFuncSetAttribute(bip_batch_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kBipFieldSmem);
    if (e != cudaSuccess) return (int)e;
    bip_batch_persistent<<<grid, 256, kBipFieldSmem, (cudaStream_t)stream>>>(d_tasks, d_nTasks, nTasks, d_order,
                                                                             d_pos, d_queue, stepsPerLaunch);
    return (int)cudaGetLastError();
}

extern "C" SQ103_API int sq103_bipartite_anneal(const sq103_bipartite_task *task, void *stream) {
    if (!task) return kErrBadShape;
    const sq103_bipartite_task &T = *task;
    if (T.N0 <= 0 || T.N1 <= 0 || T.m <= 0) return kErrBadShape;
    cudaStream_t st = (cudaStream_t)stream;
    const int m = T.m, m2 = (m / 2) * 2;
    for (int s = 0; s < T.nSteps; ++s) {
        const uint32_t step = T.step0 + (uint32_t)s;
        if (T.algo == kNaive || T.algo == kSANaive) {
            bip_naive<<<T.algo == kSANaive ? m : 1, 256, 0, st>>>(T, s);
            continue;
        }
        const bool sa = T.algo == kSAColoring;
        const unsigned long long wordsPerStep = ((unsigned long long)m * (T.N0 + T.N1) + 31) / 32;
        uint32_t *trace = T.trace ? T.trace + (size_t)s * wordsPerStep : nullptr;
        unsigned long long bitBase = 0;
        for (int hs = 0; hs < 2; ++hs) {
            const int side = hs == 0 ? 1 : 0;
            const int Ns = side ? T.N1 : T.N0;
            int8_t *qA = side ? T.q1 : T.q0;
            float *F = side ? T.F1 : T.F0;
            const float *h = side ? T.h1 : T.h0;
            if (T.digits1 && T.digits0) {
                // side 1: F1 = q0 J^T (rows of J, K = N0); side 0: F0 = q1 J (rows of J^T, K = N1)
                const int rc = side ? sq103_tc_refresh(T.digits1, T.N1, T.N0, T.q0, T.N0, m, T.spinsBf16, F, T.N1,
                                                       0, T.status, stream)
                                    : sq103_tc_refresh(T.digits0, T.N0, T.N1, T.q1, T.N1, m, T.spinsBf16, F, T.N0,
                                                       0, T.status, stream);
                if (rc != 0) return rc;
            } else {
                sq103_bipartite_fields(T.J, T.N0, T.N1, side ? T.q0 : T.q1, side, F, m, stream);
            }
            const uint32_t tag = (uint32_t)(sa ? kTagBipSA : kTagBipSweep) | ((uint32_t)side << 8);
            const BipFixed fixedSide{T.J, T.N0, side ? T.q0 : T.q1, side ? T.N0 : T.N1, side, 0.f, 0.f, T.J64,
                                     side ? T.h1_64 : T.h0_64};
            if (!sa) {
                // every colour phase of the half-step in one launch (blocks own whole columns)
                const int C = flip_half_cols(m);
                bip_flip_half<<<(Ns + C - 1) / C, 256, 0, st>>>(qA, F, h, Ns, m, C, T.seed, step, tag,
                                                               T.G ? T.G + s : nullptr, T.beta ? T.beta + s : nullptr,
                                                               T.Gs, T.betas, T.algo, trace, bitBase, T.accepted,
                                                               fixedSide);
                bitBase += (unsigned long long)m * Ns;
                continue;
            }
            for (int ph = 0; ph < 3; ++ph) {
                int yb, ys, cnt;
                if (sa) {
                    if (ph) break;
                    yb = 0; ys = 1; cnt = m;
                } else if (ph == 0) {
                    yb = 0; ys = 2; cnt = m2 / 2;
                } else if (ph == 1) {
                    if (!(m & 1)) continue;
                    yb = m - 1; ys = 1; cnt = 1;
                } else {
                    yb = 1; ys = 2; cnt = m2 / 2;
                }
                if (cnt == 0) continue;
                long long n = (long long)cnt * Ns;
                bip_flip_phase<<<(int)((n + 255) / 256), 256, 0, st>>>(qA, F, h, Ns, m, yb, ys, cnt, T.seed, step, tag,
                                                                       T.G ? T.G + s : nullptr,
                                                                       T.beta ? T.beta + s : nullptr, T.Gs, T.betas,
                                                                       T.algo, trace, bitBase, T.accepted,
                                                                       BipFixed{T.J, T.N0, side ? T.q0 : T.q1,
                                                                                side ? T.N0 : T.N1, side, 0.f, 0.f,
                                                                                T.J64, side ? T.h1_64 : T.h0_64});
            }
            bitBase += (unsigned long long)m * Ns;
        }
    }
    return (int)cudaGetLastError();
}
