// dense_multi.cu -- one CTA per trotter: the dense coloring / SA sweep of one
// large instance across the whole GPU (cooperative launch, all CTAs resident).
//
// It runs the same trials, in the same colour order and with the same fp32
// arithmetic, as the one-CTA-per-instance kernel in dense.cu, so both give
// bit-identical spins and fields.
//
// Per CTA (trotter y), 256 threads:
//   warp 0  decider: trials in batches of 32 iterations, lane i = iteration g0+i.
//           Lane i starts from its site's resident field F[y][x_i] (exact
//           through the previous batch) and, as earlier lanes accept, adds
//           d_j * J[x_j][x_i] in trial order (the gathers J[x_j][x_i] are
//           loaded one batch ahead).  The batch's accept bits go to a global
//           accept log, followed by a release store of the progress word.
//   warp 1  helper: for each ring neighbour n (trotters y-1, y+1 in other
//           CTAs) it replays n's Philox site stream into a ring of sites, and
//           applies n's published accept log to a ghost bit row of n's spins.
//   warps 2-7 updaters: after each batch, F[y][:] += d * J[x][:] for the batch's
//           accepted flips, in trial order (float4 rows of J from L2/HBM).
// Colour order: trial (y, k) must see neighbour n after every neighbour trial
// that precedes it (iteration < k, or = k when n's colour phase comes first:
// even trotters, then trotter m-1 if m is odd, then odd trotters).  Only
// neighbour trials at the same site matter, so a trial waits only when a
// neighbour trial inside the not-yet-applied window hit its site; the wait is
// bounded (global timer) and ends the kernel with a timeout status instead of
// hanging.  Before waiting a CTA publishes its own progress, so waits always
// point to strictly earlier trials and cannot form a cycle.
#include <cooperative_groups.h>

#include "sq_common.cuh"
#include "sq_kernels.h"

namespace sq103 {

constexpr int kMcThreads = 256;
constexpr int kMcUpdaters = kMcThreads - 64;
constexpr int kRing = 256;  // iterations of neighbour sites kept (power of two)
constexpr unsigned long long kWaitLimitNs = 4000000000ull;
constexpr int kProgStride = 32;  // progress words on their own 128-byte lines

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void named_bar(int id, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

__host__ __device__ __forceinline__ int colour_phase(int y, int m) {
    if ((m & 1) && y == m - 1) return 1;
    return (y & 1) ? 2 : 0;
}

struct McShared {
    volatile int applied[2];   // neighbour iterations applied to the ghost rows
    volatile int ringHead[2];  // neighbour sites computed for iterations < ringHead
    volatile int done;
    volatile int nflip;
};

__global__ void __launch_bounds__(kMcThreads) dense_sweep_multi(sq103_dense_task T, uint32_t *outLog,
                                                                unsigned *progress, int nWords) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ McShared S;
    const unsigned FULL = 0xffffffffu;
    const int y = blockIdx.x, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = T.N, m = T.m;
    const bool sa = T.algo == kSANaive;
    const int nNbr = sa ? 0 : (m == 2 ? 1 : 2);
    const int nbr0 = (y + m - 1) % m, nbr1 = (y + 1) % m;
    const int Itot = T.nSteps * N;
    const int nWG = (N + 31) / 32;
    const uint32_t tag = sa ? kTagDenseSA : kTagDenseSweep;

    float *Fs = reinterpret_cast<float *>(smem);                 // N
    float *hs = Fs + N;                                          // N
    float *Jgs = hs + N;                                         // 32 x 33 gathers
    uint32_t *ghost = reinterpret_cast<uint32_t *>(Jgs + 32 * 33);  // 2 x nWG
    int *ring = reinterpret_cast<int *>(ghost + 2 * nWG);         // 2 x kRing
    int2 *flips = reinterpret_cast<int2 *>(ring + 2 * kRing);     // 32
    int8_t *qs = reinterpret_cast<int8_t *>(flips + 32);          // N

    for (int i = tid; i < N; i += kMcThreads) {
        Fs[i] = T.F[(size_t)y * N + i];
        hs[i] = T.h[i];
        qs[i] = T.q[(size_t)y * N + i];
    }
    for (int n = 0; n < nNbr; ++n) {
        const int8_t *qn = T.q + (size_t)(n ? nbr1 : nbr0) * N;
        for (int w = tid; w < nWG; w += kMcThreads) {
            uint32_t bits = 0;
            for (int b = 0; b < 32 && w * 32 + b < N; ++b) bits |= (qn[w * 32 + b] > 0 ? 1u : 0u) << b;
            ghost[n * nWG + w] = bits;
        }
    }
    if (tid == 0) {
        S.applied[0] = S.applied[1] = 0;
        S.ringHead[0] = S.ringHead[1] = 0;
        S.done = 0;
        S.nflip = 0;
    }
    // every CTA has read its neighbours' rows before any CTA can finish and
    // write its own row back
    cooperative_groups::this_grid().sync();

    if (warp == 0) {
        // ------------------------------------------------------------ decider
        const int myPh = colour_phase(y, m);
        const int before0 = colour_phase(nbr0, m) < myPh ? 1 : 0;
        const int before1 = colour_phase(nbr1, m) < myPh ? 1 : 0;
        const uint32_t wordsPerStep = (uint32_t)(((size_t)N * m + 31) / 32);
        unsigned long long accepted = 0;
        bool aborted = false;

        // per-lane trial state of the current batch and the next one
        auto trial_setup = [&](int g, int &x, float &u, StepConst &sc, int &s, int &k) {
            s = g / N;
            k = g - s * N;
            u32x4 r = draw(T.seed, (uint32_t)k, (uint32_t)y, T.step0 + (uint32_t)s, tag);
            x = draw_index(r.x, N);
            u = draw_unit(r.y);
            float G = T.G ? T.G[s] : T.Gs, beta = T.beta ? T.beta[s] : T.betas;
            sc = step_const(T.algo, m, G, beta);
        };

        int x = 0, s = 0, k = 0;
        float u = 0.f;
        StepConst sc = {0.f, 0.f, 0.f};
        {
            int g = lane;
            if (g < Itot) trial_setup(g, x, u, sc, s, k);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                int xi = __shfl_sync(FULL, x, i);
                Jgs[lane * 33 + i] = (i < lane && g < Itot) ? __ldg(T.J + (size_t)xi * T.ldJ + x) : 0.f;
            }
            __syncwarp();
        }

        for (int g0 = 0; g0 < Itot && !aborted; g0 += 32) {
            const int nValid = min(32, Itot - g0);
            const bool valid = lane < nValid;
            float Fv = valid ? Fs[x] : 0.f;
            const float hx = valid ? hs[x] : 0.f;

            // next batch: sites and gathers in flight while this batch is decided
            int xN = 0, sN = 0, kN = 0;
            float uN = 0.f;
            StepConst scN = {0.f, 0.f, 0.f};
            const int gN = g0 + 32 + lane;
            const bool validN = gN < Itot;
            if (validN) trial_setup(gN, xN, uN, scN, sN, kN);
            float Jn[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                int xi = __shfl_sync(FULL, xN, i);
                Jn[i] = (i < lane && validN) ? __ldg(T.J + (size_t)xi * T.ldJ + xN) : 0.f;
            }

            unsigned accBits = 0;
            int nf = 0;
            int published = g0;  // iterations [0, published) are visible to the neighbours
            for (int i = 0; i < nValid; ++i) {
                const int xi = __shfl_sync(FULL, x, i);
                const int gi = g0 + i;
                float qn[2] = {0.f, 0.f};
                for (int n = 0; n < nNbr; ++n) {
                    const int Jlim = gi - 1 + (n ? before1 : before0);
                    unsigned long long tStart = 0;
                    int bit = 0;
                    for (;;) {
                        int a = __shfl_sync(FULL, S.applied[n], 0);
                        int head = __shfl_sync(FULL, S.ringHead[n], 0);
                        bool ready = false;
                        if (Jlim < a) {
                            ready = true;
                        } else if (Jlim < head && Jlim - a < kRing) {
                            int jc = -1;
                            for (int j0 = a; j0 <= Jlim; j0 += 32) {
                                int j = j0 + lane;
                                bool hit = j <= Jlim && ring[n * kRing + (j & (kRing - 1))] == xi;
                                unsigned b = __ballot_sync(FULL, hit);
                                if (b) jc = j0 + 31 - __clz(b);
                            }
                            ready = jc < 0;
                        }
                        if (ready) break;
                        if (published < gi) {  // publish everything decided before waiting
                            if (lane == 0) {
                                __stcg(outLog + (size_t)y * nWords + (g0 >> 5), accBits);
                                st_release_gpu(progress + (size_t)y * kProgStride, (unsigned)gi);
                            }
                            published = gi;
                        }
                        if (tStart == 0) tStart = global_ns();
                        if (global_ns() - tStart > kWaitLimitNs) {
                            aborted = true;
                            break;
                        }
                        __nanosleep(64);
                    }
                    if (aborted) break;
                    __threadfence_block();
                    bit = (ghost[n * nWG + (xi >> 5)] >> (xi & 31)) & 1u;
                    qn[n] = bit ? 1.f : -1.f;
                }
                if (aborted) break;
                if (nNbr == 1) qn[1] = qn[0];
                int acc = 0;
                float d = 0.f;
                if (lane == i) {
                    float qyx = qs[x];
                    float dE = sa ? dense_sa_dE(qyx, hx, Fv)
                                  : dense_sqa_dE(qyx, hx, Fv, qn[0], qn[1], sc.twoDivM, sc.coef);
                    acc = metropolis(dE, sc.rate, u);
                    if (acc) {
                        qs[x] = (int8_t)(-qyx);
                        d = -2.f * qyx;
                        flips[nf] = make_int2(x, __float_as_int(d));
                        if (T.trace) {
                            uint32_t bitIdx = (uint32_t)k * (uint32_t)m + (uint32_t)y;
                            atomicOr(&T.trace[(size_t)s * wordsPerStep + (bitIdx >> 5)], 1u << (bitIdx & 31));
                        }
                    }
                }
                acc = __shfl_sync(FULL, acc, i);
                if (acc) {
                    d = __shfl_sync(FULL, d, i);
                    if (lane > i) Fv = __fmaf_rn(d, Jgs[lane * 33 + i], Fv);
                    accBits |= 1u << i;
                    ++nf;
                }
            }
            if (aborted) break;
            accepted += (unsigned long long)nf;
            if (lane == 0) {
                __stcg(outLog + (size_t)y * nWords + (g0 >> 5), accBits);
                st_release_gpu(progress + (size_t)y * kProgStride, (unsigned)(g0 + nValid));
                S.nflip = nf;
            }
            __syncwarp();
            named_bar(1, 32 + kMcUpdaters);  // flips ready
#pragma unroll
            for (int i = 0; i < 32; ++i) Jgs[lane * 33 + i] = Jn[i];
            x = xN;
            u = uN;
            sc = scN;
            s = sN;
            k = kN;
            named_bar(2, 32 + kMcUpdaters);  // fields updated
        }
        if (lane == 0) {
            if (aborted && T.status) atomicExch(T.status, (int)kErrTimeout);
            if (T.accepted) atomicAdd(T.accepted, accepted);
            S.nflip = -1;
            S.done = 1;
        }
        __syncwarp();
        named_bar(1, 32 + kMcUpdaters);
    } else if (warp == 1) {
        // ------------------------------------------------------------- helper
        while (nNbr > 0 && !S.done) {
            for (int n = 0; n < nNbr; ++n) {
                const int nb = n ? nbr1 : nbr0;
                const int a = S.applied[n];
                int head = S.ringHead[n];
                const int lim = min(a + kRing, Itot);
                if (head < lim) {
                    int j = head + lane;
                    if (j < lim) {
                        int sj = j / N, kj = j - sj * N;
                        u32x4 r = draw(T.seed, (uint32_t)kj, (uint32_t)nb, T.step0 + (uint32_t)sj, tag);
                        ring[n * kRing + (j & (kRing - 1))] = draw_index(r.x, N);
                    }
                    __syncwarp();
                    __threadfence_block();
                    head = min(head + 32, lim);
                    if (lane == 0) S.ringHead[n] = head;
                    __syncwarp();
                }
                const unsigned P = ld_acquire_gpu(progress + (size_t)nb * kProgStride);
                const int cnt = min(min((int)P - a, 32), head - a);
                if (cnt > 0) {
                    const int j = a + lane;
                    if (lane < cnt) {
                        uint32_t w = __ldcg(outLog + (size_t)nb * nWords + (j >> 5));
                        if ((w >> (j & 31)) & 1u) {
                            int site = ring[n * kRing + (j & (kRing - 1))];
                            atomicXor(&ghost[n * nWG + (site >> 5)], 1u << (site & 31));
                        }
                    }
                    __syncwarp();
                    __threadfence_block();
                    if (lane == 0) S.applied[n] = a + cnt;
                    __syncwarp();
                }
            }
        }
    } else {
        // ----------------------------------------------------------- updaters
        const int ut = tid - 64;
        const int n4 = N / 4;
        float4 *F4 = reinterpret_cast<float4 *>(Fs);
        for (;;) {
            named_bar(1, 32 + kMcUpdaters);
            const int nf = S.nflip;
            if (nf < 0) break;
            for (int c0 = ut; c0 < n4; c0 += 4 * kMcUpdaters) {
                float4 f[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    int c = c0 + t * kMcUpdaters;
                    if (c < n4) f[t] = F4[c];
                }
                for (int q = 0; q < nf; ++q) {
                    const int2 fl = flips[q];
                    const float d = __int_as_float(fl.y);
                    const float4 *Jr = reinterpret_cast<const float4 *>(T.J + (size_t)fl.x * T.ldJ);
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        int c = c0 + t * kMcUpdaters;
                        if (c < n4) {
                            float4 j = __ldg(Jr + c);
                            f[t].x = __fmaf_rn(d, j.x, f[t].x);
                            f[t].y = __fmaf_rn(d, j.y, f[t].y);
                            f[t].z = __fmaf_rn(d, j.z, f[t].z);
                            f[t].w = __fmaf_rn(d, j.w, f[t].w);
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    int c = c0 + t * kMcUpdaters;
                    if (c < n4) F4[c] = f[t];
                }
            }
            named_bar(2, 32 + kMcUpdaters);
        }
    }
    __syncthreads();
    for (int i = tid; i < N; i += kMcThreads) {
        T.F[(size_t)y * N + i] = Fs[i];
        T.q[(size_t)y * N + i] = qs[i];
    }
}

static size_t multi_smem_bytes(int N) {
    int nWG = (N + 31) / 32;
    return (size_t)N * 4 * 2 + 32 * 33 * 4 + (size_t)2 * nWG * 4 + 2 * kRing * 4 + 32 * 8 + (size_t)N + 16;
}

static int multi_capacity(int N) {
    static int cachedN = -1, cachedCap = 0;
    if (N == cachedN) return cachedCap;
    int dev = 0, sms = 0, perSm = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    size_t smem = multi_smem_bytes(N);
    cudaFuncAttributes fa;
    cudaFuncGetAttributes(&fa, dense_sweep_multi);
    if (smem + fa.sharedSizeBytes > (size_t)optin) return 0;
    if (cudaFuncSetAttribute(dense_sweep_multi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, dense_sweep_multi, kMcThreads, smem);
    cachedN = N;
    cachedCap = perSm * sms;
    return cachedCap;
}

}  // namespace sq103

using namespace sq103;

extern "C" {

SQ103_API unsigned long long sq103_dense_ws_bytes(int N, int m, int nSteps) {
    unsigned long long nWords = ((unsigned long long)nSteps * N + 31) / 32;
    return (unsigned long long)m * kProgStride * 4 + (unsigned long long)m * nWords * 4 + 256;
}

SQ103_API int sq103_dense_multicta_ok(int N, int m, int algo) {
    if (algo != kColoring && algo != kSANaive) return 0;
    if (N < 64 || (N & 3) || m < 2) return 0;
    return m <= multi_capacity(N) ? 1 : 0;
}

// launched from sq103_dense_anneal (dense.cu) when the shape and workspace allow it
int sq103_dense_anneal_multi(const sq103_dense_task *t, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    const int N = t->N, m = t->m;
    if ((long long)t->nSteps * N >= (1ll << 31)) return kErrBadShape;
    if (!t->ws || t->wsBytes < sq103_dense_ws_bytes(N, m, t->nSteps)) return kErrCapacity;
    unsigned *progress = reinterpret_cast<unsigned *>(t->ws);
    uint32_t *outLog = reinterpret_cast<uint32_t *>(progress + (size_t)m * kProgStride);
    int nWords = (int)(((long long)t->nSteps * N + 31) / 32);
    cudaError_t e = cudaMemsetAsync(progress, 0, (size_t)m * kProgStride * 4, st);
    if (e != cudaSuccess) return (int)e;
    if (multi_capacity(N) < m) return kErrCapacity;
    sq103_dense_task task = *t;
    void *args[] = {&task, &outLog, &progress, &nWords};
    e = cudaLaunchCooperativeKernel((const void *)dense_sweep_multi, dim3(m), dim3(kMcThreads), args,
                                    multi_smem_bytes(N), st);
    return (int)e;
}

}  // extern "C"
