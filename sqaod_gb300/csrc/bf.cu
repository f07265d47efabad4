// bf.cu -- brute-force QUBO search (dense and bipartite graphs).
//
// Dense: E(x) = x^T W x over packed states x (variable i at bit N-1-i,
// sqaodc/common/Common.cpp:79-93).  A state splits into hi = x >> L (the
// first N-L variables) and lo = x & (2^L - 1) (the last L variables,
// L = min(N, 14)):
//   E = E_hh(hi) + E_ll(lo) + sum_{b in lo} x_b C_hi[b],   C_hi[b] = 2 sum_{i in hi} W_{i,b}
// One CTA per hi value; E_ll is a 2^L table shared by all CTAs and the cross
// term is two table lookups over the halves of lo.  The search runs in three
// passes: fp32 minimum, collection of every x with E32 <= Emin32 + slack, and
// an FP64 re-evaluation of the candidates (tie-break) done by the caller
// through sq103_dense_bf_refine.  For integer-valued W every fp32 value is
// exact, so Emin and the argmin set equal the reference CPU searcher's
// (sqaodc/cpu/CPUDenseGraphBatchSearch.cpp:26-50).
//
// Bipartite: E(x0, x1) = b0.x0 + b1.x1 + x1^T W x0 (sqaodc/cpu/SharedFormulas.cpp:123-144).
// One CTA per x1 value; D[j] = b0[j] + sum_{i in x1} W[i][j]; E is the sum of
// 7-bit-group lookups over x0 plus b1.x1.
#include <cstdint>
#include <cstring>

#include "sq_common.cuh"
#include "sq_kernels.h"

namespace sq103 {

constexpr int kLoBits = 14;
constexpr int kBfThreads = 256;

struct BfWorkspace {
    float ell[1 << kLoBits];
    unsigned int minEnc;
    int count;
    int pad[62];
};

__device__ __forceinline__ unsigned int enc_float(float f) {
    unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float dec_float(unsigned int e) {
    unsigned int u = (e & 0x80000000u) ? (e & 0x7fffffffu) : ~e;
    return __uint_as_float(u);
}

__global__ void bf_init_ws(BfWorkspace *ws) {
    ws->minEnc = 0xffffffffu;
    ws->count = 0;
}

// E_ll table: lo bit b <-> variable N-1-b
__global__ void bf_lo_table(const float *W, int N, int L, BfWorkspace *ws) {
    int lo = blockIdx.x * blockDim.x + threadIdx.x;
    if (lo >= (1 << L)) return;
    double e = 0.;
    for (int a = 0; a < L; ++a) {
        if (!((lo >> a) & 1)) continue;
        int va = N - 1 - a;
        for (int b = 0; b < L; ++b)
            if ((lo >> b) & 1) e += (double)W[(size_t)va * N + (N - 1 - b)];
    }
    ws->ell[lo] = (float)e;
}

// per-CTA set-up for the K consecutive hi values hi0 .. hi0 + K - 1 that are <= he:
// each hi value's set-up (C_hi, E_hh) runs in its own group of kBfThreads / K
// threads, all at once: base = E_hh(hi), C_hi, and the cross-term half tables
template <int K>
__device__ void bf_block_setup_k(const float *W, int N, int L, uint64_t hi0, uint64_t he, float *base,
                                 float (*tabHi)[128], float (*tabLo)[128], float (*C)[kLoBits], int Lh, int Ll) {
    static_assert(kBfThreads / K >= 64 && kBfThreads % K == 0, "a group needs two warps");
    constexpr int kGroup = kBfThreads / K;
    const int H = N - L;
    const int tid = threadIdx.x, g = tid / kGroup, t = tid % kGroup;
    const uint64_t hi = hi0 + g;
    if (hi <= he) {
        if (t < L) {
            double s = 0.;
            for (int c = 0; c < H; ++c)
                if ((hi >> c) & 1ull) s += (double)W[(size_t)(H - 1 - c) * N + (N - 1 - t)];
            C[g][t] = (float)(2. * s);
        }
        if (t >= 32 && t < 64) {
            double e = 0.;
            for (int c = t - 32; c < H; c += 32) {
                if (!((hi >> c) & 1ull)) continue;
                const float *row = W + (size_t)(H - 1 - c) * N;
                for (int d = 0; d < H; ++d)
                    if ((hi >> d) & 1ull) e += (double)row[H - 1 - d];
            }
            for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
            if (t == 32) base[g] = (float)e;
        }
    }
    __syncthreads();
    for (int idx = tid; idx < (K << Lh); idx += blockDim.x) {
        const int k = idx >> Lh, u = idx & ((1 << Lh) - 1);
        float s = 0.f;
        for (int b = 0; b < Lh; ++b)
            if ((u >> b) & 1) s += C[k][Ll + b];
        tabHi[k][u] = s;
    }
    for (int idx = tid; idx < (K << Ll); idx += blockDim.x) {
        const int k = idx >> Ll, u = idx & ((1 << Ll) - 1);
        float s = 0.f;
        for (int b = 0; b < Ll; ++b)
            if ((u >> b) & 1) s += C[k][b];
        tabLo[k][u] = s;
    }
    __syncthreads();
}

// PASS 0: minimum; PASS 1: collect x with E <= thr.  A CTA takes kBfHiPerRound hi
// values per round of set-up.
constexpr int kBfHiPerRound = 4;
template <int PASS>
__global__ void __launch_bounds__(kBfThreads) bf_dense_pass(const float *W, int N, int L, uint64_t xb, uint64_t xe,
                                                            float slack, BfWorkspace *ws, uint64_t *cand, int cap) {
    constexpr int K = kBfHiPerRound;
    __shared__ float tabHi[K][128], tabLo[K][128], C[K][kLoBits];
    __shared__ float base[K];
    __shared__ unsigned int blockMin;
    const int Lh = L / 2, Ll = L - Lh;
    const uint64_t hb = xb >> L, he = (xe - 1) >> L;
    float thr = 0.f;
    if (PASS == 1) thr = dec_float(ws->minEnc) + slack;
    const uint32_t mask = (1u << Ll) - 1u;
    for (uint64_t hi0 = hb + (uint64_t)blockIdx.x * K; hi0 <= he; hi0 += (uint64_t)gridDim.x * K) {
        bf_block_setup_k<K>(W, N, L, hi0, he, base, tabHi, tabLo, C, Lh, Ll);
        if (PASS == 0 && threadIdx.x == 0) blockMin = 0xffffffffu;
        __syncthreads();
        float lmin = __int_as_float(0x7f800000);
        for (int k = 0; k < K && hi0 + k <= he; ++k) {
            const float bk = base[k];
            const float *tH = tabHi[k], *tL = tabLo[k];
            const uint64_t x0 = (hi0 + k) << L;
            const uint32_t loB = (uint32_t)(xb > x0 ? xb - x0 : 0);
            const uint32_t loE = (uint32_t)min((uint64_t)1 << L, xe - x0);
            auto visit = [&](uint32_t lo, float e) {
                if (PASS == 0) {
                    lmin = fminf(lmin, e);
                } else if (e <= thr) {
                    int slot = atomicAdd(&ws->count, 1);
                    if (slot < cap) cand[slot] = x0 | lo;
                }
            };
            // four consecutive states per thread: one 16-byte load of the E_ll table and one
            // tabHi lookup for the four; a thread's tabLo entries stay the same across its
            // iterations (the stride 4 * blockDim.x is a multiple of 2^Ll), so they are
            // kept in registers.  Every energy is summed in the same order as one at a time.
            const uint32_t vb = (loB + 3u) & ~3u, ve = loE & ~3u;
            const uint32_t step4 = 4u * blockDim.x;
            if (vb < ve && (step4 & mask) == 0 && !(reinterpret_cast<uintptr_t>(ws->ell) & 15)) {
                for (uint32_t lo = loB + threadIdx.x; lo < vb; lo += blockDim.x)
                    visit(lo, (bk + ws->ell[lo]) + (tH[lo >> Ll] + tL[lo & mask]));
                for (uint32_t lo = ve + threadIdx.x; lo < loE; lo += blockDim.x)
                    visit(lo, (bk + ws->ell[lo]) + (tH[lo >> Ll] + tL[lo & mask]));
                const uint32_t first = vb + 4u * threadIdx.x;
                const float t0 = tL[first & mask], t1 = tL[(first + 1u) & mask];
                const float t2 = tL[(first + 2u) & mask], t3 = tL[(first + 3u) & mask];
                uint32_t lo = first;
                for (; lo + step4 < ve; lo += 2u * step4) {
                    const float4 l = *reinterpret_cast<const float4 *>(&ws->ell[lo]);
                    const float4 q = *reinterpret_cast<const float4 *>(&ws->ell[lo + step4]);
                    const float th = tH[lo >> Ll], tq = tH[(lo + step4) >> Ll];
                    visit(lo, (bk + l.x) + (th + t0));
                    visit(lo + 1u, (bk + l.y) + (th + t1));
                    visit(lo + 2u, (bk + l.z) + (th + t2));
                    visit(lo + 3u, (bk + l.w) + (th + t3));
                    visit(lo + step4, (bk + q.x) + (tq + t0));
                    visit(lo + step4 + 1u, (bk + q.y) + (tq + t1));
                    visit(lo + step4 + 2u, (bk + q.z) + (tq + t2));
                    visit(lo + step4 + 3u, (bk + q.w) + (tq + t3));
                }
                for (; lo < ve; lo += step4) {
                    const float4 l = *reinterpret_cast<const float4 *>(&ws->ell[lo]);
                    const float th = tH[lo >> Ll];  // the four share lo >> Ll (2^Ll is a multiple of 4)
                    visit(lo, (bk + l.x) + (th + t0));
                    visit(lo + 1u, (bk + l.y) + (th + t1));
                    visit(lo + 2u, (bk + l.z) + (th + t2));
                    visit(lo + 3u, (bk + l.w) + (th + t3));
                }
            } else {
                for (uint32_t lo = loB + threadIdx.x; lo < loE; lo += blockDim.x)
                    visit(lo, (bk + ws->ell[lo]) + (tH[lo >> Ll] + tL[lo & mask]));
            }
        }
        if (PASS == 0) {
            for (int o = 16; o > 0; o >>= 1) lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
            if ((threadIdx.x & 31) == 0) atomicMin(&blockMin, enc_float(lmin));
            __syncthreads();
            if (threadIdx.x == 0) atomicMin(&ws->minEnc, blockMin);
        }
        __syncthreads();
    }
}

// bipartite: x1 per CTA; x0 through 7-bit-group tables
template <int PASS>
__global__ void __launch_bounds__(kBfThreads) bf_bip_pass(const float *b0, const float *b1, const float *W, int N0,
                                                          int N1, uint64_t x0b, uint64_t x0e, uint64_t x1b,
                                                          uint64_t x1e, float slack, BfWorkspace *ws,
                                                          uint64_t *cand, int cap) {
    __shared__ float tab[9][128];
    __shared__ float D[64];
    __shared__ float base;
    __shared__ unsigned int blockMin;
    const int nG = (N0 + 6) / 7;
    float thr = 0.f;
    if (PASS == 1) thr = dec_float(ws->minEnc) + slack;
    for (uint64_t x1 = x1b + blockIdx.x; x1 < x1e; x1 += gridDim.x) {
        int tid = threadIdx.x;
        // x0 bit c <-> variable N0-1-c ; x1 bit c <-> variable N1-1-c
        if (tid < N0) {
            int j = N0 - 1 - tid;  // D indexed by x0 bit position
            double s = (double)b0[j];
            for (int c = 0; c < N1; ++c)
                if ((x1 >> c) & 1ull) s += (double)W[(size_t)(N1 - 1 - c) * N0 + j];
            D[tid] = (float)s;
        }
        if (tid == 64) {
            double s = 0.;
            for (int c = 0; c < N1; ++c)
                if ((x1 >> c) & 1ull) s += (double)b1[N1 - 1 - c];
            base = (float)s;
        }
        if (PASS == 0 && tid == 0) blockMin = 0xffffffffu;
        __syncthreads();
        for (int t = tid; t < nG * 128; t += blockDim.x) {
            int g = t >> 7, v = t & 127;
            float s = 0.f;
            for (int k = 0; k < 7; ++k) {
                int bit = g * 7 + k;
                if (bit < N0 && ((v >> k) & 1)) s += D[bit];
            }
            tab[g][v] = s;
        }
        __syncthreads();
        float lmin = __int_as_float(0x7f800000);
        auto visit = [&](uint64_t x0, float e) {
            if (PASS == 0) {
                lmin = fminf(lmin, e);
            } else if (e <= thr) {
                int slot = atomicAdd(&ws->count, 1);
                if (slot < cap) {
                    cand[2 * slot] = x0;
                    cand[2 * slot + 1] = x1;
                }
            }
        };
        auto energy = [&](uint64_t x0) {
            float e = base;
            for (int g = 0; g < nG; ++g) e += tab[g][(x0 >> (7 * g)) & 127];
            return e;
        };
        // four consecutive x0 per thread: their first-group entries stay the same across
        // the thread's iterations (the stride 4 * blockDim.x is a multiple of 128), so
        // they are kept in registers, and the four share every higher group's lookup.
        // Each energy adds its groups in the same order as one at a time.
        const uint64_t vb = (x0b + 3) & ~3ull, ve = x0e & ~3ull;
        const uint32_t step4 = 4u * blockDim.x;
        if (nG >= 2 && vb < ve && (step4 & 127u) == 0) {
            for (uint64_t x0 = x0b + tid; x0 < vb && x0 < x0e; x0 += blockDim.x) visit(x0, energy(x0));
            for (uint64_t x0 = ve + tid; x0 < x0e; x0 += blockDim.x) visit(x0, energy(x0));
            const uint64_t first = vb + 4u * tid;
            const float t0 = base + tab[0][first & 127], t1 = base + tab[0][(first + 1) & 127];
            const float t2 = base + tab[0][(first + 2) & 127], t3 = base + tab[0][(first + 3) & 127];
            for (uint64_t x0 = first; x0 < ve; x0 += step4) {
                float e0 = t0, e1 = t1, e2 = t2, e3 = t3;
                for (int g = 1; g < nG; ++g) {
                    const float tg = tab[g][(x0 >> (7 * g)) & 127];  // the same for x0 .. x0 + 3
                    e0 += tg;
                    e1 += tg;
                    e2 += tg;
                    e3 += tg;
                }
                visit(x0, e0);
                visit(x0 + 1, e1);
                visit(x0 + 2, e2);
                visit(x0 + 3, e3);
            }
        } else {
            for (uint64_t x0 = x0b + tid; x0 < x0e; x0 += blockDim.x) visit(x0, energy(x0));
        }
        if (PASS == 0) {
            for (int o = 16; o > 0; o >>= 1) lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
            if ((tid & 31) == 0) atomicMin(&blockMin, enc_float(lmin));
            __syncthreads();
            if (tid == 0) atomicMin(&ws->minEnc, blockMin);
        }
        __syncthreads();
    }
}

// FP64 energies of packed dense states, one warp per state (W float, or double
// for the double-precision searchers)
template <class T>
__global__ void bf_dense_refine(const T *W, int N, const uint64_t *xs, int n, double *E) {
    int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= n) return;
    uint64_t x = xs[w];
    double s = 0.;
    for (int i = lane; i < N; i += 32) {
        if (!((x >> (N - 1 - i)) & 1ull)) continue;
        for (int j = 0; j < N; ++j)
            if ((x >> (N - 1 - j)) & 1ull) s += (double)W[(size_t)i * N + j];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) E[w] = s;
}

template <class T>
__global__ void bf_bip_refine(const T *b0, const T *b1, const T *W, int N0, int N1, const uint64_t *pairs, int n,
                              double *E) {
    int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= n) return;
    uint64_t x0 = pairs[2 * w], x1 = pairs[2 * w + 1];
    double s = 0.;
    for (int j = lane; j < N0; j += 32)
        if ((x0 >> (N0 - 1 - j)) & 1ull) s += (double)b0[j];
    for (int i = lane; i < N1; i += 32) {
        if (!((x1 >> (N1 - 1 - i)) & 1ull)) continue;
        s += (double)b1[i];
        for (int j = 0; j < N0; ++j)
            if ((x0 >> (N0 - 1 - j)) & 1ull) s += (double)W[(size_t)i * N0 + j];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) E[w] = s;
}

static int bf_grid(uint64_t units) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t g = (uint64_t)sms * 8;
    return (int)(units < g ? units : g);
}

}  // namespace sq103

using namespace sq103;

extern "C" {

SQ103_API size_t sq103_bf_workspace_bytes(int N) {
    (void)N;
    return sizeof(BfWorkspace);
}

SQ103_API int sq103_dense_bf_range(const float *W, int N, uint64_t xBegin, uint64_t xEnd, float slack, void *ws,
                                   uint64_t *cand, int cap, int *count, float *Emin32, void *stream) {
    if (N <= 0 || N > 63 || xEnd <= xBegin || xEnd > (1ull << N)) return kErrBadShape;
    cudaStream_t s = (cudaStream_t)stream;
    BfWorkspace *w = (BfWorkspace *)ws;
    int L = N < kLoBits ? N : kLoBits;
    bf_init_ws<<<1, 1, 0, s>>>(w);
    bf_lo_table<<<((1 << L) + 255) / 256, 256, 0, s>>>(W, N, L, w);
    uint64_t nHi = ((xEnd - 1) >> L) - (xBegin >> L) + 1;
    int grid = bf_grid((nHi + kBfHiPerRound - 1) / kBfHiPerRound);
    bf_dense_pass<0><<<grid, kBfThreads, 0, s>>>(W, N, L, xBegin, xEnd, slack, w, cand, cap);
    bf_dense_pass<1><<<grid, kBfThreads, 0, s>>>(W, N, L, xBegin, xEnd, slack, w, cand, cap);
    unsigned int enc = 0;
    cudaMemcpyAsync(count, &w->count, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&enc, &w->minEnc, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return (int)e;
    unsigned int u = (enc & 0x80000000u) ? (enc & 0x7fffffffu) : ~enc;
    memcpy(Emin32, &u, sizeof(float));
    return (int)cudaGetLastError();
}

SQ103_API int sq103_dense_bf_refine(const float *W, int N, const uint64_t *x, int n, double *E, void *stream) {
    if (n <= 0) return 0;
    bf_dense_refine<float><<<(n * 32 + 255) / 256, 256, 0, (cudaStream_t)stream>>>(W, N, x, n, E);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_dense_bf_refine64(const double *W, int N, const uint64_t *x, int n, double *E, void *stream) {
    if (n <= 0) return 0;
    bf_dense_refine<double><<<(n * 32 + 255) / 256, 256, 0, (cudaStream_t)stream>>>(W, N, x, n, E);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_bipartite_bf_range(const float *b0, const float *b1, const float *W, int N0, int N1,
                                       uint64_t x0b, uint64_t x0e, uint64_t x1b, uint64_t x1e, float slack,
                                       void *ws, uint64_t *cand, int cap, int *count, float *Emin32,
                                       void *stream) {
    if (N0 <= 0 || N1 <= 0 || N0 > 63 || N1 > 63 || x0e <= x0b || x1e <= x1b) return kErrBadShape;
    cudaStream_t s = (cudaStream_t)stream;
    BfWorkspace *w = (BfWorkspace *)ws;
    bf_init_ws<<<1, 1, 0, s>>>(w);
    int grid = bf_grid(x1e - x1b);
    bf_bip_pass<0><<<grid, kBfThreads, 0, s>>>(b0, b1, W, N0, N1, x0b, x0e, x1b, x1e, slack, w, cand, cap);
    bf_bip_pass<1><<<grid, kBfThreads, 0, s>>>(b0, b1, W, N0, N1, x0b, x0e, x1b, x1e, slack, w, cand, cap);
    unsigned int enc = 0;
    cudaMemcpyAsync(count, &w->count, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&enc, &w->minEnc, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return (int)e;
    unsigned int u = (enc & 0x80000000u) ? (enc & 0x7fffffffu) : ~enc;
    memcpy(Emin32, &u, sizeof(float));
    return (int)cudaGetLastError();
}

SQ103_API int sq103_bipartite_bf_refine(const float *b0, const float *b1, const float *W, int N0, int N1,
                                        const uint64_t *pairs, int n, double *E, void *stream) {
    if (n <= 0) return 0;
    bf_bip_refine<float><<<(n * 32 + 255) / 256, 256, 0, (cudaStream_t)stream>>>(b0, b1, W, N0, N1, pairs, n, E);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_bipartite_bf_refine64(const double *b0, const double *b1, const double *W, int N0, int N1,
                                          const uint64_t *pairs, int n, double *E, void *stream) {
    if (n <= 0) return 0;
    bf_bip_refine<double><<<(n * 32 + 255) / 256, 256, 0, (cudaStream_t)stream>>>(b0, b1, W, N0, N1, pairs, n, E);
    return (int)cudaGetLastError();
}

}  // extern "C"
