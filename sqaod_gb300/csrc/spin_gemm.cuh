// spin_gemm.cuh -- the spin x coupling GEMM C[y][n] = sum_k A[y][k] B(k, n), A in {-1, +1}.
//
// One 64 x 64 output tile per call of spin_gemm_tile (256 threads, 4 x 4
// outputs each, k in 32-wide chunks).  fp32 outputs are the FP64 sum, in k
// order, of fp32 partial sums over each chunk (sequential FMAs); FP64 outputs
// accumulate every product in FP64.  The products are exact, so the result is
// deterministic and does not depend on which kernel runs the tile: the
// stand-alone GEMM (one tile per CTA) and the batched bipartite sweep (one CTA
// looping over the tiles of its instance) give bit-identical fields.
//
// A int8 spins (M x K, row stride lda);
// TRANS_B = false: B(k, n) = Bm[k * ldb + n];  true: B(k, n) = Bm[n * ldb + k].
#pragma once

#include <cstdint>
#include <type_traits>

namespace sq103 {

template <bool TRANS_B, typename OutT>
__device__ __forceinline__ void spin_gemm_tile(const int8_t *A, int lda, const float *Bm, int ldb, OutT *C, int ldc,
                                               int M, int Nn, int K, int y0, int n0) {
    constexpr bool EXACT = std::is_same<OutT, double>::value;
    __shared__ float As[32][64 + 4];
    __shared__ float Bs[32][64 + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
    float part[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.;
    for (int k0 = 0; k0 < K; k0 += 32) {
        for (int idx = threadIdx.x; idx < 64 * 32; idx += 256) {
            int r = idx >> 5, kk = idx & 31;
            int y = y0 + r, k = k0 + kk;
            As[kk][r] = (y < M && k < K) ? (float)A[(size_t)y * lda + k] : 0.f;
        }
        if (!TRANS_B) {
            for (int idx = threadIdx.x; idx < 32 * 64; idx += 256) {
                int kk = idx >> 6, c = idx & 63;
                int k = k0 + kk, n = n0 + c;
                Bs[kk][c] = (k < K && n < Nn) ? Bm[(size_t)k * ldb + n] : 0.f;
            }
        } else {
            for (int idx = threadIdx.x; idx < 32 * 64; idx += 256) {
                int c = idx >> 5, kk = idx & 31;
                int k = k0 + kk, n = n0 + c;
                Bs[kk][c] = (k < K && n < Nn) ? Bm[(size_t)n * ldb + k] : 0.f;
            }
        }
        __syncthreads();
        if (EXACT) {
#pragma unroll 4
            for (int kk = 0; kk < 32; ++kk) {
                double av[4], bv[4];
#pragma unroll
                for (int a = 0; a < 4; ++a) av[a] = As[kk][ty * 4 + a];
#pragma unroll
                for (int b = 0; b < 4; ++b) bv[b] = Bs[kk][tx * 4 + b];
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
            }
        } else {
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) part[a][b] = 0.f;
#pragma unroll 8
            for (int kk = 0; kk < 32; ++kk) {
                float av[4], bv[4];
#pragma unroll
                for (int a = 0; a < 4; ++a) av[a] = As[kk][ty * 4 + a];
#pragma unroll
                for (int b = 0; b < 4; ++b) bv[b] = Bs[kk][tx * 4 + b];
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) part[a][b] = __fmaf_rn(av[a], bv[b], part[a][b]);
            }
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] += (double)part[a][b];
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        int y = y0 + ty * 4 + a;
        if (y >= M) continue;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            int n = n0 + tx * 4 + b;
            if (n < Nn) C[(size_t)y * ldc + n] = (OutT)acc[a][b];
        }
    }
}

template <bool TRANS_B, typename OutT>
__global__ void __launch_bounds__(256) spin_gemm_kernel(const int8_t *A, int lda, const float *Bm, int ldb,
                                                        OutT *C, int ldc, int M, int Nn, int K) {
    spin_gemm_tile<TRANS_B, OutT>(A, lda, Bm, ldb, C, ldc, M, Nn, K, blockIdx.y * 64, blockIdx.x * 64);
}

}  // namespace sq103
