// field_gemm.cuh -- dense local fields and energy row sums without FP64 arithmetic.
//
// Both compute C[y][n] = sum_k A[y][k] B[k][n] with A in {-1, +1} (int8 spins,
// M x K) and B fp32 (K x N, row stride ldb): every product is an exact fp32
// value (+-B or 0 past the edge), so only the summation rounds.  GB300 runs
// FP64 at 1/64 of the fp32 rate, so both kernels sum in fp32 with error-free
// transformations instead:
//   fields (fp32 out): fp32 partial sums over 32-wide k chunks (sequential,
//     k ascending), the chunk sums added with TwoSum into a (sum, compensation)
//     pair; the result is sum + compensation.  About 1e-7 of the row scale.
//   energies (FP64 out): every product added with TwoSum into a (sum,
//     compensation) pair -- a double-float accumulator, about 2^-44 relative --
//     returned as sum + compensation in FP64.
// Tiles of 64 x 64 outputs per CTA of 256 threads (4 x 4 per thread), k in
// chunks of 32 staged in shared memory with the next chunk's loads in flight.
// The order of every addition is fixed, so results do not depend on the launch.
#pragma once

#include <cstdint>

namespace sq103 {

__device__ __forceinline__ void two_sum_acc(float &s, float &c, float x) {
    const float t = __fadd_rn(s, x);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp));
    s = t;
    c = __fadd_rn(c, err);
}

// The 64 x 64 output tile at rows y0.., columns n0.. of C = A B, by a CTA of 256
// threads.  EXACT = false: fp32 fields; true: double-float energy row sums (OutT
// double).
template <bool EXACT, typename OutT>
__device__ __forceinline__ void field_gemm_tile(const int8_t *A, int lda, const float *B, int ldb, OutT *C, int ldc,
                                                int M, int Nn, int K, int y0, int n0) {
    __shared__ __align__(16) float As[2][32][68];  // rows padded against store conflicts
    __shared__ __align__(16) float Bs[2][32][68];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    // loader roles: A row ar, k ak..ak+7; B row bk, columns bc..bc+3 and bc+32..bc+35
    const int ar = tid >> 2, ak = (tid & 3) * 8;
    const int bk = tid >> 3, bc = (tid & 7) * 4;
    float la[8], lb[8];
    // chunks inside the matrices take vector loads without bounds checks (same values)
    const bool inside = y0 + 64 <= M && n0 + 64 <= Nn;
    const bool vecA = !(lda & 7) && !(reinterpret_cast<uintptr_t>(A) & 7);
    const bool vecB = !(ldb & 3) && !(reinterpret_cast<uintptr_t>(B) & 15);
    auto load = [&](int k0) {
        const int y = y0 + ar;
        if (inside && k0 + 32 <= K) {
            if (vecA) {
                const int2 v = *reinterpret_cast<const int2 *>(A + (size_t)y * lda + k0 + ak);
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    la[i] = (float)(int8_t)(((i < 4 ? v.x : v.y) >> (8 * (i & 3))) & 0xff);
            } else {
#pragma unroll
                for (int i = 0; i < 8; ++i) la[i] = (float)A[(size_t)y * lda + k0 + ak + i];
            }
            const float *Bk = B + (size_t)(k0 + bk) * ldb + n0 + bc;
            if (vecB) {
                const float4 b0 = *reinterpret_cast<const float4 *>(Bk);
                const float4 b1 = *reinterpret_cast<const float4 *>(Bk + 32);
                lb[0] = b0.x, lb[1] = b0.y, lb[2] = b0.z, lb[3] = b0.w;
                lb[4] = b1.x, lb[5] = b1.y, lb[6] = b1.z, lb[7] = b1.w;
            } else {
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int i = 0; i < 4; ++i) lb[4 * h + i] = Bk[32 * h + i];
            }
            return;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int k = k0 + ak + i;
            la[i] = (y < M && k < K) ? (float)A[(size_t)y * lda + k] : 0.f;
        }
        const int k = k0 + bk;
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int n = n0 + bc + 32 * h + i;
                lb[4 * h + i] = (k < K && n < Nn) ? B[(size_t)k * ldb + n] : 0.f;
            }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int i = 0; i < 8; ++i) As[buf][ak + i][ar] = la[i];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int i = 0; i < 4; ++i) Bs[buf][bk][bc + 32 * h + i] = lb[4 * h + i];
    };

    float s[4][4], c[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) s[a][b] = c[a][b] = 0.f;

    const int nChunks = (K + 31) / 32;
    load(0);
    store(0);
    __syncthreads();
    for (int ch = 0; ch < nChunks; ++ch) {
        const int buf = ch & 1;
        if (ch + 1 < nChunks) load((ch + 1) * 32);  // in flight during this chunk
        float part[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) part[a][b] = 0.f;
#pragma unroll 8
        for (int kk = 0; kk < 32; ++kk) {
            const float4 av = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 4]);
            const float4 bv = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 4]);
            const float a4[4] = {av.x, av.y, av.z, av.w}, b4[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    if (EXACT)
                        two_sum_acc(s[a][b], c[a][b], __fmul_rn(a4[a], b4[b]));
                    else
                        part[a][b] = __fmaf_rn(a4[a], b4[b], part[a][b]);
                }
        }
        if (!EXACT) {
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) two_sum_acc(s[a][b], c[a][b], part[a][b]);
        }
        if (ch + 1 < nChunks) store(buf ^ 1);
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int y = y0 + ty * 4 + a;
        if (y >= M) continue;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int n = n0 + tx * 4 + b;
            if (n >= Nn) continue;
            if (EXACT)
                C[(size_t)y * ldc + n] = (OutT)((double)s[a][b] + (double)c[a][b]);
            else
                C[(size_t)y * ldc + n] = (OutT)__fadd_rn(s[a][b], c[a][b]);
        }
    }
}

template <bool EXACT, typename OutT>
__global__ void __launch_bounds__(256) field_gemm_kernel(const int8_t *A, int lda, const float *B, int ldb, OutT *C,
                                                         int ldc, int M, int Nn, int K) {
    field_gemm_tile<EXACT, OutT>(A, lda, B, ldb, C, ldc, M, Nn, K, blockIdx.y * 64, blockIdx.x * 64);
}

}  // namespace sq103
