// bip_field.cuh -- bipartite local fields and energy row sums,
// C[y][n] = sum_k A[y][k] B(k, n), A in {-1, +1} (int8 spins, M x K), B fp32.
//
// The half-step GEMMs of the bipartite sweep are small (m = 64, N0 = N1 = 1024
// is 67 M multiply-adds): 64 x 64 output tiles give 16 CTAs, a tenth of the
// GPU.  Here a CTA owns a 16 x 32 output tile and splits K over its 8 warps:
//   - k runs in 32-wide chunks; the nChunks = ceil(K / 32) chunks are dealt
//     to 8 groups in contiguous, balanced runs (group g gets q or q + 1 chunks,
//     q = nChunks / 8, the first nChunks % 8 groups one more);
//   - fields (fp32): a chunk's partial is the sequential fp32 FMA sum over its
//     32 k (ascending, +0 start); a group adds its chunk partials in order with
//     TwoSum into (s_g, c_g);
//   - energies (FP64 out): a group adds every product with TwoSum into
//     (s_g, c_g) (a double-float accumulator);
//   - the 8 groups are folded in order: (S, C) = (0, 0); for g = 0..7:
//     TwoSum-add s_g into (S, C), then C += c_g; the result is S + C.
// Every addition is in a fixed order that depends only on K, so a tile gives
// the same bits whichever kernel runs it: the stand-alone launch (one tile per
// CTA) and the persistent bipartite batch kernel (one CTA looping over the
// tiles of its instance) produce bit-identical fields.
//
// TRANS_B = false: B(k, n) = Bm[k * ldb + n];  true: B(k, n) = Bm[n * ldb + k].
// Shared memory: kBipFieldSmem bytes (dynamic), 256 threads.
#pragma once

#include <cstdint>

#include "field_gemm.cuh"

namespace sq103 {

constexpr int kBipTileM = 16, kBipTileN = 32, kBipGroups = 8;
constexpr int kBipWarpFloats = 32 * 16 + 32 * 32;                     // A chunk + B chunk per warp
constexpr int kBipFieldSmem = kBipGroups * kBipWarpFloats * 4;       // 49152 bytes
static_assert(kBipGroups * 2 * kBipTileM * kBipTileN <= kBipGroups * kBipWarpFloats, "fold buffer fits");

// Shared-memory swizzles (float4 reads; the permutations inside a float4 depend
// only on k mod 8, so they are compile-time constants in the 8-way unrolled loop):
//   A chunk [32 k][16 rows]: row r of k lives at r ^ ((k >> 1) & 15) (conflict-free stores)
//   B chunk [32 k][32 cols]: col n of k lives at n ^ ((k & 7) << 2) (conflict-free stores
//     for B(k, n) = Bm[k * ldb + n], 4-way for the transposed layout)
__device__ __forceinline__ int bip_swz_b(int k) { return (k & 7) << 2; }

template <bool TRANS_B, bool EXACT, typename OutT>
__device__ __forceinline__ void bip_field_tile(const int8_t *A, int lda, const float *Bm, int ldb, OutT *C, int ldc,
                                               int M, int Nn, int K, int y0, int n0, float *smem) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *As = smem + warp * kBipWarpFloats;
    float *Bs = As + 32 * 16;
    const int nChunks = (K + 31) >> 5;
    const int q = nChunks / kBipGroups, r = nChunks % kBipGroups;
    const int cb = warp * q + min(warp, r), ce = cb + q + (warp < r ? 1 : 0);
    const int lr = lane >> 3, lc = lane & 7;  // this lane's outputs: rows lr*4.., cols lc*4..

    float s[4][4], c[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) s[a][b] = c[a][b] = 0.f;

    float ra[16], rb[32];
    const bool rowsIn = y0 + 16 <= M && n0 + 32 <= Nn;
    auto load = [&](int ch) {
        const int k0 = ch << 5, k = k0 + lane;
        if (rowsIn && k0 + 32 <= K) {  // the whole chunk is inside: no bounds checks
            const int8_t *Ap = A + (size_t)y0 * lda + k;
#pragma unroll
            for (int i = 0; i < 16; ++i) ra[i] = (float)Ap[(size_t)i * lda];
            const float *Bp = TRANS_B ? Bm + (size_t)n0 * ldb + k : Bm + (size_t)k0 * ldb + n0 + lane;
#pragma unroll
            for (int j = 0; j < 32; ++j) rb[j] = Bp[(size_t)j * ldb];
            return;
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int y = y0 + i;
            ra[i] = (y < M && k < K) ? (float)A[(size_t)y * lda + k] : 0.f;
        }
        if (!TRANS_B) {  // lane = column
            const int n = n0 + lane;
#pragma unroll
            for (int kk = 0; kk < 32; ++kk) {
                const int kq = k0 + kk;
                rb[kk] = (n < Nn && kq < K) ? Bm[(size_t)kq * ldb + n] : 0.f;
            }
        } else {  // lane = k
#pragma unroll
            for (int nn = 0; nn < 32; ++nn) {
                const int n = n0 + nn;
                rb[nn] = (n < Nn && k < K) ? Bm[(size_t)n * ldb + k] : 0.f;
            }
        }
    };
    auto store = [&]() {
        const int sa = (lane >> 1) & 15;
#pragma unroll
        for (int i = 0; i < 16; ++i) As[lane * 16 + (i ^ sa)] = ra[i];
        if (!TRANS_B) {
#pragma unroll
            for (int kk = 0; kk < 32; ++kk) Bs[kk * 32 + (lane ^ bip_swz_b(kk))] = rb[kk];
        } else {
            const int f = bip_swz_b(lane);
#pragma unroll
            for (int nn = 0; nn < 32; ++nn) Bs[lane * 32 + (nn ^ f)] = rb[nn];
        }
    };

    if (cb < ce) load(cb);
    for (int ch = cb; ch < ce; ++ch) {
        __syncwarp();  // the previous chunk's reads are done
        store();
        __syncwarp();
        if (ch + 1 < ce) load(ch + 1);  // in flight during this chunk
        float part[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) part[a][b] = 0.f;
        for (int k8 = 0; k8 < 32; k8 += 8) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int kk = k8 + j, pA = (j >> 1) & 3;  // ((kk >> 1) & 15) & 3, k8 a multiple of 8
                const float4 av = *reinterpret_cast<const float4 *>(&As[kk * 16 + ((lr ^ ((kk >> 3) & 3)) << 2)]);
                const float4 bv = *reinterpret_cast<const float4 *>(&Bs[kk * 32 + ((lc ^ j) << 2)]);
                const float ar4[4] = {av.x, av.y, av.z, av.w}, br4[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        const float av1 = ar4[a ^ pA], bv1 = br4[b];
                        if (EXACT)
                            two_sum_acc(s[a][b], c[a][b], __fmul_rn(av1, bv1));
                        else
                            part[a][b] = __fmaf_rn(av1, bv1, part[a][b]);
                    }
            }
        }
        if (!EXACT) {
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) two_sum_acc(s[a][b], c[a][b], part[a][b]);
        }
    }

    // fold the 8 groups in order
    __syncthreads();  // every warp is done with its staging area
    float *red = smem;  // [group][s|c][16 rows][32 cols]
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int o = (lr * 4 + a) * kBipTileN + lc * 4 + b;
            red[(warp * 2) * (kBipTileM * kBipTileN) + o] = s[a][b];
            red[(warp * 2 + 1) * (kBipTileM * kBipTileN) + o] = c[a][b];
        }
    __syncthreads();
    for (int o = threadIdx.x; o < kBipTileM * kBipTileN; o += blockDim.x) {
        float S = 0.f, Cc = 0.f;
#pragma unroll
        for (int g = 0; g < kBipGroups; ++g) {
            two_sum_acc(S, Cc, red[(g * 2) * (kBipTileM * kBipTileN) + o]);
            Cc = __fadd_rn(Cc, red[(g * 2 + 1) * (kBipTileM * kBipTileN) + o]);
        }
        const int y = y0 + o / kBipTileN, n = n0 + o % kBipTileN;
        if (y < M && n < Nn) {
            if (EXACT)
                C[(size_t)y * ldc + n] = (OutT)((double)S + (double)Cc);
            else
                C[(size_t)y * ldc + n] = (OutT)__fadd_rn(S, Cc);
        }
    }
    __syncthreads();  // the staging area is reused by the next tile
}

template <bool TRANS_B, bool EXACT, typename OutT>
__global__ void __launch_bounds__(256) bip_field_kernel(const int8_t *A, int lda, const float *Bm, int ldb, OutT *C,
                                                        int ldc, int M, int Nn, int K) {
    extern __shared__ __align__(16) float bip_smem[];
    bip_field_tile<TRANS_B, EXACT, OutT>(A, lda, Bm, ldb, C, ldc, M, Nn, K, blockIdx.y * kBipTileM,
                                         blockIdx.x * kBipTileN, bip_smem);
}

}  // namespace sq103
