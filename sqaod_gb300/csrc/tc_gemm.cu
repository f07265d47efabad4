// tc_gemm.cu -- local-field refresh on the 5th-generation tensor cores
// (tcgen05), operands staged by TMA, accumulators in TMEM.
//
//   F[y][r] = sum_k q[y][k] B[r][k]      (dense: B = J, symmetric, so F = q J;
//                                          bipartite: B = J or J^T)
//
// The refresh replaces the reference's J.q contractions
// (DeviceDotJqVec4, sqaodc/cuda/DeviceBatchedDot.cuh:247-262, and the cuBLAS
// SGEMMs of CUDABipartiteGraphAnnealer.cu:393-401).
//
// Exactness.  The couplings are held as 31-bit fixed point, B ~ 2^-S * (D0 +
// 2^8 D1 + 2^16 D2 + 2^24 D3), with S chosen from the matrix's largest
// magnitude and every digit D_t a signed integer of magnitude <= 128, exact in
// bf16.  The spins are +-1, so each digit's contraction P_t = q . D_t is a sum
// of integers of magnitude <= 128, and every partial sum is an integer below
// 2^24 for K < 2^17: the fp32 accumulation in TMEM is exact whatever the
// tensor core's adder order, alignment or truncation.  The epilogue combines
// sum_t 2^(8t) P_t in 64-bit integers and rounds once to fp32.  The only error
// left is the quantisation of B (below 2^-29 of the largest |B| per element),
// far below the fp32 rounding of the result.
//
// Kernel (one CTA per 128 x 64 output tile, 128 threads):
//   thread 0    TMA producer: per 64-wide K block, the spin tile (128 x 64 bf16)
//               and the four digit tiles (64 x 64 bf16 each) into a 4-stage
//               shared-memory ring (128B swizzle), mbarrier-tracked;
//   thread 32   MMA issuer: per K block 4 x 4 tcgen05.mma kind::f16
//               (M = 128, N = 64, K = 16), one TMEM accumulator per digit;
//               tcgen05.commit frees each stage;
//   all 4 warps epilogue: tcgen05.ld of the four accumulators (a trotter row
//               per thread), integer combination, fp32 store.
// Every mbarrier wait is bounded by the global timer; on timeout the CTA
// records status 1, lets the copies it issued land (bounded), frees TMEM and
// returns.  Two test flags make a wait run out on purpose: the producer skips
// the first K block's copies, and waits give up after 1 ms.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "sq_common.cuh"
#include "sq_kernels.h"

namespace sq103 {

constexpr int kTcBM = 128, kTcBN = 64, kTcBK = 64, kTcStages = 4, kTcThreads = 128, kTcDigits = 4;
constexpr int kTcATile = kTcBM * kTcBK * 2;  // 16 KB
constexpr int kTcBTile = kTcBN * kTcBK * 2;  // 8 KB
constexpr int kTcStageBytes = kTcATile + kTcDigits * kTcBTile;
constexpr int kTcSmemBytes = kTcStages * kTcStageBytes + 1024 + 256;
constexpr int kTcTmemCols = 256;  // 4 accumulators of 64 fp32 columns
constexpr unsigned long long kTcWaitNs = 2000000000ull, kTcShortWaitNs = 1000000ull;
constexpr int kTcHeader = 256;  // digit buffer: exponent word, int shift S, then the four planes

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long tc_now() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait for the phase with the given parity; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, unsigned long long limitNs) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = tc_now();
    while (!mbar_try_wait(bar, parity))
        if (tc_now() - t0 > limitNs) return false;
    return true;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_addr(dst)),
        "l"((uint64_t)map), "r"(smem_addr(bar)), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::
            "r"(smem_addr(dst)),
        "l"((uint64_t)map), "r"(smem_addr(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}

// shared-memory matrix descriptor: K-major, 128B swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused with swizzle)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;             // descriptor version
    d |= (uint64_t)2 << 61;             // 128B swizzle
    return d;
}

// instruction descriptor, kind::f16: bf16 x bf16 -> f32, A and B K-major, M x N
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// 16 consecutive fp32 columns of the warp's 32 TMEM lanes (one lane per thread)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// F tile (128 trotters x 64 outputs) = sum_t 2^(8t - S) (q . D_t)
__global__ void __launch_bounds__(kTcThreads) tc_digit_gemm(const __grid_constant__ CUtensorMap tmA,
                                                            const __grid_constant__ CUtensorMap tmB,
                                                            const int *shiftPtr, float *F, int ldF, int M, int R,
                                                            int Kp, int flags, int *status) {
    extern __shared__ __align__(16) unsigned char tc_smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)tc_smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kTcStages * kTcStageBytes);
    uint64_t *empty = full + kTcStages;
    uint64_t *done = empty + kTcStages;
    uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(done + 1);
    __shared__ int abortFlag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kTcBM, n0 = blockIdx.x * kTcBN;
    const int nK = Kp / kTcBK;
    const unsigned long long waitNs = (flags & 2) ? kTcShortWaitNs : kTcWaitNs;

    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmemSlot)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmemSlot;

    if (tid == 0) {
        // ---------------------------------------------------------- producer
        // issued[s]: the parity of the latest copy issued into stage s, -1 if none is outstanding
        int issued[kTcStages];
        for (int s = 0; s < kTcStages; ++s) issued[s] = -1;
        for (int kb = 0; kb < nK; ++kb) {
            const int s = kb % kTcStages;
            if (kb >= kTcStages && !mbar_wait(&empty[s], ((kb / kTcStages) - 1) & 1, waitNs)) {
                abortFlag = 1;
                break;
            }
            if ((flags & 1) && kb == 0) continue;  // test hook: stage 0's first copies never come
            unsigned char *a = smem + s * kTcStageBytes;
            mbar_expect_tx(&full[s], kTcStageBytes);
            tma_load_2d(a, &tmA, &full[s], kb * kTcBK, m0);
#pragma unroll
            for (int t = 0; t < kTcDigits; ++t) tma_load_3d(a + kTcATile + t * kTcBTile, &tmB, &full[s], kb * kTcBK, n0, t);
            issued[s] = (kb / kTcStages) & 1;
        }
        // let every copy still in flight land before the CTA can leave
        for (int s = 0; s < kTcStages; ++s)
            if (issued[s] >= 0) mbar_wait(&full[s], (uint32_t)issued[s], waitNs);
    } else if (tid == 32) {
        // ---------------------------------------------------------- MMA issuer
        constexpr uint32_t idesc = umma_idesc_bf16(kTcBM, kTcBN);
        bool ok = true;
        for (int kb = 0; kb < nK; ++kb) {
            const int s = kb % kTcStages;
            if (!mbar_wait(&full[s], (kb / kTcStages) & 1, waitNs) || abortFlag) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = smem_addr(smem + s * kTcStageBytes);
            const uint64_t adesc = sw128_desc(a);
#pragma unroll
            for (int kk = 0; kk < kTcBK / 16; ++kk)  // K = 16 per MMA: +32 B in the swizzled row
#pragma unroll
                for (int t = 0; t < kTcDigits; ++t)
                    umma_bf16(tmem + (uint32_t)(t * kTcBN), adesc + 2 * kk,
                              sw128_desc(a + kTcATile + t * kTcBTile) + 2 * kk, idesc, (kb | kk) ? 1u : 0u);
            umma_commit(&empty[s]);
        }
        if (!ok) abortFlag = 1;
        umma_commit(done);
    }
    __syncwarp();
    // ---------------------------------------------------------------- epilogue
    const bool got = mbar_wait(done, 0, waitNs);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (!got || abortFlag) {
        if (tid == 0 && status) atomicExch(status, (int)kErrTimeout);
    } else {
        const int S = *shiftPtr;
        const float scale = __int_as_float((127 - S) << 23);  // 2^-S, S in [-126, 126]
        const int row = m0 + warp * 32 + lane;
        const uint32_t lanes = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
        for (int c0 = 0; c0 < kTcBN; c0 += 16) {
            uint32_t p[kTcDigits][16];
#pragma unroll
            for (int t = 0; t < kTcDigits; ++t) tmem_ld16(tmem + lanes + (uint32_t)(t * kTcBN + c0), p[t]);
            tmem_wait_ld();
            if (row < M) {
                float *dst = F + (size_t)row * ldF + n0 + c0;
                const int nv = min(16, R - (n0 + c0));
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    long long v = 0;
#pragma unroll
                    for (int t = kTcDigits - 1; t >= 0; --t)
                        v = (v << 8) + (long long)__float2int_rn(__uint_as_float(p[t][j]));
                    if (j < nv) dst[j] = __fmul_rn(__ll2float_rn(v), scale);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols)
                     : "memory");
}

// largest biased exponent of the matrix (atomicMax over the float bit patterns)
__global__ void tc_max_exponent(const float *B, int ld, int rows, int cols, unsigned *out) {
    unsigned e = 0;
    const size_t n = (size_t)rows * cols;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / cols, c = i - r * cols;
        e = max(e, __float_as_uint(B[r * ld + c]) & 0x7f800000u);
    }
    e = __reduce_max_sync(0xffffffffu, e);
    if ((threadIdx.x & 31) == 0) atomicMax(out, e);
}

// shift S: |B| < 2^(E - 126) for the largest biased exponent E, so |B 2^S| < 2^30 with S = 156 - E
__device__ __forceinline__ int tc_shift(unsigned maxExpBits) {
    return min(max(156 - (int)(maxExpBits >> 23), -126), 126);
}

// digit planes D_t[r][k] (r < R rows of output, k < K, row stride ldD, zero padded to ldD):
// B[r][k] = J[r][k] (transpose = 0) or J[k][r] (transpose = 1), J with row stride ldJ
__global__ void tc_make_digits(const float *J, int ldJ, int R, int K, int ldD, int transpose, const unsigned *maxExp,
                               int *shiftOut, __nv_bfloat16 *D) {
    const int S = tc_shift(*maxExp);
    if (blockIdx.x == 0 && threadIdx.x == 0) *shiftOut = S;
    const float scale = __int_as_float((S + 127) << 23);
    const size_t n = (size_t)R * ldD, plane = n;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / ldD), k = (int)(i - (size_t)r * ldD);
        int v = 0;
        if (k < K) v = __float2int_rn(__fmul_rn(transpose ? J[(size_t)k * ldJ + r] : J[(size_t)r * ldJ + k], scale));
        // balanced base-256 digits: v = d0 + 2^8 d1 + 2^16 d2 + 2^24 d3, d0..d2 in [-128, 127],
        // |d3| <= 64 since |v| < 2^30
#pragma unroll
        for (int t = 0; t < kTcDigits; ++t) {
            const int d = t == kTcDigits - 1 ? v : (int)(int8_t)(v & 0xff);
            D[t * plane + i] = __int2bfloat16_rn(d);
            v = (v - d) >> 8;
        }
    }
}

// spins (m x K int8, row stride ldq) -> bf16 (m x ldA), zero beyond K
__global__ void tc_spins_bf16(const int8_t *q, int ldq, int m, int K, int ldA, __nv_bfloat16 *A) {
    const size_t n = (size_t)m * ldA;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int y = (int)(i / ldA), k = (int)(i - (size_t)y * ldA);
        A[i] = __int2bfloat16_rn(k < K ? (int)q[(size_t)y * ldq + k] : 0);
    }
}

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

static int ld_pad(int K) { return (K + kTcBK - 1) / kTcBK * kTcBK; }

static int grid_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, (size_t)152 * 16); }

}  // namespace sq103

using namespace sq103;

extern "C" {

SQ103_API unsigned long long sq103_tc_digits_bytes(int R, int K) {
    return (unsigned long long)kTcHeader + (unsigned long long)kTcDigits * R * (unsigned long long)ld_pad(K) * 2ull;
}

SQ103_API unsigned long long sq103_tc_spins_bytes(int m, int K) {
    return (unsigned long long)m * (unsigned long long)ld_pad(K) * 2ull;
}

SQ103_API int sq103_tc_make_digits(const float *J, int ldJ, int R, int K, int transpose, void *digits, void *stream) {
    if (R <= 0 || K <= 0 || K >= (1 << 17) || !J || !digits || (reinterpret_cast<uintptr_t>(digits) & 255))
        return kErrBadShape;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *base = static_cast<unsigned char *>(digits);
    unsigned *maxExp = reinterpret_cast<unsigned *>(base);
    int *shift = reinterpret_cast<int *>(base + 16);
    cudaError_t e = cudaMemsetAsync(maxExp, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return (int)e;
    const int rowsJ = transpose ? K : R, colsJ = transpose ? R : K;
    tc_max_exponent<<<grid_for((size_t)rowsJ * colsJ), 256, 0, st>>>(J, ldJ, rowsJ, colsJ, maxExp);
    const int ldD = ld_pad(K);
    tc_make_digits<<<grid_for((size_t)R * ldD), 256, 0, st>>>(J, ldJ, R, K, ldD, transpose, maxExp, shift,
                                                              reinterpret_cast<__nv_bfloat16 *>(base + kTcHeader));
    return (int)cudaGetLastError();
}

SQ103_API int sq103_tc_refresh(const void *digits, int R, int K, const int8_t *q, int ldq, int m, void *spinsBf16,
                               float *F, int ldF, int flags, int *status, void *stream) {
    if (R <= 0 || K <= 0 || m <= 0 || K >= (1 << 17) || !digits || !q || !spinsBf16 || !F ||
        (reinterpret_cast<uintptr_t>(digits) & 255) || (reinterpret_cast<uintptr_t>(spinsBf16) & 15) ||
        (flags & ~3))
        return kErrBadShape;
    auto enc = tensor_map_encoder();
    if (!enc) return kErrBadShape;
    cudaStream_t st = (cudaStream_t)stream;
    const int ldD = ld_pad(K);
    tc_spins_bf16<<<grid_for((size_t)m * ldD), 256, 0, st>>>(q, ldq, m, K, ldD,
                                                            reinterpret_cast<__nv_bfloat16 *>(spinsBf16));
    const unsigned char *base = static_cast<const unsigned char *>(digits);
    CUtensorMap tmA, tmB;
    {
        cuuint64_t dims[2] = {(cuuint64_t)ldD, (cuuint64_t)m};
        cuuint64_t strides[1] = {(cuuint64_t)ldD * 2};
        cuuint32_t box[2] = {(cuuint32_t)kTcBK, (cuuint32_t)kTcBM};
        cuuint32_t estr[2] = {1, 1};
        if (enc(&tmA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, spinsBf16, dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return kErrBadShape;
    }
    {
        cuuint64_t dims[3] = {(cuuint64_t)ldD, (cuuint64_t)R, (cuuint64_t)kTcDigits};
        cuuint64_t strides[2] = {(cuuint64_t)ldD * 2, (cuuint64_t)R * ldD * 2};
        cuuint32_t box[3] = {(cuuint32_t)kTcBK, (cuuint32_t)kTcBN, 1};
        cuuint32_t estr[3] = {1, 1, 1};
        if (enc(&tmB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<unsigned char *>(base + kTcHeader), dims,
                strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return kErrBadShape;
    }
    // the shared-memory limit is a per-device kernel attribute: set once per device, under a lock
    {
        static std::mutex mu;
        static bool attrSet[256] = {};
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return (int)e;
        std::lock_guard<std::mutex> lock(mu);
        if (dev < 0 || dev >= 256 || !attrSet[dev]) {
            e = cudaFuncSetAttribute(tc_digit_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes);
            if (e != cudaSuccess) return (int)e;
            if (dev >= 0 && dev < 256) attrSet[dev] = true;
        }
    }
    dim3 grid((R + kTcBN - 1) / kTcBN, (m + kTcBM - 1) / kTcBM);
    tc_digit_gemm<<<grid, kTcThreads, kTcSmemBytes, st>>>(tmA, tmB, reinterpret_cast<const int *>(base + 16), F, ldF,
                                                          m, R, ldD, flags, status);
    return (int)cudaGetLastError();
}

// The dense refresh every path runs (single annealer, batch, server, bench): the
// tensor-core digit contraction when a digit buffer is given, else the SIMT spin
// GEMM.  Which one a path uses is decided by sq103_dense_refresh_uses_tc(N) alone,
// so every path that anneals the same instance holds the same fields.
SQ103_API int sq103_dense_refresh_uses_tc(int N) { return N >= 1024 ? 1 : 0; }

// Bipartite half-step fields on the tensor cores for problems of at least 2^20
// couplings whose output tiles (128 trotters x 64 spins) give each half step a
// grid of at least 64 CTAs; smaller grids leave most SMs idle, and the SIMT
// field kernel is faster there (N0 = N1 = 1024, m = 64: 16 CTAs).
SQ103_API int sq103_bipartite_refresh_uses_tc(int N0, int N1, int m) {
    if ((long long)N0 * (long long)N1 < (1ll << 20) || m < 1) return 0;
    const long long tiles = (long long)((m + 127) / 128) * ((std::min(N0, N1) + 63) / 64);
    return tiles >= 64 ? 1 : 0;
}

SQ103_API int sq103_dense_refresh(const float *J, int ldJ, const void *digits, void *spinsBf16, const int8_t *q,
                                  float *F, int N, int m, int *status, void *stream) {
    if (digits) return sq103_tc_refresh(digits, N, N, q, N, m, spinsBf16, F, N, 0, status, stream);
    return sq103_dense_field_refresh(J, ldJ, q, F, N, m, stream);
}

}  // extern "C"
