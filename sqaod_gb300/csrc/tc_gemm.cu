// tc_gemm.cu -- 5th-generation tensor-core (tcgen05) GEMM for the local-field
// refresh, fed by TMA, accumulating in TMEM.
//
// F[y][n] = sum_k Q[y][k] J[n][k]   (J symmetric, so this is F = q J)
// with J split exactly into three bf16 parts, J = J_hi + J_mid + J_lo
// (8 + 8 + 8 significand bits = fp32's 24), and the spins q in {-1, +1} as
// bf16: every product is exact and the accumulation is fp32 in TMEM.  The
// operands are concatenated along K: A' = [q q q] (m x 3N), B' = [J_hi J_mid
// J_lo] (N x 3N), both K-major bf16 with the row stride padded to 64 elements.
//
// One CTA per 128 x 128 output tile, 128 threads:
//   thread 0        TMA producer: 64-wide K blocks of A' and B' into a
//                   4-stage shared-memory ring (128B swizzle), mbarrier-tracked;
//   thread 32       MMA issuer: tcgen05.mma kind::f16 (M=128, N=128, K=16) x 4
//                   per stage, tcgen05.commit frees the stage;
//   all 4 warps     epilogue: tcgen05.ld 32x32b rows of the TMEM accumulator
//                   and store fp32 to F.
// Every mbarrier wait is bounded by the global timer; on timeout the CTA
// records a status, lets its issued copies land (bounded), frees TMEM and
// returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "sq_common.cuh"
#include "sq_kernels.h"

namespace sq103 {

constexpr int kTcBM = 128, kTcBN = 128, kTcBK = 64, kTcStages = 4, kTcThreads = 128;
constexpr int kTcTileBytes = kTcBM * kTcBK * 2;  // 16 KB (A and B tiles alike)
constexpr int kTcStageBytes = 2 * kTcTileBytes;
constexpr int kTcSmemBytes = kTcStages * kTcStageBytes + 1024 + 256;
constexpr unsigned long long kTcWaitNs = 2000000000ull;

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
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    unsigned long long t0 = tc_now();
    while (!mbar_try_wait(bar, parity))
        if (tc_now() - t0 > kTcWaitNs) return false;
    return true;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_addr(dst)),
        "l"((uint64_t)map), "r"(smem_addr(bar)), "r"(x), "r"(y)
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

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(kTcThreads) tc_field_gemm(const __grid_constant__ CUtensorMap tmA,
                                                            const __grid_constant__ CUtensorMap tmB, float *F,
                                                            int ldF, int M, int Nout, int Kp, int *status) {
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

    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {  // 128 TMEM columns = one 128 x 128 fp32 accumulator
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmemSlot)),
                     "r"(128)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmemSlot;

    if (tid == 0) {
        // ---------------------------------------------------------- producer
        int issued = 0;
        for (int kb = 0; kb < nK; ++kb) {
            const int s = kb % kTcStages;
            if (kb >= kTcStages && !mbar_wait(&empty[s], ((kb / kTcStages) - 1) & 1)) {
                abortFlag = 1;
                break;
            }
            unsigned char *a = smem + s * kTcStageBytes;
            mbar_expect_tx(&full[s], kTcStageBytes);
            tma_load_2d(a, &tmA, &full[s], kb * kTcBK, m0);
            tma_load_2d(a + kTcTileBytes, &tmB, &full[s], kb * kTcBK, n0);
            ++issued;
        }
        // let every issued copy land before the CTA can leave
        for (int kb = (issued > kTcStages ? issued - kTcStages : 0); kb < issued; ++kb)
            mbar_wait(&full[kb % kTcStages], (kb / kTcStages) & 1);
    } else if (tid == 32) {
        // ---------------------------------------------------------- MMA issuer
        constexpr uint32_t idesc = umma_idesc_bf16(kTcBM, kTcBN);
        bool ok = true;
        for (int kb = 0; kb < nK; ++kb) {
            const int s = kb % kTcStages;
            if (!mbar_wait(&full[s], (kb / kTcStages) & 1) || abortFlag) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = smem_addr(smem + s * kTcStageBytes);
            const uint64_t adesc = sw128_desc(a), bdesc = sw128_desc(a + kTcTileBytes);
#pragma unroll
            for (int kk = 0; kk < kTcBK / 16; ++kk)  // K = 16 per MMA: +32 B in the swizzled row
                umma_bf16(tmem, adesc + 2 * kk, bdesc + 2 * kk, idesc, (kb | kk) ? 1u : 0u);
            umma_commit(&empty[s]);
        }
        if (!ok) abortFlag = 1;
        umma_commit(done);
    }
    __syncwarp();
    // ---------------------------------------------------------------- epilogue
    bool got = mbar_wait(done, 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (!got || abortFlag) {
        if (tid == 0 && status) atomicExch(status, (int)kErrTimeout);
    } else {
        const int row = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int c0 = 0; c0 < kTcBN; c0 += 32) {
            uint32_t r[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
            if (row < M) {
                float *dst = F + (size_t)row * ldF + n0 + c0;
                const int nv = min(32, Nout - (n0 + c0));
                if (nv == 32 && (((uintptr_t)dst) & 15) == 0) {
#pragma unroll
                    for (int j = 0; j < 32; j += 4)
                        *reinterpret_cast<float4 *>(dst + j) =
                            make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]), __uint_as_float(r[j + 2]),
                                        __uint_as_float(r[j + 3]));
                } else {
                    for (int j = 0; j < nv; ++j) dst[j] = __uint_as_float(r[j]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128) : "memory");
}

// J (N x N fp32, ld) -> B' = [J_hi | J_mid | J_lo] (N x Kp bf16), exact three-way split
__global__ void split3_kernel(const float *J, int ld, int N, int Kp, __nv_bfloat16 *B) {
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)N * Kp) return;
    int r = (int)(idx / Kp), c = (int)(idx - (size_t)r * Kp);
    float v = 0.f;
    int part = c / N, k = c - part * N;
    if (part < 3) {
        float x = J[(size_t)r * ld + k];
        float hi = __bfloat162float(__float2bfloat16_rn(x));
        float r1 = x - hi;
        float mid = __bfloat162float(__float2bfloat16_rn(r1));
        float r2 = r1 - mid;
        v = part == 0 ? hi : (part == 1 ? mid : r2);
    }
    B[idx] = __float2bfloat16_rn(v);
}

// spins (m x N int8) -> A' = [q | q | q] (m x Kp bf16)
__global__ void spins3_kernel(const int8_t *q, int N, int m, int Kp, __nv_bfloat16 *A) {
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)m * Kp) return;
    int r = (int)(idx / Kp), c = (int)(idx - (size_t)r * Kp);
    int part = c / N, k = c - part * N;
    A[idx] = __float2bfloat16_rn(part < 3 ? (float)q[(size_t)r * N + k] : 0.f);
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

static int make_map(CUtensorMap *map, const void *base, int rows, int Kp) {
    auto enc = tensor_map_encoder();
    if (!enc) return kErrBadShape;
    cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
    cuuint32_t box[2] = {(cuuint32_t)kTcBK, (cuuint32_t)kTcBM};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? 0 : kErrBadShape;
}

}  // namespace sq103

using namespace sq103;

extern "C" {

SQ103_API int sq103_tc_kpad(int N) { return (3 * N + kTcBK - 1) / kTcBK * kTcBK; }

SQ103_API int sq103_tc_split_couplings(const float *J, int ldJ, int N, void *Bsplit, void *stream) {
    if (N <= 0) return kErrBadShape;
    int Kp = sq103_tc_kpad(N);
    size_t n = (size_t)N * Kp;
    split3_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(J, ldJ, N, Kp,
                                                                               (__nv_bfloat16 *)Bsplit);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_tc_field_refresh(const void *Bsplit, const int8_t *q, void *Aspins, float *F, int N, int m,
                                     int *status, void *stream) {
    if (N <= 0 || m <= 0 || (N % 4)) return kErrBadShape;
    cudaStream_t st = (cudaStream_t)stream;
    int Kp = sq103_tc_kpad(N);
    size_t na = (size_t)m * Kp;
    spins3_kernel<<<(unsigned)((na + 255) / 256), 256, 0, st>>>(q, N, m, Kp, (__nv_bfloat16 *)Aspins);
    CUtensorMap tmA, tmB;
    int rc = make_map(&tmA, Aspins, m, Kp);
    if (rc == 0) rc = make_map(&tmB, Bsplit, N, Kp);
    if (rc != 0) return rc;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(tc_field_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes);
        if (e != cudaSuccess) return (int)e;
        attr = true;
    }
    dim3 grid((N + kTcBN - 1) / kTcBN, (m + kTcBM - 1) / kTcBM);
    tc_field_gemm<<<grid, kTcThreads, kTcSmemBytes, st>>>(tmA, tmB, F, N, m, N, Kp, status);
    return (int)cudaGetLastError();
}

}  // extern "C"
