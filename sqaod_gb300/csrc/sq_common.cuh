// sq_common.cuh -- shared device helpers of the GB300 sqaod hot path.
//
// Random numbers: every random draw of the annealers is one Philox4x32-10
// evaluation (Salmon, Moraes, Dror, Shaw, SC'11) at counter
// (c0, c1, step, tag | side << 8) under key (seed_lo, seed_hi).  The tags and
// counter meanings are fixed so that any kernel (single instance, batched,
// served) and the FP64 host replay draw the same numbers for the same trial.
//
// Metropolis arithmetic: the decision helpers use explicitly rounded
// intrinsics (no contraction into FMA), so every kernel that evaluates a
// trial from the same field value takes the same decision.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sq103 {

enum Tag : uint32_t {
    kTagDenseSweep = 0x11,    // dense coloring: c0 = iteration k, c1 = trotter y
    kTagDenseSA = 0x12,       // dense SA: c0 = iteration k, c1 = trotter y
    kTagDenseNaive = 0x13,    // dense naive: c0 = trial t
    kTagRandomize = 0x21,     // randomizeSpin: c0 = 128-spin chunk, c1 = trotter
    kTagBipSweep = 0x31,      // bipartite coloring: c0 = spin, c1 = trotter
    kTagBipSA = 0x32,         // bipartite SA coloring
    kTagBipNaive = 0x33,      // bipartite naive: c0 = trial
    kTagBipSANaive = 0x34,    // bipartite SA naive: c0 = trial, c1 = trotter
};

enum Algo : int { kNaive = 0, kColoring = 1, kSANaive = 2, kSAColoring = 3 };

// device status words (written by kernels, read by the host)
enum Status : int {
    kOk = 0,
    kErrTimeout = 1,      // a bounded wait gave up
    kErrBadShape = 2,
    kErrCapacity = 3,     // an output buffer was too small
};

struct u32x4 {
    uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

// Philox4x32-10
__host__ __device__ __forceinline__ u32x4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                 uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t lo0 = 0xD2511F53u * c0, hi0 = mulhi32(0xD2511F53u, c0);
        uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = mulhi32(0xCD9E8D57u, c2);
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return u32x4{c0, c1, c2, c3};
}

__host__ __device__ __forceinline__ u32x4 draw(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t step,
                                               uint32_t tag) {
    return philox(c0, c1, step, tag, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// index in [0, n)
__host__ __device__ __forceinline__ int draw_index(uint32_t w, int n) { return (int)mulhi32(w, (uint32_t)n); }

// uniform in [0, 1), 24-bit resolution, exact in fp32
__host__ __device__ __forceinline__ float draw_unit(uint32_t w) {
    return (float)(w >> 8) * (1.0f / 16777216.0f);
}

#ifdef __CUDACC__
// dE of a Suzuki-Trotter trial on a dense graph:
//   dE = (2/m) q (h + 2 F) - q (qL + qR) coef
__device__ __forceinline__ float dense_sqa_dE(float q, float h, float F, float qL, float qR,
                                              float twoDivM, float coef) {
    float t = __fadd_rn(h, __fmul_rn(2.f, F));
    float a = __fmul_rn(__fmul_rn(twoDivM, q), t);
    float b = __fmul_rn(__fmul_rn(q, __fadd_rn(qL, qR)), coef);
    return __fsub_rn(a, b);
}

// dE of an SA trial on a dense graph: 2 q (h + 2 F)
__device__ __forceinline__ float dense_sa_dE(float q, float h, float F) {
    return __fmul_rn(__fmul_rn(2.f, q), __fadd_rn(h, __fmul_rn(2.f, F)));
}

// bipartite: (2/m) q (h + F) - q (qL + qR) coef  /  2 q (h + F)
__device__ __forceinline__ float bip_sqa_dE(float q, float h, float F, float qL, float qR,
                                            float twoDivM, float coef) {
    float a = __fmul_rn(__fmul_rn(twoDivM, q), __fadd_rn(h, F));
    float b = __fmul_rn(__fmul_rn(q, __fadd_rn(qL, qR)), coef);
    return __fsub_rn(a, b);
}

__device__ __forceinline__ float bip_sa_dE(float q, float h, float F) {
    return __fmul_rn(__fmul_rn(2.f, q), __fadd_rn(h, F));
}

// accept iff dE < 0 or exp(-dE * rate) > u   (rate = beta for SQA, 1/kT for SA)
__device__ __forceinline__ bool metropolis(float dE, float rate, float u) {
    if (dE < 0.f) return true;
    return expf(__fmul_rn(-dE, rate)) > u;
}

// per-step constants, evaluated on the device by every kernel with the same code
struct StepConst {
    float twoDivM, coef, rate;
};

__device__ __forceinline__ StepConst step_const(int algo, int m, float G, float beta) {
    StepConst s;
    s.twoDivM = __fdiv_rn(2.f, (float)m);
    if (algo == kSANaive || algo == kSAColoring) {
        s.coef = 0.f;
        s.rate = __fdiv_rn(1.f, G);
    } else {
        float arg = __fdiv_rn(__fmul_rn(G, beta), (float)m);
        s.coef = __fdiv_rn(logf(tanhf(arg)), beta);
        s.rate = beta;
    }
    return s;
}
#endif

}  // namespace sq103
