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

// sq103_dense_task.flags: bits 0-1 choose the kernel (0 auto, 1 one CTA per
// instance, 2 one CTA per trotter); the other bits are test hooks of the
// one-CTA-per-trotter sweep that make its bounded waits give up
enum TaskFlags : int {
    kFlagKernelMask = 3,
    kFlagShortWaits = 16,        // every wait gives up after 1 ms instead of 4 s
    kFlagWithholdTrotter0 = 32,  // trotter 0 never publishes its accept words
};

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

// ------------------------------------------------------------ exact decisions
// The resident fp32 fields drift from the exact local fields by the rounding
// of their rank-1 updates (about 15 ulps after a few thousand updates).  Every
// kernel takes its fp32 decision in the log form of the Metropolis test,
//   accept iff dE < 0 or x = rate dE < L = -ln u,
// and flags the trial when |x - L| lies within a bound on the fp32 error of x;
// a flagged trial is decided again from its exact field, with the FP64
// arithmetic of the host replay (exact_accept).  The sweeps thus take the FP64
// decision on every trial whose FP64 acceptance margin is above about 1e-12,
// and every kernel that runs the same trial takes the same decision.

// -ln u of a uniform draw (+inf for u = 0: every finite x accepts, as exp(-x) > 0)
__device__ __forceinline__ float neg_log_unit(float u) { return u > 0.f ? -logf(u) : __int_as_float(0x7f800000); }

// The error bound of x = rate dE for a trial with field F: the field error is
// taken as 2^-16 (|h| + |F| + 1) (dense fields enter dE as 2F, bipartite as F),
// about 25 times the largest drift seen over the 8 steps between field
// refreshes (6e-6 at |F| ~ 10, a random walk of rank-1 update roundings); the
// rest covers the rounding of the ring term, of x and of -ln u.
struct DecisionTol {
    float kF, kC;  // x tolerance = kF (|h| + |F'| + 1) + kC + 2.4e-7 L, F' = 2F (dense) or F
};
__device__ __forceinline__ DecisionTol decision_tol(bool sa, bool dense, float twoDivM, float coef, float rate) {
    DecisionTol t;
    const float dF = sa ? 2.f : twoDivM;  // d(dE) / d(h + F')
    t.kF = __fmul_rn(__fmul_rn(rate, dF), 1.52587890625e-5f);
    t.kC = __fadd_rn(__fmul_rn(__fmul_rn(rate, 1e-6f), fabsf(coef)), 2e-6f);
    (void)dense;
    return t;
}

// accept iff dE < 0 or rate dE < L; nearFlag set when |rate dE - L| <= xtol
__device__ __forceinline__ int metropolis_log(float dE, float rate, float L, float xtol, int &nearFlag) {
    const float x = __fmul_rn(dE, rate);
    if (fabsf(__fsub_rn(x, L)) <= xtol) nearFlag = 1;
    return (dE < 0.f || x < L) ? 1 : 0;
}

// x tolerance of a trial: kF (|h| + |Fp| + 1) + kC + 2.4e-7 L (Fp = 2F dense, F bipartite)
__device__ __forceinline__ float trial_xtol(const DecisionTol &t, float h, float Fp, float L) {
    const float base = __fadd_rn(t.kC, __fmul_rn(2.4e-7f, fminf(L, 1e30f)));
    return __fmaf_rn(t.kF, __fadd_rn(__fadd_rn(fabsf(h), fabsf(Fp)), 1.f), base);
}

// The exact local field sum_j J[j] q[j] (q = +-1) as an integer sum: every J[j]
// is scaled by 2^S and rounded to an int64, S chosen from the row's largest
// exponent and N so that no partial sum reaches 2^62.  Integer addition does not
// depend on order, so a thread summing the row alone and a warp summing it in
// 32 strands get the same value.  For fp32 couplings it is within N 2^-(S+1)
// of the exact sum (4.5e-13 for |J| < 0.5 and N = 4096); the FP64 couplings of
// the <double> annealers take the same scheme with the double exponent.
template <class R>
struct ExactFx;
template <>
struct ExactFx<float> {
    static __device__ __forceinline__ unsigned expo(float v) { return (__float_as_uint(v) >> 23) & 0xffu; }
    // |J| < 2^(E - 126) for biased exponent E
    static __device__ __forceinline__ int shift(unsigned E, int lg) { return min(max(188 - lg - (int)E, -126), 127); }
    static __device__ __forceinline__ long long term(float J, int S) {
        return __float2ll_rn(__fmul_rn(J, __int_as_float((S + 127) << 23)));
    }
};
template <>
struct ExactFx<double> {
    static __device__ __forceinline__ unsigned expo(double v) {
        return (unsigned)((__double_as_longlong(v) >> 52) & 0x7ff);
    }
    // |J| < 2^(E - 1022) for biased exponent E
    static __device__ __forceinline__ int shift(unsigned E, int lg) { return min(max(1084 - lg - (int)E, -1000), 1000); }
    static __device__ __forceinline__ long long term(double J, int S) {
        return __double2ll_rn(__dmul_rn(J, __longlong_as_double((long long)(1023 + S) << 52)));
    }
};
__device__ __forceinline__ int log2_ceil(int N) { return N > 1 ? 32 - __clz(N - 1) : 0; }
__device__ __forceinline__ double exact_value(long long s, int S) {
    return __dmul_rn(__ll2double_rn(s), __longlong_as_double((long long)(1023 - S) << 52));
}

// The exact-decision helpers are kept out of line by default (they are rare,
// and inlined copies grow every kernel's hot code); a file may define
// SQ103_EXACT_ATTR as __forceinline__ before including this header when that
// measures faster (the one-CTA-per-trotter sweep, which calls them from a warp
// of their own).
#ifndef SQ103_EXACT_ATTR
#define SQ103_EXACT_ATTR __noinline__
#endif

// one thread; the couplings are Jx[j * stride] (a row of J, or a column with stride = ld)
template <class R>
static __device__ SQ103_EXACT_ATTR double exact_field_thread(const R *Jx, size_t stride, const int8_t *q, int N) {
    unsigned e = 0;
    for (int j = 0; j < N; ++j) e = max(e, ExactFx<R>::expo(Jx[j * stride]));
    const int S = ExactFx<R>::shift(e, log2_ceil(N));
    long long s = 0;
    for (int j = 0; j < N; ++j) {
        const long long v = ExactFx<R>::term(Jx[j * stride], S);
        s += q[j] > 0 ? v : -v;
    }
    return exact_value(s, S);
}

// warp-wide: every lane of the (converged) warp calls it and gets the sum
template <class R>
static __device__ SQ103_EXACT_ATTR double exact_field_warp(const R *Jx, const int8_t *q, int N) {
    const int lane = threadIdx.x & 31;
    unsigned e = 0;
    for (int j = lane; j < N; j += 32) e = max(e, ExactFx<R>::expo(Jx[j]));
    e = __reduce_max_sync(0xffffffffu, e);
    const int S = ExactFx<R>::shift(e, log2_ceil(N));
    long long s = 0;
    for (int j = lane; j < N; j += 32) {
        const long long v = ExactFx<R>::term(Jx[j], S);
        s += q[j] > 0 ? v : -v;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return exact_value(s, S);
}

// fp32 rows on a 16-byte boundary are read as float4 with eight loads in flight
// per lane (the row of N = 4096 in four rounds); the second pass finds the row
// in L1.  The same integer sum as the generic form.
template <>
__device__ SQ103_EXACT_ATTR double exact_field_warp<float>(const float *Jx, const int8_t *q, int N) {
    typedef ExactFx<float> X;
    const int lane = threadIdx.x & 31;
    const bool vec = (reinterpret_cast<uintptr_t>(Jx) & 15) == 0 && (reinterpret_cast<uintptr_t>(q) & 3) == 0;
    const int n4 = vec ? N / 4 : 0;
    const float4 *J4 = reinterpret_cast<const float4 *>(Jx);
    const char4 *q4 = reinterpret_cast<const char4 *>(q);
    unsigned e = 0;
#pragma unroll 8
    for (int c = lane; c < n4; c += 32) {
        const float4 v = __ldg(J4 + c);
        e = max(e, max(max(X::expo(v.x), X::expo(v.y)), max(X::expo(v.z), X::expo(v.w))));
    }
    for (int j = 4 * n4 + lane; j < N; j += 32) e = max(e, X::expo(__ldg(Jx + j)));
    e = __reduce_max_sync(0xffffffffu, e);
    const int S = X::shift(e, log2_ceil(N));
    long long s = 0;
#pragma unroll 8
    for (int c = lane; c < n4; c += 32) {
        const float4 v = __ldg(J4 + c);
        const char4 qq = q4[c];
        const long long a = X::term(v.x, S), b = X::term(v.y, S), cc = X::term(v.z, S), d = X::term(v.w, S);
        s += (qq.x > 0 ? a : -a) + (qq.y > 0 ? b : -b) + (qq.z > 0 ? cc : -cc) + (qq.w > 0 ? d : -d);
    }
    for (int j = 4 * n4 + lane; j < N; j += 32) {
        const long long v = X::term(__ldg(Jx + j), S);
        s += q[j] > 0 ? v : -v;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return exact_value(s, S);
}

// The FP64 ring coefficient log(tanh(G beta / m)) / beta of a step (SQA only)
__device__ __forceinline__ double exact_ring_coef(float G, float beta, int m) {
    const double Gd = G, bd = beta;
    return log(tanh(__dmul_rn(Gd, bd) / (double)m)) / bd;
}

// exact_accept with the step's ring coefficient already evaluated (exact_ring_coef;
// ignored for SA) and the neighbours' spin sum qL + qR given as `sum`
__device__ __forceinline__ int exact_accept_coef(bool sa, bool twoF, float q, double h, double F, int sum, int m,
                                                 float G, float beta, double coef, float u) {
    const double qd = q, Gd = G, bd = beta;
    const double t = __dadd_rn(h, twoF ? __dmul_rn(2.0, F) : F);
    double dE, rate;
    if (sa) {
        dE = __dmul_rn(__dmul_rn(2.0, qd), t);
        rate = 1.0 / Gd;
    } else {
        const double a = __dmul_rn(__dmul_rn(2.0 / (double)m, qd), t);
        const double b = __dmul_rn(__dmul_rn(qd, (double)sum), coef);
        dE = __dsub_rn(a, b);
        rate = bd;
    }
    if (dE < 0.0) return 1;
    return exp(__dmul_rn(-dE, rate)) > (double)u ? 1 : 0;
}

// FP64 decision of a dense trial from its exact field F, in the host replay's
// order of operations: SQA dE = (2/m) q (h + 2F) - q (qL + qR) coef with
// coef = log(tanh(G beta / m)) / beta, rate beta; SA dE = 2 q (h + 2F), rate 1/G;
// accept iff dE < 0 or exp(-dE rate) > u.  For bipartite trials (dE with h + F)
// pass twoF = false.
static __device__ SQ103_EXACT_ATTR int exact_accept(bool sa, bool twoF, float q, double h, double F, float qL, float qR,
                                                int m, float G, float beta, float u) {
    const double coef = sa ? 0.0 : exact_ring_coef(G, beta, m);
    return exact_accept_coef(sa, twoF, q, h, F, (int)qL + (int)qR, m, G, beta, coef, u);
}
#endif

}  // namespace sq103
