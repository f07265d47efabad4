// formulas.cu -- QUBO -> Ising conversion, local-field refresh and FP64 energies.
//
// Dense QUBO -> Ising (sqaodc/cuda/DeviceFormulas.cpp:24-31 /
// sqaodc/cpu/SharedFormulas.cpp:36-55):
//   h_i = -1/2 sum_j W_ij,  J = -W/4 with zero diagonal,
//   c = sum(-W/4) + sum(diag(-W/4)); maximisation negates W first.
// Bipartite (sqaodc/cpu/SharedFormulas.cpp:148-167):
//   J = -W/4 (N1 x N0), h0 = -1/4 colsum(W) - b0/2, h1 = -1/4 rowsum(W) - b1/2,
//   c = -1/4 sum(W) - 1/2 (sum b0 + sum b1).
// Sums are accumulated in FP64 with fixed reduction trees (deterministic).
//
// Spin x coupling products C[y][n] = sum_k q[y][k] * B(k, n), q in {-1, +1}
// (int8), every product exact:
//   field_gemm (field_gemm.cuh): the dense field refresh F = q J (fp32 partial
//     sums over 32-wide k chunks, compensated fp32 sum of the chunks) and the
//     dense energy row sums (double-float accumulation of every product);
//   bip_field (bip_field.cuh): the bipartite half-step fields and energy row
//     sums, K split over the 8 warps of a CTA, groups folded in a fixed order.
// All are deterministic: the order of every addition is fixed.
#include <cstdio>
#include <mutex>
#include <type_traits>

#include "field_gemm.cuh"
#include "bip_field.cuh"
#include "sq_common.cuh"
#include "sq_kernels.h"

namespace sq103 {

// ------------------------------------------------------------ reductions
template <int BLOCK>
__device__ double block_sum_f64(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double r = 0.;
    if (warp == 0) {
        r = lane < BLOCK / 32 ? red[lane] : 0.;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;  // valid in thread 0
}

// ----------------------------------------------------- dense hamiltonian
// one block per row: h, J row, per-row contribution to c
__global__ void __launch_bounds__(256) dg_hamiltonian_rows(const float *W, int ldW, int N, float sign,
                                                           float *h, float *J, int ldJ, double *rowc) {
    __shared__ double red[8];
    int i = blockIdx.x;
    const float *Wi = W + (size_t)i * ldW;
    float *Ji = J + (size_t)i * ldJ;
    double s = 0.;
    for (int j = threadIdx.x; j < N; j += 256) {
        float w = sign * Wi[j];
        s += (double)w;
        Ji[j] = (j == i) ? 0.f : -0.25f * w;
    }
    double rs = block_sum_f64<256>(s, red);
    if (threadIdx.x == 0) {
        float wii = sign * Wi[i];
        h[i] = (float)(-0.5 * rs);
        rowc[i] = -0.25 * rs + -0.25 * (double)wii;
    }
}

// single block: c = sum(rowc) (+ extra), written as fp32 and FP64
__global__ void __launch_bounds__(256) reduce_constant(const double *parts, int n, double extra, float *c,
                                                       double *c64) {
    __shared__ double red[8];
    double s = 0.;
    for (int i = threadIdx.x; i < n; i += 256) s += parts[i];
    double r = block_sum_f64<256>(s, red);
    if (threadIdx.x == 0) {
        r += extra;
        if (c) *c = (float)r;
        if (c64) *c64 = r;
    }
}

// ------------------------------------------------- bipartite hamiltonian
// one block per row i of W (N1 x N0): J row, h1[i], row part of c
__global__ void __launch_bounds__(256) bg_hamiltonian_rows(const float *W, int N0, int N1, float sign,
                                                           const float *b1, float *h1, float *J,
                                                           double *rowc) {
    __shared__ double red[8];
    int i = blockIdx.x;
    const float *Wi = W + (size_t)i * N0;
    float *Ji = J + (size_t)i * N0;
    double s = 0.;
    for (int j = threadIdx.x; j < N0; j += 256) {
        float w = sign * Wi[j];
        s += (double)w;
        Ji[j] = -0.25f * w;
    }
    double rs = block_sum_f64<256>(s, red);
    if (threadIdx.x == 0) {
        double bi = (double)(sign * b1[i]);
        h1[i] = (float)(-0.25 * rs - 0.5 * bi);
        rowc[i] = -0.25 * rs - 0.5 * bi;
    }
}

// one thread per column j: h0[j], column part of c (b0 only)
__global__ void bg_hamiltonian_cols(const float *W, int N0, int N1, float sign, const float *b0, float *h0,
                                    double *colc) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N0) return;
    double s = 0.;
    for (int i = 0; i < N1; ++i) s += (double)(sign * W[(size_t)i * N0 + j]);
    double bj = (double)(sign * b0[j]);
    h0[j] = (float)(-0.25 * s - 0.5 * bj);
    colc[j] = -0.5 * bj;
}

// ------------------------------------------------------- bipartite GEMM
// (bip_field.cuh)

template <bool TRANS_B, bool EXACT, typename OutT>
static void launch_bip_field(const int8_t *A, int lda, const float *B, int ldb, OutT *C, int ldc, int M, int Nn,
                             int K, cudaStream_t s) {
    dim3 grid((Nn + kBipTileN - 1) / kBipTileN, (M + kBipTileM - 1) / kBipTileM);
    bip_field_kernel<TRANS_B, EXACT, OutT><<<grid, 256, kBipFieldSmem, s>>>(A, lda, B, ldb, C, ldc, M, Nn, K);
}

// ------------------------------------------------------------ energies
// dense: E[y] = -c - sum_i q_yi (h_i + r_yi),  r = q J  (FP64)
__global__ void __launch_bounds__(256) dg_energy_finish(const int8_t *q, int N, const float *h,
                                                        const double *r, const double *c64, double sign,
                                                        double *E64, float *E32) {
    __shared__ double red[8];
    int y = blockIdx.x;
    double s = 0.;
    for (int i = threadIdx.x; i < N; i += 256) {
        double qi = q[(size_t)y * N + i];
        s += qi * ((double)h[i] + r[(size_t)y * N + i]);
    }
    double t = block_sum_f64<256>(s, red);
    if (threadIdx.x == 0) {
        double e = sign * (-*c64 - t);
        if (E64) E64[y] = e;
        if (E32) E32[y] = (float)e;
    }
}

// bipartite: E[y] = -(h0.q0 + h1.q1 + q1.r1) - c, r1 = q0 J^T (FP64)
__global__ void __launch_bounds__(256) bg_energy_finish(const int8_t *q0, const int8_t *q1, int N0, int N1,
                                                        const float *h0, const float *h1, const double *r1,
                                                        const double *c64, double sign, double *E64,
                                                        float *E32) {
    __shared__ double red[8];
    int y = blockIdx.x;
    double s = 0.;
    for (int j = threadIdx.x; j < N0; j += 256) s += (double)q0[(size_t)y * N0 + j] * (double)h0[j];
    for (int i = threadIdx.x; i < N1; i += 256) {
        double qi = q1[(size_t)y * N1 + i];
        s += qi * ((double)h1[i] + r1[(size_t)y * N1 + i]);
    }
    double t = block_sum_f64<256>(s, red);
    if (threadIdx.x == 0) {
        double e = sign * (-t - *c64);
        if (E64) E64[y] = e;
        if (E32) E32[y] = (float)e;
    }
}

// spin-ring sum for getSystemE: sum_y sum_i q_yi q_{(y+1)%m, i}
__global__ void __launch_bounds__(256) ring_dot(const int8_t *q, int N, int m, long long *out) {
    __shared__ double red[8];
    long long s = 0;
    for (size_t idx = (size_t)blockIdx.x * 256 + threadIdx.x; idx < (size_t)m * N;
         idx += (size_t)gridDim.x * 256) {
        size_t y = idx / N, i = idx - y * N;
        size_t y1 = (y + 1) % m;
        s += (int)q[y * N + i] * (int)q[y1 * N + i];
    }
    double t = block_sum_f64<256>((double)s, red);
    if (threadIdx.x == 0) atomicAdd((unsigned long long *)out, (unsigned long long)(long long)t);
}

// One 64 x 64 tile of one job's fields per CTA; the tile arithmetic is the one
// of field_gemm_kernel, so each job's fields equal its own refresh bit for bit.
__global__ void __launch_bounds__(256) field_gemm_batch_kernel(const sq103_field_job *jobs, const int *tileJob) {
    const sq103_field_job jb = jobs[tileJob[blockIdx.x]];
    const int local = (int)blockIdx.x - jb.tile0, tilesN = (jb.N + 63) / 64;
    const int ty = local / tilesN, tx = local - ty * tilesN;
    field_gemm_tile<false, float>(jb.q, jb.N, jb.J, jb.ldJ, jb.F, jb.N, jb.m, jb.N, jb.N, ty * 64, tx * 64);
}

}  // namespace sq103

using namespace sq103;

extern "C" {

SQ103_API int sq103_dense_hamiltonian(const float *W, int ldW, int N, int maximize, float *h, float *J, int ldJ,
                            float *c, double *c64, double *scratch, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (N <= 0) return kErrBadShape;
    float sign = maximize ? -1.f : 1.f;
    dg_hamiltonian_rows<<<N, 256, 0, s>>>(W, ldW, N, sign, h, J, ldJ, scratch);
    reduce_constant<<<1, 256, 0, s>>>(scratch, N, 0., c, c64);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_bipartite_hamiltonian(const float *b0, const float *b1, const float *W, int N0, int N1,
                                int maximize, float *h0, float *h1, float *J, float *c, double *c64,
                                double *scratch, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (N0 <= 0 || N1 <= 0) return kErrBadShape;
    float sign = maximize ? -1.f : 1.f;
    bg_hamiltonian_rows<<<N1, 256, 0, s>>>(W, N0, N1, sign, b1, h1, J, scratch);
    bg_hamiltonian_cols<<<(N0 + 127) / 128, 128, 0, s>>>(W, N0, N1, sign, b0, h0, scratch + N1);
    reduce_constant<<<1, 256, 0, s>>>(scratch, N0 + N1, 0., c, c64);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_dense_field_refresh(const float *J, int ldJ, const int8_t *q, float *F, int N, int m,
                              void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    dim3 grid((N + 63) / 64, (m + 63) / 64);
    field_gemm_kernel<false, float><<<grid, 256, 0, s>>>(q, N, J, ldJ, F, N, m, N, N);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_dense_field_refresh_batch(const sq103_field_job *jobs, const int *tileJob, int nTiles,
                                              void *stream) {
    if (nTiles < 0 || (nTiles > 0 && (!jobs || !tileJob))) return kErrBadShape;
    if (nTiles == 0) return 0;
    field_gemm_batch_kernel<<<nTiles, 256, 0, (cudaStream_t)stream>>>(jobs, tileJob);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_bipartite_fields(const float *J, int N0, int N1, const int8_t *qFixed, int side, float *F, int m,
                           void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (side == 1)  // F1[y][i] = sum_j J[i][j] q0[y][j]
        launch_bip_field<true, false, float>(qFixed, N0, J, N0, F, N1, m, N1, N0, s);
    else  // F0[y][j] = sum_i q1[y][i] J[i][j]
        launch_bip_field<false, false, float>(qFixed, N1, J, N0, F, N0, m, N0, N1, s);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_dense_energy(const float *J, int ldJ, const float *h, const double *c64, const int8_t *q, int N,
                       int m, int maximize, double *r_scratch, double *E64, float *E32, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    dim3 grid((N + 63) / 64, (m + 63) / 64);
    field_gemm_kernel<true, double><<<grid, 256, 0, s>>>(q, N, J, ldJ, r_scratch, N, m, N, N);
    dg_energy_finish<<<m, 256, 0, s>>>(q, N, h, r_scratch, c64, maximize ? -1. : 1., E64, E32);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_bipartite_energy(const float *J, const float *h0, const float *h1, const double *c64,
                           const int8_t *q0, const int8_t *q1, int N0, int N1, int m, int maximize,
                           double *r_scratch, double *E64, float *E32, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    launch_bip_field<true, true, double>(q0, N0, J, N0, r_scratch, N1, m, N1, N0, s);
    bg_energy_finish<<<m, 256, 0, s>>>(q0, q1, N0, N1, h0, h1, r_scratch, c64, maximize ? -1. : 1., E64,
                                       E32);
    return (int)cudaGetLastError();
}

}  // extern "C"

// ------------------------------------------------ no-allocation energy entry point
// sq103_dense_energy_static serves callers that cannot allocate device memory:
// code running inside a framework whose memory pool owns the whole device (a
// cudaMalloc there fails or fragments the pool), or a long-lived service that
// must keep its footprint fixed after start-up.  Its scratch, one m x N block
// of FP64 row sums, is this file-scope device array: every GPU that loads the
// library holds its kStaticEnergyElems doubles (2 MiB) until the process
// exits.  The spin GEMM writes every value it later reads, so nothing has to
// be cleared between calls.  There is one array per device: two calls that
// overlap in time (different streams or threads) race on it, so callers must
// serialise them.
static constexpr size_t kStaticEnergyElems = (size_t)1 << 18;
static __device__ __align__(256) double g_energy_scratch[kStaticEnergyElems];

namespace {
// device address of g_energy_scratch, looked up with cudaGetSymbolAddress by
// the first call on each device, with that device current (the host-side
// name is only a stand-in for the symbol).  That lookup is the call's only
// set-up work; make the first call on a device before any stream capture.
std::mutex g_scratch_mutex;
double *g_scratch_addr[256] = {};

int static_scratch(double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    if (dev < 0 || dev >= 256) return kErrBadShape;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_energy_scratch);
        if (e != cudaSuccess) return (int)e;
        g_scratch_addr[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_addr[dev];
    return 0;
}
}  // namespace

extern "C" {

SQ103_API unsigned long long sq103_dense_energy_static_max(void) { return (unsigned long long)kStaticEnergyElems; }

SQ103_API int sq103_dense_energy_static(const float *J, int ldJ, const float *h, const double *c64, const int8_t *q,
                                        int N, int m, int maximize, double *E64, float *E32, void *stream) {
    if (N <= 0 || m <= 0) {
        sq103_set_error("sq103_dense_energy_static: N and m must be positive.");
        return kErrBadShape;
    }
    if ((size_t)N * (size_t)m > kStaticEnergyElems) {
        char msg[160];
        snprintf(msg, sizeof(msg), "sq103_dense_energy_static: m * N = %zu exceeds the static scratch of %zu values.",
                 (size_t)N * (size_t)m, kStaticEnergyElems);
        sq103_set_error(msg);
        return kErrCapacity;
    }
    double *scratch = nullptr;
    int rc = static_scratch(&scratch);
    if (rc == kErrBadShape) {
        sq103_set_error("sq103_dense_energy_static: the current device number is 256 or more; the static "
                        "scratch addresses are kept for devices 0-255 only.");
        return rc;
    }
    if (rc != 0) {
        char msg[160];
        snprintf(msg, sizeof(msg), "sq103_dense_energy_static: looking up the static scratch failed: %s.",
                 cudaGetErrorString((cudaError_t)rc));
        sq103_set_error(msg);
        return rc;
    }
    return sq103_dense_energy(J, ldJ, h, c64, q, N, m, maximize, scratch, E64, E32, stream);
}

SQ103_API int sq103_ring_dot(const int8_t *q, int N, int m, long long *out, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemsetAsync(out, 0, sizeof(long long), s);
    int blocks = (int)(((size_t)m * N + 255) / 256);
    if (blocks > 1024) blocks = 1024;
    ring_dot<<<blocks, 256, 0, s>>>(q, N, m, out);
    return (int)cudaGetLastError();
}

}  // extern "C"

// ------------------------------------------------------------ FP64 formula sets
// The double-precision formula kernels (sqaodc/cuda/DeviceFormulas.cpp:24-140
// instantiated with real = double): plain FP64 sums over a fixed thread
// assignment and reduction tree, so a result does not depend on the launch.
// Bits (0 / 1) and spins (+-1) times FP64 couplings are exact products.
namespace sq103 {

// h_i = -1/2 sum_j W_ij, J = -W / 4 with a zero diagonal; rs_i = sum_j W_ij + W_ii
__global__ void __launch_bounds__(256) dg_hamiltonian64_rows(const double *W, int N, double *h, double *J,
                                                             double *rs) {
    __shared__ double red[8];
    const int i = blockIdx.x;
    double s = 0.;
    for (int j = threadIdx.x; j < N; j += 256) {
        const double w = W[(size_t)i * N + j];
        s += w;
        J[(size_t)i * N + j] = i == j ? 0. : -0.25 * w;
    }
    const double t = block_sum_f64<256>(s, red);
    if (threadIdx.x == 0) {
        h[i] = -0.5 * t;
        rs[i] = t + W[(size_t)i * N + i];
    }
}

// out = scale * sum v + add (one CTA)
__global__ void __launch_bounds__(256) sum_scaled64(const double *v, int n, double scale, const double *v2, int n2,
                                                    double scale2, double *out) {
    __shared__ double red[8];
    double s = 0., s2 = 0.;
    for (int i = threadIdx.x; i < n; i += 256) s += v[i];
    for (int i = threadIdx.x; i < n2; i += 256) s2 += v2[i];
    const double t = block_sum_f64<256>(s, red);
    const double t2 = block_sum_f64<256>(s2, red);
    if (threadIdx.x == 0) *out = scale * t + scale2 * t2;
}

// bipartite, W N1 x N0: h1_i = -1/4 sum_j W_ij - b1_i / 2, J = -W / 4, rs_i = sum_j W_ij
__global__ void __launch_bounds__(256) bg_hamiltonian64_rows(const double *W, const double *b1, int N0, double *h1,
                                                             double *J, double *rs) {
    __shared__ double red[8];
    const int i = blockIdx.x;
    double s = 0.;
    for (int j = threadIdx.x; j < N0; j += 256) {
        const double w = W[(size_t)i * N0 + j];
        s += w;
        J[(size_t)i * N0 + j] = -0.25 * w;
    }
    const double t = block_sum_f64<256>(s, red);
    if (threadIdx.x == 0) {
        h1[i] = -0.25 * t - 0.5 * b1[i];
        rs[i] = t;
    }
}

// h0_j = -1/4 sum_i W_ij - b0_j / 2 (a thread per column, rows ascending)
__global__ void bg_hamiltonian64_cols(const double *W, const double *b0, int N0, int N1, double *h0) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N0) return;
    double s = 0.;
    for (int i = 0; i < N1; ++i) s += W[(size_t)i * N0 + j];
    h0[j] = -0.25 * s - 0.5 * b0[j];
}

// E[y] = sign (-c - sum_i q_i (h_i + sum_j J_ij q_j)); h may be null (zero)
__global__ void __launch_bounds__(256) dense_energy64(const double *J, const double *h, double c, const int8_t *q,
                                                      int N, double sign, double *E) {
    __shared__ double red[8];
    const int y = blockIdx.x;
    const int8_t *qy = q + (size_t)y * N;
    double s = 0.;
    for (int i = threadIdx.x; i < N; i += 256) {
        const int qi = qy[i];
        if (qi == 0) continue;
        const double *Ji = J + (size_t)i * N;
        double d = 0.;
        for (int j = 0; j < N; ++j) d += Ji[j] * (double)qy[j];
        s += (double)qi * ((h ? h[i] : 0.) + d);
    }
    const double t = block_sum_f64<256>(s, red);
    if (threadIdx.x == 0) E[y] = sign * (-c - t);
}

// E[y] = sign (-c - h0.q0 - sum_i q1_i (h1_i + sum_j J_ij q0_j)), J N1 x N0
__global__ void __launch_bounds__(256) bipartite_energy64(const double *J, const double *h0, const double *h1,
                                                          double c, const int8_t *q0, const int8_t *q1, int N0,
                                                          int N1, double sign, double *E) {
    __shared__ double red[8];
    const int y = blockIdx.x;
    const int8_t *a = q0 + (size_t)y * N0, *b = q1 + (size_t)y * N1;
    double s = 0.;
    for (int j = threadIdx.x; j < N0; j += 256) s += (double)a[j] * h0[j];
    for (int i = threadIdx.x; i < N1; i += 256) {
        const int bi = b[i];
        if (bi == 0) continue;
        const double *Ji = J + (size_t)i * N0;
        double d = 0.;
        for (int j = 0; j < N0; ++j) d += Ji[j] * (double)a[j];
        s += (double)bi * (h1[i] + d);
    }
    const double t = block_sum_f64<256>(s, red);
    if (threadIdx.x == 0) E[y] = sign * (-c - t);
}

}  // namespace sq103

extern "C" {

SQ103_API int sq103_dense_hamiltonian64(const double *W, int N, double *h, double *J, double *c, double *scratch,
                                        void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (N <= 0) return kErrBadShape;
    dg_hamiltonian64_rows<<<N, 256, 0, s>>>(W, N, h, J, scratch);
    sum_scaled64<<<1, 256, 0, s>>>(scratch, N, -0.25, nullptr, 0, 0., c);  // c = -(sum W + tr W) / 4
    return (int)cudaGetLastError();
}

SQ103_API int sq103_dense_energy64(const double *J, const double *h, double c, const int8_t *q, int N, int m,
                                   int maximize, double *E, void *stream) {
    if (N <= 0 || m <= 0) return kErrBadShape;
    dense_energy64<<<m, 256, 0, (cudaStream_t)stream>>>(J, h, c, q, N, maximize ? -1. : 1., E);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_bipartite_hamiltonian64(const double *b0, const double *b1, const double *W, int N0, int N1,
                                            double *h0, double *h1, double *J, double *c, double *scratch,
                                            void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (N0 <= 0 || N1 <= 0) return kErrBadShape;
    bg_hamiltonian64_rows<<<N1, 256, 0, s>>>(W, b1, N0, h1, J, scratch);
    bg_hamiltonian64_cols<<<(N0 + 127) / 128, 128, 0, s>>>(W, b0, N0, N1, h0);
    // c = -(sum W) / 4 - (sum b0 + sum b1) / 2: the row sums, then b0 and b1 (copied after them)
    cudaMemcpyAsync(scratch + N1, b0, sizeof(double) * N0, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(scratch + N1 + N0, b1, sizeof(double) * N1, cudaMemcpyDeviceToDevice, s);
    sum_scaled64<<<1, 256, 0, s>>>(scratch, N1, -0.25, scratch + N1, N0 + N1, -0.5, c);
    return (int)cudaGetLastError();
}

SQ103_API int sq103_bipartite_energy64(const double *J, const double *h0, const double *h1, double c,
                                       const int8_t *q0, const int8_t *q1, int N0, int N1, int m, int maximize,
                                       double *E, void *stream) {
    if (N0 <= 0 || N1 <= 0 || m <= 0) return kErrBadShape;
    bipartite_energy64<<<m, 256, 0, (cudaStream_t)stream>>>(J, h0, h1, c, q0, q1, N0, N1, maximize ? -1. : 1., E);
    return (int)cudaGetLastError();
}

}  // extern "C"
