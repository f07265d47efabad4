/*
 * oracle.c -- CPU oracle for the sqaod annealing / brute-force-search hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): used by tests/, smoke() and the
 * cpu_baseline / reference legs of bench.py; never linked into the product.
 *
 * Compiled with -ffp-contract=off so that every fused multiply-add below is
 * an explicit fmaf() and the arithmetic order is exactly the one written.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MIN(a, b) ((a) < (b) ? (a) : (b))
#define ORC_MAX(a, b) ((a) > (b) ? (a) : (b))

static int round_up(int v, int base) { return (v + base - 1) / base * base; }

static int omp_workers(int n) {
#ifdef _OPENMP
    return n > 0 ? n : omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

static int omp_tid(void) {
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

/* ===================================================== Philox4x32-10 ==== */
/* Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
 * SC'11: 10 rounds of the 4x32 Philox S-box with multipliers 0xD2511F53 and
 * 0xCD9E8D57 and Weyl key increments 0x9E3779B9 / 0xBB67AE85. */
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static void philox_draw(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t step, uint32_t tag,
                        uint32_t out[4]) {
    uint32_t ctr[4] = {c0, c1, step, tag};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    orc_philox(ctr, key, out);
}

/* index in [0, n): high word of w * n (the build's site / trotter draw) */
static int mulhi_index(uint32_t w, int n) { return (int)(((uint64_t)w * (uint32_t)n) >> 32); }
/* uniform in [0, 1) with 24-bit resolution, exact in fp32 */
static float unit_float(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }

/* ============================================================ MT19937 ==== */
/* Matsumoto & Nishimura's MT19937 as used by sqaod::Random
 * (sqaodc/common/Random.cpp:70-168): init_genrand seeding, 624-word twist,
 * tempering; randInt(n) = u32 % n; random<float>() = float(u32) * 2^-32;
 * random<double>() = 53-bit from two words. */
enum { MT_N = 624, MT_M = 397 };

void orc_mt_seed(orc_mt *r, unsigned long long s) {
    r->mt[0] = (uint32_t)(s & 0xffffffffULL);
    for (int i = 1; i < MT_N; ++i)
        r->mt[i] = 1812433253u * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t)i;
    r->mti = MT_N;
}

uint32_t orc_mt_u32(orc_mt *r) {
    static const uint32_t mag01[2] = {0x0u, 0x9908b0dfu};
    uint32_t y;
    if (r->mti >= MT_N) {
        int kk;
        for (kk = 0; kk < MT_N - MT_M; ++kk) {
            y = (r->mt[kk] & 0x80000000u) | (r->mt[kk + 1] & 0x7fffffffu);
            r->mt[kk] = r->mt[kk + MT_M] ^ (y >> 1) ^ mag01[y & 1u];
        }
        for (; kk < MT_N - 1; ++kk) {
            y = (r->mt[kk] & 0x80000000u) | (r->mt[kk + 1] & 0x7fffffffu);
            r->mt[kk] = r->mt[kk + (MT_M - MT_N)] ^ (y >> 1) ^ mag01[y & 1u];
        }
        y = (r->mt[MT_N - 1] & 0x80000000u) | (r->mt[0] & 0x7fffffffu);
        r->mt[MT_N - 1] = r->mt[MT_M - 1] ^ (y >> 1) ^ mag01[y & 1u];
        r->mti = 0;
    }
    y = r->mt[r->mti++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}

uint32_t orc_mt_randint(orc_mt *r, int n) { return orc_mt_u32(r) % (uint32_t)n; }

float orc_mt_f32(orc_mt *r) { return (float)orc_mt_u32(r) * (float)(1. / 4294967296.); }

double orc_mt_f64(orc_mt *r) {
    uint32_t a = orc_mt_u32(r) >> 5, b = orc_mt_u32(r) >> 6;
    return (a * 67108864.0 + b) * (1.0 / 9007199254740992.0);
}

void orc_mt_stream(unsigned long long s, int n, uint32_t *out) {
    orc_mt r;
    orc_mt_seed(&r, s);
    for (int i = 0; i < n; ++i)
        out[i] = orc_mt_u32(&r);
}

/* =============================================== reference dot (AVX2) ==== */
/* sqaodc/cpu/Dot_SIMD.cpp:160-210 (float dot_avx2): two 8-lane FMA
 * accumulators over 16-float blocks, then lane sum, quad fold, dual fold. */
float orc_dot_ref(const float *v0, const float *v1, int N) {
    float s0[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float s1[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int nBlocks = (N + 15) / 16;
    for (int b = 0; b < nBlocks; ++b) {
        const float *a = v0 + 16 * b, *c = v1 + 16 * b;
        for (int l = 0; l < 8; ++l)
            s0[l] = fmaf(a[l], c[l], s0[l]);
        for (int l = 0; l < 8; ++l)
            s1[l] = fmaf(a[8 + l], c[8 + l], s1[l]);
    }
    float s[8];
    for (int l = 0; l < 8; ++l)
        s[l] = s0[l] + s1[l];
    float q0 = s[0] + s[4], q1 = s[1] + s[5], q2 = s[2] + s[6], q3 = s[3] + s[7];
    float d0 = q0 + q2, d1 = q1 + q3;
    return d0 + d1;
}

/* =========================================================== formulas ==== */
/* sqaodc/cpu/SharedFormulas.cpp:36-55 / sqaodpy/sqaod/py/formulas.py:6-33:
 * h_i = -1/2 sum_j W_ij ; J = -W/4 with zero diagonal ;
 * c = sum(-W/4) + sum(diag(-W/4)). */
void orc_dg_hamiltonian(const double *W, int N, double *h, double *J, double *c) {
    double sumJ = 0., diag = 0.;
    for (int i = 0; i < N; ++i) {
        double rs = 0.;
        for (int j = 0; j < N; ++j) {
            rs += W[(size_t)i * N + j];
            double v = -0.25 * W[(size_t)i * N + j];
            sumJ += v;
            J[(size_t)i * N + j] = (i == j) ? 0. : v;
        }
        h[i] = -0.5 * rs;
        diag += -0.25 * W[(size_t)i * N + i];
    }
    *c = sumJ + diag;
}

/* E = x^T W x (sqaodc/cpu/SharedFormulas.cpp:10-33; py/formulas.py:37-76) */
void orc_dg_energy_qubo(const double *W, int N, const int8_t *x, int n, double *E) {
    for (int s = 0; s < n; ++s) {
        const int8_t *xs = x + (size_t)s * N;
        double e = 0.;
        for (int i = 0; i < N; ++i) {
            if (!xs[i]) continue;
            double r = 0.;
            for (int j = 0; j < N; ++j)
                r += W[(size_t)i * N + j] * xs[j];
            e += r;
        }
        E[s] = e;
    }
}

/* E = -c - h.q - q^T J q (sqaodc/cpu/SharedFormulas.cpp:58-85; py/formulas.py:79-116) */
void orc_dg_energy_ising(const double *h, const double *J, double c, int N,
                         const int8_t *q, int m, double *E) {
    for (int y = 0; y < m; ++y) {
        const int8_t *qy = q + (size_t)y * N;
        double hq = 0., qJq = 0.;
        for (int i = 0; i < N; ++i) {
            hq += h[i] * qy[i];
            double r = 0.;
            for (int j = 0; j < N; ++j)
                r += J[(size_t)i * N + j] * qy[j];
            qJq += qy[i] * r;
        }
        E[y] = -c - hq - qJq;
    }
}

/* sqaodc/cpu/SharedFormulas.cpp:148-167: J = -W/4 (N1 x N0);
 * h0 = -1/4 colsum(W) - b0/2; h1 = -1/4 rowsum(W) - b1/2;
 * c = -1/4 sum(W) - 1/2 (sum b0 + sum b1). */
void orc_bg_hamiltonian(const double *b0, const double *b1, const double *W, int N0, int N1,
                        double *h0, double *h1, double *J, double *c) {
    double sumW = 0., sb0 = 0., sb1 = 0.;
    for (int j = 0; j < N0; ++j) h0[j] = 0.;
    for (int i = 0; i < N1; ++i) {
        double rs = 0.;
        for (int j = 0; j < N0; ++j) {
            double w = W[(size_t)i * N0 + j];
            J[(size_t)i * N0 + j] = -0.25 * w;
            rs += w;
            h0[j] += w;
            sumW += w;
        }
        h1[i] = -0.25 * rs - 0.5 * b1[i];
        sb1 += b1[i];
    }
    for (int j = 0; j < N0; ++j) {
        h0[j] = -0.25 * h0[j] - 0.5 * b0[j];
        sb0 += b0[j];
    }
    *c = -0.25 * sumW - 0.5 * (sb0 + sb1);
}

static double bg_qubo_one(const double *b0, const double *b1, const double *W, int N0, int N1,
                          const int8_t *x0, const int8_t *x1) {
    double e = 0.;
    for (int j = 0; j < N0; ++j) e += b0[j] * x0[j];
    for (int i = 0; i < N1; ++i) {
        e += b1[i] * x1[i];
        if (!x1[i]) continue;
        double r = 0.;
        for (int j = 0; j < N0; ++j) r += W[(size_t)i * N0 + j] * x0[j];
        e += r;
    }
    return e;
}

/* E = b0.x0 + b1.x1 + x1^T W x0 (sqaodc/cpu/SharedFormulas.cpp:91-120) */
void orc_bg_energy_qubo(const double *b0, const double *b1, const double *W, int N0, int N1,
                        const int8_t *x0, const int8_t *x1, int n, double *E) {
    for (int s = 0; s < n; ++s)
        E[s] = bg_qubo_one(b0, b1, W, N0, N1, x0 + (size_t)s * N0, x1 + (size_t)s * N1);
}

/* E[i1][i0] over all pairs (sqaodc/cpu/SharedFormulas.cpp:123-144) */
void orc_bg_energy_qubo_2d(const double *b0, const double *b1, const double *W, int N0, int N1,
                           const int8_t *x0, int n0, const int8_t *x1, int n1, double *E) {
    for (int s1 = 0; s1 < n1; ++s1)
        for (int s0 = 0; s0 < n0; ++s0)
            E[(size_t)s1 * n0 + s0] =
                bg_qubo_one(b0, b1, W, N0, N1, x0 + (size_t)s0 * N0, x1 + (size_t)s1 * N1);
}

/* E = -(h0.q0 + h1.q1 + q1^T J q0) - c (sqaodc/cpu/SharedFormulas.cpp:171-202) */
void orc_bg_energy_ising(const double *h0, const double *h1, const double *J, double c,
                         int N0, int N1, const int8_t *q0, const int8_t *q1, int m, double *E) {
    for (int y = 0; y < m; ++y) {
        const int8_t *a = q0 + (size_t)y * N0, *b = q1 + (size_t)y * N1;
        double e = 0.;
        for (int j = 0; j < N0; ++j) e += h0[j] * a[j];
        for (int i = 0; i < N1; ++i) {
            e += h1[i] * b[i];
            double r = 0.;
            for (int j = 0; j < N0; ++j) r += J[(size_t)i * N0 + j] * a[j];
            e += b[i] * r;
        }
        E[y] = -e - c;
    }
}

/* ======================================================= BF searchers ==== */

static float dg_state_energy(const double *Wd, int N, uint64_t x) {
    /* bit (N-1-i) of x is variable i: MSB-first (sqaodc/common/Common.cpp:79-93) */
    double e = 0.;
    for (int i = 0; i < N; ++i) {
        if (!((x >> (N - 1 - i)) & 1ull)) continue;
        const double *row = Wd + (size_t)i * N;
        for (int j = 0; j < N; ++j)
            if ((x >> (N - 1 - j)) & 1ull)
                e += row[j];
    }
    return (float)e;
}

static int cmp_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : (x > y);
}

typedef struct {
    float Emin;
    uint64_t *list;
    int n;
} bf_worker;

/* sqaodc/cpu/CPUDenseGraphBatchSearch.cpp:26-50: per-tile scan */
static void dg_batch_search(const double *Wd, int N, uint64_t xb, uint64_t xe, int tileSize,
                            bf_worker *w) {
    for (uint64_t x = xb; x < xe; ++x) {
        float e = dg_state_energy(Wd, N, x);
        if (e > w->Emin) continue;
        if (e == w->Emin) {
            if (w->n < tileSize) w->list[w->n++] = x;
        } else {
            w->Emin = e;
            w->n = 0;
            w->list[w->n++] = x;
        }
    }
}

/* sqaodc/cpu/CPUDenseGraphBFSearcher.cpp:29-139,166-198 */
int orc_dg_bf_search_ref(const float *W, int N, int om, int tileSize, int nWorkers,
                         float *Emin, uint64_t *xout, int cap) {
    int nw = omp_workers(nWorkers);
    double *Wd = (double *)malloc(sizeof(double) * N * N);
    for (int i = 0; i < N * N; ++i) Wd[i] = (om == 1) ? -(double)W[i] : (double)W[i];
    uint64_t xMax = 1ull << N;
    if (xMax < (uint64_t)tileSize) tileSize = (int)xMax;
    bf_worker *ws = (bf_worker *)calloc(nw, sizeof(bf_worker));
    for (int t = 0; t < nw; ++t) {
        ws[t].Emin = FLT_MAX;
        ws[t].list = (uint64_t *)malloc(sizeof(uint64_t) * tileSize);
    }
    for (uint64_t x = 0; x < xMax; x = ORC_MIN(x + (uint64_t)tileSize * nw, xMax)) {
#pragma omp parallel for num_threads(nw) schedule(static, 1)
        for (int t = 0; t < nw; ++t) {
            uint64_t b = ORC_MIN(x + (uint64_t)tileSize * t, xMax);
            uint64_t e = ORC_MIN(x + (uint64_t)tileSize * (t + 1), xMax);
            if (b < e) dg_batch_search(Wd, N, b, e, tileSize, &ws[t]);
        }
    }
    /* merge (CPUDenseGraphBFSearcher.cpp:104-131) */
    float E = FLT_MAX;
    uint64_t *merged = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)tileSize * (nw + 1));
    int nm = 0;
    for (int t = 0; t < nw; ++t) {
        if (ws[t].Emin < E) {
            E = ws[t].Emin;
            memcpy(merged, ws[t].list, sizeof(uint64_t) * ws[t].n);
            nm = ws[t].n;
        } else if (ws[t].Emin == E) {
            if (nm < tileSize) {
                memcpy(merged + nm, ws[t].list, sizeof(uint64_t) * ws[t].n);
                nm += ws[t].n;
            }
        }
    }
    qsort(merged, nm, sizeof(uint64_t), cmp_u64);
    int nsol = ORC_MIN(ORC_MIN(tileSize, nm), cap);
    memcpy(xout, merged, sizeof(uint64_t) * nsol);
    *Emin = (om == 1) ? -E : E;
    for (int t = 0; t < nw; ++t) free(ws[t].list);
    free(ws);
    free(merged);
    free(Wd);
    return nsol;
}

int orc_dg_bf_search_range(const float *W, int N, int om, uint64_t xBegin, uint64_t xEnd,
                           int cap, float *Emin, uint64_t *xout) {
    double *Wd = (double *)malloc(sizeof(double) * N * N);
    for (int i = 0; i < N * N; ++i) Wd[i] = (om == 1) ? -(double)W[i] : (double)W[i];
    float E = FLT_MAX;
    int n = 0;
    for (uint64_t x = xBegin; x < xEnd; ++x) {
        float e = dg_state_energy(Wd, N, x);
        if (e > E) continue;
        if (e < E) { E = e; n = 0; }
        if (n < cap) xout[n] = x;
        ++n;
    }
    *Emin = (om == 1) ? -E : E;
    free(Wd);
    return ORC_MIN(n, cap);
}

/* Per-tile fp32 formulation of sqaodc/cpu/CPUDenseGraphBatchSearch.cpp:26-50
 * (bits matrix, X*W, row-wise dot with X, scan), for the CPU baseline. */
float orc_dg_bf_sweep_tiles(const float *W, int N, uint64_t xBegin, int tileSize, int nTiles,
                            int nWorkers) {
    int nw = omp_workers(nWorkers);
    float gmin = FLT_MAX;
#pragma omp parallel num_threads(nw)
    {
        float *X = (float *)malloc(sizeof(float) * tileSize * N);
        float *t = (float *)malloc(sizeof(float) * N);
        float lmin = FLT_MAX;
        int nlist = 0;
#pragma omp for schedule(static, 1)
        for (int tile = 0; tile < nTiles; ++tile) {
            uint64_t xb = xBegin + (uint64_t)tile * tileSize;
            for (int s = 0; s < tileSize; ++s)
                for (int p = 0; p < N; ++p)
                    X[(size_t)s * N + p] = (float)(((xb + s) >> (N - 1 - p)) & 1ull);
            for (int s = 0; s < tileSize; ++s) {
                const float *xs = X + (size_t)s * N;
                for (int i = 0; i < N; ++i) t[i] = 0.f;
                for (int j = 0; j < N; ++j) {
                    float xj = xs[j];
                    const float *wr = W + (size_t)j * N;
                    for (int i = 0; i < N; ++i) t[i] = fmaf(xj, wr[i], t[i]);
                }
                float e = 0.f;
                for (int i = 0; i < N; ++i) e = fmaf(t[i], xs[i], e);
                if (e > lmin) continue;
                if (e == lmin) { ++nlist; } else { lmin = e; nlist = 1; }
            }
        }
#pragma omp critical
        { if (lmin < gmin) gmin = lmin; }
        (void)nlist;
        free(X);
        free(t);
    }
    return gmin;
}

typedef struct {
    float Emin;
    uint64_t *pairs; /* 2 words per entry */
    int n;
} bg_worker;

static float bg_pair_energy(const double *b0, const double *b1, const double *W, int N0, int N1,
                            uint64_t x0, uint64_t x1) {
    double e = 0.;
    for (int j = 0; j < N0; ++j)
        if ((x0 >> (N0 - 1 - j)) & 1ull) e += b0[j];
    for (int i = 0; i < N1; ++i) {
        if (!((x1 >> (N1 - 1 - i)) & 1ull)) continue;
        e += b1[i];
        const double *row = W + (size_t)i * N0;
        for (int j = 0; j < N0; ++j)
            if ((x0 >> (N0 - 1 - j)) & 1ull) e += row[j];
    }
    return (float)e;
}

/* sqaodc/cpu/CPUBipartiteGraphBatchSearch.cpp:29-66 */
static void bg_batch_search(const double *b0, const double *b1, const double *W, int N0, int N1,
                            uint64_t x0b, uint64_t x0e, uint64_t x1b, uint64_t x1e, bg_worker *w) {
    int maxN = N0 + N1;
    for (uint64_t x1 = x1b; x1 < x1e; ++x1)
        for (uint64_t x0 = x0b; x0 < x0e; ++x0) {
            float e = bg_pair_energy(b0, b1, W, N0, N1, x0, x1);
            if (e > w->Emin) continue;
            if (e == w->Emin) {
                if (w->n < maxN) {
                    w->pairs[2 * w->n] = x0;
                    w->pairs[2 * w->n + 1] = x1;
                    w->n++;
                }
            } else {
                w->Emin = e;
                w->n = 0;
                w->pairs[0] = x0;
                w->pairs[1] = x1;
                w->n = 1;
            }
        }
}

/* sqaodc/cpu/CPUBipartiteGraphBFSearcher.cpp:29-293 */
int orc_bg_bf_search_ref(const float *b0f, const float *b1f, const float *Wf, int N0, int N1,
                         int om, int tileSize0, int tileSize1, int nWorkers,
                         float *Emin, uint64_t *xout, int cap) {
    int nw = omp_workers(nWorkers);
    double sgn = (om == 1) ? -1. : 1.;
    double *b0 = (double *)malloc(sizeof(double) * N0), *b1 = (double *)malloc(sizeof(double) * N1);
    double *W = (double *)malloc(sizeof(double) * N0 * N1);
    for (int j = 0; j < N0; ++j) b0[j] = sgn * b0f[j];
    for (int i = 0; i < N1; ++i) b1[i] = sgn * b1f[i];
    for (int k = 0; k < N0 * N1; ++k) W[k] = sgn * Wf[k];
    uint64_t x0max = 1ull << N0, x1max = 1ull << N1;
    if (x0max < (uint64_t)tileSize0) tileSize0 = (int)x0max;
    if (x1max < (uint64_t)tileSize1) tileSize1 = (int)x1max;
    bg_worker *ws = (bg_worker *)calloc(nw, sizeof(bg_worker));
    for (int t = 0; t < nw; ++t) {
        ws[t].Emin = FLT_MAX;
        ws[t].pairs = (uint64_t *)malloc(sizeof(uint64_t) * 2 * (N0 + N1));
    }
    uint64_t *bb0 = (uint64_t *)malloc(sizeof(uint64_t) * nw), *be0 = (uint64_t *)malloc(sizeof(uint64_t) * nw);
    uint64_t *bb1 = (uint64_t *)malloc(sizeof(uint64_t) * nw), *be1 = (uint64_t *)malloc(sizeof(uint64_t) * nw);
    uint64_t x0 = 0, x1 = 0;
    while (x0 != x0max) {
        uint64_t cx0 = x0, cx0end = ORC_MIN(cx0 + tileSize0, x0max), cx1 = x1;
        for (int t = 0; t < nw; ++t) {
            bb1[t] = cx1;
            uint64_t cx1end = ORC_MIN(cx1 + tileSize1, x1max);
            be1[t] = cx1end;
            bb0[t] = cx0;
            be0[t] = cx0end;
            cx1 = cx1end;
            if (cx1 == x1max) {
                cx1 = 0;
                cx0 = ORC_MIN(cx0 + tileSize0, x0max);
                cx0end = ORC_MIN(cx0 + tileSize0, x0max);
            }
        }
#pragma omp parallel for num_threads(nw) schedule(static, 1)
        for (int t = 0; t < nw; ++t)
            if (bb0[t] < be0[t] && bb1[t] < be1[t])
                bg_batch_search(b0, b1, W, N0, N1, bb0[t], be0[t], bb1[t], be1[t], &ws[t]);
        x0 = bb0[nw - 1];
        x1 = be1[nw - 1];
        if (x1 == x1max) {
            x1 = 0;
            x0 = ORC_MIN(x0 + tileSize0, x0max);
        }
    }
    /* merge (CPUBipartiteGraphBFSearcher.cpp:117-151): no sort */
    int nMax = tileSize0 + tileSize1;
    float E = FLT_MAX;
    uint64_t *merged = (uint64_t *)malloc(sizeof(uint64_t) * 2 * (size_t)(N0 + N1) * (nw + 1));
    int nm = 0;
    for (int t = 0; t < nw; ++t) {
        if (ws[t].Emin < E) {
            E = ws[t].Emin;
            memcpy(merged, ws[t].pairs, sizeof(uint64_t) * 2 * ws[t].n);
            nm = ws[t].n;
        } else if (ws[t].Emin == E) {
            if (nm < nMax) {
                memcpy(merged + 2 * nm, ws[t].pairs, sizeof(uint64_t) * 2 * ws[t].n);
                nm += ws[t].n;
            }
        }
    }
    int nsol = ORC_MIN(ORC_MIN(nMax, nm), cap);
    memcpy(xout, merged, sizeof(uint64_t) * 2 * nsol);
    *Emin = (om == 1) ? -E : E;
    for (int t = 0; t < nw; ++t) free(ws[t].pairs);
    free(ws); free(merged); free(b0); free(b1); free(W);
    free(bb0); free(be0); free(bb1); free(be1);
    return nsol;
}

int orc_bg_bf_search_sorted(const float *b0f, const float *b1f, const float *Wf, int N0, int N1,
                            int om, int cap, float *Emin, uint64_t *xout) {
    double sgn = (om == 1) ? -1. : 1.;
    double *b0 = (double *)malloc(sizeof(double) * N0), *b1 = (double *)malloc(sizeof(double) * N1);
    double *W = (double *)malloc(sizeof(double) * N0 * N1);
    for (int j = 0; j < N0; ++j) b0[j] = sgn * b0f[j];
    for (int i = 0; i < N1; ++i) b1[i] = sgn * b1f[i];
    for (int k = 0; k < N0 * N1; ++k) W[k] = sgn * Wf[k];
    float E = FLT_MAX;
    int n = 0;
    for (uint64_t x0 = 0; x0 < (1ull << N0); ++x0)
        for (uint64_t x1 = 0; x1 < (1ull << N1); ++x1) {
            float e = bg_pair_energy(b0, b1, W, N0, N1, x0, x1);
            if (e > E) continue;
            if (e < E) { E = e; n = 0; }
            if (n < cap) { xout[2 * n] = x0; xout[2 * n + 1] = x1; }
            ++n;
        }
    *Emin = (om == 1) ? -E : E;
    free(b0); free(b1); free(W);
    return ORC_MIN(n, cap);
}

/* ========================================= reference CPU annealers ==== */

struct orc_dga {
    int N, m, stride, nw;
    float *h, *J, c; /* J rows zero-padded to stride */
    float *q;        /* m x stride, zero-padded */
    orc_mt *rng;     /* one per worker, seed + 17 * idx */
};

orc_dga *orc_dga_new(int N, int m, int nWorkers) {
    orc_dga *a = (orc_dga *)calloc(1, sizeof(orc_dga));
    a->N = N;
    a->m = m;
    a->stride = round_up(N, 16);
    a->nw = omp_workers(nWorkers);
    a->h = (float *)calloc(N, sizeof(float));
    a->J = (float *)calloc((size_t)N * a->stride, sizeof(float));
    a->q = (float *)calloc((size_t)m * a->stride, sizeof(float));
    a->rng = (orc_mt *)calloc(a->nw, sizeof(orc_mt));
    for (int t = 0; t < a->nw; ++t) orc_mt_seed(&a->rng[t], 5489u + 17u * t);
    return a;
}

void orc_dga_free(orc_dga *a) {
    if (!a) return;
    free(a->h); free(a->J); free(a->q); free(a->rng); free(a);
}

int orc_dga_workers(const orc_dga *a) { return a->nw; }

void orc_dga_set_hamiltonian(orc_dga *a, const float *h, const float *J, float c) {
    memcpy(a->h, h, sizeof(float) * a->N);
    for (int i = 0; i < a->N; ++i)
        memcpy(a->J + (size_t)i * a->stride, J + (size_t)i * a->N, sizeof(float) * a->N);
    a->c = c;
}

/* CPUDenseGraphAnnealer.cpp:29-33 */
void orc_dga_seed(orc_dga *a, unsigned long long seed) {
    for (int t = 0; t < a->nw; ++t) orc_mt_seed(&a->rng[t], seed + 17ull * t);
}

/* CPUDenseGraphAnnealer.cpp:151-161 */
void orc_dga_randomize(orc_dga *a) {
    for (int y = 0; y < a->m; ++y)
        for (int x = 0; x < a->N; ++x)
            a->q[(size_t)y * a->stride + x] = orc_mt_randint(&a->rng[0], 2) ? 1.f : -1.f;
}

void orc_dga_set_q(orc_dga *a, const int8_t *q) {
    for (int y = 0; y < a->m; ++y)
        for (int x = 0; x < a->N; ++x)
            a->q[(size_t)y * a->stride + x] = (float)q[(size_t)y * a->N + x];
}

void orc_dga_get_q(const orc_dga *a, int8_t *q) {
    for (int y = 0; y < a->m; ++y)
        for (int x = 0; x < a->N; ++x)
            q[(size_t)y * a->N + x] = (int8_t)a->q[(size_t)y * a->stride + x];
}

/* tryFlip, CPUDenseGraphAnnealer.cpp:251-265 */
static void dga_try_flip(orc_dga *a, int y, orc_mt *r, float twoDivM, float coef, float beta) {
    int N = a->N, m = a->m;
    int x = (int)orc_mt_randint(r, N);
    float *qy = a->q + (size_t)y * a->stride;
    float qyx = qy[x];
    float sum = orc_dot_ref(a->J + (size_t)x * a->stride, qy, N);
    float dE = twoDivM * qyx * (a->h[x] + 2.f * sum);
    int n0 = (y == 0) ? m - 1 : y - 1;
    int n1 = (y == m - 1) ? 0 : y + 1;
    dE -= qyx * (a->q[(size_t)n0 * a->stride + x] + a->q[(size_t)n1 * a->stride + x]) * coef;
    float threshold = (dE < 0.f) ? 1.f : expf(-dE * beta);
    if (threshold > orc_mt_f32(r)) qy[x] = -qyx;
}

/* tryFlipSA, CPUDenseGraphAnnealer.cpp:342-352 */
static void dga_try_flip_sa(orc_dga *a, int y, orc_mt *r, float invKT) {
    int N = a->N;
    int x = (int)orc_mt_randint(r, N);
    float *qy = a->q + (size_t)y * a->stride;
    float qyx = qy[x];
    float sum = orc_dot_ref(a->J + (size_t)x * a->stride, qy, N);
    float dE = 2.f * qyx * (a->h[x] + 2.f * sum);
    float threshold = (dE < 0.f) ? 1.f : expf(-dE * invKT);
    if (threshold > orc_mt_f32(r)) qy[x] = -qyx;
}

void orc_dga_step(orc_dga *a, int algo, float G, float beta) {
    int N = a->N, m = a->m;
    float twoDivM = 2.f / (float)m;
    float coef = logf(tanhf(G * beta / (float)m)) / beta;
    if (algo == ORC_ALGO_NAIVE) {
        /* annealOneStepNaive, CPUDenseGraphAnnealer.cpp:268-279 */
        orc_mt *r = &a->rng[0];
        for (long loop = 0; loop < (long)N * m; ++loop) {
            int y = (int)orc_mt_randint(r, m);
            dga_try_flip(a, y, r, twoDivM, coef, beta);
        }
    } else if (algo == ORC_ALGO_COLORING) {
        if (a->nw == 1) {
            /* annealOneStepColoring / annealColoredPlane, :282-301 */
            for (int idx = 0; idx < N; ++idx)
                for (int off = 0; off < 2; ++off)
                    for (int y = off; y < m; y += 2)
                        dga_try_flip(a, y, &a->rng[0], twoDivM, coef, beta);
        } else {
            /* annealOneStepColoringParallel / annealColoredPlaneParallel, :304-338 */
            int m2 = (m / 2) * 2;
            for (int idx = 0; idx < N; ++idx) {
#pragma omp parallel num_threads(a->nw)
                {
                    orc_mt *r = &a->rng[omp_tid()];
#pragma omp for schedule(static)
                    for (int y = 0; y < m2; y += 2)
                        dga_try_flip(a, y, r, twoDivM, coef, beta);
                }
                if (m % 2) dga_try_flip(a, m - 1, &a->rng[0], twoDivM, coef, beta);
#pragma omp parallel num_threads(a->nw)
                {
                    orc_mt *r = &a->rng[omp_tid()];
#pragma omp for schedule(static)
                    for (int y = 1; y < m2; y += 2)
                        dga_try_flip(a, y, r, twoDivM, coef, beta);
                }
            }
        }
    } else {
        /* annealOneStepSANaive, :355-371.  The reference takes the worker's
         * generator outside the parallel region (every thread then shares
         * random_[0]); here each thread uses its own generator. */
        float invKT = 1.f / G;
#pragma omp parallel num_threads(a->nw)
        {
            orc_mt *r = &a->rng[omp_tid()];
#pragma omp for schedule(static)
            for (int y = 0; y < m; ++y)
                for (int loop = 0; loop < N; ++loop)
                    dga_try_flip_sa(a, y, r, invKT);
        }
    }
}

void orc_dga_energy(const orc_dga *a, double *E) {
    int N = a->N;
    for (int y = 0; y < a->m; ++y) {
        const float *qy = a->q + (size_t)y * a->stride;
        double hq = 0., qJq = 0.;
        for (int i = 0; i < N; ++i) {
            hq += (double)a->h[i] * qy[i];
            double r = 0.;
            const float *Ji = a->J + (size_t)i * a->stride;
            for (int j = 0; j < N; ++j) r += (double)Ji[j] * qy[j];
            qJq += qy[i] * r;
        }
        E[y] = -(double)a->c - hq - qJq;
    }
}

struct orc_bga {
    int N0, N1, m, nw;
    float *h0, *h1, *J, c; /* J: N1 x N0 */
    float *q0, *q1;        /* m x N0, m x N1 */
    float *dE;             /* scratch m x max(N0, N1) */
    orc_mt *rng;
};

orc_bga *orc_bga_new(int N0, int N1, int m, int nWorkers) {
    orc_bga *a = (orc_bga *)calloc(1, sizeof(orc_bga));
    a->N0 = N0; a->N1 = N1; a->m = m;
    a->nw = omp_workers(nWorkers);
    a->h0 = (float *)calloc(N0, sizeof(float));
    a->h1 = (float *)calloc(N1, sizeof(float));
    a->J = (float *)calloc((size_t)N0 * N1, sizeof(float));
    a->q0 = (float *)calloc((size_t)m * N0, sizeof(float));
    a->q1 = (float *)calloc((size_t)m * N1, sizeof(float));
    a->dE = (float *)calloc((size_t)m * ORC_MAX(N0, N1), sizeof(float));
    a->rng = (orc_mt *)calloc(a->nw, sizeof(orc_mt));
    for (int t = 0; t < a->nw; ++t) orc_mt_seed(&a->rng[t], 5489u + 17u * t);
    return a;
}

int orc_bga_workers(const orc_bga *a) { return a->nw; }

void orc_bga_free(orc_bga *a) {
    if (!a) return;
    free(a->h0); free(a->h1); free(a->J); free(a->q0); free(a->q1); free(a->dE); free(a->rng);
    free(a);
}

void orc_bga_set_hamiltonian(orc_bga *a, const float *h0, const float *h1, const float *J, float c) {
    memcpy(a->h0, h0, sizeof(float) * a->N0);
    memcpy(a->h1, h1, sizeof(float) * a->N1);
    memcpy(a->J, J, sizeof(float) * a->N0 * a->N1);
    a->c = c;
}

void orc_bga_seed(orc_bga *a, unsigned long long seed) {
    for (int t = 0; t < a->nw; ++t) orc_mt_seed(&a->rng[t], seed + 17ull * t);
}

/* CPUBipartiteGraphAnnealer.cpp:188-228 */
void orc_bga_randomize(orc_bga *a) {
#pragma omp parallel num_threads(a->nw)
    {
        orc_mt *r = &a->rng[omp_tid()];
#pragma omp for schedule(static)
        for (int im = 0; im < a->m; ++im) {
            float *q = a->q0 + (size_t)im * a->N0;
            for (int i = 0; i < a->N0; ++i) q[i] = orc_mt_randint(r, 2) ? 1.f : -1.f;
            q = a->q1 + (size_t)im * a->N1;
            for (int i = 0; i < a->N1; ++i) q[i] = orc_mt_randint(r, 2) ? 1.f : -1.f;
        }
    }
}

void orc_bga_set_q(orc_bga *a, const int8_t *q0, const int8_t *q1) {
    for (size_t k = 0; k < (size_t)a->m * a->N0; ++k) a->q0[k] = q0[k];
    for (size_t k = 0; k < (size_t)a->m * a->N1; ++k) a->q1[k] = q1[k];
}

void orc_bga_get_q(const orc_bga *a, int8_t *q0, int8_t *q1) {
    for (size_t k = 0; k < (size_t)a->m * a->N0; ++k) q0[k] = (int8_t)a->q0[k];
    for (size_t k = 0; k < (size_t)a->m * a->N1; ++k) q1[k] = (int8_t)a->q1[k];
}

/* dEmat = qFixed * J^T for side 1 (J: N1 x N0, qFixed = q0) or qFixed * J for side 0 */
static void bga_fields(orc_bga *a, int side) {
    int N0 = a->N0, N1 = a->N1, m = a->m;
#pragma omp parallel for num_threads(a->nw) schedule(static)
    for (int y = 0; y < m; ++y) {
        if (side == 1) {
            const float *qf = a->q0 + (size_t)y * N0;
            for (int i = 0; i < N1; ++i) {
                const float *Ji = a->J + (size_t)i * N0;
                float s = 0.f;
                for (int j = 0; j < N0; ++j) s = fmaf(qf[j], Ji[j], s);
                a->dE[(size_t)y * N1 + i] = s;
            }
        } else {
            const float *qf = a->q1 + (size_t)y * N1;
            float *out = a->dE + (size_t)y * N0;
            for (int j = 0; j < N0; ++j) out[j] = 0.f;
            for (int i = 0; i < N1; ++i) {
                const float *Ji = a->J + (size_t)i * N0;
                float qi = qf[i];
                for (int j = 0; j < N0; ++j) out[j] = fmaf(qi, Ji[j], out[j]);
            }
        }
    }
}

/* tryFlip (row), CPUBipartiteGraphAnnealer.cpp:331-344 */
static void bga_flip_row(orc_bga *a, float *qA, const float *h, int N, int im, float twoDivM,
                         float beta, float coef, orc_mt *r) {
    int m = a->m;
    for (int iq = 0; iq < N; ++iq) {
        float q = qA[(size_t)im * N + iq];
        float dE = twoDivM * q * (h[iq] + a->dE[(size_t)im * N + iq]);
        int n0 = (im + m - 1) % m, n1 = (im + 1) % m;
        dE -= q * (qA[(size_t)n0 * N + iq] + qA[(size_t)n1 * N + iq]) * coef;
        float thresh = dE < 0.f ? 1.f : expf(-dE * beta);
        if (thresh > orc_mt_f32(r)) qA[(size_t)im * N + iq] = -q;
    }
}

/* tryFlipSA (row), CPUBipartiteGraphAnnealer.cpp:485-496 */
static void bga_flip_row_sa(orc_bga *a, float *qA, const float *h, int N, int im, float invKT,
                            orc_mt *r) {
    for (int iq = 0; iq < N; ++iq) {
        float q = qA[(size_t)im * N + iq];
        float dE = 2.f * q * (h[iq] + a->dE[(size_t)im * N + iq]);
        float thresh = dE < 0.f ? 1.f : expf(-dE * invKT);
        if (thresh > orc_mt_f32(r)) qA[(size_t)im * N + iq] = -q;
    }
}

static void bga_half_coloring(orc_bga *a, int side, float G, float beta) {
    int m = a->m;
    float twoDivM = 2.f / (float)m;
    float coef = logf(tanhf(G * beta / (float)m)) / beta;
    float *qA = side == 1 ? a->q1 : a->q0;
    const float *h = side == 1 ? a->h1 : a->h0;
    int N = side == 1 ? a->N1 : a->N0;
    bga_fields(a, side);
    if (a->nw == 1) {
        /* annealHalfStepColoring, :347-365 */
        for (int off = 0; off < 2; ++off)
            for (int im = off; im < m; im += 2)
                bga_flip_row(a, qA, h, N, im, twoDivM, beta, coef, &a->rng[0]);
        return;
    }
    /* annealHalfStepColoringParallel, :378-431 */
    int m2 = (m / 2) * 2;
#pragma omp parallel num_threads(a->nw)
    {
        orc_mt *r = &a->rng[omp_tid()];
#pragma omp for schedule(static)
        for (int im = 0; im < m2; im += 2)
            bga_flip_row(a, qA, h, N, im, twoDivM, beta, coef, r);
    }
    if (m % 2) bga_flip_row(a, qA, h, N, m - 1, twoDivM, beta, coef, &a->rng[0]);
#pragma omp parallel num_threads(a->nw)
    {
        orc_mt *r = &a->rng[omp_tid()];
#pragma omp for schedule(static)
        for (int im = 1; im < m2; im += 2)
            bga_flip_row(a, qA, h, N, im, twoDivM, beta, coef, r);
    }
}

static void bga_half_sa_coloring(orc_bga *a, int side, float invKT) {
    float *qA = side == 1 ? a->q1 : a->q0;
    const float *h = side == 1 ? a->h1 : a->h0;
    int N = side == 1 ? a->N1 : a->N0;
    bga_fields(a, side);
#pragma omp parallel num_threads(a->nw)
    {
        orc_mt *r = &a->rng[omp_tid()];
#pragma omp for schedule(static)
        for (int im = 0; im < a->m; ++im)
            bga_flip_row_sa(a, qA, h, N, im, invKT, r);
    }
}

static float bga_field_at(const orc_bga *a, int side, int y, int x) {
    float s = 0.f;
    if (side == 0) { /* column x of J dotted with q1[y] */
        for (int i = 0; i < a->N1; ++i)
            s = fmaf(a->J[(size_t)i * a->N0 + x], a->q1[(size_t)y * a->N1 + i], s);
    } else {
        for (int j = 0; j < a->N0; ++j)
            s = fmaf(a->J[(size_t)x * a->N0 + j], a->q0[(size_t)y * a->N0 + j], s);
    }
    return s;
}

void orc_bga_step(orc_bga *a, int algo, float G, float beta) {
    int N0 = a->N0, N1 = a->N1, m = a->m, N = N0 + N1;
    if (algo == ORC_ALGO_NAIVE) {
        /* annealOneStepNaive, :290-328 */
        float twoDivM = 2.f / (float)m;
        float coef = logf(tanhf(G * beta / (float)m)) / beta;
        orc_mt *r = &a->rng[0];
        for (long loop = 0; loop < (long)N * m; ++loop) {
            int x = (int)orc_mt_randint(r, N);
            int y = (int)orc_mt_randint(r, m);
            int side = x < N0 ? 0 : 1;
            if (side == 1) x -= N0;
            float *qA = side ? a->q1 : a->q0;
            int Ns = side ? N1 : N0;
            const float *h = side ? a->h1 : a->h0;
            float qyx = qA[(size_t)y * Ns + x];
            float sum = bga_field_at(a, side, y, x);
            float dE = twoDivM * qyx * (h[x] + sum);
            int n0 = (y == 0) ? m - 1 : y - 1, n1 = (y == m - 1) ? 0 : y + 1;
            dE -= qyx * (qA[(size_t)n0 * Ns + x] + qA[(size_t)n1 * Ns + x]) * coef;
            float thr = (dE < 0.f) ? 1.f : expf(-dE * beta);
            if (thr > orc_mt_f32(r)) qA[(size_t)y * Ns + x] = -qyx;
        }
    } else if (algo == ORC_ALGO_COLORING) {
        bga_half_coloring(a, 1, G, beta);
        bga_half_coloring(a, 0, G, beta);
    } else if (algo == ORC_ALGO_SA_NAIVE) {
        /* annealOneStepSANaive, :446-480 (N*m trials per trotter) */
        float invKT = 1.f / G;
        orc_mt *r = &a->rng[0];
        for (int y = 0; y < m; ++y)
            for (long loop = 0; loop < (long)N * m; ++loop) {
                int x = (int)orc_mt_randint(r, N);
                int side = x < N0 ? 0 : 1;
                if (side == 1) x -= N0;
                float *qA = side ? a->q1 : a->q0;
                int Ns = side ? N1 : N0;
                const float *h = side ? a->h1 : a->h0;
                float qyx = qA[(size_t)y * Ns + x];
                float sum = bga_field_at(a, side, y, x);
                float dE = 2.f * qyx * (h[x] + sum);
                float thr = (dE < 0.f) ? 1.f : expf(-dE * invKT);
                if (thr > orc_mt_f32(r)) qA[(size_t)y * Ns + x] = -qyx;
            }
    } else {
        /* annealOneStepSAColoring, :528-537 */
        float invKT = 1.f / G;
        bga_half_sa_coloring(a, 1, invKT);
        bga_half_sa_coloring(a, 0, invKT);
    }
}

void orc_bga_energy(const orc_bga *a, double *E) {
    int N0 = a->N0, N1 = a->N1;
    for (int y = 0; y < a->m; ++y) {
        const float *q0 = a->q0 + (size_t)y * N0, *q1 = a->q1 + (size_t)y * N1;
        double e = 0.;
        for (int j = 0; j < N0; ++j) e += (double)a->h0[j] * q0[j];
        for (int i = 0; i < N1; ++i) {
            e += (double)a->h1[i] * q1[i];
            double r = 0.;
            for (int j = 0; j < N0; ++j) r += (double)a->J[(size_t)i * N0 + j] * q0[j];
            e += q1[i] * r;
        }
        E[y] = -e - (double)a->c;
    }
}

/* ====================================== FP64 replay of the GPU sweeps ==== */
/*
 * The GPU build's algorithms (the device code documents the same rules):
 *
 *  dense coloring, one annealOneStep with step counter s:
 *    for k in [0, N): phase A = even y < 2*(m/2), phase B = {m-1} if m is odd,
 *    phase C = odd y; within a phase every trotter makes one trial:
 *      (w0..w3) = philox((k, y, s, TAG_DSWEEP)), x = hi(w0 * N), u = (w1 >> 8) 2^-24
 *      dE = (2/m) q_yx (h_x + 2 sum_j J_xj q_yj) - q_yx (q_{y-1,x} + q_{y+1,x}) coef
 *      coef = log(tanh(G beta / m)) / beta ; accept iff dE < 0 or exp(-beta dE) > u
 *    trace bit k*m + y = accepted.
 *  dense SA (sa_naive): per trotter y, for k in [0, N): philox((k, y, s, TAG_DSA)),
 *    dE = 2 q (h + 2 J.q), accept iff dE < 0 or exp(-dE / G) > u; bit k*m + y.
 *  dense naive: for t in [0, N m): philox((t, 0, s, TAG_DNAIVE)): y = hi(w0 m),
 *    x = hi(w1 N), u from w2; SQA rule; bit t.
 *  bipartite coloring: half-step on side 1 (fields q0 J^T) then side 0 (q1 J);
 *    phases as above, spin i of trotter y: u from philox((i, y, s, TAG_BSWEEP | side << 8)).w1;
 *    dE = (2/m) q (h + F) - q (q_{y-1} + q_{y+1}) coef.  trace: [m x N1 bits][m x N0 bits].
 *  bipartite SA coloring: same with TAG_BSA, one phase, dE = 2 q (h + F), exp(-dE / G).
 *  bipartite naive: t in [0, (N0+N1) m): x = hi(w0 (N0+N1)), y = hi(w1 m), u from w2.
 *  bipartite SA naive: per trotter y, t in [0, (N0+N1) m): x = hi(w0 (N0+N1)), u from w1;
 *    trace bit y (N0+N1) m + t.
 */

static int trace_bit(const uint32_t *trace, long long i) { return (trace[i >> 5] >> (i & 31)) & 1; }

typedef struct {
    double tol;
    orc_replay_stats *st;
} replay_ctx;

/* compares the FP64 decision with the device decision; returns the device decision */
static int replay_decide(replay_ctx *ctx, double dE, double rate, float u, int dev) {
    double p = dE < 0. ? 1. : exp(-dE * rate);
    int host = p > (double)u;
    double margin = fabs(ORC_MIN(p, 1.) - (double)u);
    orc_replay_stats *st = ctx->st;
    st->n_trials++;
    st->n_accept += dev;
    if (margin < ctx->tol) st->n_small_margin++;
    if (host != dev) {
        st->n_mismatch++;
        if (margin < ctx->tol) st->n_mismatch_small++;
        if (margin > st->max_mismatch_margin) st->max_mismatch_margin = margin;
    }
    return dev;
}

static double dg_field64(const float *J, int N, const int8_t *qy, int x) {
    double s = 0.;
    const float *Jx = J + (size_t)x * N;
    for (int j = 0; j < N; ++j) s += (double)Jx[j] * qy[j];
    return s;
}

void orc_gpu_randomize(uint64_t seed, uint32_t step, int tagSide, int m, int N, int8_t *q) {
    for (int y = 0; y < m; ++y)
        for (int chunk = 0; chunk * 128 < N; ++chunk) {
            uint32_t w[4];
            philox_draw(seed, (uint32_t)chunk, (uint32_t)y, step,
                        (uint32_t)ORC_TAG_RAND | ((uint32_t)tagSide << 8), w);
            for (int b = 0; b < 128 && chunk * 128 + b < N; ++b) {
                int bit = (w[b >> 5] >> (b & 31)) & 1;
                q[(size_t)y * N + chunk * 128 + b] = bit ? 1 : -1;
            }
        }
}

void orc_dg_replay(const float *h, const float *J, int N, int m, int algo,
                   uint64_t seed, uint32_t step, float G, float beta,
                   int8_t *q, const uint32_t *trace, double tol, orc_replay_stats *st) {
    replay_ctx ctx = {tol, st};
    double Gd = G, bd = beta;
    double twoDivM = 2. / m;
    double coef = log(tanh(Gd * bd / m)) / bd;
    if (algo == ORC_ALGO_COLORING || algo == ORC_ALGO_NAIVE) {
        long long nTrials = (long long)N * m;
        if (algo == ORC_ALGO_NAIVE) {
            for (long long t = 0; t < nTrials; ++t) {
                uint32_t w[4];
                philox_draw(seed, (uint32_t)t, 0u, step, ORC_TAG_DNAIVE, w);
                int y = mulhi_index(w[0], m), x = mulhi_index(w[1], N);
                float u = unit_float(w[2]);
                int8_t *qy = q + (size_t)y * N;
                double qyx = qy[x];
                int yl = (y + m - 1) % m, yr = (y + 1) % m;
                double dE = twoDivM * qyx * ((double)h[x] + 2. * dg_field64(J, N, qy, x)) -
                            qyx * (q[(size_t)yl * N + x] + q[(size_t)yr * N + x]) * coef;
                if (replay_decide(&ctx, dE, bd, u, trace_bit(trace, t))) qy[x] = (int8_t)-qy[x];
            }
            return;
        }
        int m2 = (m / 2) * 2;
        for (int k = 0; k < N; ++k) {
            for (int phase = 0; phase < 3; ++phase) {
                int yb, ye, ys;
                if (phase == 0) { yb = 0; ye = m2; ys = 2; }
                else if (phase == 1) { if (!(m % 2)) continue; yb = m - 1; ye = m; ys = 1; }
                else { yb = 1; ye = m2; ys = 2; }
                /* decisions of one phase are independent: evaluate, then apply */
                for (int y = yb; y < ye; y += ys) {
                    uint32_t w[4];
                    philox_draw(seed, (uint32_t)k, (uint32_t)y, step, ORC_TAG_DSWEEP, w);
                    int x = mulhi_index(w[0], N);
                    float u = unit_float(w[1]);
                    int8_t *qy = q + (size_t)y * N;
                    double qyx = qy[x];
                    int yl = (y + m - 1) % m, yr = (y + 1) % m;
                    double dE = twoDivM * qyx * ((double)h[x] + 2. * dg_field64(J, N, qy, x)) -
                                qyx * (q[(size_t)yl * N + x] + q[(size_t)yr * N + x]) * coef;
                    if (replay_decide(&ctx, dE, bd, u, trace_bit(trace, (long long)k * m + y)))
                        qy[x] = (int8_t)-qy[x];
                }
            }
        }
        return;
    }
    /* SA naive */
    double invKT = 1. / Gd;
    for (int y = 0; y < m; ++y) {
        int8_t *qy = q + (size_t)y * N;
        for (int k = 0; k < N; ++k) {
            uint32_t w[4];
            philox_draw(seed, (uint32_t)k, (uint32_t)y, step, ORC_TAG_DSA, w);
            int x = mulhi_index(w[0], N);
            float u = unit_float(w[1]);
            double qyx = qy[x];
            double dE = 2. * qyx * ((double)h[x] + 2. * dg_field64(J, N, qy, x));
            if (replay_decide(&ctx, dE, invKT, u, trace_bit(trace, (long long)k * m + y)))
                qy[x] = (int8_t)-qy[x];
        }
    }
}

/*
 * Same decisions as orc_dg_replay over nSteps consecutive annealOneSteps (step
 * counters step0 .. step0 + nSteps - 1, trace of step s at trace + s * words),
 * but with FP64 local fields kept resident: F[y][i] = sum_j J_ij q_yj is
 * computed once (threads over trotters) and every flip the device reports adds
 * -2 s J[x][:] to its trotter's row.  Each addend is an fp32 value, exact in
 * FP64, so the fields stay within a few FP64 ulps of the direct dot products;
 * the cost per step is N m trials plus N per accepted flip, which makes the
 * benchmark size (N = 4096, m = 256) replayable.  J must be symmetric with a
 * zero diagonal (the Ising J of the dense formulas).
 */
void orc_dg_replay_steps(const double *h, const double *J, int N, int m, int algo, uint64_t seed,
                         uint32_t step0, int nSteps, const float *G, const float *beta, int8_t *q,
                         const uint32_t *trace, double tol, orc_replay_stats *st) {
    replay_ctx ctx = {tol, st};
    double *F = (double *)malloc(sizeof(double) * (size_t)m * N);
    if (!F) return;
#pragma omp parallel
    {
        double *qd = (double *)malloc(sizeof(double) * (size_t)N);
#pragma omp for schedule(static)
        for (int y = 0; y < m; ++y) {
            const int8_t *qy = q + (size_t)y * N;
            for (int j = 0; j < N; ++j) qd[j] = qy[j];
            for (int i = 0; i < N; ++i) {
                const double *Ji = J + (size_t)i * N;
                double s = 0.;
                for (int j = 0; j < N; ++j) s += Ji[j] * qd[j];
                F[(size_t)y * N + i] = s;
            }
        }
        free(qd);
    }
    const size_t words = ((size_t)N * m + 31) / 32;
    for (int s = 0; s < nSteps; ++s) {
        const uint32_t *tr = trace + words * (size_t)s;
        const uint32_t step = step0 + (uint32_t)s;
        const double Gd = G[s], bd = beta[s];
        const double twoDivM = 2. / m;
        const double coef = log(tanh(Gd * bd / m)) / bd;
        const double invKT = 1. / Gd;
#define ORC_FLIP(Y, X)                                                   \
    do {                                                                 \
        int8_t *qy_ = q + (size_t)(Y) * N;                               \
        double d_ = -2. * qy_[(X)];                                      \
        double *Fy_ = F + (size_t)(Y) * N;                               \
        const double *Jx_ = J + (size_t)(X) * N;                         \
        for (int i_ = 0; i_ < N; ++i_) Fy_[i_] += d_ * Jx_[i_];         \
        qy_[(X)] = (int8_t)-qy_[(X)];                                    \
    } while (0)
        if (algo == ORC_ALGO_NAIVE) {
            const long long nTrials = (long long)N * m;
            for (long long t = 0; t < nTrials; ++t) {
                uint32_t w[4];
                philox_draw(seed, (uint32_t)t, 0u, step, ORC_TAG_DNAIVE, w);
                int y = mulhi_index(w[0], m), x = mulhi_index(w[1], N);
                float u = unit_float(w[2]);
                double qyx = q[(size_t)y * N + x];
                int yl = (y + m - 1) % m, yr = (y + 1) % m;
                double dE = twoDivM * qyx * ((double)h[x] + 2. * F[(size_t)y * N + x]) -
                            qyx * (q[(size_t)yl * N + x] + q[(size_t)yr * N + x]) * coef;
                if (replay_decide(&ctx, dE, bd, u, trace_bit(tr, t))) ORC_FLIP(y, x);
            }
        } else if (algo == ORC_ALGO_COLORING) {
            const int m2 = (m / 2) * 2;
            for (int k = 0; k < N; ++k)
                for (int phase = 0; phase < 3; ++phase) {
                    int yb, ye, ys;
                    if (phase == 0) { yb = 0; ye = m2; ys = 2; }
                    else if (phase == 1) { if (!(m % 2)) continue; yb = m - 1; ye = m; ys = 1; }
                    else { yb = 1; ye = m2; ys = 2; }
                    /* trotters of one phase are never ring neighbours: flipping at once is the same
                       as evaluating the phase first */
                    for (int y = yb; y < ye; y += ys) {
                        uint32_t w[4];
                        philox_draw(seed, (uint32_t)k, (uint32_t)y, step, ORC_TAG_DSWEEP, w);
                        int x = mulhi_index(w[0], N);
                        float u = unit_float(w[1]);
                        double qyx = q[(size_t)y * N + x];
                        int yl = (y + m - 1) % m, yr = (y + 1) % m;
                        double dE = twoDivM * qyx * ((double)h[x] + 2. * F[(size_t)y * N + x]) -
                                    qyx * (q[(size_t)yl * N + x] + q[(size_t)yr * N + x]) * coef;
                        if (replay_decide(&ctx, dE, bd, u, trace_bit(tr, (long long)k * m + y))) ORC_FLIP(y, x);
                    }
                }
        } else {
            for (int y = 0; y < m; ++y)
                for (int k = 0; k < N; ++k) {
                    uint32_t w[4];
                    philox_draw(seed, (uint32_t)k, (uint32_t)y, step, ORC_TAG_DSA, w);
                    int x = mulhi_index(w[0], N);
                    float u = unit_float(w[1]);
                    double qyx = q[(size_t)y * N + x];
                    double dE = 2. * qyx * ((double)h[x] + 2. * F[(size_t)y * N + x]);
                    if (replay_decide(&ctx, dE, invKT, u, trace_bit(tr, (long long)k * m + y))) ORC_FLIP(y, x);
                }
        }
#undef ORC_FLIP
    }
    free(F);
}

/* field on spin x of `side` in trotter y from the other side (FP64) */
static double bg_field64(const double *J, int N0, int N1, const int8_t *q0, const int8_t *q1,
                         int side, int y, int x) {
    double s = 0.;
    if (side == 1) {
        const double *Jx = J + (size_t)x * N0;
        const int8_t *qf = q0 + (size_t)y * N0;
        for (int j = 0; j < N0; ++j) s += Jx[j] * qf[j];
    } else {
        const int8_t *qf = q1 + (size_t)y * N1;
        for (int i = 0; i < N1; ++i) s += J[(size_t)i * N0 + x] * qf[i];
    }
    return s;
}

void orc_bg_replay(const double *h0, const double *h1, const double *J, int N0, int N1, int m,
                   int algo, uint64_t seed, uint32_t step, float G, float beta,
                   int8_t *q0, int8_t *q1, const uint32_t *trace, double tol,
                   orc_replay_stats *st) {
    replay_ctx ctx = {tol, st};
    double Gd = G, bd = beta;
    double twoDivM = 2. / m;
    double coef = log(tanh(Gd * bd / m)) / bd;
    double invKT = 1. / Gd;
    int Ntot = N0 + N1;
    if (algo == ORC_ALGO_NAIVE || algo == ORC_ALGO_SA_NAIVE) {
        int sa = algo == ORC_ALGO_SA_NAIVE;
        int ny = sa ? m : 1;
        long long perY = (long long)Ntot * m;
        for (int yy = 0; yy < ny; ++yy)
            for (long long t = 0; t < perY; ++t) {
                uint32_t w[4];
                philox_draw(seed, (uint32_t)t, sa ? (uint32_t)yy : 0u, step,
                            sa ? ORC_TAG_BSANAIVE : ORC_TAG_BNAIVE, w);
                int x = mulhi_index(w[0], Ntot);
                int y = sa ? yy : mulhi_index(w[1], m);
                float u = unit_float(sa ? w[1] : w[2]);
                int side = x < N0 ? 0 : 1;
                if (side) x -= N0;
                int Ns = side ? N1 : N0;
                int8_t *qA = side ? q1 : q0;
                const double *h = side ? h1 : h0;
                double qyx = qA[(size_t)y * Ns + x];
                double F = bg_field64(J, N0, N1, q0, q1, side, y, x);
                double dE;
                if (sa) {
                    dE = 2. * qyx * ((double)h[x] + F);
                } else {
                    int yl = (y + m - 1) % m, yr = (y + 1) % m;
                    dE = twoDivM * qyx * ((double)h[x] + F) -
                         qyx * (qA[(size_t)yl * Ns + x] + qA[(size_t)yr * Ns + x]) * coef;
                }
                long long bit = sa ? (long long)yy * perY + t : t;
                if (replay_decide(&ctx, dE, sa ? invKT : bd, u, trace_bit(trace, bit)))
                    qA[(size_t)y * Ns + x] = (int8_t)-qA[(size_t)y * Ns + x];
            }
        return;
    }
    int sa = algo == ORC_ALGO_SA_COLORING;
    long long bitBase = 0;
    double *F = (double *)malloc(sizeof(double) * (size_t)m * ORC_MAX(N0, N1));
    for (int hs = 0; hs < 2; ++hs) {
        int side = hs == 0 ? 1 : 0;
        int Ns = side ? N1 : N0;
        int8_t *qA = side ? q1 : q0;
        const double *h = side ? h1 : h0;
        for (int y = 0; y < m; ++y)
            for (int i = 0; i < Ns; ++i)
                F[(size_t)y * Ns + i] = bg_field64(J, N0, N1, q0, q1, side, y, i);
        int m2 = (m / 2) * 2;
        for (int phase = 0; phase < 3; ++phase) {
            int yb, ye, ys;
            if (sa) { if (phase) break; yb = 0; ye = m; ys = 1; }
            else if (phase == 0) { yb = 0; ye = m2; ys = 2; }
            else if (phase == 1) { if (!(m % 2)) continue; yb = m - 1; ye = m; ys = 1; }
            else { yb = 1; ye = m2; ys = 2; }
            for (int y = yb; y < ye; y += ys)
                for (int i = 0; i < Ns; ++i) {
                    uint32_t w[4];
                    philox_draw(seed, (uint32_t)i, (uint32_t)y, step,
                                (uint32_t)(sa ? ORC_TAG_BSA : ORC_TAG_BSWEEP) | ((uint32_t)side << 8), w);
                    float u = unit_float(w[1]);
                    double qyx = qA[(size_t)y * Ns + i];
                    double dE;
                    if (sa) {
                        dE = 2. * qyx * ((double)h[i] + F[(size_t)y * Ns + i]);
                    } else {
                        int yl = (y + m - 1) % m, yr = (y + 1) % m;
                        dE = twoDivM * qyx * ((double)h[i] + F[(size_t)y * Ns + i]) -
                             qyx * (qA[(size_t)yl * Ns + i] + qA[(size_t)yr * Ns + i]) * coef;
                    }
                    long long bit = bitBase + (long long)y * Ns + i;
                    if (replay_decide(&ctx, dE, sa ? invKT : bd, u, trace_bit(trace, bit)))
                        qA[(size_t)y * Ns + i] = (int8_t)-qA[(size_t)y * Ns + i];
                }
        }
        bitBase += (long long)m * Ns;
    }
    free(F);
}

/* ========================== exact integer BF in Gray-code order (checker) ==== */
typedef struct {
    int64_t best;
    uint64_t *list;
    long long n, cap;
    int overflow;
} gray_worker;

int orc_dg_bf_search_exact_int(const float *W, int N, int om, int cap, int nWorkers,
                               double *Emin, uint64_t *xout, long long *nMin) {
    if (N < 1 || N > 40) return -2;
    int32_t *Wz = (int32_t *)malloc(sizeof(int32_t) * (size_t)N * N);
    int32_t *diag = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
    double tot = 0.;
    int bad = 0;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
            double w = om == 1 ? -(double)W[(size_t)i * N + j] : (double)W[(size_t)i * N + j];
            if (w != floor(w) || W[(size_t)i * N + j] != W[(size_t)j * N + i]) bad = 1;
            tot += fabs(w);
            Wz[(size_t)i * N + j] = i == j ? 0 : (int32_t)w;
            if (i == j) diag[i] = (int32_t)w;
        }
    if (bad || tot >= 1073741824.) {
        free(Wz);
        free(diag);
        return -3;
    }
    const int nw = omp_workers(nWorkers);
    const uint64_t total = 1ull << N;
    gray_worker *ws = (gray_worker *)calloc(nw, sizeof(gray_worker));
#pragma omp parallel num_threads(nw)
    {
        const int t = omp_tid();
        gray_worker *me = &ws[t];
        me->cap = 1 << 16;
        me->list = (uint64_t *)malloc(sizeof(uint64_t) * me->cap);
        const uint64_t n0 = total / nw * t + ORC_MIN((uint64_t)t, total % nw);
        const uint64_t n1 = n0 + total / nw + ((uint64_t)t < total % nw ? 1 : 0);
        if (n0 < n1) {
            int32_t g[64];  /* g_k = sum_{j != k} W_kj x_j; packed bit b is variable N-1-b */
            uint64_t v = n0 ^ (n0 >> 1);
            int64_t E = 0;
            for (int k = 0; k < N; ++k) {
                int32_t s = 0;
                for (int j = 0; j < N; ++j) s += Wz[(size_t)k * N + j] * (int32_t)((v >> (N - 1 - j)) & 1);
                g[k] = s;
                if ((v >> (N - 1 - k)) & 1) E += diag[k] + s;
            }
            me->best = E;
            me->list[me->n++] = v;
            for (uint64_t n = n0 + 1; n < n1; ++n) {
                const int b = __builtin_ctzll(n);
                const int k = N - 1 - b;
                const int xk = (int)((v >> b) & 1);
                const int32_t d = diag[k] + 2 * g[k];
                E += xk ? -(int64_t)d : (int64_t)d;
                const int32_t sgn = xk ? -1 : 1;
                const int32_t *Wk = Wz + (size_t)k * N;
                for (int j = 0; j < N; ++j) g[j] += sgn * Wk[j];
                v ^= 1ull << b;
                if (E <= me->best) {
                    if (E < me->best) {
                        me->best = E;
                        me->n = 0;
                        me->overflow = 0;
                    }
                    if (me->n < me->cap) me->list[me->n++] = v;
                    else me->overflow = 1;
                }
            }
        } else {
            me->best = INT64_MAX;
        }
    }
    int64_t best = INT64_MAX;
    for (int t = 0; t < nw; ++t) best = ORC_MIN(best, ws[t].best);
    long long count = 0;
    int overflow = 0;
    for (int t = 0; t < nw; ++t)
        if (ws[t].best == best) {
            count += ws[t].n;
            overflow |= ws[t].overflow;
        }
    uint64_t *all = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)ORC_MAX(count, 1));
    long long k = 0;
    for (int t = 0; t < nw; ++t)
        if (ws[t].best == best) {
            memcpy(all + k, ws[t].list, sizeof(uint64_t) * ws[t].n);
            k += ws[t].n;
        }
    qsort(all, (size_t)count, sizeof(uint64_t), cmp_u64);
    int nout = (int)ORC_MIN((long long)cap, count);
    memcpy(xout, all, sizeof(uint64_t) * nout);
    *Emin = om == 1 ? -(double)best : (double)best;
    *nMin = count;
    for (int t = 0; t < nw; ++t) free(ws[t].list);
    free(ws);
    free(all);
    free(Wz);
    free(diag);
    return overflow ? -4 : nout;
}
