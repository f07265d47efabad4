// dense_multi.cu -- one CTA per trotter: the dense coloring / SA sweep of one
// large instance across the whole GPU (cooperative launch, all CTAs resident).
//
// It runs the same trials, in the same colour order and with the same fp32
// arithmetic, as the one-CTA-per-instance kernel in dense.cu, so both give
// bit-identical spins and fields.
//
// Per CTA (trotter y), 256 threads:
//   warp 0  decider: the trotter's trials in batches of 32 iterations, lane i =
//           iteration g0 + i.  A batch is decided in rounds: every undecided
//           lane evaluates its trial with its current field and neighbour
//           spins; the lowest accepting lane is final (all undecided lanes
//           below it reject), and the lanes above it add d * J[x_f][x_i] to
//           their fields and flip their spin copy when they share its site.
//           A batch takes (accepted flips + 1) rounds instead of 32 sequential
//           trials.  The batch's fields start from the resident row F[y][:],
//           which the updaters keep one batch behind, plus the previous
//           batch's flips d_f * J[x_f][x_i], gathered at the batch boundary and
//           added after the next batch's ghost-row update.
//           Decisions are published as one 64-bit word per batch (accept
//           bits, decided count, batch tag) with a single relaxed store after
//           every accepting round and at the end of the batch: a reader that
//           sees the tag of the batch it wants sees consistent bits, so no
//           fence is needed.
//   warp 1  helper: polls the two neighbours' accept words (both neighbours,
//           two words ahead, in one round trip) and copies them into shared
//           memory.
//   warps 2-3 prefetchers, alternate batches: this trotter's own sites,
//           uniforms and step constants, the in-batch gathers J[x_j][x_i]
//           (j < i) for the lanes j predicted to accept, the neighbours' sites of the same iterations (a ring of
//           sites and one hashed-site bitmap per batch), and per lane the
//           neighbour iterations of this and the previous batch that hit its
//           site, into a ring of kPre batch buffers with a ready tag each.
//   warps 4-6 updaters: F[y][:] += d * J[x][:] for the flips of the previous
//           batch, in trial order, while the decider works on the next one.
//   warp 7  exact decisions: a trial whose fp32 outcome the rounding of the
//           resident field could change is decided in FP64 from its exact field
//           (sq_common.cuh); the warp sleeps on a named barrier between requests
//           and answers through a shared word the decider waits on (bounded).
// Colour order: trial (y, k) must see neighbour n after every neighbour trial
// that precedes it (iteration < k, or = k when n's colour phase comes first:
// even trotters, then trotter m-1 if m is odd, then odd trotters).  The
// decider applies neighbour flips to a ghost bit row of n only up to the
// first trial of its current batch; each lane's bit is corrected for the
// neighbour trials between that point and the lane's own limit, which the
// prefetched lists show to be none for almost every lane.  A lane waits only when such
// a neighbour trial is not yet published.  Every wait is bounded (global
// timer) and ends the kernel with a timeout status instead of hanging; before
// waiting a CTA publishes the trials it has decided, so waits always point to
// strictly earlier trials and cannot form a cycle.
#include <cooperative_groups.h>

#include <algorithm>
#include <array>
#include <mutex>

// the exact warp's helpers inlined: measured 1.8 % faster at N=4096 m=256
#define SQ103_EXACT_ATTR __forceinline__
#include "sq_common.cuh"
#include "sq_kernels.h"

namespace sq103 {

constexpr int kMcThreads = 256;
constexpr int kPf = 2;                            // prefetcher warps (2 .. 1 + kPf)
constexpr int kUpdWarp0 = 2 + kPf;                // first updater warp
constexpr int kExactWarp = kMcThreads / 32 - 1;   // the last warp: exact decisions
constexpr int kMcUpdaters = kMcThreads - 32 * kUpdWarp0 - 32;
constexpr int kBarCount = 32 + kMcUpdaters;       // decider + updaters (barriers 1, 2)
constexpr int kBarExReq = 3;                      // wakes the exact warp (decider + exact warp, 64 threads)
constexpr int kRing = 256;      // neighbour sites kept per neighbour (power of two)
constexpr int kLogWords = 32;   // neighbour accept words kept per neighbour (power of two)
constexpr int kBmBits = 2048;   // bits of a batch's neighbour-site bitmap (hashed sites, power of two)
constexpr int kBmWords = kBmBits / 32;
constexpr int kBmSlots = kRing / 32;  // bitmaps kept per neighbour (one per ring batch)
constexpr int kPre = 4;         // prefetched batches (power of two)
constexpr int kJgStride = 32 * 33;
constexpr int kGv = 8;          // flips of a batch whose gathers are deferred to the next batch
constexpr int kCand = 2;        // neighbour iterations per lane and batch found by the prefetchers
constexpr int kPredRows = 8;    // predicted accepting lanes whose gathers are kept in registers
constexpr float kFieldDrift = 1.f;  // assumed field change between prefetch and decision
constexpr unsigned long long kWaitLimitNs = 4000000000ull;
constexpr unsigned long long kShortWaitNs = 1000000ull;  // task flag kFlagShortWaits (tests)
// the prefetchers run ahead and mostly wait: they poll gently, which leaves the
// SM's shared load/store path to the decider
constexpr int kPrefetchSleepNs = 128;
constexpr unsigned FULL = 0xffffffffu;
constexpr int kSmallN = 1024;  // rows up to this many spins take the kSmall instance (measured: 1024 faster, 2048 slower)

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void bar_sync(int id, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_arrive(int id, int n) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ unsigned smem_addr(const volatile void *p) {
    return (unsigned)__cvta_generic_to_shared((const void *)p);
}
__device__ __forceinline__ int ld_acquire_cta(const volatile int *p) {
    int v;
    asm volatile("ld.acquire.cta.shared.b32 %0, [%1];" : "=r"(v) : "r"(smem_addr(p)) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_acquire_cta64(const volatile unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.cta.shared.b64 %0, [%1];" : "=l"(v) : "r"(smem_addr(p)) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_cta(volatile int *p, int v) {
    asm volatile("st.release.cta.shared.b32 [%0], %1;" ::"r"(smem_addr(p)), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release_cta64(volatile unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.cta.shared.b64 [%0], %1;" ::"r"(smem_addr(p)), "l"(v) : "memory");
}

// accept word of batch b: bits 0-31 accept bits, 32-37 decided count, 38-63 b + 1
__device__ __forceinline__ unsigned long long log_word(int b, int cnt, unsigned bits) {
    return ((unsigned long long)(b + 1) << 38) | ((unsigned long long)cnt << 32) | bits;
}

__host__ __device__ __forceinline__ int colour_phase(int y, int m) {
    if ((m & 1) && y == m - 1) return 1;
    return (y & 1) ? 2 : 0;
}

struct McShared {
    volatile unsigned long long logAvail;  // neighbour accept bits known below (lo: neighbour 0, hi: 1) (helper)
    volatile int applied[2];               // neighbour iterations applied to the ghost rows (decider)
    volatile int readyTag[kPre];           // p + 1 once buffer p % kPre holds batch p (prefetchers)
    volatile int decDone;                  // batches [0, decDone) no longer read from the buffers (decider)
    volatile int done;
    int nflip;
    // exact decisions (rare): the decider posts a trial, the exact warp answers
    int exX, exBits;       // the trial's site; its FP64 outcomes for qL + qR = -2, 0, +2 (bits 0-2)
    volatile int exDone;   // number of the latest answer (exact warp; the decider counts its requests)
    float exQ, exU, exG, exBeta;
};

// every lane loads the flag with acquire semantics (one broadcast access); the
// value of lane 0 keeps control flow uniform
__device__ __forceinline__ int uniform_acquire(const volatile int *p) { return __shfl_sync(FULL, ld_acquire_cta(p), 0); }
__device__ __forceinline__ unsigned long long uniform_acquire64(const volatile unsigned long long *p) {
    return __shfl_sync(FULL, ld_acquire_cta64(p), 0);
}
__device__ __forceinline__ int avail_of(unsigned long long v, int n) { return (int)(n ? v >> 32 : v & 0xffffffffu); }

// bounded wait on a warp-uniform condition; false on timeout
template <int SLEEP_NS = 32, class F>
__device__ __forceinline__ bool wait_until(unsigned long long limitNs, F &&ready) {
    unsigned long long t0 = 0;
    while (!ready()) {
        if (t0 == 0) t0 = global_ns();
        if (global_ns() - t0 > limitNs) return false;
        __nanosleep(SLEEP_NS);
    }
    return true;
}

// Warp-wide.  The spin bit of a neighbour at the lane's site x after its
// iteration Ji, from `bit` (its value after every published iteration below
// j0) and the iterations j in [j0, Ji] that hit x: published ones (j < avail)
// flip it when accepted; need returns the latest unpublished one (-1: none).
// The batch bitmaps flag the lanes whose hashed site an iteration of that
// batch hit; one ballot per flagged lane over the batch's sites finds them.
// j0 and pLast (the batch of the latest Ji) are warp-uniform; only `active`
// lanes take part.
__device__ __forceinline__ void window_bits(int x, int Ji, int j0, int pLast, int avail, bool active,
                                            const uint32_t *bmn, const int *rg, const uint32_t *nl, int Itot,
                                            int &bit, int &need) {
    const int lane = threadIdx.x & 31;
    const int hb = x & (kBmBits - 1);
    need = -1;
    for (int p = j0 >> 5; p <= pLast; ++p) {
        const int jlo = max(j0, 32 * p);
        const bool hit = active && Ji >= jlo && ((bmn[(p & (kBmSlots - 1)) * kBmWords + (hb >> 5)] >> (hb & 31)) & 1u);
        unsigned hits = __ballot_sync(FULL, hit);
        if (!hits) continue;
        const int jl = 32 * p + lane;
        const int sj = jl < Itot ? rg[jl & (kRing - 1)] : -1;
        const uint32_t accw = nl[p & (kLogWords - 1)];  // accept bits, valid below avail
        while (hits) {
            const int i = __ffs(hits) - 1;
            hits &= hits - 1u;
            const int xi = __shfl_sync(FULL, x, i), Jii = __shfl_sync(FULL, Ji, i);
            const unsigned mt = __ballot_sync(FULL, sj == xi && jl >= jlo && jl <= Jii);
            if (lane == i) {
                for (unsigned r = mt; r; r &= r - 1u) {
                    const int j = 32 * p + __ffs(r) - 1;
                    if (j < avail)
                        bit ^= (accw >> (j & 31)) & 1u;
                    else
                        need = j;
                }
            }
        }
    }
}

// Up to kMaxPack independent instances in one cooperative launch: CTAs
// [base[i], base[i+1]) are the trotters of task t[i], whose accept words live in
// outLog[i] (nWords[i] per trotter).  Instances do not interact (the prologue's
// grid sync is the only common step), so each runs exactly as alone.
constexpr int kMaxPack = 16;
struct McPack {
    sq103_dense_task t[kMaxPack];
    unsigned long long *outLog[kMaxPack];
    int nWords[kMaxPack];
    int base[kMaxPack + 1];
    int n;
};

// kHooks: the test hooks of the task flags are compiled in (short waits, a
// trotter that withholds its accept words); the production instance has none.
// kSmall: rows of at most kSmallN spins, where the neighbours' sites hit a lane's
// site often: each prefetcher finds a lane's neighbour candidates from a table
// of the positions at each site of batches p - 2 .. p (one per batch and
// neighbour, in shared memory, cleared after use), with the sites of p - 1 and
// p - 2 drawn again from the neighbours' Philox streams, instead of a ballot per
// hit over the hashed-site bitmaps of the other prefetcher's batches (which
// makes the prefetchers wait for each other).  Both give the same candidates.
template <bool kHooks, bool kSmall>
__global__ void __launch_bounds__(kMcThreads, 2) dense_sweep_multi(const McPack P) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ McShared S;
    __shared__ sq103_dense_task task;
    __shared__ unsigned long long *sLog;
    __shared__ int sWords, sBase;
    if (threadIdx.x == 0) {
        int ti = 0;
#pragma unroll
        for (int i = 1; i < kMaxPack; ++i)
            if (i < P.n && (int)blockIdx.x >= P.base[i]) ti = i;
        // constant indices only (a runtime index into the parameters would copy them all)
        switch (ti) {
#define SQ103_PICK(i)            \
    case i:                      \
        task = P.t[i];           \
        sLog = P.outLog[i];      \
        sWords = P.nWords[i];    \
        sBase = P.base[i];       \
        break;
            SQ103_PICK(0) SQ103_PICK(1) SQ103_PICK(2) SQ103_PICK(3)
            SQ103_PICK(4) SQ103_PICK(5) SQ103_PICK(6) SQ103_PICK(7)
            SQ103_PICK(8) SQ103_PICK(9) SQ103_PICK(10) SQ103_PICK(11)
            SQ103_PICK(12) SQ103_PICK(13) SQ103_PICK(14) SQ103_PICK(15)
#undef SQ103_PICK
        }
    }
    __syncthreads();
    static_assert(kMaxPack == 16, "one case per pack entry");
    const sq103_dense_task &T = task;
    unsigned long long *const outLog = sLog;
    const int nWords = sWords;
    const int y = (int)blockIdx.x - sBase, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = T.N, m = T.m;
    const bool sa = T.algo == kSANaive;
    const int nNbr = sa ? 0 : (m == 2 ? 1 : 2);
    const int nbr0 = (y + m - 1) % m, nbr1 = (y + 1) % m;
    const int myPh = colour_phase(y, m);
    const int before0 = colour_phase(nbr0, m) < myPh ? 1 : 0;
    const int before1 = colour_phase(nbr1, m) < myPh ? 1 : 0;
    const int Itot = T.nSteps * N;
    const int nBatches = (Itot + 31) / 32;
    const int nWG = (N + 31) / 32;
    const int ghostStride = (nWG + 1) & ~1;
    const uint32_t tag = sa ? kTagDenseSA : kTagDenseSweep;
    // test hooks (task flags): every wait gives up after 1 ms; trotter 0 never
    // publishes its accept words, so its neighbours' waits run out
    const unsigned long long waitNs = (kHooks && (T.flags & kFlagShortWaits)) ? kShortWaitNs : kWaitLimitNs;
    const bool publish = !(kHooks && (T.flags & kFlagWithholdTrotter0) && y == 0);

    float *Fs = reinterpret_cast<float *>(smem);                        // N
    float *hs = Fs + N;                                                 // N
    float *Jg = hs + N;                                                 // kPre x 32 x 33
    float *preU = Jg + kPre * kJgStride;                                // kPre x 32
    float *preC = preU + kPre * 32;                                     // kPre x 3 x 32
    float *preL = preC + kPre * 96;                                     // kPre x 32: -ln u
    int *preX = reinterpret_cast<int *>(preL + kPre * 32);              // kPre x 32
    uint32_t *ghost = reinterpret_cast<uint32_t *>(preX + kPre * 32);   // 2 x ghostStride
    uint32_t *bm = ghost + 2 * ghostStride;                             // 2 x kBmSlots x kBmWords
    int *ring = reinterpret_cast<int *>(bm + 2 * kBmSlots * kBmWords);  // 2 x kRing
    uint32_t *nlog = reinterpret_cast<uint32_t *>(ring + 2 * kRing);    // 2 x kLogWords
    int *cand = reinterpret_cast<int *>(nlog + 2 * kLogWords);          // kPre x 2 x kCand x 32
    unsigned *prePred = reinterpret_cast<unsigned *>(cand + kPre * 2 * kCand * 32);  // kPre
    int2 *flips = reinterpret_cast<int2 *>(prePred + kPre);             // 32
    int8_t *qs = reinterpret_cast<int8_t *>(flips + 32);                // N
    // kSmall: one site table of kSmallN words per prefetcher (positions of a batch by site)
    uint32_t *siteTab = reinterpret_cast<uint32_t *>(qs + ((N + 15) & ~15));

    if (kSmall)
        for (int i = tid; i < kPf * kSmallN; i += kMcThreads) siteTab[i] = 0u;
    for (int i = tid; i < N; i += kMcThreads) {
        Fs[i] = T.F[(size_t)y * N + i];
        hs[i] = T.h[i];
        qs[i] = T.q[(size_t)y * N + i];
    }
    for (int n = 0; n < nNbr; ++n) {
        const int8_t *qn = T.q + (size_t)(n ? nbr1 : nbr0) * N;
        for (int w = tid; w < nWG; w += kMcThreads) {
            uint32_t bits = 0;
            for (int b = 0; b < 32 && w * 32 + b < N; ++b) bits |= (qn[w * 32 + b] > 0 ? 1u : 0u) << b;
            ghost[n * ghostStride + w] = bits;
        }
    }
    if (tid == 0) {
        S.logAvail = 0;
        S.applied[0] = S.applied[1] = 0;
        for (int i = 0; i < kPre; ++i) S.readyTag[i] = 0;
        S.decDone = 0;
        S.exDone = 0;
        S.done = 0;
        S.nflip = 0;
    }
    // every CTA has read its neighbours' rows before any CTA can finish and
    // write its own row back
    cooperative_groups::this_grid().sync();

    if (warp == 0) {
        // ------------------------------------------------------------ decider
        const uint32_t wordsPerStep = (uint32_t)(((size_t)N * m + 31) / 32);
        unsigned long long accepted = 0;
        bool aborted = false;
        int nfPrev = 0;      // flips of the previous batch still to be added to Fv
        int qb0 = 0, qb1 = 0, nd0 = -1, nd1 = -1;  // neighbour bits of the lane's site, unknown iterations
        int x = 0;                                  // the lane's site in the current batch
        float gv[kGv];       // their gathers J[x_f][x] (at this batch's sites)
#pragma unroll
        for (int t = 0; t < kGv; ++t) gv[t] = 0.f;

        int A0 = 0, A1 = 0;  // neighbour iterations applied to the ghost rows
        int exSeq = 0;       // exact-decision requests posted

        // Applies the published neighbour iterations below lim0 / lim1 (their sites
        // are in the ring) to the ghost rows; returns the helper's availability word.
        auto apply_nbr = [&](int lim0, int lim1) {
            const unsigned long long av = uniform_acquire64(&S.logAvail);
            lim0 = min(avail_of(av, 0), lim0);
            lim1 = nNbr > 1 ? min(avail_of(av, 1), lim1) : 0;
            const int span = max(lim0 - A0, lim1 - A1);
            for (int j0 = 0; j0 < span; j0 += 32) {
#pragma unroll
                for (int n = 0; n < 2; ++n) {
                    const int j = (n ? A1 : A0) + j0 + lane;
                    if (n < nNbr && j < (n ? lim1 : lim0) &&
                        ((nlog[n * kLogWords + ((j >> 5) & (kLogWords - 1))] >> (j & 31)) & 1u)) {
                        const int site = ring[n * kRing + (j & (kRing - 1))];
                        atomicXor(&ghost[n * ghostStride + (site >> 5)], 1u << (site & 31));
                    }
                }
            }
            if (span > 0) {
                A0 = max(A0, lim0);
                if (nNbr > 1) A1 = max(A1, lim1);
                __syncwarp();
                if (lane == 0) {
                    S.applied[0] = A0;
                    S.applied[1] = A1;
                }
            }
            return av;
        };

        // Neighbour bits at the lane's site for batch b: the ghost row (iterations
        // < A applied) corrected by the neighbour iterations in [A, Ji] at the site,
        // which the prefetchers listed (the latest kCand of the last three batches).
        // A neighbour more than two batches behind, or a longer list, takes the
        // bitmap scan of window_bits.  need: latest unpublished such iteration (-1: none).
        auto nbr_bits = [&](int b, int g0, bool valid, unsigned long long av) {
            const int buf = b & (kPre - 1);
            bool slow = false;
#pragma unroll
            for (int n = 0; n < 2; ++n) {
                if (n >= nNbr) break;
                const int A = n ? A1 : A0, avail = avail_of(av, n);
                int bit = (ghost[n * ghostStride + (x >> 5)] >> (x & 31)) & 1, need = -1;
                const int ca = cand[((buf * 2 + n) * kCand) * 32 + lane];
                const int cb = cand[((buf * 2 + n) * kCand + 1) * 32 + lane];
                slow |= ca == -2 || A < 32 * (b - 2);
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const int j = c ? cb : ca;
                    if (j >= A) {
                        if (j < avail)
                            bit ^= (nlog[n * kLogWords + ((j >> 5) & (kLogWords - 1))] >> (j & 31)) & 1u;
                        else
                            need = max(need, j);
                    }
                }
                if (n) {
                    qb1 = bit;
                    nd1 = valid ? need : -1;
                } else {
                    qb0 = bit;
                    nd0 = valid ? need : -1;
                }
            }
            slow = slow && valid;
            if (__any_sync(FULL, slow)) {
#pragma unroll
                for (int n = 0; n < 2; ++n) {
                    if (n >= nNbr) break;
                    int bit = (ghost[n * ghostStride + (x >> 5)] >> (x & 31)) & 1, need;
                    window_bits(x, g0 + lane - 1 + (n ? before1 : before0), n ? A1 : A0, b, avail_of(av, n), slow,
                                bm + n * kBmSlots * kBmWords, ring + n * kRing, nlog + n * kLogWords, Itot, bit, need);
                    if (slow) {
                        if (n) {
                            qb1 = bit;
                            nd1 = need;
                        } else {
                            qb0 = bit;
                            nd0 = need;
                        }
                    }
                }
            }
        };

        aborted = !wait_until(waitNs, [&] { return uniform_acquire(&S.readyTag[0]) == 1; });
        x = preX[lane];
        float Fv = Fs[x];

        for (int b = 0; b < nBatches && !aborted; ++b) {
            const int g0 = b * 32;
            const int buf = b & (kPre - 1);
            const int nValid = min(32, Itot - g0);
            const bool valid = lane < nValid;
            const float u = preU[buf * 32 + lane], Lu = preL[buf * 32 + lane];
            const StepConst sc = {preC[buf * 96 + lane], preC[buf * 96 + 32 + lane], preC[buf * 96 + 64 + lane]};
            const float *jg = Jg + buf * kJgStride + lane * 33;
            const unsigned pred = prePred[buf];  // lanes whose row of in-batch gathers is in jg
            const float hx = valid ? hs[x] : 0.f;
            float qx = valid ? (float)qs[x] : 1.f;

            // neighbour spins at this batch's sites: apply the published neighbour
            // iterations before this batch's first trial (their sites are in the ring
            // since this batch's buffer is ready); each lane's site is corrected at the
            // top of the first round
            qb0 = qb1 = 0;
            nd0 = nd1 = -1;
            unsigned blocked = 0;
            unsigned long long avEval = 0;  // availability the lanes' neighbour bits are evaluated with
            if (nNbr > 0) avEval = apply_nbr(g0 + before0, g0 + before1);

            // the previous batch's flips (gathered at the end of that batch)
#pragma unroll
            for (int t = 0; t < kGv; ++t) {
                if (t >= nfPrev) break;
                Fv = __fmaf_rn(__int_as_float(flips[t].y), gv[t], Fv);
            }

            // decide the batch in rounds
            unsigned pending = __ballot_sync(FULL, valid), accBits = 0;
            float d = 0.f;
            bool exValid = false;  // exBits holds the FP64 outcomes of the lane's trial
            int exBits = 0;
            const DecisionTol tolD = decision_tol(sa, true, sc.twoDivM, sc.coef, sc.rate);
            float xt = trial_xtol(tolD, hx, __fmul_rn(2.f, Fv), Lu);  // updated when Fv changes
            bool evalNbr = nNbr > 0;  // (one instance of nbr_bits keeps the loop's code small)
            while (pending) {
                if (evalNbr) {
                    nbr_bits(b, g0, valid, avEval);
                    blocked = __ballot_sync(FULL, nd0 >= 0 || nd1 >= 0) & pending;
                    evalNbr = false;
                }
                // a lane with unknown neighbour bits is decided anyway when every value
                // those bits can take gives the same outcome; it blocks otherwise.  The
                // outcomes come from the fp32 field, or from the FP64 outcomes of a
                // flagged lane's trial; a flagged lane (one whose fp32 outcome the field's
                // rounding could change) blocks too, until it has its FP64 outcomes
                int acc = 0, amb = 0, nearT = 0;
                if ((pending >> lane) & 1u) {
                    const float qn0 = qb0 ? 1.f : -1.f, qn1 = nNbr == 1 ? qn0 : (qb1 ? 1.f : -1.f);
                    auto accept = [&](float a, float c) -> int {
                        if (exValid) return (exBits >> (((int)a + (int)c + 2) >> 1)) & 1;
                        const float dE = sa ? dense_sa_dE(qx, hx, Fv)
                                            : dense_sqa_dE(qx, hx, Fv, a, c, sc.twoDivM, sc.coef);
                        return metropolis_log(dE, sc.rate, Lu, xt, nearT);
                    };
                    acc = accept(qn0, qn1);
                    if ((blocked >> lane) & 1u) {
                        const bool u0 = nd0 >= 0, u1 = nNbr > 1 && nd1 >= 0;
                        if (u0 && accept(-qn0, nNbr == 1 ? -qn0 : qn1) != acc) amb = 1;
                        if (u1 && accept(qn0, -qn1) != acc) amb = 1;
                        if (u0 && u1 && accept(-qn0, -qn1) != acc) amb = 1;
                    }
                }
                amb |= nearT;
                const unsigned accM = __ballot_sync(FULL, acc && !amb) & pending;
                const unsigned blkM = __ballot_sync(FULL, amb) & pending;
                const int fa = accM ? __ffs(accM) - 1 : 32;
                const int fb = blkM ? __ffs(blkM) - 1 : 32;
                if (fb < fa) {
                    // undecided lanes below fb reject
                    pending &= ~((1u << fb) - 1u);
                    if (lane == 0 && publish) st_relaxed_u64(outLog + (size_t)y * nWords + b, log_word(b, fb, accBits));
                    if (__shfl_sync(FULL, nearT, fb)) {
                        // fb is flagged: the exact warp decides its trial in FP64 from the
                        // exact field (every flip before the trial is in qs), for each value
                        // of the neighbours' spin sum; then the round is evaluated again.
                        // (The decider's arrival on a named barrier wakes the exact warp, which
                        // sleeps there between requests; the decider's wait is bounded.)
                        if (lane == fb) {
                            const int sl = (g0 + lane) / N;
                            S.exX = x;
                            S.exQ = qx;
                            S.exU = u;
                            S.exG = T.G ? T.G[sl] : T.Gs;
                            S.exBeta = T.beta ? T.beta[sl] : T.betas;
                        }
                        ++exSeq;
                        __syncwarp();
                        __threadfence_block();
                        bar_arrive(kBarExReq, 64);
                        if (!wait_until(waitNs, [&] { return uniform_acquire(&S.exDone) == exSeq; })) {
                            aborted = true;
                            break;
                        }
                        if (lane == fb) {
                            exBits = S.exBits;
                            exValid = true;
                        }
                        continue;
                    }
                    // fb waits for its neighbour trials
                    const int w0 = __shfl_sync(FULL, nd0, fb), w1 = __shfl_sync(FULL, nd1, fb);
                    unsigned long long av = 0;
                    if (!wait_until(waitNs, [&] {
                            av = uniform_acquire64(&S.logAvail);
                            return avail_of(av, 0) > w0 && (nNbr < 2 || avail_of(av, 1) > w1);
                        })) {
                        aborted = true;
                        break;
                    }
                    // re-evaluate (the ghost rows and A are unchanged within the batch)
                    avEval = av;
                    evalNbr = true;
                    continue;
                }
                if (fa == 32) break;  // every undecided lane rejects
                // undecided lanes below fa reject; fa flips
                const int xf = __shfl_sync(FULL, x, fa);
                const float df = -2.f * __shfl_sync(FULL, qx, fa);
                if (lane == fa) {
                    qs[x] = (int8_t)(qx > 0.f ? -1 : 1);
                    d = df;
                    if (T.trace) {
                        const int s = (g0 + lane) / N, k = g0 + lane - s * N;
                        uint32_t bitIdx = (uint32_t)k * (uint32_t)m + (uint32_t)y;
                        atomicOr(&T.trace[(size_t)s * wordsPerStep + (bitIdx >> 5)], 1u << (bitIdx & 31));
                    }
                }
                if (lane > fa) {
                    const float jv = ((pred >> fa) & 1u) ? jg[fa] : __ldg(T.J + (size_t)xf * T.ldJ + x);
                    Fv = __fmaf_rn(df, jv, Fv);
                    xt = trial_xtol(tolD, hx, __fmul_rn(2.f, Fv), Lu);
                    if (x == xf) qx = -qx;
                    exValid = false;  // the trial now follows another flip
                }
                accBits |= 1u << fa;
                pending &= ~((2u << fa) - 1u);
                // trials through fa are decided: make them visible to the neighbours
                if (lane == 0 && pending && publish) st_relaxed_u64(outLog + (size_t)y * nWords + b, log_word(b, fa + 1, accBits));
            }
            if (aborted) break;
            __syncwarp();
            if (lane == 0) {
                S.decDone = b + 1;  // this batch's buffer is free
                if (publish) st_relaxed_u64(outLog + (size_t)y * nWords + b, log_word(b, nValid, accBits));
            }
            const int nf = __popc(accBits);
            accepted += (unsigned long long)nf;

            // the next batch's sites
            const bool more = b + 1 < nBatches;
            // (while waiting, keep applying published neighbour iterations of this and
            // earlier batches: the prefetchers may need those ring slots)
            if (more && !wait_until(waitNs, [&] {
                    if (uniform_acquire(&S.readyTag[(b + 1) & (kPre - 1)]) == b + 2) return true;
                    if (nNbr > 0) apply_nbr(g0 + 32, g0 + 32);
                    return false;
                })) {
                aborted = true;
                break;
            }
            const int xN = more ? preX[((b + 1) & (kPre - 1)) * 32 + lane] : 0;
            const bool validN = g0 + 32 + lane < Itot;
            // the next batch's fields start from the resident row once the updaters
            // are done with the previous batch's flips; this batch's flips are
            // gathered now and added after the next batch's neighbour work
            const bool defer = nf <= kGv;
            if (defer && accBits) {
                unsigned rem = accBits;
#pragma unroll
                for (int t = 0; t < kGv; ++t) {
                    const int xf = __shfl_sync(FULL, x, __ffs(rem) - 1);
                    gv[t] = validN ? __ldg(T.J + (size_t)xf * T.ldJ + xN) : 0.f;
                    rem &= rem - 1u;
                    if (!rem) break;
                }
            }
            bar_sync(2, kBarCount);
            float FvN = validN ? Fs[xN] : 0.f;
            if ((accBits >> lane) & 1u) flips[__popc(accBits & ((1u << lane) - 1u))] = make_int2(x, __float_as_int(d));
            if (lane == 0) S.nflip = nf;
            __syncwarp();
            __threadfence_block();
            bar_arrive(1, kBarCount);
            nfPrev = defer ? nf : 0;
            if (!defer) {
                // many flips: add them all now, in trial order
                unsigned rem = accBits;
                while (rem) {
                    const int f = __ffs(rem) - 1;
                    rem &= rem - 1u;
                    const int xf = __shfl_sync(FULL, x, f);
                    const float df = __shfl_sync(FULL, d, f);
                    if (validN) FvN = __fmaf_rn(df, __ldg(T.J + (size_t)xf * T.ldJ + xN), FvN);
                }
            }
            x = xN;
            Fv = FvN;
        }
        bar_sync(2, kBarCount);  // the updaters are done with the last flips
        if (lane == 0) {
            if (aborted && T.status) atomicExch(T.status, (int)kErrTimeout);
            if (T.accepted) atomicAdd(T.accepted, accepted);
            S.nflip = -1;
            S.done = 1;
        }
        __syncwarp();
        __threadfence_block();
        bar_arrive(1, kBarCount);
        bar_arrive(kBarExReq, 64);  // the exact warp sees done and leaves
    } else if (warp == 1) {
        // -------------------------------------------------------------- helper
        // lane l < 4 polls word (avail[n] >> 5) + dw of neighbour n = l & 1, dw = l >> 1
        int avail0 = 0, avail1 = 0;
        const int n = lane & 1, dw = lane >> 1;
        const unsigned long long *nbLog = outLog + (size_t)(n ? nbr1 : nbr0) * nWords;
        while (nNbr > 0 && !__shfl_sync(FULL, (int)S.done, 0)) {
            const int an = n ? avail1 : avail0;
            const int w = (an >> 5) + dw;
            unsigned long long v = 0;
            if (lane < 4 && n < nNbr && w * 32 < Itot && w < (S.applied[n] >> 5) + kLogWords)
                v = ld_relaxed_u64(nbLog + w);
            bool moved = false;
#pragma unroll
            for (int nn = 0; nn < 2; ++nn) {
                int &a = nn ? avail1 : avail0;
#pragma unroll
                for (int ww = 0; ww < 2; ++ww) {
                    const unsigned long long vv = __shfl_sync(FULL, v, nn + 2 * ww);
                    const int wv = __shfl_sync(FULL, w, nn + 2 * ww);
                    // words are consumed in order: the second only after the first is complete
                    if (nn >= nNbr || wv != (a >> 5) || (int)(vv >> 38) != wv + 1) break;
                    const int c = (int)((vv >> 32) & 63u);
                    if (wv * 32 + c <= a) break;
                    if (lane == 0) nlog[nn * kLogWords + (wv & (kLogWords - 1))] = (uint32_t)vv;
                    a = wv * 32 + c;
                    moved = true;
                    if (c < min(32, Itot - wv * 32)) break;  // batch still being decided
                }
            }
            if (moved) {
                __syncwarp();
                if (lane == 0)
                    st_release_cta64(&S.logAvail, (unsigned long long)(unsigned)avail0 |
                                                      ((unsigned long long)(unsigned)avail1 << 32));
            }
        }
    } else if (warp == kExactWarp) {
        // --------------------------------------------------------- exact warp
        // Sleeps on a named barrier until the decider posts a flagged trial (or
        // the end of the sweep) and arrives on it: sums
        // its exact field (the integer row sum, as the one-CTA kernel computes it)
        // and decides it in FP64 for each value of the neighbours' spin sum (lane
        // k < 3: the sum 2k - 2).
        for (int seq = 1;; ++seq) {
            bar_sync(kBarExReq, 64);
            if (S.done) break;
            const int xr = S.exX;
            const float qr = S.exQ, ur = S.exU, Gr = S.exG, br = S.exBeta;
            const double hr = T.h64 ? T.h64[xr] : (double)hs[xr];
            const double F = T.J64 ? exact_field_warp(T.J64 + (size_t)xr * N, qs, N)
                                   : exact_field_warp(T.J + (size_t)xr * T.ldJ, qs, N);
            const int ok = lane < 3 ? exact_accept(sa, true, qr, hr, F, lane == 0 ? -1.f : 1.f, lane == 2 ? 1.f : -1.f,
                                                   m, Gr, br, ur)
                                    : 0;
            const unsigned bits = __ballot_sync(FULL, ok) & 7u;
            if (lane == 0) {
                S.exBits = (int)bits;
                st_release_cta(&S.exDone, seq);
            }
            __syncwarp();
        }
    } else if (warp < kUpdWarp0) {
        // --------------------------------------------------------- prefetchers
        const int pw = warp - 2;
        int s = 0, k = lane + 32 * pw, cs = -1;
        while (k >= N) {
            k -= N;
            ++s;
        }
        StepConst sc = {0.f, 0.f, 0.f};
        for (int p = pw; p < nBatches; p += kPf) {
            // buffer p % kPre is free once the decider has finished batch p - kPre,
            // and ring slots j - kRing are applied for the neighbours' iterations j of batch p
            const int jEnd = 32 * p + 32;
            int stop = 0;
            if (!wait_until<kPrefetchSleepNs>(waitNs, [&] {
                    int ok = 0;
                    if (lane == 0) {
                        stop = S.done;
                        ok = stop || (S.decDone > p - kPre && (nNbr < 1 || S.applied[0] + kRing >= jEnd) &&
                                      (nNbr < 2 || S.applied[1] + kRing >= jEnd));
                    }
                    return __shfl_sync(FULL, ok, 0) != 0;
                }))
                break;
            if (__shfl_sync(FULL, stop, 0)) break;
            __threadfence_block();
            const int buf = p & (kPre - 1);
            const int j = 32 * p + lane;
            const bool valid = j < Itot;
            int x = 0;
            float u = 0.f;
            if (valid) {
                u32x4 r = draw(T.seed, (uint32_t)k, (uint32_t)y, T.step0 + (uint32_t)s, tag);
                x = draw_index(r.x, N);
                u = draw_unit(r.y);
                if (s != cs) {
                    const float G = T.G ? T.G[s] : T.Gs, beta = T.beta ? T.beta[s] : T.betas;
                    sc = step_const(T.algo, m, G, beta);
                    cs = s;
                }
            }
            // the in-batch gathers J[x_f][x_i] (i > f) are needed only for the lanes f
            // that accept: predict them from the current (a few batches stale) field,
            // spins and ghost rows with a margin for the drift; the decider gathers
            // the row of an accepting lane that was not predicted itself
            unsigned pred;
            {
                const volatile float *vF = Fs, *vh = hs;
                const volatile int8_t *vq = qs;
                const volatile uint32_t *vg = ghost;
                const float qx = (float)vq[x], hx = vh[x], fx = vF[x];
                float qn0 = ((vg[x >> 5] >> (x & 31)) & 1u) ? 1.f : -1.f;
                float qn1 = nNbr > 1 ? (((vg[ghostStride + (x >> 5)] >> (x & 31)) & 1u) ? 1.f : -1.f) : qn0;
                const float dE = sa ? dense_sa_dE(qx, hx, fx) : dense_sqa_dE(qx, hx, fx, qn0, qn1, sc.twoDivM, sc.coef);
                const float margin = (sa ? 4.f : 2.f * sc.twoDivM) * kFieldDrift;
                const float dEm = dE - margin;
                pred = __ballot_sync(FULL, valid && (dEm < 0.f || __fmul_rn(dEm, sc.rate) < neg_log_unit(u)));
            }
            float v[kPredRows];
            {
                unsigned r = pred;
#pragma unroll
                for (int t = 0; t < kPredRows; ++t) {
                    if (!r) break;
                    const int f = __ffs(r) - 1;
                    r &= r - 1u;
                    const int xf = __shfl_sync(FULL, x, f);
                    v[t] = (lane > f && valid) ? __ldg(T.J + (size_t)xf * T.ldJ + x) : 0.f;
                }
            }
            // the neighbours' sites of the same iterations (while the gathers are in
            // flight): ring entries and the batch's site bitmaps; then, per lane and
            // neighbour, the latest kCand iterations of batches p - 2 .. p that hit
            // the lane's site up to its limit (-2: more than kCand)
            if (nNbr > 0) {
                uint32_t *bp = bm + (p & (kBmSlots - 1)) * kBmWords;
                bp[lane] = 0u;
                bp[lane + 32] = 0u;
                if (nNbr > 1) {
                    bp[kBmSlots * kBmWords + lane] = 0u;
                    bp[kBmSlots * kBmWords + lane + 32] = 0u;
                }
                __syncwarp();
                int cur0 = -1, cur1 = -1;
                if (valid) {
                    cur0 = draw_index(draw(T.seed, (uint32_t)k, (uint32_t)nbr0, T.step0 + (uint32_t)s, tag).x, N);
                    ring[j & (kRing - 1)] = cur0;
                    atomicOr(&bp[(cur0 & (kBmBits - 1)) >> 5], 1u << (cur0 & 31));
                    if (nNbr > 1) {
                        cur1 = draw_index(draw(T.seed, (uint32_t)k, (uint32_t)nbr1, T.step0 + (uint32_t)s, tag).x, N);
                        ring[kRing + (j & (kRing - 1))] = cur1;
                        atomicOr(&bp[kBmSlots * kBmWords + ((cur1 & (kBmBits - 1)) >> 5)], 1u << (cur1 & 31));
                    }
                }
                // batch p - 1 (the other prefetcher's) must be in the ring; its buffer
                // slot may already hold a later batch (batch p - 2 is this warp's own)
                if (!kSmall && p > 0 &&
                    !wait_until<kPrefetchSleepNs>(waitNs, [&] { return uniform_acquire(&S.readyTag[(p - 1) & (kPre - 1)]) >= p; }))
                    break;
                __syncwarp();
                const int hb = x & (kBmBits - 1);
                if (kSmall) {
                    // the sites of the neighbours' iterations 32 (p - q) + lane, q = 1, 2,
                    // drawn again (the ring's entries for them are the other prefetcher's)
                    int sites[2][3];
#pragma unroll
                    for (int nn = 0; nn < 2; ++nn) {
                        sites[nn][0] = nn ? cur1 : cur0;
#pragma unroll
                        for (int q = 1; q < 3; ++q) {
                            const int jq = 32 * (p - q) + lane;
                            int sq = -1;
                            if (nn < nNbr && jq >= 0) {
                                const int s2 = jq / N, k2 = jq - s2 * N;
                                sq = draw_index(draw(T.seed, (uint32_t)k2, (uint32_t)(nn ? nbr1 : nbr0),
                                                     T.step0 + (uint32_t)s2, tag).x, N);
                            }
                            sites[nn][q] = sq;
                        }
                    }
                    // per batch and neighbour: the positions of each site in a table
                    // (cleared again after use), read at the lane's own site
                    uint32_t *tab = siteTab + pw * kSmallN;
#pragma unroll
                    for (int nn = 0; nn < 2; ++nn) {
                        if (nn >= nNbr) break;
                        const int lim = lane - 1 + (nn ? before1 : before0);
                        int c0 = -1, c1 = -1, cnt = 0;
                        // latest first: batch p, then p - 1, then p - 2, each from its last iteration
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            const int sq = sites[nn][q];
                            if (sq >= 0) atomicOr(&tab[sq], 1u << lane);
                            __syncwarp();
                            unsigned mk = valid ? tab[x] : 0u;
                            __syncwarp();
                            if (sq >= 0) tab[sq] = 0u;
                            __syncwarp();
                            if (q == 0) mk &= lim < 0 ? 0u : (lim >= 31 ? ~0u : (2u << lim) - 1u);
                            cnt += __popc(mk);
                            while (mk) {
                                const int t = 31 - __clz(mk);
                                mk &= ~(1u << t);
                                const int jj = 32 * (p - q) + t;
                                if (c0 < 0)
                                    c0 = jj;
                                else if (c1 < 0)
                                    c1 = jj;
                            }
                        }
                        if (cnt > kCand) c0 = -2;
                        cand[((buf * 2 + nn) * kCand) * 32 + lane] = c0;
                        cand[((buf * 2 + nn) * kCand + 1) * 32 + lane] = cnt > kCand ? -1 : c1;
                    }
                } else {
#pragma unroll
                for (int nn = 0; nn < 2; ++nn) {
                    if (nn >= nNbr) break;
                    const uint32_t *bmn = bm + nn * kBmSlots * kBmWords;
                    const int prev = p > 0 ? ring[nn * kRing + ((32 * (p - 1) + lane) & (kRing - 1))] : -1;
                    const int prev2 = p > 1 ? ring[nn * kRing + ((32 * (p - 2) + lane) & (kRing - 1))] : -1;
                    const int cur = nn ? cur1 : cur0;
                    const int lim = lane - 1 + (nn ? before1 : before0);  // latest iteration of batch p a lane needs
                    auto marked = [&](int q) {
                        return q >= 0 && ((bmn[(q & (kBmSlots - 1)) * kBmWords + (hb >> 5)] >> (hb & 31)) & 1u);
                    };
                    const bool flag = valid && (marked(p) || marked(p - 1) || marked(p - 2));
                    int c0 = -1, c1 = -1;
                    unsigned hits = __ballot_sync(FULL, flag);
                    while (hits) {
                        const int i = __ffs(hits) - 1;
                        hits &= hits - 1u;
                        const int xi = __shfl_sync(FULL, x, i), li = __shfl_sync(FULL, lim, i);
                        const unsigned mc = __ballot_sync(FULL, cur == xi && lane <= li);
                        const unsigned mp = __ballot_sync(FULL, prev == xi);
                        const unsigned mq = __ballot_sync(FULL, prev2 == xi);
                        if (lane == i) {
                            if (__popc(mc) + __popc(mp) + __popc(mq) > kCand) {
                                c0 = -2;
                            } else {
                                // the latest two: batch p first, then p - 1, then p - 2
                                const unsigned ms[3] = {mc, mp, mq};
#pragma unroll
                                for (int q = 0; q < 3; ++q) {
                                    for (unsigned r = ms[q]; r; r &= ~(1u << (31 - __clz(r)))) {
                                        const int jj = 32 * (p - q) + 31 - __clz(r);
                                        if (c0 < 0)
                                            c0 = jj;
                                        else
                                            c1 = jj;
                                    }
                                }
                            }
                        }
                    }
                    cand[((buf * 2 + nn) * kCand) * 32 + lane] = c0;
                    cand[((buf * 2 + nn) * kCand + 1) * 32 + lane] = c1;
                }
                }
            }
            float *jg = Jg + buf * kJgStride + lane * 33;
            {
                unsigned r = pred;
#pragma unroll
                for (int t = 0; t < kPredRows; ++t) {
                    if (!r) break;
                    const int f = __ffs(r) - 1;
                    r &= r - 1u;
                    jg[f] = v[t];
                }
                for (; r; r &= r - 1u) {  // more predicted rows than registers: gather the rest here
                    const int f = __ffs(r) - 1;
                    const int xf = __shfl_sync(FULL, x, f);
                    jg[f] = (lane > f && valid) ? __ldg(T.J + (size_t)xf * T.ldJ + x) : 0.f;
                }
            }
            if (lane == 0) prePred[buf] = pred;
            preX[buf * 32 + lane] = x;
            preU[buf * 32 + lane] = u;
            preL[buf * 32 + lane] = neg_log_unit(u);
            preC[buf * 96 + lane] = sc.twoDivM;
            preC[buf * 96 + 32 + lane] = sc.coef;
            preC[buf * 96 + 64 + lane] = sc.rate;
            __syncwarp();
            if (lane == 0) st_release_cta(&S.readyTag[buf], p + 1);
            k += 32 * kPf;
            while (k >= N) {
                k -= N;
                ++s;
            }
        }
    } else {
        // ----------------------------------------------------------- updaters
        const int ut = tid - 32 * kUpdWarp0;
        const int n4 = N / 4;
        float4 *F4 = reinterpret_cast<float4 *>(Fs);
        bar_arrive(2, kBarCount);
        for (;;) {
            bar_sync(1, kBarCount);
            const int nf = S.nflip;
            if (nf < 0) break;
            for (int c0 = ut; c0 < n4; c0 += 4 * kMcUpdaters) {
                float4 f[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    int c = c0 + t * kMcUpdaters;
                    if (c < n4) f[t] = F4[c];
                }
                for (int q = 0; q < nf; ++q) {
                    const int2 fl = flips[q];
                    const float d = __int_as_float(fl.y);
                    const float4 *Jr = reinterpret_cast<const float4 *>(T.J + (size_t)fl.x * T.ldJ);
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        int c = c0 + t * kMcUpdaters;
                        if (c < n4) {
                            float4 j = __ldg(Jr + c);
                            f[t].x = __fmaf_rn(d, j.x, f[t].x);
                            f[t].y = __fmaf_rn(d, j.y, f[t].y);
                            f[t].z = __fmaf_rn(d, j.z, f[t].z);
                            f[t].w = __fmaf_rn(d, j.w, f[t].w);
                        }
                    }
                }
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    int c = c0 + t * kMcUpdaters;
                    if (c < n4) F4[c] = f[t];
                }
            }
            // the last N % 4 fields (J rows start on 16-byte boundaries: ldJ % 4 == 0)
            if (ut < N - 4 * n4) {
                const int i = 4 * n4 + ut;
                float f = Fs[i];
                for (int q = 0; q < nf; ++q) {
                    const int2 fl = flips[q];
                    f = __fmaf_rn(__int_as_float(fl.y), __ldg(T.J + (size_t)fl.x * T.ldJ + i), f);
                }
                Fs[i] = f;
            }
            __threadfence_block();
            bar_arrive(2, kBarCount);
        }
    }
    __syncthreads();
    for (int i = tid; i < N; i += kMcThreads) {
        T.F[(size_t)y * N + i] = Fs[i];
        T.q[(size_t)y * N + i] = qs[i];
    }
}

static size_t multi_smem_bytes(int N) {
    size_t ghostStride = (size_t)((N + 31) / 32 + 1) & ~(size_t)1;
    return (size_t)N * 4 * 2 + (size_t)kPre * (kJgStride + 32 + 96 + 32 + 32) * 4 + 2 * ghostStride * 4 +
           (size_t)2 * kBmSlots * kBmWords * 4 + 2 * kRing * 4 + 2 * kLogWords * 4 + (size_t)kPre * 2 * kCand * 32 * 4 + kPre * 4 +
           32 * 8 + (size_t)((N + 15) & ~15) + 16 + (N <= kSmallN ? (size_t)kPf * kSmallN * 4 : 0);
}

static std::array<const void *, 4> multi_kernels() {
    return {(const void *)dense_sweep_multi<false, false>, (const void *)dense_sweep_multi<true, false>,
            (const void *)dense_sweep_multi<false, true>, (const void *)dense_sweep_multi<true, true>};
}

static int multi_capacity(int N) {
    // the last answer is cached; callers on several host threads share it
    static std::mutex mu;
    static int cachedN = -1, cachedCap = 0;
    std::lock_guard<std::mutex> lock(mu);
    if (N == cachedN) return cachedCap;
    int dev = 0, sms = 0, perSm = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    size_t smem = multi_smem_bytes(N);
    cudaFuncAttributes fa;
    cudaFuncGetAttributes(&fa, dense_sweep_multi<false, false>);
    if (smem + fa.sharedSizeBytes > (size_t)optin) return 0;
    // every instance: the launch takes the one the tasks' flags and sizes ask for
    perSm = 1 << 30;
    for (const void *k : multi_kernels()) {
        int ps = 0;
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, k, kMcThreads, smem) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        perSm = std::min(perSm, ps);
    }
    cachedN = N;
    cachedCap = perSm * sms;
    return cachedCap;
}

}  // namespace sq103

using namespace sq103;

extern "C" {

SQ103_API unsigned long long sq103_dense_ws_bytes(int N, int m, int nSteps) {
    unsigned long long nWords = ((unsigned long long)nSteps * N + 31) / 32;
    return (unsigned long long)m * nWords * 8 + 256;
}

SQ103_API int sq103_dense_multicta_ok(int N, int m, int algo) {
    if (algo != kColoring && algo != kSANaive) return 0;
    if (N < 64 || m < 2) return 0;
    return m <= multi_capacity(N) ? 1 : 0;
}

// n instances in one cooperative launch (see McPack)
static int launch_pack(const sq103_dense_task *tasks, int n, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n < 1 || n > kMaxPack) return kErrBadShape;
    McPack P = {};
    P.n = n;
    int maxN = 0, ctas = 0;
    bool hooks = false;
    for (int i = 0; i < n; ++i) {
        const sq103_dense_task &t = tasks[i];
        hooks |= (t.flags & (kFlagShortWaits | kFlagWithholdTrotter0)) != 0;
        const int N = t.N, m = t.m;
        if (t.algo != kColoring && t.algo != kSANaive) return kErrBadShape;
        if (N < 64 || m < 2 || t.nSteps < 1) return kErrBadShape;
        if ((long long)t.nSteps * N >= (1ll << 31)) return kErrBadShape;
        // rows of J are read as float4
        if ((t.ldJ & 3) || (reinterpret_cast<uintptr_t>(t.J) & 15)) return kErrBadShape;
        if (!t.ws || t.wsBytes < sq103_dense_ws_bytes(N, m, t.nSteps)) return kErrCapacity;
        P.t[i] = t;
        P.outLog[i] = reinterpret_cast<unsigned long long *>(t.ws);
        P.nWords[i] = (int)(((long long)t.nSteps * N + 31) / 32);
        P.base[i] = ctas;
        ctas += m;
        maxN = std::max(maxN, N);
    }
    for (int i = n; i <= kMaxPack; ++i) P.base[i] = ctas;
    // every CTA resident at once (cooperative launch); also sets the kernel's shared-memory limit
    if (multi_capacity(maxN) < ctas) return kErrCapacity;
    for (int i = 0; i < n; ++i) {
        // the accept words carry their batch tag; zero means "not published"
        cudaError_t e = cudaMemsetAsync(P.outLog[i], 0, (size_t)tasks[i].m * P.nWords[i] * 8, st);
        if (e != cudaSuccess) return (int)e;
    }
    void *args[] = {&P};
    const bool small = maxN <= kSmallN;
    const void *kernel = small ? (hooks ? (const void *)dense_sweep_multi<true, true>
                                        : (const void *)dense_sweep_multi<false, true>)
                               : (hooks ? (const void *)dense_sweep_multi<true, false>
                                        : (const void *)dense_sweep_multi<false, false>);
    return (int)cudaLaunchCooperativeKernel(kernel, dim3(ctas), dim3(kMcThreads), args, multi_smem_bytes(maxN), st);
}

// launched from sq103_dense_anneal (dense.cu) when the shape and workspace allow it
int sq103_dense_anneal_multi(const sq103_dense_task *t, void *stream) { return launch_pack(t, 1, stream); }

SQ103_API int sq103_dense_anneal_pack(const sq103_dense_task *tasks, int n, void *stream) {
    if (!tasks) return kErrBadShape;
    return launch_pack(tasks, n, stream);
}

SQ103_API int sq103_dense_multicta_capacity(int N) { return N >= 64 ? multi_capacity(N) : 0; }

}  // extern "C"
