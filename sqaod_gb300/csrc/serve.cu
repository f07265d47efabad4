// serve.cu -- continuous-batching request server for anneals of mixed size and type.
//
// Requests (dense or bipartite QUBO, own N, m, seed and G/beta schedule) are
// admitted in arrival order as soon as their device-memory footprint fits the
// budget and a slot is free (a request that cannot start yet does not block
// the ones behind it).  Admitted instances stay resident (couplings,
// spins, fields; the RNG state is (seed, step) and lives in the task).  Every
// tick advances every active instance by 8 annealOneSteps (one field-refresh
// period):
//   - dense instances whose spins and fields fit in shared memory, and small
//     bipartite instances, in the persistent batch kernels (one launch each,
//     instance count read on the device);
//   - large dense instances with the one-CTA-per-trotter kernel and large
//     bipartite instances with the per-instance kernels, a few at a time;
//   - dense fields are refreshed every 8 steps, as the single-instance annealer
//     does, so each instance ends exactly as it would alone.
// Finished instances get their FP64 energies and spins copied out, and their
// slot and memory are released in the same tick, so a waiting request can be
// admitted by the next tick.
// Dense brute-force searches are served too: each tick searches the next 2^30
// packed states of every active search with the single-instance searcher's own
// range search (its own stream, so the sub-range runs while the tick's anneals
// do), and a search that reaches 2^N completes with its exact minimum and
// minimisers.  No counterpart in the reference.
#include <algorithm>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <vector>

#include "host_util.h"
#include "sq_common.cuh"
#include "sq_kernels.h"

namespace sq103 {

namespace sq = sqaod;

class Server : public sq::NullBase {
public:
    static constexpr int kRefreshPeriod = 8;
    static constexpr int kStepsPerTick = kRefreshPeriod;  // refreshes fall on tick boundaries
    // bipartite instances with more spin x coupling products per half step than this
    // take the per-instance path (GEMMs over the whole GPU) instead of one CTA
    static constexpr size_t kBipLargeWork = (size_t)1 << 22;
    enum State { kQueued = 0, kActive = 1, kDone = 2 };
    enum Kind { kDenseAnneal = 0, kBipartiteAnneal = 1, kSearch = 2 };
    static constexpr uint64_t kSearchChunk = 1ull << 30;  // states per search per tick
    static constexpr int kMaxSearches = 4;                 // active searches

    // device memory of one request, allocated and freed in stream order (no
    // device-wide synchronisation per request)
    struct AsyncMem {
        unsigned char *p = nullptr;
        void alloc(size_t bytes, cudaStream_t s) {
            release(s);
            SQ_CHECK(cudaMallocAsync((void **)&p, bytes, s));
        }
        void release(cudaStream_t s) {
            if (p) cudaFreeAsync(p, s);
            p = nullptr;
        }
        ~AsyncMem() {
            if (p) cudaFree(p);
        }
    };

    // Pinned staging for every host-to-device copy of the server: from pageable
    // memory cudaMemcpyAsync may wait for the stream, stalling the host behind
    // every queued tick.  Two halves are used in turn; a half is reused only
    // after an event recorded when it was left has passed.
    struct PinnedStage {
        unsigned char *base = nullptr;
        size_t half = 0, off = 0;
        int cur = 0;
        cudaEvent_t left[2] = {nullptr, nullptr};
        bool pending[2] = {false, false};
        ~PinnedStage() {
            if (base) cudaFreeHost(base);
            for (cudaEvent_t e : left)
                if (e) cudaEventDestroy(e);
        }
        void init(size_t halfBytes) {
            SQ_CHECK(cudaMallocHost((void **)&base, 2 * halfBytes));
            half = halfBytes;
            for (cudaEvent_t &e : left) SQ_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        void copy(void *dst, const void *src, size_t n, cudaStream_t s) {
            if (n > half) {  // larger than a half: directly from the caller's memory
                SQ_CHECK(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, s));
                return;
            }
            const size_t need = (n + 255) & ~(size_t)255;
            if (off + need > half) {
                SQ_CHECK(cudaEventRecord(left[cur], s));
                pending[cur] = true;
                cur ^= 1;
                if (pending[cur]) SQ_CHECK(cudaEventSynchronize(left[cur]));
                pending[cur] = false;
                off = 0;
            }
            unsigned char *p = base + cur * half + off;
            memcpy(p, src, n);
            off += need;
            SQ_CHECK(cudaMemcpyAsync(dst, p, n, cudaMemcpyHostToDevice, s));
        }
    };

    struct Request {
        int id, kind;  // Kind
        int N0, N1, m, optimize, nSteps;
        unsigned long long seed;
        std::vector<float> W, b0, b1, G, beta;
        int state = kQueued;
        // resident state
        AsyncMem mem;
        double *dE = nullptr;          // FP64 energies, computed when the last step is queued
        cudaEvent_t done = nullptr;    // recorded after them
        size_t bytes = 0;
        int pos = 0;     // steps done
        int slot = -1;   // batch slot, -1 for the per-instance kernel
        bool large = false;
        sq103_dense_task dt = {};
        sq103_bipartite_task bt = {};
        double *c64 = nullptr;
        int *dStatus = nullptr;        // this request's own timeout status word (dense sweeps)
        void *digits = nullptr;        // tensor-core refresh of a dense request with N >= 1024
        void *spinsBf16 = nullptr;
        int status = 0;                // its value once the request is done
        // a search: the searcher handle, the next state to search, 2^N, the list cap
        void *bf = nullptr;
        uint64_t xNext = 0, xMax = 0;
        int tile = 0;
        // results
        std::vector<double> E;
        std::vector<int8_t> q0, q1;
        ~Request() {
            if (bf) sq103_dg_bf_delete(bf);
        }
    };

    Server(unsigned long long budget, int maxSlots) : budget_(budget), maxSlots_(maxSlots) {
        dTasks_.ensure(maxSlots);
        bTasks_.ensure(maxSlots);
        dPos_.ensure(maxSlots);
        bPos_.ensure(maxSlots);
        counts_.ensure(2);
        queues_.ensure(4);
        stage_.init((size_t)96 << 20);
        SQ_CHECK(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
        for (cudaEvent_t &e : join_) SQ_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        SQ_CHECK(cudaMemsetAsync(queues_.p, 0, sizeof(int) * 4, st_.get()));
        SQ_CHECK(cudaMemsetAsync(counts_.p, 0, sizeof(int) * 2, st_.get()));
        int dev = 0;
        SQ_CHECK(cudaGetDevice(&dev));
        SQ_CHECK(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
        stageSmem_ = std::min(sq103_dense_batch_max_smem(), 96 * 1024);
        denseGrid_ = sms_ * std::max(1, sq103_dense_batch_ctas_per_sm(stageSmem_));
        bipGrid_ = sms_ * 4;
        // request memory comes from the device's stream-ordered pool: keep what is
        // freed for the next requests instead of returning it at every sync
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        st_.sync();
    }

    ~Server() {
        for (Request *r : finishing_)
            if (r->done) cudaEventDestroy(r->done);
        cudaEventDestroy(fork_);
        for (cudaEvent_t e : join_) cudaEventDestroy(e);
    }

    int submitDense(const float *W, int N, int m, int optimize, unsigned long long seed, const float *G,
                    const float *beta, int nSteps) {
        throwErrorIf(N <= 0 || m <= 0 || nSteps <= 0, "bad request shape.");
        throwErrorIf(sq103_dense_batch_min_smem(m) > stageSmem_ && !sq103_dense_multicta_ok(N, m, kColoring),
                     "%d trotters of %d spins fit neither kernel.", m, N);
        throwErrorIf(!sqaod::isSymmetric(W, (size_t)N, (size_t)N), "%s, Matrix is not symmetric.", __func__);
        auto rq = std::make_unique<Request>();
        rq->kind = 0;
        rq->N0 = N;
        rq->N1 = 0;
        rq->W.assign(W, W + (size_t)N * N);
        return enqueue(std::move(rq), m, optimize, seed, G, beta, nSteps);
    }

    int submitBipartite(const float *b0, const float *b1, const float *W, int N0, int N1, int m, int optimize,
                        unsigned long long seed, const float *G, const float *beta, int nSteps) {
        throwErrorIf(N0 <= 0 || N1 <= 0 || m <= 0 || nSteps <= 0, "bad request shape.");
        auto rq = std::make_unique<Request>();
        rq->kind = 1;
        rq->N0 = N0;
        rq->N1 = N1;
        rq->W.assign(W, W + (size_t)N0 * N1);
        rq->b0.assign(b0, b0 + N0);
        rq->b1.assign(b1, b1 + N1);
        return enqueue(std::move(rq), m, optimize, seed, G, beta, nSteps);
    }

    int submitSearch(const float *W, int N, int optimize, int tileSize) {
        throwErrorIf(N <= 0 || N > 63, "a search needs 0 < N < 64, N=%d.", N);
        throwErrorIf(tileSize <= 0, "tile size must be positive.");
        throwErrorIf(!sqaod::isSymmetric(W, (size_t)N, (size_t)N), "%s, Matrix is not symmetric.", __func__);
        auto rq = std::make_unique<Request>();
        rq->kind = kSearch;
        rq->N0 = N;
        rq->N1 = 0;
        rq->tile = tileSize;
        rq->W.assign(W, W + (size_t)N * N);
        const float none = 0.f;
        return enqueue(std::move(rq), 1, optimize, 0, &none, &none, 1);
    }

    // kStepsPerTick steps (one refresh period) of every active instance and the
    // next range of every active search; returns the number of requests completed
    int tick() {
        const int nDone = finalizeReady(false);
        admit();
        const int nD = (int)denseSlots_.size(), nB = (int)bipSlots_.size();
        if (nD > 0)
            SQ_CHECK(sq103_dense_batch_launch(dTasks_.p, nD, counts_.p, nullptr, dPos_.p, queues_.p, kStepsPerTick,
                                              std::min(denseGrid_, nD), stageSmem_, st_.get()));
        if (nB > 0)
            SQ_CHECK(sq103_bipartite_batch_launch(bTasks_.p, nB, counts_.p + 1, nullptr, bPos_.p, queues_.p + 2,
                                                  kStepsPerTick, std::min(bipGrid_, nB), st_.get()));
        // large dense instances: packed cooperative launches (instances of similar
        // size together, as many trotters as can be resident); large bipartite: one by one
        std::vector<Request *> big;
        for (Request *r : large_)
            if (r->kind == 0) big.push_back(r);
        std::sort(big.begin(), big.end(), [](const Request *a, const Request *b) { return a->N0 < b->N0; });
        std::vector<sq103_dense_task> pack;
        int packM = 0, packN = 0;
        auto flush = [&]() {
            if (!pack.empty()) SQ_CHECK(sq103_dense_anneal_pack(pack.data(), (int)pack.size(), st_.get()));
            pack.clear();
            packM = packN = 0;
        };
        for (Request *r : big) {
            sq103_dense_task t = r->dt;
            t.G = r->dt.G + r->pos;
            t.beta = r->dt.beta + r->pos;
            t.step0 = 1 + (uint32_t)r->pos;
            t.nSteps = std::min(kStepsPerTick, r->nSteps - r->pos);
            const int N2 = std::max(packN, r->N0);
            if (pack.size() == (size_t)kMaxPack || packM + r->m > sq103_dense_multicta_capacity(N2)) flush();
            pack.push_back(t);
            packM += r->m;
            packN = std::max(packN, r->N0);
        }
        flush();
        // large bipartite requests: each one's launches in order on one of the side
        // streams, the requests side by side (each fills only part of the GPU)
        int nBig = 0;
        for (Request *r : large_) {
            if (r->kind != 1) continue;
            if (nBig == 0) fork();
            sq103_bipartite_task t = r->bt;
            t.G = r->bt.G + r->pos;
            t.beta = r->bt.beta + r->pos;
            t.step0 = 1 + (uint32_t)r->pos;
            t.nSteps = std::min(kStepsPerTick, r->nSteps - r->pos);
            SQ_CHECK(sq103_bipartite_anneal(&t, side_[nBig % kRefreshStreams].get()));
            ++nBig;
        }
        if (nBig > 0) join();
        std::vector<Request *> finished;
        jobs_.clear();
        tileJob_.clear();
        int nTc = 0;  // tensor-core refreshes queued on the side streams
        for (auto &kv : active_) {
            Request *r = kv.second;
            if (r->kind == kSearch) continue;   // advanced below
            if (r->pos >= r->nSteps) continue;  // finishing: its results are being collected
            r->pos = std::min(r->pos + kStepsPerTick, r->nSteps);
            if (r->kind == 0 && r->pos < r->nSteps && r->pos % kRefreshPeriod == 0) {
                if (r->digits) {  // on the side streams, forked from the work stream at the first
                    if (nTc == 0) fork();
                    SQ_CHECK(sq103_dense_refresh(r->dt.J, r->dt.ldJ, r->digits, r->spinsBf16, r->dt.q, r->dt.F, r->N0,
                                                 r->m, r->dStatus, side_[nTc % kRefreshStreams].get()));
                    ++nTc;
                } else {  // below the tensor-core size: with the others, in one launch
                    sq103_field_job j = {};
                    j.J = r->dt.J;
                    j.q = r->dt.q;
                    j.F = r->dt.F;
                    j.N = r->N0;
                    j.m = r->m;
                    j.ldJ = r->dt.ldJ;
                    j.tile0 = (int)tileJob_.size();
                    tileJob_.insert(tileJob_.end(), ((r->N0 + 63) / 64) * ((r->m + 63) / 64), (int)jobs_.size());
                    jobs_.push_back(j);
                }
            }
            if (r->pos >= r->nSteps) finished.push_back(r);
        }
        if (!jobs_.empty()) {
            // grown rarely (a larger buffer frees the old one, which waits for the device)
            dJobs_.ensure(std::max<size_t>(jobs_.size(), 1024));
            dTileJob_.ensure(std::max<size_t>(tileJob_.size(), 16384));
            stage_.copy(dJobs_.p, jobs_.data(), sizeof(sq103_field_job) * jobs_.size(), st_.get());
            stage_.copy(dTileJob_.p, tileJob_.data(), sizeof(int) * tileJob_.size(), st_.get());
            SQ_CHECK(sq103_dense_field_refresh_batch(dJobs_.p, dTileJob_.p, (int)tileJob_.size(), st_.get()));
        }
        if (nTc > 0) join();  // the next work on the stream sees every refreshed field
        for (Request *r : finished) finish(r);
        // searches: the next range of each, on the searcher's stream (the anneals
        // queued above run meanwhile)
        int nSearched = 0;
        for (size_t i = 0; i < searches_.size();) {
            Request *r = searches_[i];
            const uint64_t e = std::min<uint64_t>(r->xMax, r->xNext + kSearchChunk);
            bfCheck(sq103_dg_bf_search_subrange(r->bf, r->xNext, e));
            r->xNext = e;
            if (e < r->xMax) {
                ++i;
                continue;
            }
            searches_.erase(searches_.begin() + i);
            finishSearch(r);
            ++nSearched;
        }
        ++ticks_;
        // nothing left to step (queued requests wait for memory or slots that only
        // collected results free): wait for the results still being computed
        if (active_.size() == finishing_.size()) return nDone + nSearched + finalizeReady(true);
        return nDone + nSearched;
    }

    // the side streams start after the work queued so far on the work stream ...
    void fork() {
        SQ_CHECK(cudaEventRecord(fork_, st_.get()));
        for (Stream &x : side_) SQ_CHECK(cudaStreamWaitEvent(x.get(), fork_, 0));
    }
    // ... and the work stream continues after everything queued on them
    void join() {
        for (int k = 0; k < kRefreshStreams; ++k) {
            SQ_CHECK(cudaEventRecord(join_[k], side_[k].get()));
            SQ_CHECK(cudaStreamWaitEvent(st_.get(), join_[k], 0));
        }
    }

    int state(int id) const {
        auto it = all_.find(id);
        throwErrorIf(it == all_.end(), "unknown request id %d.", id);
        return it->second->state;
    }

    const Request &request(int id) const {
        auto it = all_.find(id);
        throwErrorIf(it == all_.end(), "unknown request id %d.", id);
        return *it->second;
    }

    void release(int id) {
        auto it = all_.find(id);
        throwErrorIf(it == all_.end(), "unknown request id %d.", id);
        throwErrorIf(it->second->state != kDone, "request %d is not done.", id);
        all_.erase(it);
    }

    // ids completed since the last call, in completion order
    int drainCompleted(int *ids, int cap) {
        const int n = std::min<int>(cap, (int)completed_.size());
        for (int i = 0; i < n; ++i) ids[i] = completed_[i];
        completed_.erase(completed_.begin(), completed_.begin() + n);
        return n;
    }

    // Fault injection from the host (tests): writes `value` into an active dense
    // request's status word, in stream order, as a sweep that gave up a bounded
    // wait would.  Only that request then reports the error.
    void injectStatus(int id, int value) {
        auto it = all_.find(id);
        throwErrorIf(it == all_.end(), "unknown request id %d.", id);
        Request *r = it->second.get();
        throwErrorIf(r->state != kActive || r->dStatus == nullptr, "request %d is not an active request.", id);
        stage_.copy(r->dStatus, &value, sizeof(int), st_.get());
    }

    void setLargeLimit(int n) {
        throwErrorIf(n < 1, "the large-instance limit must be at least 1.");
        maxLarge_ = n;
    }

    int rows(int id) const {
        const Request &r = request(id);
        throwErrorIf(r.state != kDone, "request %d is not done.", id);
        return r.kind == kSearch ? (int)(r.q0.size() / (size_t)r.N0) : r.m;
    }

    void stats(int *queued, int *active, int *done, unsigned long long *bytes) const {
        if (queued) *queued = (int)queue_.size();
        if (active) *active = (int)active_.size();
        if (done) *done = done_;
        if (bytes) *bytes = used_;
    }

private:
    int enqueue(std::unique_ptr<Request> rq, int m, int optimize, unsigned long long seed, const float *G,
                const float *beta, int nSteps) {
        rq->id = nextId_++;
        rq->m = m;
        rq->optimize = optimize ? 1 : 0;
        rq->seed = seed;
        rq->nSteps = nSteps;
        rq->G.assign(G, G + nSteps);
        rq->beta.assign(beta, beta + nSteps);
        rq->bytes = footprint(*rq);
        throwErrorIf(rq->bytes > budget_, "request of %llu bytes exceeds the device-memory budget of %llu bytes.",
                     (unsigned long long)rq->bytes, budget_);
        Request *p = rq.get();
        all_[p->id] = std::move(rq);
        queue_.push_back(p);
        return p->id;
    }

    static size_t al(size_t b) { return (b + 255) & ~(size_t)255; }
    static size_t ldj(size_t N) { return (N + 3) & ~(size_t)3; }

    static size_t footprint(const Request &r) {
        size_t s = 8 * 256 + al(r.nSteps * 4) * 2;
        if (r.kind == kSearch) {
            // the searcher's couplings, workspace and candidate buffers
            const size_t N = r.N0, cap = std::min<size_t>(std::max<size_t>((size_t)r.tile, 1u << 16), 1u << 22);
            return s + al(N * N * 4) + al(sq103_bf_workspace_bytes((int)N)) + 2 * al(cap * 8);
        }
        if (r.kind == 0) {
            size_t N = r.N0, m = r.m;
            s += al(N * ldj(N) * 4) + al(N * 4) + al(m * N * 4) + al(m * N) + al(m * N * 8);
            if (sq103_dense_refresh_uses_tc((int)N))
                s += al(sq103_tc_digits_bytes((int)N, (int)N)) + al(sq103_tc_spins_bytes((int)m, (int)N));
        } else {
            size_t N0 = r.N0, N1 = r.N1, m = r.m;
            s += al(N0 * N1 * 4) + al(N0 * 4) + al(N1 * 4) + al(m * N0) + al(m * N1) + al(m * N0 * 4) +
                 al(m * N1 * 4) + al(m * N1 * 8);
            if (sq103_bipartite_refresh_uses_tc((int)N0, (int)N1, (int)m))
                s += al(sq103_tc_digits_bytes((int)N1, (int)N0)) + al(sq103_tc_digits_bytes((int)N0, (int)N1)) +
                     al(sq103_tc_spins_bytes((int)m, (int)std::max(N0, N1)));
        }
        return s;
    }

    bool fitsStaging(const Request &r) const {
        const size_t base = (size_t)sq103_dense_batch_min_smem(r.m);  // the flip lists
        return base + (size_t)r.m * r.N0 * 5 + (size_t)r.N0 * 4 <= (size_t)stageSmem_;
    }

    // Admits queued requests in arrival order as memory, slots and the large-instance
    // limit allow; a request that cannot start yet keeps its place and does not
    // block the ones behind it.
    void admit() {
        bool changed = false;
        size_t i = 0;
        while (i < queue_.size()) {
            Request *r = queue_[i];
            // bipartite requests whose fields the single-instance annealer computes on the
            // tensor cores take the per-instance kernels, which do the same
            const bool large = r->kind == kSearch ? false
                               : r->kind == 0 ? !fitsStaging(*r) && sq103_dense_multicta_ok(r->N0, r->m, kColoring)
                                              : (size_t)r->m * r->N0 * r->N1 > kBipLargeWork ||
                                                    sq103_bipartite_refresh_uses_tc(r->N0, r->N1, r->m);
            const bool fits =
                used_ + r->bytes <= budget_ &&
                (r->kind == kSearch ? (int)searches_.size() < kMaxSearches
                 : large            ? (int)large_.size() < maxLarge_  // each steps with the whole GPU every tick
                                    : (int)(r->kind == 0 ? denseSlots_.size() : bipSlots_.size()) < maxSlots_);
            if (!fits) {
                ++i;
                continue;
            }
            queue_.erase(queue_.begin() + i);
            r->large = large;
            setup(r);
            used_ += r->bytes;
            r->state = kActive;
            active_[r->id] = r;
            changed = true;
        }
        if (changed) {
            int c[2] = {(int)denseSlots_.size(), (int)bipSlots_.size()};
            // (through the pinned stage: the host does not wait for the stream)
            stage_.copy(counts_.p, c, sizeof(c), st_.get());
        }
    }

    static void bfCheck(int rc) {
        if (rc != 0) sqaod::throwError("search: %s", sq103_last_error());
    }

    void setup(Request *r) {
        const int m = r->m, n = r->nSteps;
        if (r->kind == kSearch) {
            // the single-instance searcher with the request's tile size: its range
            // searches give the result a whole search gives
            bfCheck(sq103_dg_bf_new(&r->bf));
            bfCheck(sq103_dg_bf_set_qubo(r->bf, r->W.data(), r->N0, r->optimize));
            char tile[32];
            snprintf(tile, sizeof(tile), "%d", r->tile);
            bfCheck(sq103_dg_bf_set_preference(r->bf, "tile_size", tile));
            bfCheck(sq103_dg_bf_prepare(r->bf));
            r->xNext = 0;
            r->xMax = 1ull << r->N0;
            searches_.push_back(r);
            r->W.clear();
            r->W.shrink_to_fit();
            return;
        }
        if (r->kind == 0) {
            const size_t N = r->N0;
            const size_t ldJ = ldj(N);  // rows padded to 16 bytes for the one-CTA-per-trotter sweep
            const bool tc = sq103_dense_refresh_uses_tc((int)N);  // as the single-instance annealer
            size_t oG = 0, oB = al(n * 4), oJ = oB + al(n * 4), oh = oJ + al(N * ldJ * 4), oc = oh + al(N * 4),
                   oF = oc + 512, oq = oF + al(m * N * 4), oR = oq + al(m * N), oE = oR + al(m * N * 8),
                   oD = oE + al(m * 8), oA = oD + (tc ? al(sq103_tc_digits_bytes((int)N, (int)N)) : 0),
                   oWs = oA + (tc ? al(sq103_tc_spins_bytes(m, (int)N)) : 0),
                   tot = oWs + (r->large ? al(sq103_dense_ws_bytes((int)N, m, kStepsPerTick)) : 0);
            r->bytes += tot - oWs;  // the accept-word workspace of a large instance
            r->mem.alloc(tot, st_.get());
            r->digits = tc ? r->mem.p + oD : nullptr;
            r->spinsBf16 = tc ? r->mem.p + oA : nullptr;
            unsigned char *b = r->mem.p;
            r->dE = (double *)(b + oE);
            float *G = (float *)(b + oG), *beta = (float *)(b + oB), *J = (float *)(b + oJ), *h = (float *)(b + oh);
            float *c32 = (float *)(b + oc);
            r->c64 = (double *)(b + oc + 256);
            r->dStatus = (int *)(b + oc + 384);
            SQ_CHECK(cudaMemsetAsync(r->dStatus, 0, sizeof(int), st_.get()));
            float *F = (float *)(b + oF);
            int8_t *q = (int8_t *)(b + oq);
            double *scratch = (double *)(b + oR);  // N doubles for the hamiltonian, m N for energies
            stage_.copy(G, r->G.data(), 4 * n, st_.get());
            stage_.copy(beta, r->beta.data(), 4 * n, st_.get());
            dW_.ensure(N * N);
            stage_.copy(dW_.p, r->W.data(), 4 * N * N, st_.get());
            SQ_CHECK(cudaMemsetAsync(J, 0, sizeof(float) * N * ldJ, st_.get()));
            SQ_CHECK(sq103_dense_hamiltonian(dW_.p, (int)N, (int)N, r->optimize, h, J, (int)ldJ, c32, r->c64, scratch,
                                             st_.get()));
            if (r->digits) SQ_CHECK(sq103_tc_make_digits(J, (int)ldJ, (int)N, (int)N, 0, r->digits, st_.get()));
            SQ_CHECK(sq103_randomize_spins(q, (int)N, m, r->seed, 0, 0, st_.get()));
            SQ_CHECK(sq103_dense_refresh(J, (int)ldJ, r->digits, r->spinsBf16, q, F, (int)N, m, r->dStatus,
                                         st_.get()));
            sq103_dense_task &t = r->dt;
            t = sq103_dense_task{};
            t.J = J; t.h = h; t.q = q; t.F = F; t.G = G; t.beta = beta;
            t.seed = r->seed; t.step0 = 1; t.N = (int)N; t.m = m; t.ldJ = (int)ldJ;
            t.algo = m == 1 ? kSANaive : kColoring;
            t.nSteps = n;
            t.status = r->dStatus;
            if (r->large) {
                t.ws = b + oWs;  // its own: large instances step together in packed launches
                t.wsBytes = sq103_dense_ws_bytes((int)N, m, kStepsPerTick);
                large_.push_back(r);
            } else {
                r->slot = (int)denseSlots_.size();
                denseSlots_.push_back(r);
                int zero = 0;
                stage_.copy(dTasks_.p + r->slot, &t, sizeof(t), st_.get());
                stage_.copy(dPos_.p + r->slot, &zero, sizeof(int), st_.get());
            }
        } else {
            const size_t N0 = r->N0, N1 = r->N1;
            const bool tc = sq103_bipartite_refresh_uses_tc((int)N0, (int)N1, m);  // as the single-instance annealer
            size_t oG = 0, oB = al(n * 4), oJ = oB + al(n * 4), oh0 = oJ + al(N0 * N1 * 4), oh1 = oh0 + al(N0 * 4),
                   oc = oh1 + al(N1 * 4), oq0 = oc + 512, oq1 = oq0 + al(m * N0), oF0 = oq1 + al(m * N1),
                   oF1 = oF0 + al(m * N0 * 4), oR = oF1 + al(m * N1 * 4), oE = oR + al(std::max(m * N1, N0 + N1) * 8),
                   oD1 = oE + al(m * 8), oD0 = oD1 + (tc ? al(sq103_tc_digits_bytes((int)N1, (int)N0)) : 0),
                   oA = oD0 + (tc ? al(sq103_tc_digits_bytes((int)N0, (int)N1)) : 0),
                   tot = oA + (tc ? al(sq103_tc_spins_bytes(m, (int)std::max(N0, N1))) : 0);
            r->mem.alloc(tot, st_.get());
            unsigned char *b = r->mem.p;
            r->dE = (double *)(b + oE);
            float *G = (float *)(b + oG), *beta = (float *)(b + oB), *J = (float *)(b + oJ);
            float *h0 = (float *)(b + oh0), *h1 = (float *)(b + oh1), *c32 = (float *)(b + oc);
            r->c64 = (double *)(b + oc + 256);
            int8_t *q0 = (int8_t *)(b + oq0), *q1 = (int8_t *)(b + oq1);
            float *F0 = (float *)(b + oF0), *F1 = (float *)(b + oF1);
            double *scratch = (double *)(b + oR);
            stage_.copy(G, r->G.data(), 4 * n, st_.get());
            stage_.copy(beta, r->beta.data(), 4 * n, st_.get());
            dW_.ensure(N0 * N1 + N0 + N1);
            stage_.copy(dW_.p, r->W.data(), 4 * N0 * N1, st_.get());
            stage_.copy(dW_.p + N0 * N1, r->b0.data(), 4 * N0, st_.get());
            stage_.copy(dW_.p + N0 * N1 + N0, r->b1.data(), 4 * N1, st_.get());
            SQ_CHECK(sq103_bipartite_hamiltonian(dW_.p + N0 * N1, dW_.p + N0 * N1 + N0, dW_.p, (int)N0, (int)N1,
                                                 r->optimize, h0, h1, J, c32, r->c64, scratch, st_.get()));
            SQ_CHECK(sq103_randomize_spins(q0, (int)N0, m, r->seed, 0, 0, st_.get()));
            SQ_CHECK(sq103_randomize_spins(q1, (int)N1, m, r->seed, 0, 1, st_.get()));
            r->dStatus = (int *)(b + oc + 384);
            SQ_CHECK(cudaMemsetAsync(r->dStatus, 0, sizeof(int), st_.get()));
            if (tc) {
                SQ_CHECK(sq103_tc_make_digits(J, (int)N0, (int)N1, (int)N0, 0, b + oD1, st_.get()));
                SQ_CHECK(sq103_tc_make_digits(J, (int)N0, (int)N0, (int)N1, 1, b + oD0, st_.get()));
            }
            sq103_bipartite_task &t = r->bt;
            t = sq103_bipartite_task{};
            t.J = J; t.h0 = h0; t.h1 = h1; t.q0 = q0; t.q1 = q1; t.F0 = F0; t.F1 = F1;
            if (tc) {
                t.digits1 = b + oD1;
                t.digits0 = b + oD0;
                t.spinsBf16 = b + oA;
            }
            t.status = r->dStatus;
            t.G = G; t.beta = beta; t.seed = r->seed; t.step0 = 1;
            t.N0 = (int)N0; t.N1 = (int)N1; t.m = m;
            t.algo = m == 1 ? kSAColoring : kColoring;
            t.nSteps = n;
            if (r->large) {
                large_.push_back(r);
            } else {
                r->slot = (int)bipSlots_.size();
                bipSlots_.push_back(r);
                int zero = 0;
                stage_.copy(bTasks_.p + r->slot, &t, sizeof(t), st_.get());
                stage_.copy(bPos_.p + r->slot, &zero, sizeof(int), st_.get());
            }
        }
        // copies from pageable host memory return once the data is staged, so
        // r->W and the task structs above may go now
        r->W.clear();
        r->W.shrink_to_fit();
    }

    // FP64 energies and spins out, memory and slot released
    // The request has queued its last step: its FP64 energies are queued behind
    // it and collected by finalizeReady() once an event says they are done, so
    // the host never waits for the GPU here.
    void finish(Request *r) {
        const int m = r->m;
        if (r->kind == 0) {
            const int N = r->N0;
            double *scratch = (double *)((unsigned char *)r->dt.q + al((size_t)m * N));
            SQ_CHECK(sq103_dense_energy(r->dt.J, r->dt.ldJ, r->dt.h, r->c64, r->dt.q, N, m, r->optimize, scratch,
                                        r->dE, nullptr, st_.get()));
        } else {
            double *scratch = (double *)((unsigned char *)r->bt.F1 + al((size_t)m * r->N1 * 4));
            SQ_CHECK(sq103_bipartite_energy(r->bt.J, r->bt.h0, r->bt.h1, r->c64, r->bt.q0, r->bt.q1, r->N0, r->N1,
                                            m, r->optimize, scratch, r->dE, nullptr, st_.get()));
        }
        SQ_CHECK(cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming));
        SQ_CHECK(cudaEventRecord(r->done, st_.get()));
        // free the slot now (the kernels skip finished instances anyway): the last slot moves into it
        if (r->kind == 0 && !r->large) removeSlot(denseSlots_, r, dTasks_.p, dPos_.p, 0);
        if (r->kind == 1 && !r->large) removeSlot(bipSlots_, r, bTasks_.p, bPos_.p, 1);
        if (r->large) large_.erase(std::find(large_.begin(), large_.end(), r));
        finishing_.push_back(r);
    }

    // A search that has covered its 2^N states: its minimum and minimisers out,
    // the searcher released, done in this tick.
    void finishSearch(Request *r) {
        bfCheck(sq103_dg_bf_make_solution(r->bf));
        double E = 0.;
        bfCheck(sq103_dg_bf_get_E64(r->bf, &E));
        int n = 0;
        bfCheck(sq103_dg_bf_solution_count(r->bf, &n));
        r->E.assign(1, E);
        r->q0.assign((size_t)std::max(n, 0) * r->N0, 0);
        int got = 0;
        if (n > 0) bfCheck(sq103_dg_bf_get_x(r->bf, r->q0.data(), n, &got));
        bfCheck(sq103_dg_bf_delete(r->bf));
        r->bf = nullptr;
        used_ -= r->bytes;
        active_.erase(r->id);
        r->state = kDone;
        completed_.push_back(r->id);
        ++done_;
    }

    // Collects, in completion order, the requests whose energies are done (all
    // of them when wait): energies, spins and the status word are copied on the
    // result stream, which waits only for that request's event, and its memory
    // is released.  Returns how many became done.
    int finalizeReady(bool wait) {
        int n = 0;
        while (!finishing_.empty()) {
            Request *r = finishing_.front();
            if (wait) {
                SQ_CHECK(cudaEventSynchronize(r->done));
            } else {
                const cudaError_t q = cudaEventQuery(r->done);
                if (q == cudaErrorNotReady) break;
                SQ_CHECK(q);
            }
            finishing_.pop_front();
            const int m = r->m;
            cudaStream_t rs = res_.get();
            SQ_CHECK(cudaStreamWaitEvent(rs, r->done, 0));
            r->E.resize(m);
            SQ_CHECK(cudaMemcpyAsync(r->E.data(), r->dE, sizeof(double) * m, cudaMemcpyDeviceToHost, rs));
            const int8_t *dq0 = r->kind == 0 ? r->dt.q : r->bt.q0;
            r->q0.resize((size_t)m * r->N0);
            SQ_CHECK(cudaMemcpyAsync(r->q0.data(), dq0, r->q0.size(), cudaMemcpyDeviceToHost, rs));
            if (r->kind == 1) {
                r->q1.resize((size_t)m * r->N1);
                SQ_CHECK(cudaMemcpyAsync(r->q1.data(), r->bt.q1, r->q1.size(), cudaMemcpyDeviceToHost, rs));
            }
            int status = 0;
            if (r->dStatus)
                SQ_CHECK(cudaMemcpyAsync(&status, r->dStatus, sizeof(int), cudaMemcpyDeviceToHost, rs));
            SQ_CHECK(cudaStreamSynchronize(rs));
            r->status = status;
            cudaEventDestroy(r->done);
            r->done = nullptr;
            r->mem.release(st_.get());
            used_ -= r->bytes;
            active_.erase(r->id);
            r->state = kDone;
            completed_.push_back(r->id);
            ++done_;
            ++n;
        }
        return n;
    }

    template <class T>
    void removeSlot(std::vector<Request *> &slots, Request *r, T *dTasks, int *dPos, int which) {
        const int s = r->slot, last = (int)slots.size() - 1;
        if (s != last) {
            Request *mv = slots[last];
            SQ_CHECK(cudaMemcpyAsync(dTasks + s, dTasks + last, sizeof(T), cudaMemcpyDeviceToDevice, st_.get()));
            SQ_CHECK(cudaMemcpyAsync(dPos + s, dPos + last, sizeof(int), cudaMemcpyDeviceToDevice, st_.get()));
            slots[s] = mv;
            mv->slot = s;
        }
        slots.pop_back();
        r->slot = -1;
        int c = (int)slots.size();
        hostCount_[which] = c;
        stage_.copy(counts_.p + which, &hostCount_[which], sizeof(int), st_.get());
    }

    Stream st_, res_;  // work; result copies
    // side streams for a tick's large bipartite requests and tensor-core field
    // refreshes, which each fill only part of the GPU
    static constexpr int kRefreshStreams = 4;
    Stream side_[kRefreshStreams];
    cudaEvent_t fork_ = nullptr, join_[kRefreshStreams] = {};
    // this tick's SIMT field refreshes (host table, device copy)
    std::vector<sq103_field_job> jobs_;
    std::vector<int> tileJob_;
    DevBuf<sq103_field_job> dJobs_;
    DevBuf<int> dTileJob_;
    PinnedStage stage_;
    unsigned long long budget_, used_ = 0;
    int maxSlots_, maxLarge_ = 64, sms_ = 0, denseGrid_ = 1, bipGrid_ = 1, stageSmem_ = 0, nextId_ = 0, done_ = 0;
    long long ticks_ = 0;
    int hostCount_[2] = {0, 0};
    std::map<int, std::unique_ptr<Request>> all_;
    std::deque<Request *> queue_;
    std::deque<int> completed_;
    std::map<int, Request *> active_;
    std::vector<Request *> denseSlots_, bipSlots_, large_, searches_;
    std::deque<Request *> finishing_;  // last step queued, results not yet collected
    DevBuf<sq103_dense_task> dTasks_;
    DevBuf<sq103_bipartite_task> bTasks_;
    DevBuf<int> dPos_, bPos_, counts_, queues_;
    DevBuf<float> dW_;
    static constexpr int kMaxPack = 16;  // instances per packed launch (sq103_dense_anneal_pack)
};

}  // namespace sq103

using namespace sq103;

namespace {
template <class F>
int serve_guard(F &&f) {
    try {
        f();
        return 0;
    } catch (const std::exception &e) {
        sq103_set_error(e.what());
    } catch (...) {
        sq103_set_error("unknown error");
    }
    return -1;
}
Server *as_server(void *h) {
    throwErrorIf(h == nullptr, "null handle or argument");
    Server *s = dynamic_cast<Server *>(static_cast<sqaod::NullBase *>(h));
    throwErrorIf(s == nullptr, "handle of the wrong type");
    return s;
}
}  // namespace

extern "C" {

SQ103_API int sq103_server_new(void **handle, unsigned long long budgetBytes, int maxSlots) {
    return serve_guard([&] {
        throwErrorIf(handle == nullptr, "null handle");
        *handle = static_cast<sqaod::NullBase *>(new Server(budgetBytes, maxSlots > 0 ? maxSlots : 4096));
    });
}
SQ103_API int sq103_server_delete(void *h) { return serve_guard([&] { delete as_server(h); }); }
SQ103_API int sq103_server_submit_dense(void *h, const float *W, int N, int m, int optimize, unsigned long long seed,
                                        const float *G, const float *beta, int nSteps, int *id) {
    return serve_guard([&] {
        throwErrorIf(!W || !G || !beta, "null argument");
        int i = as_server(h)->submitDense(W, N, m, optimize, seed, G, beta, nSteps);
        if (id) *id = i;
    });
}
SQ103_API int sq103_server_submit_bipartite(void *h, const float *b0, const float *b1, const float *W, int N0, int N1,
                                            int m, int optimize, unsigned long long seed, const float *G,
                                            const float *beta, int nSteps, int *id) {
    return serve_guard([&] {
        throwErrorIf(!b0 || !b1 || !W || !G || !beta, "null argument");
        int i = as_server(h)->submitBipartite(b0, b1, W, N0, N1, m, optimize, seed, G, beta, nSteps);
        if (id) *id = i;
    });
}
SQ103_API int sq103_server_submit_search(void *h, const float *W, int N, int optimize, int tileSize, int *id) {
    return serve_guard([&] {
        throwErrorIf(!W, "null argument");
        int i = as_server(h)->submitSearch(W, N, optimize, tileSize);
        if (id) *id = i;
    });
}
SQ103_API int sq103_server_result_rows(void *h, int id, int *rows) {
    return serve_guard([&] {
        throwErrorIf(!rows, "null argument");
        *rows = as_server(h)->rows(id);
    });
}
SQ103_API int sq103_server_tick(void *h, int *completed) {
    return serve_guard([&] {
        int c = as_server(h)->tick();
        if (completed) *completed = c;
    });
}
SQ103_API int sq103_server_state(void *h, int id, int *state) {
    return serve_guard([&] { *state = as_server(h)->state(id); });
}
SQ103_API int sq103_server_result(void *h, int id, double *E, int capE, int *m, int8_t *q0, int8_t *q1,
                                  long long capBytes, int release) {
    return serve_guard([&] {
        Server *s = as_server(h);
        const Server::Request &r = s->request(id);
        throwErrorIf(r.state != Server::kDone, "request %d is not done.", id);
        if (r.status != 0) {
            const int st = r.status;
            if (release) s->release(id);
            sqaod::throwError("request %d: its sweep gave up a bounded device wait (status %d); its spins and "
                       "energies are not valid.", id, st);
        }
        throwErrorIf((int)r.E.size() > capE, "energy capacity %d is smaller than %d.", capE, (int)r.E.size());
        if (E) memcpy(E, r.E.data(), sizeof(double) * r.E.size());
        if (m) *m = s->rows(id);
        throwErrorIf((long long)r.q0.size() > capBytes || (long long)r.q1.size() > capBytes, "spin capacity too small.");
        if (q0) memcpy(q0, r.q0.data(), r.q0.size());
        if (q1 && !r.q1.empty()) memcpy(q1, r.q1.data(), r.q1.size());
        if (release) s->release(id);
    });
}
SQ103_API int sq103_server_inject_status(void *h, int id, int value) {
    return serve_guard([&] { as_server(h)->injectStatus(id, value); });
}
SQ103_API int sq103_server_set_large_limit(void *h, int n) {
    return serve_guard([&] { as_server(h)->setLargeLimit(n); });
}
SQ103_API int sq103_server_completed(void *h, int *ids, int cap, int *n) {
    return serve_guard([&] {
        throwErrorIf(ids == nullptr && cap > 0, "null argument");
        const int k = as_server(h)->drainCompleted(ids, cap);
        if (n) *n = k;
    });
}
SQ103_API int sq103_server_stats(void *h, int *queued, int *active, int *done, unsigned long long *bytesInUse) {
    return serve_guard([&] { as_server(h)->stats(queued, active, done, bytesInUse); });
}

}  // extern "C"
