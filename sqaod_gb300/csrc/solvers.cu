// solvers.cu -- the sqaod::cuda solver classes (float) on the sm_103a kernels.
//
// Behaviour follows the reference's CUDA solvers (state machine, algorithm
// selection, preference handling, error messages):
//   dense annealer     sqaodc/cuda/CUDADenseGraphAnnealer.cu:26-375
//   bipartite annealer sqaodc/cuda/CUDABipartiteGraphAnnealer.cu
//   dense BF           sqaodc/cuda/CUDADenseGraphBFSearcher.cpp:15-185
//   bipartite BF       sqaodc/cuda/CUDABipartiteGraphBFSearcher.cpp
// with these differences, each deliberate:
//   - the naive sweeps (dense naive, bipartite naive and sa_naive) are
//     kernel-layer entry points; the annealers select algorithms as the
//     reference's CUDA annealers do (naive runs coloring);
//   - random numbers come from the in-kernel Philox stream
//     (seed, step counter), so a seeded run replays bit-exactly;
//   - returned energies are evaluated in FP64 on the GPU;
//   - BF ties are broken by an FP64 re-evaluation of the candidates; the
//     result is the first tileSize minimisers in ascending order (the
//     CUDA reference's append-while-short rule).
#include <float.h>
#include <math.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include <sqaodc/sqaodc.h>

#include "host_util.h"
#include "sq_common.cuh"
#include "sq_kernels.h"

namespace sq103 {

namespace sq = sqaod;

// Exact W == W^T on the device (the host check of sqaodc/common/Common.cpp:97-104,
// `!=` per element pair): each 32 x 32 tile on or below the diagonal is
// compared with its mirror tile, staged transposed in shared memory.
__global__ void sym_check_kernel(const float *W, int N, int ld, int *bad) {
    __shared__ float t[32][33];
    const int bx = blockIdx.x, by = blockIdx.y, tx = threadIdx.x, ty = threadIdx.y;
    if (bx > by) return;
    for (int j = ty; j < 32; j += 8) {
        const int r = bx * 32 + j, c = by * 32 + tx;
        t[j][tx] = (r < N && c < N) ? W[(size_t)r * ld + c] : 0.f;
    }
    __syncthreads();
    int mismatch = 0;
    for (int j = ty; j < 32; j += 8) {
        const int r = by * 32 + j, c = bx * 32 + tx;
        if (r < N && c < N && W[(size_t)r * ld + c] != t[tx][j]) mismatch = 1;
    }
    if (__syncthreads_or(mismatch) && tx == 0 && ty == 0) atomicOr(bad, 1);
}

// dst (rows x cols, row stride ldd) = fp32 rounding of src (row stride lds): the
// fp32 copy of a <double> problem that the sweeps run on
__global__ void round_to_f32(const double *src, int rows, int cols, int lds, float *dst, int ldd) {
    const size_t n = (size_t)rows * cols;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / cols, c = i - r * cols;
        dst[r * ldd + c] = (float)src[r * lds + c];
    }
}

static void round_problem(const double *src, int rows, int cols, int lds, float *dst, int ldd, cudaStream_t st) {
    const size_t n = (size_t)rows * cols;
    const int grid = (int)std::min<size_t>((n + 255) / 256, 4096);
    round_to_f32<<<grid, 256, 0, st>>>(src, rows, cols, lds, dst, ldd);
    SQ_CHECK(cudaGetLastError());
}

// a matrix with row stride = columns
template <class real>
static std::vector<real> dense_copy(const sq::MatrixType<real> &M) {
    std::vector<real> d((size_t)M.rows * M.cols);
    for (int i = 0; i < M.rows; ++i)
        memcpy(d.data() + (size_t)i * M.cols, M.data + (size_t)i * M.stride, sizeof(real) * M.cols);
    return d;
}
// host check of int8 bits (0 / 1) or spins (-1 / +1)
static void check_values(const int8_t *v, size_t n, bool spins, const char *fn) {
    for (size_t i = 0; i < n; ++i) {
        const int8_t a = v[i];
        if (spins ? (a != 1 && a != -1) : (a != 0 && a != 1))
            sq::throwError("%s, %s must be %s, got %d.", fn, spins ? "q" : "x", spins ? "-1 or +1" : "0 or 1", (int)a);
    }
}

class DeviceImpl : public sq::cuda::Device {
public:
    explicit DeviceImpl(int devNo) { initialize(devNo < 0 ? 0 : devNo); }
    void initialize(int devNo) override {
        devNo_ = devNo;
        SQ_CHECK(cudaSetDevice(devNo));
    }
    void finalize() override {}
    int devNo_ = 0;
};

static unsigned long long time_seed() { return (unsigned long long)time(nullptr); }

// ======================================================= dense annealer
class DenseAnnealer : public sq::cuda::DenseGraphAnnealer<float> {
public:
    typedef sq::MatrixType<float> Matrix;
    typedef sq::VectorType<float> Vector;

    DenseAnnealer() {
        m_ = -1;
        selectAlgorithm(sq::algoDefault);
    }

    void assignDevice(sq::cuda::Device &device) override {
        SQ_CHECK(cudaSetDevice(static_cast<DeviceImpl &>(device).devNo_));
    }

    // As the reference's CUDA annealer (CUDADenseGraphAnnealer.cu): coloring for
    // naive, sa_naive for sa_coloring.  The naive sweep kernels stay available at
    // the kernel layer (sq103_dense_anneal with algo 0).
    sq::Algorithm selectAlgorithm(sq::Algorithm algo) override {
        switch (algo) {
        case sq::algoColoring:
        case sq::algoSANaive:
            algo_ = algo;
            break;
        case sq::algoNaive:
            algo_ = sq::algoColoring;
            break;
        case sq::algoSAColoring:
            algo_ = sq::algoSANaive;
            break;
        default:
            selectDefaultAlgorithm(algo, sq::algoColoring, sq::algoSANaive);
            break;
        }
        return algo_;
    }

    sq::Preferences getPreferences() const override {
        sq::Preferences prefs = sq::Annealer<float>::getPreferences();
        prefs.pushBack(sq::Preference(sq::pnDevice, "cuda"));
        return prefs;
    }

    void seed(unsigned long long s) override {
        seed_ = s;
        step_ = 0;
        setState(solRandSeedGiven);
    }

    // <double> problems (sq::cuda::DenseGraphAnnealer<double>): the FP64 couplings
    // are kept for the trials the fp32 sweep flags (their exact decisions) and for
    // the energies; the sweep runs on their fp32 rounding.  W is N x N row-major.
    void setQUBO64(const double *W, int N, sq::OptimizeMethod om) {
        throwErrorIf(N <= 0, "%s, Shape does not match.", __func__);
        throwErrorIf(!sq::isSymmetric(W, (size_t)N, (size_t)N), "%s, Matrix is not symmetric.", __func__);
        clearState(solProblemSet);
        N_ = N;
        m_ = N_ / 4;
        om_ = om;
        allocProblem();
        allocFP64();
        const double sgn = om == sq::optMaximize ? -1. : 1.;  // maximize negates W (CUDADenseGraphAnnealer.cu:148-149)
        std::vector<double> w((size_t)N * N);
        for (size_t i = 0; i < w.size(); ++i) w[i] = sgn * W[i];
        DevBuf<double> dW;
        dW.ensure(w.size());
        SQ_CHECK(cudaMemcpyAsync(dW.p, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(sq103_dense_hamiltonian64(dW.p, N_, d_h64_.p, d_J64_.p, d_c64_.p, d_scratchN_.p, st_.get()));
        finishFP64();
        setState(solProblemSet);
    }

    void setHamiltonian64(const double *h, const double *J, double c, int N) {
        throwErrorIf(N <= 0, "%s, Shape does not match.", __func__);
        throwErrorIf(!sq::isSymmetric(J, (size_t)N, (size_t)N), "%s, Matrix is not symmetric.", __func__);
        clearState(solProblemSet);
        N_ = N;
        m_ = N_ / 4;
        om_ = sq::optMinimize;
        allocProblem();
        allocFP64();
        SQ_CHECK(cudaMemcpyAsync(d_h64_.p, h, sizeof(double) * N_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_J64_.p, J, sizeof(double) * N_ * N_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_c64_.p, &c, sizeof(double), cudaMemcpyHostToDevice, st_.get()));
        finishFP64();
        setState(solProblemSet);
    }

    void getHamiltonian64(double *h, double *J, double *c) {
        throwErrorIfProblemNotSet();
        throwErrorIf(!fp64_, "%s, the problem is not a double-precision one.", __func__);
        SQ_CHECK(cudaMemcpyAsync(h, d_h64_.p, sizeof(double) * N_, cudaMemcpyDeviceToHost, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(J, d_J64_.p, sizeof(double) * N_ * N_, cudaMemcpyDeviceToHost, st_.get()));
        *c = c64h_;
        st_.sync();
    }
    bool isFP64() const { return fp64_; }

    double getSystemE64(double G, double beta) {
        calculate_E();
        double E = 0.;
        for (int y = 0; y < m_; ++y) E += h_E64_.p[y];
        E /= m_;
        if (sq::isSQAAlgorithm(algo_)) {
            d_ring_.ensure(1);
            SQ_CHECK(sq103_ring_dot(d_q_.p, N_, m_, d_ring_.p, st_.get()));
            long long ring = 0;
            SQ_CHECK(cudaMemcpyAsync(&ring, d_ring_.p, sizeof(ring), cudaMemcpyDeviceToHost, st_.get()));
            st_.sync();
            E -= (double)ring * 0.5 / beta * std::log(std::tanh(G * beta / (double)m_));
        }
        return om_ == sq::optMaximize ? -E : E;
    }

    void setQUBO(const Matrix &W, sq::OptimizeMethod om) override {
        throwErrorIf(W.rows != W.cols, "%s, W is not a sqare matrix.", __func__);
        // the exact symmetry check (Common.cpp:97-104) runs on the uploaded copy,
        // before any state changes
        const int N = W.rows;
        DevBuf<float> dW;
        dW.ensure((size_t)N * N);
        upload(dW.p, N, W);
        throwErrorIf(!deviceSymmetric(dW.p, N, N), "%s, Matrix is not symmetric.", __func__);
        clearState(solProblemSet);
        N_ = N;
        m_ = N_ / 4;
        om_ = om;
        allocProblem();
        SQ_CHECK(sq103_dense_hamiltonian(dW.p, N_, N_, om == sq::optMaximize, d_h_.p, d_J_.p, ldJ_, d_c_.p,
                                         d_c64_.p, d_scratchN_.p, st_.get()));
        makeDigits();
        st_.sync();
        dropFP64();
        setState(solProblemSet);
    }

    bool deviceSymmetric(const float *dW, int N, int ld) {
        d_flag_.ensure(1);
        SQ_CHECK(cudaMemsetAsync(d_flag_.p, 0, sizeof(int), st_.get()));
        const int nT = (N + 31) / 32;
        sym_check_kernel<<<dim3(nT, nT), dim3(32, 8), 0, st_.get()>>>(dW, N, ld, d_flag_.p);
        SQ_CHECK(cudaGetLastError());
        int bad = 0;
        SQ_CHECK(cudaMemcpyAsync(&bad, d_flag_.p, sizeof(int), cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        return bad == 0;
    }

    void setHamiltonian(const Vector &h, const Matrix &J, float c) override {
        throwErrorIf(J.rows != J.cols, "%s, J is not a sqare matrix.", __func__);
        throwErrorIf(h.size != J.cols, "%s, Shape does not match.", __func__);
        throwErrorIf(!sq::isSymmetric(J), "%s, Matrix is not symmetric.", __func__);
        clearState(solProblemSet);
        N_ = J.rows;
        m_ = N_ / 4;
        om_ = sq::optMinimize;
        allocProblem();
        SQ_CHECK(cudaMemcpyAsync(d_h_.p, h.data, sizeof(float) * N_, cudaMemcpyHostToDevice, st_.get()));
        upload(d_J_.p, ldJ_, J);
        makeDigits();
        double c64 = (double)c;
        SQ_CHECK(cudaMemcpyAsync(d_c_.p, &c, sizeof(float), cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_c64_.p, &c64, sizeof(double), cudaMemcpyHostToDevice, st_.get()));
        st_.sync();
        dropFP64();
        setState(solProblemSet);
    }

    void getHamiltonian(Vector *h, Matrix *J, float *c) const override {
        throwErrorIfProblemNotSet();
        h->resize(N_);
        J->resize(N_, N_);
        SQ_CHECK(cudaMemcpyAsync(h->data, d_h_.p, sizeof(float) * N_, cudaMemcpyDeviceToHost, st_.get()));
        SQ_CHECK(cudaMemcpy2DAsync(J->data, sizeof(float) * J->stride, d_J_.p, sizeof(float) * ldJ_,
                                   sizeof(float) * N_, N_, cudaMemcpyDeviceToHost, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(c, d_c_.p, sizeof(float), cudaMemcpyDeviceToHost, st_.get()));
        const_cast<Stream &>(st_).sync();
    }

    void prepare() override {
        throwErrorIfProblemNotSet();
        throwErrorIf(m_ <= 0, "# trotters must be a positive integer.");
        if (!isRandSeedGiven()) seed(time_seed());
        setState(solRandSeedGiven);
        clearState(solPrepared);
        if (m_ == 1) selectDefaultSAAlgorithm(algo_, sq::algoSANaive);
        size_t mn = (size_t)m_ * N_;
        d_q_.ensure(mn);
        d_F_.ensure(mn);
        if (d_digits_.p) d_Abf_.ensure(sq103_tc_spins_bytes(m_, N_));
        d_E64_.ensure(m_);
        d_E32_.ensure(m_);
        h_E64_.ensure(m_);
        h_q_.ensure(mn);
        E_.resize(m_);
        setState(solPrepared);
    }

    void randomizeSpin() override {
        throwErrorIfNotPrepared();
        SQ_CHECK(sq103_randomize_spins(d_q_.p, N_, m_, seed_, step_++, 0, st_.get()));
        refreshFields();
        setState(solQSet);
    }

    void set_q(const sq::BitSet &q) override {
        throwErrorIfNotPrepared();
        throwErrorIf(q.size != N_, "Dimension of q, %d, should be equal to N, %d.", q.size, N_);
        for (int y = 0; y < m_; ++y) memcpy(h_q_.p + (size_t)y * N_, q.data, N_);
        uploadQ();
    }

    void set_qset(const sq::BitSetArray &qs) override {
        throwErrorIfProblemNotSet();
        for (int i = 0; i < qs.size(); ++i)
            throwErrorIf(qs[i].size != N_, "%s, Shape does not match.", __func__);
        throwErrorIf(qs.size() <= 0, "%s, empty q set.", __func__);
        m_ = qs.size();
        prepare();
        for (int y = 0; y < m_; ++y) memcpy(h_q_.p + (size_t)y * N_, qs[y].data, N_);
        uploadQ();
    }

    const sq::BitSetArray &get_q() const override {
        if (!isSolutionAvailable()) const_cast<DenseAnnealer *>(this)->makeSolution();
        return qlist_;
    }

    const sq::BitSetArray &get_x() const override {
        if (!isSolutionAvailable()) const_cast<DenseAnnealer *>(this)->makeSolution();
        return xlist_;
    }

    const Vector &get_E() const override {
        if (!isEAvailable()) const_cast<DenseAnnealer *>(this)->calculate_E();
        return E_;
    }

    void calculate_E() override {
        throwErrorIfQNotSet();
        checkStatus();
        d_r_.ensure((size_t)m_ * N_);
        if (fp64_)
            SQ_CHECK(sq103_dense_energy64(d_J64_.p, d_h64_.p, c64h_, d_q_.p, N_, m_, om_ == sq::optMaximize,
                                          d_E64_.p, st_.get()));
        else
            SQ_CHECK(sq103_dense_energy(d_J_.p, ldJ_, d_h_.p, d_c64_.p, d_q_.p, N_, m_, om_ == sq::optMaximize,
                                        d_r_.p, d_E64_.p, d_E32_.p, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(h_E64_.p, d_E64_.p, sizeof(double) * m_, cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        E_.resize(m_);
        for (int y = 0; y < m_; ++y) E_(y) = (float)h_E64_.p[y];
        setState(solEAvailable);
    }

    void makeSolution() override {
        throwErrorIfQNotSet();
        syncBits();
        setState(solSolutionAvailable);
        calculate_E();
    }

    float getSystemE(float G, float beta) const override {
        auto self = const_cast<DenseAnnealer *>(this);
        self->calculate_E();
        double E = 0.;
        for (int y = 0; y < m_; ++y) E += E_(y);
        E /= m_;
        if (sq::isSQAAlgorithm(algo_)) {
            self->d_ring_.ensure(1);
            SQ_CHECK(sq103_ring_dot(d_q_.p, N_, m_, self->d_ring_.p, st_.get()));
            long long ring = 0;
            SQ_CHECK(cudaMemcpyAsync(&ring, d_ring_.p, sizeof(long long), cudaMemcpyDeviceToHost, st_.get()));
            self->st_.sync();
            float coef = 0.5f / beta * std::log(std::tanh(G * beta / (float)m_));
            E -= (double)ring * coef;
        }
        if (om_ == sq::optMaximize) E = -E;
        return (float)E;
    }

    void annealOneStep(float G, float beta) override {
        throwErrorIfNotPrepared();
        throwErrorIfQNotSet();
        runSteps(nullptr, nullptr, G, beta, 1);
    }

    // extension: a whole schedule (host arrays) in one call
    void anneal(const float *G, const float *beta, int nSteps) {
        throwErrorIfNotPrepared();
        throwErrorIfQNotSet();
        if (nSteps <= 0) return;
        d_sched_.ensure(2 * (size_t)nSteps);
        SQ_CHECK(cudaMemcpyAsync(d_sched_.p, G, sizeof(float) * nSteps, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_sched_.p + nSteps, beta, sizeof(float) * nSteps, cudaMemcpyHostToDevice, st_.get()));
        runSteps(d_sched_.p, d_sched_.p + nSteps, 0.f, 0.f, nSteps);
    }

    void getE64(std::vector<double> &out) {
        get_E();
        out.assign(h_E64_.p, h_E64_.p + m_);
    }
    unsigned long long accepted() {
        if (!d_acc_.p) return 0;
        unsigned long long v = 0;
        SQ_CHECK(cudaMemcpyAsync(&v, d_acc_.p, sizeof(v), cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        return v;
    }
    void rngState(unsigned long long *s, uint32_t *step) const {
        *s = seed_;
        *step = step_;
    }
    // Checkpoint (no counterpart in the reference, whose cuRAND generator state
    // cannot be exported): the spins and resident local fields of every
    // trotter, the Philox key and step counter, and the steps since the last
    // field refresh.  Restored into a prepared annealer of the same problem,
    // algorithm and trotter count, the run continues bit for bit as the
    // annealer the checkpoint was taken from.
    void getCheckpoint(int8_t *q, float *F, unsigned long long *s, uint32_t *step, int *since) {
        throwErrorIfQNotSet();
        checkStatus();
        SQ_CHECK(cudaMemcpyAsync(q, d_q_.p, (size_t)m_ * N_, cudaMemcpyDeviceToHost, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(F, d_F_.p, sizeof(float) * m_ * N_, cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        *s = seed_;
        *step = step_;
        *since = stepsSinceRefresh_;
    }
    void setCheckpoint(const int8_t *q, const float *F, int m, int N, unsigned long long s, uint32_t step, int since) {
        throwErrorIfNotPrepared();
        throwErrorIf(m != m_ || N != N_, "%s, Shape does not match: (%d, %d) for an annealer of (%d, %d).", __func__, m,
                     N, m_, N_);
        throwErrorIf(since < 0 || since > refreshPeriod_, "%s, steps since the field refresh out of range.", __func__);
        check_values(q, (size_t)m_ * N_, true, __func__);
        SQ_CHECK(cudaMemcpyAsync(d_q_.p, q, (size_t)m_ * N_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_F_.p, F, sizeof(float) * m_ * N_, cudaMemcpyHostToDevice, st_.get()));
        st_.sync();
        seed_ = s;
        step_ = step;
        stepsSinceRefresh_ = since;
        setState(solRandSeedGiven);
        setState(solQSet);
    }
    void setTrace(bool on) { trace_ = on; }
    void getTrace(uint32_t *bits, int nwords) {
        throwErrorIf(!trace_ || !d_trace_.p, "trace is not enabled.");
        size_t n = std::min((size_t)nwords, d_trace_.n);
        SQ_CHECK(cudaMemcpyAsync(bits, d_trace_.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
    }
    int numTrotters() const { return m_; }
    int problemSize() const { return N_; }

private:
    void allocProblem() {
        // rows of J padded to 16 bytes (the one-CTA-per-trotter sweep reads them as float4)
        ldJ_ = (N_ + 3) & ~3;
        d_J_.ensure((size_t)N_ * ldJ_);
        SQ_CHECK(cudaMemsetAsync(d_J_.p, 0, sizeof(float) * N_ * ldJ_, st_.get()));
        d_h_.ensure(N_);
        d_c_.ensure(1);
        d_c64_.ensure(1);
        d_scratchN_.ensure(N_);
        d_status_.ensure(1);
        SQ_CHECK(cudaMemsetAsync(d_status_.p, 0, sizeof(int), st_.get()));
        // large instances refresh their fields on the tensor cores from digit planes of J
        if (sq103_dense_refresh_uses_tc(N_))
            d_digits_.ensure(sq103_tc_digits_bytes(N_, N_));
        else
            d_digits_.release();
    }

    void makeDigits() {
        if (d_digits_.p) SQ_CHECK(sq103_tc_make_digits(d_J_.p, ldJ_, N_, N_, 0, d_digits_.p, st_.get()));
    }

    void allocFP64() {
        d_J64_.ensure((size_t)N_ * N_);
        d_h64_.ensure(N_);
    }
    // the fp32 copies of an uploaded FP64 problem (h64, J64, c64), their digits, and c64 on the host
    void finishFP64() {
        round_problem(d_h64_.p, 1, N_, N_, d_h_.p, N_, st_.get());
        round_problem(d_J64_.p, N_, N_, N_, d_J_.p, ldJ_, st_.get());
        round_problem(d_c64_.p, 1, 1, 1, d_c_.p, 1, st_.get());
        makeDigits();
        SQ_CHECK(cudaMemcpyAsync(&c64h_, d_c64_.p, sizeof(double), cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        fp64_ = true;
    }
    void dropFP64() {
        fp64_ = false;
        d_J64_.release();
        d_h64_.release();
    }

    void upload(float *dst, int ldDst, const Matrix &M) {
        SQ_CHECK(cudaMemcpy2DAsync(dst, sizeof(float) * ldDst, M.data, sizeof(float) * M.stride,
                                   sizeof(float) * M.cols, M.rows, cudaMemcpyHostToDevice, st_.get()));
        st_.sync();  // M may be a temporary of the caller
    }

    void uploadQ() {
        SQ_CHECK(cudaMemcpyAsync(d_q_.p, h_q_.p, (size_t)m_ * N_, cudaMemcpyHostToDevice, st_.get()));
        refreshFields();
        st_.sync();
        setState(solQSet);
    }

    void refreshFields() {
        SQ_CHECK(sq103_dense_refresh(d_J_.p, ldJ_, d_digits_.p, d_Abf_.p, d_q_.p, d_F_.p, N_, m_, d_status_.p,
                                     st_.get()));
        stepsSinceRefresh_ = 0;
    }

    void runSteps(const float *dG, const float *dBeta, float G, float beta, int nSteps) {
        int algo = algo_ == sq::algoNaive ? kNaive : (algo_ == sq::algoSANaive ? kSANaive : kColoring);
        d_acc_.ensure(1);
        if (!accInit_) {
            d_status_.ensure(1);
            SQ_CHECK(cudaMemsetAsync(d_acc_.p, 0, sizeof(unsigned long long), st_.get()));
            SQ_CHECK(cudaMemsetAsync(d_status_.p, 0, sizeof(int), st_.get()));
            accInit_ = true;
        }
        size_t words = ((size_t)N_ * m_ + 31) / 32;
        if (trace_) {
            d_trace_.ensure(words * nSteps);
            SQ_CHECK(cudaMemsetAsync(d_trace_.p, 0, sizeof(uint32_t) * words * nSteps, st_.get()));
        }
        // periodic refresh of the resident fields bounds fp32 drift of the rank-1 updates
        int done = 0;
        while (done < nSteps) {
            int chunk = nSteps - done;
            if (refreshPeriod_ > 0) chunk = std::min(chunk, refreshPeriod_ - stepsSinceRefresh_);
            if (chunk <= 0) {
                refreshFields();
                continue;
            }
            sq103_dense_task t = {};
            t.J = d_J_.p;
            t.h = d_h_.p;
            t.q = d_q_.p;
            t.F = d_F_.p;
            t.trace = trace_ ? d_trace_.p + words * done : nullptr;
            t.accepted = d_acc_.p;
            t.G = dG ? dG + done : nullptr;
            t.beta = dBeta ? dBeta + done : nullptr;
            t.Gs = G;
            t.betas = beta;
            t.seed = seed_;
            t.step0 = step_;
            t.N = N_;
            t.m = m_;
            t.ldJ = ldJ_;
            t.algo = algo;
            t.nSteps = chunk;
            t.status = d_status_.p;
            t.flags = kernelFlags_;
            t.J64 = fp64_ ? d_J64_.p : nullptr;
            t.h64 = fp64_ ? d_h64_.p : nullptr;
            if (algo != kNaive) {
                unsigned long long wsb = sq103_dense_ws_bytes(N_, m_, chunk);
                d_ws_.ensure(wsb);
                t.ws = d_ws_.p;
                t.wsBytes = wsb;
            }
            SQ_CHECK(sq103_dense_anneal(&t, st_.get()));
            step_ += (uint32_t)chunk;
            stepsSinceRefresh_ += chunk;
            done += chunk;
        }
        clearState(solSolutionAvailable);
    }

    // a kernel that gave up a bounded wait leaves a status word: report it at the next sync
    void checkStatus() {
        if (!d_status_.p) return;
        int v = 0;
        SQ_CHECK(cudaMemcpyAsync(&v, d_status_.p, sizeof(int), cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        if (v != 0) {
            SQ_CHECK(cudaMemsetAsync(d_status_.p, 0, sizeof(int), st_.get()));
            sq::throwError("annealOneStep: device wait timed out (status %d); spins are not valid.", v);
        }
    }

    void syncBits() {
        size_t mn = (size_t)m_ * N_;
        h_q_.ensure(mn);
        checkStatus();
        SQ_CHECK(cudaMemcpyAsync(h_q_.p, d_q_.p, mn, cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        qlist_.clear();
        xlist_.clear();
        for (int y = 0; y < m_; ++y) {
            sq::BitSet q(N_);
            memcpy(q.data, h_q_.p + (size_t)y * N_, N_);
            xlist_.pushBack(sq::x_from_q(q));
            qlist_.pushBack(q);
        }
    }

    mutable Stream st_;
    DevBuf<float> d_J_, d_h_, d_c_, d_F_, d_E32_, d_sched_;
    DevBuf<unsigned char> d_digits_, d_Abf_;  // tensor-core refresh: digit planes of J, spins in bf16
    DevBuf<double> d_J64_, d_h64_;            // FP64 problem of a <double> annealer (J64 row stride N)
    double c64h_ = 0.;
    bool fp64_ = false;
    int ldJ_ = 0;  // row stride of J
    DevBuf<double> d_c64_, d_scratchN_, d_E64_, d_r_;
    DevBuf<int8_t> d_q_;
    DevBuf<unsigned long long> d_acc_;
    DevBuf<long long> d_ring_;
    DevBuf<uint32_t> d_trace_;
    HostBuf<double> h_E64_;
    HostBuf<int8_t> h_q_;
    Vector E_;
    sq::BitSetArray xlist_, qlist_;
    unsigned long long seed_ = 0;
    uint32_t step_ = 0;
    bool trace_ = false, accInit_ = false;
    int refreshPeriod_ = 8, stepsSinceRefresh_ = 0;
    int kernelFlags_ = 0;
    DevBuf<unsigned char> d_ws_;
    DevBuf<int> d_status_, d_flag_;

public:
    void setKernel(int flags) {
        throwErrorIf(flags < 0 || (flags & kFlagKernelMask) > 2 ||
                         (flags & ~(kFlagKernelMask | kFlagShortWaits | kFlagWithholdTrotter0)),
                     "kernel selector must be 0 (auto), 1 (one CTA) or 2 (CTA per trotter), optionally with the "
                     "test flags 16 (1 ms waits) and 32 (trotter 0 withholds its accept words).");
        kernelFlags_ = flags;
    }
};

// =================================================== bipartite annealer
class BipartiteAnnealer : public sq::cuda::BipartiteGraphAnnealer<float> {
public:
    typedef sq::MatrixType<float> Matrix;
    typedef sq::VectorType<float> Vector;

    BipartiteAnnealer() {
        m_ = -1;
        selectAlgorithm(sq::algoDefault);
    }

    void assignDevice(sq::cuda::Device &device) override {
        SQ_CHECK(cudaSetDevice(static_cast<DeviceImpl &>(device).devNo_));
    }

    // As the reference's CUDA annealer (CUDABipartiteGraphAnnealer.cu): coloring
    // for naive, sa_coloring for sa_naive.  The naive and sa_naive kernels stay
    // available at the kernel layer (sq103_bipartite_anneal with algo 0 / 2).
    sq::Algorithm selectAlgorithm(sq::Algorithm algo) override {
        switch (algo) {
        case sq::algoColoring:
        case sq::algoSAColoring:
            algo_ = algo;
            break;
        case sq::algoNaive:
            algo_ = sq::algoColoring;
            break;
        case sq::algoSANaive:
            algo_ = sq::algoSAColoring;
            break;
        default:
            selectDefaultAlgorithm(algo, sq::algoColoring, sq::algoSAColoring);
            break;
        }
        return algo_;
    }

    sq::Preferences getPreferences() const override {
        sq::Preferences prefs = sq::Annealer<float>::getPreferences();
        prefs.pushBack(sq::Preference(sq::pnDevice, "cuda"));
        return prefs;
    }

    void seed(unsigned long long s) override {
        seed_ = s;
        step_ = 0;
        setState(solRandSeedGiven);
    }

    // <double> problems: the FP64 couplings decide the flagged trials and give the
    // energies; the sweeps run on their fp32 rounding.  W is N1 x N0 row-major.
    void setQUBO64(const double *b0, const double *b1, const double *W, int N0, int N1, sq::OptimizeMethod om) {
        throwErrorIf(N0 <= 0 || N1 <= 0, "%s, Shape does not match.", __func__);
        clearState(solProblemSet);
        N0_ = N0;
        N1_ = N1;
        m_ = (N0_ + N1_) / 4;
        om_ = om;
        allocProblem();
        allocFP64();
        const double sgn = om == sq::optMaximize ? -1. : 1.;
        std::vector<double> v((size_t)N0 * N1 + N0 + N1);
        for (size_t i = 0; i < (size_t)N0 * N1; ++i) v[i] = sgn * W[i];
        for (int i = 0; i < N0; ++i) v[(size_t)N0 * N1 + i] = sgn * b0[i];
        for (int i = 0; i < N1; ++i) v[(size_t)N0 * N1 + N0 + i] = sgn * b1[i];
        DevBuf<double> dv, scr;
        dv.ensure(v.size());
        scr.ensure((size_t)N0 + 2 * N1);
        SQ_CHECK(cudaMemcpyAsync(dv.p, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(sq103_bipartite_hamiltonian64(dv.p + (size_t)N0 * N1, dv.p + (size_t)N0 * N1 + N0, dv.p, N0, N1,
                                               d_h0_64_.p, d_h1_64_.p, d_J64_.p, d_c64_.p, scr.p, st_.get()));
        finishFP64();
        setState(solProblemSet);
    }

    void setHamiltonian64(const double *h0, const double *h1, const double *J, double c, int N0, int N1) {
        throwErrorIf(N0 <= 0 || N1 <= 0, "%s, Shape does not match.", __func__);
        clearState(solProblemSet);
        N0_ = N0;
        N1_ = N1;
        m_ = (N0_ + N1_) / 4;
        om_ = sq::optMinimize;
        allocProblem();
        allocFP64();
        SQ_CHECK(cudaMemcpyAsync(d_h0_64_.p, h0, sizeof(double) * N0_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_h1_64_.p, h1, sizeof(double) * N1_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_J64_.p, J, sizeof(double) * N0_ * N1_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_c64_.p, &c, sizeof(double), cudaMemcpyHostToDevice, st_.get()));
        finishFP64();
        setState(solProblemSet);
    }

    void getHamiltonian64(double *h0, double *h1, double *J, double *c) {
        throwErrorIfProblemNotSet();
        throwErrorIf(!fp64_, "%s, the problem is not a double-precision one.", __func__);
        SQ_CHECK(cudaMemcpyAsync(h0, d_h0_64_.p, sizeof(double) * N0_, cudaMemcpyDeviceToHost, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(h1, d_h1_64_.p, sizeof(double) * N1_, cudaMemcpyDeviceToHost, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(J, d_J64_.p, sizeof(double) * N0_ * N1_, cudaMemcpyDeviceToHost, st_.get()));
        *c = c64h_;
        st_.sync();
    }
    bool isFP64() const { return fp64_; }

    double getSystemE64(double G, double beta) {
        calculate_E();
        double E = 0.;
        for (int y = 0; y < m_; ++y) E += h_E64_.p[y];
        E /= m_;
        if (sq::isSQAAlgorithm(algo_)) {
            d_ring_.ensure(2);
            SQ_CHECK(sq103_ring_dot(d_q0_.p, N0_, m_, d_ring_.p, st_.get()));
            SQ_CHECK(sq103_ring_dot(d_q1_.p, N1_, m_, d_ring_.p + 1, st_.get()));
            long long ring[2] = {0, 0};
            SQ_CHECK(cudaMemcpyAsync(ring, d_ring_.p, sizeof(ring), cudaMemcpyDeviceToHost, st_.get()));
            st_.sync();
            E -= (double)(ring[0] + ring[1]) * 0.5 / beta * std::log(std::tanh(G * beta / (double)m_));
        }
        return om_ == sq::optMaximize ? -E : E;
    }

    void setQUBO(const Vector &b0, const Vector &b1, const Matrix &W, sq::OptimizeMethod om) override {
        throwErrorIf(W.cols != b0.size || W.rows != b1.size, "%s, Shape does not match.", __func__);
        clearState(solProblemSet);
        N0_ = b0.size;
        N1_ = b1.size;
        m_ = (N0_ + N1_) / 4;
        om_ = om;
        allocProblem();
        DevBuf<float> db0, db1, dW;
        db0.ensure(N0_);
        db1.ensure(N1_);
        dW.ensure((size_t)N0_ * N1_);
        SQ_CHECK(cudaMemcpyAsync(db0.p, b0.data, sizeof(float) * N0_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(db1.p, b1.data, sizeof(float) * N1_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpy2DAsync(dW.p, sizeof(float) * N0_, W.data, sizeof(float) * W.stride, sizeof(float) * N0_, N1_,
                                   cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(sq103_bipartite_hamiltonian(db0.p, db1.p, dW.p, N0_, N1_, om == sq::optMaximize, d_h0_.p, d_h1_.p,
                                             d_J_.p, d_c_.p, d_c64_.p, d_scratch_.p, st_.get()));
        makeDigits();
        st_.sync();
        dropFP64();
        setState(solProblemSet);
    }

    void setHamiltonian(const Vector &h0, const Vector &h1, const Matrix &J, float c) override {
        throwErrorIf(J.cols != h0.size || J.rows != h1.size, "%s, Shape does not match.", __func__);
        clearState(solProblemSet);
        N0_ = h0.size;
        N1_ = h1.size;
        m_ = (N0_ + N1_) / 4;
        om_ = sq::optMinimize;
        allocProblem();
        double c64 = c;
        SQ_CHECK(cudaMemcpyAsync(d_h0_.p, h0.data, sizeof(float) * N0_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_h1_.p, h1.data, sizeof(float) * N1_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpy2DAsync(d_J_.p, sizeof(float) * N0_, J.data, sizeof(float) * J.stride, sizeof(float) * N0_,
                                   N1_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_c_.p, &c, sizeof(float), cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_c64_.p, &c64, sizeof(double), cudaMemcpyHostToDevice, st_.get()));
        makeDigits();
        st_.sync();
        dropFP64();
        setState(solProblemSet);
    }

    void getHamiltonian(Vector *h0, Vector *h1, Matrix *J, float *c) const override {
        throwErrorIfProblemNotSet();
        h0->resize(N0_);
        h1->resize(N1_);
        J->resize(N1_, N0_);
        SQ_CHECK(cudaMemcpyAsync(h0->data, d_h0_.p, sizeof(float) * N0_, cudaMemcpyDeviceToHost, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(h1->data, d_h1_.p, sizeof(float) * N1_, cudaMemcpyDeviceToHost, st_.get()));
        SQ_CHECK(cudaMemcpy2DAsync(J->data, sizeof(float) * J->stride, d_J_.p, sizeof(float) * N0_, sizeof(float) * N0_,
                                   N1_, cudaMemcpyDeviceToHost, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(c, d_c_.p, sizeof(float), cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
    }

    void prepare() override {
        throwErrorIfProblemNotSet();
        throwErrorIf(m_ <= 0, "# trotters must be a positive integer.");
        if (!isRandSeedGiven()) seed(time_seed());
        setState(solRandSeedGiven);
        clearState(solPrepared);
        if (m_ == 1) selectDefaultSAAlgorithm(algo_, sq::algoSAColoring);
        d_q0_.ensure((size_t)m_ * N0_);
        d_q1_.ensure((size_t)m_ * N1_);
        d_F0_.ensure((size_t)m_ * N0_);
        d_F1_.ensure((size_t)m_ * N1_);
        if (useTc()) d_Abf_.ensure(sq103_tc_spins_bytes(m_, std::max(N0_, N1_)));
        d_E64_.ensure(m_);
        h_E64_.ensure(m_);
        h_q0_.ensure((size_t)m_ * N0_);
        h_q1_.ensure((size_t)m_ * N1_);
        E_.resize(m_);
        setState(solPrepared);
    }

    void randomizeSpin() override {
        throwErrorIfNotPrepared();
        uint32_t step = step_++;
        SQ_CHECK(sq103_randomize_spins(d_q0_.p, N0_, m_, seed_, step, 0, st_.get()));
        SQ_CHECK(sq103_randomize_spins(d_q1_.p, N1_, m_, seed_, step, 1, st_.get()));
        setState(solQSet);
    }

    void set_q(const sq::BitSetPair &qp) override {
        throwErrorIfNotPrepared();
        throwErrorIf(qp.bits0.size != N0_, "Dimension of q0, %d,  should be equal to N0, %d.", qp.bits0.size, N0_);
        throwErrorIf(qp.bits1.size != N1_, "Dimension of q1, %d,  should be equal to N1, %d.", qp.bits1.size, N1_);
        for (int y = 0; y < m_; ++y) {
            memcpy(h_q0_.p + (size_t)y * N0_, qp.bits0.data, N0_);
            memcpy(h_q1_.p + (size_t)y * N1_, qp.bits1.data, N1_);
        }
        uploadQ();
    }

    void set_qset(const sq::BitSetPairArray &qs) override {
        throwErrorIfProblemNotSet();
        throwErrorIf(qs.size() <= 0, "%s, empty q set.", __func__);
        for (int i = 0; i < qs.size(); ++i)
            throwErrorIf(qs[i].bits0.size != N0_ || qs[i].bits1.size != N1_, "%s, Shape does not match.", __func__);
        m_ = qs.size();
        prepare();
        for (int y = 0; y < m_; ++y) {
            memcpy(h_q0_.p + (size_t)y * N0_, qs[y].bits0.data, N0_);
            memcpy(h_q1_.p + (size_t)y * N1_, qs[y].bits1.data, N1_);
        }
        uploadQ();
    }

    const sq::BitSetPairArray &get_q() const override {
        if (!isSolutionAvailable()) const_cast<BipartiteAnnealer *>(this)->makeSolution();
        return qlist_;
    }
    const sq::BitSetPairArray &get_x() const override {
        if (!isSolutionAvailable()) const_cast<BipartiteAnnealer *>(this)->makeSolution();
        return xlist_;
    }
    const Vector &get_E() const override {
        if (!isEAvailable()) const_cast<BipartiteAnnealer *>(this)->calculate_E();
        return E_;
    }

    void calculate_E() override {
        throwErrorIfQNotSet();
        d_r_.ensure((size_t)m_ * N1_);
        if (fp64_)
            SQ_CHECK(sq103_bipartite_energy64(d_J64_.p, d_h0_64_.p, d_h1_64_.p, c64h_, d_q0_.p, d_q1_.p, N0_, N1_, m_,
                                              om_ == sq::optMaximize, d_E64_.p, st_.get()));
        else
            SQ_CHECK(sq103_bipartite_energy(d_J_.p, d_h0_.p, d_h1_.p, d_c64_.p, d_q0_.p, d_q1_.p, N0_, N1_, m_,
                                            om_ == sq::optMaximize, d_r_.p, d_E64_.p, nullptr, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(h_E64_.p, d_E64_.p, sizeof(double) * m_, cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        E_.resize(m_);
        for (int y = 0; y < m_; ++y) E_(y) = (float)h_E64_.p[y];
        setState(solEAvailable);
    }

    void makeSolution() override {
        throwErrorIfNotPrepared();
        throwErrorIfQNotSet();
        syncBits();
        setState(solSolutionAvailable);
        calculate_E();
    }

    float getSystemE(float G, float beta) const override {
        auto self = const_cast<BipartiteAnnealer *>(this);
        self->calculate_E();
        double E = 0.;
        for (int y = 0; y < m_; ++y) E += E_(y);
        E /= m_;
        if (sq::isSQAAlgorithm(algo_)) {
            self->d_ring_.ensure(2);
            SQ_CHECK(sq103_ring_dot(d_q0_.p, N0_, m_, self->d_ring_.p, st_.get()));
            SQ_CHECK(sq103_ring_dot(d_q1_.p, N1_, m_, self->d_ring_.p + 1, st_.get()));
            long long ring[2] = {0, 0};
            SQ_CHECK(cudaMemcpyAsync(ring, d_ring_.p, sizeof(ring), cudaMemcpyDeviceToHost, st_.get()));
            self->st_.sync();
            float coef = 0.5f / beta * std::log(std::tanh(G * beta / (float)m_));
            E -= (double)(ring[0] + ring[1]) * coef;
        }
        if (om_ == sq::optMaximize) E = -E;
        return (float)E;
    }

    void annealOneStep(float G, float beta) override {
        throwErrorIfNotPrepared();
        throwErrorIfQNotSet();
        runSteps(nullptr, nullptr, G, beta, 1);
    }

    void anneal(const float *G, const float *beta, int nSteps) {
        throwErrorIfNotPrepared();
        throwErrorIfQNotSet();
        if (nSteps <= 0) return;
        d_sched_.ensure(2 * (size_t)nSteps);
        SQ_CHECK(cudaMemcpyAsync(d_sched_.p, G, sizeof(float) * nSteps, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_sched_.p + nSteps, beta, sizeof(float) * nSteps, cudaMemcpyHostToDevice, st_.get()));
        runSteps(d_sched_.p, d_sched_.p + nSteps, 0.f, 0.f, nSteps);
    }

    void getE64(std::vector<double> &out) {
        get_E();
        out.assign(h_E64_.p, h_E64_.p + m_);
    }
    unsigned long long accepted() {
        if (!d_acc_.p) return 0;
        unsigned long long v = 0;
        SQ_CHECK(cudaMemcpyAsync(&v, d_acc_.p, sizeof(v), cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        return v;
    }
    void rngState(unsigned long long *s, uint32_t *step) const {
        *s = seed_;
        *step = step_;
    }
    // Checkpoint: the spins of every trotter and the Philox key and step
    // counter (the fields are recomputed from the spins every half step, so
    // nothing else carries over).  Restored into a prepared annealer of the same
    // problem, algorithm and trotter count, the run continues bit for bit.
    void getCheckpoint(int8_t *q0, int8_t *q1, unsigned long long *s, uint32_t *step) {
        throwErrorIfQNotSet();
        SQ_CHECK(cudaMemcpyAsync(q0, d_q0_.p, (size_t)m_ * N0_, cudaMemcpyDeviceToHost, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(q1, d_q1_.p, (size_t)m_ * N1_, cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        *s = seed_;
        *step = step_;
    }
    void setCheckpoint(const int8_t *q0, const int8_t *q1, int m, int N0, int N1, unsigned long long s,
                       uint32_t step) {
        throwErrorIfNotPrepared();
        throwErrorIf(m != m_ || N0 != N0_ || N1 != N1_, "%s, Shape does not match.", __func__);
        check_values(q0, (size_t)m_ * N0_, true, __func__);
        check_values(q1, (size_t)m_ * N1_, true, __func__);
        SQ_CHECK(cudaMemcpyAsync(d_q0_.p, q0, (size_t)m_ * N0_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_q1_.p, q1, (size_t)m_ * N1_, cudaMemcpyHostToDevice, st_.get()));
        st_.sync();
        seed_ = s;
        step_ = step;
        setState(solRandSeedGiven);
        setState(solQSet);
    }
    void setTrace(bool on) { trace_ = on; }
    void getTrace(uint32_t *bits, int nwords) {
        throwErrorIf(!trace_ || !d_trace_.p, "trace is not enabled.");
        size_t n = std::min((size_t)nwords, d_trace_.n);
        SQ_CHECK(cudaMemcpyAsync(bits, d_trace_.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
    }
    int numTrotters() const { return m_; }

private:
    void allocProblem() {
        d_J_.ensure((size_t)N0_ * N1_);
        d_h0_.ensure(N0_);
        d_h1_.ensure(N1_);
        d_c_.ensure(1);
        d_c64_.ensure(1);
        d_scratch_.ensure(N0_ + N1_);
        d_status_.ensure(1);
        SQ_CHECK(cudaMemsetAsync(d_status_.p, 0, sizeof(int), st_.get()));
        // large problems may compute the half-step fields on the tensor cores from
        // digit planes of J (for F1) and of J^T (for F0): made with the problem, used
        // when the trotter count also allows (sq103_bipartite_refresh_uses_tc)
        if ((long long)N0_ * N1_ >= (1ll << 20)) {
            d_digits1_.ensure(sq103_tc_digits_bytes(N1_, N0_));
            d_digits0_.ensure(sq103_tc_digits_bytes(N0_, N1_));
        } else {
            d_digits1_.release();
            d_digits0_.release();
        }
    }

    bool useTc() const { return d_digits1_.p && sq103_bipartite_refresh_uses_tc(N0_, N1_, m_); }

    void makeDigits() {
        if (!d_digits1_.p) return;
        SQ_CHECK(sq103_tc_make_digits(d_J_.p, N0_, N1_, N0_, 0, d_digits1_.p, st_.get()));
        SQ_CHECK(sq103_tc_make_digits(d_J_.p, N0_, N0_, N1_, 1, d_digits0_.p, st_.get()));
    }

    void allocFP64() {
        d_J64_.ensure((size_t)N0_ * N1_);
        d_h0_64_.ensure(N0_);
        d_h1_64_.ensure(N1_);
    }
    void finishFP64() {
        round_problem(d_h0_64_.p, 1, N0_, N0_, d_h0_.p, N0_, st_.get());
        round_problem(d_h1_64_.p, 1, N1_, N1_, d_h1_.p, N1_, st_.get());
        round_problem(d_J64_.p, N1_, N0_, N0_, d_J_.p, N0_, st_.get());
        round_problem(d_c64_.p, 1, 1, 1, d_c_.p, 1, st_.get());
        makeDigits();
        SQ_CHECK(cudaMemcpyAsync(&c64h_, d_c64_.p, sizeof(double), cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        fp64_ = true;
    }
    void dropFP64() {
        fp64_ = false;
        d_J64_.release();
        d_h0_64_.release();
        d_h1_64_.release();
    }

    void uploadQ() {
        SQ_CHECK(cudaMemcpyAsync(d_q0_.p, h_q0_.p, (size_t)m_ * N0_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_q1_.p, h_q1_.p, (size_t)m_ * N1_, cudaMemcpyHostToDevice, st_.get()));
        st_.sync();
        setState(solQSet);
    }

    void runSteps(const float *dG, const float *dBeta, float G, float beta, int nSteps) {
        int algo = algo_ == sq::algoNaive ? kNaive
                   : algo_ == sq::algoSANaive ? kSANaive
                   : algo_ == sq::algoSAColoring ? kSAColoring
                                                  : kColoring;
        d_acc_.ensure(1);
        if (!accInit_) {
            SQ_CHECK(cudaMemsetAsync(d_acc_.p, 0, sizeof(unsigned long long), st_.get()));
            accInit_ = true;
        }
        size_t perStep = (size_t)m_ * (N0_ + N1_);
        if (algo == kNaive) perStep = (size_t)(N0_ + N1_) * m_;
        if (algo == kSANaive) perStep = (size_t)(N0_ + N1_) * m_ * m_;
        size_t words = (perStep + 31) / 32;
        if (trace_) {
            d_trace_.ensure(words * nSteps);
            SQ_CHECK(cudaMemsetAsync(d_trace_.p, 0, sizeof(uint32_t) * words * nSteps, st_.get()));
        }
        sq103_bipartite_task t = {};
        t.J = d_J_.p;
        t.h0 = d_h0_.p;
        t.h1 = d_h1_.p;
        t.q0 = d_q0_.p;
        t.q1 = d_q1_.p;
        t.F0 = d_F0_.p;
        t.F1 = d_F1_.p;
        t.trace = trace_ ? d_trace_.p : nullptr;
        t.accepted = d_acc_.p;
        t.G = dG;
        t.beta = dBeta;
        t.Gs = G;
        t.betas = beta;
        t.seed = seed_;
        t.step0 = step_;
        t.N0 = N0_;
        t.N1 = N1_;
        t.m = m_;
        t.algo = algo;
        t.nSteps = nSteps;
        t.J64 = fp64_ ? d_J64_.p : nullptr;
        t.h0_64 = fp64_ ? d_h0_64_.p : nullptr;
        t.h1_64 = fp64_ ? d_h1_64_.p : nullptr;
        const bool tc = useTc();
        t.digits1 = tc ? d_digits1_.p : nullptr;
        t.digits0 = tc ? d_digits0_.p : nullptr;
        t.spinsBf16 = tc ? d_Abf_.p : nullptr;
        t.status = d_status_.p;
        SQ_CHECK(sq103_bipartite_anneal(&t, st_.get()));
        step_ += (uint32_t)nSteps;
        clearState(solSolutionAvailable);
    }

    void syncBits() {
        SQ_CHECK(cudaMemcpyAsync(h_q0_.p, d_q0_.p, (size_t)m_ * N0_, cudaMemcpyDeviceToHost, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(h_q1_.p, d_q1_.p, (size_t)m_ * N1_, cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
        qlist_.clear();
        xlist_.clear();
        for (int y = 0; y < m_; ++y) {
            sq::BitSet q0(N0_), q1(N1_);
            memcpy(q0.data, h_q0_.p + (size_t)y * N0_, N0_);
            memcpy(q1.data, h_q1_.p + (size_t)y * N1_, N1_);
            xlist_.pushBack(sq::BitSetPair(sq::x_from_q(q0), sq::x_from_q(q1)));
            qlist_.pushBack(sq::BitSetPair(q0, q1));
        }
    }

    mutable Stream st_;
    DevBuf<float> d_J_, d_h0_, d_h1_, d_c_, d_F0_, d_F1_, d_sched_;
    DevBuf<double> d_c64_, d_scratch_, d_E64_, d_r_;
    DevBuf<double> d_J64_, d_h0_64_, d_h1_64_;        // FP64 problem of a <double> annealer
    DevBuf<unsigned char> d_digits1_, d_digits0_, d_Abf_;  // tensor-core half-step fields
    DevBuf<int> d_status_;
    DevBuf<int8_t> d_q0_, d_q1_;
    DevBuf<unsigned long long> d_acc_;
    DevBuf<long long> d_ring_;
    DevBuf<uint32_t> d_trace_;
    HostBuf<double> h_E64_;
    HostBuf<int8_t> h_q0_, h_q1_;
    Vector E_;
    sq::BitSetPairArray xlist_, qlist_;
    unsigned long long seed_ = 0;
    uint32_t step_ = 0;
    double c64h_ = 0.;
    bool fp64_ = false;
    bool trace_ = false, accInit_ = false;
};

// ============================================== <double> annealers
// sq::cuda::{Dense,Bipartite}GraphAnnealer<double> (the reference instantiates
// both, CUDADenseGraphAnnealer.cu:607-608, CUDABipartiteGraphAnnealer.cu:647-648).
// A float annealer carries the FP64 problem and does the work: its sweeps run on
// the fp32 rounding of the couplings, every trial they flag is decided from the
// FP64 couplings, and the energies are summed from them in FP64.  G and beta are
// taken in fp32, the schedule's precision in every kernel.
static sq::Preferences as_double_prefs(sq::Preferences prefs) {
    for (int i = 0; i < (int)prefs.size(); ++i)
        if (prefs[i].name == sq::pnPrecision) prefs[i] = sq::Preference(sq::pnPrecision, "double");
    return prefs;
}

class DenseAnnealer64 : public sq::cuda::DenseGraphAnnealer<double> {
public:
    typedef sq::MatrixType<double> Matrix;
    typedef sq::VectorType<double> Vector;

    DenseAnnealer &inner() { return f_; }

    void assignDevice(sq::cuda::Device &device) override { f_.assignDevice(device); }
    sq::Algorithm selectAlgorithm(sq::Algorithm algo) override { return f_.selectAlgorithm(algo); }
    sq::Algorithm getAlgorithm() const override { return f_.getAlgorithm(); }
    sq::Preferences getPreferences() const override { return as_double_prefs(f_.getPreferences()); }
    void setPreference(const sq::Preference &pref) override { f_.setPreference(pref); }
    void seed(unsigned long long s) override { f_.seed(s); }

    void setQUBO(const Matrix &W, sq::OptimizeMethod om) override {
        throwErrorIf(W.rows != W.cols, "%s, W is not a sqare matrix.", __func__);
        std::vector<double> d = dense_copy(W);
        f_.setQUBO64(d.data(), W.rows, om);
        N_ = W.rows;
    }
    void setHamiltonian(const Vector &h, const Matrix &J, double c) override {
        throwErrorIf(J.rows != J.cols, "%s, J is not a sqare matrix.", __func__);
        throwErrorIf(h.size != J.cols, "%s, Shape does not match.", __func__);
        std::vector<double> d = dense_copy(J);
        f_.setHamiltonian64(h.data, d.data(), c, J.rows);
        N_ = J.rows;
    }
    void getHamiltonian(Vector *h, Matrix *J, double *c) const override {
        h->resize(N_);
        J->resize(N_, N_);
        std::vector<double> d((size_t)N_ * N_);
        f_.getHamiltonian64(h->data, d.data(), c);
        for (int i = 0; i < N_; ++i) memcpy(&(*J)(i, 0), d.data() + (size_t)i * N_, sizeof(double) * N_);
    }
    void prepare() override { f_.prepare(); }
    void randomizeSpin() override { f_.randomizeSpin(); }
    void set_q(const sq::BitSet &q) override { f_.set_q(q); }
    void set_qset(const sq::BitSetArray &q) override { f_.set_qset(q); }
    const sq::BitSetArray &get_q() const override { return f_.get_q(); }
    const sq::BitSetArray &get_x() const override { return f_.get_x(); }
    void annealOneStep(double G, double beta) override { f_.annealOneStep((float)G, (float)beta); }
    void calculate_E() override { f_.calculate_E(); }
    void makeSolution() override { f_.makeSolution(); }
    double getSystemE(double G, double beta) const override { return f_.getSystemE64(G, beta); }
    const Vector &get_E() const override {
        std::vector<double> e;
        f_.getE64(e);
        E_.resize((sq::SizeType)e.size());
        for (size_t i = 0; i < e.size(); ++i) E_((sq::IdxType)i) = e[i];
        return E_;
    }

private:
    mutable DenseAnnealer f_;
    mutable Vector E_;
};

class BipartiteAnnealer64 : public sq::cuda::BipartiteGraphAnnealer<double> {
public:
    typedef sq::MatrixType<double> Matrix;
    typedef sq::VectorType<double> Vector;

    BipartiteAnnealer &inner() { return f_; }

    void assignDevice(sq::cuda::Device &device) override { f_.assignDevice(device); }
    sq::Algorithm selectAlgorithm(sq::Algorithm algo) override { return f_.selectAlgorithm(algo); }
    sq::Algorithm getAlgorithm() const override { return f_.getAlgorithm(); }
    sq::Preferences getPreferences() const override { return as_double_prefs(f_.getPreferences()); }
    void setPreference(const sq::Preference &pref) override { f_.setPreference(pref); }
    void seed(unsigned long long s) override { f_.seed(s); }

    void setQUBO(const Vector &b0, const Vector &b1, const Matrix &W, sq::OptimizeMethod om) override {
        throwErrorIf(W.cols != b0.size || W.rows != b1.size, "%s, Shape does not match.", __func__);
        std::vector<double> d = dense_copy(W);
        f_.setQUBO64(b0.data, b1.data, d.data(), b0.size, b1.size, om);
        N0_ = b0.size;
        N1_ = b1.size;
    }
    void setHamiltonian(const Vector &h0, const Vector &h1, const Matrix &J, double c) override {
        throwErrorIf(J.cols != h0.size || J.rows != h1.size, "%s, Shape does not match.", __func__);
        std::vector<double> d = dense_copy(J);
        f_.setHamiltonian64(h0.data, h1.data, d.data(), c, h0.size, h1.size);
        N0_ = h0.size;
        N1_ = h1.size;
    }
    void getHamiltonian(Vector *h0, Vector *h1, Matrix *J, double *c) const override {
        h0->resize(N0_);
        h1->resize(N1_);
        J->resize(N1_, N0_);
        std::vector<double> d((size_t)N0_ * N1_);
        f_.getHamiltonian64(h0->data, h1->data, d.data(), c);
        for (int i = 0; i < N1_; ++i) memcpy(&(*J)(i, 0), d.data() + (size_t)i * N0_, sizeof(double) * N0_);
    }
    void prepare() override { f_.prepare(); }
    void randomizeSpin() override { f_.randomizeSpin(); }
    void set_q(const sq::BitSetPair &q) override { f_.set_q(q); }
    void set_qset(const sq::BitSetPairArray &q) override { f_.set_qset(q); }
    const sq::BitSetPairArray &get_q() const override { return f_.get_q(); }
    const sq::BitSetPairArray &get_x() const override { return f_.get_x(); }
    void annealOneStep(double G, double beta) override { f_.annealOneStep((float)G, (float)beta); }
    void calculate_E() override { f_.calculate_E(); }
    void makeSolution() override { f_.makeSolution(); }
    double getSystemE(double G, double beta) const override { return f_.getSystemE64(G, beta); }
    const Vector &get_E() const override {
        std::vector<double> e;
        f_.getE64(e);
        E_.resize((sq::SizeType)e.size());
        for (size_t i = 0; i < e.size(); ++i) E_((sq::IdxType)i) = e[i];
        return E_;
    }

private:
    mutable BipartiteAnnealer f_;
    mutable Vector E_;
};

// ========================================================== BF searchers
// Running result of a brute-force search: exact FP64 minimum and the first
// `cap` minimisers in ascending order of the packed value.
template <class Key>
struct BfResult {
    double Emin = DBL_MAX;
    std::vector<Key> xs;
    void reset() {
        Emin = DBL_MAX;
        xs.clear();
    }
    // merge candidates (with FP64 energies) of a range that comes after every range merged so far
    void merge(const std::vector<Key> &cand, const std::vector<double> &E, size_t cap) {
        double m = DBL_MAX;
        for (double e : E) m = std::min(m, e);
        if (cand.empty()) return;
        std::vector<Key> sel;
        for (size_t i = 0; i < cand.size(); ++i)
            if (E[i] == m) sel.push_back(cand[i]);
        std::sort(sel.begin(), sel.end());
        if (m < Emin) {
            Emin = m;
            xs.clear();
        } else if (m > Emin) {
            return;
        }
        for (size_t i = 0; i < sel.size() && xs.size() < cap; ++i) xs.push_back(sel[i]);
    }
};

struct Pair {
    uint64_t x0, x1;
    bool operator<(const Pair &o) const { return x0 != o.x0 ? x0 < o.x0 : x1 < o.x1; }
};

// The <double> searchers screen every state with fp32 copies of the FP64
// couplings: a value outside the fp32 range would become inf, and inf - inf
// energies (NaN) fail every comparison, so true minimisers could be dropped
// before the FP64 re-evaluation.  Such problems are refused, as is a total
// magnitude at which some state's fp32 energy could overflow.
static void checkScreeningRange(const double *a, size_t na, const double *b = nullptr, size_t nb = 0,
                                const double *c = nullptr, size_t nc = 0) {
    double total = 0.;
    for (const auto &part : {std::make_pair(a, na), std::make_pair(b, nb), std::make_pair(c, nc)})
        for (size_t i = 0; i < part.second; ++i) {
            const double v = std::fabs(part.first[i]);
            throwErrorIf(!(v <= (double)FLT_MAX), "setQUBO: a coupling of magnitude %g is not finite in float32, "
                         "the precision of the screening pass.", part.first[i]);
            total += v;
        }
    throwErrorIf(!(total <= 1e37), "setQUBO: the couplings' total magnitude %g could overflow the float32 "
                 "energies of the screening pass.", total);
}

static float bf_slack(const std::vector<float> &vals) {
    bool integer = true;
    double s = 0.;
    for (float v : vals) {
        if (v != std::floor(v)) integer = false;
        s += std::fabs((double)v);
    }
    if (integer && s < 16777216.) return 0.f;
    return (float)(16. * s * 5.96e-8);
}

class DenseBFSearcher : public sq::cuda::DenseGraphBFSearcher<float> {
public:
    typedef sq::MatrixType<float> Matrix;
    typedef sq::VectorType<float> Vector;

    DenseBFSearcher() { tileSize_ = 1 << 18; }

    void assignDevice(sq::cuda::Device &device) override {
        SQ_CHECK(cudaSetDevice(static_cast<DeviceImpl &>(device).devNo_));
    }

    sq::Preferences getPreferences() const override {
        sq::Preferences prefs = sq::DenseGraphBFSearcher<float>::getPreferences();
        prefs.pushBack(sq::Preference(sq::pnDevice, "cuda"));
        return prefs;
    }

    void setQUBO(const Matrix &W, sq::OptimizeMethod om) override {
        throwErrorIf(W.rows != W.cols, "%s, W is not a sqare matrix.", __func__);
        throwErrorIf(!sq::isSymmetric(W), "%s, Matrix is not symmetric.", __func__);
        throwErrorIf(63 < W.rows, "N must be smaller than 64, N=%d.", W.rows);
        clearState(solProblemSet);
        N_ = W.rows;
        om_ = om;
        W_.assign((size_t)N_ * N_, 0.f);
        float sgn = om == sq::optMaximize ? -1.f : 1.f;
        for (int r = 0; r < N_; ++r)
            for (int c = 0; c < N_; ++c) W_[(size_t)r * N_ + c] = sgn * W(r, c);
        W64_.clear();
        extraSlack_ = 0.;
        setState(solProblemSet);
    }

    // The FP64 problem of the <double> searcher: the screening runs on the
    // fp32-rounded couplings, its slack widened by twice their total rounding
    // (a bound on how far any state's fp32 energy moves), and the candidates are
    // re-evaluated with the FP64 couplings.
    void setQUBO64(const double *W, int N, sq::OptimizeMethod om) {
        throwErrorIf(N <= 0, "%s, Shape does not match.", __func__);
        throwErrorIf(!sq::isSymmetric(W, (size_t)N, (size_t)N), "%s, Matrix is not symmetric.", __func__);
        throwErrorIf(63 < N, "N must be smaller than 64, N=%d.", N);
        checkScreeningRange(W, (size_t)N * N);
        clearState(solProblemSet);
        N_ = N;
        om_ = om;
        const double sgn = om == sq::optMaximize ? -1. : 1.;
        W64_.resize((size_t)N * N);
        W_.resize((size_t)N * N);
        double r = 0.;
        for (size_t i = 0; i < W64_.size(); ++i) {
            W64_[i] = sgn * W[i];
            W_[i] = (float)W64_[i];
            r += std::fabs(W64_[i] - (double)W_[i]);
        }
        extraSlack_ = 2. * r;
        setState(solProblemSet);
    }

    void prepare() override {
        throwErrorIfProblemNotSet();
        x_ = 0;
        xMax_ = 1ull << N_;
        if (xMax_ < (sq::PackedBitSet)tileSize_) tileSize_ = (sq::SizeType)xMax_;
        d_W_.ensure((size_t)N_ * N_);
        SQ_CHECK(cudaMemcpyAsync(d_W_.p, W_.data(), sizeof(float) * N_ * N_, cudaMemcpyHostToDevice, st_.get()));
        d_ws_.ensure(sq103_bf_workspace_bytes(N_));
        slack_ = bf_slack(W_);
        if (!W64_.empty()) {
            d_W64_.ensure((size_t)N_ * N_);
            SQ_CHECK(cudaMemcpyAsync(d_W64_.p, W64_.data(), sizeof(double) * N_ * N_, cudaMemcpyHostToDevice,
                                     st_.get()));
            slack_ = (float)((double)slack_ + extraSlack_ * (1. + 1e-6));  // rounded up past the cast
        }
        res_.reset();
        xList_.clear();
        st_.sync();
        setState(solPrepared);
    }

    bool searchRange(sq::PackedBitSet *curXEnd) override {
        throwErrorIfNotPrepared();
        clearState(solSolutionAvailable);
        uint64_t b = x_, e = std::min<uint64_t>(x_ + tileSize_, xMax_);
        if (b < e) runRange(b, e);
        x_ = e;
        if (curXEnd) *curXEnd = x_;
        return x_ == xMax_;
    }

    // whole-range fast path: same result as prepare() + searchRange() until done + makeSolution()
    void search() override {
        prepare();
        const uint64_t chunk = 1ull << 34;
        for (uint64_t b = 0; b < xMax_; b += chunk) runRange(b, std::min<uint64_t>(xMax_, b + chunk));
        x_ = xMax_;
        makeSolution();
    }

    void calculate_E() override {
        throwErrorIfNotPrepared();
        E_.resize(xList_.size() ? xList_.size() : 1);
        float E = (float)res_.Emin;
        if (res_.Emin == DBL_MAX) E = FLT_MAX;
        E_ = (om_ == sq::optMaximize) ? -E : E;
        setState(solEAvailable);
    }

    void makeSolution() override {
        throwErrorIfNotPrepared();
        xList_.clear();
        size_t n = std::min(res_.xs.size(), (size_t)tileSize_);
        for (size_t i = 0; i < n; ++i) {
            sq::BitSet bits;
            sq::unpackBitSet(&bits, res_.xs[i], N_);
            xList_.pushBack(bits);
        }
        setState(solSolutionAvailable);
        calculate_E();
    }

    const sq::BitSetArray &get_x() const override {
        if (!isSolutionAvailable()) const_cast<DenseBFSearcher *>(this)->makeSolution();
        return xList_;
    }
    const Vector &get_E() const override {
        if (!isEAvailable()) const_cast<DenseBFSearcher *>(this)->calculate_E();
        return E_;
    }
    double EminExact() const { return om_ == sq::optMaximize ? -res_.Emin : res_.Emin; }

    // one shard of a multi-GPU search: searches [b, e) after prepare() (ranges
    // of one searcher in ascending order), merged into the running result
    void searchSubrange(uint64_t b, uint64_t e) {
        throwErrorIfNotPrepared();
        throwErrorIf(b > e || e > xMax_, "range [%llu, %llu) is outside [0, 2^%d).", (unsigned long long)b,
                     (unsigned long long)e, N_);
        throwErrorIf(b < x_, "ranges must be searched in ascending order.");
        clearState(solSolutionAvailable);
        const uint64_t chunk = 1ull << 34;
        for (uint64_t c = b; c < e; c += chunk) runRange(c, std::min<uint64_t>(e, c + chunk));
        x_ = e;
    }

private:
    // one range in ascending order; splits itself when the candidates overflow
    void runRange(uint64_t b, uint64_t e) {
        int cap = (int)std::min<uint64_t>(std::max<uint64_t>((uint64_t)tileSize_, 1u << 16), 1u << 22);
        d_cand_.ensure(cap);
        int count = 0;
        float emin32 = 0.f;
        SQ_CHECK(sq103_dense_bf_range(d_W_.p, N_, b, e, slack_, d_ws_.p, d_cand_.p, cap, &count, &emin32, st_.get()));
        if (count > cap) {
            uint64_t mid = b + (e - b) / 2;
            runRange(b, mid);
            // with exact energies every candidate of a heavy tie equals Emin: stop once the list is full
            if (slack_ == 0.f && res_.xs.size() >= (size_t)tileSize_ && (double)emin32 >= res_.Emin) return;
            runRange(mid, e);
            return;
        }
        std::vector<uint64_t> cand(count);
        std::vector<double> E(count);
        if (count > 0) {
            d_E_.ensure(count);
            if (W64_.empty())
                SQ_CHECK(sq103_dense_bf_refine(d_W_.p, N_, d_cand_.p, count, d_E_.p, st_.get()));
            else
                SQ_CHECK(sq103_dense_bf_refine64(d_W64_.p, N_, d_cand_.p, count, d_E_.p, st_.get()));
            SQ_CHECK(cudaMemcpyAsync(cand.data(), d_cand_.p, sizeof(uint64_t) * count, cudaMemcpyDeviceToHost, st_.get()));
            SQ_CHECK(cudaMemcpyAsync(E.data(), d_E_.p, sizeof(double) * count, cudaMemcpyDeviceToHost, st_.get()));
            st_.sync();
        }
        res_.merge(cand, E, (size_t)tileSize_);
    }

    Stream st_;
    std::vector<float> W_;
    std::vector<double> W64_;  // the FP64 couplings of a <double> problem (empty otherwise)
    DevBuf<float> d_W_;
    DevBuf<double> d_W64_;
    DevBuf<unsigned char> d_ws_;
    DevBuf<uint64_t> d_cand_;
    DevBuf<double> d_E_;
    BfResult<uint64_t> res_;
    float slack_ = 0.f;
    double extraSlack_ = 0.;
    sq::BitSetArray xList_;
    Vector E_;
};

class BipartiteBFSearcher : public sq::cuda::BipartiteGraphBFSearcher<float> {
public:
    typedef sq::MatrixType<float> Matrix;
    typedef sq::VectorType<float> Vector;

    BipartiteBFSearcher() {
        tileSize0_ = 8192;
        tileSize1_ = 8192;
    }

    void assignDevice(sq::cuda::Device &device) override {
        SQ_CHECK(cudaSetDevice(static_cast<DeviceImpl &>(device).devNo_));
    }

    sq::Preferences getPreferences() const override {
        sq::Preferences prefs = sq::BipartiteGraphBFSearcher<float>::getPreferences();
        prefs.pushBack(sq::Preference(sq::pnDevice, "cuda"));
        return prefs;
    }

    void setQUBO(const Vector &b0, const Vector &b1, const Matrix &W, sq::OptimizeMethod om) override {
        throwErrorIf(W.cols != b0.size || W.rows != b1.size, "%s, Shape does not match.", __func__);
        throwErrorIf(63 < b0.size, "N0 must be smaller than 64, N0=%d.", b0.size);
        throwErrorIf(63 < b1.size, "N1 must be smaller than 64, N1=%d.", b1.size);
        clearState(solProblemSet);
        N0_ = b0.size;
        N1_ = b1.size;
        om_ = om;
        float sgn = om == sq::optMaximize ? -1.f : 1.f;
        b0_.resize(N0_);
        b1_.resize(N1_);
        W_.resize((size_t)N0_ * N1_);
        for (int j = 0; j < N0_; ++j) b0_[j] = sgn * b0(j);
        for (int i = 0; i < N1_; ++i) b1_[i] = sgn * b1(i);
        for (int i = 0; i < N1_; ++i)
            for (int j = 0; j < N0_; ++j) W_[(size_t)i * N0_ + j] = sgn * W(i, j);
        b064_.clear();
        b164_.clear();
        W64_.clear();
        extraSlack_ = 0.;
        setState(solProblemSet);
    }

    // The FP64 problem of the <double> searcher (W: N1 x N0): fp32-rounded
    // screening with the slack widened by twice the total rounding, FP64
    // re-evaluation of the candidates.
    void setQUBO64(const double *b0, const double *b1, const double *W, int N0, int N1, sq::OptimizeMethod om) {
        throwErrorIf(N0 <= 0 || N1 <= 0, "%s, Shape does not match.", __func__);
        throwErrorIf(63 < N0, "N0 must be smaller than 64, N0=%d.", N0);
        throwErrorIf(63 < N1, "N1 must be smaller than 64, N1=%d.", N1);
        checkScreeningRange(b0, N0, b1, N1, W, (size_t)N0 * N1);
        clearState(solProblemSet);
        N0_ = N0;
        N1_ = N1;
        om_ = om;
        const double sgn = om == sq::optMaximize ? -1. : 1.;
        double r = 0.;
        auto round = [&](const double *src, size_t n, std::vector<double> &v64, std::vector<float> &v32) {
            v64.resize(n);
            v32.resize(n);
            for (size_t i = 0; i < n; ++i) {
                v64[i] = sgn * src[i];
                v32[i] = (float)v64[i];
                r += std::fabs(v64[i] - (double)v32[i]);
            }
        };
        round(b0, N0, b064_, b0_);
        round(b1, N1, b164_, b1_);
        round(W, (size_t)N0 * N1, W64_, W_);
        extraSlack_ = 2. * r;
        setState(solProblemSet);
    }
    double EminExact() const { return om_ == sq::optMaximize ? -res_.Emin : res_.Emin; }

    void prepare() override {
        throwErrorIfProblemNotSet();
        x0_ = x1_ = 0;
        x0max_ = 1ull << N0_;
        x1max_ = 1ull << N1_;
        if (x0max_ < (sq::PackedBitSet)tileSize0_) tileSize0_ = (sq::SizeType)x0max_;
        if (x1max_ < (sq::PackedBitSet)tileSize1_) tileSize1_ = (sq::SizeType)x1max_;
        d_b0_.ensure(N0_);
        d_b1_.ensure(N1_);
        d_W_.ensure((size_t)N0_ * N1_);
        SQ_CHECK(cudaMemcpyAsync(d_b0_.p, b0_.data(), sizeof(float) * N0_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_b1_.p, b1_.data(), sizeof(float) * N1_, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(d_W_.p, W_.data(), sizeof(float) * N0_ * N1_, cudaMemcpyHostToDevice, st_.get()));
        d_ws_.ensure(sq103_bf_workspace_bytes(N0_ + N1_));
        std::vector<float> all(W_);
        all.insert(all.end(), b0_.begin(), b0_.end());
        all.insert(all.end(), b1_.begin(), b1_.end());
        slack_ = bf_slack(all);
        if (!W64_.empty()) {
            d_b064_.ensure(N0_);
            d_b164_.ensure(N1_);
            d_W64_.ensure((size_t)N0_ * N1_);
            SQ_CHECK(cudaMemcpyAsync(d_b064_.p, b064_.data(), sizeof(double) * N0_, cudaMemcpyHostToDevice, st_.get()));
            SQ_CHECK(cudaMemcpyAsync(d_b164_.p, b164_.data(), sizeof(double) * N1_, cudaMemcpyHostToDevice, st_.get()));
            SQ_CHECK(cudaMemcpyAsync(d_W64_.p, W64_.data(), sizeof(double) * N0_ * N1_, cudaMemcpyHostToDevice,
                                     st_.get()));
            slack_ = (float)((double)slack_ + extraSlack_ * (1. + 1e-6));  // rounded up past the cast
        }
        res_.reset();
        xList_.clear();
        st_.sync();
        setState(solPrepared);
    }

    // tiles advance x1 first, then x0 (CUDABipartiteGraphBFSearcher.cpp:168-211)
    bool searchRange(sq::PackedBitSet *curX0, sq::PackedBitSet *curX1) override {
        throwErrorIfNotPrepared();
        clearState(solSolutionAvailable);
        uint64_t b0 = x0_, e0 = std::min<uint64_t>(x0_ + tileSize0_, x0max_);
        uint64_t b1 = x1_, e1 = std::min<uint64_t>(x1_ + tileSize1_, x1max_);
        if (b0 < e0 && b1 < e1) runRange(b0, e0, b1, e1);
        x1_ = e1;
        if (x1_ == x1max_) {
            x1_ = 0;
            x0_ = std::min<uint64_t>(x0_ + tileSize0_, x0max_);
        }
        if (curX0) *curX0 = x0_;
        if (curX1) *curX1 = x1_;
        return x0_ == x0max_;
    }

    void search() override {
        prepare();
        runRange(0, x0max_, 0, x1max_);
        x0_ = x0max_;
        x1_ = 0;
        makeSolution();
    }

    void calculate_E() override {
        throwErrorIfNotPrepared();
        E_.resize(xList_.size() ? xList_.size() : 1);
        float E = res_.Emin == DBL_MAX ? FLT_MAX : (float)res_.Emin;
        E_ = (om_ == sq::optMaximize) ? -E : E;
        setState(solEAvailable);
    }

    void makeSolution() override {
        throwErrorIfNotPrepared();
        xList_.clear();
        // result order: ascending (x0, x1); at most tileSize0 + tileSize1 pairs
        // (the merge cap of CPUBipartiteGraphBFSearcher.cpp:117-151)
        std::vector<Pair> xs = res_.xs;
        std::sort(xs.begin(), xs.end());
        size_t n = std::min(xs.size(), (size_t)(tileSize0_ + tileSize1_));
        for (size_t i = 0; i < n; ++i) {
            sq::BitSet a, b;
            sq::unpackBitSet(&a, xs[i].x0, N0_);
            sq::unpackBitSet(&b, xs[i].x1, N1_);
            xList_.pushBack(sq::BitSetPair(a, b));
        }
        setState(solSolutionAvailable);
        calculate_E();
    }

    const sq::BitSetPairArray &get_x() const override {
        if (!isSolutionAvailable()) const_cast<BipartiteBFSearcher *>(this)->makeSolution();
        return xList_;
    }
    const Vector &get_E() const override {
        if (!isEAvailable()) const_cast<BipartiteBFSearcher *>(this)->calculate_E();
        return E_;
    }

private:
    void runRange(uint64_t b0, uint64_t e0, uint64_t b1, uint64_t e1) {
        int cap = 1 << 20;
        d_cand_.ensure(2 * (size_t)cap);
        int count = 0;
        float emin32 = 0.f;
        SQ_CHECK(sq103_bipartite_bf_range(d_b0_.p, d_b1_.p, d_W_.p, N0_, N1_, b0, e0, b1, e1, slack_, d_ws_.p,
                                          d_cand_.p, cap, &count, &emin32, st_.get()));
        if (count > cap) {
            // split the x1 range (or x0 when x1 is a single value)
            if (e1 - b1 > 1) {
                uint64_t mid = b1 + (e1 - b1) / 2;
                runRange(b0, e0, b1, mid);
                runRange(b0, e0, mid, e1);
            } else {
                uint64_t mid = b0 + (e0 - b0) / 2;
                runRange(b0, mid, b1, e1);
                runRange(mid, e0, b1, e1);
            }
            return;
        }
        std::vector<uint64_t> raw(2 * (size_t)count);
        std::vector<double> E(count);
        if (count > 0) {
            d_E_.ensure(count);
            if (W64_.empty())
                SQ_CHECK(sq103_bipartite_bf_refine(d_b0_.p, d_b1_.p, d_W_.p, N0_, N1_, d_cand_.p, count, d_E_.p,
                                                   st_.get()));
            else
                SQ_CHECK(sq103_bipartite_bf_refine64(d_b064_.p, d_b164_.p, d_W64_.p, N0_, N1_, d_cand_.p, count,
                                                     d_E_.p, st_.get()));
            SQ_CHECK(cudaMemcpyAsync(raw.data(), d_cand_.p, sizeof(uint64_t) * 2 * count, cudaMemcpyDeviceToHost, st_.get()));
            SQ_CHECK(cudaMemcpyAsync(E.data(), d_E_.p, sizeof(double) * count, cudaMemcpyDeviceToHost, st_.get()));
            st_.sync();
        }
        std::vector<Pair> cand(count);
        for (int i = 0; i < count; ++i) cand[i] = Pair{raw[2 * i], raw[2 * i + 1]};
        // ranges of one search are not visited in (x0, x1) order: keep all ties, cap at the end
        res_.merge(cand, E, (size_t)1 << 24);
    }

    Stream st_;
    std::vector<float> b0_, b1_, W_;
    std::vector<double> b064_, b164_, W64_;  // the FP64 problem of a <double> searcher (empty otherwise)
    DevBuf<float> d_b0_, d_b1_, d_W_;
    DevBuf<double> d_b064_, d_b164_, d_W64_;
    double extraSlack_ = 0.;
    DevBuf<unsigned char> d_ws_;
    DevBuf<uint64_t> d_cand_;
    DevBuf<double> d_E_;
    BfResult<Pair> res_;
    float slack_ = 0.f;
    sq::BitSetPairArray xList_;
    Vector E_;
};

// ---------------------------------------------- double-precision BF searchers
// The reference's <double> searchers (CUDADenseGraphBFSearcher<double>, ...):
// a float searcher carries the FP64 problem (setQUBO64) and does the work, so
// Emin and the argmin set are those of the FP64 couplings.  Preferences live
// in both objects; energies are returned as the FP64 minimum.
class DenseBFSearcher64 : public sq::cuda::DenseGraphBFSearcher<double> {
public:
    typedef sq::MatrixType<double> Matrix;
    typedef sq::VectorType<double> Vector;

    DenseBFSearcher64() { tileSize_ = 1 << 18; }
    DenseBFSearcher &inner() { return f_; }

    void assignDevice(sq::cuda::Device &device) override { f_.assignDevice(device); }
    sq::Preferences getPreferences() const override {
        sq::Preferences prefs = sq::DenseGraphBFSearcher<double>::getPreferences();
        prefs.pushBack(sq::Preference(sq::pnDevice, "cuda"));
        return prefs;
    }
    void setPreference(const sq::Preference &pref) override {
        f_.setPreference(pref);
        sq::DenseGraphBFSearcher<double>::setPreference(pref);
    }
    void setQUBO(const Matrix &W, sq::OptimizeMethod om) override {
        throwErrorIf(W.rows != W.cols, "%s, W is not a sqare matrix.", __func__);
        std::vector<double> d = dense_copy(W);
        setQUBO64(d.data(), W.rows, om);
    }
    void setQUBO64(const double *W, int N, sq::OptimizeMethod om) {
        f_.setQUBO64(W, N, om);
        N_ = N;
    }
    void prepare() override { f_.prepare(); }
    bool searchRange(sq::PackedBitSet *curXEnd) override { return f_.searchRange(curXEnd); }
    void search() override { f_.search(); }
    void calculate_E() override { f_.calculate_E(); }
    void makeSolution() override { f_.makeSolution(); }
    const sq::BitSetArray &get_x() const override { return f_.get_x(); }
    const Vector &get_E() const override {
        const int n = f_.get_E().size;
        E_.resize(n);
        for (int i = 0; i < n; ++i) E_(i) = f_.EminExact();
        return E_;
    }

private:
    mutable DenseBFSearcher f_;
    mutable Vector E_;
};

class BipartiteBFSearcher64 : public sq::cuda::BipartiteGraphBFSearcher<double> {
public:
    typedef sq::MatrixType<double> Matrix;
    typedef sq::VectorType<double> Vector;

    BipartiteBFSearcher64() {
        tileSize0_ = 8192;
        tileSize1_ = 8192;
    }
    BipartiteBFSearcher &inner() { return f_; }

    void assignDevice(sq::cuda::Device &device) override { f_.assignDevice(device); }
    sq::Preferences getPreferences() const override {
        sq::Preferences prefs = sq::BipartiteGraphBFSearcher<double>::getPreferences();
        prefs.pushBack(sq::Preference(sq::pnDevice, "cuda"));
        return prefs;
    }
    void setPreference(const sq::Preference &pref) override {
        f_.setPreference(pref);
        sq::BipartiteGraphBFSearcher<double>::setPreference(pref);
    }
    void setQUBO(const Vector &b0, const Vector &b1, const Matrix &W, sq::OptimizeMethod om) override {
        throwErrorIf(W.cols != b0.size || W.rows != b1.size, "%s, Shape does not match.", __func__);
        std::vector<double> d = dense_copy(W);
        setQUBO64(b0.data, b1.data, d.data(), b0.size, b1.size, om);
    }
    void setQUBO64(const double *b0, const double *b1, const double *W, int N0, int N1, sq::OptimizeMethod om) {
        f_.setQUBO64(b0, b1, W, N0, N1, om);
        N0_ = N0;
        N1_ = N1;
    }
    void prepare() override { f_.prepare(); }
    bool searchRange(sq::PackedBitSet *curX0, sq::PackedBitSet *curX1) override {
        return f_.searchRange(curX0, curX1);
    }
    void search() override { f_.search(); }
    void calculate_E() override { f_.calculate_E(); }
    void makeSolution() override { f_.makeSolution(); }
    const sq::BitSetPairArray &get_x() const override { return f_.get_x(); }
    const Vector &get_E() const override {
        const int n = f_.get_E().size;
        E_.resize(n);
        for (int i = 0; i < n; ++i) E_(i) = f_.EminExact();
        return E_;
    }

private:
    mutable BipartiteBFSearcher f_;
    mutable Vector E_;
};

// ===================================================== batched annealer
// Many independent dense instances annealed together: every annealOneStep of
// all of them is one persistent launch (sq103_dense_batch_launch) replayed
// from a CUDA graph.  Each instance follows exactly the rules of the
// single-instance annealer (same Philox stream for the same seed, same field
// refresh every kRefreshPeriod steps), so its result is bit-identical to
// annealing it alone.
class DenseBatch : public sq::NullBase {
public:
    static constexpr int kRefreshPeriod = 8;
    static constexpr int kPackMax = 8;           // instances per packed launch (16 measured slower on C4)
    static constexpr int kDefaultMultiMinN = 1024;

    // Instances of at least multiMinN_ spins (with m >= 2 that fit the device) run
    // on the one-CTA-per-trotter sweep in packed cooperative launches: its decider
    // takes 32 iterations per round trip, where the persistent one-CTA kernel
    // takes one per colour phase, and the serial chain of the largest instances
    // sets the batch's step time.  Both kernels give bit-identical results.
    struct Inst {
        int N, m, ldJ;  // J rows on a 16-byte stride (the one-CTA-per-trotter sweep reads them as float4)
        bool multi = false;
        unsigned long long seed;
        DevBuf<unsigned char> mem, ws;
        DevBuf<unsigned char> digits, Abf;  // tensor-core refresh (N >= 1024), as the single annealer
        unsigned long long wsBytes = 0;
        float *J, *h, *c32, *F;
        double *c64;
        int8_t *q;
        int *status;
    };

    ~DenseBatch() {
        if (graph_) cudaGraphExecDestroy(graph_);
        if (fork_) cudaEventDestroy(fork_);
        for (cudaEvent_t e : join_)
            if (e) cudaEventDestroy(e);
    }

    int add(const float *W, int N, int m, int optimize, unsigned long long seed) {
        throwErrorIf(prepared_, "instances must be added before prepare().");
        throwErrorIf(N <= 0 || m <= 0, "N and m must be positive.");
        throwErrorIf(!sqaod::isSymmetric(W, (size_t)N, (size_t)N), "%s, Matrix is not symmetric.", __func__);
        insts_.emplace_back(new Inst());
        Inst &in = *insts_.back();
        in.N = N;
        in.m = m;
        in.ldJ = (N + 3) & ~3;
        in.seed = seed;
        auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
        size_t oJ = 0, oh = oJ + al((size_t)N * in.ldJ * 4), oc = oh + al((size_t)N * 4), oc64 = oc + 256,
               oF = oc64 + 256, oq = oF + al((size_t)m * N * 4), total = oq + al((size_t)m * N);
        in.mem.ensure(total);
        unsigned char *b = in.mem.p;
        in.J = (float *)(b + oJ);
        in.h = (float *)(b + oh);
        in.c32 = (float *)(b + oc);
        in.c64 = (double *)(b + oc64);
        in.status = (int *)(b + oc64 + 8);
        in.F = (float *)(b + oF);
        in.q = (int8_t *)(b + oq);
        SQ_CHECK(cudaMemsetAsync(in.status, 0, sizeof(int), st_.get()));
        if (sq103_dense_refresh_uses_tc(N)) {
            in.digits.ensure(sq103_tc_digits_bytes(N, N));
            in.Abf.ensure(sq103_tc_spins_bytes(m, N));
        }
        dW_.ensure((size_t)N * N);
        scratch_.ensure(N);
        SQ_CHECK(cudaMemcpyAsync(dW_.p, W, sizeof(float) * N * N, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemsetAsync(in.J, 0, sizeof(float) * N * in.ldJ, st_.get()));  // zero row padding
        SQ_CHECK(sq103_dense_hamiltonian(dW_.p, N, N, optimize, in.h, in.J, in.ldJ, in.c32, in.c64, scratch_.p,
                                         st_.get()));
        if (in.digits.p) SQ_CHECK(sq103_tc_make_digits(in.J, in.ldJ, N, N, 0, in.digits.p, st_.get()));
        st_.sync();
        optimize_.push_back(optimize);
        return (int)insts_.size() - 1;
    }

    void setSchedule(const float *G, const float *beta, int nSteps) {
        throwErrorIf(nSteps <= 0, "schedule must have at least one step.");
        sched_.ensure(2 * (size_t)nSteps);
        SQ_CHECK(cudaMemcpyAsync(sched_.p, G, sizeof(float) * nSteps, cudaMemcpyHostToDevice, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(sched_.p + nSteps, beta, sizeof(float) * nSteps, cudaMemcpyHostToDevice, st_.get()));
        nSched_ = nSteps;
        st_.sync();
        prepared_ = false;
    }

    // randomize every instance (Philox step 0 of its seed), refresh fields, upload tasks
    void prepare() {
        throwErrorIf(insts_.empty(), "no instance added.");
        throwErrorIf(nSched_ <= 0, "set a schedule before prepare().");
        const int nAll = (int)insts_.size();
        std::vector<sq103_dense_task> tasks;
        std::vector<Inst *> smallInsts;
        multi_.clear();
        int maxN = 0, maxM = 0;
        for (int i = 0; i < nAll; ++i) {
            Inst &in = *insts_[i];
            SQ_CHECK(sq103_randomize_spins(in.q, in.N, in.m, in.seed, 0, 0, st_.get()));
            in.multi = multiMinN_ > 0 && in.N >= multiMinN_ && in.m >= 2 && sq103_dense_multicta_ok(in.N, in.m, kColoring);
            if (in.multi) {
                in.wsBytes = sq103_dense_ws_bytes(in.N, in.m, kRefreshPeriod);
                in.ws.ensure(in.wsBytes);
                multi_.push_back(&in);
                continue;
            }
            sq103_dense_task t = {};
            t.J = in.J;
            t.h = in.h;
            t.q = in.q;
            t.F = in.F;
            t.accepted = nullptr;
            t.G = sched_.p;
            t.beta = sched_.p + nSched_;
            t.seed = in.seed;
            t.step0 = 1;  // step 0 of the Philox counter is the randomisation
            t.N = in.N;
            t.m = in.m;
            t.ldJ = in.ldJ;
            t.algo = in.m == 1 ? kSANaive : kColoring;
            t.nSteps = nSched_;
            tasks.push_back(t);
            smallInsts.push_back(&in);
            maxN = std::max(maxN, in.N);
            maxM = std::max(maxM, in.m);
        }
        buildRefreshJobs();
        refreshAll();
        // packed launches take instances of similar size together
        std::stable_sort(multi_.begin(), multi_.end(), [](const Inst *a, const Inst *b) { return a->N < b->N; });
        // largest instances first: the queue then balances the tail
        const int n = (int)tasks.size();
        nSmall_ = n;
        std::vector<int> order(n);
        for (int i = 0; i < n; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            return (long long)smallInsts[a]->N * smallInsts[a]->m > (long long)smallInsts[b]->N * smallInsts[b]->m;
        });
        const int nAlloc = std::max(n, 1);
        dTasks_.ensure(nAlloc);
        dOrder_.ensure(nAlloc);
        dPos_.ensure(nAlloc);
        dQueue_.ensure(2);
        dStatus_.ensure(1);
        if (n > 0) {
            SQ_CHECK(cudaMemcpyAsync(dTasks_.p, tasks.data(), sizeof(sq103_dense_task) * n, cudaMemcpyHostToDevice,
                                     st_.get()));
            SQ_CHECK(cudaMemcpyAsync(dOrder_.p, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st_.get()));
        }
        SQ_CHECK(cudaMemsetAsync(dPos_.p, 0, sizeof(int) * nAlloc, st_.get()));
        SQ_CHECK(cudaMemsetAsync(dQueue_.p, 0, sizeof(int) * 2, st_.get()));
        SQ_CHECK(cudaMemsetAsync(dStatus_.p, 0, sizeof(int), st_.get()));
        st_.sync();
        pos_ = 0;
        if (smem_ < 0) chooseConfig(-1);
        if (graph_) {
            cudaGraphExecDestroy(graph_);
            graph_ = nullptr;
        }
        prepared_ = true;
    }

    // the launch configuration (shared memory per CTA -> CTAs per SM) only
    // changes speed, never results
    void chooseConfig(int smemBytes) {
        int dev = 0, sms = 0;
        SQ_CHECK(cudaGetDevice(&dev));
        SQ_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        int maxS = sq103_dense_batch_max_smem(), maxM = 1;
        for (auto &p : insts_) maxM = std::max(maxM, p->m);
        const int minS = sq103_dense_batch_min_smem(maxM);  // the flip lists of the largest m
        throwErrorIf(minS > maxS, "%d trotters exceed the shared memory of one CTA.", maxM);
        smem_ = smemBytes < 0 ? std::min(maxS, 96 * 1024) : std::min(smemBytes, maxS);
        smem_ = std::max(smem_, minS);
        int per = std::max(1, sq103_dense_batch_ctas_per_sm(smem_));
        grid_ = std::max(1, std::min(std::max(nSmall_, 1), per * sms));
        if (graph_) {
            cudaGraphExecDestroy(graph_);
            graph_ = nullptr;
        }
    }

    // times a few candidate configurations on copies of the instance state and keeps the fastest
    // Trotters per CTA, by measurement: for each candidate size limit (instances of
    // at least that many spins take one CTA per trotter in packed launches, the
    // rest one CTA per instance in the persistent kernel; 0: every instance in the
    // persistent kernel) the batch is prepared and `trialSteps` steps from the start
    // of the schedule are timed; the fastest limit is kept and the batch prepared
    // again, so the results do not depend on the choice.  Returns the limit.
    int autotuneRouting(int trialSteps, const int *cands, int nCands) {
        throwErrorIf(!cands || nCands < 1, "no candidate size limit.");
        throwErrorIf(insts_.empty() || nSched_ <= 0, "add instances and set a schedule first.");
        const int steps = std::max(1, std::min(trialSteps, nSched_));
        cudaEvent_t e0, e1;
        SQ_CHECK(cudaEventCreate(&e0));
        SQ_CHECK(cudaEventCreate(&e1));
        float best = 1e30f;
        int bestN = multiMinN_;
        for (int i = 0; i < nCands; ++i) {
            throwErrorIf(cands[i] < 0, "size limits must not be negative.");
            multiMinN_ = cands[i];
            prepare();
            SQ_CHECK(cudaEventRecord(e0, st_.get()));
            anneal(steps, true);
            SQ_CHECK(cudaEventRecord(e1, st_.get()));
            sync();
            float ms = 0.f;
            SQ_CHECK(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                bestN = cands[i];
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        multiMinN_ = bestN;
        prepare();
        return bestN;
    }

    int autotune(int trialSteps) {
        throwErrorIf(!prepared_, "prepare() first.");
        const int n = (int)insts_.size();
        std::vector<DevBuf<unsigned char>> saveQ(n), saveF(n);
        for (int i = 0; i < n; ++i) {
            Inst &in = *insts_[i];
            saveQ[i].ensure((size_t)in.m * in.N);
            saveF[i].ensure((size_t)in.m * in.N * 4);
            SQ_CHECK(cudaMemcpyAsync(saveQ[i].p, in.q, (size_t)in.m * in.N, cudaMemcpyDeviceToDevice, st_.get()));
            SQ_CHECK(cudaMemcpyAsync(saveF[i].p, in.F, (size_t)in.m * in.N * 4, cudaMemcpyDeviceToDevice, st_.get()));
        }
        int maxS = sq103_dense_batch_max_smem();
        int cands[] = {0, 24 * 1024, 48 * 1024, 96 * 1024, maxS};
        float best = 1e30f;
        int bestS = smem_;
        cudaEvent_t e0, e1;
        SQ_CHECK(cudaEventCreate(&e0));
        SQ_CHECK(cudaEventCreate(&e1));
        for (int c : cands) {
            if (c > maxS) continue;
            chooseConfig(c);
            SQ_CHECK(cudaMemsetAsync(dPos_.p, 0, sizeof(int) * std::max(nSmall_, 1), st_.get()));
            SQ_CHECK(cudaEventRecord(e0, st_.get()));
            for (int s = 0; s < trialSteps; ++s) launchOne();
            SQ_CHECK(cudaEventRecord(e1, st_.get()));
            SQ_CHECK(cudaEventSynchronize(e1));
            float ms = 0.f;
            SQ_CHECK(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                bestS = c;
            }
            for (int i = 0; i < n; ++i) {  // restore the state
                Inst &in = *insts_[i];
                SQ_CHECK(cudaMemcpyAsync(in.q, saveQ[i].p, (size_t)in.m * in.N, cudaMemcpyDeviceToDevice, st_.get()));
                SQ_CHECK(cudaMemcpyAsync(in.F, saveF[i].p, (size_t)in.m * in.N * 4, cudaMemcpyDeviceToDevice, st_.get()));
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        SQ_CHECK(cudaMemsetAsync(dPos_.p, 0, sizeof(int) * std::max(nSmall_, 1), st_.get()));
        st_.sync();
        chooseConfig(bestS);
        return bestS;
    }

    // nSteps further steps of every instance (bounded by the schedule length), in
    // chunks that end at the field refreshes (every kRefreshPeriod steps, as the
    // single-instance solver refreshes)
    void anneal(int nSteps, bool useGraph) {
        throwErrorIf(!prepared_, "prepare() first.");
        int left = std::min(nSteps, nSched_ - pos_);
        while (left > 0) {
            if (pos_ > 0 && pos_ % kRefreshPeriod == 0) refreshAll();
            const int chunk = std::min(left, kRefreshPeriod - pos_ % kRefreshPeriod);
            for (int s = 0; s < chunk && nSmall_ > 0; ++s) {
                if (useGraph) {
                    if (!graph_) captureStep();
                    SQ_CHECK(cudaGraphLaunch(graph_, st_.get()));
                } else {
                    launchOne();
                }
            }
            launchMulti(chunk);
            pos_ += chunk;
            left -= chunk;
        }
    }

    void sync() {
        st_.sync();
        if (multi_.empty()) return;
        int status = 0;
        SQ_CHECK(cudaMemcpy(&status, dStatus_.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (status != 0) throw_cuda(status, "one-CTA-per-trotter batch sweep");
    }

    // instances of at least N spins take the one-CTA-per-trotter sweep (0: none); before prepare()
    void setMultiMinN(int N) {
        throwErrorIf(N < 0, "the size limit must not be negative.");
        multiMinN_ = N;
        prepared_ = false;
    }
    int multiCount() const { return (int)multi_.size(); }
    int size() const { return (int)insts_.size(); }
    int position() const { return pos_; }
    int grid() const { return grid_; }
    int smem() const { return smem_; }
    const Inst &inst(int i) const {
        throwErrorIf(i < 0 || i >= (int)insts_.size(), "instance index out of range.");
        return *insts_[i];
    }

    void energies(int i, double *E) {
        const Inst &in = inst(i);
        r_.ensure((size_t)in.m * in.N);
        E64_.ensure(in.m);
        SQ_CHECK(sq103_dense_energy(in.J, in.ldJ, in.h, in.c64, in.q, in.N, in.m, optimize_[i], r_.p, E64_.p,
                                    nullptr, st_.get()));
        SQ_CHECK(cudaMemcpyAsync(E, E64_.p, sizeof(double) * in.m, cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
    }

    void spins(int i, int8_t *q) {
        const Inst &in = inst(i);
        SQ_CHECK(cudaMemcpyAsync(q, in.q, (size_t)in.m * in.N, cudaMemcpyDeviceToHost, st_.get()));
        st_.sync();
    }

private:
    void launchOne() {
        SQ_CHECK(sq103_dense_batch_launch(dTasks_.p, nSmall_, nullptr, dOrder_.p, dPos_.p, dQueue_.p, 1, grid_, smem_,
                                          st_.get()));
    }

    // `chunk` steps of the large instances from pos_: packed cooperative launches of
    // instances of similar size, as many trotters as can be resident at once
    void launchMulti(int chunk) {
        std::vector<sq103_dense_task> pack;
        int packM = 0, packN = 0;
        auto flush = [&]() {
            if (!pack.empty()) SQ_CHECK(sq103_dense_anneal_pack(pack.data(), (int)pack.size(), st_.get()));
            pack.clear();
            packM = packN = 0;
        };
        for (Inst *in : multi_) {
            sq103_dense_task t = {};
            t.J = in->J;
            t.h = in->h;
            t.q = in->q;
            t.F = in->F;
            t.G = sched_.p + pos_;
            t.beta = sched_.p + nSched_ + pos_;
            t.status = dStatus_.p;
            t.seed = in->seed;
            t.step0 = 1 + (uint32_t)pos_;  // step 0 of the Philox counter is the randomisation
            t.N = in->N;
            t.m = in->m;
            t.ldJ = in->ldJ;
            t.algo = kColoring;
            t.nSteps = chunk;
            t.ws = in->ws.p;
            t.wsBytes = in->wsBytes;
            const int N2 = std::max(packN, in->N);
            if ((int)pack.size() == kPackMax || packM + in->m > sq103_dense_multicta_capacity(N2)) flush();
            pack.push_back(t);
            packM += in->m;
            packN = std::max(packN, in->N);
        }
        flush();
    }

    // Instances below the tensor-core refresh size take the SIMT refresh, all of
    // them in one launch (one CTA per 64 x 64 tile of any instance's fields);
    // the others refresh on the tensor cores one by one.
    void buildRefreshJobs() {
        std::vector<sq103_field_job> jobs;
        std::vector<int> tileJob;
        tcInsts_.clear();
        for (auto &p : insts_) {
            Inst &in = *p;
            if (in.digits.p) {
                tcInsts_.push_back(&in);
                continue;
            }
            sq103_field_job j = {};
            j.J = in.J;
            j.q = in.q;
            j.F = in.F;
            j.N = in.N;
            j.m = in.m;
            j.ldJ = in.ldJ;
            j.tile0 = (int)tileJob.size();
            const int tiles = ((in.N + 63) / 64) * ((in.m + 63) / 64);
            tileJob.insert(tileJob.end(), tiles, (int)jobs.size());
            jobs.push_back(j);
        }
        nTiles_ = (int)tileJob.size();
        if (jobs.empty()) return;
        dJobs_.ensure(jobs.size());
        dTileJob_.ensure(tileJob.size());
        SQ_CHECK(cudaMemcpyAsync(dJobs_.p, jobs.data(), sizeof(sq103_field_job) * jobs.size(), cudaMemcpyHostToDevice,
                                 st_.get()));
        SQ_CHECK(cudaMemcpyAsync(dTileJob_.p, tileJob.data(), sizeof(int) * tileJob.size(), cudaMemcpyHostToDevice,
                                 st_.get()));
        st_.sync();
    }

    // The tensor-core refreshes are independent and each fills only part of the
    // GPU: they run on kRefreshStreams side streams, forked from and joined back
    // into the batch's stream with events (the same kernels, so the same fields).
    void refreshAll() {
        SQ_CHECK(sq103_dense_field_refresh_batch(dJobs_.p, dTileJob_.p, nTiles_, st_.get()));
        if (tcInsts_.empty()) return;
        const int ns = (int)std::min<size_t>(kRefreshStreams, tcInsts_.size());
        if (!fork_) {
            SQ_CHECK(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
            for (cudaEvent_t &e : join_) SQ_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        SQ_CHECK(cudaEventRecord(fork_, st_.get()));
        for (int k = 0; k < ns; ++k) SQ_CHECK(cudaStreamWaitEvent(side_[k].get(), fork_, 0));
        for (size_t i = 0; i < tcInsts_.size(); ++i) {
            Inst &in = *tcInsts_[i];
            SQ_CHECK(sq103_dense_refresh(in.J, in.ldJ, in.digits.p, in.Abf.p, in.q, in.F, in.N, in.m, in.status,
                                         side_[i % ns].get()));
        }
        for (int k = 0; k < ns; ++k) {
            SQ_CHECK(cudaEventRecord(join_[k], side_[k].get()));
            SQ_CHECK(cudaStreamWaitEvent(st_.get(), join_[k], 0));
        }
    }

    void captureStep() {
        cudaGraph_t g;
        SQ_CHECK(cudaStreamBeginCapture(st_.get(), cudaStreamCaptureModeThreadLocal));
        launchOne();
        SQ_CHECK(cudaStreamEndCapture(st_.get(), &g));
        SQ_CHECK(cudaGraphInstantiate(&graph_, g, 0));
        cudaGraphDestroy(g);
    }

    Stream st_;
    std::vector<std::unique_ptr<Inst>> insts_;
    std::vector<int> optimize_;
    DevBuf<float> dW_, sched_;
    DevBuf<double> scratch_, r_, E64_;
    DevBuf<sq103_dense_task> dTasks_;
    DevBuf<int> dOrder_, dPos_, dQueue_, dStatus_;
    DevBuf<sq103_field_job> dJobs_;  // the SIMT refresh of every instance below the tensor-core size
    DevBuf<int> dTileJob_;
    int nTiles_ = 0;
    std::vector<Inst *> tcInsts_;     // instances refreshed on the tensor cores
    static constexpr int kRefreshStreams = 4;
    Stream side_[kRefreshStreams];
    cudaEvent_t fork_ = nullptr, join_[kRefreshStreams] = {};
    std::vector<Inst *> multi_;  // the instances on the one-CTA-per-trotter sweep, by N
    cudaGraphExec_t graph_ = nullptr;
    int nSched_ = 0, pos_ = 0, grid_ = 1, smem_ = -1, nSmall_ = 0, multiMinN_ = kDefaultMultiMinN;
    bool prepared_ = false;
};

// ============================================================= formulas
// The CUDA formula sets (sqaodc/cuda/CUDAFormulas.cpp:8-294), for real = float
// and real = double: each call uploads its host arguments, runs the
// Hamiltonian or energy kernels of formulas.cu on the object's stream and
// copies the result back.  Energies are FP64 (float: fp32 inputs with
// double-float row sums; double: FP64 throughout) and rounded to real only
// where the interface returns real.  A QUBO energy is the Ising energy kernel
// run with J = W, h = b, c = 0 and the sign of a maximisation: bits times the
// couplings are exact products, so the result is x W x^T to FP64 accuracy and
// a zero x gives exactly 0.  Bits must be 0 / 1 and spins -1 / +1 (checked).
// Rows are processed in chunks that keep the device scratch under
// kFormulaScratch doubles.
static constexpr size_t kFormulaScratch = (size_t)1 << 25;

// real-typed rows (the reference's bit / spin vectors) -> int8, checked
template <class Row>
static std::vector<int8_t> rows_to_int8(const Row *rows, int nRows, int len, bool spins, const char *fn) {
    std::vector<int8_t> out((size_t)nRows * len);
    for (int r = 0; r < nRows; ++r)
        for (int i = 0; i < len; ++i) {
            const double v = (double)rows[r](i);
            throwErrorIf(spins ? (v != 1. && v != -1.) : (v != 0. && v != 1.), "%s, %s must be %s.", fn,
                         spins ? "q" : "x", spins ? "-1 or +1" : "0 or 1");
            out[(size_t)r * len + i] = (int8_t)v;
        }
    return out;
}

// row accessors over the reference's Vector / Matrix types
template <class real>
struct VecRow {
    const sq::VectorType<real> *v;
    real operator()(int i) const { return v->data[i]; }
};
template <class real>
struct MatRow {
    const sq::MatrixType<real> *m;
    int r;
    real operator()(int i) const { return m->data[(size_t)r * m->stride + i]; }
};
template <class real>
static std::vector<MatRow<real>> mat_rows(const sq::MatrixType<real> &m) {
    std::vector<MatRow<real>> rows;
    for (int r = 0; r < m.rows; ++r) rows.push_back(MatRow<real>{&m, r});
    return rows;
}
template <class real>
static void to_vector(sq::VectorType<real> *E, const std::vector<double> &e) {
    E->resize((int)e.size());
    for (size_t i = 0; i < e.size(); ++i) E->data[i] = (real)e[i];
}

template <class real>
class DenseFormulasT : public sq::cuda::DenseGraphFormulas<real> {
public:
    typedef sq::MatrixType<real> Matrix;
    typedef sq::VectorType<real> Vector;
    static constexpr bool kF64 = std::is_same<real, double>::value;

    void assignDevice(sq::cuda::Device &device) override {
        SQ_CHECK(cudaSetDevice(static_cast<DeviceImpl &>(device).devNo_));
    }

    // E[i] = x_i W x_i^T for the m rows of x (int8 bits, row stride N)
    void quboEnergies(const real *W, int ldW, int N, const int8_t *x, int m, double *E) {
        check_shape(N, m, __func__);
        throwErrorIf(!sq::isSymmetric(W, (size_t)N, (size_t)ldW), "%s, Matrix is not symmetric.", __func__);
        check_values(x, (size_t)m * N, false, __func__);
        energies(W, ldW, nullptr, 0.0, N, x, m, /*maximize*/ true, E);
    }

    // E[i] = -c - h q_i^T - q_i J q_i^T (int8 spins)
    void isingEnergies(const real *h, const real *J, int ldJ, real c, int N, const int8_t *q, int m, double *E) {
        check_shape(N, m, __func__);
        throwErrorIf(!sq::isSymmetric(J, (size_t)N, (size_t)ldJ), "%s, Matrix is not symmetric.", __func__);
        check_values(q, (size_t)m * N, true, __func__);
        energies(J, ldJ, h, (double)c, N, q, m, false, E);
    }

    void hamiltonian(const real *W, int ldW, int N, real *h, real *J, real *c) {
        check_shape(N, 1, __func__);
        throwErrorIf(!sq::isSymmetric(W, (size_t)N, (size_t)ldW), "%s, Matrix is not symmetric.", __func__);
        cudaStream_t s = st_.get();
        dW_.ensure((size_t)N * N);
        dh_.ensure(N);
        dJ_.ensure((size_t)N * N);
        dc_.ensure(1);
        dc64_.ensure(1);
        dscr_.ensure(N);
        SQ_CHECK(cudaMemcpy2DAsync(dW_.p, sizeof(real) * N, W, sizeof(real) * ldW, sizeof(real) * N, N,
                                   cudaMemcpyHostToDevice, s));
        if constexpr (kF64)
            SQ_CHECK(sq103_dense_hamiltonian64(dW_.p, N, dh_.p, dJ_.p, dc_.p, dscr_.p, s));
        else
            SQ_CHECK(sq103_dense_hamiltonian(dW_.p, N, N, 0, dh_.p, dJ_.p, N, dc_.p, dc64_.p, dscr_.p, s));
        SQ_CHECK(cudaMemcpyAsync(h, dh_.p, sizeof(real) * N, cudaMemcpyDeviceToHost, s));
        SQ_CHECK(cudaMemcpyAsync(J, dJ_.p, sizeof(real) * N * N, cudaMemcpyDeviceToHost, s));
        SQ_CHECK(cudaMemcpyAsync(c, dc_.p, sizeof(real), cudaMemcpyDeviceToHost, s));
        st_.sync();
    }

    // ---- the reference's interface
    void calculate_E(real *E, const Matrix &W, const Vector &x) override {
        throwErrorIf(E == nullptr, "%s, E is null.", __func__);
        throwErrorIf(W.rows != W.cols || x.size != W.cols, "%s, Shape does not match.", __func__);
        VecRow<real> r{&x};
        std::vector<int8_t> xi = rows_to_int8(&r, 1, x.size, false, __func__);
        double e;
        quboEnergies(W.data, W.stride, W.rows, xi.data(), 1, &e);
        *E = (real)e;
    }
    void calculate_E(Vector *E, const Matrix &W, const Matrix &x) override {
        throwErrorIf(E == nullptr, "%s, E is null.", __func__);
        throwErrorIf(W.rows != W.cols || x.cols != W.cols, "%s, Shape does not match.", __func__);
        auto rows = mat_rows(x);
        std::vector<int8_t> xi = rows_to_int8(rows.data(), x.rows, x.cols, false, __func__);
        std::vector<double> e(x.rows);
        quboEnergies(W.data, W.stride, W.rows, xi.data(), x.rows, e.data());
        to_vector(E, e);
    }
    void calculateHamiltonian(Vector *h, Matrix *J, real *c, const Matrix &W) override {
        throwErrorIf(h == nullptr || J == nullptr || c == nullptr, "%s, null output.", __func__);
        throwErrorIf(W.rows != W.cols, "%s, W is not a sqare matrix.", __func__);
        const int N = W.rows;
        h->resize(N);
        std::vector<real> Jd((size_t)N * N);
        hamiltonian(W.data, W.stride, N, h->data, Jd.data(), c);
        J->resize(N, N);
        for (int i = 0; i < N; ++i) memcpy(J->data + (size_t)i * J->stride, Jd.data() + (size_t)i * N, sizeof(real) * N);
    }
    void calculate_E(real *E, const Vector &h, const Matrix &J, real c, const Vector &q) override {
        throwErrorIf(E == nullptr, "%s, E is null.", __func__);
        throwErrorIf(J.rows != J.cols || h.size != J.cols || q.size != J.cols, "%s, Shape does not match.", __func__);
        VecRow<real> r{&q};
        std::vector<int8_t> qi = rows_to_int8(&r, 1, q.size, true, __func__);
        double e;
        isingEnergies(h.data, J.data, J.stride, c, J.rows, qi.data(), 1, &e);
        *E = (real)e;
    }
    void calculate_E(Vector *E, const Vector &h, const Matrix &J, real c, const Matrix &q) override {
        throwErrorIf(E == nullptr, "%s, E is null.", __func__);
        throwErrorIf(J.rows != J.cols || h.size != J.cols || q.cols != J.cols, "%s, Shape does not match.", __func__);
        auto rows = mat_rows(q);
        std::vector<int8_t> qi = rows_to_int8(rows.data(), q.rows, q.cols, true, __func__);
        std::vector<double> e(q.rows);
        isingEnergies(h.data, J.data, J.stride, c, J.rows, qi.data(), q.rows, e.data());
        to_vector(E, e);
    }

private:
    static void check_shape(int N, int m, const char *fn) {
        throwErrorIf(N <= 0 || m <= 0, "%s, Shape does not match.", fn);
    }

    // sign * (-c - h q^T - q J q^T) of every row, h = 0 when null
    void energies(const real *J, int ldJ, const real *h, double c, int N, const int8_t *q, int m, bool maximize,
                  double *E) {
        cudaStream_t s = st_.get();
        dJ_.ensure((size_t)N * N);
        dh_.ensure(N);
        dc64_.ensure(1);
        SQ_CHECK(cudaMemcpy2DAsync(dJ_.p, sizeof(real) * N, J, sizeof(real) * ldJ, sizeof(real) * N, N,
                                   cudaMemcpyHostToDevice, s));
        if (h)
            SQ_CHECK(cudaMemcpyAsync(dh_.p, h, sizeof(real) * N, cudaMemcpyHostToDevice, s));
        else
            SQ_CHECK(cudaMemsetAsync(dh_.p, 0, sizeof(real) * N, s));
        SQ_CHECK(cudaMemcpyAsync(dc64_.p, &c, sizeof(double), cudaMemcpyHostToDevice, s));
        const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)m, kFormulaScratch / (size_t)N));
        dq_.ensure((size_t)chunk * N);
        if (!kF64) dr_.ensure((size_t)chunk * N);
        dE_.ensure(chunk);
        for (int r0 = 0; r0 < m; r0 += chunk) {
            const int rows = std::min(chunk, m - r0);
            SQ_CHECK(cudaMemcpyAsync(dq_.p, q + (size_t)r0 * N, (size_t)rows * N, cudaMemcpyHostToDevice, s));
            if constexpr (kF64)
                SQ_CHECK(sq103_dense_energy64(dJ_.p, dh_.p, c, dq_.p, N, rows, maximize ? 1 : 0, dE_.p, s));
            else
                SQ_CHECK(sq103_dense_energy(dJ_.p, N, dh_.p, dc64_.p, dq_.p, N, rows, maximize ? 1 : 0, dr_.p,
                                            dE_.p, nullptr, s));
            SQ_CHECK(cudaMemcpyAsync(E + r0, dE_.p, sizeof(double) * rows, cudaMemcpyDeviceToHost, s));
            st_.sync();  // the next chunk reuses the staging buffers
        }
    }

    Stream st_;
    DevBuf<real> dW_, dh_, dJ_, dc_;
    DevBuf<double> dc64_, dscr_, dr_, dE_;
    DevBuf<int8_t> dq_;
};

template <class real>
class BipartiteFormulasT : public sq::cuda::BipartiteGraphFormulas<real> {
public:
    typedef sq::MatrixType<real> Matrix;
    typedef sq::VectorType<real> Vector;
    static constexpr bool kF64 = std::is_same<real, double>::value;

    void assignDevice(sq::cuda::Device &device) override {
        SQ_CHECK(cudaSetDevice(static_cast<DeviceImpl &>(device).devNo_));
    }

    // E[i] = b0 x0_i^T + b1 x1_i^T + x1_i W x0_i^T (W: N1 x N0, row stride N0)
    void quboEnergies(const real *b0, const real *b1, const real *W, int N0, int N1, const int8_t *x0,
                      const int8_t *x1, int m, double *E) {
        check_shape(N0, N1, m, __func__);
        check_values(x0, (size_t)m * N0, false, __func__);
        check_values(x1, (size_t)m * N1, false, __func__);
        energies(b0, b1, W, 0.0, N0, N1, x0, x1, m, true, E);
    }

    // E[i1 * m0 + i0] = the QUBO energy of (x0_i0, x1_i1)
    void quboEnergies2d(const real *b0, const real *b1, const real *W, int N0, int N1, const int8_t *x0, int m0,
                        const int8_t *x1, int m1, double *E) {
        check_shape(N0, N1, m0, __func__);
        check_shape(N0, N1, m1, __func__);
        check_values(x0, (size_t)m0 * N0, false, __func__);
        check_values(x1, (size_t)m1 * N1, false, __func__);
        // pairs in row-major (i1, i0) order, expanded a block of i1 rows at a time
        const size_t pairsPer = std::max<size_t>((size_t)m0, kFormulaScratch / (size_t)N1);
        const int i1Block = (int)std::max<size_t>(1, pairsPer / (size_t)m0);
        std::vector<int8_t> p0, p1;
        for (int a = 0; a < m1; a += i1Block) {
            const int nb = std::min(i1Block, m1 - a);
            const size_t np = (size_t)nb * m0;
            p0.resize(np * N0);
            p1.resize(np * N1);
            for (int i1 = 0; i1 < nb; ++i1)
                for (int i0 = 0; i0 < m0; ++i0) {
                    const size_t k = (size_t)i1 * m0 + i0;
                    memcpy(p0.data() + k * N0, x0 + (size_t)i0 * N0, N0);
                    memcpy(p1.data() + k * N1, x1 + (size_t)(a + i1) * N1, N1);
                }
            energies(b0, b1, W, 0.0, N0, N1, p0.data(), p1.data(), (int)np, true, E + (size_t)a * m0);
        }
    }

    // E[i] = -c - h0 q0_i^T - h1 q1_i^T - q1_i J q0_i^T
    void isingEnergies(const real *h0, const real *h1, const real *J, real c, int N0, int N1, const int8_t *q0,
                       const int8_t *q1, int m, double *E) {
        check_shape(N0, N1, m, __func__);
        check_values(q0, (size_t)m * N0, true, __func__);
        check_values(q1, (size_t)m * N1, true, __func__);
        energies(h0, h1, J, (double)c, N0, N1, q0, q1, m, false, E);
    }

    void hamiltonian(const real *b0, const real *b1, const real *W, int N0, int N1, real *h0, real *h1, real *J,
                     real *c) {
        check_shape(N0, N1, 1, __func__);
        cudaStream_t s = st_.get();
        upload_problem(b0, b1, W, N0, N1);
        dJ2_.ensure((size_t)N0 * N1);
        dh0o_.ensure(N0);
        dh1o_.ensure(N1);
        dc_.ensure(1);
        dc64_.ensure(1);
        dscr_.ensure((size_t)N0 + 2 * N1);
        if constexpr (kF64)
            SQ_CHECK(sq103_bipartite_hamiltonian64(dh0_.p, dh1_.p, dJ_.p, N0, N1, dh0o_.p, dh1o_.p, dJ2_.p, dc_.p,
                                                   dscr_.p, s));
        else
            SQ_CHECK(sq103_bipartite_hamiltonian(dh0_.p, dh1_.p, dJ_.p, N0, N1, 0, dh0o_.p, dh1o_.p, dJ2_.p, dc_.p,
                                                 dc64_.p, dscr_.p, s));
        SQ_CHECK(cudaMemcpyAsync(h0, dh0o_.p, sizeof(real) * N0, cudaMemcpyDeviceToHost, s));
        SQ_CHECK(cudaMemcpyAsync(h1, dh1o_.p, sizeof(real) * N1, cudaMemcpyDeviceToHost, s));
        SQ_CHECK(cudaMemcpyAsync(J, dJ2_.p, sizeof(real) * N0 * N1, cudaMemcpyDeviceToHost, s));
        SQ_CHECK(cudaMemcpyAsync(c, dc_.p, sizeof(real), cudaMemcpyDeviceToHost, s));
        st_.sync();
    }

    // ---- the reference's interface
    void calculate_E(real *E, const Vector &b0, const Vector &b1, const Matrix &W, const Vector &x0,
                     const Vector &x1) override {
        throwErrorIf(E == nullptr, "%s, E is null.", __func__);
        check_problem(b0, b1, W, __func__);
        throwErrorIf(x0.size != b0.size || x1.size != b1.size, "%s, Shape does not match.", __func__);
        VecRow<real> r0{&x0}, r1{&x1};
        std::vector<int8_t> a = rows_to_int8(&r0, 1, x0.size, false, __func__);
        std::vector<int8_t> b = rows_to_int8(&r1, 1, x1.size, false, __func__);
        std::vector<real> Wd = dense_copy(W);
        double e;
        quboEnergies(b0.data, b1.data, Wd.data(), b0.size, b1.size, a.data(), b.data(), 1, &e);
        *E = (real)e;
    }
    void calculate_E(Vector *E, const Vector &b0, const Vector &b1, const Matrix &W, const Matrix &x0,
                     const Matrix &x1) override {
        throwErrorIf(E == nullptr, "%s, E is null.", __func__);
        check_problem(b0, b1, W, __func__);
        throwErrorIf(x0.cols != b0.size || x1.cols != b1.size, "%s, Shape does not match.", __func__);
        throwErrorIf(x0.rows != x1.rows, "%s, Different batch dims between x0 and x1.", __func__);
        auto r0 = mat_rows(x0), r1 = mat_rows(x1);
        std::vector<int8_t> a = rows_to_int8(r0.data(), x0.rows, x0.cols, false, __func__);
        std::vector<int8_t> b = rows_to_int8(r1.data(), x1.rows, x1.cols, false, __func__);
        std::vector<real> Wd = dense_copy(W);
        std::vector<double> e(x0.rows);
        quboEnergies(b0.data, b1.data, Wd.data(), b0.size, b1.size, a.data(), b.data(), x0.rows, e.data());
        to_vector(E, e);
    }
    void calculate_E_2d(Matrix *E, const Vector &b0, const Vector &b1, const Matrix &W, const Matrix &x0,
                        const Matrix &x1) override {
        throwErrorIf(E == nullptr, "%s, E is null.", __func__);
        check_problem(b0, b1, W, __func__);
        throwErrorIf(x0.cols != b0.size || x1.cols != b1.size, "%s, Shape does not match.", __func__);
        auto r0 = mat_rows(x0), r1 = mat_rows(x1);
        std::vector<int8_t> a = rows_to_int8(r0.data(), x0.rows, x0.cols, false, __func__);
        std::vector<int8_t> b = rows_to_int8(r1.data(), x1.rows, x1.cols, false, __func__);
        std::vector<real> Wd = dense_copy(W);
        std::vector<double> e((size_t)x0.rows * x1.rows);
        quboEnergies2d(b0.data, b1.data, Wd.data(), b0.size, b1.size, a.data(), x0.rows, b.data(), x1.rows, e.data());
        E->resize(x1.rows, x0.rows);
        for (int i1 = 0; i1 < x1.rows; ++i1)
            for (int i0 = 0; i0 < x0.rows; ++i0)
                E->data[(size_t)i1 * E->stride + i0] = (real)e[(size_t)i1 * x0.rows + i0];
    }
    void calculateHamiltonian(Vector *h0, Vector *h1, Matrix *J, real *c, const Vector &b0, const Vector &b1,
                              const Matrix &W) override {
        throwErrorIf(h0 == nullptr || h1 == nullptr || J == nullptr || c == nullptr, "%s, null output.", __func__);
        check_problem(b0, b1, W, __func__);
        const int N0 = b0.size, N1 = b1.size;
        std::vector<real> Wd = dense_copy(W), Jd((size_t)N0 * N1);
        h0->resize(N0);
        h1->resize(N1);
        hamiltonian(b0.data, b1.data, Wd.data(), N0, N1, h0->data, h1->data, Jd.data(), c);
        J->resize(N1, N0);
        for (int i = 0; i < N1; ++i) memcpy(J->data + (size_t)i * J->stride, Jd.data() + (size_t)i * N0, sizeof(real) * N0);
    }
    void calculate_E(real *E, const Vector &h0, const Vector &h1, const Matrix &J, real c, const Vector &q0,
                     const Vector &q1) override {
        throwErrorIf(E == nullptr, "%s, E is null.", __func__);
        check_problem(h0, h1, J, __func__);
        throwErrorIf(q0.size != h0.size || q1.size != h1.size, "%s, Shape does not match.", __func__);
        VecRow<real> r0{&q0}, r1{&q1};
        std::vector<int8_t> a = rows_to_int8(&r0, 1, q0.size, true, __func__);
        std::vector<int8_t> b = rows_to_int8(&r1, 1, q1.size, true, __func__);
        std::vector<real> Jd = dense_copy(J);
        double e;
        isingEnergies(h0.data, h1.data, Jd.data(), c, h0.size, h1.size, a.data(), b.data(), 1, &e);
        *E = (real)e;
    }
    void calculate_E(Vector *E, const Vector &h0, const Vector &h1, const Matrix &J, real c, const Matrix &q0,
                     const Matrix &q1) override {
        throwErrorIf(E == nullptr, "%s, E is null.", __func__);
        check_problem(h0, h1, J, __func__);
        throwErrorIf(q0.cols != h0.size || q1.cols != h1.size, "%s, Shape does not match.", __func__);
        throwErrorIf(q0.rows != q1.rows, "%s, Different batch dims between q0 and q1.", __func__);
        auto r0 = mat_rows(q0), r1 = mat_rows(q1);
        std::vector<int8_t> a = rows_to_int8(r0.data(), q0.rows, q0.cols, true, __func__);
        std::vector<int8_t> b = rows_to_int8(r1.data(), q1.rows, q1.cols, true, __func__);
        std::vector<real> Jd = dense_copy(J);
        std::vector<double> e(q0.rows);
        isingEnergies(h0.data, h1.data, Jd.data(), c, h0.size, h1.size, a.data(), b.data(), q0.rows, e.data());
        to_vector(E, e);
    }

private:
    static void check_shape(int N0, int N1, int m, const char *fn) {
        throwErrorIf(N0 <= 0 || N1 <= 0 || m <= 0, "%s, Shape does not match.", fn);
    }
    static void check_problem(const Vector &v0, const Vector &v1, const Matrix &M, const char *fn) {
        throwErrorIf(M.rows != v1.size || M.cols != v0.size, "%s, Shape does not match.", fn);
    }

    void upload_problem(const real *v0, const real *v1, const real *M, int N0, int N1) {
        cudaStream_t s = st_.get();
        dh0_.ensure(N0);
        dh1_.ensure(N1);
        dJ_.ensure((size_t)N0 * N1);
        SQ_CHECK(cudaMemcpyAsync(dh0_.p, v0, sizeof(real) * N0, cudaMemcpyHostToDevice, s));
        SQ_CHECK(cudaMemcpyAsync(dh1_.p, v1, sizeof(real) * N1, cudaMemcpyHostToDevice, s));
        SQ_CHECK(cudaMemcpyAsync(dJ_.p, M, sizeof(real) * N0 * N1, cudaMemcpyHostToDevice, s));
    }

    // sign * (-c - h0 q0^T - h1 q1^T - q1 J q0^T) of every pair of rows
    void energies(const real *h0, const real *h1, const real *J, double c, int N0, int N1, const int8_t *q0,
                  const int8_t *q1, int m, bool maximize, double *E) {
        cudaStream_t s = st_.get();
        upload_problem(h0, h1, J, N0, N1);
        dc64_.ensure(1);
        SQ_CHECK(cudaMemcpyAsync(dc64_.p, &c, sizeof(double), cudaMemcpyHostToDevice, s));
        const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)m, kFormulaScratch / (size_t)N1));
        dq0_.ensure((size_t)chunk * N0);
        dq1_.ensure((size_t)chunk * N1);
        if (!kF64) dr_.ensure((size_t)chunk * N1);
        dE_.ensure(chunk);
        for (int r0 = 0; r0 < m; r0 += chunk) {
            const int rows = std::min(chunk, m - r0);
            SQ_CHECK(cudaMemcpyAsync(dq0_.p, q0 + (size_t)r0 * N0, (size_t)rows * N0, cudaMemcpyHostToDevice, s));
            SQ_CHECK(cudaMemcpyAsync(dq1_.p, q1 + (size_t)r0 * N1, (size_t)rows * N1, cudaMemcpyHostToDevice, s));
            if constexpr (kF64)
                SQ_CHECK(sq103_bipartite_energy64(dJ_.p, dh0_.p, dh1_.p, c, dq0_.p, dq1_.p, N0, N1, rows,
                                                  maximize ? 1 : 0, dE_.p, s));
            else
                SQ_CHECK(sq103_bipartite_energy(dJ_.p, dh0_.p, dh1_.p, dc64_.p, dq0_.p, dq1_.p, N0, N1, rows,
                                                maximize ? 1 : 0, dr_.p, dE_.p, nullptr, s));
            SQ_CHECK(cudaMemcpyAsync(E + r0, dE_.p, sizeof(double) * rows, cudaMemcpyDeviceToHost, s));
            st_.sync();
        }
    }

    Stream st_;
    DevBuf<real> dh0_, dh1_, dJ_, dJ2_, dh0o_, dh1o_, dc_;
    DevBuf<double> dc64_, dscr_, dr_, dE_;
    DevBuf<int8_t> dq0_, dq1_;
};

typedef DenseFormulasT<float> DenseFormulas;
typedef DenseFormulasT<double> DenseFormulas64;
typedef BipartiteFormulasT<float> BipartiteFormulas;
typedef BipartiteFormulasT<double> BipartiteFormulas64;

}  // namespace sq103

// ============================================================ factories
namespace sqaod {
namespace cuda {

template <>
DenseGraphAnnealer<float> *newDenseGraphAnnealer<float>() {
    return new sq103::DenseAnnealer();
}
template <>
BipartiteGraphAnnealer<float> *newBipartiteGraphAnnealer<float>() {
    return new sq103::BipartiteAnnealer();
}
template <>
DenseGraphAnnealer<double> *newDenseGraphAnnealer<double>() {
    return new sq103::DenseAnnealer64();
}
template <>
BipartiteGraphAnnealer<double> *newBipartiteGraphAnnealer<double>() {
    return new sq103::BipartiteAnnealer64();
}
template <>
DenseGraphBFSearcher<float> *newDenseGraphBFSearcher<float>() {
    return new sq103::DenseBFSearcher();
}
template <>
BipartiteGraphBFSearcher<float> *newBipartiteGraphBFSearcher<float>() {
    return new sq103::BipartiteBFSearcher();
}
template <>
DenseGraphBFSearcher<double> *newDenseGraphBFSearcher<double>() {
    return new sq103::DenseBFSearcher64();
}
template <>
BipartiteGraphBFSearcher<double> *newBipartiteGraphBFSearcher<double>() {
    return new sq103::BipartiteBFSearcher64();
}
template <>
DenseGraphFormulas<float> *newDenseGraphFormulas<float>() {
    return new sq103::DenseFormulas();
}
template <>
BipartiteGraphFormulas<float> *newBipartiteGraphFormulas<float>() {
    return new sq103::BipartiteFormulas();
}
template <>
DenseGraphFormulas<double> *newDenseGraphFormulas<double>() {
    return new sq103::DenseFormulas64();
}
template <>
BipartiteGraphFormulas<double> *newBipartiteGraphFormulas<double>() {
    return new sq103::BipartiteFormulas64();
}
Device *newDevice(int devNo) { return new sq103::DeviceImpl(devNo); }

}  // namespace cuda
}  // namespace sqaod

extern "C" SQ103_API void sqaodc_cuda_version(int *version, int *cuda_version) {
    *version = 10003;
    int v = 0;
    cudaRuntimeGetVersion(&v);
    *cuda_version = v;
}

#include "capi_impl.inc"
