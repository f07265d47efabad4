// host_util.h -- host-side helpers shared by the solver translation units:
// CUDA error checks that throw (the reference's throwOnError,
// sqaodc/cuda/cudafuncs.h:37), owning device / pinned buffers, a lazily
// created non-blocking stream.
#pragma once

#include <cuda_runtime.h>

#include <sqaodc/common/Common.h>

namespace sq103 {

[[noreturn]] inline void throw_cuda(int code, const char *what) {
    sqaod::throwError("%s failed: %s (%d)", what,
                      code > 0 && code < 1000 ? cudaGetErrorString((cudaError_t)code) : "device status", code);
}

inline void check(int code, const char *what) {
    if (code != 0) throw_cuda(code, what);
}
#define SQ_CHECK(call) ::sq103::check((int)(call), #call)

// owning device buffer
template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void ensure(size_t count) {
        if (count <= n && p) return;
        release();
        if (count == 0) return;
        SQ_CHECK(cudaMalloc((void **)&p, sizeof(T) * count));
        n = count;
    }
};

// owning pinned host buffer
template <class T>
struct HostBuf {
    T *p = nullptr;
    size_t n = 0;
    HostBuf() = default;
    HostBuf(const HostBuf &) = delete;
    HostBuf &operator=(const HostBuf &) = delete;
    ~HostBuf() {
        if (p) cudaFreeHost(p);
    }
    void ensure(size_t count) {
        if (count <= n && p) return;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        if (count == 0) return;
        SQ_CHECK(cudaMallocHost((void **)&p, sizeof(T) * count));
        n = count;
    }
};

// solver stream, created on first use so that a solver object can be built
// (and its preferences and state rules used) before any CUDA work
struct Stream {
    cudaStream_t h = nullptr;
    Stream() = default;
    Stream(const Stream &) = delete;
    ~Stream() {
        if (h) cudaStreamDestroy(h);
    }
    cudaStream_t get() {
        if (!h) SQ_CHECK(cudaStreamCreateWithFlags(&h, cudaStreamNonBlocking));
        return h;
    }
    void sync() { SQ_CHECK(cudaStreamSynchronize(get())); }
};

}  // namespace sq103
