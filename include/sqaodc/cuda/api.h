// api.h -- CUDA solver interfaces of the sqaod C++ solver API
// (sqaodc/cuda/api.h:16-83 of the reference): Device, DeviceAssigner and the
// CUDA flavours of the four solvers and the two formula sets.  Implemented for sm_103a by
// libsqaod_gb300.so: the annealers for <float>; the BF searchers and the
// formula sets for <float> and <double>.
#pragma once

#include <sqaodc/common/Common.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

extern "C" void sqaodc_cuda_version(int *version, int *cuda_version);

namespace sqaod {
namespace cuda {

class Device : public NullBase {
public:
    Device() {}
    virtual ~Device() {}
    virtual void initialize(int devNo = 0) = 0;
    virtual void finalize() = 0;

private:
    Device(const Device &);
};

struct DeviceAssigner {
    virtual ~DeviceAssigner() {}
    virtual void assignDevice(Device &device) = 0;
};

template <class real>
struct DenseGraphAnnealer : DeviceAssigner, sqaod::DenseGraphAnnealer<real> {
    virtual ~DenseGraphAnnealer() {}
};

template <class real>
struct BipartiteGraphAnnealer : DeviceAssigner, sqaod::BipartiteGraphAnnealer<real> {
    virtual ~BipartiteGraphAnnealer() {}
};

template <class real>
struct DenseGraphBFSearcher : DeviceAssigner, sqaod::DenseGraphBFSearcher<real> {
    virtual ~DenseGraphBFSearcher() {}
};

template <class real>
struct BipartiteGraphBFSearcher : DeviceAssigner, sqaod::BipartiteGraphBFSearcher<real> {
    virtual ~BipartiteGraphBFSearcher() {}
};

template <class real>
struct DenseGraphFormulas : DeviceAssigner, sqaod::DenseGraphFormulas<real> {
    virtual ~DenseGraphFormulas() {}
};

template <class real>
struct BipartiteGraphFormulas : DeviceAssigner, sqaod::BipartiteGraphFormulas<real> {
    virtual ~BipartiteGraphFormulas() {}
};

}  // namespace cuda
}  // namespace sqaod

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
