// sqaodc.h -- factories of the sqaod C++ solver API (sqaodc/sqaodc.h:41-59 of
// the reference), CUDA flavour only.  Objects are freed with
// sqaod::deleteInstance().  Only real = float is instantiated.
#pragma once

#include <sqaodc/common/Common.h>
#include <sqaodc/cuda/api.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

namespace sqaod {
namespace cuda {

template <class real>
DenseGraphBFSearcher<real> *newDenseGraphBFSearcher();

template <class real>
DenseGraphAnnealer<real> *newDenseGraphAnnealer();

template <class real>
BipartiteGraphBFSearcher<real> *newBipartiteGraphBFSearcher();

template <class real>
BipartiteGraphAnnealer<real> *newBipartiteGraphAnnealer();

template <class real>
DenseGraphFormulas<real> *newDenseGraphFormulas();

template <class real>
BipartiteGraphFormulas<real> *newBipartiteGraphFormulas();

Device *newDevice(int devNo = -1);

}  // namespace cuda
}  // namespace sqaod

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
