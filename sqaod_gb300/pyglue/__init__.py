"""The reference's CUDA extension modules, on libsqaod_gb300.so.

sqaodpy's CUDA package (sqaodpy/sqaod/cuda/*.py) drives its solvers through
six C extension modules built from sqaodc/pyglue:

    cuda_device          sqaodpy/sqaod/cuda/src/cuda_device.cpp
    cuda_dg_annealer     annealer.inc, method table annealer.inc:885-908
    cuda_bg_annealer     the same table, bipartite signatures
    cuda_dg_bf_searcher  bf_searcher.inc, method table bf_searcher.inc:479-494
    cuda_bg_bf_searcher  the same table, bipartite signatures
    cuda_formulas        formulas.inc, method table formulas.inc:586-605

Each module here has the same function names, argument order and meaning:
a solver handle first, the dtype (numpy.float32 or numpy.float64) last,
results returned or written into the arrays passed in exactly as the
reference's extension does, and user errors raised as RuntimeError.  A
maintainer swaps the backend by importing these modules under the names
sqaod.cuda imports (`from . import cuda_dg_annealer as cext`); the Python
layer above them (sqaodpy/sqaod/common/*_base.py) is unchanged.

The handles are the solver objects of sqaod_gb300.cuda; every call is one
entry point of the C ABI (include/sqaod_gb300.h).  There is no CPU fallback.
"""
