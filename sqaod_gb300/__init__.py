"""sqaod_gb300: GB300-native (sm_103a) annealing and brute-force search for QUBO
problems, with the sqaod solver API.

    import sqaod_gb300 as sq
    ann = sq.cuda.dense_graph_annealer(W, sq.minimize, n_trotters=16)

The compute path is libsqaod_gb300.so (built in-tree by sqaod_gb300.build);
there is no CPU fallback.
"""
from .common import (Summary, algorithm, anneal, bit_from_spin, bit_to_spin, create_bitset_sequence,
                     generate_random_symmetric_W, make_summary, maximize, minimize, randomize_spin, symmetrize,
                     unique_x)
from ._lib import SqaodError

__version__ = "1.0.3"


def is_cuda_available():
    try:
        import ctypes
        cudart = ctypes.CDLL("libcuda.so.1")
        n = ctypes.c_int()
        return cudart.cuInit(0) == 0 and cudart.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


def __getattr__(name):
    if name == "cuda":
        import importlib
        mod = importlib.import_module(".cuda", __name__)
        globals()["cuda"] = mod
        return mod
    raise AttributeError(name)
