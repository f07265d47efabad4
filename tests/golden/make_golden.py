"""Generates tests/golden/golden.npz from the reference's own numpy backend.

The reference package ``sqaod`` refuses to import without its C extensions,
so this script registers a bare package object for ``sqaod`` that points at the
reference's ``sqaodpy/sqaod`` directory and imports only the pure-numpy
modules (``sqaod.common`` and ``sqaod.py``).  The reference tree is the first
argument, else $SQAOD_REFERENCE_ROOT, else a directory named ``reference``
beside this repository's root:

    python tests/golden/make_golden.py [path/to/sqaod]

The output is small (a few hundred KB) and is committed, so that the tests
need no reference tree at run time.

Problems generated (all seeded):
  - sqaodpy/tests/example_problems.py shapes: the 8x8 dense W, quantised
    random dense W (rint(W * 16384) / 16384), quantised bipartite problems;
  - the integer matrix of sqaodc/tests/utils.h:75-90 (upper triangle cycling
    -2..2, mirrored), the "minimum run" BF problem of
    sqaodc/tests/CUDADenseGraphBFSolverTest.cpp:218-247 (N = 16);
  - +/- ones matrices of sqaodpy/tests/test_dense_graph_bf_searcher.py:79-98.
Outputs: h, J, c from py.formulas; QUBO and Ising energies; BF searcher
Emin and argmin sets from py.dense_graph_bf_searcher /
py.bipartite_graph_bf_searcher.
"""
import importlib
import os
import sys
import types

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF = (sys.argv[1] if len(sys.argv) > 1 else
       os.environ.get("SQAOD_REFERENCE_ROOT", os.path.join(os.path.dirname(REPO), "reference")))
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")


def load_reference_py():
    pkgdir = os.path.join(REF, "sqaodpy", "sqaod")
    sq = types.ModuleType("sqaod")
    sq.__path__ = [pkgdir]
    sys.modules["sqaod"] = sq
    pref = importlib.import_module("sqaod.common.preference")
    sq.algorithm = pref.algorithm
    sq.minimize = pref.minimize
    sq.maximize = pref.maximize
    common = importlib.import_module("sqaod.common")
    for k in dir(common):
        if not k.startswith("_"):
            setattr(sq, k, getattr(common, k))
    sq.common = common
    py = importlib.import_module("sqaod.py")
    sq.py = py
    return sq


def int_test_matrix(dim):
    """Integer pattern of sqaodc/tests/utils.h:75-90 (cycling -2..2)."""
    W = np.zeros((dim, dim), np.float64)
    v = -2
    for r in range(dim):
        for c in range(r, dim):
            W[r, c] = W[c, r] = v
            v += 1
            if v == 3:
                v = -2
    return W


def quantize(W):
    return np.rint(W * 16384) / 16384.


def bits_of(x, n):
    return np.array([(x >> (n - 1 - i)) & 1 for i in range(n)], np.int8)


def main():
    sq = load_reference_py()
    f = sq.py.formulas
    out = {}
    np.random.seed(0)

    # dense formulas
    Wex = np.array([[-32 if i == j else 4 for j in range(8)] for i in range(8)], np.float64)
    Wr16 = quantize(sq.generate_random_symmetric_W(16))
    Wr100 = quantize(sq.generate_random_symmetric_W(100))
    for name, W in (("ex8", Wex), ("r16", Wr16), ("r100", Wr100)):
        h, J, c = f.dense_graph_calculate_hamiltonian(W.copy())
        out["dg_%s_W" % name] = W
        out["dg_%s_h" % name] = h
        out["dg_%s_J" % name] = J
        out["dg_%s_c" % name] = np.float64(c)
    # all 2^8 states of a random N=8 problem
    W8 = quantize(sq.generate_random_symmetric_W(8))
    X8 = np.array([bits_of(i, 8) for i in range(256)], np.int8)
    out["dg_r8_W"] = W8
    out["dg_r8_X"] = X8
    out["dg_r8_E"] = f.dense_graph_batch_calculate_E(W8, X8)
    h8, J8, c8 = f.dense_graph_calculate_hamiltonian(W8.copy())
    Q8 = (2 * X8 - 1).astype(np.int8)
    out["dg_r8_Eising"] = f.dense_graph_batch_calculate_E_from_spin(h8, J8, c8, Q8)

    # bipartite formulas
    N0, N1 = 12, 10
    b0 = quantize(np.random.random(N0) - 0.5)
    b1 = quantize(np.random.random(N1) - 0.5)
    Wb = quantize(np.random.random((N1, N0)) - 0.5)
    h0, h1, Jb, cb = f.bipartite_graph_calculate_hamiltonian(b0, b1, Wb)
    x0 = np.random.randint(0, 2, (20, N0)).astype(np.int8)
    x1 = np.random.randint(0, 2, (20, N1)).astype(np.int8)
    out.update({"bg_b0": b0, "bg_b1": b1, "bg_W": Wb, "bg_h0": h0, "bg_h1": h1, "bg_J": Jb,
                "bg_c": np.float64(cb), "bg_x0": x0, "bg_x1": x1,
                "bg_E": f.bipartite_graph_batch_calculate_E(b0, b1, Wb, x0, x1),
                "bg_E2d": f.bipartite_graph_batch_calculate_E_2d(b0, b1, Wb, x0[:7], x1[:7]),
                "bg_Eising": f.bipartite_graph_batch_calculate_E_from_spin(
                    h0, h1, Jb, cb, (2 * x0 - 1).astype(np.int8), (2 * x1 - 1).astype(np.int8))})

    # dense brute-force searches (py backend)
    cases = {
        "int12": (int_test_matrix(12), sq.minimize),
        "int16": (int_test_matrix(16), sq.minimize),
        "int16max": (int_test_matrix(16), sq.maximize),
        "ex8": (Wex, sq.minimize),
        "pos8min": (np.ones((8, 8)), sq.minimize),
        "neg8min": (-np.ones((8, 8)), sq.minimize),
        "pos8max": (np.ones((8, 8)), sq.maximize),
        "r10": (quantize(sq.generate_random_symmetric_W(10)), sq.minimize),
    }
    for name, (W, opt) in cases.items():
        # py.dense_graph_bf_searcher.search_range ends its range at tile_size
        # (not xbegin + tile_size), so one tile must cover all 2^N states.
        s = sq.py.dense_graph_bf_searcher(W, opt, tile_size=1 << W.shape[0])
        s.search()
        out["bf_%s_W" % name] = W
        out["bf_%s_om" % name] = np.int32(1 if opt is sq.maximize else 0)
        out["bf_%s_E" % name] = np.asarray(s.get_E())
        out["bf_%s_x" % name] = np.asarray(s.get_x(), np.int8)

    # bipartite brute-force search
    bN0, bN1 = 6, 5
    bb0 = quantize(np.random.random(bN0) - 0.5)
    bb1 = quantize(np.random.random(bN1) - 0.5)
    bW = quantize(np.random.random((bN1, bN0)) - 0.5)
    s = sq.py.bipartite_graph_bf_searcher(bb0, bb1, bW, sq.minimize)
    s.search()
    xs = s.get_x()
    out.update({"bbf_b0": bb0, "bbf_b1": bb1, "bbf_W": bW, "bbf_E": np.asarray(s.get_E()),
                "bbf_x0": np.asarray([p[0] for p in xs], np.int8),
                "bbf_x1": np.asarray([p[1] for p in xs], np.int8)})
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, len(out), "arrays")


if __name__ == "__main__":
    main()
