"""Argument rules of sqaod_gb300.cuda.formulas that hold before any device work
(sqaodpy/sqaod/common/checkers.py, formulas_base.py): no GPU needed."""
import numpy as np
import pytest

import sqaod_gb300 as sq

F32 = np.float32


def test_only_float32_and_float64_are_provided():
    # sqaodpy/tests/test_wrong_type.py: an integer dtype raises RuntimeError
    with pytest.raises(RuntimeError):
        sq.cuda.formulas.dense_graph_calculate_hamiltonian(np.ones((4, 4), np.int32), np.int32)
    W = np.eye(4)
    with pytest.raises(RuntimeError, match="float32 or float64"):
        sq.cuda.formulas.dense_graph_calculate_E(W, np.zeros(4, np.int8), np.float16)
    with pytest.raises(RuntimeError, match="float32 or float64"):
        sq.cuda.formulas.bipartite_graph_calculate_hamiltonian(np.zeros(2), np.zeros(3), np.zeros((3, 2)),
                                                              np.int32)


def test_shape_and_type_checks():
    f = sq.cuda.formulas
    W = np.eye(4, dtype=F32)
    with pytest.raises(RuntimeError, match="dimension mismatch"):
        f.dense_graph_calculate_E(W, np.zeros(5, np.int8), F32)
    with pytest.raises(RuntimeError, match="wrong shape"):
        f.dense_graph_calculate_hamiltonian(np.zeros((3, 4), F32), F32)
    with pytest.raises(RuntimeError, match="np.int8"):
        # the batched spin form takes int8 spins as given, as the reference's does
        f.dense_graph_batch_calculate_E_from_spin(np.zeros(4, F32), W, 0., np.ones((2, 4), np.int32), F32)
    with pytest.raises(RuntimeError, match="not a scalar"):
        f.dense_graph_batch_calculate_E_from_spin(np.zeros(4, F32), W, np.zeros(2), np.ones((2, 4), np.int8), F32)
    b0, b1, Wb = np.zeros(3, F32), np.zeros(2, F32), np.zeros((2, 3), F32)
    with pytest.raises(RuntimeError, match="dimension mismatch"):
        f.bipartite_graph_calculate_E(b0, b1, Wb.T, np.zeros(3, np.int8), np.zeros(2, np.int8), F32)
    with pytest.raises(RuntimeError, match="dimension mismatch"):
        f.bipartite_graph_batch_calculate_E_2d(b0, b1, Wb, np.zeros((4, 2), np.int8), np.zeros((4, 2), np.int8),
                                               F32)


def test_searcher_dtypes():
    # the BF searchers come in float32 and float64; other dtypes raise before any device work
    for make in (lambda d: sq.cuda.dense_graph_bf_searcher(dtype=d),
                 lambda d: sq.cuda.bipartite_graph_bf_searcher(dtype=d)):
        with pytest.raises(RuntimeError, match="float32 or float64"):
            make(np.float16)
    # so do the annealers (the <double> annealers keep FP64 couplings); other dtypes raise
    for make in (lambda d: sq.cuda.dense_graph_annealer(dtype=d),
                 lambda d: sq.cuda.bipartite_graph_annealer(dtype=d)):
        with pytest.raises(RuntimeError, match="float32 or float64"):
            make(np.float16)
