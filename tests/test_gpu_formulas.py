"""sqaod_gb300.cuda.formulas on the GPU against the FP64 oracle, for float32
and float64.

The cases follow the reference's formula tests
(sqaodpy/tests/test_dense_graph_formulas.py, test_bipartite_graph_formulas.py):
zero and all-one bit vectors, every state of a small problem single and
batched, Hamiltonian identities and QUBO == Ising energies, plus larger ragged
sizes and the reference's error rules.  Tolerances, written out:
  * float32: the device sums energies in FP64 from the fp32 inputs, so a
    returned float32 energy lies within one float32 ulp of the oracle's FP64
    energy of the same inputs;
  * float64: FP64 throughout, within 1e-12 relative of the oracle (the
    reference's own float64 tests use 1e-12).
"""
import numpy as np
import pytest

import sqaod_gb300 as sq
from oracle import oracle_ctypes as orc

pytestmark = pytest.mark.gpu
F32, F64 = np.float32, np.float64
DTYPES = [F32, F64]


def formulas():
    return sq.cuda.formulas


def sym_W(N, seed, dtype=F32):
    rng = np.random.default_rng(seed)
    W = rng.uniform(-0.5, 0.5, (N, N))
    return ((W + W.T) * 0.5).astype(dtype)


def bip_problem(N0, N1, seed, dtype=F32):
    rng = np.random.default_rng(seed)
    return (rng.uniform(-0.5, 0.5, N0).astype(dtype), rng.uniform(-0.5, 0.5, N1).astype(dtype),
            rng.uniform(-0.5, 0.5, (N1, N0)).astype(dtype))


def close(E, E64, dtype):
    """(ok, worst excess) of E against FP64 values under the tolerance of dtype."""
    E = np.asarray(E, np.float64)
    E64 = np.asarray(E64, np.float64)
    if dtype is F32:
        tol = np.spacing(np.abs(E64).astype(F32)).astype(np.float64)
    else:
        tol = 1e-12 * np.maximum(1., np.abs(E64))
    return np.all(np.abs(E - E64) <= tol), np.max(np.abs(E - E64) - tol)


# ------------------------------------------------------------------ dense graph

@pytest.mark.parametrize("dtype", DTYPES)
def test_dense_energy_of_zero_and_one_bits(dtype):
    f = formulas()
    W = sym_W(8, 0, dtype)
    assert f.dense_graph_calculate_E(W, np.zeros(8, np.int8), dtype) == 0.
    E1 = f.dense_graph_calculate_E(W, np.ones(8, np.int8), dtype)
    assert type(E1) is dtype
    ok, err = close([E1], [np.sum(W.astype(np.float64))], dtype)
    assert ok, err


@pytest.mark.parametrize("dtype", DTYPES)
def test_dense_energy_every_state_single_and_batched(dtype):
    f = formulas()
    N = 8
    W = sym_W(N, 1, dtype)
    xs = sq.create_bitset_sequence(range(2 ** N), N)
    Eb = f.dense_graph_batch_calculate_E(W, xs, dtype)
    Es = np.array([f.dense_graph_calculate_E(W, x, dtype) for x in xs])
    Eb1 = np.array([f.dense_graph_batch_calculate_E(W, x, dtype)[0] for x in xs])
    assert Eb.dtype == dtype and Eb.shape == (2 ** N,)
    assert np.array_equal(Eb, Es) and np.array_equal(Eb, Eb1)
    ok, err = close(Eb, orc.dg_energy_qubo(W, xs), dtype)
    assert ok, err


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("N,m", [(1030, 40), (64, 1), (333, 257)])
def test_dense_energy_ragged_sizes(N, m, dtype):
    f = formulas()
    W = sym_W(N, N, dtype)
    x = (np.random.default_rng(N + m).random((m, N)) < 0.5).astype(np.int8)
    ok, err = close(f.dense_graph_batch_calculate_E(W, x, dtype), orc.dg_energy_qubo(W, x), dtype)
    assert ok, err


def test_dense_triangular_W_is_symmetrized():
    f = formulas()
    W = sym_W(40, 2)
    U = np.triu(W) + np.triu(W, 1)  # upper triangle carrying W_ij + W_ji
    x = (np.random.default_rng(3).random((16, 40)) < 0.5).astype(np.int8)
    E = f.dense_graph_batch_calculate_E(W, x, F32)
    assert np.array_equal(f.dense_graph_batch_calculate_E(U, x, F32), E)
    assert np.array_equal(f.dense_graph_batch_calculate_E(U.T.copy(), x, F32), E)  # lower triangle
    h, J, c = f.dense_graph_calculate_hamiltonian(W, F32)
    for T in (U, U.T.copy()):  # sqaodpy/tests/test_symmetrize_formulas.py
        hT, JT, cT = f.dense_graph_calculate_hamiltonian(T, F32)
        assert np.array_equal(hT, h) and np.array_equal(JT, J) and cT == c


@pytest.mark.parametrize("dtype", DTYPES)
def test_dense_hamiltonian_against_oracle(dtype):
    f = formulas()
    W = sym_W(100, 4, dtype)
    h, J, c = f.dense_graph_calculate_hamiltonian(W, dtype)
    h64, J64, c64 = orc.dg_hamiltonian(W)
    assert h.dtype == dtype and J.shape == (100, 100) and isinstance(c, dtype)
    assert np.array_equal(J, J64.astype(dtype))  # J = -W / 4 off the diagonal: exact
    rtol = 1e-6 if dtype is F32 else 1e-13
    assert np.max(np.abs(h - h64)) <= rtol * np.max(np.abs(h64))
    assert abs(c - c64) <= rtol * max(1., abs(c64))
    # identity of the conversion: -sum(h) + sum(J) + c == 0
    assert abs(-np.sum(h64) + np.sum(J64) + c64) < 1e-9
    atol = 1e-4 if dtype is F32 else 1e-11
    assert abs(-np.sum(h.astype(np.float64)) + np.sum(J.astype(np.float64)) + float(c)) < atol


@pytest.mark.parametrize("dtype", DTYPES)
def test_dense_qubo_energy_equals_ising_energy(dtype):
    f = formulas()
    N = 8
    W = sym_W(N, 5, dtype)
    h, J, c = f.dense_graph_calculate_hamiltonian(W, dtype)
    xs = sq.create_bitset_sequence(range(2 ** N), N)
    qs = (2 * xs - 1).astype(np.int8)
    Eq = f.dense_graph_batch_calculate_E(W, xs, dtype)
    Ei = f.dense_graph_batch_calculate_E_from_spin(h, J, c, qs, dtype)
    Ei1 = np.array([f.dense_graph_calculate_E_from_spin(h, J, c, q, dtype) for q in qs])
    assert np.array_equal(Ei, Ei1)
    assert np.allclose(Eq, Ei, atol=1e-5 if dtype is F32 else 1e-12)


@pytest.mark.parametrize("dtype", DTYPES)
def test_dense_ising_energy_against_oracle(dtype):
    f = formulas()
    N, m = 300, 24
    rng = np.random.default_rng(6)
    h = rng.uniform(-1, 1, N).astype(dtype)
    J = sym_W(N, 7, dtype)
    np.fill_diagonal(J, 0.)
    c = dtype(0.75)
    q = np.where(rng.random((m, N)) < 0.5, 1, -1).astype(np.int8)
    ok, err = close(f.dense_graph_batch_calculate_E_from_spin(h, J, c, q, dtype),
                    orc.dg_energy_ising(h, J, float(c), q), dtype)
    assert ok, err


@pytest.mark.parametrize("dtype", DTYPES)
def test_dense_formulas_reject_bad_input(dtype):
    f = formulas()
    W = sym_W(16, 8, dtype)
    with pytest.raises(sq.SqaodError, match="x must be 0 or 1"):
        f.dense_graph_calculate_E(W, np.full(16, 2, np.int8), dtype)
    h, J, c = f.dense_graph_calculate_hamiltonian(W, dtype)
    with pytest.raises(sq.SqaodError, match="q must be -1 or"):
        f.dense_graph_calculate_E_from_spin(h, J, c, np.zeros(16, np.int8), dtype)
    A = W.copy()
    A[0, 5] += 1.
    A[3, 9] -= 1.
    with pytest.raises(RuntimeError, match="triangular nor symmetric"):
        f.dense_graph_calculate_E(A, np.zeros(16, np.int8), dtype)


# --------------------------------------------------------------- bipartite graph

@pytest.mark.parametrize("dtype", DTYPES)
def test_bipartite_energy_of_zero_and_one_bits(dtype):
    f = formulas()
    b0, b1, W = bip_problem(8, 8, 10, dtype)
    assert f.bipartite_graph_calculate_E(b0, b1, W, np.zeros(8, np.int8), np.zeros(8, np.int8), dtype) == 0.
    E1 = f.bipartite_graph_calculate_E(b0, b1, W, np.ones(8, np.int8), np.ones(8, np.int8), dtype)
    ok, err = close([E1], [np.sum(b0, dtype=np.float64) + np.sum(b1, dtype=np.float64) +
                           np.sum(W, dtype=np.float64)], dtype)
    assert ok, err


def _all_pairs(N0, N1):
    xs = sq.create_bitset_sequence(range(2 ** (N0 + N1)), N0 + N1)
    return np.ascontiguousarray(xs[:, :N0]), np.ascontiguousarray(xs[:, N0:])


@pytest.mark.parametrize("dtype", DTYPES)
def test_bipartite_energy_every_state_single_and_batched(dtype):
    f = formulas()
    N0, N1 = 4, 8
    b0, b1, W = bip_problem(N0, N1, 11, dtype)
    x0, x1 = _all_pairs(N0, N1)
    Eb = f.bipartite_graph_batch_calculate_E(b0, b1, W, x0, x1, dtype)
    assert Eb.dtype == dtype and Eb.shape == (2 ** (N0 + N1),)
    sel = range(0, 2 ** (N0 + N1), 37)
    Es = np.array([f.bipartite_graph_calculate_E(b0, b1, W, x0[i], x1[i], dtype) for i in sel])
    assert np.array_equal(Eb[list(sel)], Es)
    ok, err = close(Eb, orc.bg_energy_qubo(b0, b1, W, x0, x1), dtype)
    assert ok, err


@pytest.mark.parametrize("dtype", DTYPES)
def test_bipartite_energy_2d(dtype):
    f = formulas()
    N0, N1 = 37, 70
    b0, b1, W = bip_problem(N0, N1, 12, dtype)
    rng = np.random.default_rng(13)
    x0 = (rng.random((5, N0)) < 0.5).astype(np.int8)
    x1 = (rng.random((7, N1)) < 0.5).astype(np.int8)
    E2 = f.bipartite_graph_batch_calculate_E_2d(b0, b1, W, x0, x1, dtype)
    assert E2.shape == (7, 5) and E2.dtype == dtype
    # every entry is the batched energy of that pair, bit for bit
    for i1 in range(7):
        Ep = f.bipartite_graph_batch_calculate_E(b0, b1, W, x0, np.repeat(x1[i1:i1 + 1], 5, 0), dtype)
        assert np.array_equal(E2[i1], Ep)
    ok, err = close(E2, orc.bg_energy_qubo_2d(b0, b1, W, x0, x1), dtype)
    assert ok, err


@pytest.mark.parametrize("dtype", DTYPES)
def test_bipartite_hamiltonian_and_ising_energy(dtype):
    f = formulas()
    N0, N1 = 4, 8
    b0, b1, W = bip_problem(N0, N1, 14, dtype)
    h0, h1, J, c = f.bipartite_graph_calculate_hamiltonian(b0, b1, W, dtype)
    r0, r1, RJ, rc = orc.bg_hamiltonian(b0, b1, W)
    assert J.shape == (N1, N0) and isinstance(c, dtype)
    assert np.array_equal(J, RJ.astype(dtype))  # J = -W / 4: exact
    tol = 1e-6 if dtype is F32 else 1e-14
    assert np.max(np.abs(h0 - r0)) <= tol and np.max(np.abs(h1 - r1)) <= tol
    assert abs(c - rc) <= tol * max(1., abs(rc))
    x0, x1 = _all_pairs(N0, N1)
    q0, q1 = (2 * x0 - 1).astype(np.int8), (2 * x1 - 1).astype(np.int8)
    Eq = f.bipartite_graph_batch_calculate_E(b0, b1, W, x0, x1, dtype)
    Ei = f.bipartite_graph_batch_calculate_E_from_spin(h0, h1, J, c, q0, q1, dtype)
    assert np.allclose(Eq, Ei, atol=1e-5 if dtype is F32 else 1e-12)
    Ei1 = np.array([f.bipartite_graph_calculate_E_from_spin(h0, h1, J, c, q0[i], q1[i], dtype)
                    for i in range(0, len(q0), 101)])
    assert np.array_equal(Ei[::101], Ei1)
    ok, err = close(Ei, orc.bg_energy_ising(h0, h1, J, float(c), q0, q1), dtype)
    assert ok, err


@pytest.mark.parametrize("dtype", DTYPES)
def test_bipartite_energy_large_ragged(dtype):
    f = formulas()
    N0, N1, m = 1000, 333, 48
    b0, b1, W = bip_problem(N0, N1, 15, dtype)
    rng = np.random.default_rng(16)
    x0 = (rng.random((m, N0)) < 0.5).astype(np.int8)
    x1 = (rng.random((m, N1)) < 0.5).astype(np.int8)
    ok, err = close(f.bipartite_graph_batch_calculate_E(b0, b1, W, x0, x1, dtype),
                    orc.bg_energy_qubo(b0, b1, W, x0, x1), dtype)
    assert ok, err


def test_bipartite_formulas_reject_bad_input():
    f = formulas()
    b0, b1, W = bip_problem(6, 5, 17)
    with pytest.raises(sq.SqaodError, match="x must be 0 or 1"):
        f.bipartite_graph_calculate_E(b0, b1, W, np.full(6, 3, np.int8), np.zeros(5, np.int8), F32)
    with pytest.raises(RuntimeError, match="Different batch dims"):
        f.bipartite_graph_batch_calculate_E(b0, b1, W, np.zeros((3, 6), np.int8), np.zeros((2, 5), np.int8), F32)
