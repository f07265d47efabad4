"""The reference's CUDA extension modules on libsqaod_gb300.so (sqaod_gb300.pyglue),
called as sqaodpy's base classes call them (sqaodpy/sqaod/common/*_base.py,
formulas_base.py): handle first, dtype last, output arrays passed in.  Each
case is one of the reference tests' known answers or an FP64 oracle check, for
float32 and float64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DTYPES = [np.float32, np.float64]


class _Tag:
    """The reference's minimize / maximize tags convert to 0 / 1 (preference.py:61-76)."""

    def __init__(self, v):
        self.v = v

    def __int__(self):
        return self.v


MIN, MAX = _Tag(0), _Tag(1)


@pytest.fixture(scope="module")
def glue():
    from sqaod_gb300 import pyglue  # noqa: F401
    from sqaod_gb300.pyglue import (cuda_bg_annealer, cuda_bg_bf_searcher, cuda_device, cuda_dg_annealer,
                                    cuda_dg_bf_searcher, cuda_formulas)
    dev = cuda_device.new()
    cuda_device.initialize(dev, 0)
    return dict(dev=dev, dg=cuda_dg_annealer, bg=cuda_bg_annealer, dgbf=cuda_dg_bf_searcher,
                bgbf=cuda_bg_bf_searcher, f=cuda_formulas, device=cuda_device)


@pytest.mark.parametrize("dtype", DTYPES)
def test_dense_annealer_module(glue, orc, dtype):
    ext = glue["dg"]
    N, m = 24, 6
    rng = np.random.default_rng(3)
    W = rng.uniform(-1, 1, (N, N))
    W = ((np.triu(W) + np.triu(W, 1).T)).astype(dtype)
    a = ext.new(dtype)
    ext.assign_device(a, glue["dev"], dtype)
    ext.set_qubo(a, W, MIN, dtype)
    assert ext.get_problem_size(a, dtype) == N
    ext.set_preferences(a, {"n_trotters": m, "algorithm": "coloring"}, dtype)
    prefs = ext.get_preferences(a, dtype)
    assert prefs["n_trotters"] == m and prefs["device"] == "cuda"
    assert prefs["precision"] == ("double" if dtype == np.float64 else "float")
    h, J, c = np.empty(N, dtype), np.empty((N, N), dtype), np.empty(1, dtype)
    ext.get_hamiltonian(a, h, J, c, dtype)
    h0, J0, c0 = orc.dg_hamiltonian(W.astype(np.float64))
    tol = 1e-6 if dtype == np.float32 else 1e-12
    assert np.allclose(h, h0, atol=tol) and np.allclose(J, J0, atol=tol) and abs(c[0] - c0) <= tol * N * N
    ext.seed(a, 7, dtype)
    ext.prepare(a, dtype)
    ext.randomize_spin(a, dtype)
    G = 5.0
    while G > 0.01:
        ext.anneal_one_step(a, G, 50.0, dtype)
        G *= 0.9
    ext.make_solution(a, dtype)
    E = ext.get_E(a, dtype)
    assert isinstance(E, np.ndarray) and E.dtype == dtype and len(E) == m
    x = ext.get_x(a, dtype)
    assert len(x) == m and all(v.dtype == np.int8 for v in x)
    E_x = orc.dg_energy_qubo(W.astype(np.float64), np.array(x))
    assert np.allclose(E, E_x, rtol=1e-5 if dtype == np.float32 else 1e-12)
    q = ext.get_q(a, dtype)
    assert np.array_equal(np.array(x), (np.array(q) + 1) // 2)
    # set_q / set_qset with the reference's int8 vectors (dense_graph_annealer_base.py:54-63)
    ext.set_qset(a, [np.ones(N, np.int8), -np.ones(N, np.int8)], dtype)
    ext.calculate_E(a, dtype)
    E2 = ext.get_E(a, dtype)
    assert len(E2) == 2
    sysE = ext.get_system_E(a, 0.5, 50.0, dtype)
    assert np.isfinite(sysE)
    ext.delete(a, dtype)


@pytest.mark.parametrize("dtype", DTYPES)
def test_bipartite_annealer_module(glue, orc, dtype):
    ext = glue["bg"]
    N0, N1, m = 12, 10, 4
    b0, b1, W = np.ones(N0, dtype), np.ones(N1, dtype), np.ones((N1, N0), dtype)
    a = ext.new(dtype)
    ext.set_qubo(a, b0, b1, W, MIN, dtype)
    assert tuple(ext.get_problem_size(a, dtype)) == (N0, N1)
    ext.set_preferences(a, {"n_trotters": m}, dtype)
    ext.seed(a, 1, dtype)
    ext.prepare(a, dtype)
    ext.randomize_spin(a, dtype)
    G = 5.0
    while G > 0.01:
        ext.anneal_one_step(a, G, 50.0, dtype)
        G *= 0.9
    ext.make_solution(a, dtype)
    # W = b = ones: the minimum is x = 0 with E = 0 (test_bipartite_graph_annealer.py:223-282)
    assert abs(ext.get_E(a, dtype).min()) < 1e-6
    h0, h1, J, c = np.empty(N0, dtype), np.empty(N1, dtype), np.empty((N1, N0), dtype), np.empty(1, dtype)
    ext.get_hamiltonian(a, h0, h1, J, c, dtype)
    r0, r1, rJ, rc = orc.bg_hamiltonian(b0, b1, W)
    assert np.allclose(h0, r0) and np.allclose(h1, r1) and np.allclose(J, rJ) and abs(c[0] - rc) < 1e-9
    pairs = ext.get_x(a, dtype)
    assert len(pairs) == m and all(len(p) == 2 for p in pairs)
    ext.set_q(a, (np.ones(N0, np.int8), np.ones(N1, np.int8)), dtype)
    ext.calculate_E(a, dtype)
    # q = +1 everywhere: E = N0 N1 + N0 + N1 (test_bipartite_graph_annealer.py:170-182)
    assert np.allclose(ext.get_E(a, dtype), N0 * N1 + N0 + N1)
    ext.delete(a, dtype)


@pytest.mark.parametrize("dtype", DTYPES)
def test_dense_bf_module(glue, orc, dtype):
    ext = glue["dgbf"]
    N = 12
    rng = np.random.default_rng(4)
    U = np.triu(rng.integers(-8, 9, (N, N)))
    W = (U + np.triu(U, 1).T).astype(dtype)
    s = ext.new(dtype)
    ext.set_qubo(s, W, MIN, dtype)
    ext.set_preferences(s, {"tile_size": 256}, dtype)
    ext.prepare(s, dtype)
    steps = 0
    while True:  # the loop of dense_graph_bf_searcher_base.py:60-66
        done, curx = ext.search_range(s, dtype)
        steps += 1
        assert isinstance(curx, int)
        if done:
            break
    assert steps > 1 and curx == 1 << N
    ext.make_solution(s, dtype)
    E_ref, xs = orc.dg_bf_search_ref(W.astype(np.float32))
    assert float(ext.get_E(s, dtype)[0]) == E_ref
    assert np.array_equal(np.array(ext.get_x(s, dtype)), orc.unpack_bits(xs, N))
    s2 = ext.new(dtype)
    ext.set_qubo(s2, W, MAX, dtype)
    ext.search(s2, dtype)
    E_max, _ = orc.dg_bf_search_ref(W.astype(np.float32), om=1)
    assert float(ext.get_E(s2, dtype)[0]) == E_max
    ext.delete(s, dtype)
    ext.delete(s2, dtype)


@pytest.mark.parametrize("dtype", DTYPES)
def test_bipartite_bf_module(glue, dtype):
    ext = glue["bgbf"]
    N0, N1 = 6, 5
    s = ext.new(dtype)
    ext.set_qubo(s, -np.ones(N0, dtype), -np.ones(N1, dtype), -np.ones((N1, N0), dtype), MIN, dtype)
    ext.prepare(s, dtype)
    while True:
        done, cur0, cur1 = ext.search_range(s, dtype)
        if done:
            break
    ext.make_solution(s, dtype)
    # all ones minimise: E = -(N0 N1 + N0 + N1) (test_bipartite_graph_bf_searcher.py)
    assert float(ext.get_E(s, dtype)[0]) == -(N0 * N1 + N0 + N1)
    x0, x1 = ext.get_x(s, dtype)[0]
    assert x0.all() and x1.all()
    ext.delete(s, dtype)


@pytest.mark.parametrize("dtype", DTYPES)
def test_formulas_module(glue, orc, dtype):
    f = glue["f"]
    dg, bg = f.dg_formulas_new(), f.bg_formulas_new()
    f.dg_formulas_assign_device(dg, glue["dev"])
    f.bg_formulas_assign_device(bg, glue["dev"])
    rng = np.random.default_rng(5)
    N = 16
    W = rng.uniform(-1, 1, (N, N))
    W = (np.triu(W) + np.triu(W, 1).T).astype(dtype)
    x = rng.integers(0, 2, (5, N)).astype(np.int8)
    E = np.empty(5, dtype)
    f.dense_graph_batch_calculate_E(dg, E, W, x, dtype)
    assert np.allclose(E, orc.dg_energy_qubo(W.astype(np.float64), x), rtol=1e-6)
    h, J, c = np.empty(N, dtype), np.empty((N, N), dtype), np.empty(1, dtype)
    f.dense_graph_calculate_hamiltonian(dg, h, J, c, W, dtype)
    h0, J0, c0 = orc.dg_hamiltonian(W.astype(np.float64))
    assert np.allclose(h, h0, atol=1e-6) and np.allclose(J, J0, atol=1e-6)
    # the identity -sum h + sum J + c = 0 at q = -1 ... (test_dense_graph_formulas.py:56-80): E(q = -1) = E(x = 0) = 0
    E1 = np.empty(1, dtype)
    f.dense_graph_calculate_E_from_spin(dg, E1, h, J, c[0], -np.ones(N, np.int8), dtype)
    assert abs(E1[0]) < 1e-4
    N0, N1 = 7, 9
    b0, b1 = rng.uniform(-1, 1, N0).astype(dtype), rng.uniform(-1, 1, N1).astype(dtype)
    Wb = rng.uniform(-1, 1, (N1, N0)).astype(dtype)
    x0, x1 = rng.integers(0, 2, (3, N0)).astype(np.int8), rng.integers(0, 2, (3, N1)).astype(np.int8)
    Eb = np.empty(3, dtype)
    f.bipartite_graph_batch_calculate_E(bg, Eb, b0, b1, Wb, x0, x1, dtype)
    assert np.allclose(Eb, orc.bg_energy_qubo(b0, b1, Wb, x0, x1), rtol=1e-6)
    f.dg_formulas_delete(dg)
    f.bg_formulas_delete(bg)


def test_wrong_dtype_raises_runtime_error(glue):
    """sqaodpy/tests/test_wrong_type.py: a dtype other than float32 / float64."""
    for ext in (glue["dg"], glue["bg"], glue["dgbf"], glue["bgbf"]):
        with pytest.raises(RuntimeError, match="dtype is not float64 nor float32"):
            ext.new(np.int32)


def test_user_errors_are_runtime_errors(glue):
    ext = glue["dg"]
    a = ext.new(np.float64)
    with pytest.raises(RuntimeError):
        ext.anneal_one_step(a, 1.0, 1.0, np.float64)  # before set_qubo / prepare
    with pytest.raises(RuntimeError):
        ext.set_qubo(a, np.array([[0.0, 1.0], [2.0, 0.0]]), MIN, np.float64)  # not symmetric
