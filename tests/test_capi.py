"""CPU-only checks of the C ABI library and of the host-side logic.

The library must build, load without a GPU and export every entry point that
include/sqaod_gb300.h declares; solver objects must apply the reference's
preference and state rules (sqaodc/common/Solver.cpp, Preference.cpp) before
any device work.
"""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from sqaod_gb300 import _lib
    return _lib.lib()


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "sqaod_gb300.h")).read()
    return sorted(set(re.findall(r"SQ103_API[^;(]*?\b(sq103_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_cpp_api_symbols_exported(lib):
    # the C++ factories of include/sqaodc/sqaodc.h are exported for C++ callers
    import subprocess
    from sqaod_gb300 import build
    out = subprocess.run(["nm", "-DC", "--defined-only", build.lib_path()], capture_output=True, text=True).stdout
    for sym in ("sqaod::cuda::newDenseGraphAnnealer<float>", "sqaod::cuda::newBipartiteGraphAnnealer<float>",
                "sqaod::cuda::newDenseGraphBFSearcher<float>", "sqaod::cuda::newBipartiteGraphBFSearcher<float>",
                "sqaod::cuda::newDenseGraphFormulas<float>", "sqaod::cuda::newBipartiteGraphFormulas<float>",
                "sqaod::cuda::newDenseGraphBFSearcher<double>", "sqaod::cuda::newBipartiteGraphBFSearcher<double>",
                "sqaod::deleteInstance", "sqaod::cuda::newDevice"):
        assert sym in out, sym


def test_version(lib):
    assert lib.sq103_version() == 10003


def test_annealer_preferences_on_host():
    import sqaod_gb300 as sq
    a = sq.cuda.dense_graph_annealer()
    p = a.get_preferences()
    assert p["algorithm"] == "coloring" and p["precision"] == "float" and p["device"] == "cuda"
    # as the reference's CUDA annealers (sqaodpy/tests/test_dense_graph_annealer.py:453-471)
    a.set_preferences(algorithm=sq.algorithm.naive, n_trotters=7)
    p = a.get_preferences()
    assert p["algorithm"] == "coloring" and p["n_trotters"] == 7
    a.set_preferences(algorithm=sq.algorithm.sa_default)
    assert a.get_preferences()["algorithm"] == "sa_naive"
    a.set_preferences(algorithm=sq.algorithm.sa_coloring)
    assert a.get_preferences()["algorithm"] == "sa_naive"
    a.set_preferences(algorithm=sq.algorithm.default)
    assert a.get_preferences()["algorithm"] == "coloring"
    b = sq.cuda.bipartite_graph_annealer()
    b.set_preferences(algorithm=sq.algorithm.sa_default)
    assert b.get_preferences()["algorithm"] == "sa_coloring"
    b.set_preferences(algorithm=sq.algorithm.naive)
    assert b.get_preferences()["algorithm"] == "coloring"
    b.set_preferences(algorithm=sq.algorithm.sa_naive)
    assert b.get_preferences()["algorithm"] == "sa_coloring"


def test_searcher_preferences_on_host():
    import sqaod_gb300 as sq
    s = sq.cuda.dense_graph_bf_searcher()
    p = s.get_preferences()
    assert p["algorithm"] == "brute_force_search" and p["tile_size"] == 1 << 18
    s.set_preferences(tile_size=1000)  # rounded up to a multiple of 256
    assert s.get_preferences()["tile_size"] == 1024
    s.set_preferences(algorithm=sq.algorithm.naive)
    assert s.get_preferences()["algorithm"] == "brute_force_search"
    b = sq.cuda.bipartite_graph_bf_searcher()
    b.set_preferences(tile_size_0=300, tile_size_1=512)
    p = b.get_preferences()
    assert p["tile_size_0"] == 512 and p["tile_size_1"] == 512


def test_state_machine_errors_on_host():
    import sqaod_gb300 as sq
    a = sq.cuda.dense_graph_annealer()
    for call in (a.prepare, a.randomize_spin, lambda: a.anneal_one_step(1., 1.), a.calculate_E,
                 a.make_solution):
        with pytest.raises(RuntimeError):
            call()
    with pytest.raises(RuntimeError):
        a.set_preferences(n_trotters=0)
    with pytest.raises(RuntimeError):
        a.set_preferences(no_such_pref=1)
    s = sq.cuda.dense_graph_bf_searcher()
    with pytest.raises(RuntimeError):
        s.search_range()


def test_input_checks_on_host():
    import sqaod_gb300 as sq
    for make in (sq.cuda.dense_graph_annealer, sq.cuda.bipartite_graph_annealer, sq.cuda.dense_graph_bf_searcher):
        with pytest.raises(RuntimeError, match="float32 or float64"):
            make(dtype=np.int32)
    a = sq.cuda.dense_graph_annealer()
    W = np.random.default_rng(0).uniform(-1, 1, (6, 6)).astype(np.float32)
    with pytest.raises(RuntimeError):  # neither symmetric nor triangular
        a.set_qubo(W)
    with pytest.raises(RuntimeError):
        a.set_qubo(np.zeros((3, 4), np.float32))
    with pytest.raises(RuntimeError):  # N > 63 for a brute-force searcher
        sq.cuda.dense_graph_bf_searcher().set_qubo(np.zeros((64, 64), np.float32))
    with pytest.raises(RuntimeError):
        sq.cuda.bipartite_graph_annealer().set_qubo(np.zeros(3), np.zeros(4), np.zeros((3, 3)))


def test_field_refresh_batch_argument_checks_on_host(lib):
    """The batched field refresh checks its table before any launch: no tiles is
    a no-op, tiles without a table or a negative count are rejected."""
    assert lib.sq103_dense_field_refresh_batch(None, None, 0, None) == 0
    assert lib.sq103_dense_field_refresh_batch(None, None, 5, None) != 0
    assert lib.sq103_dense_field_refresh_batch(None, None, -1, None) != 0


def test_symmetrize_rules():
    import sqaod_gb300 as sq
    W = np.triu(np.arange(16, dtype=np.float32).reshape(4, 4))
    S = sq.symmetrize(W)
    assert np.allclose(S, S.T) and np.allclose(np.diag(S), np.diag(W))
    assert sq.symmetrize(S) is S


def test_generators_match_reference_draws(golden):
    """generate_random_symmetric_W draws like sqaodpy's (same np.random calls)."""
    import sqaod_gb300 as sq
    np.random.seed(0)
    W = sq.generate_random_symmetric_W(16)
    assert np.allclose(np.rint(W * 16384) / 16384., golden["dg_r16_W"])
    assert np.array_equal(sq.create_bitset_sequence([5], 4), np.array([[0, 1, 0, 1]], np.int8))


def test_cpp_headers_compile(tmp_path):
    """A C++ caller written against the reference's API compiles against include/
    (factories, solver and formula interfaces, deleteInstance)."""
    import shutil
    import subprocess
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "caller.cpp"
    src.write_text(r'''
#include <sqaodc/sqaodc.h>
namespace sq = sqaod;
void use() {
    sq::cuda::DenseGraphAnnealer<float> *a = sq::cuda::newDenseGraphAnnealer<float>();
    sq::MatrixType<float> W(4, 4);
    a->setQUBO(W, sq::optMinimize);
    a->setPreference(sq::Preference(sq::pnNumTrotters, 8));
    a->prepare();
    a->randomizeSpin();
    a->annealOneStep(1.f, 10.f);
    a->makeSolution();
    const sq::VectorType<float> &E = a->get_E();
    (void)E;
    sq::deleteInstance(a);
    sq::cuda::DenseGraphFormulas<double> *f = sq::cuda::newDenseGraphFormulas<double>();
    sq::MatrixType<double> Wd(4, 4);
    sq::VectorType<double> x(4), h;
    sq::MatrixType<double> J;
    double e = 0., c = 0.;
    f->calculate_E(&e, Wd, x);
    f->calculateHamiltonian(&h, &J, &c, Wd);
    sq::deleteInstance(f);
    sq::cuda::BipartiteGraphFormulas<float> *g = sq::cuda::newBipartiteGraphFormulas<float>();
    sq::deleteInstance(g);
    sq::cuda::DenseGraphBFSearcher<double> *s = sq::cuda::newDenseGraphBFSearcher<double>();
    s->setQUBO(Wd, sq::optMinimize);
    s->search();
    const sq::VectorType<double> &Es = s->get_E();
    (void)Es;
    sq::deleteInstance(s);
}
''')
    import os
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-I", inc, "-c", str(src), "-o", str(tmp_path / "caller.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_factory_default_dtypes_on_host():
    """The sqaod_gb300.cuda factories default to float32 (the benchmark
    precision); the reference's default float64 is one argument away."""
    import numpy as np
    import sqaod_gb300 as sq
    for make in (sq.cuda.dense_graph_annealer, sq.cuda.bipartite_graph_annealer, sq.cuda.dense_graph_bf_searcher,
                 sq.cuda.bipartite_graph_bf_searcher):
        assert make().dtype is np.float32
        assert make(dtype=np.float64).dtype is np.float64
