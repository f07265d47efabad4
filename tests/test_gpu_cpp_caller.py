"""A C++ caller of the reference's solver API (tests/cpp/caller.cpp, the shape
of sqaodc/tests/perf.cpp:87-112) compiled against include/, linked with
libsqaod_gb300.so and run on the GPU: float and double dense annealers and
brute-force searchers through the sqaod::cuda factories.  Every printed result
is checked against the FP64 oracle."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bits(s):
    return np.array([int(c) for c in s], np.int8)


def test_cpp_caller_links_and_runs(orc, tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    from sqaod_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "caller")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "caller.cpp"), "-L", libdir, "-lsqaod_gb300",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe, "64", "8", "3"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = [json.loads(ln) for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert [(d["solver"], d.get("precision")) for d in lines] == [
        ("dense_annealer", "float"), ("dense_annealer", "double"), ("dense_bf_searcher", None),
        ("dense_bf_searcher", None)]
    for d in lines:
        N = d["N"]
        W = np.array(d["W"], np.float64).reshape(N, N)
        x = _bits(d["x"])
        E_x = float(orc.dg_energy_qubo(W, x)[0])
        if d["solver"] == "dense_annealer":
            tol = 1e-5 if d["precision"] == "float" else 1e-12
            assert abs(d["E"] - E_x) <= tol * max(1.0, abs(E_x)), d["E"]
            print("C++ caller, %s annealer: min E %.6f" % (d["precision"], d["E"]))
        else:
            E_ref, xs = orc.dg_bf_search_ref(W.astype(np.float32))
            assert d["E"] == E_ref == E_x
            assert np.array_equal(x, orc.unpack_bits(xs, N)[0])
