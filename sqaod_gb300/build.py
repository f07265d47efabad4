"""Builds libsqaod_gb300.so (the C ABI + the sm_103a kernels) in-tree.

nvcc compiles every translation unit of sqaod_gb300/csrc for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, and links them into
sqaod_gb300/lib/libsqaod_gb300.so.  Nothing is installed outside the tree.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libsqaod_gb300.so"

SOURCES = ["formulas.cu", "tc_gemm.cu", "dense.cu", "dense_multi.cu", "bipartite.cu", "bf.cu", "solvers.cu", "serve.cu", "common_api.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def lib_path():
    return os.path.join(OUT_DIR, LIB_NAME)


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsqaod_gb300.so")


def _deps():
    files = []
    for d in (CSRC, os.path.join(INCLUDE), os.path.join(INCLUDE, "sqaodc"),
              os.path.join(INCLUDE, "sqaodc", "common"), os.path.join(INCLUDE, "sqaodc", "cuda")):
        if os.path.isdir(d):
            files += [os.path.join(d, f) for f in os.listdir(d) if os.path.isfile(os.path.join(d, f))]
    return files + [__file__]


def _up_to_date(target):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False):
    out = lib_path()
    if not force and _up_to_date(out):
        return out
    nvcc = _nvcc()
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                     "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr"]

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, src + ".o")
        cmd = [nvcc] + common + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc] + common + ["-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = out + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
