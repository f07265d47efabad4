"""Build recipe for the CPU oracle (test infrastructure).

``build_oracle()`` compiles oracle/oracle.c into oracle/liboracle.so with gcc
(OpenMP, -ffp-contract=off so the written arithmetic order is kept).  It runs
on x86_64 and aarch64 alike.

``build_ref()`` compiles the reference's own sqaodc/common/Random.cpp,
sqaodc/common/os_dependent_linux.cpp and sqaodc/cpu/Dot_SIMD.cpp, straight from
the reference tree where they lie, together with oracle/ref_harness.cpp, into
oracle/_ref/libsqaod_ref.so.  Only the reference's generated config header is
written (into oracle/_ref/include).  It is skipped when the reference tree is
absent or the host is not x86_64 (Dot_SIMD.cpp includes <x86intrin.h>).
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree: $SQAOD_REFERENCE_ROOT, else a directory named "reference"
# beside this repository's root; build_ref() skips the build when it is absent
REF_ROOT = os.environ.get("SQAOD_REFERENCE_ROOT",
                          os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def _run(cmd):
    subprocess.check_call(cmd)


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def oracle_lib_path():
    return os.path.join(HERE, "liboracle.so")


def ref_lib_path():
    return os.path.join(HERE, "_ref", "libsqaod_ref.so")


def build_oracle(force=False):
    src = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "oracle.h")]
    out = oracle_lib_path()
    if not force and _newer(out, src + [__file__]):
        return out
    flags = ["-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags += ["-mavx2", "-mfma"]
    _run(["gcc"] + flags + [src[0], "-o", out + ".tmp", "-lm"])
    os.replace(out + ".tmp", out)
    return out


def build_ref(force=False):
    """Returns the library path, or None when the reference cannot be built here."""
    sq = os.path.join(REF_ROOT, "sqaodc")
    if not os.path.isdir(sq) or platform.machine() not in ("x86_64", "AMD64"):
        return None
    out_dir = os.path.join(HERE, "_ref")
    inc = os.path.join(out_dir, "include", "sqaodc", "common")
    os.makedirs(inc, exist_ok=True)
    cfg = os.path.join(inc, "sqaod_config.h")
    if not os.path.exists(cfg):
        with open(cfg, "w") as f:
            f.write("#pragma once\n/* generated for the oracle build: no BLAS, no CUDA */\n")
    srcs = [os.path.join(sq, "common", "Random.cpp"),
            os.path.join(sq, "common", "os_dependent_linux.cpp"),
            os.path.join(sq, "cpu", "Dot_SIMD.cpp"),
            os.path.join(HERE, "ref_harness.cpp")]
    out = ref_lib_path()
    if not force and _newer(out, srcs):
        return out
    # the reference's own flags (configure.ac: SIMD_OPT=avx2 -> -mavx2 -mfma, -O2, OpenMP)
    cmd = ["g++", "-std=c++11", "-O2", "-mavx2", "-mfma", "-fopenmp", "-fPIC", "-shared",
           "-I", os.path.join(out_dir, "include"), "-I", REF_ROOT, "-I", sq]
    _run(cmd + srcs + ["-o", out + ".tmp"])
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
