"""Kernel skeletons of the GB300 Kokkos backend on the GPU
(tests/cpp/test_backend_skel.cu): parallel_for / parallel_reduce (scalar,
array-valued with a runtime count, a reducer with final(), MinLoc with ties),
the look-back parallel_scan with its total at tile-edge sizes, and the
TeamPolicy reduce at team sizes 128, 100, 33 and 1 (partial warps), driven
through closures shaped like the backend's adapters of a Kokkos functor and
FunctorAnalysis reducer.  Compiled here (CPU) and run on the GPU, exact
checks against host computations."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_backend_skel.cu")
BIN = os.path.join(ROOT, "kokkos_gb300", "_build", "test_backend_skel")
LIBDIR = os.path.join(ROOT, "kokkos_gb300")


def compile_skel():
    if not os.path.exists(os.path.join(LIBDIR, "libgbk.so")):
        import __graft_entry__
        __graft_entry__.build()
    deps = [SRC, os.path.join(LIBDIR, "libgbk.so"),
            os.path.join(ROOT, "include", "gb300_backend", "GB300", "Kokkos_GB300_Skeletons.hpp")]
    if os.path.exists(BIN) and all(os.path.getmtime(BIN) >= os.path.getmtime(f) for f in deps):
        return BIN
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-lineinfo",
           "-I" + os.path.join(ROOT, "include"), SRC, "-L" + LIBDIR, "-lgbk", "-Xlinker", "-rpath", "-Xlinker", LIBDIR,
           "-o", BIN]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-4000:]
    return BIN


def test_backend_skeletons_compile():
    assert os.path.exists(compile_skel())


@pytest.mark.gpu
def test_backend_skeletons_on_gpu():
    r = subprocess.run([compile_skel()], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0 and "FAIL" not in r.stdout, r.stdout[-4000:]
    assert r.stdout.count("ok ") >= 20, r.stdout
