"""The C++ header-template path (include/Kokkos_GB300.hpp): tests/cpp/test_api.cu
uses the Kokkos API of this path with user lambdas (Range / MDRange / Team
parallel_reduce and parallel_scan, built-in reducers, ScatterView, sort,
sort_by_key, BinSort, std algorithms, Graph).  It is compiled with nvcc for
sm_103a (CPU test: it must compile here) and run on the GPU, where every
check must pass."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_api.cu")
BIN = os.path.join(ROOT, "kokkos_gb300", "_build", "test_api")
LIBDIR = os.path.join(ROOT, "kokkos_gb300")


def _deps():
    inc = os.path.join(ROOT, "include")
    files = [SRC, os.path.join(LIBDIR, "libgbk.so")]
    for d, _, fs in os.walk(inc):
        files += [os.path.join(d, f) for f in fs]
    files += [os.path.join(LIBDIR, "csrc", f) for f in os.listdir(os.path.join(LIBDIR, "csrc")) if f.endswith(".cuh")]
    return files


def compile_test():
    if not os.path.exists(os.path.join(LIBDIR, "libgbk.so")):
        import __graft_entry__
        __graft_entry__.build()
    if os.path.exists(BIN) and all(os.path.getmtime(BIN) >= os.path.getmtime(f) for f in _deps()):
        return BIN
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "--extended-lambda",
           "-I" + os.path.join(ROOT, "include"), SRC, "-L" + LIBDIR, "-lgbk", "-Xlinker", "-rpath", "-Xlinker", LIBDIR,
           "-o", BIN]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-4000:]
    return BIN


def test_header_path_compiles_for_sm103a():
    assert os.path.exists(compile_test())


@pytest.mark.gpu
def test_header_path_runs():
    b = compile_test()
    r = subprocess.run([b], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    fails = [ln for ln in r.stdout.splitlines() if ln.startswith("FAIL")]
    assert r.returncode == 0 and not fails and "ALL PASS" in r.stdout, r.stdout[-4000:]
    assert sum(ln.startswith("PASS") for ln in r.stdout.splitlines()) >= 30
