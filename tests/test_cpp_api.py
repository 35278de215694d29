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


TOOL_SRC = os.path.join(ROOT, "tests", "cpp", "tool_counter.cpp")
TOOL = os.path.join(ROOT, "kokkos_gb300", "_build", "libtool_counter.so")


def compile_tool():
    if os.path.exists(TOOL) and os.path.getmtime(TOOL) >= os.path.getmtime(TOOL_SRC):
        return TOOL
    os.makedirs(os.path.dirname(TOOL), exist_ok=True)
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", TOOL_SRC, "-o", TOOL],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-2000:]
    return TOOL


def test_profiling_tool_compiles():
    assert os.path.exists(compile_tool())


@pytest.mark.gpu
def test_header_path_calls_a_kokkos_tool():
    """With KOKKOS_TOOLS_LIBS naming a profiling tool, every parallel_for /
    parallel_reduce / parallel_scan of the header path calls the tool's
    begin and end callbacks in pairs, with the label given and a CUDA device
    id, and the tool is initialised and finalised once."""
    b = compile_test()
    env = dict(os.environ, KOKKOS_TOOLS_LIBS=compile_tool())
    r = subprocess.run([b], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600, env=env)
    assert r.returncode == 0 and "ALL PASS" in r.stdout, r.stdout[-4000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("KOKKOS_TOOL")]
    assert len(line) == 1, r.stdout[-2000:]
    f = dict(kv.split("=") for kv in line[0].split()[1:])
    for k in ("for", "reduce", "scan"):
        b_, e_ = (int(v) for v in f[k].split("/"))
        assert b_ > 0 and b_ == e_, (k, f[k])
    assert f["unmatched"] == "0" and f["open"] == "0" and f["devtype"] == "2", f
    assert f["saw_sum"] == "1" and f["version_ok"] == "1", f
