"""Build libgbk.so (CUDA, sm_103a) and libgbk_host.so (host data generator).

Each .cu translation unit is compiled by its own nvcc process in parallel,
then linked into one shared library in the package directory (in-tree; the
outputs are git-ignored).  Rebuilds only what changed (mtime of the unit or
of any header in csrc/ and include/).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]

LIB = os.path.join(HERE, "libgbk.so")
HOSTLIB = os.path.join(HERE, "libgbk_host.so")
# thrust comparator for the sort benchmarks (not part of libgbk.so)
CMP_SRC = os.path.join(HERE, "comparators", "thrust_sort.cu")
CMP_LIB = os.path.join(HERE, "comparators", "libgbk_thrust.so")
# throughput of the header-template path for user functors (run by bench.py)
HP_SRC = os.path.join(HERE, "bench_header_path.cu")
HP_BIN = os.path.join(OBJ, "bench_header_path")


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    hdrs = _headers()
    units = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    objs, todo = [], []
    for u in units:
        o = os.path.join(OBJ, os.path.basename(u)[:-3] + ".o")
        objs.append(o)
        if _stale(o, [u] + hdrs):
            todo.append((u, o))
    jobs = jobs or max(1, min(len(todo) + 1, os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_run, [nvcc()] + ARCH + NVFLAGS + ["-c", u, "-o", o]) for u, o in todo]
        if _stale(CMP_LIB, [CMP_SRC]):
            futs.append(ex.submit(_run, [nvcc()] + ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                                                           CMP_SRC, "-o", CMP_LIB]))
        for f in futs:
            out = f.result()
            if verbose and out.strip():
                print(out)
    if todo or _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs)
    hp_deps = [HP_SRC, LIB] + glob.glob(os.path.join(ROOT, "include", "gb300", "*.hpp")) + hdrs
    if _stale(HP_BIN, hp_deps):
        _run([nvcc()] + ARCH + ["-O3", "-std=c++17", "--extended-lambda", "-I" + os.path.join(ROOT, "include"), HP_SRC,
                                "-L" + HERE, "-lgbk", "-Xlinker", "-rpath", "-Xlinker", HERE, "-o", HP_BIN])
    src = os.path.join(CSRC, "gbk_datagen.c")
    if _stale(HOSTLIB, [src]):
        _run(["gcc", "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-Wall", src, "-o", HOSTLIB, "-lm"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
