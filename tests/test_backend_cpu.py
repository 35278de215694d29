"""The GB300 execution space as a Kokkos backend (include/gb300_backend/).

Built the way Kokkos builds a backend: the Kokkos sources' own core units and
the backend's unit (include/gb300_backend/GB300/Kokkos_GB300.cpp) compiled by
nvcc for sm_103a with the backend's configuration headers ahead of the Kokkos
sources, then tests/backend/backend_api.cu - Kokkos user code on
Kokkos::Experimental::GB300: RangePolicy / MDRangePolicy (tiles, Iterate::Right,
rank 6) / TeamPolicy parallel_for, parallel_reduce (built-in, combined, array
and final() reducers, View results), parallel_scan with and without a total,
TeamThreadRange / team_scan / team scratch, ScatterView + contribute,
Kokkos::sort, sort_by_key, the std reduce / exclusive_scan, deep_copy - linked
against them and libgbk.so (tests/backend/Makefile).

Needs the Kokkos sources (KOKKOS_REF_SRC, default: a `reference` checkout
beside this repository); skipped without them.  Without a GPU the program
runs in --no-device mode: Kokkos::initialize must reach the space's
impl_initialize through Kokkos' ExecSpaceManager (the space is registered)
and report the missing device.  Kokkos' execution-space concept check
(check_valid_execution_space) is a static_assert compiled into the
backend's unit.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("KOKKOS_REF_SRC", os.path.join(ROOT, os.pardir, "reference"))
BIN = os.path.join(ROOT, "tests", "backend", "_build", "backend_api")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "core", "src")),
                                reason="Kokkos sources not present")


def build():
    lib = os.path.join(ROOT, "kokkos_gb300", "libgbk.so")
    if not os.path.exists(lib):
        import __graft_entry__
        __graft_entry__.build()
    jobs = str(max(2, min(16, os.cpu_count() or 4)))
    r = subprocess.run(["make", "-s", "-f", "tests/backend/Makefile", f"REF={os.path.abspath(REF)}", "-j" + jobs],
                       cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-6000:]
    return BIN


def test_backend_builds_against_kokkos_and_registers():
    b = build()
    from tests.conftest import has_gpu
    if has_gpu():
        pytest.skip("a GPU is present: the full program is the GPU check")
    r = subprocess.run([b, "--no-device"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
    assert r.returncode == 0, r.stdout
    assert r.stdout.startswith("registered: Kokkos::Experimental::GB300: initialize"), r.stdout


def test_reference_unit_test_compiles_for_the_space():
    """One of the reference's own unit-test headers (core/unit_test/
    TestReduce.hpp) compiles for the GB300 space through the test category
    of tests/backend/unit, with the reference's googletest; the whole set
    runs on a GPU machine from a copy of the Kokkos sources."""
    if not os.path.isdir(os.path.join(REF, "core", "unit_test")) or \
            not os.path.isdir(os.path.join(REF, "tpls", "gtest")):
        pytest.skip("Kokkos unit-test sources not present")
    build()
    target = "tests/backend/_build/unit/gb300_Reduce.o"  # the Makefile's default OUT, relative to the repository
    obj = os.path.join(ROOT, target)
    r = subprocess.run(["make", "-s", "-f", "tests/backend/Makefile", f"REF={os.path.abspath(REF)}", target],
                       cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-6000:]
    assert os.path.getsize(obj) > 0
