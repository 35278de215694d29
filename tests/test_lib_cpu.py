"""CPU-only checks: the C-ABI library loads and exports every symbol the
header declares, status strings, and the host-side generator's determinism.
No kernel is launched here."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def gbk():
    lib = os.path.join(ROOT, "kokkos_gb300", "libgbk.so")
    if not os.path.exists(lib):
        import __graft_entry__
        __graft_entry__.build()
    from kokkos_gb300 import gbk as g
    return g


def test_exports_every_declared_symbol(gbk):
    names = gbk.declared_symbols()
    assert len(names) >= 80
    out = subprocess.run(["nm", "-D", "--defined-only", gbk.LIB_PATH], capture_output=True, text=True, check=True)
    exported = {ln.split()[-1] for ln in out.stdout.splitlines() if ln.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(gbk.lib, n)


def test_status_strings_and_version(gbk):
    assert gbk.lib.gbk_version() >= 100
    for s in range(0, 8):
        assert gbk.lib.gbk_status_string(s)
    assert b"unknown" in gbk.lib.gbk_status_string(99)


def test_argument_errors_without_device(gbk):
    # Invalid arguments are rejected before any device call.
    assert gbk.lib.gbk_reduce(0, 0, None, -1, ctypes.c_void_p(8), None, None) == 1
    assert gbk.lib.gbk_reduce(4, 4, None, 0, ctypes.c_void_p(8), None, None) == 2  # LAnd on float
    assert gbk.lib.gbk_reduce(99, 0, None, 0, ctypes.c_void_p(8), None, None) == 2
    assert gbk.lib.gbk_scan(0, 0, 4, None, 0, None, None, None, None, None) == 2  # i32 -> f32 not a pair
    assert gbk.lib.gbk_scan(0, 0, 1, None, 5, None, None, None, None, None) == 1  # null buffers
    assert gbk.lib.gbk_histogram_i32_i64(None, 10, None, 0, None, None) == 1
    assert gbk.lib.gbk_set_wait_limit(0) == 1
    buf = ctypes.create_string_buffer(512)
    assert gbk.lib.gbk_fence_read(None, ctypes.c_void_p(8), buf, 257) == 1  # more than the 256-byte slot
    assert gbk.lib.gbk_fence_read(None, None, buf, 8) == 1                  # no source
    assert gbk.lib.gbk_fence_read(None, ctypes.c_void_p(8), buf, -1) == 1


def test_datagen_deterministic_and_blocked():
    from kokkos_gb300 import datagen
    a = datagen.uniform_f64(200000, seed=0)
    b = datagen.uniform_f64(200000, seed=0)
    assert a.tobytes() == b.tobytes()
    c = datagen.uniform_f64(70000, seed=0)
    assert c.tobytes() == a[:70000].tobytes()  # block-seeded: prefix independent of n
    assert 0.0 <= a.min() and a.max() < 1.0 and abs(a.mean() - 0.5) < 0.01
    z = datagen.zipf_i32(1 << 20, 1 << 16, 1.1, seed=0)
    assert z.min() >= 0 and z.max() < (1 << 16)
    frac0 = (z == 0).mean()
    assert 0.12 < frac0 < 0.15  # p(rank 1) = 1/H_{65536,1.1} ~ 0.137
    k, pos = datagen.lowentropy_u64(1 << 16, 8, seed=0)
    assert len(np.unique(k)) <= 256 and len(set(pos.tolist())) == 8
    lens, sigma = datagen.lognormal_lengths(10000, seed=0)
    assert abs(lens.sum() - (1 << 28)) / (1 << 28) < 0.02 and lens.max() <= (1 << 21) and lens.min() >= 1
    assert abs(np.median(lens) - 2048) / 2048 < 0.1 and 1.5 < sigma < 3.5


def test_fill_argument_errors_without_device(gbk):
    v = ctypes.c_int64(7)
    assert gbk.lib.gbk_fill(None, ctypes.byref(v), 8, -1, None) == 1
    assert gbk.lib.gbk_fill(None, ctypes.byref(v), 3, 4, None) == 1  # element size
    assert gbk.lib.gbk_fill(None, None, 8, 4, None) == 1
    assert gbk.lib.gbk_fill(ctypes.c_void_p(12), ctypes.byref(v), 8, 4, None) == 1  # misaligned element
    assert gbk.lib.gbk_fill(None, ctypes.byref(v), 8, 0, None) == 0
