"""Data movement either side of the reduce / scan path: deep_copy(view,
value) through gbk_fill (ragged heads and tails, every element size),
deep_copy between buffers, and permute, each against numpy on the same
seeded data."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    from kokkos_gb300 import gbk
    torch.cuda.set_device(0)
    return gbk, torch


@pytest.mark.parametrize("dtype", ["uint8", "int16", "int32", "float32", "int64", "float64"])
@pytest.mark.parametrize("offset", [0, 1, 3])
@pytest.mark.parametrize("n", [0, 1, 5, 17, 4099, (1 << 20) + 3])
def test_fill_matches_full(env, dtype, offset, n):
    gbk, torch = env
    td = getattr(torch, dtype)
    base = torch.zeros(n + offset + 9, dtype=td, device="cuda")
    base.fill_(0)
    view = base[offset:offset + n]
    value = {"uint8": 201, "int16": -12345, "int32": -7, "float32": 3.25, "int64": -(1 << 40) - 3,
             "float64": -1.0e-300}[dtype]
    gbk.fill(view, value)
    gbk.stream_check()
    got = base.cpu().numpy()
    want = np.zeros_like(got)
    want[offset:offset + n] = np.array(value).astype(got.dtype)
    assert got.tobytes() == want.tobytes()


def test_fill_sixteen_byte_elements(env):
    gbk, torch = env
    n = 1000
    buf = torch.zeros(2 * n + 2, dtype=torch.int64, device="cuda")
    val = np.array([0x0123456789ABCDEF, -5], dtype=np.int64)
    assert gbk.lib.gbk_fill(ctypes.c_void_p(buf.data_ptr() + 16), ctypes.c_void_p(val.ctypes.data), 16, n - 1,
                            None) == 0
    gbk.stream_check()
    got = buf.cpu().numpy().reshape(-1, 2)
    assert np.all(got[1:n] == val) and np.all(got[0] == 0) and np.all(got[n:] == 0)


def test_deep_copy_and_permute(env):
    gbk, torch = env
    from kokkos_gb300 import datagen
    n = (1 << 22) + 7
    x = datagen.uniform_i64(n, -(1 << 40), 1 << 40, seed=3)
    hx = torch.from_numpy(x).pin_memory()
    d = torch.empty(n, dtype=torch.int64, device="cuda")
    assert gbk.lib.gbk_deep_copy(ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(hx.data_ptr()), n * 8, None) == 0
    d2 = torch.empty_like(d)
    assert gbk.lib.gbk_deep_copy(ctypes.c_void_p(d2.data_ptr()), ctypes.c_void_p(d.data_ptr()), n * 8, None) == 0
    gbk.stream_check()
    np.testing.assert_array_equal(d2.cpu().numpy(), x)
    perm = np.random.default_rng(5).permutation(n).astype(np.int64)
    for dt in (torch.int64, torch.int32, torch.int16, torch.uint8):
        src = d2.to(dt)
        got = gbk.permute(src, torch.from_numpy(perm).cuda())
        gbk.stream_check()
        np.testing.assert_array_equal(got.cpu().numpy(), src.cpu().numpy()[perm])
