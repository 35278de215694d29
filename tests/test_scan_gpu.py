"""Parity of the single-pass GPU scans (through the C ABI) with the oracle
and the reference's golden outputs; integer scans bit-exact."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")


@pytest.fixture(scope="module")
def env():
    import torch

    from kokkos_gb300 import gbk
    torch.cuda.set_device(0)
    return gbk, torch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_golden_scans(env):
    gbk, torch = env
    G = np.load(GOLDEN)
    for n in [0, 1, 1000, 20011]:
        x = G[f"scan/i32/{n}/x"]
        for init in (0, 7):
            want = np.frombuffer(G[f"exscan/i32_i64/{n}/{init}/4/out"].tobytes(), np.int64)
            y = torch.empty(n, dtype=torch.int64, device="cuda")
            gbk.scan(_dev(torch, x), y, inclusive=False, init=init)
            np.testing.assert_array_equal(y.cpu().numpy(), want)
        want = np.frombuffer(G[f"inscan/i32/{n}/4/out"].tobytes(), np.int32)
        y = torch.empty(n, dtype=torch.int32, device="cuda")
        gbk.scan(_dev(torch, x), y, inclusive=True)
        np.testing.assert_array_equal(y.cpu().numpy(), want)
        xl = G[f"scan/i64/{n}/x"]
        want = np.frombuffer(G[f"scantotal/i64/{n}/4/out"].tobytes(), np.int64)
        y = torch.empty(n, dtype=torch.int64, device="cuda")
        tot = torch.zeros(1, dtype=torch.int64, device="cuda")
        gbk.scan(_dev(torch, xl), y, inclusive=False, total=tot)
        np.testing.assert_array_equal(y.cpu().numpy(), want[:n])
        assert int(tot.item()) == int(want[n])
        xf = G[f"scan/f64/{n}/x"]
        want = np.frombuffer(G[f"inscan/f64/{n}/4/out"].tobytes(), np.float64)
        y = torch.empty(n, dtype=torch.float64, device="cuda")
        gbk.scan(_dev(torch, xf), y, inclusive=True)
        if n:
            ya = y.cpu().numpy()
            scale = np.cumsum(np.abs(xf))
            assert np.all(np.abs(ya - want) <= 1e-12 * np.maximum(scale, 1e-300))
    gbk.stream_check()


@pytest.mark.parametrize("n", [1, 5, 4095, 4096, 4097, 123457, (1 << 22) + 3])
@pytest.mark.parametrize("pair", [("i32", "i64"), ("i32", "i32"), ("i64", "i64"), ("u32", "u64"), ("u64", "u64")])
def test_int_scans_vs_oracle(env, n, pair):
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    tin, tout = gbk.NP[gbk.DT[pair[0]]], gbk.NP[gbk.DT[pair[1]]]
    x = datagen.uniform_i64(n, 0, 255, seed=n).astype(tin)
    d = _dev(torch, x)
    for incl in (False, True):
        y = torch.empty(n, dtype=getattr(torch, np.dtype(tout).name), device="cuda")
        gbk.scan(d, y, inclusive=incl, init=None if incl else 11)
        want = oracle.scan(x, tout, inclusive=incl, init=11, nthreads=3)
        np.testing.assert_array_equal(y.cpu().numpy(), want)
    gbk.stream_check()


@pytest.mark.parametrize("pair", [("f32", "f32"), ("f32", "f64"), ("f64", "f64")])
def test_float_scans(env, pair):
    gbk, torch = env
    from kokkos_gb300 import datagen
    n = 300001
    tin, tout = gbk.NP[gbk.DT[pair[0]]], gbk.NP[gbk.DT[pair[1]]]
    x = datagen.normal_f64(n, seed=4).astype(tin)
    d = _dev(torch, x)
    y = torch.empty(n, dtype=getattr(torch, np.dtype(tout).name), device="cuda")
    gbk.scan(d, y, inclusive=True)
    exact = np.cumsum(x.astype(np.float64))
    scale = np.cumsum(np.abs(x.astype(np.float64)))
    rel = 1e-12 if tout == np.float64 else 1e-5
    assert np.all(np.abs(y.cpu().numpy().astype(np.float64) - exact) <= rel * scale + 1e-30)


def test_c1_exclusive_scan_full_size(env):
    """Experimental::exclusive_scan of View<int32*> 2^24 uniform 0..15 into
    View<int64*>, seed 0: bit-exact."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    n = 1 << 24
    x = datagen.uniform_i32(n, 0, 15, seed=0)
    y = torch.empty(n, dtype=torch.int64, device="cuda")
    gbk.scan(_dev(torch, x), y, inclusive=False, init=0)
    gbk.stream_check()
    np.testing.assert_array_equal(y.cpu().numpy(), oracle.scan(x, np.int64, inclusive=False, init=0, nthreads=8))


def test_inplace_and_misaligned(env):
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    x = datagen.uniform_i64(50001, -9, 9, seed=2)
    d = _dev(torch, x)
    gbk.scan(d, d, inclusive=True)
    np.testing.assert_array_equal(d.cpu().numpy(), np.cumsum(x))
    xi = datagen.uniform_i32(70001, 0, 9, seed=3)
    di = _dev(torch, xi)[1:]
    yo = torch.empty(70001, dtype=torch.int64, device="cuda")[1:]
    gbk.scan(di, yo, inclusive=False, init=5)
    np.testing.assert_array_equal(yo.cpu().numpy(), oracle.scan(xi[1:], np.int64, inclusive=False, init=5))


@pytest.mark.parametrize("ipt,cps", [(3, 1), (3, 0), (7, 1), (7, 0), (9, 1), (9, 0)])
def test_tuned_ring_shapes(env, ipt, cps):
    """Every (vectors per thread, CTAs per SM) shape of the persistent grid,
    with few CTAs (many laps of the staging ring) and a ragged last tile;
    totals through ParallelScanWithTotal."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    for pair, n in [(("i32", "i64"), (1 << 23) + 13), (("i64", "i64"), 3 * 8192 + 1), (("u32", "u32"), 999_999)]:
        tin, tout = gbk.NP[gbk.DT[pair[0]]], gbk.NP[gbk.DT[pair[1]]]
        x = datagen.uniform_i64(n, 0, 1000, seed=ipt * 10 + cps).astype(tin)
        d = _dev(torch, x)
        y = torch.empty(n, dtype=getattr(torch, np.dtype(tout).name), device="cuda")
        tot = torch.zeros(1, dtype=y.dtype, device="cuda")
        gbk.scan(d, y, inclusive=False, init=3, total=tot, tune=(256, ipt, cps, 0))
        want = oracle.scan(x, tout, inclusive=False, init=3, nthreads=8)
        np.testing.assert_array_equal(y.cpu().numpy(), want)
        assert int(tot.item()) == int(want[-1]) + int(x[-1])
    gbk.stream_check()


def test_scan_2e28_properties(env):
    """2^28 int32 -> int64 (1 GiB in, 2 GiB out), checked on the device by
    size-independent properties: y[0] = init, y[i+1] - y[i] = x[i], total."""
    gbk, torch = env
    n = 1 << 28
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    x = torch.randint(0, 256, (n,), dtype=torch.int32, device="cuda", generator=g)
    y = torch.empty(n, dtype=torch.int64, device="cuda")
    tot = torch.zeros(1, dtype=torch.int64, device="cuda")
    gbk.scan(x, y, inclusive=False, init=-7, total=tot)
    gbk.stream_check()
    assert int(y[0].item()) == -7
    assert bool(torch.equal(y[1:] - y[:-1], x[:-1].to(torch.int64)))
    assert int(tot.item()) == -7 + int(x.sum(dtype=torch.int64).item())
    del y
    yi = torch.empty(n, dtype=torch.int32, device="cuda")
    xs = (x & 7).contiguous()
    gbk.scan(xs, yi, inclusive=True)
    gbk.stream_check()
    assert bool(torch.equal(yi[1:] - yi[:-1], xs[1:])) and int(yi[0].item()) == int(xs[0].item())


def test_many_launches_reuse_status_words(env):
    """Back-to-back scans of different sizes on one stream reuse the epoch-
    tagged status words without clearing them."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    for i, n in enumerate([100000, 7, 400000, 4096 * 3, 99999, 1 << 20]):
        x = datagen.uniform_i32(n, 0, 99, seed=i)
        y = torch.empty(n, dtype=torch.int64, device="cuda")
        gbk.scan(_dev(torch, x), y, inclusive=True)
        np.testing.assert_array_equal(y.cpu().numpy(), np.cumsum(x.astype(np.int64)))
    gbk.stream_check()


def test_bounded_wait_gives_up_cleanly(env):
    """The device-side wait bound (gbk_set_wait_limit) on the GPU: a scan of
    2^26 int32 values whose input starts off the 16-byte boundary (the
    plain-load kernel: its only waits are the look-back polls, no bulk copy is
    ever in flight) runs with a bound of one poll, so tiles whose predecessor
    has not published yet give up, publish what they have and end; the call
    reports GBK_ERR_DEVICE_TIMEOUT (or GBK_OK when no wait ran out), the GPU
    context stays usable, and the next scan at the default bound is exact."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    n = 1 << 26
    xh = datagen.uniform_i32(n, 0, 15, seed=4)
    x = _dev(torch, np.concatenate([np.zeros(1, np.int32), xh]))[1:]
    y = torch.empty(n, dtype=torch.int64, device="cuda")
    default = gbk.lib.gbk_wait_limit()
    assert default > 1000
    try:
        assert gbk.lib.gbk_set_wait_limit(1) == 0
        gbk.scan(x, y, inclusive=True)
        st = gbk.lib.gbk_stream_check(None)
        assert st in (0, 4), gbk.lib.gbk_status_string(st)
        print("bounded wait of one poll:", "timed out" if st == 4 else "no wait ran out")
    finally:
        assert gbk.lib.gbk_set_wait_limit(default) == 0
    gbk.scan(x, y, inclusive=True)
    gbk.stream_check()
    np.testing.assert_array_equal(y.cpu().numpy(), np.cumsum(xh, dtype=np.int64))
