"""Parity of the GPU radix sort, sort_by_key and BinSort (through the C ABI)
with the reference's golden outputs and the oracle; keys and stable
permutations bit-exact.  Full-size checks (2^27 u64 keys + int32 payload)
use size-independent properties that determine the stable sort uniquely:
keys non-decreasing, payload a permutation of 0..n-1, keys[i] ==
input[payload[i]], and payload increasing inside every run of equal keys."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")
SIGNED = {np.dtype(np.uint64): np.int64, np.dtype(np.uint32): np.int32}


@pytest.fixture(scope="module")
def env():
    import torch

    from kokkos_gb300 import gbk
    torch.cuda.set_device(0)
    return gbk, torch


def _dev(torch, a):
    a = np.ascontiguousarray(a)
    if a.dtype in SIGNED:
        a = a.view(SIGNED[a.dtype])
    return torch.from_numpy(a).cuda()


def _host(t, dtype):
    a = t.cpu().numpy()
    return a.view(dtype) if np.dtype(dtype) in SIGNED else a


def check_stable_sort(orig_keys, keys, payload):
    n = orig_keys.size
    assert keys.size == n and payload.size == n
    assert np.all(keys[1:] >= keys[:-1]), "keys not sorted"
    seen = np.zeros(n, dtype=bool)
    seen[payload] = True
    assert seen.all(), "payload is not a permutation"
    assert np.array_equal(orig_keys[payload], keys), "keys do not follow the payload"
    eq = keys[1:] == keys[:-1]
    assert np.all(payload[1:][eq] > payload[:-1][eq]), "equal keys out of input order"


@pytest.mark.parametrize("dist", ["uniform", "lowentropy"])
def test_golden_sorts(env, dist):
    gbk, torch = env
    G = np.load(GOLDEN)
    n = 12000
    keys = G[f"sort/{dist}/{n}/x"]
    want = np.frombuffer(G[f"sort/{dist}/{n}/out"].tobytes(), np.uint64)
    d = _dev(torch, keys)
    gbk.sort(d, dt=3)
    gbk.stream_check()
    np.testing.assert_array_equal(_host(d, np.uint64), want)
    # stable permutation = reference Kokkos::sort of (key, index) pairs
    want_perm = np.frombuffer(G[f"sortstable/{dist}/{n}/out"].tobytes(), np.int32)
    dk = _dev(torch, keys)
    dv = torch.arange(n, dtype=torch.int32, device="cuda")
    gbk.sort_by_key(dk, dv, dt=3)
    gbk.stream_check()
    np.testing.assert_array_equal(dv.cpu().numpy(), want_perm)
    np.testing.assert_array_equal(_host(dk, np.uint64), want)
    # the reference's own (unstable) sort_by_key agrees on keys
    raw = G[f"sortbykey/{dist}/{n}/out"].tobytes()
    np.testing.assert_array_equal(np.frombuffer(raw[: 8 * n], np.uint64), want)


@pytest.mark.parametrize("kdt", [np.uint32, np.uint64, np.int32, np.int64, np.float32, np.float64])
@pytest.mark.parametrize("n", [0, 1, 2, 31, 4095, 4096, 4097, 300007])
def test_sort_key_types_vs_oracle(env, kdt, n):
    gbk, torch = env
    from kokkos_gb300 import datagen
    t = np.dtype(kdt)
    if t.kind == "f":
        k = datagen.normal_f64(n, seed=n).astype(t) * 1000
        if n > 10:
            k[3] = -0.0
            k[5] = 0.0
            k[7] = np.inf
            k[9] = -np.inf
    elif t.kind == "i":
        k = datagen.uniform_i64(n, -(1 << 30), 1 << 30, seed=n).astype(t)
        if t == np.int64 and n > 4:
            k[1] = np.iinfo(np.int64).min
            k[2] = np.iinfo(np.int64).max
    else:
        k = datagen.bits_u64(n, seed=n).astype(t)
    code = {np.dtype(np.int32): 0, np.dtype(np.int64): 1, np.dtype(np.uint32): 2, np.dtype(np.uint64): 3,
            np.dtype(np.float32): 4, np.dtype(np.float64): 5}[t]
    d = _dev(torch, k)
    gbk.sort(d, dt=code)
    gbk.stream_check()
    got = _host(d, t)
    want = np.sort(k, kind="stable")
    assert got.tobytes() == want.tobytes() or (t.kind == "f" and np.array_equal(got, want))
    # pairs: 8-byte values
    dk = _dev(torch, k)
    dv = torch.arange(n, dtype=torch.int64, device="cuda")
    gbk.sort_by_key(dk, dv, dt=code)
    gbk.stream_check()
    perm = dv.cpu().numpy()
    if t.kind == "f":
        # order by the radix image: -0.0 before +0.0
        img = k.view(np.uint32 if t.itemsize == 4 else np.uint64)
        sign = img >> (8 * t.itemsize - 1)
        rad = np.where(sign == 1, ~img, img | (np.array(1, img.dtype) << (8 * t.itemsize - 1)))
        check_stable_sort(rad, rad[perm], perm)
    else:
        check_stable_sort(k, k[perm], perm)


@pytest.mark.parametrize("kdt,vbytes", [(np.uint32, 0), (np.uint32, 4), (np.uint32, 8), (np.uint64, 0),
                                        (np.uint64, 4), (np.uint64, 8)])
@pytest.mark.parametrize("n", [152 * 4096 * 2 + 3, (1 << 21) + 1, 5 * 8192 - 1])
def test_sort_ragged_chunks(env, kdt, vbytes, n):
    """Sizes that give many chunks of whole tiles with a ragged last tile and
    a tail shorter than one 16-byte group, for every key / payload width."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    k = datagen.bits_u64(n, seed=n + vbytes).astype(kdt)
    code = 2 if kdt == np.uint32 else 3
    dk = _dev(torch, k)
    if vbytes == 0:
        gbk.sort(dk, dt=code)
        gbk.stream_check()
        assert _host(dk, kdt).tobytes() == np.sort(k, kind="stable").tobytes()
        return
    dv = torch.arange(n, dtype=torch.int32 if vbytes == 4 else torch.int64, device="cuda")
    gbk.sort_by_key(dk, dv, dt=code)
    gbk.stream_check()
    check_stable_sort(k, _host(dk, kdt), dv.cpu().numpy())


@pytest.mark.parametrize("kdt,off", [(np.uint64, 1), (np.uint32, 1), (np.uint32, 3)])
def test_sort_unaligned_buffers(env, kdt, off):
    """Caller buffers that start off a 16-byte boundary: the passes that read
    them use plain loads instead of bulk copies."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    n = 300007
    k = datagen.bits_u64(n, seed=7).astype(kdt)
    base = _dev(torch, np.concatenate([np.zeros(off, dtype=kdt), k]))
    dk = base[off:]
    assert dk.data_ptr() % 16 != 0
    vbase = torch.arange(-1, n, dtype=torch.int32, device="cuda")
    dv = vbase[1:]
    assert dv.data_ptr() % 16 != 0
    gbk.sort_by_key(dk, dv, dt=2 if kdt == np.uint32 else 3)
    gbk.stream_check()
    check_stable_sort(k, _host(dk, kdt), dv.cpu().numpy())
    assert int(vbase[0].item()) == -1 and _host(base[:off], kdt).tolist() == [0] * off


@pytest.mark.parametrize("ndistinct", [1, 2, 3, 255, 257])
def test_sort_few_distinct_keys(env, ndistinct):
    """Heavy duplicates: every tile holds long runs of one digit."""
    gbk, torch = env
    n = 1 << 20
    rng = np.random.default_rng(ndistinct)
    vals = rng.integers(0, 1 << 63, size=ndistinct, dtype=np.uint64)
    k = vals[rng.integers(0, ndistinct, size=n)]
    dk, dv = _dev(torch, k), torch.arange(n, dtype=torch.int32, device="cuda")
    gbk.sort_by_key(dk, dv, dt=3)
    gbk.stream_check()
    check_stable_sort(k, _host(dk, np.uint64), dv.cpu().numpy())


def test_all_keys_equal_and_one_varying_digit(env):
    gbk, torch = env
    n = 100003
    k = np.full(n, 0xDEADBEEF12345678, dtype=np.uint64)
    dk, dv = _dev(torch, k), torch.arange(n, dtype=torch.int32, device="cuda")
    gbk.sort_by_key(dk, dv, dt=3)
    gbk.stream_check()
    np.testing.assert_array_equal(dv.cpu().numpy(), np.arange(n, dtype=np.int32))
    k2 = k.copy()
    k2 ^= (np.arange(n, dtype=np.uint64) % 7) << np.uint64(56)  # only the top digit varies
    dk, dv = _dev(torch, k2), torch.arange(n, dtype=torch.int32, device="cuda")
    gbk.sort_by_key(dk, dv, dt=3)
    gbk.stream_check()
    check_stable_sort(k2, _host(dk, np.uint64), dv.cpu().numpy())


@pytest.mark.parametrize("dist", ["uniform", "lowentropy"])
def test_c4_sort_by_key_full_size(env, dist):
    """Kokkos::sort / sort_by_key of 2^27 uint64 keys with int32 payload
    (payload = iota), stable."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    n = 1 << 27
    keys = datagen.bits_u64(n, seed=0) if dist == "uniform" else datagen.lowentropy_u64(n, 8, seed=0)[0]
    dk = _dev(torch, keys)
    dv = torch.arange(n, dtype=torch.int32, device="cuda")
    gbk.sort_by_key(dk, dv, dt=3)
    gbk.stream_check()
    check_stable_sort(keys, _host(dk, np.uint64), dv.cpu().numpy())


def test_golden_binsort(env):
    gbk, torch = env
    G = np.load(GOLDEN)
    keys = G["binsort/20000/1000/x"]
    o = np.frombuffer(G["binsort/20000/1000/out"].tobytes(), np.int64)
    nbb = int(o[0])
    mul = o[1:2].view(np.float64)[0]
    cnt, off, perm = o[2:2 + nbb], o[2 + nbb:2 + 2 * nbb], o[2 + 2 * nbb:]
    c, of, p = gbk.binsort(_dev(torch, keys), nbb, float(keys.min()), mul)
    gbk.stream_check()
    np.testing.assert_array_equal(c.cpu().numpy(), cnt)
    np.testing.assert_array_equal(of.cpu().numpy(), off)
    pp = p.cpu().numpy()
    for b in range(nbb):
        s, e = off[b], off[b] + cnt[b]
        assert sorted(perm[s:e]) == list(pp[s:e])  # same bin contents, stable order here
    # sort_within_bins: fully sorted keys; applying the permutation sorts them
    c, of, p = gbk.binsort(_dev(torch, keys), nbb, float(keys.min()), mul, sort_within_bins=True)
    sk = gbk.permute(_dev(torch, keys), p)
    gbk.stream_check()
    np.testing.assert_array_equal(_host(sk, np.uint64), np.sort(keys))
    np.testing.assert_array_equal(c.cpu().numpy(), cnt)


def test_binsort_vs_oracle_many_bins(env):
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    n = 1 << 20
    keys = datagen.uniform_i64(n, 5, 1 << 40, seed=3).astype(np.uint64)
    kmin, kmax = int(keys.min()), int(keys.max())
    nb_req = n // 2
    mul = float(nb_req) / (float(kmax) - float(kmin))
    nbb = nb_req + 1
    c, of, p = gbk.binsort(_dev(torch, keys), nbb, float(kmin), mul)
    gbk.stream_check()
    wc, wo, wp = oracle.binsort(keys, nbb, float(kmin), mul)
    np.testing.assert_array_equal(c.cpu().numpy(), wc)
    np.testing.assert_array_equal(of.cpu().numpy(), wo)
    np.testing.assert_array_equal(p.cpu().numpy(), wp)


@pytest.mark.parametrize("varying_bytes", [8, 3])
def test_graph_with_sort_replays_against_oracle(env, varying_bytes):
    """Experimental::Graph holding a sort: refill the keys and an iota payload
    (device copies), sort_by_key, exclusive_scan of the sorted payload into
    int64, and a Max of the scan, captured once and replayed three times.
    Every replay is checked against the oracle (the stable sort by key, the
    reference OpenMP scan and reduce restated).  Keys where only 3 of the 8
    bytes vary leave 5 constant-digit passes to the device-side plan and an
    odd number of passes, so the data ends in the temporaries and the final
    copy-back runs inside the graph."""
    gbk, torch = env
    import ctypes

    import oracle
    from kokkos_gb300 import datagen
    n = 300007
    kh = datagen.bits_u64(n, seed=5)
    if varying_bytes < 8:
        keep = np.uint64(sum(0xFF << (8 * b) for b in (1, 4, 6)))
        kh = (kh & keep) | np.uint64(0x0101010101010101) & ~keep
    iota = np.arange(n, dtype=np.int32)
    k0, v0 = _dev(torch, kh), _dev(torch, iota)
    k, v = torch.empty_like(k0), torch.empty_like(v0)
    y = torch.empty(n, dtype=torch.int64, device="cuda")
    res = torch.zeros(16, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    P = ctypes.c_void_p
    gbk.check(gbk.lib.gbk_workspace_reserve(sp, 64 << 20), "reserve")

    def chain():
        gbk.check(gbk.lib.gbk_deep_copy(P(k.data_ptr()), P(k0.data_ptr()), n * 8, sp), "copy keys")
        gbk.check(gbk.lib.gbk_deep_copy(P(v.data_ptr()), P(v0.data_ptr()), n * 4, sp), "copy payload")
        gbk.check(gbk.lib.gbk_sort_by_key(3, P(k.data_ptr()), 4, P(v.data_ptr()), n, sp), "sort_by_key")
        gbk.scan(v, y, inclusive=False, init=0, stream=s)
        gbk.reduce("max", y, out=res[0:8], stream=s)

    with torch.cuda.stream(s):
        chain()  # uncaptured once: the workspace exists before the capture
    gbk.stream_check(s)
    ks, perm = oracle.sort_by_key_stable(kh, iota)
    want_y = oracle.scan(perm, np.int64, inclusive=False, init=0, nthreads=4)
    want_max = oracle.reduce("max", want_y, 4)
    g = gbk.Graph(s)
    with g:
        chain()
    for _ in range(3):
        k.zero_()
        y.zero_()
        res.zero_()
        torch.cuda.synchronize()
        g.submit()
        gbk.stream_check(s)
        np.testing.assert_array_equal(_host(k, np.uint64), ks)
        np.testing.assert_array_equal(v.cpu().numpy(), perm)
        np.testing.assert_array_equal(y.cpu().numpy(), want_y)
        assert gbk.decode_result(res.cpu().numpy()[:8], 3, 1) == want_max
