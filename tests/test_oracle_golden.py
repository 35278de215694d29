"""Pin the oracle (oracle/oracle.cpp) to golden vectors produced by the
reference Kokkos OpenMP backend itself (tests/golden/make_golden.py).

Everything here is bit-exact, floating point included: the oracle restates
the OpenMP work partition and join order for the same thread count, so its
Sum/Prod of floats must reproduce the reference's bits.
"""
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")


@pytest.fixture(scope="module")
def G():
    return np.load(GOLDEN)


def _cases(G, prefix):
    return sorted({k.rsplit("/", 1)[0] for k in G.files if k.startswith(prefix) and k.endswith("/out")})


def test_reduce_all_reducers_bit_exact(G):
    n_checked = 0
    for k in _cases(G, "reduce/"):
        _, op, dt, n, P = k.split("/")
        x = G[f"reduce/{op}/{dt}/{n}/x"]
        want = G[k + "/out"].tobytes()
        got = oracle.reduce(op, x, int(P))
        got_b = np.asarray(got).tobytes()
        # Padding bytes in ValLoc<float> are not part of the value.
        rd = oracle.result_dtype(op, x.dtype)
        w = np.frombuffer(want, dtype=rd)[0]
        for name in (rd.names or [None]):
            a = got[name] if name else got
            b = w[name] if name else w
            assert np.asarray(a).tobytes() == np.asarray(b).tobytes(), (k, name, a, b)
        n_checked += 1
        del got_b
    assert n_checked > 300


def test_std_reduce(G):
    x = G["stdreduce/f64/65536/4/x"]
    want = np.frombuffer(G["stdreduce/f64/65536/4/out"].tobytes(), np.float64)[0]
    assert oracle.reduce("sum", x, 4).tobytes() == want.tobytes()


@pytest.mark.parametrize("n", [0, 1, 1000, 20011])
@pytest.mark.parametrize("P", [1, 4])
def test_scans(G, n, P):
    x = G[f"scan/i32/{n}/x"]
    for init in (0, 7):
        want = np.frombuffer(G[f"exscan/i32_i64/{n}/{init}/{P}/out"].tobytes(), np.int64)
        np.testing.assert_array_equal(oracle.scan(x, np.int64, inclusive=False, init=init, nthreads=P), want)
    want = np.frombuffer(G[f"inscan/i32/{n}/{P}/out"].tobytes(), np.int32)
    np.testing.assert_array_equal(oracle.scan(x, np.int32, inclusive=True, nthreads=P), want)
    xf = G[f"scan/f64/{n}/x"]
    want = np.frombuffer(G[f"inscan/f64/{n}/{P}/out"].tobytes(), np.float64)
    got = oracle.scan(xf, np.float64, inclusive=True, nthreads=P)
    assert got.tobytes() == want.tobytes()
    xl = G[f"scan/i64/{n}/x"]
    want = np.frombuffer(G[f"scantotal/i64/{n}/{P}/out"].tobytes(), np.int64)
    got = oracle.scan(xl, np.int64, inclusive=False, nthreads=P)
    np.testing.assert_array_equal(got, want[:n])
    assert int(want[n]) == int(xl.sum())


@pytest.mark.parametrize("shape", [(37, 19, 11), (64, 32, 16)])
def test_mdrange_leftlayout(G, shape):
    n0, n1, n2 = shape
    x = G[f"mdrange/f32/{n0}x{n1}x{n2}/x"]
    for P in (1, 4):
        for op in ("minloc", "maxloc"):
            rd = oracle.result_dtype(op, np.float32)
            want = np.frombuffer(G[f"mdrange/{op}/f32/{n0}x{n1}x{n2}/{P}/out"].tobytes(), rd)[0]
            got = oracle.mdrange_reduce(op, x, [0, 0, 0], [n0, n1, n2], [1, n0, n0 * n1], P)
            assert got["val"] == want["val"] and got["loc"] == want["loc"], (op, got, want)
        want = np.frombuffer(G[f"mdrange/sum/f32/{n0}x{n1}x{n2}/{P}/out"].tobytes(), np.float32)[0]
        got = oracle.mdrange_reduce("sum", x, [0, 0, 0], [n0, n1, n2], [1, n0, n0 * n1], P)
        # the host tile walk is restated, so the float sum matches bit for bit
        assert got.tobytes() == want.tobytes(), (P, got, want)


@pytest.mark.parametrize("case", [(100000, 4096), (5000, 65536), (0, 16)])
def test_histogram(G, case):
    n, nb = case
    keys = G[f"hist/{n}/{nb}/x"]
    for P in (1, 4):
        want = np.frombuffer(G[f"hist/{n}/{nb}/{P}/out"].tobytes(), np.int64)
        got, dropped = oracle.histogram(keys, nb, P)
        np.testing.assert_array_equal(got, want)
        assert dropped == 0


@pytest.mark.parametrize("dist", ["uniform", "lowentropy"])
def test_sorts(G, dist):
    n = 12000
    keys = G[f"sort/{dist}/{n}/x"]
    want = np.frombuffer(G[f"sort/{dist}/{n}/out"].tobytes(), np.uint64)
    np.testing.assert_array_equal(oracle.sort_u64(keys), want)
    # Stable permutation == reference Kokkos::sort with a (key, index) comparator.
    want_perm = np.frombuffer(G[f"sortstable/{dist}/{n}/out"].tobytes(), np.int32)
    k2, v2 = oracle.sort_by_key_stable(keys, np.arange(n, dtype=np.int32))
    np.testing.assert_array_equal(v2, want_perm)
    np.testing.assert_array_equal(k2, want)
    # The reference sort_by_key (unstable) agrees on keys; on distinct keys
    # it also agrees on the permutation.
    raw = G[f"sortbykey/{dist}/{n}/out"].tobytes()
    rk = np.frombuffer(raw[: 8 * n], np.uint64)
    rv = np.frombuffer(raw[8 * n:], np.int32)
    np.testing.assert_array_equal(rk, want)
    assert np.array_equal(keys[rv], rk)
    if len(np.unique(keys)) == n:
        np.testing.assert_array_equal(rv, want_perm)


def test_binsort(G):
    keys = G["binsort/20000/1000/x"]
    o = np.frombuffer(G["binsort/20000/1000/out"].tobytes(), np.int64)
    nbb = int(o[0])
    mul = o[1:2].view(np.float64)[0]
    cnt = o[2:2 + nbb]
    off = o[2 + nbb:2 + 2 * nbb]
    perm = o[2 + 2 * nbb:]
    c, of, p = oracle.binsort(keys, nbb, float(keys.min()), mul)
    np.testing.assert_array_equal(c, cnt)
    np.testing.assert_array_equal(of, off)
    # The reference bins with atomics, so the order inside a bin is
    # arbitrary; the oracle's order is the stable one.  Same bin contents:
    for b in range(nbb):
        s, e = off[b], off[b] + cnt[b]
        assert sorted(perm[s:e]) == sorted(p[s:e]) == list(p[s:e])


def test_team_reduce(G):
    offs = G["teamreduce/f64/50/offsets"]
    x = G["teamreduce/f64/50/x"]
    want = np.frombuffer(G["teamreduce/f64/50/out"].tobytes(), np.float64)
    for s in range(50):
        seg = x[offs[s]:offs[s + 1]]
        c, a, _ = oracle.sum_compensated(seg)
        assert abs(want[s] - c) <= 1e-12 * max(a, 1e-300)
