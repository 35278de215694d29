"""Batched segmented reduce / scan (one launch for all segments) through the
C ABI vs the oracle's per-segment loops, the reference's TeamPolicy golden
output, and CUDA-graph capture of dependent reduce/scan chains."""
import os

import numpy as np
import pytest

from tests._util import sum_ok

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


def lengths_cases():
    from kokkos_gb300 import datagen
    rng = np.random.default_rng(1)
    yield "lognormal", datagen.lognormal_lengths(2000, median=300.0, max_len=1 << 16, target_total=1 << 20, seed=2)[0]
    yield "with_empty", rng.integers(0, 6, size=5000)           # many empty and tiny segments
    yield "one_huge", np.array([1 << 20])                          # a segment over hundreds of tiles
    yield "tile_edges", np.array([4096, 4096, 1, 4095, 8192, 0, 4097, 3])  # boundaries on tile edges
    yield "mixed", np.concatenate([rng.integers(1, 50, 300), [300000], rng.integers(0, 3000, 200)])


@pytest.mark.parametrize("case", list(lengths_cases()), ids=lambda c: c[0])
def test_segmented_vs_oracle(env, case):
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    _, lens = case
    offs = datagen.offsets_from_lengths(np.asarray(lens, dtype=np.int64))
    n = int(offs[-1])
    xf = datagen.normal_f32(n, seed=5)
    xi = datagen.uniform_i32(n, 0, 255, seed=6)
    do = _dev(torch, offs)
    nseg = offs.size - 1
    # float Sum per segment (tolerance), vs compensated sums
    out = torch.empty(nseg, dtype=torch.float32, device="cuda")
    gbk.segmented_reduce("sum", _dev(torch, xf), do, out)
    gbk.stream_check()
    got = out.cpu().numpy()
    _, comp, absum = oracle.seg_sum_f32(xf, offs, 4)
    for s in range(nseg):
        seg = xf[offs[s]:offs[s + 1]]
        ok, info = sum_ok(got[s], seg, 1e-5) if seg.size else (got[s] == 0.0, got[s])
        assert ok, (s, info)
    # int Sum / Min / Max exact
    for op in ("sum", "min", "max"):
        o = torch.empty(nseg, dtype=torch.int32, device="cuda")
        gbk.segmented_reduce(op, _dev(torch, xi), do, o)
        gbk.stream_check()
        w = np.array([getattr(np, {"sum": "sum", "min": "min", "max": "max"}[op])(xi[offs[s]:offs[s + 1]])
                      if offs[s + 1] > offs[s] else {"sum": 0, "min": 2**31 - 1, "max": -2**31}[op]
                      for s in range(nseg)], dtype=np.int64).astype(np.int32)
        np.testing.assert_array_equal(o.cpu().numpy(), w)
    # int32 inclusive scan per segment, exact
    y = torch.empty(n, dtype=torch.int32, device="cuda")
    gbk.segmented_scan(_dev(torch, xi), do, y, inclusive=True)
    gbk.stream_check()
    np.testing.assert_array_equal(y.cpu().numpy(), oracle.seg_inclusive_scan_i32(xi, offs, 4))
    # exclusive, widening to int64
    y64 = torch.empty(n, dtype=torch.int64, device="cuda")
    gbk.segmented_scan(_dev(torch, xi), do, y64, inclusive=False)
    gbk.stream_check()
    inc = oracle.seg_inclusive_scan_i32(xi, offs, 4).astype(np.int64)
    np.testing.assert_array_equal(y64.cpu().numpy(), inc - xi.astype(np.int64))


@pytest.mark.parametrize("ipt,cps", [(7, 0), (7, 1), (5, 0), (5, 1), (3, 0), (3, 2)])
def test_segmented_shapes(env, ipt, cps):
    """Every tile shape of the persistent kernel (7, 5 (scans: three stages)
    or 3 vectors per thread, all-resident or fewer CTAs), with segment
    boundaries on the tile edges of the shapes (7168 / 5120 / 3072 elements
    for 4-byte types, 3584 / 2560 / 1536 for 8-byte), empty segments next to
    them, and an unaligned input view."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    rng = np.random.default_rng(ipt * 10 + cps)
    lens = np.concatenate([[7168, 7168, 0, 1, 7167, 3584, 3584, 0, 0, 3072, 1536, 5, 14336, 6144, 5120, 0, 5120,
                            2560, 10240, 2559, 1],
                           rng.integers(0, 40, 400), [100000], rng.integers(0, 9000, 60)]).astype(np.int64)
    offs = datagen.offsets_from_lengths(lens)
    n = int(offs[-1])
    nseg = lens.size
    do = _dev(torch, offs)
    tune = (256, ipt, cps, 0)
    xi = datagen.uniform_i32(n + 1, 0, 255, seed=7)
    xl = datagen.uniform_i64(n, -1000, 1000, seed=8)
    for name, x in (("aligned", _dev(torch, xi[:n])), ("unaligned", _dev(torch, xi)[1:])):
        xh = xi[:n] if name == "aligned" else xi[1:]
        for op in ("sum", "min", "max"):
            o = torch.empty(nseg, dtype=torch.int32, device="cuda")
            gbk.segmented_reduce(op, x, do, o, tune=tune)
            gbk.stream_check()
            f = {"sum": np.sum, "min": np.min, "max": np.max}[op]
            ident = {"sum": 0, "min": 2**31 - 1, "max": -2**31}[op]
            w = np.array([f(xh[offs[s]:offs[s + 1]]) if lens[s] else ident for s in range(nseg)],
                         dtype=np.int64).astype(np.int32)
            np.testing.assert_array_equal(o.cpu().numpy(), w, err_msg=f"{name} {op}")
        y = torch.empty(n, dtype=torch.int32, device="cuda")
        gbk.segmented_scan(x, do, y, inclusive=True, tune=tune)
        gbk.stream_check()
        inc = oracle.seg_inclusive_scan_i32(np.ascontiguousarray(xh), offs, 4)
        np.testing.assert_array_equal(y.cpu().numpy(), inc, err_msg=name)
        y64 = torch.empty(n, dtype=torch.int64, device="cuda")
        gbk.segmented_scan(x, do, y64, inclusive=False, tune=tune)
        gbk.stream_check()
        np.testing.assert_array_equal(y64.cpu().numpy(), inc.astype(np.int64) - xh.astype(np.int64), err_msg=name)
    # 8-byte elements: tile edges at 3584 / 1536
    o = torch.empty(nseg, dtype=torch.int64, device="cuda")
    gbk.segmented_reduce("sum", _dev(torch, xl), do, o, tune=tune)
    gbk.stream_check()
    w = np.array([xl[offs[s]:offs[s + 1]].sum() for s in range(nseg)], dtype=np.int64)
    np.testing.assert_array_equal(o.cpu().numpy(), w)
    yl = torch.empty(n, dtype=torch.int64, device="cuda")
    gbk.segmented_scan(_dev(torch, xl), do, yl, inclusive=True, tune=tune)
    gbk.stream_check()
    cs = np.cumsum(xl)
    base = np.repeat(np.concatenate([[0], cs[offs[1:-1] - 1]]), lens) if n else cs
    np.testing.assert_array_equal(yl.cpu().numpy(), cs - base)


def test_segmented_all_empty(env):
    """n = 0 with segments: every segment is empty and gets the identity."""
    gbk, torch = env
    offs = np.zeros(9, dtype=np.int64)
    x = torch.empty(0, dtype=torch.float32, device="cuda")
    o = torch.full((8,), 5.0, dtype=torch.float32, device="cuda")
    gbk.segmented_reduce("sum", x, _dev(torch, offs), o)
    gbk.stream_check()
    assert o.cpu().numpy().tolist() == [0.0] * 8
    om = torch.zeros(8, dtype=torch.float32, device="cuda")
    gbk.segmented_reduce("max", x, _dev(torch, offs), om)
    gbk.stream_check()
    assert np.all(om.cpu().numpy() == np.float32(-3.402823466e38))


def test_golden_team_reduce(env):
    """TeamPolicy league of per-segment sums (reference TeamThreadRange
    reduce) — the batched reduce gives the same sums within 1e-12."""
    gbk, torch = env
    G = np.load(GOLDEN)
    offs = G["teamreduce/f64/50/offsets"]
    x = G["teamreduce/f64/50/x"]
    want = np.frombuffer(G["teamreduce/f64/50/out"].tobytes(), np.float64)
    out = torch.empty(50, dtype=torch.float64, device="cuda")
    gbk.segmented_reduce("sum", _dev(torch, x), _dev(torch, offs), out)
    gbk.stream_check()
    got = out.cpu().numpy()
    for s in range(50):
        a = np.abs(x[offs[s]:offs[s + 1]]).sum()
        assert abs(got[s] - want[s]) <= 1e-12 * max(a, 1e-300)


def test_c3_batched_full_size(env):
    """10,000 lognormal segments (median 2,048, max 2^21, total ~2^28):
    per-segment float Sum and int32 inclusive_scan, one launch each."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    lens, sigma = datagen.lognormal_lengths(10000, median=2048.0, max_len=1 << 21, target_total=1 << 28, seed=0)
    offs = datagen.offsets_from_lengths(lens)
    n = int(offs[-1])
    assert abs(n - (1 << 28)) / (1 << 28) < 0.02
    xf = datagen.normal_f32(n, seed=0)
    xi = datagen.uniform_i32(n, 0, 255, seed=0)
    do = _dev(torch, offs)
    out = torch.empty(10000, dtype=torch.float32, device="cuda")
    gbk.segmented_reduce("sum", _dev(torch, xf), do, out)
    y = torch.empty(n, dtype=torch.int32, device="cuda")
    gbk.segmented_scan(_dev(torch, xi), do, y, inclusive=True)
    gbk.stream_check()
    _, comp, absum = oracle.seg_sum_f32(xf, offs, 16)
    got = out.cpu().numpy().astype(np.float64)
    l2 = np.sqrt(np.add.reduceat(xf.astype(np.float64) ** 2, offs[:-1]))
    err = np.abs(got - comp)
    assert np.all((err <= 1e-5 * np.abs(comp)) | (err <= 1e-5 * l2))
    np.testing.assert_array_equal(y.cpu().numpy(), oracle.seg_inclusive_scan_i32(xi, offs, 16))


def test_graph_chain_of_dependent_nodes(env):
    """A CUDA graph of 8 dependent reduce/scan nodes (each node reads the
    previous node's output) replays to the results of the oracle (the
    reference's OpenMP scan and reduce restated, int64 arithmetic wrapping
    as two's complement in both) and of the same chain as stream launches,
    several times, interleaved with uncaptured scans."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    s = torch.cuda.Stream()
    n = 1 << 20
    xh = datagen.uniform_i32(n, 0, 15, seed=1)
    x = _dev(torch, xh)
    o0 = oracle.scan(xh, np.int64, inclusive=False, init=0, nthreads=4)
    o1 = oracle.scan(o0, np.int64, inclusive=True, nthreads=4)
    o2 = oracle.scan(o1, np.int64, inclusive=False, init=3, nthreads=4)
    o3 = oracle.scan(o2, np.int64, inclusive=True, nthreads=4)
    want_oracle = b"".join(np.asarray(r).tobytes() for r in (
        oracle.reduce("max", o0, 4), oracle.reduce("sum", o1, 4), oracle.reduce("minloc", o2[1:], 4),
        oracle.reduce("maxloc", o3, 4)))
    bufs = [torch.empty(n, dtype=torch.int64, device="cuda") for _ in range(4)]
    res = torch.zeros(64, dtype=torch.uint8, device="cuda")
    gbk.lib.gbk_workspace_reserve(__import__("ctypes").c_void_p(s.cuda_stream), 64 << 20)

    def chain():
        gbk.scan(x, bufs[0], inclusive=False, init=0, stream=s)           # 1 exclusive_scan i32 -> i64
        gbk.reduce("max", bufs[0], out=res[0:8], stream=s)                # 2 reduce of node 1's output
        gbk.scan(bufs[0], bufs[1], inclusive=True, stream=s)              # 3 inclusive scan of node 1
        gbk.reduce("sum", bufs[1], out=res[8:16], stream=s)               # 4
        gbk.scan(bufs[1], bufs[2], inclusive=False, init=3, stream=s)     # 5
        gbk.reduce("minloc", bufs[2][1:], out=res[16:32], stream=s)       # 6
        gbk.scan(bufs[2], bufs[3], inclusive=True, stream=s)              # 7
        gbk.reduce("maxloc", bufs[3], out=res[32:48], stream=s)           # 8

    with torch.cuda.stream(s):
        chain()
    s.synchronize()
    want = (res.cpu().numpy().copy(), bufs[3].cpu().numpy().copy())
    assert want[0][:48].tobytes() == want_oracle
    np.testing.assert_array_equal(want[1], o3)
    g = gbk.Graph(s)
    with g:
        chain()
    for rep in range(3):
        res.zero_()
        bufs[3].zero_()
        torch.cuda.synchronize()
        g.submit()
        # an uncaptured scan on the same stream between replays
        junk = torch.empty(n, dtype=torch.int64, device="cuda")
        gbk.scan(x, junk, inclusive=True, stream=s)
        s.synchronize()
        np.testing.assert_array_equal(res.cpu().numpy(), want[0])
        np.testing.assert_array_equal(bufs[3].cpu().numpy(), want[1])
    gbk.stream_check(s)


def share_cases():
    rng = np.random.default_rng(11)
    yield "one_segment_with_tail", np.array([(1 << 22) + 3])
    yield "empty_at_both_ends", np.concatenate([[0, 0, 0], rng.integers(1000, 200000, 40), [0, 0]])
    # more than 256 starts inside one 4096-element chunk (several windows of starts)
    yield "tiny_run", np.concatenate([rng.integers(5000, 100000, 20), rng.integers(0, 4, 30000),
                                      rng.integers(5000, 100000, 20), [7]])
    yield "random_sizes", rng.integers(0, 20000, 800)
    yield "chunk_multiples", np.array([4096] * 300 + [1024] * 100 + [24576] * 50 + [0, 4096, 0])


def _seg_expect(x, offs, op):
    lens = np.diff(offs)
    if op == "sum":
        cs = np.concatenate([[0], np.cumsum(x.astype(np.int64))])
        return (cs[offs[1:]] - cs[offs[:-1]]).astype(x.dtype)
    info = np.iinfo(x.dtype)
    out = np.full(lens.size, info.max if op == "min" else info.min, dtype=x.dtype)
    nz = lens > 0
    f = np.minimum if op == "min" else np.maximum
    out[nz] = f.reduceat(x, offs[:-1][nz])
    return out


@pytest.mark.parametrize("case", list(share_cases()), ids=lambda c: c[0])
def test_segmented_reduce_contiguous_shares(env, case):
    """The contiguous-share segmented reduce (the default for 16-byte aligned
    input of at least one chunk): segments across share and chunk edges,
    starts on them, more than 256 starts in one chunk, empty segments at both
    ends, a tail after the last whole vector, one segment over everything.
    Integers exact against numpy and against the tile-pipeline variant
    (variant 1); float and double Sum within the stated tolerances."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    _, lens = case
    offs = datagen.offsets_from_lengths(np.asarray(lens, dtype=np.int64))
    n = int(offs[-1])
    nseg = offs.size - 1
    do = _dev(torch, offs)
    xi = datagen.uniform_i32(n, 0, 255, seed=21)
    xl = datagen.uniform_i64(n, -(1 << 40), 1 << 40, seed=22)
    for x in (xi, xl):
        dx = _dev(torch, x)
        for op in ("sum", "min", "max"):
            want = _seg_expect(x, offs, op)
            for variant in (0, 1):
                o = torch.empty(nseg, dtype=dx.dtype, device="cuda")
                gbk.segmented_reduce(op, dx, do, o, tune=(256, 7, 0, variant))
                gbk.stream_check()
                np.testing.assert_array_equal(o.cpu().numpy(), want, err_msg=f"{x.dtype} {op} variant {variant}")
    for dt, rel in ((np.float32, 1e-5), (np.float64, 1e-12)):
        xf = datagen.normal_f64(n, seed=23).astype(dt)
        o = torch.empty(nseg, dtype=torch.float32 if dt == np.float32 else torch.float64, device="cuda")
        gbk.segmented_reduce("sum", _dev(torch, xf), do, o)
        gbk.stream_check()
        got = o.cpu().numpy()
        big = [s for s in range(nseg) if offs[s + 1] - offs[s] > 64] + list(range(min(nseg, 50)))
        for s in big:
            seg = xf[offs[s]:offs[s + 1]]
            ok, info = sum_ok(got[s], seg, rel) if seg.size else (got[s] == 0.0, got[s])
            assert ok, (dt, s, info)
        # the same call twice gives the same bits (fixed join order)
        o2 = torch.empty_like(o)
        gbk.segmented_reduce("sum", _dev(torch, xf), do, o2)
        gbk.stream_check()
        assert o2.cpu().numpy().tobytes() == got.tobytes()
