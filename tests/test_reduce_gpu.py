"""Parity of the GPU reduce / MDRange reduce (through the C ABI) with the
oracle and with the reference's own golden outputs."""
import os

import numpy as np
import pytest

from tests._util import prod_ok, sum_ok, sum_tol

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")
INT_OPS = ["sum", "prod", "min", "max", "land", "lor", "band", "bor", "minloc", "maxloc", "minmax", "minmaxloc"]
FLT_OPS = ["sum", "prod", "min", "max", "minloc", "maxloc", "minmax", "minmaxloc"]


@pytest.fixture(scope="module")
def env():
    import torch

    from kokkos_gb300 import gbk
    torch.cuda.set_device(0)
    return gbk, torch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def compare(op, got, want, x):
    """got/want: numpy scalars / structured records of the reducer layout."""
    names = got.dtype.names
    fl = x.dtype.kind == "f"
    if op == "sum" and fl:
        ok, info = sum_ok(got, x, sum_tol(x.dtype))
        assert ok, info
        return
    if op == "prod" and fl:
        ok, info = prod_ok(got, x)
        assert ok, info
        return
    if names:
        for nm in names:
            assert np.asarray(got[nm]).tobytes() == np.asarray(want[nm]).tobytes(), (op, nm, got, want)
    else:
        assert np.asarray(got).tobytes() == np.asarray(want).tobytes(), (op, got, want)


def test_golden_reducers_all_dtypes(env):
    """GPU result vs the reference's own output for every reducer x dtype x
    size in the golden set (floats within the stated tolerances)."""
    gbk, torch = env
    G = np.load(GOLDEN)
    cases = sorted({k.rsplit("/", 2)[0] for k in G.files if k.startswith("reduce/") and k.endswith("/out")})
    assert len(cases) > 200
    for c in cases:
        _, op, dt, n = c.split("/")
        x = G[c + "/x"]
        want = np.frombuffer(G[c + "/4/out"].tobytes(), dtype=gbk.result_dtype(gbk.OPS[op], gbk.DT[{
            "int32": "i32", "int64": "i64", "uint32": "u32", "uint64": "u64", "float32": "f32", "float64": "f64"}[dt]]))[0]
        got = gbk.reduce_value(op, _dev(torch, x))
        compare(op, got, want, x)


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint32, np.uint64, np.float32, np.float64])
@pytest.mark.parametrize("n", [0, 1, 3, 33, 4097, (1 << 20) + 5])
def test_reducers_vs_oracle(env, dtype, n):
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    t = np.dtype(dtype)
    if t.kind == "f":
        x = datagen.normal_f64(n, seed=n).astype(t)
    elif t.kind == "i":
        x = datagen.uniform_i64(n, -1000, 1000, seed=n).astype(t)
    else:
        x = datagen.uniform_i64(n, 0, 100000, seed=n).astype(t)
    ops = FLT_OPS if t.kind == "f" else INT_OPS
    for op in ops:
        xx = x
        if op == "prod":
            xx = np.ones(n, dtype=t) if t.kind != "f" else (1 + 1e-4 * datagen.normal_f64(n, seed=1)).astype(t)
            if n > 2 and t.kind != "f":
                xx[n // 3] = 3
                xx[n // 2] = 2
        if op in ("land", "lor"):
            xx = (x % 5 != 0).astype(t) if op == "land" else (x % 997 == 3).astype(t)
        d = _dev(torch, xx)
        got = gbk.reduce_value(op, d)
        want = oracle.reduce(op, xx, 4)
        compare(op, got, want, xx)


@pytest.mark.parametrize("offset", [1, 2, 3])
def test_misaligned_views(env, offset):
    """Views that start off a 16-byte boundary (subviews) take the scalar
    head path."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    base = datagen.uniform_i32(100003, -50, 50, seed=7)
    d = _dev(torch, base)
    sub = d[offset:]
    for op in ("sum", "minloc", "maxloc", "minmaxloc"):
        got = gbk.reduce_value(op, sub)
        want = oracle.reduce(op, base[offset:], 1)
        compare(op, got, want, base[offset:])


def test_c1_sum_f64_full_size(env):
    """parallel_reduce Sum over View<double*> 2^24 uniform[0,1), seed 0:
    rel err <= 1e-12 vs the compensated FP64 sum."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    x = datagen.uniform_f64(1 << 24, seed=0)
    got = gbk.reduce_value("sum", _dev(torch, x))
    ok, info = sum_ok(got, x, 1e-12)
    assert ok, info
    import oracle
    s, _, _ = oracle.sum_compensated(x)
    assert abs(float(got) - s) <= 1e-12 * abs(s)


def test_c2_mdrange_full_size(env):
    """MDRangePolicy<Rank<3>> MinLoc / MaxLoc / Sum over LayoutLeft
    View<float***> 512x512x256 of N(0,1); the extremum is unique, so value
    and loc are exact."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    n0, n1, n2 = 512, 512, 256
    x = datagen.normal_f32(n0 * n1 * n2, seed=0)
    d = _dev(torch, x)
    lo, up, st = [0, 0, 0], [n0, n1, n2], [1, n0, n0 * n1]
    imin, imax = int(np.argmin(x)), int(np.argmax(x))
    assert (x == x[imin]).sum() == 1 and (x == x[imax]).sum() == 1
    r = gbk.decode_result(gbk.mdrange_reduce("minloc", d, lo, up, st).cpu().numpy(), 8, 4)
    assert r["val"] == x[imin] and r["loc"] == imin
    r = gbk.decode_result(gbk.mdrange_reduce("maxloc", d, lo, up, st).cpu().numpy(), 9, 4)
    assert r["val"] == x[imax] and r["loc"] == imax
    s = gbk.decode_result(gbk.mdrange_reduce("sum", d, lo, up, st).cpu().numpy(), 0, 4)
    ok, info = sum_ok(s, x, 1e-5)
    assert ok, info
    gbk.stream_check()


@pytest.mark.parametrize("layout", ["left", "right"])
def test_mdrange_subbox_generic(env, layout):
    """A box that is not one contiguous run (generic row kernel), rank 3."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    n0, n1, n2 = 37, 29, 23
    x = datagen.normal_f32(n0 * n1 * n2, seed=3)
    st = [1, n0, n0 * n1] if layout == "left" else [n1 * n2, n2, 1]
    lo, up = [2, 3, 1], [35, 20, 22]
    d = _dev(torch, x)
    for op, code in (("minloc", 8), ("maxloc", 9), ("minmaxloc", 11), ("min", 2), ("max", 3)):
        got = gbk.decode_result(gbk.mdrange_reduce(op, d, lo, up, st).cpu().numpy(), code, 4)
        want = oracle.mdrange_reduce(op, x, lo, up, st, 1)
        for nm in (got.dtype.names or [None]):
            a = got[nm] if nm else got
            b = want[nm] if nm else want
            assert np.asarray(a).tobytes() == np.asarray(b).tobytes(), (op, nm, a, b)
    got = gbk.decode_result(gbk.mdrange_reduce("sum", d, lo, up, st).cpu().numpy(), 0, 4)
    idx = np.array([i * st[0] + j * st[1] + k * st[2] for i in range(lo[0], up[0]) for j in range(lo[1], up[1])
                    for k in range(lo[2], up[2])])
    ok, info = sum_ok(got, x[idx], 1e-5)
    assert ok, info


def test_mdrange_golden(env):
    gbk, torch = env
    G = np.load(GOLDEN)
    for (n0, n1, n2) in [(37, 19, 11), (64, 32, 16)]:
        x = G[f"mdrange/f32/{n0}x{n1}x{n2}/x"]
        d = _dev(torch, x)
        for op, code in (("minloc", 8), ("maxloc", 9)):
            want = np.frombuffer(G[f"mdrange/{op}/f32/{n0}x{n1}x{n2}/4/out"].tobytes(), gbk.result_dtype(code, 4))[0]
            got = gbk.decode_result(gbk.mdrange_reduce(op, d, [0, 0, 0], [n0, n1, n2], [1, n0, n0 * n1]).cpu().numpy(),
                                    code, 4)
            assert got["val"] == want["val"] and got["loc"] == want["loc"]


def test_host_buffer_entry(env):
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    x = datagen.normal_f32(1 << 18, seed=11)
    r = gbk.mdrange_reduce_host("minmaxloc", x, [0], [x.size], [1])
    w = oracle.reduce("minmaxloc", x, 1)
    for nm in ("min_val", "max_val", "min_loc", "max_loc"):
        assert r[nm] == w[nm]


def test_fence_read_returns_result_and_status(env):
    """gbk_fence_read: the reduce's device result comes back into host memory
    behind the same synchronisation as the stream's status (the host-scalar
    parallel_reduce path), on the default and on a created stream, twice in a
    row (the pinned slot is reused); a device-side status raised earlier on the
    stream comes back with it and is cleared."""
    import ctypes

    import oracle
    gbk, torch = env
    from kokkos_gb300 import datagen
    x = datagen.uniform_i32((1 << 20) + 7, -50, 50, seed=3)
    dx = _dev(torch, x)
    want = int(oracle.reduce("sum", x, 4))
    for st in (None, torch.cuda.Stream()):
        sp = ctypes.c_void_p(st.cuda_stream) if st is not None else None
        d = torch.zeros(8, dtype=torch.int64, device="cuda")
        for _ in range(2):
            d.zero_()
            torch.cuda.synchronize()
            assert gbk.lib.gbk_reduce(0, 0, ctypes.c_void_p(dx.data_ptr()), x.size,
                                      ctypes.c_void_p(d.data_ptr()), sp, None) == 0
            h = ctypes.c_int64(-1)
            assert gbk.lib.gbk_fence_read(sp, ctypes.c_void_p(d.data_ptr()), ctypes.byref(h), 8) == 0
            assert h.value == want
    # a key outside the bins raises the stream's status; fence_read reports it once
    keys = torch.tensor([1, 2, 70000], dtype=torch.int32, device="cuda")
    bins = torch.zeros(16, dtype=torch.int64, device="cuda")
    assert gbk.lib.gbk_histogram_i32_i64(ctypes.c_void_p(keys.data_ptr()), 3, ctypes.c_void_p(bins.data_ptr()),
                                         16, None, None) == 0
    h = ctypes.c_int64(-1)
    assert gbk.lib.gbk_fence_read(None, ctypes.c_void_p(bins.data_ptr() + 8), ctypes.byref(h), 8) == 6
    assert h.value == 1
    assert gbk.lib.gbk_stream_check(None) == 0


def test_tuning_configs_agree(env):
    """Every compiled launch configuration gives a correct (in-tolerance,
    exact for integers) result."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    x = datagen.uniform_i32((1 << 22) + 17, -3, 3, seed=5)
    xf = datagen.normal_f32((1 << 22) + 17, seed=5)
    d, df = _dev(torch, x), _dev(torch, xf)
    w = oracle.reduce("sum", x, 1)
    wl = oracle.reduce("minloc", xf, 1)
    wm = oracle.reduce("maxloc", xf, 1)
    for blk, un, cps in [(256, 2, 8), (256, 4, 8), (512, 2, 4), (512, 4, 2), (128, 8, 16), (256, 8, 4), (1024, 2, 2),
                         (256, 4, 1)]:
        for var in (0, 1):  # 0: the ring kernel at this size; 1: the load-pipelined kernel with this shape
            tune = (blk, un, cps, var)
            got = gbk.decode_result(gbk.reduce("sum", d, tune=tune).cpu().numpy(), 0, 0)
            assert got == w, tune
            gl = gbk.decode_result(gbk.reduce("minloc", df, tune=tune).cpu().numpy(), 8, 4)
            assert gl["val"] == wl["val"] and gl["loc"] == wl["loc"], tune
            gm = gbk.decode_result(gbk.reduce("maxloc", df, tune=tune).cpu().numpy(), 9, 4)
            assert gm["val"] == wm["val"] and gm["loc"] == wm["loc"], tune
            gs = gbk.decode_result(gbk.reduce("sum", df, tune=tune).cpu().numpy(), 0, 4)
            ok, info = sum_ok(gs, xf, 1e-5)
            assert ok, (tune, info)


@pytest.mark.parametrize("n", [4099, (1 << 21) + 7, (1 << 22) + 3])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32])
def test_loc_ties_nan_signed_zero(env, n, dtype):
    """*Loc reducers on data full of ties (few distinct values), NaNs and
    signed zeros, through the flat (< 4 MiB) and the ring kernel: the value
    and the first-occurrence loc equal the oracle's element-by-element strict
    comparison."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    t = np.dtype(dtype)
    x = datagen.uniform_i64(n, -3, 3, seed=n + 11).astype(t)
    if t.kind == "f":
        x[x == 0] = -0.0
        x[::7] = 0.0
        x[5::13] = np.nan
        x[: min(n, 64)] = np.nan  # a NaN-only prefix: the running value stays the identity for a while
    cases = [x]
    if t.kind == "f":
        z = (x > 0).astype(t)  # minimum 0: the first zero wins, whatever its sign
        zi = np.flatnonzero(z == 0)
        z[zi[::2]] = -0.0
        z[5::13] = np.nan
        z[: min(n, 64)] = np.nan
        cases.append(z)
    for i, a in enumerate(cases):
        d = _dev(torch, a)
        # plain Min over {-0.0, +0.0} may return either zero (partials join in tree order); the *Loc
        # reducers return the first occurrence, sign included
        for op in ("minloc", "maxloc", "minmaxloc") + (("min", "max") if i == 0 else ()):
            got = gbk.reduce_value(op, d)
            want = oracle.reduce(op, a, 1)
            compare(op, got, want, a)


SPLIT_TUNES = [(256, 4, 0, 3), (256, 3, 0, 3), (256, 5, 0, 3), (256, 6, 2, 3), (256, 4, 1, 4)]


@pytest.mark.parametrize("tune", SPLIT_TUNES)
def test_sum_f64_split_pipes(env, tune):
    """Sum<double> with the adds split between the FP64 pipe and the exact
    fixed-point accumulator on the integer pipes (every launch shape):
    uniform, mixed-sign, exponent ranges far wider than 53 bits, subnormals,
    unaligned heads and odd tails, within 1e-12 of the compensated sum."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    rng = np.random.default_rng(7)
    n = (1 << 20) + 3
    cases = {
        "uniform": datagen.uniform_f64(n, seed=3),
        "normal": datagen.normal_f64(n, seed=4),
        "wide": datagen.normal_f64(n, seed=5) * 10.0 ** rng.integers(-250, 250, n),
        "cancel": np.concatenate([datagen.normal_f64(n // 2, seed=6) * 1e30, -datagen.normal_f64(n // 2, seed=6) * 1e30,
                                  datagen.uniform_f64(3, seed=8)]),
        "subnormal": datagen.uniform_f64(n, seed=9) * 1e-310,
        "ints": rng.integers(-1 << 20, 1 << 20, n).astype(np.float64),
    }
    for name, x in cases.items():
        for off in (0, 1):
            sub = x[off:]
            got = gbk.reduce_value("sum", _dev(torch, sub), tune=tune)
            ok, info = sum_ok(got, sub, 1e-12)
            assert ok, (name, off, info)
            if name == "ints":  # every partial is an integer below 2^53: exact
                assert float(got) == float(np.sum(sub.astype(np.int64))), (name, off)
    gbk.stream_check()


def test_sum_f64_split_nonfinite(env):
    """Infinities and NaNs keep their FP64 meaning on the split kernel."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    n = 1 << 20
    x = datagen.uniform_f64(n, seed=1)
    for tune in ((256, 4, 0, 3), (256, 4, 0, 4)):
        y = x.copy()
        y[12345] = np.inf
        assert float(gbk.reduce_value("sum", _dev(torch, y), tune=tune)) == np.inf
        y[777777] = -np.inf
        assert np.isnan(float(gbk.reduce_value("sum", _dev(torch, y), tune=tune)))
        y = x.copy()
        y[n - 1] = np.nan
        assert np.isnan(float(gbk.reduce_value("sum", _dev(torch, y), tune=tune)))
        y = np.full(n, 1.5e308)
        assert float(gbk.reduce_value("sum", _dev(torch, y), tune=tune)) == np.inf
        y[1::2] = -1.5e308  # exact cancellation of huge values
        assert float(gbk.reduce_value("sum", _dev(torch, y), tune=tune)) == 0.0
    gbk.stream_check()


def test_sum_f64_split_fold_interval(env):
    """2^30 doubles on one CTA per SM: each thread folds its fixed-point
    accumulator into FP64 mid-way (more than 2^14 elements per thread).  The
    values are multiples of 2^-20 below 2^31 in every partial, so the sum is
    exact and compared bit for bit."""
    gbk, torch = env
    n = 1 << 30
    i = torch.arange(n, dtype=torch.int64, device="cuda")
    x = (1.0 + (i % 7).to(torch.float64) * 2.0 ** -20) * torch.where(i % 3 == 0, -1.0, 1.0).to(torch.float64)
    del i
    k = np.arange(21)
    pat = (1.0 + (k % 7) * 2.0 ** -20) * np.where(k % 3 == 0, -1.0, 1.0)
    want = (n // 21) * int(np.sum(pat * 2 ** 20)) + int(np.sum(pat[: n % 21] * 2 ** 20))
    for tune in ((256, 4, 1, 3), (256, 4, 1, 4)):
        got = float(gbk.reduce_value("sum", x, tune=tune))
        assert got * 2 ** 20 == want, (tune, got, want / 2 ** 20)
    del x
    torch.cuda.empty_cache()
    gbk.stream_check()


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint32, np.float32, np.float64])
@pytest.mark.parametrize("n", [0, 1, 33, 4097, (1 << 20) + 5])
def test_minmaxloc_sum_one_pass(env, dtype, n):
    """MinMaxLoc and Sum as two reducers of one parallel_reduce (one pass):
    the MinMaxLoc half equals the MinMaxLoc reducer's result exactly (ties:
    first index), the Sum half matches the oracle (exact for integers,
    within the Sum tolerances for floats); head/tail offsets included."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    t = np.dtype(dtype)
    if t.kind == "f":
        x = datagen.normal_f64(n + 3, seed=n + 11).astype(t)
    elif t.kind == "i":
        x = datagen.uniform_i64(n + 3, -1000, 1000, seed=n + 11).astype(t)
    else:
        x = datagen.uniform_i64(n + 3, 0, 100000, seed=n + 11).astype(t)
    for off in (0, 1, 3):
        xx = x[off:off + n]
        got = gbk.reduce_value("minmaxloc_sum", _dev(torch, xx))
        want = oracle.reduce("minmaxloc", xx, 4)
        for nm in ("min_val", "max_val", "min_loc", "max_loc"):
            assert np.asarray(got[nm]).tobytes() == np.asarray(want[nm]).tobytes(), (nm, off, got, want)
        if t.kind == "f":
            ok, info = sum_ok(got["sum"], xx, sum_tol(t))
            assert ok, (off, info)
        else:
            assert np.asarray(got["sum"]).tobytes() == np.asarray(oracle.reduce("sum", xx, 4)).tobytes(), off
    gbk.stream_check()


def test_c2_minmaxloc_sum_one_pass_full_size(env):
    """The C2 box (LayoutLeft View<float***> 512x512x256 of N(0,1)) reduced
    once for MinLoc, MaxLoc and Sum together, and a strided sub-box through
    the generic row kernel."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    n0, n1, n2 = 512, 512, 256
    x = datagen.normal_f32(n0 * n1 * n2, seed=0)
    d = _dev(torch, x)
    st = [1, n0, n0 * n1]
    imin, imax = int(np.argmin(x)), int(np.argmax(x))
    r = gbk.decode_result(gbk.mdrange_reduce("minmaxloc_sum", d, [0, 0, 0], [n0, n1, n2], st).cpu().numpy(), 12, 4)
    assert r["min_val"] == x[imin] and r["min_loc"] == imin
    assert r["max_val"] == x[imax] and r["max_loc"] == imax
    ok, info = sum_ok(r["sum"], x, 1e-5)
    assert ok, info
    lo, up = [3, 5, 7], [500, 300, 200]
    r = gbk.decode_result(gbk.mdrange_reduce("minmaxloc_sum", d, lo, up, st).cpu().numpy(), 12, 4)
    want = oracle.mdrange_reduce("minmaxloc", x, lo, up, st, 4)
    for nm in ("min_val", "max_val", "min_loc", "max_loc"):
        assert np.asarray(r[nm]).tobytes() == np.asarray(want[nm]).tobytes(), nm
    sub = x.reshape(n2, n1, n0)[7:200, 5:300, 3:500]
    ok, info = sum_ok(r["sum"], np.ascontiguousarray(sub).ravel(), 1e-5)
    assert ok, info
    gbk.stream_check()
