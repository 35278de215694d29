"""Parity of the ScatterView histogram and scatter ops (through the C ABI)
with the oracle / reference golden outputs; counts bit-exact."""
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


def test_golden_histograms(env):
    gbk, torch = env
    G = np.load(GOLDEN)
    for (n, nb) in [(100000, 4096), (5000, 65536), (0, 16)]:
        keys = G[f"hist/{n}/{nb}/x"]
        want = np.frombuffer(G[f"hist/{n}/{nb}/4/out"].tobytes(), np.int64)
        bins = torch.zeros(nb, dtype=torch.int64, device="cuda")
        gbk.histogram(_dev(torch, keys), bins)
        gbk.stream_check()
        np.testing.assert_array_equal(bins.cpu().numpy(), want)


@pytest.mark.parametrize("variant", [0, 1, 2, 4, 8, 0x11, 0x12, 0x14, 0x18, 0x20, 0x30, 0x40, 0x80, 0x100, 0x200])
@pytest.mark.parametrize("nbins", [16, 1000, 4096, 1 << 16])
def test_histogram_variants(env, variant, nbins):
    """Every privatisation variant (cluster size 1/2/4/8, with/without warp
    aggregation) counts exactly; contributions add to existing bins."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    cl = variant & 0xF
    if cl and (nbins + cl - 1) // cl * 4 > 200 * 1024:
        pytest.skip("bins do not fit this cluster size")
    n = 1000003
    keys = datagen.zipf_i32(n, nbins, 1.1, seed=nbins)
    init = datagen.uniform_i64(nbins, 0, 5, seed=1)
    bins = _dev(torch, init.copy())
    gbk.histogram(_dev(torch, keys), bins, tune=(0, 0, 0, variant))
    gbk.stream_check()
    want, _ = oracle.histogram(keys, nbins, 4, bins=init.copy())
    np.testing.assert_array_equal(bins.cpu().numpy(), want)


@pytest.mark.parametrize("variant", [0x20, 0x30, 0, 0x80, 0x100, 0x200])
def test_hist16_saturating_bins(env, variant):
    """16-bit privatised counters: one bin taking every key, and two bins
    sharing one 32-bit word both taking millions of keys (low halves, then
    a low and a high half), stay exact."""
    gbk, torch = env
    nb = 1 << 16
    for keys in (np.full(3000001, 7, dtype=np.int32),
                 np.tile(np.array([6, 7, 7, 6, 6, 9], dtype=np.int32), 1000003),
                 np.tile(np.array([7, 32775, 32775, 7, 65535, 32775], dtype=np.int32), 1000003)):
        bins = torch.zeros(nb, dtype=torch.int64, device="cuda")
        gbk.histogram(_dev(torch, keys), bins, tune=(0, 0, 0, variant))
        gbk.stream_check()
        want = np.bincount(keys, minlength=nb)
        np.testing.assert_array_equal(bins.cpu().numpy(), want)


@pytest.mark.parametrize("variant", [0x20, 0x30, 0x80, 0x100])
def test_hist16_saturating_ragged_words(env, variant):
    """16-bit counters when the word count is not a multiple of four (4,099
    bins: 2,050 words): the hot bins sit in the last words, which the drain
    scans one by one, and share a word (bins 2,048 and 4,098)."""
    gbk, torch = env
    nb = 4099
    keys = np.tile(np.array([2048, 4098, 2048, 2049, 4098, 0], dtype=np.int32), 700001)
    bins = torch.zeros(nb, dtype=torch.int64, device="cuda")
    gbk.histogram(_dev(torch, keys), bins, tune=(0, 0, 0, variant))
    gbk.stream_check()
    np.testing.assert_array_equal(bins.cpu().numpy(), np.bincount(keys, minlength=nb))


@pytest.mark.parametrize("variant", [0, 0x20, 0x80, 0x100, 0x200])
@pytest.mark.parametrize("offset", [1, 2, 3])
def test_hist16_unaligned_keys(env, variant, offset):
    """Keys that start off the 16-byte boundary (a ragged head and tail go
    through the edge kernel), power-of-two and odd bin counts."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    for nb in (1 << 16, 30001):
        keys = datagen.zipf_i32(777777 + offset, nb, 1.1, seed=offset)
        d = _dev(torch, np.concatenate([np.zeros(offset, np.int32), keys]))[offset:]
        bins = torch.zeros(nb, dtype=torch.int64, device="cuda")
        gbk.histogram(d, bins, tune=(0, 0, 0, variant))
        gbk.stream_check()
        want, _ = oracle.histogram(keys, nb, 4)
        np.testing.assert_array_equal(bins.cpu().numpy(), want)


def test_c2_histogram_full_size(env):
    """ScatterView histogram of 2^26 int32 Zipf(1.1) keys over 2^16 bins into
    int64 counts: bit-exact."""
    gbk, torch = env
    import oracle
    from kokkos_gb300 import datagen
    n, nb = 1 << 26, 1 << 16
    keys = datagen.zipf_i32(n, nb, 1.1, seed=0)
    bins = torch.zeros(nb, dtype=torch.int64, device="cuda")
    gbk.histogram(_dev(torch, keys), bins)
    gbk.stream_check()
    want, _ = oracle.histogram(keys, nb, 8)
    np.testing.assert_array_equal(bins.cpu().numpy(), want)
    assert int(bins.sum().item()) == n


def test_out_of_range_keys_flagged(env):
    gbk, torch = env
    keys = np.array([0, 1, 5, -1, 7, 100, 3], dtype=np.int32)
    bins = torch.zeros(8, dtype=torch.int64, device="cuda")
    gbk.histogram(_dev(torch, keys), bins)
    with pytest.raises(gbk.GbkError) as e:
        gbk.stream_check()
    assert e.value.status == 6
    assert bins.cpu().numpy().tolist() == [1, 1, 0, 1, 0, 1, 0, 1]
    gbk.stream_check()  # the flag was cleared


@pytest.mark.parametrize("variant", [0x20, 0x30, 0x80, 0x100, 0x200])
def test_hist16_out_of_range_keys(env, variant):
    """16-bit counters: keys below 0 or at and above nbins (odd nbins, so
    the last word's high half is not a bin) are left out of every bin and
    raise the key-range status; the valid keys count exactly."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    nb = 40001
    keys = datagen.uniform_i64(2000003, -50, nb + 50, seed=3).astype(np.int32)
    bins = torch.zeros(nb, dtype=torch.int64, device="cuda")
    gbk.histogram(_dev(torch, keys), bins, tune=(0, 0, 0, variant))
    with pytest.raises(gbk.GbkError) as e:
        gbk.stream_check()
    assert e.value.status == 6
    ok = keys[(keys >= 0) & (keys < nb)]
    np.testing.assert_array_equal(bins.cpu().numpy(), np.bincount(ok, minlength=nb))
    gbk.stream_check()


@pytest.mark.parametrize("variant", [0x100, 0x200])
def test_hist16_multiply_form_out_of_range_keys(env, variant):
    """The multiply forms (power-of-two bins): rounds holding a key below 0 or
    at and above nbins take the general path; those keys raise the key-range
    status and the rest count exactly."""
    gbk, torch = env
    from kokkos_gb300 import datagen
    nb = 1 << 15
    for lo, hi, n in ((-3, nb + 3, 2000003), (0, nb - 1, 1999999)):
        keys = datagen.uniform_i64(n, lo, hi, seed=5).astype(np.int32)
        if lo == 0:
            keys[::100003] = nb  # a few rounds with one bad key
        bins = torch.zeros(nb, dtype=torch.int64, device="cuda")
        gbk.histogram(_dev(torch, keys), bins, tune=(0, 0, 0, variant))
        with pytest.raises(gbk.GbkError) as e:
            gbk.stream_check()
        assert e.value.status == 6
        ok = keys[(keys >= 0) & (keys < nb)]
        np.testing.assert_array_equal(bins.cpu().numpy(), np.bincount(ok, minlength=nb))
        gbk.stream_check()


@pytest.mark.parametrize("op", ["sum", "min", "max", "prod"])
@pytest.mark.parametrize("dt", ["i32", "i64", "u64", "f32", "f64"])
def test_scatter_ops(env, op, dt):
    gbk, torch = env
    from kokkos_gb300 import datagen
    t = gbk.NP[gbk.DT[dt]]
    n, nd = 200000, 1000
    idx = datagen.uniform_i32(n, 0, nd - 1, seed=9)
    if op == "prod":
        vals = np.where(datagen.uniform_i32(n, 0, 999, seed=3) == 0, 2, 1).astype(t)
    elif np.dtype(t).kind == "f":
        vals = datagen.uniform_i32(n, -100, 100, seed=3).astype(t)  # exactly representable sums
    else:
        vals = datagen.uniform_i64(n, 0, 1000, seed=3).astype(t)
    init = {"sum": 0, "prod": 1, "min": 10**6, "max": 0}[op]
    dest = np.full(nd, init, dtype=t)
    want = dest.copy()
    if op == "sum":
        np.add.at(want, idx, vals)
    elif op == "prod":
        np.multiply.at(want, idx, vals)
    elif op == "min":
        np.minimum.at(want, idx, vals)
    else:
        np.maximum.at(want, idx, vals)
    d = _dev(torch, dest)
    gbk.scatter(op, _dev(torch, idx), _dev(torch, vals), d)
    gbk.stream_check()
    np.testing.assert_array_equal(d.cpu().numpy(), want)
