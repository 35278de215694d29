"""Host logic of the autotuner's candidate sets (kokkos_gb300/tuner.py): the
double Sum offers the FP64 / integer split kernel (variant 3) beside the
load-pipelined and ring kernels, other reducers do not, the index of the
library's own default matches the entry points' rule, and the features tell
the kernel families apart."""
import numpy as np

from kokkos_gb300 import tuner


def test_split_candidates_only_for_double_sum():
    w = {"kind": tuner.KIND_REDUCE, "op": 0, "dtype": 5, "n": 1 << 24}
    cs = tuner.candidates(w)
    split = [c for c in cs if c["variant"] == 3]
    assert [(c["ipt"], c["cps"]) for c in split] == list(tuner.SPLIT_CFGS)
    for op, dt in ((0, 4), (8, 4), (9, 4), (0, 0), (0, 1)):
        cs = tuner.candidates({"kind": tuner.KIND_REDUCE, "op": op, "dtype": dt, "n": 1 << 24})
        assert all(c["variant"] in (1, 2) for c in cs), (op, dt)


def test_default_index_follows_the_library_rule():
    big = {"kind": tuner.KIND_REDUCE, "op": 0, "dtype": 5, "n": 1 << 23}
    cs = tuner.candidates(big)
    c = cs[tuner.default_cfg_index(big, cs)]
    assert (c["variant"], c["ipt"], c["cps"]) == (3, 5, 0)  # the split kernel from 2^23 doubles
    small = {"kind": tuner.KIND_REDUCE, "op": 0, "dtype": 5, "n": 1 << 18}
    cs = tuner.candidates(small)
    c = cs[tuner.default_cfg_index(small, cs)]
    assert (c["variant"], c["block"], c["ipt"], c["cps"]) == (1, 256, 4, 8)  # under 4 MiB: load-pipelined 256 x 4
    mid = {"kind": tuner.KIND_REDUCE, "op": 8, "dtype": 4, "n": 1 << 24}
    cs = tuner.candidates(mid)
    c = cs[tuner.default_cfg_index(mid, cs)]
    assert (c["variant"], c["cps"]) == (2, 0)  # 4 MiB and more: the ring kernel


def test_features_separate_kernel_families():
    w = {"kind": tuner.KIND_REDUCE, "op": 0, "dtype": 5, "n": 1 << 24}
    f = {v: tuner.features(w, {"block": 256, "ipt": 4, "cps": 0, "variant": v}) for v in (1, 2, 3)}
    assert f[1][20] == 0 and f[1][21] == 0
    assert f[2][20] == 1 and f[2][21] == 0
    assert f[3][20] == 0 and f[3][21] == 1
    assert all(len(x) == tuner.NFEAT and np.isfinite(x).all() for x in f.values())


def test_new_candidate_families():
    h = {"kind": tuner.KIND_HIST, "dtype": 0, "n": 1 << 24, "nbins": 65536}
    cs = tuner.candidates(h)
    c = cs[tuner.default_cfg_index(h, cs)]
    assert (c["variant"], c["cps"]) == (0x100, 1)  # 65536 bins: the drain-free 16-bit kernel, multiply form
    f = tuner.features(h, c)
    assert f[22] == 1 and f[26] == 2
    f80 = tuner.features(h, next(x for x in cs if x["variant"] == 0x80))
    assert f80[22] == 1 and f80[26] == 1
    f20 = tuner.features(h, next(x for x in cs if x["variant"] == 0x20))
    assert f20[22] == 1 and f20[26] == 0
    small = {"kind": tuner.KIND_HIST, "dtype": 0, "n": 1 << 24, "nbins": 4096}
    cs = tuner.candidates(small)
    assert (cs[tuner.default_cfg_index(small, cs)]["variant"], cs[tuner.default_cfg_index(small, cs)]["cps"]) == (1, 2)
    s = {"kind": tuner.KIND_SEGSCAN, "op": 1, "dtype": 0, "n": 1 << 22, "nseg": 1024}
    cs = tuner.candidates(s)
    assert [(c["ipt"], c["cps"]) for c in cs] == list(tuner.SEGSCAN_CFGS)
    assert (cs[tuner.default_cfg_index(s, cs)]["ipt"], cs[tuner.default_cfg_index(s, cs)]["cps"]) == (5, 0)
    fs = tuner.features(s, cs[0])
    assert fs[3] == 1 and fs[24] == 1 and fs[27] == 1
    m = {"kind": tuner.KIND_REDUCE, "op": 12, "dtype": 4, "n": 1 << 22}
    fm = tuner.features(m, tuner.candidates(m)[0])
    assert fm[10] == 1 and fm[25] == 1


def test_lookup_keys_follow_the_entry_points():
    # gbk_scan: (1, inclusive, in*8+out); histogram: (2, 0, i32, n, ceil log2 bins * 8);
    # segmented: (3, op or 16+inclusive, dtype, n, ceil log2 mean length)
    assert tuner.lookup_key({"kind": tuner.KIND_SCAN, "op": 1, "n": 5}) == (1, 1, 1, 5, 0)
    assert tuner.lookup_key({"kind": tuner.KIND_HIST, "n": 9, "nbins": 4000}) == (2, 0, 0, 9, 96)
    assert tuner.lookup_key({"kind": tuner.KIND_SEG, "n": 1000, "nseg": 10}) == (3, 0, 4, 1000, 7)
    assert tuner.lookup_key({"kind": tuner.KIND_SEGSCAN, "op": 0, "n": 1024, "nseg": 16}) == (3, 16, 1, 1024, 6)


def test_table_round_trip_through_the_library(tmp_path):
    """A table written from per-bucket choices and loaded into libgbk gives
    every bucket back the candidate it was written with (the method without
    the MLP that the held-out evaluation compares against)."""
    import os

    from kokkos_gb300 import gbk
    if not os.path.exists(gbk.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    rng = np.random.default_rng(0)
    rows = []
    for w in tuner.grid_workloads():
        if "nseg" in w:
            w = dict(w, n=w["n"] + int(rng.integers(0, 1000)))  # realised segment totals are not powers of two
        cs = tuner.candidates(w)
        ts = list(rng.uniform(1.0, 2.0, len(cs)))
        rows.append((w, cs, ts))
    path = tuner.table_exhaustive(rows, str(tmp_path / "t.txt"))
    assert gbk.lib.gbk_tuner_load(path.encode()) == 0
    try:
        for w, cs, ts in rows:
            assert tuner.table_pick(w, cs) == int(np.argmin(ts)), w
        # a workload between buckets takes the choice of the bucket nearest
        # to its ceil(log2 n)
        w = dict(rows[0][0], n=(1 << 16) - 3)
        assert tuner.table_pick(w, rows[0][1]) == int(np.argmin(rows[0][2]))
    finally:
        gbk.lib.gbk_tuner_clear()
