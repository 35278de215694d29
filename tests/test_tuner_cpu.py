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
