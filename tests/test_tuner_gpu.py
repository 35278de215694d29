"""End-to-end learned-tuner pipeline at reduced scale on the GPU: exhaustive
sweeps through the C ABI, MLP training with the library's kernels, held-out
evaluation against the exhaustive best and the untuned default, and the
tuning table consulted by the entry points.  The full-scale run (about
20,000 training timings, 2,000 held-out workloads) is
`python -m kokkos_gb300.tuner`."""
import ctypes
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_small_pipeline_and_table():
    import torch

    from kokkos_gb300 import gbk, tuner
    bench = tuner.Bench(max_n=1 << 22)
    train = tuner.collect(tuner.sample_workloads(60, seed=11), bench, log_every=0)
    held = tuner.collect(tuner.sample_workloads(40, seed=12), bench, log_every=0)
    X, T, _ = tuner.dataset(train)
    assert X.shape[0] > 600 and X.shape[1] == tuner.NFEAT
    m = tuner.MLP(seed=0)
    hist = m.train(X, T, epochs=120, batch=512, lr=3e-3)
    assert hist[-1][1] < hist[0][1]
    rep = tuner.evaluate(m, held)
    assert rep["workloads"] == 40
    assert 0.0 < rep["default_mean_throughput_vs_best"] <= 1.0
    assert rep["mlp_mean_throughput_vs_best"] > 0.7
    grid = tuner.collect(tuner.grid_workloads(), bench, log_every=0)
    with tempfile.TemporaryDirectory() as d:
        ratio = tuner.table_from_model(m, grid, os.path.join(d, "mlp.txt"))
        assert 0.0 < ratio <= 1.0
        assert gbk.lib.gbk_tuner_load(os.path.join(d, "mlp.txt").encode()) == 0
        path = tuner.table_exhaustive(grid, os.path.join(d, "t.txt"))
        assert gbk.lib.gbk_tuner_load(path.encode()) == 0
    # (sizes above the small bench's 2^22 fold into fewer buckets)
    assert gbk.lib.gbk_tuner_size() >= 50
    gbk.lib.gbk_tuner_enable(1)
    try:
        # entry points called without a configuration now use the table;
        # results are unchanged
        from kokkos_gb300 import datagen
        x = datagen.uniform_i32((1 << 20) + 3, -5, 5, seed=1)
        got = gbk.reduce_value("sum", torch.from_numpy(x).cuda())
        assert int(got) == int(x.astype(np.int64).sum())
        t = gbk.Tuning()
        assert gbk.lib.gbk_tuner_lookup(0, 0, 0, 1 << 20, 0, ctypes.byref(t)) == 0 and t.block in (128, 256, 512, 1024)
    finally:
        gbk.lib.gbk_tuner_enable(0)
        gbk.lib.gbk_tuner_clear()


def test_mlp_gains_over_the_methods_without_it():
    """On held-out workloads (sizes, segment statistics and key distributions
    the training set never held) the learned tuner's choice (an ensemble of
    five MLPs trained by the library's kernels) is compared with the
    exhaustive best, with the library's untuned default, and with the tuning
    table the exhaustive autotuner writes for its buckets (the method without
    the MLP: nearest bucket by ceil(log2 n), as the entry points look it up).
    Margins (mean throughput relative to the best, and the fraction of
    workloads within 5 % of the best):
      MLP >= default + 0.02;  MLP >= table + 0.005;
      MLP within 5 % on >= 0.88 of the workloads and on more of them than the table."""
    from kokkos_gb300 import gbk, tuner
    GAIN_DEFAULT, GAIN_TABLE, WITHIN_5PCT = 0.02, 0.005, 0.88
    bench = tuner.Bench(max_n=1 << 26)
    train = tuner.collect(tuner.sample_workloads(500, seed=21), bench, log_every=0)
    held = tuner.collect(tuner.sample_workloads(250, seed=22), bench, log_every=0)
    grid = tuner.collect(tuner.grid_workloads(), bench, log_every=0)
    X, T, _ = tuner.dataset(train)
    m = tuner.Ensemble(k=5)
    m.train(X, T, epochs=300)
    with tempfile.TemporaryDirectory() as d:
        path = tuner.table_exhaustive(grid, os.path.join(d, "t.txt"))
        assert gbk.lib.gbk_tuner_load(path.encode()) == 0
        try:
            rep = tuner.evaluate(m, held, table=True)
        finally:
            gbk.lib.gbk_tuner_clear()
    print({k: (round(v, 4) if isinstance(v, float) else v) for k, v in rep.items() if k != "per_kind"})
    assert rep["workloads"] == 250
    mlp, dflt, table = (rep[f"{k}_mean_throughput_vs_best"] for k in ("mlp", "default", "table"))
    assert mlp >= dflt + GAIN_DEFAULT, rep
    assert mlp >= table + GAIN_TABLE, rep
    assert rep["mlp_frac_within_5pct"] >= WITHIN_5PCT, rep
    assert rep["mlp_frac_within_5pct"] > rep["table_frac_within_5pct"], rep
