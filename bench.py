"""Benchmark of the GB300 reduce / scatter hot path on the MDRange +
ScatterView workload:

  step = MDRangePolicy<Rank<3>> MinLoc, MaxLoc and Sum over a LayoutLeft
         View<float***> 512x512x256 of N(0,1) values (three reduces), plus a
         ScatterView histogram of 2^26 int32 Zipf(s=1.1) keys over 2^16 bins
         into int64 counts (bins zeroed, then contributed).
  metric = algorithmic HBM bytes of the step / step time, in GB/s:
           3 x 268,435,456 (reduces) + 268,435,456 + 524,288 (histogram).

`value` times the device path (inputs resident in HBM; every input is
268 MB, larger than the 129 MB L2, so no flush is needed).  `e2e` times the
same step through the C ABI from pinned HOST buffers: deep_copy of the view
and the keys to the device, the four operations, and the results copied
back, every step.  `roofline` is the dominant kernel (the flat reduce the
contiguous MDRange box collapses to).  `cpu_baseline` is the oracle (CPU
restatement of the reference OpenMP algorithms) on this host.
`other_configs` (N = 1 only) times the other headline workloads after the
step, outside the timed region: the RangePolicy Sum and exclusive_scan of
2^24 values, the batched segmented Sum / inclusive_scan over 10,000
lognormal segments against the one-launch-per-segment loop, a Graph of 8
dependent reduce / scan nodes, sort_by_key, sort and BinSort of 2^27 uint64
keys, and deep_copy / fill / permute.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbk|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own
GPU (the path does not shard across GPUs here); value = all ranks' bytes /
the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N0, N1, N2 = 512, 512, 256
NX = N0 * N1 * N2
NKEYS = 1 << 26
NBINS = 1 << 16
RED_BYTES = NX * 4
HIST_BYTES = NKEYS * 4 + NBINS * 8
STEP_BYTES = 3 * RED_BYTES + HIST_BYTES
# The dominant kernel and its DRAM traffic per launch (dram__bytes_read.sum +
# dram__bytes_write.sum from one ncu capture of the same launch, as recorded
# in profiles/).
ROOF_KERNEL = "flat reduce of the box, MinLoc/MaxLoc/Sum f32"
ROOF_TRAFFIC = 272140000  # MinLoc f32 over the box, ring kernel: 268.48 MB read + 3.66 MB written (ncu, MB precision)
METRIC = "HBM GB/s (algorithmic bytes / step time) of MDRange reduce + ScatterView histogram"
WORKLOAD = ("MDRange<Rank<3>> MinLoc+MaxLoc+Sum over LayoutLeft View<float***> 512x512x256 N(0,1) "
            "+ ScatterView histogram 2^26 int32 Zipf(1.1) keys -> 2^16 int64 bins")


def launch_shapes(gbk, tuned):
    """The kernel each operation of the step runs with (from the tuning table
    when it is in use, else the library defaults)."""
    import ctypes
    out = {}
    for name, op in (("MinLoc", 8), ("MaxLoc", 9), ("Sum", 0)):
        t = gbk.Tuning()
        if tuned and gbk.lib.gbk_tuner_lookup(0, op, 4, NX, 0, ctypes.byref(t)) == 0:
            cps = f"{t.ctas_per_sm} CTAs/SM" if t.ctas_per_sm else "all resident CTAs"
            out[name] = (f"k_reduce_flat load-pipelined {t.block} x {t.items_per_thread}, {cps}" if t.variant == 1
                         else f"k_reduce_tma shared-memory ring, {cps}")
        else:
            out[name] = "k_reduce_tma shared-memory ring, all resident CTAs (default)"
    t = gbk.Tuning()
    hv = t.variant if tuned and gbk.lib.gbk_tuner_lookup(2, 0, 0, NKEYS, 16 * 8, ctypes.byref(t)) == 0 else 0
    out["histogram"] = {0: "default (16-bit drain-free, multiply form)", 0x20: "k_hist16 with drains",
                        0x80: "k_hist16 drain-free", 0x100: "k_hist16 drain-free, multiply form"}.get(hv, hex(hv))
    return out


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def job_gbs(world, steps, ms_total):
    """Whole-job throughput of independent replicas: every rank processes
    STEP_BYTES per step, the job takes the slowest rank's time."""
    return world * STEP_BYTES * steps / (ms_total / 1e3) / 1e9


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.p = None
        self.path = os.path.join(tempfile.gettempdir(), f"gbk_clocks_{os.getpid()}.csv")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in open(self.path):
            c = [x.strip() for x in ln.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                mx.append(float(c[2]))
                power.append(float(c[3]))
            except ValueError:
                continue
            for nm, v in zip(names, c[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        try:
            os.remove(self.path)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": float(max(power)) if power else None}


def cpu_baseline(budget_s=12.0):
    """Oracle (CPU restatement of the reference OpenMP MDRange reduce and
    Duplicated ScatterView algorithms) over the same workload on this host's
    cores: full-size inputs, as many whole steps as fit in the time budget
    (at least one).  The reduces walk the box as the reference's host
    backend does for MDRangePolicy<Rank<3>> (Iterate::Right outer and inner,
    default tiles {2, 2, 256}) over the LayoutLeft view, i.e. the stride-
    n0*n1 dimension innermost; the same three reduces with
    Rank<3, Iterate::Left, Iterate::Left> (unit stride innermost) are timed
    once beside it as `iterate_left_step_s`."""
    import oracle
    from kokkos_gb300 import datagen
    P = oracle.max_threads()
    x = datagen.normal_f32(NX, seed=0)
    keys = datagen.zipf_i32(NKEYS, NBINS, 1.1, seed=0)
    box = ([0, 0, 0], [N0, N1, N2], [1, N0, N0 * N1])
    steps, t0 = 0, time.perf_counter()
    while True:
        oracle.mdrange_reduce("minloc", x, *box, P)
        oracle.mdrange_reduce("maxloc", x, *box, P)
        oracle.mdrange_reduce("sum", x, *box, P)
        oracle.histogram(keys, NBINS, P)
        steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s:
            break
    gbs = steps * STEP_BYTES / el / 1e9
    t1 = time.perf_counter()
    for op in ("minloc", "maxloc", "sum"):
        oracle.mdrange_reduce(op, x, *box, P, outer="left", inner="left")
    oracle.histogram(keys, NBINS, P)
    left_s = time.perf_counter() - t1
    return {"value": round(gbs, 3), "unit": "GB/s", "cores": P, "kind": "port",
            "sample": (f"{steps} full-size steps ({el:.1f} s) of the same workload, OpenMP threads={P}; "
                       "MDRangePolicy<Rank<3>> host defaults (Iterate::Right) over the LayoutLeft view"),
            "iterate_left_step_s": round(left_s, 4),
            "iterate_left_GBps": round(STEP_BYTES / left_s / 1e9, 3)}


def other_configs(torch, gbk, datagen, stream, dev, hbm, peak_kind, reps=10):
    """The other headline workloads of the path, timed after the step with CUDA
    events around each call on the launching stream (not part of `value`):
      c1: Sum over 2^24 uniform doubles and exclusive_scan int32 -> int64 of
          2^24 values 0..15, inputs rotated over 4 copies (each call starts
          with its input out of L2), 40 calls back to back between two events;
      c3: 10,000 lognormal segments (median 2,048, max 2^21, total ~2^28):
          per-segment Sum f32 and inclusive_scan int32, one launch each (10
          back to back; inputs of 1 GB), and one pass of the
          one-launch-per-segment loop for comparison;
      c4: sort_by_key of 2^27 uint64 keys + int32 iota payload, uniform and
          low-entropy keys (inputs refilled on the stream before each sort);
      data movement: deep_copy of 1 GiB device to device (read + write
          bytes), deep_copy(view, value) of 1 GiB, permute (gather) of 2^26
          int32 by a random permutation (4 + 8 + 4 bytes per element)."""
    lib = gbk.lib
    sp = ctypes.c_void_p(stream.cuda_stream)
    P = ctypes.c_void_p
    out = {}

    def timed(calls, n_reps, prep=None, batch=False):
        """Median per-call ms with events around each call, or (batch) the
        mean over n_reps back-to-back calls between two events."""
        evs = []
        with torch.cuda.stream(stream):
            for c in calls:
                if prep:
                    prep(c)
                c()
            if batch:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for r in range(n_reps):
                    calls[r % len(calls)]()
                e1.record(stream)
                torch.cuda.synchronize()
                gbk.stream_check(stream)
                return e0.elapsed_time(e1) / n_reps
            for r in range(n_reps):
                c = calls[r % len(calls)]
                if prep:
                    prep(c)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                c()
                e1.record(stream)
                evs.append((e0, e1))
        torch.cuda.synchronize()
        gbk.stream_check(stream)
        return float(np.median([a.elapsed_time(b) for a, b in evs]))

    def rate(nbytes, ms):
        g = nbytes / (ms / 1e3) / 1e9
        return {"ms": round(ms, 5), "GB/s": round(g, 1), "frac_of_" + peak_kind + "_hbm": round(g / hbm, 4)}

    # ---- c1 -----------------------------------------------------------------
    n = 1 << 24
    res = torch.zeros(64, dtype=torch.uint8, device=dev)
    xs = [torch.from_numpy(datagen.uniform_f64(n, seed=c)).to(dev) for c in range(4)]
    calls = [lambda x=x: gbk.check(lib.gbk_reduce(0, 5, P(x.data_ptr()), n, P(res.data_ptr()), sp, None), "sum")
             for x in xs]
    out["c1_sum_f64_2^24"] = rate(n * 8, timed(calls, 40, batch=True))
    del xs, calls
    iv = ctypes.c_int64(0)
    xi = [torch.from_numpy(datagen.uniform_i32(n, 0, 15, seed=c)).to(dev) for c in range(4)]
    ys = [torch.empty(n, dtype=torch.int64, device=dev) for _ in range(4)]
    calls = [lambda x=x, y=y: gbk.check(lib.gbk_scan(0, 0, 1, P(x.data_ptr()), n, ctypes.byref(iv), P(y.data_ptr()),
                                                     None, sp, None), "exscan") for x, y in zip(xi, ys)]
    out["c1_exclusive_scan_i32_i64_2^24"] = rate(n * 12, timed(calls, 40, batch=True))
    del xi, ys, calls

    # ---- c3 -----------------------------------------------------------------
    lens, sigma = datagen.lognormal_lengths(10000, median=2048.0, max_len=1 << 21, target_total=1 << 28, seed=0)
    offs = datagen.offsets_from_lengths(lens)
    ns, nseg = int(offs[-1]), len(lens)
    do = torch.from_numpy(offs).to(dev)
    xf = torch.from_numpy(datagen.normal_f32(ns, seed=0)).to(dev)
    xq = torch.from_numpy(datagen.uniform_i32(ns, 0, 255, seed=0)).to(dev)
    segout = torch.empty(nseg, dtype=torch.float32, device=dev)
    yq = torch.empty(ns, dtype=torch.int32, device=dev)
    ms_sum = timed([lambda: gbk.check(lib.gbk_segmented_reduce(0, 4, P(xf.data_ptr()), P(do.data_ptr()), nseg, ns,
                                                                P(segout.data_ptr()), sp, None), "seg sum")], reps,
                   batch=True)
    ms_scan = timed([lambda: gbk.check(lib.gbk_segmented_scan(1, 0, 0, P(xq.data_ptr()), P(do.data_ptr()), nseg, ns,
                                                               P(yq.data_ptr()), sp, None), "seg scan")], reps,
                    batch=True)
    ob = [int(v) for v in offs]

    def loop_sum():
        for s_ in range(nseg):
            gbk.check(lib.gbk_reduce(0, 4, P(xf.data_ptr() + 4 * ob[s_]), ob[s_ + 1] - ob[s_],
                                     P(segout.data_ptr() + 4 * s_), sp, None), "loop sum")

    def loop_scan():
        for s_ in range(nseg):
            gbk.check(lib.gbk_scan(1, 0, 0, P(xq.data_ptr() + 4 * ob[s_]), ob[s_ + 1] - ob[s_], None,
                                   P(yq.data_ptr() + 4 * ob[s_]), None, sp, None), "loop scan")

    ms_lsum = timed([loop_sum], 1)
    ms_lscan = timed([loop_scan], 1)
    ob_bytes = (nseg + 1) * 8
    out["c3_segmented_sum_f32"] = dict(rate(ns * 4 + ob_bytes + nseg * 4, ms_sum), per_segment_loop_ms=round(ms_lsum, 3),
                                       speedup=round(ms_lsum / ms_sum, 1))
    out["c3_segmented_inclusive_scan_i32"] = dict(rate(ns * 8 + ob_bytes, ms_scan),
                                                  per_segment_loop_ms=round(ms_lscan, 3),
                                                  speedup=round(ms_lscan / ms_scan, 1))
    out["c3_data"] = {"segments": nseg, "elements": ns, "lognormal_sigma": round(float(sigma), 4)}
    del xf, xq, yq, do, segout

    # ---- c3 graph: 8 dependent reduce / scan nodes, replayed as one CUDA graph
    # vs issued as 8 stream launches; nodes of 2^24 values (bandwidth-bound)
    # and of 2^16 values (where launch overhead dominates) ---------------------
    gbk.check(lib.gbk_workspace_reserve(sp, 64 << 20), "workspace_reserve")
    for lg in (24, 16):
        n = 1 << lg
        xg = torch.from_numpy(datagen.uniform_i32(n, 0, 15, seed=1)).to(dev)
        gb = [torch.empty(n, dtype=torch.int64, device=dev) for _ in range(4)]
        gres = torch.zeros(64, dtype=torch.uint8, device=dev)

        def chain():
            gbk.scan(xg, gb[0], inclusive=False, init=0, stream=stream)      # each node reads the previous one
            gbk.reduce("max", gb[0], out=gres[0:8], stream=stream)
            gbk.scan(gb[0], gb[1], inclusive=True, stream=stream)
            gbk.reduce("sum", gb[1], out=gres[8:16], stream=stream)
            gbk.scan(gb[1], gb[2], inclusive=False, init=3, stream=stream)
            gbk.reduce("minloc", gb[2], out=gres[16:32], stream=stream)
            gbk.scan(gb[2], gb[3], inclusive=True, stream=stream)
            gbk.reduce("maxloc", gb[3], out=gres[32:48], stream=stream)

        graph = gbk.Graph(stream)
        with graph:
            chain()
        ms_stream = timed([chain], reps, batch=True)
        ms_graph = timed([graph.submit], reps, batch=True)
        node_bytes = 4 * (n * 12) + 4 * (n * 8)  # scans i32->i64 / i64->i64 read + write, reduces read
        out[f"c3_graph_8_nodes_2^{lg}"] = dict(rate(node_bytes, ms_graph), stream_launches_ms=round(ms_stream, 4),
                                              graph_speedup=round(ms_stream / ms_graph, 3))
        del graph, xg, gb

    # ---- c4 -----------------------------------------------------------------
    thr = None
    thr_path = os.path.join(ROOT, "kokkos_gb300", "comparators", "libgbk_thrust.so")
    if os.path.exists(thr_path):
        thr = ctypes.CDLL(thr_path)
        thr.gbk_cmp_thrust_sort_by_key_u64_i32.argtypes = [P, P, ctypes.c_int64, P]
        thr.gbk_cmp_thrust_sort_u64.argtypes = [P, ctypes.c_int64, P]
    n = 1 << 27
    iota = torch.arange(n, dtype=torch.int32, device=dev)
    dk, dv = torch.empty(n, dtype=torch.int64, device=dev), torch.empty_like(iota)
    for name, kh in (("uniform", datagen.bits_u64(n, seed=0)), ("lowentropy", datagen.lowentropy_u64(n, 8, seed=0)[0])):
        passes = sum(1 for p_ in range(8) if np.any(((kh >> np.uint64(8 * p_)) & np.uint64(255)) !=
                                                  ((kh[0] >> np.uint64(8 * p_)) & np.uint64(255))))
        k0 = torch.from_numpy(kh.view(np.int64)).to(dev)

        def refill(_c, k0=k0):
            dk.copy_(k0)
            dv.copy_(iota)

        ms = timed([lambda: gbk.check(lib.gbk_sort_by_key(3, P(dk.data_ptr()), 4, P(dv.data_ptr()), n, sp),
                                      "sort_by_key")], 3, prep=refill)
        pass_bytes = n * 8 + max(passes - 1, 0) * n * 8 + passes * n * 24
        out["c4_sort_by_key_u64_i32_2^27_" + name] = dict(
            rate(pass_bytes, ms), digit_passes=passes, Gpairs_per_s=round(n / (ms / 1e3) / 1e9, 3),
            min_bytes_GBps=round(n * 24 / (ms / 1e3) / 1e9, 1))
        if thr is not None:
            # the reference's CUDA path: thrust::sort_by_key on the same keys and stream
            ms_t = timed([lambda: thr.gbk_cmp_thrust_sort_by_key_u64_i32(P(dk.data_ptr()), P(dv.data_ptr()), n, sp)],
                         3, prep=refill)
            out["c4_sort_by_key_u64_i32_2^27_" + name].update(
                thrust_sort_by_key_ms=round(ms_t, 4), speedup_vs_thrust=round(ms_t / ms, 3))
        del k0
    # Kokkos::sort of the uniform keys alone, and BinSort with BinOp1D(n / 2 bins, min, max) (the bins the
    # reference's host sort path uses): the bin permutation (stable within a bin), then applying it to the keys
    kh = datagen.bits_u64(n, seed=0)
    k0 = torch.from_numpy(kh.view(np.int64)).to(dev)

    def refill_keys(_c):
        dk.copy_(k0)

    ms = timed([lambda: gbk.check(lib.gbk_sort(3, P(dk.data_ptr()), n, sp), "sort")], 3, prep=refill_keys)
    passes = 8
    out["c4_sort_u64_2^27_uniform"] = dict(rate(n * 8 + (passes - 1) * n * 8 + passes * n * 16, ms),
                                           Gkeys_per_s=round(n / (ms / 1e3) / 1e9, 3))
    if thr is not None:
        ms_t = timed([lambda: thr.gbk_cmp_thrust_sort_u64(P(dk.data_ptr()), n, sp)], 3, prep=refill_keys)
        out["c4_sort_u64_2^27_uniform"].update(thrust_sort_ms=round(ms_t, 4), speedup_vs_thrust=round(ms_t / ms, 3))
    kmin, kmax = float(kh.min()), float(kh.max())
    nb_req = n // 2
    mul = float(nb_req) / (kmax - kmin)
    nbb = nb_req + 1
    bcnt = torch.empty(nbb, dtype=torch.int32, device=dev)
    boff = torch.empty(nbb, dtype=torch.int64, device=dev)
    bperm = torch.empty(n, dtype=torch.int64, device=dev)
    ms_bin = timed([lambda: gbk.check(lib.gbk_binsort_u64(P(k0.data_ptr()), n, nbb, kmin, mul, 0, P(bcnt.data_ptr()),
                                                          P(boff.data_ptr()), P(bperm.data_ptr()), sp), "binsort")], 3)
    ms_perm = timed([lambda: gbk.check(lib.gbk_permute(8, P(k0.data_ptr()), P(bperm.data_ptr()), n, P(dk.data_ptr()), sp),
                                       "permute")], 3)
    out["c4_binsort_u64_2^27_uniform"] = {"binsort_ms": round(ms_bin, 3), "permute_ms": round(ms_perm, 3),
                                          "bins": nbb, "Gkeys_per_s": round(n / ((ms_bin + ms_perm) / 1e3) / 1e9, 3)}
    del k0, bcnt, boff, bperm
    del iota, dk, dv

    # ---- the header-template path for user functors (C++ program) -------------
    hp = os.path.join(ROOT, "kokkos_gb300", "_build", "bench_header_path")
    if os.path.exists(hp):
        lens_h, _ = datagen.lognormal_lengths(10000, median=2048.0, max_len=1 << 21, target_total=1 << 28, seed=0)
        offs_h = datagen.offsets_from_lengths(lens_h)
        with tempfile.TemporaryDirectory() as td:
            fo = os.path.join(td, "offsets.bin")
            offs_h.astype(np.int64).tofile(fo)
            torch.cuda.synchronize()
            r = subprocess.run([hp, fo, str(len(lens_h)), "20"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                               text=True, timeout=600)
        if r.returncode == 0:
            hj = json.loads(r.stdout.strip().splitlines()[-1])
            for v in hj.values():
                for k in ("GB/s", "library_GB/s"):
                    if k in v:
                        v[k.replace("GB/s", "frac_of_" + peak_kind + "_hbm")] = round(v[k] / hbm, 4)
            out["header_path_user_functors"] = hj
        else:
            out["header_path_user_functors"] = {"error": r.stdout[-300:]}

    # ---- data movement either side of the path --------------------------------
    nb = 1 << 30
    a_ = torch.empty(nb // 4, dtype=torch.int32, device=dev)
    b_ = torch.empty_like(a_)
    a_.fill_(1)
    v32 = np.array([7], dtype=np.int32)
    out["deep_copy_d2d_1GiB"] = rate(2 * nb, timed(
        [lambda: gbk.check(lib.gbk_deep_copy(P(b_.data_ptr()), P(a_.data_ptr()), nb, sp), "deep_copy")], reps))
    out["fill_i32_1GiB"] = rate(nb, timed(
        [lambda: gbk.check(lib.gbk_fill(P(b_.data_ptr()), P(v32.ctypes.data), 4, nb // 4, sp), "fill")], reps))
    np_ = 1 << 26
    perm = torch.from_numpy(np.random.default_rng(0).permutation(np_).astype(np.int64)).to(dev)
    out["permute_i32_2^26_random"] = rate(np_ * 16, timed(
        [lambda: gbk.check(lib.gbk_permute(4, P(a_.data_ptr()), P(perm.data_ptr()), np_, P(b_.data_ptr()), sp),
                           "permute")], reps))
    del a_, b_, perm
    return out


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU implementation of the path on
    this host.  The reference build (oracle/_ref) is produced in a container
    with the reference sources and is x86-only; on any other host the oracle
    port of the same algorithms is timed."""
    if rank != 0:
        return
    cb = cpu_baseline(budget_s=max(5.0, 2.0 * (args.steps + args.warmup)))
    line = {"metric": METRIC, "value": cb["value"], "unit": "GB/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(STEP_BYTES / (cb["value"] * 1e9) * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, seed 0)",
            "config": {"workload": WORKLOAD, "step_bytes": STEP_BYTES}, "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbk", choices=["gbk", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other headline workloads (C1 sum/scan, C3 segmented, C4 sort) timed after the step")
    ap.add_argument("--no-tuning-table", action="store_true",
                    help="use the library defaults instead of the autotuner's table (kokkos_gb300/tuning_table.txt)")
    ap.add_argument("--only", default=None,
                    choices=["minloc", "maxloc", "sum", "hist", "sum_f64", "exscan", "sort", "segsum", "segscan"],
                    help="run just this operation warmup+steps times (for profiler captures): the bench ops on the "
                         "bench inputs, or sum_f64 / exscan on 2^24 doubles / int32 (the RangePolicy Sum and "
                         "exclusive_scan i32->i64 workload), or sort: sort_by_key of --sort-n uniform uint64 keys "
                         "with an int32 iota payload (the sort_by_key workload, 2^27 by default), or segsum / segscan: the "
                         "segmented Sum (f32) / inclusive_scan (i32) of --seg-total elements in lognormal segments")
    ap.add_argument("--sort-n", type=int, default=1 << 27)
    ap.add_argument("--sum-n", type=int, default=1 << 24, help="elements for --only sum_f64 / exscan")
    ap.add_argument("--seg-total", type=int, default=1 << 28,
                    help="--only segsum: elements of the lognormal segments (10,000 segments per 2^28, median 2,048)")
    ap.add_argument("--sort-keys", default="uniform", choices=["uniform", "lowentropy"],
                    help="--only sort keys: uniform 64-bit, or a seeded base pattern with 8 random bit positions")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    args.warmup = max(args.warmup, 3)

    import torch

    from kokkos_gb300 import datagen, gbk
    dist = init_dist(world)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    lib = gbk.lib
    table = os.path.join(ROOT, "kokkos_gb300", "tuning_table.txt")
    tuned = False
    if not args.no_tuning_table and os.path.exists(table):
        tuned = lib.gbk_tuner_load(table.encode()) == 0 and lib.gbk_tuner_enable(1) == 0

    if args.only == "sort":
        n = args.sort_n
        kh = datagen.bits_u64(n, seed=0) if args.sort_keys == "uniform" else datagen.lowentropy_u64(n, 8, seed=0)[0]
        k0 = torch.from_numpy(kh.view(np.int64)).to(dev)
        iota = torch.arange(n, dtype=torch.int32, device=dev)
        dk, dv = torch.empty_like(k0), torch.empty_like(iota)
        evs = []
        for _ in range(args.warmup + args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                # refill on the sort's own stream: the previous sort must finish before its input changes
                dk.copy_(k0)
                dv.copy_(iota)
                e0.record(stream)
                gbk.check(lib.gbk_sort_by_key(3, ctypes.c_void_p(dk.data_ptr()), 4, ctypes.c_void_p(dv.data_ptr()),
                                              n, sp), "sort_by_key")
                e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        gbk.stream_check(stream)
        ms = [a.elapsed_time(b) for a, b in evs[args.warmup:]]
        print(json.dumps({"only": "sort", "keys": args.sort_keys, "n": n, "ms": ms, "Gpairs/s": [round(n / m / 1e6, 3) for m in ms]}))
        return
    if args.only in ("segsum", "segscan"):
        total = args.seg_total
        nseg = max(1, int(round(10000 * total / (1 << 28))))
        lens, _ = datagen.lognormal_lengths(nseg, median=2048.0, max_len=1 << 21, target_total=total, seed=0)
        offs = datagen.offsets_from_lengths(lens)
        ns = int(offs[-1])
        do = torch.from_numpy(offs).to(dev)
        if args.only == "segsum":
            xf = torch.from_numpy(datagen.normal_f32(ns, seed=0)).to(dev)
            so = torch.empty(nseg, dtype=torch.float32, device=dev)
            call = lambda: gbk.check(lib.gbk_segmented_reduce(  # noqa: E731
                0, 4, ctypes.c_void_p(xf.data_ptr()), ctypes.c_void_p(do.data_ptr()), nseg, ns,
                ctypes.c_void_p(so.data_ptr()), sp, None), "segsum")
        else:
            xq = torch.from_numpy(datagen.uniform_i32(ns, 0, 255, seed=0)).to(dev)
            yq = torch.empty(ns, dtype=torch.int32, device=dev)
            call = lambda: gbk.check(lib.gbk_segmented_scan(  # noqa: E731
                1, 0, 0, ctypes.c_void_p(xq.data_ptr()), ctypes.c_void_p(do.data_ptr()), nseg, ns,
                ctypes.c_void_p(yq.data_ptr()), sp, None), "segscan")
        with torch.cuda.stream(stream):
            for _ in range(args.warmup + args.steps):
                call()
        torch.cuda.synchronize()
        gbk.stream_check(stream)
        print(json.dumps({"only": args.only, "elements": ns, "segments": nseg, "launches": args.warmup + args.steps}))
        return
    if args.only in ("sum_f64", "exscan"):
        n = args.sum_n
        res = torch.zeros(64, dtype=torch.uint8, device=dev)
        if args.only == "sum_f64":
            x = torch.from_numpy(datagen.uniform_f64(n, seed=0)).to(dev)
            call = lambda: gbk.check(lib.gbk_reduce(0, 5, ctypes.c_void_p(x.data_ptr()), n,  # noqa: E731
                                                    ctypes.c_void_p(res.data_ptr()), sp, None), "sum_f64")
        else:
            x = torch.from_numpy(datagen.uniform_i32(n, 0, 15, seed=0)).to(dev)
            y = torch.empty(n, dtype=torch.int64, device=dev)
            iv = ctypes.c_int64(0)
            call = lambda: gbk.check(lib.gbk_scan(0, 0, 1, ctypes.c_void_p(x.data_ptr()), n, ctypes.byref(iv),  # noqa: E731
                                                  ctypes.c_void_p(y.data_ptr()), None, sp, None), "exscan")
        with torch.cuda.stream(stream):
            for _ in range(args.warmup + args.steps):
                call()
        torch.cuda.synchronize()
        gbk.stream_check(stream)
        print(json.dumps({"only": args.only, "launches": args.warmup + args.steps}))
        return

    # ---- inputs (pinned host, seeded) and their device copies --------------
    hx = torch.empty(NX, dtype=torch.float32, pin_memory=True)
    hk = torch.empty(NKEYS, dtype=torch.int32, pin_memory=True)
    datagen.normal_f32(NX, seed=0 + rank, out=hx.numpy())
    datagen.zipf_i32(NKEYS, NBINS, 1.1, seed=0 + rank, out=hk.numpy())
    dx = hx.to(dev, non_blocking=False)
    dk = hk.to(dev, non_blocking=False)
    dbins = torch.zeros(NBINS, dtype=torch.int64, device=dev)
    dres = torch.zeros(256, dtype=torch.uint8, device=dev)
    hres = torch.zeros(256, dtype=torch.uint8, pin_memory=True)
    hbins = torch.zeros(NBINS, dtype=torch.int64, pin_memory=True)
    torch.cuda.synchronize()

    rk = 3
    lo = (ctypes.c_int64 * rk)(0, 0, 0)
    up = (ctypes.c_int64 * rk)(N0, N1, N2)
    st = (ctypes.c_int64 * rk)(1, N0, N0 * N1)
    X, K, B, R = (ctypes.c_void_p(t.data_ptr()) for t in (dx, dk, dbins, dres))
    R0, R1, R2 = (ctypes.c_void_p(dres.data_ptr() + o) for o in (0, 64, 128))

    def op_minloc():
        gbk.check(lib.gbk_mdrange_reduce(8, 4, X, rk, lo, up, st, R0, sp, None), "minloc")

    def op_maxloc():
        gbk.check(lib.gbk_mdrange_reduce(9, 4, X, rk, lo, up, st, R1, sp, None), "maxloc")

    def op_sum():
        gbk.check(lib.gbk_mdrange_reduce(0, 4, X, rk, lo, up, st, R2, sp, None), "sum")

    zero8 = np.zeros(1, dtype=np.int64)
    Z8 = ctypes.c_void_p(zero8.ctypes.data)

    def op_hist():
        # deep_copy(bins, 0) then the contribution (both kernels, launched back to back)
        gbk.check(lib.gbk_fill(B, Z8, 8, NBINS, sp), "zero bins")
        gbk.check(lib.gbk_histogram_i32_i64(K, NKEYS, B, NBINS, sp, None), "histogram")

    ops = [("mdrange_minloc_f32", op_minloc, RED_BYTES), ("mdrange_maxloc_f32", op_maxloc, RED_BYTES),
           ("mdrange_sum_f32", op_sum, RED_BYTES), ("histogram_zipf_2^16", op_hist, HIST_BYTES)]

    if args.only:
        f = {"minloc": op_minloc, "maxloc": op_maxloc, "sum": op_sum, "hist": op_hist}[args.only]
        with torch.cuda.stream(stream):
            for _ in range(args.warmup + args.steps):
                f()
        torch.cuda.synchronize()
        gbk.stream_check(stream)
        print(json.dumps({"only": args.only, "launches": args.warmup + args.steps}))
        return

    def step(evs=None):
        for i, (_, f, _) in enumerate(ops):
            if evs is not None:
                evs[i][0].record(stream)
            f()
            if evs is not None:
                evs[i][1].record(stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    gbk.stream_check(stream)

    # ---- timed region: device path ------------------------------------------
    evs = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in ops]
           for _ in range(args.steps)]
    clocks = Clocks(local)
    barrier(dist)
    torch.cuda.synchronize()
    l0 = gbk.launch_count()
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        t_start.record(stream)
        for s_ in range(args.steps):
            step()
        t_end.record(stream)
    torch.cuda.synchronize()
    barrier(dist)
    launches = gbk.launch_count() - l0
    clk = clocks.stop()
    gbk.stream_check(stream)
    # Per operation: the same K steps again, with events around each operation
    # (outside the timed region: an event between two kernels keeps the
    # second from being scheduled while the first runs).
    with torch.cuda.stream(stream):
        for s_ in range(args.steps):
            step(evs[s_])
    torch.cuda.synchronize()
    ms_total = t_start.elapsed_time(t_end)
    ms_total = max_over_ranks(dist, ms_total)
    ms_step = ms_total / args.steps
    value = job_gbs(world, args.steps, ms_total)

    per_op = {}
    hbm, peak_kind = peaks()
    for i, (name, _, nbytes) in enumerate(ops):
        ts = [evs[s_][i][0].elapsed_time(evs[s_][i][1]) for s_ in range(args.steps)]
        avg = float(np.mean(ts))
        gbs = nbytes / (avg / 1e3) / 1e9
        per_op[name] = {"ms": round(avg, 5), "GB/s": round(gbs, 1), "frac_of_" + peak_kind + "_hbm": round(gbs / hbm, 4)}
    red_ms = np.mean([per_op[n]["ms"] for n in ("mdrange_minloc_f32", "mdrange_maxloc_f32", "mdrange_sum_f32")])
    red_gbs = RED_BYTES / (red_ms / 1e3) / 1e9

    # Each operation again with L2 emptied of its input first: a read of a
    # 256 MiB buffer (clean lines, so no write-back is charged to the timed
    # call) between calls; median of 10 calls per operation.  In the step,
    # MaxLoc and Sum follow MinLoc over the same view, so part of their input
    # can still be in L2; these numbers have none of that.
    flush = torch.empty(1 << 26, dtype=torch.float32, device=dev).fill_(1.0)
    FL = ctypes.c_void_p(flush.data_ptr())
    fres = torch.zeros(64, dtype=torch.uint8, device=dev)
    FR = ctypes.c_void_p(fres.data_ptr())
    cold = {}
    with torch.cuda.stream(stream):
        for name, f, nbytes in ops:
            ce = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(10)]
            for a_, b_ in ce:
                gbk.check(lib.gbk_reduce(3, 4, FL, 1 << 26, FR, sp, None), "flush")  # Max: a plain read
                a_.record(stream)
                f()
                b_.record(stream)
            torch.cuda.synchronize()
            gbk.stream_check(stream)
            c_ms = float(np.median([a_.elapsed_time(b_) for a_, b_ in ce]))
            gbs = nbytes / (c_ms / 1e3) / 1e9
            cold[name] = {"ms": round(c_ms, 5), "GB/s": round(gbs, 1), "frac_of_" + peak_kind + "_hbm": round(gbs / hbm, 4)}
    del flush
    red_cold_ms = np.mean([cold[n]["ms"] for n in ("mdrange_minloc_f32", "mdrange_maxloc_f32", "mdrange_sum_f32")])
    red_cold_gbs = RED_BYTES / (red_cold_ms / 1e3) / 1e9

    # Each reduce launched 20 times back to back between two events, the view
    # and a copy of it taking turns (268 MB each, twice the L2, so every launch
    # reads its input from HBM): the kernel's own duration, its launch latency
    # hidden as in the step.  This is the roofline's `achieved`.
    dx2 = dx.clone()
    X2 = ctypes.c_void_p(dx2.data_ptr())
    b2b = {}
    with torch.cuda.stream(stream):
        for name, code, outp in (("mdrange_minloc_f32", 8, R0), ("mdrange_maxloc_f32", 9, R1), ("mdrange_sum_f32", 0, R2)):
            def call(i, code=code, outp=outp, name=name):
                gbk.check(lib.gbk_mdrange_reduce(code, 4, X if i % 2 == 0 else X2, rk, lo, up, st, outp, sp, None), name)
            for i in range(4):
                call(i)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for i in range(20):
                call(i)
            e1.record(stream)
            torch.cuda.synchronize()
            gbk.stream_check(stream)
            b_ms = e0.elapsed_time(e1) / 20
            gbs = RED_BYTES / (b_ms / 1e3) / 1e9
            b2b[name] = {"ms": round(b_ms, 5), "GB/s": round(gbs, 1), "frac_of_" + peak_kind + "_hbm": round(gbs / hbm, 4)}
    del dx2
    red_b2b_gbs = RED_BYTES / (np.mean([v["ms"] for v in b2b.values()]) / 1e3) / 1e9

    # The same three results from one pass: MinMaxLoc and Sum as two reducers
    # of one parallel_reduce over the box (reported beside the step, not in it).
    R3 = ctypes.c_void_p(dres.data_ptr() + 192)
    fev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(20)]
    with torch.cuda.stream(stream):
        for a_, b_ in [(None, None)] * 3 + fev:
            if a_ is not None:
                a_.record(stream)
            gbk.check(lib.gbk_mdrange_reduce(12, 4, X, rk, lo, up, st, R3, sp, None), "minmaxloc_sum")
            if b_ is not None:
                b_.record(stream)
    torch.cuda.synchronize()
    gbk.stream_check(stream)
    f_ms = float(np.median([a_.elapsed_time(b_) for a_, b_ in fev]))
    f_gbs = RED_BYTES / (f_ms / 1e3) / 1e9
    fused = {"ms": round(f_ms, 5), "GB/s": round(f_gbs, 1), "frac_of_" + peak_kind + "_hbm": round(f_gbs / hbm, 4),
             "three_passes_ms": round(3 * red_ms, 5)}

    # ---- e2e: through the C ABI from pinned host buffers ---------------------
    HX, HK = ctypes.c_void_p(hx.data_ptr()), ctypes.c_void_p(hk.data_ptr())
    HR, HB = ctypes.c_void_p(hres.data_ptr()), ctypes.c_void_p(hbins.data_ptr())

    # Three streams, as an application would issue them.  The host link
    # carries about 211 GB/s to the device however the copies are issued
    # (one or several copy engines, or kernels reading pinned host memory),
    # so the step keeps it busy: the keys are copied on a second stream once
    # the view's copy is done, so the three reduces over the view overlap the
    # keys' copy, and in KCH pieces, each counted into the bins (on a third
    # stream) while the next piece is copied; only the last piece's histogram
    # and the result copies follow the link.
    stream2 = torch.cuda.Stream(device=dev)
    stream3 = torch.cuda.Stream(device=dev)
    sp2 = ctypes.c_void_p(stream2.cuda_stream)
    sp3 = ctypes.c_void_p(stream3.cuda_stream)
    x_in = torch.cuda.Event()
    KCH = 8
    kch = NKEYS // KCH
    k_in = [torch.cuda.Event() for _ in range(KCH)]

    def e2e_step():
        gbk.check(lib.gbk_deep_copy(X, HX, NX * 4, sp), "h2d x")
        x_in.record(stream)
        stream2.wait_event(x_in)
        gbk.check(lib.gbk_memset(B, 0, NBINS * 8, sp3), "memset")
        for i in range(KCH):
            off = i * kch * 4
            gbk.check(lib.gbk_deep_copy(ctypes.c_void_p(K.value + off), ctypes.c_void_p(HK.value + off), kch * 4,
                                        sp2), "h2d keys")
            k_in[i].record(stream2)
            stream3.wait_event(k_in[i])
            gbk.check(lib.gbk_histogram_i32_i64(ctypes.c_void_p(K.value + off), kch, B, NBINS, sp3, None),
                      "histogram")
        op_minloc()
        op_maxloc()
        op_sum()
        gbk.check(lib.gbk_deep_copy(HR, R, 192, sp), "d2h results")
        gbk.check(lib.gbk_deep_copy(HB, B, NBINS * 8, sp3), "d2h bins")
        stream.synchronize()
        stream3.synchronize()

    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(2):
        e2e_step()
    barrier(dist)
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e_ms = (time.perf_counter() - e0) * 1e3 / e2e_steps
    e_ms = max_over_ranks(dist, e_ms)
    e2e_val = job_gbs(world, 1, e_ms)
    gbk.stream_check(stream)
    gbk.stream_check(stream3)

    # correctness spot check of the last step's results (rank-local, cheap)
    r = hres.numpy()
    mn = gbk.decode_result(r[0:16], 8, 4)
    hx_np = hx.numpy()
    ok = bool(mn["val"] == hx_np.min() and int(hbins.numpy().sum()) == NKEYS)

    line = {
        "metric": METRIC,
        "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded xoshiro256**, seed 0; N(0,1) floats, Zipf(1.1) keys)",
        "config": {"workload": WORKLOAD, "step_bytes": STEP_BYTES, "l2": ("inputs 268 MB each > 129 MB L2, no flush in the step; MaxLoc and Sum re-read the view MinLoc "
                          "just read, so part of it can still be in L2 (ops_cold_l2: each op after a 256 MiB read)"),
                   "parallelism": f"replicas x{world}",
                   "launch_config": "autotuner table" if tuned else "library defaults",
                   "kernels": launch_shapes(gbk, tuned)},
        "roofline": {"bound": "hbm", "kernel": ROOF_KERNEL,
                     "achieved": round(red_b2b_gbs, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(red_b2b_gbs / hbm, 4), "peak_kind": peak_kind + " hbm_gbs (burst copy)",
                     "traffic": ROOF_TRAFFIC,
                     "achieved_how": "20 back-to-back launches per reducer, two copies of the view taking turns "
                                     "(each twice the L2), CUDA events around the 20",
                     "achieved_in_step": round(red_gbs, 1), "frac_in_step": round(red_gbs / hbm, 4),
                     "achieved_cold_l2": round(red_cold_gbs, 1), "frac_cold_l2": round(red_cold_gbs / hbm, 4)},
        "ops_back_to_back": b2b,
        "ops": per_op,
        "ops_cold_l2": cold,
        "e2e": {"value": round(e2e_val, 1), "unit": "GB/s", "ms_per_step": round(e_ms, 3),
                "h2d_bytes_per_step": NX * 4 + NKEYS * 4, "d2h_bytes_per_step": 192 + NBINS * 8},
        "gpu_launches": int(launches),
        "gpu_launches_per_step": launches / args.steps,
        "clocks": clk,
        "result_check": ok,
    }
    if world == 1 and not args.no_configs:
        line["other_configs"] = other_configs(torch, gbk, datagen, stream, dev, hbm, peak_kind)
        line["other_configs"]["c2_minmaxloc_sum_one_pass_f32"] = fused
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
