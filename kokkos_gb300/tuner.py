"""Autotuner and learned tuner for libgbk launch configurations.

* Exhaustive autotuner: for a workload (operation kind, element type, size,
  segment statistics, histogram bins and key entropy) every candidate launch
  configuration is timed through the C ABI with CUDA events: inputs of at
  least twice the L2 as consecutive calls (two copies taking turns where the
  buffer has room; launch latency hidden, as in a stream of kernels), smaller
  ones one call at a time after a read that empties L2 of them (median of 3).
* Learned tuner: an ensemble of five 3-layer, 64-hidden FP32 MLPs (features
  of the workload and of a candidate configuration -> log time relative to
  the workload's mean), trained with the library's own CUDA kernels
  (gbk_mlp_forward / backward / mse / adam); for an unseen workload it picks
  the candidate with the smallest mean predicted time.  The exhaustive tuner
  stays the fallback and the yardstick of its regret; the tuning table (the
  exhaustive best per bucket, looked up at the nearest bucket) is the method
  without the MLP that it is compared with.
* The tuning table (text, loaded by gbk_tuner_load) maps (kind, op, dtype,
  log2 n, extra) to the chosen configuration; the entry points consult it
  when called without an explicit configuration.

    python -m kokkos_gb300.tuner --train-workloads 1350 --eval-workloads 2000 --out <dir>
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import time

import numpy as np

KIND_REDUCE, KIND_SCAN, KIND_HIST, KIND_SEG, KIND_SEGSCAN = 0, 1, 2, 3, 4
REDUCE_CFGS = [(b, u, c) for (b, u) in [(256, 2), (256, 4), (256, 8), (512, 2), (512, 4), (128, 8), (1024, 2)]
               for c in (1, 2, 4, 8)]
SCAN_CFGS = [(9, 0), (7, 0), (3, 0), (9, 1)]  # (vectors per thread, CTAs per SM; 0 = all resident)
# segmented reduce (variant, vectors per thread, CTAs per SM; 0 = all resident): variant 0 is the
# contiguous-share kernel (its shape is fixed), variant 1 the tile pipeline
SEG_CFGS = [(0, 7, 0), (1, 7, 0), (1, 3, 0), (1, 7, 1)]
# segmented scan (the tile pipeline; vectors per thread, CTAs per SM; 5 runs three stages)
SEGSCAN_CFGS = [(7, 0), (5, 0), (3, 0), (7, 1), (5, 1), (3, 1)]
# histogram (variant, ctas_per_sm): 32-bit privatised (cluster 1/2), 16-bit with periodic drains (0x20),
# drain-free (0x80), drain-free in the multiply form for power-of-two bins (0x100) and the same with one
# crossing test per round (0x200), no privatisation (0x40)
HIST_CFGS_SMALL = [(0x01, 1), (0x01, 2), (0x11, 2), (0x20, 1), (0x30, 1), (0x40, 1)]
HIST_CFGS_2E16 = [(0x02, 1), (0x12, 1), (0x04, 1), (0x20, 1), (0x30, 1), (0x80, 1), (0x100, 1), (0x200, 1),
                  (0x40, 1)]
SPLIT_CFGS = [(3, 0), (4, 0), (5, 0), (6, 0), (5, 2)]  # double Sum, variant 3: (vectors per thread, CTAs per SM)
# (op, dtype code); "mmls" is the fused MinMaxLoc+Sum reducer
REDUCE_OPS = [("sum", 5), ("sum", 4), ("minloc", 4), ("maxloc", 4), ("mmls", 4), ("sum", 0), ("sum", 1)]
OPC = {"sum": 0, "minloc": 8, "maxloc": 9, "mmls": 12}
NFEAT = 34
# Timing regime: inputs of at least twice the 129 MB L2 are timed as BACK_TO_BACK
# consecutive calls (launch latency hidden, as in a stream of kernels); smaller
# ones one call at a time after a 256 MiB read that empties L2 of them.
BACK_TO_BACK_BYTES = 2 * 129 * 1000 * 1000
BACK_TO_BACK = 6


def candidates(w):
    k = w["kind"]
    if k == KIND_REDUCE:
        # variant 1: load-pipelined kernel; variant 2: shared-memory ring kernel; variant 3 (double
        # Sum only): adds split between the FP64 pipe and an integer fixed-point accumulator
        cs = [{"block": b, "ipt": u, "cps": c, "variant": 1} for (b, u, c) in REDUCE_CFGS] + \
             [{"block": 256, "ipt": 4, "cps": c, "variant": 2} for c in (0, 2)]
        if w.get("op", 0) == 0 and w["dtype"] == 5:
            cs += [{"block": 256, "ipt": u, "cps": c, "variant": 3} for (u, c) in SPLIT_CFGS]
        return cs
    if k == KIND_SCAN:
        return [{"block": 256, "ipt": u, "cps": c, "variant": 0} for (u, c) in SCAN_CFGS]
    if k == KIND_SEG:
        return [{"block": 256, "ipt": u, "cps": c, "variant": v} for (v, u, c) in SEG_CFGS]
    if k == KIND_SEGSCAN:
        return [{"block": 256, "ipt": u, "cps": c, "variant": 1} for (u, c) in SEGSCAN_CFGS]
    cf = HIST_CFGS_2E16 if w["nbins"] > 24576 else HIST_CFGS_SMALL
    return [{"block": 0, "ipt": 0, "cps": c, "variant": v} for (v, c) in cf]


def features(w, c):
    """Workload + candidate features (NFEAT floats, roughly unit scale)."""
    f = np.zeros(NFEAT, dtype=np.float32)
    k = w["kind"]
    f[min(k, KIND_SEG)] = 1.0                            # 0..3 kind one-hot (both segmented kinds: 3)
    f[24] = float(k == KIND_SEGSCAN)                     # segmented scan
    f[4 + w["dtype"]] = 1.0                              # 4..9 dtype one-hot
    op = w.get("op", 0)
    if k == KIND_REDUCE:
        f[10] = float(op in (8, 9, 12))                  # *Loc reducer
        f[25] = float(op == 12)                          # fused MinMaxLoc+Sum
    elif k in (KIND_SCAN, KIND_SEGSCAN):
        f[27] = float(op & 1)                            # inclusive
    f[11] = (math.log2(max(w["n"], 1)) - 22.0) / 6.0     # size
    f[12] = (w.get("seg_log2mean", 0.0) - 11.0) / 4.0    # segment-length mean (log2)
    f[13] = w.get("seg_sigma", 0.0) / 2.0                # segment-length spread (lognormal sigma)
    f[14] = (math.log2(max(w.get("nbins", 1), 1)) - 12.0) / 4.0
    f[15] = w.get("entropy_bits", 0.0) / 16.0            # key entropy
    f[16] = (math.log2(max(w.get("inner_extent", 1), 1))) / 10.0  # MDRange inner extent
    f[17] = (math.log2(max(c["block"], 1)) - 8.0) / 2.0
    f[18] = (math.log2(max(c["ipt"], 1)) - 2.0) / 1.5
    f[19] = (math.log2(max(c["cps"], 1)) - 2.0) / 2.0
    v = c["variant"]
    if k == KIND_SEG:
        f[20] = float(v == 1)                            # segmented reduce: the tile pipeline
    elif k == KIND_REDUCE:
        f[20] = float(v == 2)                            # reduce: the ring kernel
        f[21] = float(v == 3)                            # reduce: the FP64 / integer split kernel
    elif k == KIND_HIST:
        f[20] = float((v & 0xF) > 1) if v and not (v & 0x3E0) else 0.0  # cluster-split bins
        f[21] = float((v & 0x10) != 0)                   # warp aggregation
        f[22] = float((v & 0x3A0) != 0)                  # 16-bit bins
        f[23] = float((v & 0x40) != 0)                   # no privatisation
        f[26] = float((v & 0x380) != 0) + float((v & 0x300) != 0)  # without drains (2: multiply form)
        f[25] = float((v & 0x200) != 0)                  # one crossing test per round
    # size x candidate interactions: the best tile depth, block and CTAs per SM move with the size
    f[28] = f[11] * f[18]
    f[29] = f[11] * f[19]
    f[30] = f[11] * f[17]
    f[31] = f[11] * f[11]
    f[32] = float(c["cps"] == 0)                         # all resident CTAs
    f[33] = f[11] * f[20]
    return f


def sample_workloads(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        r = rng.random()
        if r < 0.40:
            op, dt = REDUCE_OPS[rng.integers(len(REDUCE_OPS))]
            n = int(2 ** rng.uniform(16, 27 if dt in (1, 5) else 28))
            out.append({"kind": KIND_REDUCE, "op": OPC[op], "opname": op, "dtype": dt, "n": n, "inner_extent": 1})
        elif r < 0.55:
            n = int(2 ** rng.uniform(16, 28))
            out.append({"kind": KIND_SCAN, "op": int(rng.integers(2)), "dtype": 0, "n": n})
        elif r < 0.72:
            nb = int(rng.choice([256, 4096, 65536]))
            out.append({"kind": KIND_HIST, "op": 0, "dtype": 0, "n": int(2 ** rng.uniform(16, 26)), "nbins": nb,
                        "pool": int(rng.integers(5))})
        else:
            # batched segments (lognormal lengths): Sum of f32, or an int32 -> int64 scan
            nseg = int(2 ** rng.uniform(6, 13.3))
            l2m = float(rng.uniform(6, 13))
            sig = float(rng.uniform(0.3, 2.5))
            total = min(int(nseg * 2 ** l2m), 1 << 27)
            w = {"kind": KIND_SEG, "op": 0, "dtype": 4, "n": total, "nseg": nseg, "seg_log2mean": l2m,
                 "seg_sigma": sig, "seed": int(rng.integers(1 << 30))}
            if r >= 0.86:
                w.update(kind=KIND_SEGSCAN, op=int(rng.integers(2)), dtype=0)
            out.append(w)
    return out


class Bench:
    """Device buffers reused by all workloads (prefixes of large seeded arrays)."""

    def __init__(self, max_n=1 << 28):
        import torch

        from kokkos_gb300 import datagen, gbk
        self.torch, self.gbk, self.datagen = torch, gbk, datagen
        self.s = torch.cuda.Stream()
        self.sp = ctypes.c_void_p(self.s.cuda_stream)
        self.max_n = max_n
        g = torch.Generator(device="cuda")
        g.manual_seed(0)
        self.f32 = torch.randn(max_n, device="cuda", generator=g)
        self.f64 = self.f32[: max_n // 2].double()
        self.i32 = torch.randint(0, 256, (max_n,), device="cuda", dtype=torch.int32, generator=g)
        self.i64 = self.i32[: max_n // 2].long()
        self.y64 = torch.empty(max_n, dtype=torch.int64, device="cuda")
        self.res = torch.zeros(256, dtype=torch.uint8, device="cuda")
        self.pools, self.pool_entropy = [], []
        nk = min(1 << 26, max_n)
        for i, s_ in enumerate([0.0, 0.6, 0.9, 1.1, 1.4]):
            keys = datagen.uniform_i32(nk, 0, 65535, seed=i) if s_ == 0.0 else datagen.zipf_i32(nk, 65536, s_, seed=i)
            self.pools.append(torch.from_numpy(keys).cuda())
        self.bins = torch.zeros(65536, dtype=torch.int64, device="cuda")
        self._ent = {}
        self.seg_cache = {}
        # Read before every timed call: inputs start cold in L2, as in the bench, and the lines
        # that evict them are clean (a written flush buffer would be written back to HBM during
        # the timed call, which the bench step never does).
        self.flush = torch.ones(256 << 20, dtype=torch.uint8, device="cuda")
        self.flush_sink = torch.zeros(1, dtype=torch.int64, device="cuda")

    def entropy(self, pool, nbins):
        key = (pool, nbins)
        if key not in self._ent:
            k = self.pools[pool][: 1 << 22] % nbins
            c = self.torch.bincount(k.long(), minlength=nbins).double()
            p = c[c > 0] / c.sum()
            self._ent[key] = float(-(p * p.log2()).sum().item())
        return self._ent[key]

    def prepare(self, w):
        if w["kind"] == KIND_REDUCE:
            w["n"] = min(w["n"], (self.max_n // 2) if w["dtype"] in (1, 5) else self.max_n)
        if w["kind"] in (KIND_SCAN,):
            w["n"] = min(w["n"], self.max_n)
        if w["kind"] == KIND_HIST:
            w["n"] = min(w["n"], self.pools[0].numel())
            w["entropy_bits"] = self.entropy(w["pool"], w["nbins"])
            w["keys"] = (self.pools[w["pool"]][: w["n"]] % w["nbins"]).contiguous() if w["nbins"] < 65536 \
                else self.pools[w["pool"]][: w["n"]]
        if w["kind"] in (KIND_SEG, KIND_SEGSCAN):
            lens, _ = self.datagen.lognormal_lengths(w["nseg"], median=2 ** w["seg_log2mean"], max_len=1 << 24,
                                                     target_total=min(w["n"], self.max_n // 2), seed=w["seed"])
            lens = np.minimum(lens, max(1, (self.max_n // 2) // max(w["nseg"], 1)))
            offs = self.datagen.offsets_from_lengths(lens)
            w["n"] = int(offs[-1])
            w["offsets"] = self.torch.from_numpy(offs).cuda()
            w["segout"] = self.torch.empty(w["nseg"], dtype=self.torch.float32, device="cuda")

    def _half(self, buf, n, alt):
        """Address of the workload's input: the buffer's start, or (alt) its
        second half when the input fits there (a second copy of the same
        distribution)."""
        off = buf.numel() // 2 if alt and n <= buf.numel() // 2 else 0
        return ctypes.c_void_p(buf.data_ptr() + off * buf.element_size())

    def call(self, w, c, alt=False):
        gbk, lib, sp = self.gbk, self.gbk.lib, self.sp
        t = gbk.Tuning(c["block"], c["ipt"], c["cps"], c["variant"])
        k = w["kind"]
        if k == KIND_REDUCE:
            buf = {5: self.f64, 4: self.f32, 0: self.i32, 1: self.i64}[w["dtype"]]
            return lib.gbk_reduce(w["op"], w["dtype"], self._half(buf, w["n"], alt), w["n"],
                                  ctypes.c_void_p(self.res.data_ptr()), sp, ctypes.byref(t))
        if k == KIND_SCAN:
            iv = ctypes.c_int64(0)
            return lib.gbk_scan(w["op"], 0, 1, self._half(self.i32, w["n"], alt), w["n"], ctypes.byref(iv),
                                ctypes.c_void_p(self.y64.data_ptr()), None, sp, ctypes.byref(t))
        if k == KIND_HIST:
            return lib.gbk_histogram_i32_i64(ctypes.c_void_p(w["keys"].data_ptr()), w["n"],
                                             ctypes.c_void_p(self.bins.data_ptr()), w["nbins"], sp, ctypes.byref(t))
        if k == KIND_SEGSCAN:
            return lib.gbk_segmented_scan(w["op"], 0, 1, self._half(self.i32, w["n"], alt),
                                          ctypes.c_void_p(w["offsets"].data_ptr()), w["nseg"], w["n"],
                                          ctypes.c_void_p(self.y64.data_ptr()), sp, ctypes.byref(t))
        return lib.gbk_segmented_reduce(0, 4, self._half(self.f32, w["n"], alt),
                                        ctypes.c_void_p(w["offsets"].data_ptr()), w["nseg"], w["n"],
                                        ctypes.c_void_p(w["segout"].data_ptr()), sp, ctypes.byref(t))

    @staticmethod
    def input_bytes(w):
        if w["kind"] == KIND_REDUCE:
            return w["n"] * (8 if w["dtype"] in (1, 3, 5) else 4)
        return w["n"] * 4  # int32 keys, int32 scan input, float / int32 segment values

    def time(self, w, c, reps=3):
        torch = self.torch
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2 * reps)]
        st = self.call(w, c)  # warm-up
        if st:
            return float("inf")
        if self.input_bytes(w) >= BACK_TO_BACK_BYTES:
            # Inputs of at least twice the L2: BACK_TO_BACK calls between two
            # events, alternating between two copies where the buffer has room
            # (every call reads from HBM), so the launch latency is hidden as
            # in a sequence of kernels on a stream.
            self.call(w, c, alt=True)
            e0, e1 = e[0], e[1]
            e0.record(self.s)
            for i in range(BACK_TO_BACK):
                self.call(w, c, alt=bool(i & 1))
            e1.record(self.s)
            e1.synchronize()
            return e0.elapsed_time(e1) / BACK_TO_BACK * 1e3  # us
        for r in range(reps):
            with torch.cuda.stream(self.s):
                self.flush_sink.copy_(self.flush.sum(dtype=torch.int64))
            e[2 * r].record(self.s)
            self.call(w, c)
            e[2 * r + 1].record(self.s)
        e[-1].synchronize()
        return float(np.median([e[2 * r].elapsed_time(e[2 * r + 1]) for r in range(reps)])) * 1e3  # us

    def sweep(self, w):
        self.prepare(w)
        cs = candidates(w)
        ts = [self.time(w, c) for c in cs]
        for key in ("keys", "offsets", "segout"):
            w.pop(key, None)
        self.gbk.stream_check(self.s)
        return cs, ts


def collect(workloads, bench, log_every=200):
    rows = []
    t0 = time.time()
    for i, w in enumerate(workloads):
        cs, ts = bench.sweep(w)
        rows.append((dict(w), cs, ts))
        if log_every and (i + 1) % log_every == 0:
            print(f"  swept {i + 1}/{len(workloads)} workloads ({time.time() - t0:.0f} s)", flush=True)
    return rows


class MLP:
    """FP32 MLP D -> 64 -> 64 -> 1 trained and run by libgbk's CUDA kernels."""

    def __init__(self, D=NFEAT, seed=0):
        import torch

        from kokkos_gb300 import gbk
        self.torch, self.gbk, self.D = torch, gbk, D
        self.P = int(gbk.lib.gbk_mlp_param_count(D))
        rng = np.random.default_rng(seed)
        p = np.zeros(self.P, dtype=np.float32)
        H = 64
        o = 0
        p[o:o + D * H] = rng.normal(0, math.sqrt(2.0 / D), D * H)
        o += D * H + H
        p[o:o + H * H] = rng.normal(0, math.sqrt(2.0 / H), H * H)
        o += H * H + H
        p[o:o + H] = rng.normal(0, math.sqrt(1.0 / H), H)
        self.params = torch.from_numpy(p).cuda()
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grads = torch.zeros_like(self.params)
        self.t = 0
        self.mu, self.sd = 0.0, 1.0

    def _ptr(self, t):
        return ctypes.c_void_p(t.data_ptr())

    def forward(self, X):
        torch = self.torch
        B = X.shape[0]
        acts = torch.empty(B * 128, dtype=torch.float32, device="cuda")
        Y = torch.empty(B, dtype=torch.float32, device="cuda")
        self.gbk.check(self.gbk.lib.gbk_mlp_forward(self._ptr(X), B, self.D, self._ptr(self.params), self._ptr(acts),
                                                    self._ptr(Y), None), "mlp_forward")
        return Y, acts

    def train(self, X, T, epochs=300, batch=4096, lr=2e-3, seed=0):
        """X: [N, D] float32, T: [N] target log-times (standardised here)."""
        torch, lib = self.torch, self.gbk.lib
        self.mu, self.sd = float(T.mean()), float(T.std() + 1e-6)
        Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).cuda()
        Td = torch.from_numpy(((T - self.mu) / self.sd).astype(np.float32)).cuda()
        N = Xd.shape[0]
        rng = np.random.default_rng(seed)
        loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        hist = []
        for ep in range(epochs):
            perm = torch.from_numpy(rng.permutation(N)).cuda()
            el = 0.0
            nb = 0
            for s in range(0, N, batch):
                idx = perm[s:s + batch]
                xb, tb = Xd[idx].contiguous(), Td[idx].contiguous()
                B = xb.shape[0]
                Y, acts = self.forward(xb)
                dY = torch.empty(B, dtype=torch.float32, device="cuda")
                self.gbk.check(lib.gbk_mlp_mse(self._ptr(Y), self._ptr(tb), B, self._ptr(dY), self._ptr(loss), None))
                self.gbk.check(lib.gbk_mlp_backward(self._ptr(xb), B, self.D, self._ptr(self.params),
                                                    self._ptr(acts), self._ptr(dY), self._ptr(self.grads), None))
                self.t += 1
                self.gbk.check(lib.gbk_mlp_adam(self._ptr(self.params), self._ptr(self.grads), self._ptr(self.m),
                                                self._ptr(self.v), self.P, lr, 0.9, 0.999, 1e-8, self.t, None))
                if ep % 25 == 0 or ep == epochs - 1:
                    el += float(loss.item())
                    nb += 1
            if nb:
                hist.append((ep, el / nb))
        return hist

    def predict(self, X):
        Xd = self.torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).cuda()
        Y, _ = self.forward(Xd)
        return Y.cpu().numpy() * self.sd + self.mu


class Ensemble:
    """K MLPs from different initial weights, trained on the same samples;
    the prediction is their mean (less variance in the pick)."""

    def __init__(self, k=5, D=NFEAT):
        self.models = [MLP(D=D, seed=s) for s in range(k)]

    def train(self, X, T, epochs=300, **kw):
        hist = []
        for s, m in enumerate(self.models):
            h = m.train(X, T, epochs=epochs, seed=s, **kw)
            hist = h if not hist else [(a[0], a[1] + b[1]) for a, b in zip(hist, h)]
        return [(e, l / len(self.models)) for e, l in hist]

    def predict(self, X):
        return np.mean([m.predict(X) for m in self.models], axis=0)

    @property
    def params(self):
        import torch
        return torch.stack([m.params for m in self.models])


def default_cfg_index(w, cs):
    """The configuration the library uses without tuning."""
    k = w["kind"]
    for i, c in enumerate(cs):
        if k == KIND_REDUCE:
            size = {5: 8, 1: 8, 3: 8}.get(w["dtype"], 4) * w["n"]
            if w.get("op", 0) == 0 and w["dtype"] == 5 and w["n"] >= (1 << 23):
                if c["variant"] == 3 and (c["ipt"], c["cps"]) == (5, 0):
                    return i
                continue
            if (size >= (4 << 20) and c["variant"] == 2 and c["cps"] == 0) or \
                    (size < (4 << 20) and c["variant"] == 1 and (c["block"], c["ipt"], c["cps"]) == (256, 4, 8)):
                return i
        if k == KIND_SCAN and (c["ipt"], c["cps"]) == (9, 0):
            return i
        # segmented reduce: 7 vectors; segmented scans: 5 vectors with three stages
        if k == KIND_SEG and (c["ipt"], c["cps"]) == (7, 0):
            return i
        if k == KIND_SEGSCAN and (c["ipt"], c["cps"]) == (5, 0):
            return i
        if k == KIND_HIST:
            # 65536 bins: the drain-free 16-bit kernel in its multiply form; up to
            # 24576: 32-bit privatised bins, two CTAs per SM
            want = (0x100, 1) if w["nbins"] > 24576 else (0x01, 2)
            if (c["variant"], c["cps"]) == want:
                return i
    return 0


def _ceil_log2(v):
    v = max(int(v), 1)
    return (v - 1).bit_length()


def lookup_key(w):
    """(kind, op, dtype, n, extra): the key under which the entry point for
    this workload looks its configuration up in the tuning table."""
    k = w["kind"]
    if k == KIND_REDUCE:
        return 0, w["op"], w["dtype"], w["n"], 0
    if k == KIND_SCAN:
        return 1, w["op"], 0 * 8 + 1, w["n"], 0
    if k == KIND_HIST:
        return 2, 0, 0, w["n"], _ceil_log2(w["nbins"]) * 8
    extra = _ceil_log2(w["n"] // max(w["nseg"], 1))
    if k == KIND_SEG:
        return 3, 0, 4, w["n"], extra
    return 3, 16 + w["op"], 0 * 8 + 1, w["n"], extra


def table_pick(w, cs):
    """Index of the candidate the loaded tuning table gives this workload (the
    nearest log2 n of its bucket, as the entry points do), or the default's
    when the table has no entry for it.  This is the method without the MLP."""
    from kokkos_gb300 import gbk
    t = gbk.Tuning()
    if gbk.lib.gbk_tuner_lookup(*lookup_key(w), ctypes.byref(t)) == 0:
        for i, c in enumerate(cs):
            if (c["block"], c["ipt"], c["cps"], c["variant"]) == (t.block, t.items_per_thread, t.ctas_per_sm,
                                                                  t.variant):
                return i
    return default_cfg_index(w, cs)


def dataset(rows):
    """Training set: one sample per (workload, candidate).  The target is the
    candidate's log time minus the mean log time of its workload's
    candidates: only the order within a workload matters for the pick, and
    the centred target leaves the model's capacity to that order."""
    X, T, grp = [], [], []
    for gi, (w, cs, ts) in enumerate(rows):
        lt = [math.log(t) for t in ts if math.isfinite(t) and t > 0]
        if not lt:
            continue
        mu = float(np.mean(lt))
        for c, t in zip(cs, ts):
            if math.isfinite(t) and t > 0:
                X.append(features(w, c))
                T.append(math.log(t) - mu)
                grp.append(gi)
    return np.array(X, dtype=np.float32), np.array(T, dtype=np.float64), np.array(grp)


def evaluate(model, rows, table=False):
    """Throughput of the MLP's predicted-best, of the untuned default and (with
    table=True, for the tuning table loaded in the library) of the table's
    configuration, each relative to the exhaustive best, per held-out workload."""
    ratios = {"mlp": [], "default": [], "table": []}
    per_kind = {}
    for (w, cs, ts) in rows:
        ts = np.array(ts)
        ok = np.isfinite(ts)
        if not ok.any():
            continue
        best = ts[ok].min()
        X = np.stack([features(w, c) for c in cs])
        p = model.predict(X)
        p[~ok] = np.inf
        r = {"mlp": best / ts[int(np.argmin(p))], "default": best / ts[default_cfg_index(w, cs)]}
        if table:
            r["table"] = best / ts[table_pick(w, cs)]
        for key, v in r.items():
            ratios[key].append(float(v))
        per_kind.setdefault(w["kind"], []).append(r)
    rep = {"workloads": len(ratios["mlp"])}
    for key, v in ratios.items():
        if not v:
            continue
        a = np.array(v)
        rep[f"{key}_mean_throughput_vs_best"] = float(a.mean())
        rep[f"{key}_geomean_throughput_vs_best"] = float(np.exp(np.log(a).mean()))
        rep[f"{key}_frac_within_5pct"] = float((a >= 0.95).mean())
    rep["per_kind"] = {str(k): dict({"n": len(v)}, **{key: float(np.mean([r[key] for r in v])) for key in v[0]},
                                    **{key + "_within_5pct": float(np.mean([r[key] >= 0.95 for r in v]))
                                       for key in v[0]})
                       for k, v in per_kind.items()}
    return rep


def grid_workloads():
    """The workload buckets of the tuning table (kind, op, dtype, log2 n, extra)."""
    out = []
    for l2 in range(16, 29):
        for op, dt in REDUCE_OPS:
            if dt in (1, 5) and l2 > 27:
                continue
            out.append({"kind": KIND_REDUCE, "op": OPC[op], "opname": op, "dtype": dt, "n": 1 << l2,
                        "inner_extent": 1})
        for inc in (0, 1):
            out.append({"kind": KIND_SCAN, "op": inc, "dtype": 0, "n": 1 << l2})
        if l2 <= 26:
            for nb in (256, 4096, 65536):
                out.append({"kind": KIND_HIST, "op": 0, "dtype": 0, "n": 1 << l2, "nbins": nb, "pool": 3})
    # batched segments: total size x mean segment length (lognormal sigma 1.5)
    for l2 in (20, 22, 24, 26):
        for l2m in (6, 8, 10, 12):
            base = {"kind": KIND_SEG, "op": 0, "dtype": 4, "n": 1 << l2, "nseg": 1 << (l2 - l2m),
                    "seg_log2mean": float(l2m), "seg_sigma": 1.5, "seed": 7}
            out.append(dict(base))
            for inc in (0, 1):
                out.append(dict(base, kind=KIND_SEGSCAN, op=inc, dtype=0))
    return out


def table_line(w, c):
    k, op, dt, n, extra = lookup_key(w)
    l2 = int(round(math.log2(max(n, 1))))
    return f"{k} {op} {dt} {l2} {extra} {c['block']} {c['ipt']} {c['cps']} {c['variant']}"


HEADER = "# kind op dtype log2n extra block items_per_thread ctas_per_sm variant"


def table_exhaustive(grid_rows, path):
    """Tuning table from the exhaustive autotuner: the fastest measured
    candidate of every bucket."""
    lines = [HEADER]
    for (w, cs, ts) in grid_rows:
        ts = np.array(ts)
        if np.isfinite(ts).any():
            lines.append(table_line(w, cs[int(np.nanargmin(np.where(np.isfinite(ts), ts, np.nan)))]))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def table_from_model(model, grid_rows, path):
    """Tuning table from the MLP's choices on the same buckets, and the
    throughput of those choices relative to the bucket's exhaustive best."""
    lines = [HEADER]
    ratios = []
    for (w, cs, ts) in grid_rows:
        ts = np.array(ts)
        p = model.predict(np.stack([features(w, c) for c in cs]))
        i = int(np.argmin(p))
        lines.append(table_line(w, cs[i]))
        if np.isfinite(ts).any() and np.isfinite(ts[i]):
            ratios.append(float(ts[np.isfinite(ts)].min() / ts[i]))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return float(np.mean(ratios)) if ratios else float("nan")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-workloads", type=int, default=1350)  # about 20,000 timings
    ap.add_argument("--eval-workloads", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--out", default="tuner_out")
    ap.add_argument("--max-n", type=int, default=1 << 28)
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    bench = Bench(args.max_n)
    t0 = time.time()
    train_w = sample_workloads(args.train_workloads, seed=1)
    eval_w = sample_workloads(args.eval_workloads, seed=2)
    train_rows = collect(train_w, bench)
    eval_rows = collect(eval_w, bench)
    t_collect = time.time() - t0
    X, T, _ = dataset(train_rows)
    model = Ensemble(k=5)
    t1 = time.time()
    hist = model.train(X, T, epochs=args.epochs)
    t_train = time.time() - t1
    grid_rows = collect(grid_workloads(), bench, log_every=0)
    table = table_exhaustive(grid_rows, os.path.join(args.out, "tuning_table.txt"))
    from kokkos_gb300 import gbk
    gbk.check(gbk.lib.gbk_tuner_load(table.encode()), "tuner_load")
    try:
        rep = evaluate(model, eval_rows, table=True)
    finally:
        gbk.lib.gbk_tuner_clear()
    rep.update({"train_timings": int(X.shape[0]), "eval_timings": int(sum(len(r[2]) for r in eval_rows)),
                "collect_s": round(t_collect, 1), "train_s": round(t_train, 1), "loss_history": hist[::4] + hist[-1:]})
    rep["grid_buckets"] = len(grid_rows)
    rep["mlp_grid_throughput_vs_best"] = table_from_model(model, grid_rows, os.path.join(args.out, "mlp_table.txt"))
    np.save(os.path.join(args.out, "mlp_params.npy"), model.params.cpu().numpy())
    with open(os.path.join(args.out, "tuner_eval.json"), "w") as f:
        json.dump(rep, f, indent=1)
    # every timing, for re-analysis without the GPU
    with open(os.path.join(args.out, "timings.json"), "w") as f:
        json.dump({name: [[w, cs, [t if math.isfinite(t) else None for t in ts]] for (w, cs, ts) in rows]
                   for name, rows in (("train", train_rows), ("eval", eval_rows), ("grid", grid_rows))}, f)
    print(json.dumps({k: v for k, v in rep.items() if k != "loss_history"}, indent=1))


if __name__ == "__main__":
    main()
