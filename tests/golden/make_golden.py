"""Generate the golden vectors under tests/golden/ from the reference itself.

Builds the reference Kokkos OpenMP backend from its own sources
(``make -f oracle/ref.mk``, outputs in oracle/_ref/), then runs this
project's driver ``oracle/_ref/ref_runner`` on seeded inputs and stores
inputs + reference outputs in ``golden.npz``.  Run in a container that has
the reference sources:

    python tests/golden/make_golden.py [--ref /path/to/kokkos]

The fixtures are small (a few MB) and are committed; the tests never need
the reference at run time.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from kokkos_gb300 import datagen  # noqa: E402

DTYPES = {0: np.int32, 1: np.int64, 2: np.uint32, 3: np.uint64, 4: np.float32, 5: np.float64}
OPS = ["sum", "prod", "min", "max", "land", "lor", "band", "bor", "minloc", "maxloc", "minmax", "minmaxloc"]
SIZES = [0, 1, 31, 1000, 9001]
THREADS = [1, 4]


def runner():
    return os.path.join(ROOT, "oracle", "_ref", "ref_runner")


def run(nthreads, cmd, inp, *args, outsize_hint=None):
    with tempfile.TemporaryDirectory() as td:
        fi = os.path.join(td, "in.bin")
        fo = os.path.join(td, "out.bin")
        inp.tofile(fi)
        env = dict(os.environ, OMP_PROC_BIND="false")
        subprocess.run([runner(), str(nthreads), cmd, fi, fo] + [str(a) for a in args], check=True, env=env,
                       stdout=subprocess.DEVNULL)
        return np.fromfile(fo, dtype=np.uint8)


def reduce_input(op, dt, n, seed):
    t = np.dtype(DTYPES[dt])
    if op == "prod":
        if t.kind == "f":
            return (1.0 + 0.001 * datagen.normal_f64(n, seed)).astype(t)
        v = datagen.uniform_i32(n, 0, 63, seed)
        a = np.ones(n, dtype=t)
        a[v == 0] = 2
        if t.kind == "i":
            a[v == 1] = -1
        return a
    if op in ("land", "lor"):
        v = datagen.uniform_i32(n, 0, 999, seed)
        a = np.ones(n, dtype=t) if op == "land" else np.zeros(n, dtype=t)
        a[v == 0] = 0 if op == "land" else 3
        return a
    if t.kind == "f":
        return datagen.normal_f64(n, seed).astype(t) if t == np.float32 else datagen.normal_f64(n, seed)
    if op in ("band", "bor"):
        b = datagen.bits_u64(n, seed)
        if op == "band":
            b = b | np.uint64(0xF0F0F0F0F0F0F0F0) | (datagen.bits_u64(n, seed + 1) & datagen.bits_u64(n, seed + 2))
        else:
            b = b & datagen.bits_u64(n, seed + 1) & datagen.bits_u64(n, seed + 2) & np.uint64(0x0F0F0F0F0F0F0F0F)
        return b.astype(t) if t.itemsize == 8 else (b >> np.uint64(7)).astype(t)
    if t == np.int32:
        return datagen.uniform_i32(n, -1000000, 1000000, seed)
    if t == np.uint32:
        return datagen.uniform_i32(n, 0, 1 << 30, seed).astype(np.uint32)
    if t == np.int64:
        return datagen.uniform_i64(n, -(1 << 40), 1 << 40, seed)
    return datagen.uniform_i64(n, 0, 1 << 50, seed).astype(np.uint64)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("KOKKOS_REF_SRC", os.path.join(ROOT, os.pardir, "reference")))
    args = ap.parse_args()
    if not os.path.isdir(args.ref):
        sys.exit(f"reference sources not found at {args.ref}")
    subprocess.run(["make", "-s", "-f", "oracle/ref.mk", f"REF={args.ref}", "-j8"], cwd=ROOT, check=True)

    G = {}
    seed = 100
    # -- built-in reducers over RangePolicy ---------------------------------
    for dt, t in DTYPES.items():
        for op in OPS:
            if op in ("land", "lor", "band", "bor") and np.dtype(t).kind == "f":
                continue
            for n in SIZES:
                seed += 1
                x = reduce_input(op, dt, n, seed)
                key = f"reduce/{op}/{np.dtype(t).name}/{n}"
                G[key + "/x"] = x
                for P in THREADS:
                    G[f"{key}/{P}/out"] = run(P, "reduce", x, OPS.index(op), dt, n)
    # -- std reduce ---------------------------------------------------------
    x = datagen.uniform_f64(1 << 16, seed=0)
    G["stdreduce/f64/65536/4/x"] = x
    G["stdreduce/f64/65536/4/out"] = run(4, "stdreduce_f64", x, x.size)
    # -- scans --------------------------------------------------------------
    for n in [0, 1, 1000, 20011]:
        x = datagen.uniform_i32(n, 0, 15, seed=n + 7)
        xf = datagen.normal_f64(n, seed=n + 9)
        xl = datagen.uniform_i64(n, -50, 50, seed=n + 11)
        G[f"scan/i32/{n}/x"] = x
        G[f"scan/f64/{n}/x"] = xf
        G[f"scan/i64/{n}/x"] = xl
        for P in THREADS:
            for init in [0, 7]:
                G[f"exscan/i32_i64/{n}/{init}/{P}/out"] = run(P, "exscan_i32_i64", x, n, init)
            G[f"inscan/i32/{n}/{P}/out"] = run(P, "inscan", x, 0, n)
            G[f"inscan/f64/{n}/{P}/out"] = run(P, "inscan", xf, 5, n)
            G[f"scantotal/i64/{n}/{P}/out"] = run(P, "scan_total_i64", xl, n)
    # -- MDRange over LayoutLeft View<float***> -----------------------------
    for (n0, n1, n2) in [(37, 19, 11), (64, 32, 16)]:
        x = datagen.normal_f32(n0 * n1 * n2, seed=n0)
        G[f"mdrange/f32/{n0}x{n1}x{n2}/x"] = x
        for op in ["sum", "minloc", "maxloc"]:
            for P in THREADS:
                G[f"mdrange/{op}/f32/{n0}x{n1}x{n2}/{P}/out"] = run(P, "mdrange", x, OPS.index(op), 4, n0, n1, n2)
    # -- ScatterView histogram ---------------------------------------------
    for (n, nb) in [(100000, 4096), (5000, 65536), (0, 16)]:
        keys = datagen.zipf_i32(n, nb, 1.1, seed=nb)
        G[f"hist/{n}/{nb}/x"] = keys
        for P in THREADS:
            G[f"hist/{n}/{nb}/{P}/out"] = run(P, "hist", keys, n, nb)
    # -- sort / sort_by_key / BinSort ---------------------------------------
    for dist in ["uniform", "lowentropy"]:
        n = 12000
        keys = datagen.bits_u64(n, seed=5) if dist == "uniform" else datagen.lowentropy_u64(n, 8, seed=5)[0]
        G[f"sort/{dist}/{n}/x"] = keys
        G[f"sort/{dist}/{n}/out"] = run(4, "sort_u64", keys, n)
        G[f"sortstable/{dist}/{n}/out"] = run(4, "sort_pairs_stable", keys, n)
        G[f"sortbykey/{dist}/{n}/out"] = run(4, "sort_by_key", keys, n)
    keys = datagen.uniform_i64(20000, 0, 1000000, seed=3).astype(np.uint64)
    G["binsort/20000/1000/x"] = keys
    G["binsort/20000/1000/out"] = run(1, "binsort", keys, keys.size, 1000, int(keys.min()), int(keys.max()))
    # -- TeamPolicy league reduce over segments ----------------------------
    lens, _ = datagen.lognormal_lengths(50, median=64.0, max_len=4096, target_total=6000, seed=1)
    offs = datagen.offsets_from_lengths(lens)
    xv = datagen.normal_f64(int(offs[-1]), seed=2)
    G["teamreduce/f64/50/offsets"] = offs
    G["teamreduce/f64/50/x"] = xv
    G["teamreduce/f64/50/out"] = run(4, "team_reduce_sum_f64", np.concatenate([offs.view(np.uint8), xv.view(np.uint8)]), 50)

    # -- std algorithms beyond reduce/scan, nested team scan, UnorderedMap ---
    for n in (1, 1000, 65537):
        x = datagen.uniform_i64(n, -5000, 5000, seed=n + 21)
        G[f"algos/i64/{n}/x"] = x
        G[f"algos/i64/{n}/out"] = run(4, "algos_i64", x, n)
    G["teamscan/i32/50/offsets"] = offs
    xs = datagen.uniform_i32(int(offs[-1]), 0, 255, seed=4)
    G["teamscan/i32/50/x"] = xs
    G["teamscan/i32/50/out"] = run(4, "team_scan_i32", np.concatenate([offs.view(np.uint8), xs.view(np.uint8)]), 50)
    keys = datagen.zipf_i32(100000, 3000, 1.1, seed=6)
    G["umap/i32/100000/x"] = keys
    G["umap/i32/100000/4096/out"] = run(4, "umap_count", keys, keys.size, 4096)
    G["umap/i32/100000/1000/out"] = run(1, "umap_count", keys, keys.size, 1000)  # too small: failed inserts

    out = os.path.join(ROOT, "tests", "golden", "golden.npz")
    np.savez_compressed(out, **G)
    print(f"wrote {len(G)} arrays to {out} ({os.path.getsize(out) / 1e6:.2f} MB)")


if __name__ == "__main__":
    main()
