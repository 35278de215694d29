"""Small, fixed workloads for ncu captures of one kernel (measurement only).

    python -m kokkos_gb300.bench_capture hist --variants 0x100,0x200
        2^26 int32 keys into 2^16 int64 bins, Zipf(1.1) keys then uniform keys
        (seed 0), each histogram variant (gbk tuning variant bits) run twice;
        the bins are checked against numpy.
    python -m kokkos_gb300.bench_capture permute
        a seeded random permutation of 2^26 int32 values applied twice
        (gbk_permute), checked against the permutation itself.

Each run launches only the library's kernels under test (plus torch's own
fills), so an ncu launch filter such as -k regex:k_hist16 sees exactly them.
"""
import argparse
import sys

import numpy as np
import torch

from kokkos_gb300 import datagen, gbk


def hist(variants):
    n, nb = 1 << 26, 1 << 16
    bins = torch.zeros(nb, dtype=torch.int64, device="cuda")
    for dist in ("zipf", "uniform"):
        keys = datagen.zipf_i32(n, nb, 1.1, seed=0) if dist == "zipf" else datagen.uniform_i32(n, 0, nb - 1, seed=0)
        dk = torch.from_numpy(keys).cuda()
        want = np.bincount(keys, minlength=nb)
        for var in variants:
            bins.zero_()
            for _ in range(2):
                gbk.histogram(dk, bins, tune=(0, 0, 0, var))
            torch.cuda.synchronize()
            gbk.stream_check()
            assert np.array_equal(bins.cpu().numpy(), 2 * want), (dist, hex(var))


def permute():
    n = 1 << 26
    perm = torch.from_numpy(np.random.default_rng(0).permutation(n).astype(np.int64)).cuda()
    src = torch.arange(n, dtype=torch.int32, device="cuda")
    for _ in range(2):
        dst = gbk.permute(src, perm)
    torch.cuda.synchronize()
    gbk.stream_check()
    assert torch.equal(dst.long(), perm)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    sub = ap.add_subparsers(dest="what", required=True)
    h = sub.add_parser("hist")
    h.add_argument("--variants", default="0x100", help="comma-separated histogram tuning variants")
    sub.add_parser("permute")
    a = ap.parse_args(argv)
    torch.cuda.set_device(0)
    if a.what == "hist":
        hist([int(v, 0) for v in a.variants.split(",")])
    else:
        permute()
    print("ok")
    return 0


if __name__ == "__main__":
    sys.exit(main())
