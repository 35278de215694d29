"""ORACLE — test infrastructure only.

ctypes binding of ``liboracle.so`` (``oracle.cpp``), the CPU restatement of
the reference Kokkos OpenMP reduce / scan / ScatterView / sort algorithms.
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker or the timed
CPU baseline; the product path never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

DT = {np.dtype(np.int32): 0, np.dtype(np.int64): 1, np.dtype(np.uint32): 2,
      np.dtype(np.uint64): 3, np.dtype(np.float32): 4, np.dtype(np.float64): 5}
OPS = {"sum": 0, "prod": 1, "min": 2, "max": 3, "land": 4, "lor": 5, "band": 6, "bor": 7,
       "minloc": 8, "maxloc": 9, "minmax": 10, "minmaxloc": 11}


def build():
    """Compile liboracle.so with the oracle's own Makefile (g++ + OpenMP)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        vp, i64, ci, dp = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        L.orc_reduce.argtypes = [ci, ci, vp, i64, ci, vp]
        L.orc_sum_compensated.argtypes = [ci, vp, i64, vp]
        L.orc_mdrange_reduce.argtypes = [ci, ci, vp, ci, vp, vp, vp, ci, vp]
        L.orc_mdrange_reduce_ex.argtypes = [ci, ci, vp, ci, vp, vp, vp, vp, ci, ci, ci, vp]
        L.orc_scan.argtypes = [ci, ci, ci, vp, i64, vp, vp, ci]
        L.orc_histogram_i32_i64.argtypes = [vp, i64, vp, i64, ci, vp]
        L.orc_sort_u64.argtypes = [vp, i64]
        L.orc_sort_by_key_stable_u64_i32.argtypes = [vp, vp, i64]
        L.orc_sort_by_key_reference_u64_i32.argtypes = [vp, vp, i64, ci]
        L.orc_binsort_u64.argtypes = [vp, i64, i64, dp, dp, vp, vp, vp]
        L.orc_seg_sum_f32.argtypes = [vp, vp, i64, vp, vp, vp, ci]
        L.orc_seg_inclusive_scan_i32.argtypes = [vp, vp, i64, vp, ci]
        _LIB = L
    return _LIB


def _p(a):
    return ctypes.c_void_p(0 if a is None else a.ctypes.data)


def max_threads():
    return lib().orc_max_threads()


def result_dtype(op, dtype):
    """numpy structured dtype of a reducer's value_type (Kokkos layouts)."""
    t = np.dtype(dtype)
    if op in ("minloc", "maxloc"):
        return np.dtype({"names": ["val", "loc"], "formats": [t, np.int64], "offsets": [0, 8], "itemsize": 16})
    if op == "minmax":
        return np.dtype([("min_val", t), ("max_val", t)])
    if op == "minmaxloc":
        lo = (2 * t.itemsize + 7) // 8 * 8
        return np.dtype({"names": ["min_val", "max_val", "min_loc", "max_loc"],
                         "formats": [t, t, np.int64, np.int64],
                         "offsets": [0, t.itemsize, lo, lo + 8], "itemsize": lo + 16})
    return t


def reduce(op, x, nthreads):
    x = np.ascontiguousarray(x)
    out = np.zeros(1, dtype=result_dtype(op, x.dtype))
    rc = lib().orc_reduce(OPS[op], DT[x.dtype], _p(x), x.size, nthreads, _p(out))
    if rc:
        raise ValueError(f"oracle reduce {op} {x.dtype} unsupported")
    return out[0]


def sum_compensated(x):
    """(compensated FP64 sum, sum |x|, sum x^2)."""
    x = np.ascontiguousarray(x)
    out = np.zeros(3, dtype=np.float64)
    if lib().orc_sum_compensated(DT[x.dtype], _p(x), x.size, _p(out)):
        raise ValueError("sum_compensated needs float32/float64")
    return float(out[0]), float(out[1]), float(out[2])


def mdrange_reduce(op, base, lower, upper, strides, nthreads, tile=None, outer="right", inner="right"):
    """base: flat numpy array; lower/upper/strides in elements; loc = element offset.
    The reference's host tile walk: MDRangePolicy<Rank<N, outer, inner>>(lower, upper, tile),
    default tiles where tile is None or an entry is <= 0."""
    rank = len(lower)
    lo = np.asarray(lower, dtype=np.int64)
    up = np.asarray(upper, dtype=np.int64)
    st = np.asarray(strides, dtype=np.int64)
    tl = np.asarray(tile if tile is not None else [0] * rank, dtype=np.int64)
    out = np.zeros(1, dtype=result_dtype(op, base.dtype))
    rc = lib().orc_mdrange_reduce_ex(OPS[op], DT[base.dtype], _p(base), rank, _p(lo), _p(up), _p(st), _p(tl),
                                     int(outer == "left"), int(inner == "left"), nthreads, _p(out))
    if rc:
        raise ValueError("oracle mdrange_reduce failed")
    return out[0]


def scan(x, out_dtype, inclusive, init=0, nthreads=1):
    x = np.ascontiguousarray(x)
    y = np.empty(x.size, dtype=out_dtype)
    iv = np.array([init], dtype=out_dtype)
    rc = lib().orc_scan(int(inclusive), DT[x.dtype], DT[np.dtype(out_dtype)], _p(x), x.size, _p(iv), _p(y), nthreads)
    if rc:
        raise ValueError("oracle scan: unsupported dtype pair")
    return y


def histogram(keys, nbins, nthreads, bins=None):
    keys = np.ascontiguousarray(keys, dtype=np.int32)
    b = np.zeros(nbins, dtype=np.int64) if bins is None else bins
    dropped = np.zeros(1, dtype=np.int64)
    if lib().orc_histogram_i32_i64(_p(keys), keys.size, _p(b), nbins, nthreads, _p(dropped)):
        raise ValueError("oracle histogram failed")
    return b, int(dropped[0])


def sort_u64(keys):
    k = np.array(keys, dtype=np.uint64, copy=True)
    lib().orc_sort_u64(_p(k), k.size)
    return k


def sort_by_key_stable(keys, vals):
    k = np.array(keys, dtype=np.uint64, copy=True)
    v = np.array(vals, dtype=np.int32, copy=True)
    lib().orc_sort_by_key_stable_u64_i32(_p(k), _p(v), k.size)
    return k, v


def sort_by_key_reference(keys, vals, nthreads):
    k = np.array(keys, dtype=np.uint64, copy=True)
    v = np.array(vals, dtype=np.int32, copy=True)
    lib().orc_sort_by_key_reference_u64_i32(_p(k), _p(v), k.size, nthreads)
    return k, v


def binsort(keys, nbins_total, kmin, mul):
    k = np.ascontiguousarray(keys, dtype=np.uint64)
    counts = np.zeros(nbins_total, dtype=np.int32)
    offs = np.zeros(nbins_total, dtype=np.int64)
    perm = np.zeros(k.size, dtype=np.int64)
    if lib().orc_binsort_u64(_p(k), k.size, nbins_total, float(kmin), float(mul), _p(counts), _p(offs), _p(perm)):
        raise ValueError("oracle binsort failed")
    return counts, offs, perm


def seg_sum_f32(x, offsets, nthreads):
    nseg = offsets.size - 1
    out = np.zeros(nseg, dtype=np.float32)
    comp = np.zeros(nseg, dtype=np.float64)
    absum = np.zeros(nseg, dtype=np.float64)
    lib().orc_seg_sum_f32(_p(x), _p(offsets), nseg, _p(out), _p(comp), _p(absum), nthreads)
    return out, comp, absum


def seg_inclusive_scan_i32(x, offsets, nthreads):
    y = np.zeros(x.size, dtype=np.int32)
    lib().orc_seg_inclusive_scan_i32(_p(x), _p(offsets), offsets.size - 1, _p(y), nthreads)
    return y
