"""Seeded synthetic inputs for the reduce / scan / scatter / sort workloads.

Thin ctypes wrapper over ``libgbk_host.so`` (``csrc/gbk_datagen.c``): a
splitmix64-seeded xoshiro256** stream, generated in fixed 65,536-element
blocks so the bytes are independent of the host thread count.  Arrays are
written into caller-provided numpy buffers (which may be views of pinned
host tensors), so the same bytes feed the GPU path and the CPU oracle.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libgbk_host.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build() first")
        lib = ctypes.CDLL(path)
        i64, u64, i32, dbl, vp = ctypes.c_int64, ctypes.c_uint64, ctypes.c_int32, ctypes.c_double, ctypes.c_void_p
        for name, args in {
            "gbkd_uniform_f64": [vp, i64, u64],
            "gbkd_uniform_f32": [vp, i64, u64],
            "gbkd_normal_f32": [vp, i64, u64],
            "gbkd_normal_f64": [vp, i64, u64],
            "gbkd_uniform_i32": [vp, i64, i32, i32, u64],
            "gbkd_uniform_i64": [vp, i64, i64, i64, u64],
            "gbkd_bits_u64": [vp, i64, u64],
            "gbkd_bits_u32": [vp, i64, u64],
            "gbkd_zipf_i32": [vp, i64, i32, dbl, u64],
            "gbkd_lowentropy_u64": [vp, i64, ctypes.c_int, u64, vp],
            "gbkd_lognormal_lengths": [vp, i64, dbl, i64, i64, u64, ctypes.POINTER(dbl)],
            "gbkd_iota_i32": [vp, i64],
        }.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = ctypes.c_int if name in ("gbkd_zipf_i32", "gbkd_lowentropy_u64",
                                                 "gbkd_lognormal_lengths") else None
        _LIB = lib
    return _LIB


def _out(out, n, dtype):
    if out is None:
        return np.empty(n, dtype=dtype)
    assert out.dtype == np.dtype(dtype) and out.flags.c_contiguous and out.size == n
    return out


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def uniform_f64(n, seed=0, out=None):
    a = _out(out, n, np.float64)
    _lib().gbkd_uniform_f64(_p(a), n, seed)
    return a


def uniform_f32(n, seed=0, out=None):
    a = _out(out, n, np.float32)
    _lib().gbkd_uniform_f32(_p(a), n, seed)
    return a


def normal_f32(n, seed=0, out=None):
    a = _out(out, n, np.float32)
    _lib().gbkd_normal_f32(_p(a), n, seed)
    return a


def normal_f64(n, seed=0, out=None):
    a = _out(out, n, np.float64)
    _lib().gbkd_normal_f64(_p(a), n, seed)
    return a


def uniform_i32(n, lo, hi, seed=0, out=None):
    a = _out(out, n, np.int32)
    _lib().gbkd_uniform_i32(_p(a), n, lo, hi, seed)
    return a


def uniform_i64(n, lo, hi, seed=0, out=None):
    a = _out(out, n, np.int64)
    _lib().gbkd_uniform_i64(_p(a), n, lo, hi, seed)
    return a


def bits_u64(n, seed=0, out=None):
    a = _out(out, n, np.uint64)
    _lib().gbkd_bits_u64(_p(a), n, seed)
    return a


def bits_u32(n, seed=0, out=None):
    a = _out(out, n, np.uint32)
    _lib().gbkd_bits_u32(_p(a), n, seed)
    return a


def zipf_i32(n, nbins, s=1.1, seed=0, out=None):
    a = _out(out, n, np.int32)
    rc = _lib().gbkd_zipf_i32(_p(a), n, nbins, s, seed)
    if rc:
        raise ValueError(f"zipf_i32 failed ({rc})")
    return a


def lowentropy_u64(n, nbits=8, seed=0, out=None):
    """u64 keys sharing all but `nbits` seeded bit positions of a seeded base."""
    a = _out(out, n, np.uint64)
    pos = np.zeros(max(nbits, 1), dtype=np.int32)
    rc = _lib().gbkd_lowentropy_u64(_p(a), n, nbits, seed, _p(pos))
    if rc:
        raise ValueError(f"lowentropy_u64 failed ({rc})")
    return a, pos[:nbits].copy()


def lognormal_lengths(nseg, median=2048.0, max_len=1 << 21, target_total=1 << 28, seed=0):
    """Segment lengths ~ round(exp(ln(median) + sigma Z)) clipped to [1, max_len];
    sigma bisected so the total is close to `target_total`.  Returns (lengths, sigma)."""
    a = np.empty(nseg, dtype=np.int64)
    sig = ctypes.c_double(0.0)
    rc = _lib().gbkd_lognormal_lengths(_p(a), nseg, median, max_len, target_total, seed, ctypes.byref(sig))
    if rc:
        raise ValueError(f"lognormal_lengths failed ({rc})")
    return a, sig.value


def offsets_from_lengths(lengths):
    off = np.zeros(len(lengths) + 1, dtype=np.int64)
    np.cumsum(lengths, out=off[1:])
    return off


def iota_i32(n, out=None):
    a = _out(out, n, np.int32)
    _lib().gbkd_iota_i32(_p(a), n)
    return a
