"""ctypes binding of libgbk.so, the C ABI declared in include/gbk.h.

Tensors are torch CUDA tensors (device memory and streams only: torch is
plumbing here).  Every call goes through the C ABI; there is no Python or
CPU fallback: a missing library raises at import, a non-zero status raises
GbkError.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "libgbk.so")
HEADER = os.path.join(ROOT, "include", "gbk.h")

if not os.path.exists(LIB_PATH):
    raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() (nvcc, sm_103a)")
lib = ctypes.CDLL(LIB_PATH)

DT = {"i32": 0, "i64": 1, "u32": 2, "u64": 3, "f32": 4, "f64": 5}
NP = {0: np.int32, 1: np.int64, 2: np.uint32, 3: np.uint64, 4: np.float32, 5: np.float64}
OPS = {"sum": 0, "prod": 1, "min": 2, "max": 3, "land": 4, "lor": 5, "band": 6, "bor": 7,
       "minloc": 8, "maxloc": 9, "minmax": 10, "minmaxloc": 11, "minmaxloc_sum": 12}
STATUS = {0: "ok", 1: "invalid argument", 2: "unsupported", 3: "CUDA error", 4: "device timeout",
          5: "out of workspace", 6: "key out of range", 7: "no device"}


class GbkError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = lib.gbk_status_string(status).decode()
        super().__init__(f"{what}: gbk status {status} ({msg})")


class Tuning(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int32), ("items_per_thread", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32), ("variant", ctypes.c_int32)]


vp, i64, ci = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
TP = ctypes.POINTER(Tuning)
_SIGS = {
    "gbk_version": ([], ci),
    "gbk_status_string": ([ci], ctypes.c_char_p),
    "gbk_device_info": ([vp, vp, vp, vp], ci),
    "gbk_stream_check": ([vp], ci),
    "gbk_fence_read": ([vp, vp, vp, i64], ci),
    "gbk_workspace_reserve": ([vp, i64], ci),
    "gbk_workspace_release_all": ([], ci),
    "gbk_set_wait_limit": ([i64], ci),
    "gbk_wait_limit": ([], i64),
    "gbk_launch_count": ([], i64),
    "gbk_deep_copy": ([vp, vp, i64, vp], ci),
    "gbk_memset": ([vp, ci, i64, vp], ci),
    "gbk_fill": ([vp, vp, ci, i64, vp], ci),
    "gbk_reduce": ([ci, ci, vp, i64, vp, vp, TP], ci),
    "gbk_reduce_host": ([ci, ci, vp, i64, vp, vp, TP], ci),
    "gbk_mdrange_reduce": ([ci, ci, vp, ci, vp, vp, vp, vp, vp, TP], ci),
    "gbk_mdrange_reduce_host": ([ci, ci, vp, i64, ci, vp, vp, vp, vp, vp, TP], ci),
    "gbk_scan": ([ci, ci, ci, vp, i64, vp, vp, vp, vp, TP], ci),
    "gbk_exclusive_scan_i32_i64": ([vp, i64, i64, vp, vp], ci),
    "gbk_inclusive_scan_i32": ([vp, i64, vp, vp], ci),
    "gbk_inclusive_scan_f64": ([vp, i64, vp, vp], ci),
    "gbk_exclusive_scan_i32_i64_host": ([vp, i64, i64, vp, vp], ci),
    "gbk_histogram_i32_i64": ([vp, i64, vp, i64, vp, TP], ci),
    "gbk_histogram_i32_i64_host": ([vp, i64, vp, i64, vp, TP], ci),
    "gbk_scatter": ([ci, ci, vp, vp, i64, vp, i64, vp], ci),
    "gbk_reduce_noalloc": ([ci, ci, vp, i64, vp, vp, ctypes.c_int32], ci),
    "gbk_sort": ([ci, vp, i64, vp], ci),
    "gbk_sort_by_key": ([ci, vp, ci, vp, i64, vp], ci),
    "gbk_sort_u64": ([vp, i64, vp], ci),
    "gbk_sort_by_key_u64_i32": ([vp, vp, i64, vp], ci),
    "gbk_binsort_u64": ([vp, i64, i64, ctypes.c_double, ctypes.c_double, ci, vp, vp, vp, vp], ci),
    "gbk_permute": ([ci, vp, vp, i64, vp, vp], ci),
    "gbk_segmented_reduce": ([ci, ci, vp, vp, i64, i64, vp, vp, TP], ci),
    "gbk_segmented_scan": ([ci, ci, ci, vp, vp, i64, i64, vp, vp, TP], ci),
    "gbk_tuner_clear": ([], ci),
    "gbk_tuner_set": ([ci, ci, ci, ci, ci, TP], ci),
    "gbk_tuner_lookup": ([ci, ci, ci, i64, ci, TP], ci),
    "gbk_tuner_load": ([ctypes.c_char_p], ci),
    "gbk_tuner_save": ([ctypes.c_char_p], ci),
    "gbk_tuner_enable": ([ci], ci),
    "gbk_tuner_size": ([], i64),
    "gbk_mlp_param_count": ([ci], i64),
    "gbk_mlp_forward": ([vp, i64, ci, vp, vp, vp, vp], ci),
    "gbk_mlp_backward": ([vp, i64, ci, vp, vp, vp, vp, vp], ci),
    "gbk_mlp_mse": ([vp, vp, i64, vp, vp, vp], ci),
    "gbk_mlp_adam": ([vp, vp, vp, vp, i64, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, ci, vp], ci),
    "gbk_graph_begin": ([vp], ci),
    "gbk_graph_end": ([vp, ctypes.POINTER(vp)], ci),
    "gbk_graph_launch": ([vp, vp], ci),
    "gbk_graph_destroy": ([vp], ci),
}


def _bind():
    for name, (args, res) in _SIGS.items():
        f = getattr(lib, name, None)
        if f is None:
            continue
        f.argtypes = args
        f.restype = res


_bind()


def declared_symbols():
    """Every function name include/gbk.h and include/gbk_tools.h declare
    (typed reduce macros expanded, Kokkos Tools callbacks included)."""
    src = open(HEADER).read()
    tools = open(os.path.join(ROOT, "include", "gbk_tools.h")).read()
    names = set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(gbk_\w+)\s*\(", src, re.M))
    names |= set(re.findall(r"^\s*(?:int|int64_t|void)\s+((?:gbk|kokkosp)_\w+)\s*\(", tools, re.M))
    ints = ["i32", "i64", "u32", "u64"]
    alls = ints + ["f32", "f64"]
    for m in re.finditer(r"^GBK_FOR_EACH_(INT_)?DTYPE\(GBK_DECLARE_TYPED_REDUCE,\s*(\w+)\)", src, re.M):
        for dt in (ints if m.group(1) else alls):
            names.add(f"gbk_reduce_{m.group(2)}_{dt}")
    return sorted(names)


def check(status, what=""):
    if status != 0:
        raise GbkError(status, what)


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _tune(t):
    if t is None:
        return None
    if isinstance(t, Tuning):
        return ctypes.byref(t)
    return ctypes.byref(Tuning(*t))


def dtype_code(t):
    import torch
    return {torch.int32: 0, torch.int64: 1, torch.uint32: 2, torch.uint64: 3,
            torch.float32: 4, torch.float64: 5}[t]


def result_nbytes(op, dt):
    e = 4 if dt in (0, 2, 4) else 8
    if op in (8, 9):
        return 16
    if op == 10:
        return 2 * e
    if op == 11:
        return (2 * e + 7) // 8 * 8 + 16
    if op == 12:
        return (2 * e + 7) // 8 * 8 + 24
    return e


def result_dtype(op, dt):
    t = np.dtype(NP[dt])
    if op in (8, 9):
        return np.dtype({"names": ["val", "loc"], "formats": [t, np.int64], "offsets": [0, 8], "itemsize": 16})
    if op == 10:
        return np.dtype([("min_val", t), ("max_val", t)])
    if op == 11:
        lo = (2 * t.itemsize + 7) // 8 * 8
        return np.dtype({"names": ["min_val", "max_val", "min_loc", "max_loc"],
                         "formats": [t, t, np.int64, np.int64],
                         "offsets": [0, t.itemsize, lo, lo + 8], "itemsize": lo + 16})
    if op == 12:
        lo = (2 * t.itemsize + 7) // 8 * 8
        return np.dtype({"names": ["min_val", "max_val", "min_loc", "max_loc", "sum"],
                         "formats": [t, t, np.int64, np.int64, t],
                         "offsets": [0, t.itemsize, lo, lo + 8, lo + 16], "itemsize": lo + 24})
    return t


def decode_result(raw_u8, op, dt):
    return np.frombuffer(np.asarray(raw_u8).tobytes(), dtype=result_dtype(op, dt))[0]


def reduce(op, x, out=None, stream=None, tune=None):
    """parallel_reduce of a contiguous CUDA tensor with a built-in reducer.
    Returns the raw uint8 device tensor holding the result (or fills `out`)."""
    import torch
    opc = OPS[op] if isinstance(op, str) else op
    dt = dtype_code(x.dtype)
    assert x.is_cuda and x.is_contiguous()
    if out is None:
        out = torch.empty(result_nbytes(opc, dt), dtype=torch.uint8, device=x.device)
    check(lib.gbk_reduce(opc, dt, ctypes.c_void_p(x.data_ptr()), x.numel(), ctypes.c_void_p(out.data_ptr()),
                         _stream(stream), _tune(tune)), f"reduce {op}")
    return out


def reduce_value(op, x, stream=None, tune=None):
    opc = OPS[op] if isinstance(op, str) else op
    raw = reduce(opc, x, stream=stream, tune=tune)
    stream_check(stream)
    return decode_result(raw.cpu().numpy(), opc, dtype_code(x.dtype))


def mdrange_reduce(op, base, lower, upper, strides, out=None, stream=None, tune=None):
    import torch
    opc = OPS[op] if isinstance(op, str) else op
    dt = dtype_code(base.dtype)
    rank = len(lower)
    lo = (ctypes.c_int64 * rank)(*lower)
    up = (ctypes.c_int64 * rank)(*upper)
    st = (ctypes.c_int64 * rank)(*strides)
    if out is None:
        out = torch.empty(result_nbytes(opc, dt), dtype=torch.uint8, device=base.device)
    check(lib.gbk_mdrange_reduce(opc, dt, ctypes.c_void_p(base.data_ptr()), rank, lo, up, st,
                                 ctypes.c_void_p(out.data_ptr()), _stream(stream), _tune(tune)), f"mdrange {op}")
    return out


def mdrange_reduce_host(op, host_base_np, lower, upper, strides, stream=None, tune=None):
    opc = OPS[op] if isinstance(op, str) else op
    dt = {np.dtype(v): k for k, v in NP.items()}[host_base_np.dtype]
    rank = len(lower)
    lo = (ctypes.c_int64 * rank)(*lower)
    up = (ctypes.c_int64 * rank)(*upper)
    st = (ctypes.c_int64 * rank)(*strides)
    res = np.zeros(result_nbytes(opc, dt), dtype=np.uint8)
    check(lib.gbk_mdrange_reduce_host(opc, dt, ctypes.c_void_p(host_base_np.ctypes.data), host_base_np.size, rank,
                                      lo, up, st, ctypes.c_void_p(res.ctypes.data), _stream(stream), _tune(tune)),
          f"mdrange_host {op}")
    return decode_result(res, opc, dt)


def scan(x, y, inclusive, init=None, total=None, stream=None, tune=None):
    din = dtype_code(x.dtype)
    dout = dtype_code(y.dtype)
    iv = None
    if init is not None:
        arr = np.array([init], dtype=NP[dout])
        iv = ctypes.c_void_p(arr.ctypes.data)
    check(lib.gbk_scan(1 if inclusive else 0, din, dout, ctypes.c_void_p(x.data_ptr()), x.numel(), iv,
                       ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(total.data_ptr()) if total is not None else None,
                       _stream(stream), _tune(tune)), "scan")
    return y


def histogram(keys, bins, stream=None, tune=None):
    check(lib.gbk_histogram_i32_i64(ctypes.c_void_p(keys.data_ptr()), keys.numel(), ctypes.c_void_p(bins.data_ptr()),
                                    bins.numel(), _stream(stream), _tune(tune)), "histogram")
    return bins


def scatter(op, idx, vals, dest, stream=None):
    opc = OPS[op] if isinstance(op, str) else op
    check(lib.gbk_scatter(opc, dtype_code(vals.dtype), ctypes.c_void_p(idx.data_ptr()),
                          ctypes.c_void_p(vals.data_ptr()), idx.numel(), ctypes.c_void_p(dest.data_ptr()),
                          dest.numel(), _stream(stream)), "scatter")
    return dest


def sort(keys, dt=None, stream=None):
    """Kokkos::sort of a contiguous CUDA tensor in place (dt overrides the
    element type code, e.g. for unsigned data held in a signed tensor)."""
    code = dt if dt is not None else dtype_code(keys.dtype)
    check(lib.gbk_sort(code, ctypes.c_void_p(keys.data_ptr()), keys.numel(), _stream(stream)), "sort")
    return keys


def sort_by_key(keys, vals, dt=None, stream=None):
    code = dt if dt is not None else dtype_code(keys.dtype)
    check(lib.gbk_sort_by_key(code, ctypes.c_void_p(keys.data_ptr()), vals.element_size(),
                              ctypes.c_void_p(vals.data_ptr()), keys.numel(), _stream(stream)), "sort_by_key")
    return keys, vals


def binsort(keys, nbins, kmin, mul, sort_within_bins=False, stream=None):
    """BinSort(BinOp1D) permutation of u64 keys (held in an int64 tensor).
    Returns (bin_count int32, bin_offsets int64, perm int64) CUDA tensors."""
    import torch
    counts = torch.empty(nbins, dtype=torch.int32, device=keys.device)
    offs = torch.empty(nbins, dtype=torch.int64, device=keys.device)
    perm = torch.empty(keys.numel(), dtype=torch.int64, device=keys.device)
    check(lib.gbk_binsort_u64(ctypes.c_void_p(keys.data_ptr()), keys.numel(), nbins, float(kmin), float(mul),
                              1 if sort_within_bins else 0, ctypes.c_void_p(counts.data_ptr()),
                              ctypes.c_void_p(offs.data_ptr()), ctypes.c_void_p(perm.data_ptr()), _stream(stream)),
          "binsort")
    return counts, offs, perm


def fill(dst, value, stream=None):
    """deep_copy(view, value) on a contiguous device tensor: the value is
    converted to the tensor's dtype on the host and its bytes replicated."""
    import torch
    v = np.ascontiguousarray(torch.tensor([value], dtype=dst.dtype).numpy())
    check(lib.gbk_fill(ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(v.ctypes.data), dst.element_size(), dst.numel(),
                       _stream(stream)), "fill")
    return dst


def permute(src, perm, stream=None):
    import torch
    dst = torch.empty_like(src)
    check(lib.gbk_permute(src.element_size(), ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(perm.data_ptr()),
                          src.numel(), ctypes.c_void_p(dst.data_ptr()), _stream(stream)), "permute")
    return dst


def segmented_reduce(op, x, offsets, out, stream=None, tune=None):
    """out[s] = op over x[offsets[s]:offsets[s+1]] for every segment, one launch."""
    opc = OPS[op] if isinstance(op, str) else op
    check(lib.gbk_segmented_reduce(opc, dtype_code(x.dtype), ctypes.c_void_p(x.data_ptr()),
                                   ctypes.c_void_p(offsets.data_ptr()), offsets.numel() - 1, x.numel(),
                                   ctypes.c_void_p(out.data_ptr()), _stream(stream), _tune(tune)), "segmented_reduce")
    return out


def segmented_scan(x, offsets, y, inclusive=True, stream=None, tune=None):
    check(lib.gbk_segmented_scan(1 if inclusive else 0, dtype_code(x.dtype), dtype_code(y.dtype),
                                 ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(offsets.data_ptr()),
                                 offsets.numel() - 1, x.numel(), ctypes.c_void_p(y.data_ptr()), _stream(stream),
                                 _tune(tune)),
          "segmented_scan")
    return y


class Graph:
    """Kokkos::Experimental::Graph over this library's calls: the calls made
    inside `with Graph(stream) as g:` on `stream` are captured; g.submit()
    replays them."""

    def __init__(self, stream):
        self.stream = stream
        self.h = ctypes.c_void_p()

    def __enter__(self):
        check(lib.gbk_graph_begin(ctypes.c_void_p(self.stream.cuda_stream)), "graph_begin")
        return self

    def __exit__(self, et, ev, tb):
        st = lib.gbk_graph_end(ctypes.c_void_p(self.stream.cuda_stream), ctypes.byref(self.h))
        if et is None:
            check(st, "graph_end")

    def submit(self):
        check(lib.gbk_graph_launch(self.h, ctypes.c_void_p(self.stream.cuda_stream)), "graph_launch")

    def __del__(self):
        try:
            if self.h:
                lib.gbk_graph_destroy(self.h)
        except Exception:
            pass


def stream_check(stream=None):
    st = lib.gbk_stream_check(_stream(stream))
    check(st, "stream_check")


def launch_count():
    return lib.gbk_launch_count()


def device_info():
    sm, ma, mi = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    l2 = ctypes.c_int64()
    check(lib.gbk_device_info(ctypes.byref(sm), ctypes.byref(ma), ctypes.byref(mi), ctypes.byref(l2)), "device_info")
    return {"sm_count": sm.value, "cc": (ma.value, mi.value), "l2_bytes": l2.value}
