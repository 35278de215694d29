"""gbk_reduce_noalloc: the reduce for callers that may not allocate device
memory (code inside someone else's device-memory budget, or loops that must
not trigger cudaMalloc's implicit synchronisation).  Its scratch is a fixed
array inside the library instead of a cudaMalloc'd workspace.

Called through the C ABI, on two calls in a row (the array keeps the previous
call's contents, so the second call must not depend on them), and compared
both with the regular gbk_reduce on the same inputs and with the oracle (the
reference OpenMP reduce restated; the compensated FP64 sum for float and
double Sums).  Tolerances are those of the other reduce tests: exact for
integers and Min/Max/Loc, 1e-12 / 1e-5 relative for double / float Sum (the
two Sums may round differently: gbk_reduce can pick another kernel).  Cases
cover a view that does not start on a 16-byte boundary (the kernel's ragged
head), an empty view (the reducer's identity), and the bitwise and logical
reducers.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from tests._util import sum_ok

pytestmark = pytest.mark.gpu

SUM, LAND, BAND, BOR, MINLOC, MAXLOC, MINMAXLOC = 0, 4, 6, 7, 8, 9, 11
I32, I64, U64, F32, F64 = 0, 1, 3, 4, 5
NAMES = {0: "sum", 4: "land", 6: "band", 7: "bor", 8: "minloc", 9: "maxloc", 11: "minmaxloc"}


def _fn(gbk):
    f = gbk.lib.gbk_reduce_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_int32]
    f.restype = ctypes.c_int
    return f


def _cases(datagen, seed):
    """(op, dtype code, host array, offset): offset elements are dropped from
    the front of the device copy, so offset 1 starts the view off the
    16-byte boundary."""
    u64 = datagen.bits_u64(300001, seed=seed) & np.uint64(0xFFFF_FFFF_FFFF_FFF0)
    u64[7] |= np.uint64(1 << 2)
    band_src = datagen.uniform_i32(777777, 0, 255, seed=seed) | np.int32(0x7F00)
    return [
        (SUM, F64, datagen.uniform_f64((1 << 24) + 3, seed=seed), 0),
        (SUM, F64, datagen.uniform_f64((1 << 20) + 5, seed=seed), 1),
        (SUM, F32, datagen.normal_f32((1 << 22) + 1, seed=seed), 1),
        (MINLOC, F32, datagen.normal_f32(1 << 26, seed=seed), 0),
        (MAXLOC, F32, datagen.normal_f32(12345, seed=seed), 3),
        (MINMAXLOC, F64, datagen.normal_f64(1000003, seed=seed), 1),
        (SUM, I64, datagen.uniform_i64(999999, -10 ** 9, 10 ** 9, seed=seed), 1),
        (BAND, I32, band_src, 1),
        (BOR, U64, u64, 1),
        (LAND, I32, datagen.uniform_i32(5000, 1, 9, seed=seed), 2),
        (SUM, F32, np.zeros(0, dtype=np.float32), 0),
        (MINLOC, F64, np.zeros(0, dtype=np.float64), 0),
    ]


def test_noalloc_matches_workspace_reduce_and_oracle_two_calls():
    import torch

    import oracle
    from kokkos_gb300 import datagen, gbk
    torch.cuda.set_device(0)
    f = _fn(gbk)
    P = oracle.max_threads()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        for op, dt, xh, off in _cases(datagen, seed=10 + call):
            xd = torch.from_numpy(np.concatenate([np.zeros(off, xh.dtype), xh])).cuda()[off:]
            assert xd.numel() == xh.size
            a = torch.full((64,), 0xAB, dtype=torch.uint8, device="cuda")
            b = torch.full((64,), 0xCD, dtype=torch.uint8, device="cuda")
            st = f(op, dt, ctypes.c_void_p(xd.data_ptr()), xd.numel(), ctypes.c_void_p(a.data_ptr()), stream, 0)
            assert st == 0, gbk.lib.gbk_status_string(st)
            gbk.check(gbk.lib.gbk_reduce(op, dt, ctypes.c_void_p(xd.data_ptr()), xd.numel(),
                                         ctypes.c_void_p(b.data_ptr()), stream, None), "reduce")
            torch.cuda.synchronize()
            nb = gbk.result_nbytes(op, dt)
            ra = gbk.decode_result(a.cpu().numpy()[:nb], op, dt)
            rb = gbk.decode_result(b.cpu().numpy()[:nb], op, dt)
            want = oracle.reduce(NAMES[op], xh, P)
            ctx = (call, NAMES[op], dt, xh.size, off)
            if op == SUM and dt in (F32, F64):
                rel = 1e-12 if dt == F64 else 1e-5
                assert abs(float(ra) - float(rb)) <= rel * max(abs(float(rb)), 1e-30), (ctx, ra, rb)
                if xh.size:
                    ok, info = sum_ok(ra, xh, rel)
                    assert ok, (ctx, info)
                else:
                    assert float(ra) == 0.0 and float(want) == 0.0, ctx
            else:
                for nm in (rb.dtype.names or [None]):
                    va, vb = (ra[nm], rb[nm]) if nm else (ra, rb)
                    vw = want[nm] if nm else want
                    assert np.asarray(va).tobytes() == np.asarray(vb).tobytes(), (ctx, nm, va, vb)
                    assert np.asarray(va).tobytes() == np.asarray(vw).tobytes(), (ctx, nm, va, vw)
    gbk.stream_check()


def test_noalloc_rejects_more_ctas_than_its_scratch():
    import torch

    from kokkos_gb300 import gbk
    torch.cuda.set_device(0)
    f = _fn(gbk)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    x = torch.zeros(1 << 26, dtype=torch.float32, device="cuda")
    out = torch.zeros(64, dtype=torch.uint8, device="cuda")
    # 64 CTAs per SM on 152 SMs is far above the 4096 the fixed array holds.
    st = f(SUM, F32, ctypes.c_void_p(x.data_ptr()), x.numel(), ctypes.c_void_p(out.data_ptr()), stream, 64)
    assert st == 8, gbk.lib.gbk_status_string(st)
    assert b"gbk_reduce_noalloc" in gbk.lib.gbk_status_string(8)
    # The combined MinMaxLoc + Sum reducer does not fit its scratch records.
    st = f(12, F64, ctypes.c_void_p(x.data_ptr()), 1000, ctypes.c_void_p(out.data_ptr()), stream, 0)
    assert st == 2, gbk.lib.gbk_status_string(st)
    # A request that fits still works after the rejections.
    st = f(SUM, F32, ctypes.c_void_p(x.data_ptr()), x.numel(), ctypes.c_void_p(out.data_ptr()), stream, 2)
    assert st == 0
    torch.cuda.synchronize()
    assert gbk.decode_result(out.cpu().numpy()[:4], SUM, F32) == 0.0
