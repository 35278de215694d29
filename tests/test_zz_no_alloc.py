"""gbk_reduce_noalloc: the reduce for callers that may not allocate device
memory (code inside someone else's device-memory budget, or loops that must
not trigger cudaMalloc's implicit synchronisation).  Its scratch is a fixed
array inside the library instead of a cudaMalloc'd workspace.

Called through the C ABI and compared with the regular gbk_reduce on the same
inputs, on two calls in a row (the array keeps the previous call's contents,
so the second call must not depend on them).  Tolerances are those of the
other reduce tests: exact for integers and Min/Max/Loc, 1e-12 / 1e-5
relative for double / float Sum.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SUM, MINLOC, MAXLOC, MINMAXLOC = 0, 8, 9, 11
I64, F32, F64 = 1, 4, 5


def _fn(gbk):
    f = gbk.lib.gbk_reduce_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_int32]
    f.restype = ctypes.c_int
    return f


def test_noalloc_matches_workspace_reduce_two_calls():
    import torch

    from kokkos_gb300 import datagen, gbk
    torch.cuda.set_device(0)
    f = _fn(gbk)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        seed = 10 + call
        cases = [
            (SUM, F64, torch.from_numpy(datagen.uniform_f64((1 << 24) + 3, seed=seed)).cuda()),
            (SUM, F32, torch.from_numpy(datagen.normal_f32((1 << 22) + 1, seed=seed)).cuda()),
            (MINLOC, F32, torch.from_numpy(datagen.normal_f32(1 << 26, seed=seed)).cuda()),
            (MAXLOC, F32, torch.from_numpy(datagen.normal_f32(12345, seed=seed)).cuda()),
            (MINMAXLOC, F64, torch.from_numpy(datagen.normal_f64(1000003, seed=seed)).cuda()),
            (SUM, I64, torch.from_numpy(datagen.uniform_i64(999999, -10 ** 9, 10 ** 9, seed=seed)).cuda()),
        ]
        for op, dt, x in cases:
            a = torch.full((64,), 0xAB, dtype=torch.uint8, device="cuda")
            b = torch.zeros(64, dtype=torch.uint8, device="cuda")
            st = f(op, dt, ctypes.c_void_p(x.data_ptr()), x.numel(), ctypes.c_void_p(a.data_ptr()), stream, 0)
            assert st == 0, gbk.lib.gbk_status_string(st)
            gbk.check(gbk.lib.gbk_reduce(op, dt, ctypes.c_void_p(x.data_ptr()), x.numel(),
                                         ctypes.c_void_p(b.data_ptr()), stream, None), "reduce")
            torch.cuda.synchronize()
            nb = gbk.result_nbytes(op, dt)
            ra = gbk.decode_result(a.cpu().numpy()[:nb], op, dt)
            rb = gbk.decode_result(b.cpu().numpy()[:nb], op, dt)
            if op == SUM and dt in (F32, F64):
                rel = 1e-12 if dt == F64 else 1e-5
                assert abs(float(ra) - float(rb)) <= rel * max(abs(float(rb)), 1e-30), (call, op, dt, ra, rb)
            else:
                for nm in (rb.dtype.names or [None]):
                    va = ra[nm] if nm else ra
                    vb = rb[nm] if nm else rb
                    assert np.asarray(va).tobytes() == np.asarray(vb).tobytes(), (call, op, dt, nm, va, vb)
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
    # A request that fits still works after the rejection.
    st = f(SUM, F32, ctypes.c_void_p(x.data_ptr()), x.numel(), ctypes.c_void_p(out.data_ptr()), stream, 2)
    assert st == 0
    torch.cuda.synchronize()
    assert gbk.decode_result(out.cpu().numpy()[:4], SUM, F32) == 0.0
