"""The Kokkos Tools tuning-tool callbacks exported by libgbk.so, driven the
way Kokkos drives a tool (core/src/impl/Kokkos_Profiling.cpp: declare the
input and output variables, then per tuned kernel begin_context ->
request_values -> kernel -> end_context), and the in-process tuning table.
Host code only: no kernel is launched."""
import ctypes
import os
import tempfile
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class ValueUnion(ctypes.Union):
    _fields_ = [("int_value", ctypes.c_int64), ("double_value", ctypes.c_double), ("string_value", ctypes.c_char * 64)]


class ValueUnionSet(ctypes.Union):
    _fields_ = [("int_value", ctypes.POINTER(ctypes.c_int64)), ("double_value", ctypes.POINTER(ctypes.c_double)),
                ("string_value", ctypes.c_void_p)]


class ValueSet(ctypes.Structure):
    _fields_ = [("size", ctypes.c_size_t), ("values", ValueUnionSet)]


class ValueRange(ctypes.Structure):
    _fields_ = [("lower", ValueUnion), ("upper", ValueUnion), ("step", ValueUnion), ("openLower", ctypes.c_bool),
                ("openUpper", ctypes.c_bool)]


class SetOrRange(ctypes.Union):
    _fields_ = [("set", ValueSet), ("range", ValueRange)]


class VariableInfo(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("category", ctypes.c_int), ("valueQuantity", ctypes.c_int),
                ("candidates", SetOrRange), ("toolProvidedInfo", ctypes.c_void_p)]


class VariableValue(ctypes.Structure):
    _fields_ = [("type_id", ctypes.c_size_t), ("value", ValueUnion), ("metadata", ctypes.POINTER(VariableInfo))]


INT64, STRING = 1, 2
SET, RANGE, UNBOUNDED = 0, 1, 2


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(os.path.join(ROOT, "kokkos_gb300", "libgbk.so")):
        import __graft_entry__
        __graft_entry__.build()
    from kokkos_gb300 import gbk
    L = gbk.lib
    L.kokkosp_declare_input_type.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(VariableInfo)]
    L.kokkosp_declare_output_type.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(VariableInfo)]
    L.kokkosp_request_values.argtypes = [ctypes.c_size_t, ctypes.c_size_t, ctypes.POINTER(VariableValue),
                                         ctypes.c_size_t, ctypes.POINTER(VariableValue)]
    L.kokkosp_begin_context.argtypes = [ctypes.c_size_t]
    L.kokkosp_end_context.argtypes = [ctypes.c_size_t, VariableValue]
    for f in ("kokkosp_declare_input_type", "kokkosp_declare_output_type", "kokkosp_request_values",
              "kokkosp_begin_context", "kokkosp_end_context"):
        getattr(L, f).restype = None
    return L


def int_set_info(vals):
    arr = (ctypes.c_int64 * len(vals))(*vals)
    info = VariableInfo()
    info.type, info.category, info.valueQuantity = INT64, 1, SET
    info.candidates.set.size = len(vals)
    info.candidates.set.values.int_value = ctypes.cast(arr, ctypes.POINTER(ctypes.c_int64))
    return info, arr


def unbounded_info():
    info = VariableInfo()
    info.type, info.category, info.valueQuantity = INT64, 1, UNBOUNDED
    return info


def ctx_values(ids_vals, infos):
    arr = (VariableValue * len(ids_vals))()
    for i, (tid, v) in enumerate(ids_vals):
        arr[i].type_id = tid
        arr[i].value.int_value = v
        arr[i].metadata = ctypes.pointer(infos[tid])
    return arr


def test_online_exhaustive_search_picks_fastest(lib):
    infos = {}
    for tid, nm in [(101, b"gbk.kind"), (102, b"gbk.op"), (103, b"gbk.dtype"), (104, b"gbk.log2n"), (105, b"gbk.extra")]:
        infos[tid] = unbounded_info()
        lib.kokkosp_declare_input_type(nm, tid, ctypes.byref(infos[tid]))
    bi, barr = int_set_info([128, 256, 512])
    ui, uarr = int_set_info([2, 4])
    lib.kokkosp_declare_output_type(b"gbk.block", 201, ctypes.byref(bi))
    lib.kokkosp_declare_output_type(b"gbk.items_per_thread", 202, ctypes.byref(ui))
    outinfo = {201: bi, 202: ui}
    ctx = ctx_values([(101, 0), (102, 8), (103, 4), (104, 20), (105, 7)], infos)
    lib.gbk_tuner_enable(0)
    seen = []
    for trial in range(6 + 3):
        tv = (VariableValue * 2)()
        for i, tid in enumerate((201, 202)):
            tv[i].type_id = tid
            tv[i].metadata = ctypes.pointer(outinfo[tid])
            tv[i].value.int_value = -1
        lib.kokkosp_begin_context(7)
        lib.kokkosp_request_values(7, 5, ctx, 2, tv)
        choice = (tv[0].value.int_value, tv[1].value.int_value)
        seen.append(choice)
        # the "kernel": (256, 4) is fast, everything else slow
        time.sleep(0.0005 if choice == (256, 4) else 0.004)
        lib.kokkosp_end_context(7, VariableValue())
    assert sorted(seen[:6]) == sorted([(b, u) for b in (128, 256, 512) for u in (2, 4)])  # each tried once
    assert seen[6:] == [(256, 4)] * 3


def test_table_answers_immediately(lib):
    from kokkos_gb300 import gbk
    infos = {}
    for tid, nm in [(111, b"gbk.kind"), (112, b"gbk.op"), (113, b"gbk.dtype"), (114, b"gbk.log2n"), (115, b"gbk.extra")]:
        infos[tid] = unbounded_info()
        lib.kokkosp_declare_input_type(nm, tid, ctypes.byref(infos[tid]))
    outs = {}
    keep = []
    for tid, nm, vals in [(211, b"gbk.block", [128, 256, 512]), (212, b"gbk.items_per_thread", [2, 4, 8]),
                          (213, b"gbk.ctas_per_sm", [1, 2, 4, 8]), (214, b"gbk.variant", [0, 1, 2, 32])]:
        info, arr = int_set_info(vals)
        keep.append(arr)
        outs[tid] = info
        lib.kokkosp_declare_output_type(nm, tid, ctypes.byref(info))
    lib.gbk_tuner_clear()
    assert lib.gbk_tuner_set(0, 8, 4, 20, 0, ctypes.byref(gbk.Tuning(512, 2, 4, 0))) == 0
    assert lib.gbk_tuner_set(2, 0, 0, 26, 128, ctypes.byref(gbk.Tuning(0, 0, 1, 32))) == 0
    lib.gbk_tuner_enable(1)
    try:
        for ctxv, want in [([(111, 0), (112, 8), (113, 4), (114, 21), (115, 0)], (512, 2, 4, 0)),   # nearest log2n
                           ([(111, 2), (112, 0), (113, 0), (114, 26), (115, 128)], (None, None, 1, 32))]:
            ctx = ctx_values(ctxv, infos)
            tv = (VariableValue * 4)()
            for i, tid in enumerate((211, 212, 213, 214)):
                tv[i].type_id = tid
                tv[i].metadata = ctypes.pointer(outs[tid])
                tv[i].value.int_value = -7
            lib.kokkosp_begin_context(9)
            lib.kokkosp_request_values(9, 5, ctx, 4, tv)
            lib.kokkosp_end_context(9, VariableValue())
            got = tuple(tv[i].value.int_value for i in range(4))
            for g, w in zip(got, want):
                if w is not None:
                    assert g == w, (got, want)
        # in-process lookup, save / load round trip
        t = gbk.Tuning()
        assert lib.gbk_tuner_lookup(0, 8, 4, 1 << 19, 0, ctypes.byref(t)) == 0 and (t.block, t.items_per_thread) == (512, 2)
        assert lib.gbk_tuner_lookup(1, 0, 1, 1 << 19, 0, ctypes.byref(t)) != 0
        with tempfile.TemporaryDirectory() as d:
            p = os.path.join(d, "table.txt").encode()
            assert lib.gbk_tuner_save(p) == 0
            lib.gbk_tuner_clear()
            assert lib.gbk_tuner_size() == 0
            assert lib.gbk_tuner_load(p) == 0
            assert lib.gbk_tuner_size() == 2
    finally:
        lib.gbk_tuner_enable(0)
        lib.gbk_tuner_clear()


def test_range_candidates(lib):
    info = VariableInfo()
    info.type, info.category, info.valueQuantity = INT64, 1, RANGE
    info.candidates.range.lower.int_value = 1
    info.candidates.range.upper.int_value = 4
    info.candidates.range.step.int_value = 1
    info.candidates.range.openLower = False
    info.candidates.range.openUpper = False
    lib.kokkosp_declare_output_type(b"gbk.ctas_per_sm", 301, ctypes.byref(info))
    ci = unbounded_info()
    lib.kokkosp_declare_input_type(b"kokkos.kernel_id", 302, ctypes.byref(ci))
    ctx = ctx_values([(302, 12345)], {302: ci})
    got = []
    for _ in range(4):
        tv = (VariableValue * 1)()
        tv[0].type_id = 301
        tv[0].metadata = ctypes.pointer(info)
        lib.kokkosp_begin_context(3)
        lib.kokkosp_request_values(3, 1, ctx, 1, tv)
        lib.kokkosp_end_context(3, VariableValue())
        got.append(tv[0].value.int_value)
    assert sorted(got) == [1, 2, 3, 4]


REF_RUNNER = os.path.join(ROOT, "oracle", "_ref", "ref_runner")


@pytest.mark.skipif(not os.path.exists(REF_RUNNER), reason="reference build (oracle/_ref) not present")
def test_reference_loads_libgbk_as_its_tuning_tool():
    """The reference's own tool loader (KOKKOS_TOOLS_LIBS,
    core/src/impl/Kokkos_Profiling.cpp:148-165,581-705) loads libgbk.so as
    its Kokkos Tools tool, with internal tuning on (KOKKOS_TUNE_INTERNALS):
    the reference declares its context and tile-size / team-size variables
    to the tool through the struct layouts of Kokkos_Profiling_C_Interface.h,
    asks for values once per kernel, and the kernels still give the reference
    outputs (an MDRange MinLoc run six times, a TeamPolicy(AUTO) scan over
    uneven segments).  The tool's report (GBK_TOOL_REPORT) shows what it was
    told and what it answered."""
    import subprocess

    import numpy as np
    G = np.load(os.path.join(ROOT, "tests", "golden", "golden.npz"))
    lib = os.path.join(ROOT, "kokkos_gb300", "libgbk.so")
    if not os.path.exists(lib):
        import __graft_entry__
        __graft_entry__.build()
    with tempfile.TemporaryDirectory() as td:
        env = dict(os.environ, OMP_PROC_BIND="false", KOKKOS_TOOLS_LIBS=lib, KOKKOS_TUNE_INTERNALS="1")
        # MDRange MinLoc, six times: six value requests for the tile sizes
        x = G["mdrange/f32/37x19x11/x"]
        x.tofile(os.path.join(td, "x.bin"))
        rep = os.path.join(td, "md.txt")
        subprocess.run([REF_RUNNER, "2", "mdrange", os.path.join(td, "x.bin"), os.path.join(td, "o.bin"), "8", "4",
                        "37", "19", "11", "6"], env=dict(env, GBK_TOOL_REPORT=rep), check=True, capture_output=True)
        got = np.fromfile(os.path.join(td, "o.bin"), dtype=np.uint8)
        assert got.tobytes() == G["mdrange/minloc/f32/37x19x11/4/out"].tobytes()
        lines = open(rep).read().splitlines()
        assert int(lines[0].split()[1]) > 0  # the reference's tools interface version
        inputs = [ln.split()[2] for ln in lines if ln.startswith("input ")]
        assert "kokkos.kernel_name" in inputs and "kokkos.kernel_type" in inputs
        outs = [ln for ln in lines if ln.startswith("output ")]
        assert len(outs) == 3 and all("_tile_size_" in ln for ln in outs)
        assert all(int(ln.split()[-1]) > 0 for ln in outs), outs  # candidates parsed from the reference's ranges
        req = [ln for ln in lines if ln.startswith("requests ")][0].split()
        assert int(req[1]) == 6 and int(req[3]) >= 6
        assert any(ln.startswith("best ") and "tried 6 of" in ln for ln in lines)
        # TeamPolicy(AUTO): the team-size tuner; the scan result does not depend on it
        offs, xs = G["teamscan/i32/50/offsets"], G["teamscan/i32/50/x"]
        np.concatenate([offs.view(np.uint8), xs.view(np.uint8)]).tofile(os.path.join(td, "t.bin"))
        rep2 = os.path.join(td, "team.txt")
        subprocess.run([REF_RUNNER, "2", "team_scan_i32", os.path.join(td, "t.bin"), os.path.join(td, "o2.bin"), "50"],
                       env=dict(env, GBK_TOOL_REPORT=rep2), check=True, capture_output=True)
        got2 = np.fromfile(os.path.join(td, "o2.bin"), dtype=np.uint8)
        assert got2.tobytes() == G["teamscan/i32/50/out"].tobytes()
        team = open(rep2).read()
        assert "requests 1 " in team, team
