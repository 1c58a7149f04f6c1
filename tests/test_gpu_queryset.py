"""Query sets (vgpu_queryset_*): many small group-by and inner-join
instances prepared once into a CUDA graph, every instance checked against
torch, two runs of the same plan in a row, and the errors a plan reports."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib():
    import vectra_gb300
    lib = vectra_gb300.engine(0).lib
    lib.vgpu_queryset_prepare.restype = C.c_int
    lib.vgpu_queryset_prepare.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
    lib.vgpu_queryset_run.restype = C.c_int
    lib.vgpu_queryset_run.argtypes = [C.c_void_p]
    lib.vgpu_queryset_free.argtypes = [C.c_void_p]
    return lib


def test_query_set_matches_torch():
    torch = pytest.importorskip("torch")
    from vectra_gb300 import workloads as W
    lib = _lib()
    dev = torch.device("cuda", 0)
    qs = W.gen_query_set(torch, 96, 5, dev, median_rows=3000, sigma=1.5, cap_rows=200_000, max_card=20_000)
    arr, outs, out_rows, keep = W.query_set_structs(torch, qs, dev)
    torch.cuda.synchronize()
    plan = C.c_void_p()
    assert lib.vgpu_queryset_prepare(arr, len(arr), C.byref(plan)) == 0, lib.vgpu_last_error()
    try:
        for _ in range(2):                      # the same plan twice: tables are emptied each run
            out_rows.fill_(-1)
            torch.cuda.synchronize()
            assert lib.vgpu_queryset_run(plan) == 0, lib.vgpu_last_error()
            W.check_query_set(torch, qs, outs, out_rows, range(len(arr)))
    finally:
        lib.vgpu_queryset_free(plan)


def test_query_set_reports_repeated_build_keys():
    torch = pytest.importorskip("torch")
    from vectra_gb300 import workloads as W
    lib = _lib()
    dev = torch.device("cuda", 0)
    probe = torch.arange(100, dtype=torch.int64, device=dev)
    build = torch.tensor([3, 5, 3], dtype=torch.int64, device=dev)
    op = torch.empty(100, dtype=torch.int32, device=dev)
    ob = torch.empty(100, dtype=torch.int32, device=dev)
    rows = torch.zeros(1, dtype=torch.int64, device=dev)
    q = (W.SetQuery * 1)()
    q[0].kind = W.SET_JOIN
    q[0].n = 100
    q[0].key = probe.data_ptr()
    q[0].n_build = 3
    q[0].build_key = build.data_ptr()
    q[0].out_probe, q[0].out_build, q[0].out_rows = op.data_ptr(), ob.data_ptr(), rows.data_ptr()
    torch.cuda.synchronize()
    plan = C.c_void_p()
    assert lib.vgpu_queryset_prepare(q, 1, C.byref(plan)) == 0, lib.vgpu_last_error()
    try:
        assert lib.vgpu_queryset_run(plan) == -1
        assert b"repeat" in lib.vgpu_last_error()
    finally:
        lib.vgpu_queryset_free(plan)
