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


@pytest.mark.parametrize("threads,chunk,mult", [(256, 16384, 4), (1024, 262144, 2), (512, 1024, 2)])
def test_query_set_launch_parameters(threads, chunk, mult):
    """Every launch configuration the tuner tries gives the same results."""
    torch = pytest.importorskip("torch")
    from vectra_gb300 import workloads as W
    lib = _lib()
    lib.vgpu_queryset_prepare_with.restype = C.c_int
    lib.vgpu_queryset_prepare_with.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]
    dev = torch.device("cuda", 0)
    qs = W.gen_query_set(torch, 64, 8, dev, median_rows=5000, sigma=1.5, cap_rows=150_000, max_card=30_000)
    arr, outs, out_rows, keep = W.query_set_structs(torch, qs, dev)
    p = W.SetTuning(threads=threads, table_mult=mult, chunk_rows=chunk)
    plan = C.c_void_p()
    torch.cuda.synchronize()
    assert lib.vgpu_queryset_prepare_with(arr, len(arr), C.byref(p), C.byref(plan)) == 0, lib.vgpu_last_error()
    try:
        assert lib.vgpu_queryset_run(plan) == 0, lib.vgpu_last_error()
        W.check_query_set(torch, qs, outs, out_rows, range(len(arr)))
    finally:
        lib.vgpu_queryset_free(plan)


def test_query_set_autotune_records_per_shape():
    """vgpu_queryset_tune times every candidate on the set and records the
    fastest for the set's shape; prepare then uses it, and the results are
    the same."""
    torch = pytest.importorskip("torch")
    from vectra_gb300 import workloads as W
    lib = _lib()
    lib.vgpu_queryset_tune.restype = C.c_int
    lib.vgpu_queryset_tune.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    lib.vgpu_queryset_tuning.restype = C.c_int
    lib.vgpu_queryset_tuning.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    dev = torch.device("cuda", 0)
    qs = W.gen_query_set(torch, 48, 9, dev, median_rows=4000, sigma=1.2, cap_rows=100_000, max_card=10_000)
    arr, outs, out_rows, keep = W.query_set_structs(torch, qs, dev)
    torch.cuda.synchronize()
    t = W.SetTuning()
    assert lib.vgpu_queryset_tune(arr, len(arr), 1, C.byref(t)) == 0, lib.vgpu_last_error()
    assert t.candidates == 18 and t.ms > 0
    assert t.threads in (256, 512, 1024) and t.table_mult in (2, 4) and t.chunk_rows in (16384, 65536, 262144)
    r = W.SetTuning()
    assert lib.vgpu_queryset_tuning(arr, len(arr), C.byref(r)) == 1
    assert r.as_dict() == t.as_dict()
    plan = C.c_void_p()
    assert lib.vgpu_queryset_prepare(arr, len(arr), C.byref(plan)) == 0, lib.vgpu_last_error()
    try:
        out_rows.fill_(-1)
        torch.cuda.synchronize()
        assert lib.vgpu_queryset_run(plan) == 0, lib.vgpu_last_error()
        W.check_query_set(torch, qs, outs, out_rows, range(len(arr)))
    finally:
        lib.vgpu_queryset_free(plan)
