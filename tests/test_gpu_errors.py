"""Failures on the GPU path, made on the host or by a bounded wait that runs
out -- no GPU fault, trap or hang is involved:

- a device allocation that fails (fault injection, the n-th allocation of a
  join + aggregate query) surfaces as the call's error, and the query leaves
  no device memory behind once its nodes are freed: the failed call's own
  temporaries are released before the error is raised, as the reference's
  error contract asks (release device memory, then vectra_error,
  src/error.c:4-11);
- a bounded device wait that runs out (on a word nothing changes) comes back
  as an error status, and the device stays usable;
- the serving loop refuses a request whose estimate alone exceeds its
  budget, and withdraws requests still waiting for admission; the rest of
  the stream completes with the results it has without them.
"""
import ctypes as C

import numpy as np
import pytest

import cases
from engines import OracleEngine

pytestmark = pytest.mark.gpu


def _lib():
    import vectra_gb300
    lib = vectra_gb300.engine(0).lib
    lib.vgpu_device_bytes_in_use.restype = C.c_longlong
    lib.vgpu_debug_fail_alloc.argtypes = [C.c_long]
    lib.vgpu_wait_selftest.restype = C.c_int
    lib.vgpu_wait_selftest.argtypes = [C.c_longlong]
    return lib


def _join_agg(E, n=120_000, d=20_000, seed=4):
    from vectra_gb300.plan import col, tbl
    rng = np.random.default_rng(seed)
    fact = {"key": rng.integers(1, d + 1, n).astype(np.int64), "value": (rng.lognormal(0, 1, n), rng.random(n) > 0.02)}
    dim = {"id": (rng.permutation(d) + 1).astype(np.int64), "category": rng.integers(0, 64, d).astype(np.int64),
           "weight": rng.random(d)}
    return (tbl(E, fact, batch_rows=30_000).left_join(tbl(E, dim, batch_rows=7_000), {"key": "id"})
            .group_by("category").summarise(temp_dir="tmp", s=("sum", col("value") * col("weight"), True),
                                            n=("n",)).batches())


def test_failed_allocation_releases_the_calls_memory():
    import vectra_gb300
    from vectra_gb300.plan import EngineError
    lib = _lib()
    G, O = vectra_gb300.engine(0), OracleEngine()
    want = _join_agg(O)
    cases.same_batches(_join_agg(G), want, rtol=1e-12, tol_cols=("s",))   # warm: caches and kernels loaded
    lib.vgpu_synchronize()
    base = lib.vgpu_device_bytes_in_use()
    assert base >= 0
    failed = 0
    for n in range(1, 40):
        lib.vgpu_debug_fail_alloc(n)
        try:
            got = _join_agg(G)
        except EngineError as e:
            assert "device allocation" in str(e), str(e)
            failed += 1
        else:
            cases.same_batches(got, want, rtol=1e-12, tol_cols=("s",))   # n beyond the query's allocations
        finally:
            lib.vgpu_debug_fail_alloc(0)
        lib.vgpu_synchronize()
        assert lib.vgpu_device_bytes_in_use() == base, (n, lib.vgpu_device_bytes_in_use(), base)
    assert failed >= 5
    # and the library still answers
    cases.same_batches(_join_agg(G), want, rtol=1e-12, tol_cols=("s",))


def test_bounded_wait_runs_out_as_an_error():
    import vectra_gb300
    lib = _lib()
    assert lib.vgpu_wait_selftest(20_000) == -1
    assert b"bounded wait" in lib.vgpu_last_error()
    G, O = vectra_gb300.engine(0), OracleEngine()
    cases.same_batches(_join_agg(G, seed=6), _join_agg(O, seed=6), rtol=1e-12, tol_cols=("s",))


def _server(lib, W, torch, budget):
    dev = torch.device("cuda", 0)
    tables = W.gen_serve_tables(torch, [4000, 30_000, 65_000], 2, dev, ids=5000)
    torch.cuda.synchronize()
    return W.server_with_tables(lib, tables, n_streams=2, budget=budget), tables


def test_serve_refuses_requests_over_the_budget():
    torch = pytest.importorskip("torch")
    from vectra_gb300 import workloads as W
    lib = W.bind_server(_lib())
    lib.vgpu_server_cancel.restype = C.c_int
    lib.vgpu_server_cancel.argtypes = [C.c_void_p, C.c_int64]
    srv, tables = _server(lib, W, torch, budget=100_000)
    try:
        semi = W.ServeQuery(kind=W.SERVE_SEMI, table=2, build_table=1)
        assert lib.vgpu_server_submit(srv, semi) == -1
        assert b"budget" in lib.vgpu_last_error()
        filt = W.ServeQuery(kind=W.SERVE_FILTER_SUM, table=2, threshold=1.0)
        rid = lib.vgpu_server_submit(srv, filt)
        assert rid >= 0
        while lib.vgpu_server_poll(srv) > 0:
            pass
        r = W.fetch_result(lib, srv, rid, W.SERVE_FILTER_SUM)
        t = tables[2]
        m = (t["vv"] & (t["val"] > 1.0)).cpu().numpy()
        assert r[0] == int(m.sum())
        lib.vgpu_server_release(srv, rid)
    finally:
        lib.vgpu_server_free(srv)


def test_serve_cancels_queued_requests():
    torch = pytest.importorskip("torch")
    from vectra_gb300 import workloads as W
    lib = W.bind_server(_lib())
    lib.vgpu_server_cancel.restype = C.c_int
    lib.vgpu_server_cancel.argtypes = [C.c_void_p, C.c_int64]
    torch.cuda.synchronize()
    before = lib.vgpu_device_bytes_in_use()
    reqs = W.gen_requests(30, 3, 21)

    def run(cancel):
        srv, _ = _server(lib, W, torch, budget=1 << 30)
        try:
            ids = [lib.vgpu_server_submit(srv, q) for q in reqs]
            assert all(i >= 0 for i in ids)
            for k in cancel:                       # nothing polled yet: every request is still queued
                assert lib.vgpu_server_cancel(srv, ids[k]) == 0
                assert lib.vgpu_server_cancel(srv, ids[k]) == -1     # gone
            while True:
                p = lib.vgpu_server_poll(srv)
                assert p >= 0, lib.vgpu_last_error()
                if p == 0:
                    break
            out = {}
            for k, (q, rid) in enumerate(zip(reqs, ids)):
                if k in cancel:
                    assert not lib.vgpu_server_done(srv, rid)
                    continue
                assert lib.vgpu_server_cancel(srv, rid) == -1          # done: release it instead
                out[k] = W.fetch_result(lib, srv, rid, q.kind)
                lib.vgpu_server_release(srv, rid)
            return out
        finally:
            lib.vgpu_server_free(srv)
    full = run(set())
    part = run({1, 4, 5, 17, 29})
    assert set(part) == set(full) - {1, 4, 5, 17, 29}
    for k, r in part.items():
        a = full[k]
        if isinstance(r, tuple):
            for x, y in zip(r, a):
                assert np.array_equal(np.asarray(x), np.asarray(y)), k
        else:
            assert np.array_equal(r, a), k
    torch.cuda.synchronize()
    assert lib.vgpu_device_bytes_in_use() == before
