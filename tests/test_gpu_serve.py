"""The serving loop (vgpu_server_*): every request of a mixed stream gives
the same result alone as in the mix (counts, keys, selections and the
exactly rounded sums bit for bit), and the results match torch / exact
sums."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup():
    torch = pytest.importorskip("torch")
    import vectra_gb300
    from vectra_gb300 import workloads as W
    lib = W.bind_server(vectra_gb300.engine(0).lib)
    dev = torch.device("cuda", 0)
    tables = W.gen_serve_tables(torch, [3000, 20_000, 65_000], 3, dev, ids=5000)
    torch.cuda.synchronize()
    return torch, lib, W, tables


def _run(lib, W, tables, reqs, n_streams, one_at_a_time):
    srv = W.server_with_tables(lib, tables, n_streams=n_streams)
    try:
        res = []
        if one_at_a_time:
            for q in reqs:
                rid = lib.vgpu_server_submit(srv, q)
                assert rid >= 0, lib.vgpu_last_error()
                while lib.vgpu_server_poll(srv) > 0:
                    pass
                res.append(W.fetch_result(lib, srv, rid, q.kind))
                lib.vgpu_server_release(srv, rid)
        else:
            ids = []
            for q in reqs:
                ids.append(lib.vgpu_server_submit(srv, q))
                assert ids[-1] >= 0, lib.vgpu_last_error()
                assert lib.vgpu_server_poll(srv) >= 0, lib.vgpu_last_error()
            while True:
                p = lib.vgpu_server_poll(srv)
                assert p >= 0, lib.vgpu_last_error()
                if p == 0:
                    break
            for q, rid in zip(reqs, ids):
                res.append(W.fetch_result(lib, srv, rid, q.kind))
                lib.vgpu_server_release(srv, rid)
        return res
    finally:
        lib.vgpu_server_free(srv)


def _same(a, b):
    if isinstance(a, tuple):
        assert len(a) == len(b)
        for x, y in zip(a, b):
            if isinstance(x, np.ndarray):
                assert np.array_equal(x, y)
            else:
                assert x == y or (x != x and y != y)
    else:
        assert np.array_equal(a, b)


def test_alone_equals_mixed():
    torch, lib, W, tables = _setup()
    reqs = W.gen_requests(60, len(tables), 11)
    mixed = _run(lib, W, tables, reqs, n_streams=3, one_at_a_time=False)
    alone = _run(lib, W, tables, reqs, n_streams=1, one_at_a_time=True)
    for q, a, b in zip(reqs, mixed, alone):
        _same(a, b)


def test_results_match_reference_semantics():
    torch, lib, W, tables = _setup()
    reqs = W.gen_requests(24, len(tables), 12)
    got = _run(lib, W, tables, reqs, n_streams=2, one_at_a_time=False)
    host = [{k: v.cpu().numpy() for k, v in t.items() if k in ("key", "kv", "val", "vv")} for t in tables]
    for q, r in zip(reqs, got):
        t = host[q.table]
        if q.kind == W.SERVE_FILTER_SUM:
            m = t["vv"] & (t["val"] > q.threshold)
            assert r[0] == int(m.sum())
            assert r[1] == math.fsum(t["val"][m])
        elif q.kind == W.SERVE_GROUP_SUM:
            keys, kval, sums, cnt = r
            kv = t["kv"]
            uk = np.unique(t["key"][kv])
            assert np.array_equal(keys[:len(uk)], uk) and kval[:len(uk)].all()
            assert (not kval[-1]) == (not kv.all())
            for j, k in enumerate(uk[:50]):
                rows = kv & (t["key"] == k)
                assert cnt[j] == rows.sum()
                assert sums[j] == math.fsum(t["val"][rows & t["vv"]])
        else:
            b = host[q.build_table]
            hit = t["kv"] & np.isin(t["key"], b["key"][b["kv"]])
            want = np.nonzero(hit if q.kind == W.SERVE_SEMI else ~hit)[0]
            assert np.array_equal(r, want.astype(np.int32))
