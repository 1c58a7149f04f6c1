"""The benchmark workloads against the CPU oracle on the GPU, at their own
scale or on bounded samples of it (seeded numpy inputs, the same bytes for
both engines):

- filter + group-by, the whole workload: 10M rows in 100k-row batches;
- hash join + aggregate on a 1/20 sample (fact 5M x dim 500k), with and
  without na.rm: every group's n() exactly, NA poisoning exactly, and the
  na.rm sums bit for bit against the exactly rounded sum of the products;
- high-cardinality group-by on a 1/20 sample (10M rows over 2.5M keys, the
  partitioned path), also with 2% NA in x and an na.rm sum beside the plain
  one;
- a 256-instance sample of the batched query sets, every instance through the
  oracle's own plan (hash-path group-by, inner join with row ids);
- a 256-request sample of the served stream over 8 resident tables (1/200 of
  the workload's sizes), every request through the oracle's filter,
  group-by or semi / anti join plan.

Double sums: the oracle sums in row order as the reference does, so the GPU
(correctly rounded) is compared with it at 1e-12 relative (1e-12 of the sum
of magnitudes where values of both signs cancel) and bit for bit with an
exactly rounded sum (Shewchuk expansion, math.fsum).
"""
import math

import numpy as np
import pytest

import cases
from engines import OracleEngine, exact_sum, exact_sum_products

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _gpu():
    import vectra_gb300
    return vectra_gb300.engine(0)


def _exact_group_sums(groups, x, pick):
    """{g: exactly rounded sum of x over rows of group g} for g in pick."""
    order = np.argsort(groups, kind="stable")
    gs = groups[order]
    xs = x[order]
    lo = np.searchsorted(gs, pick, side="left")
    hi = np.searchsorted(gs, pick, side="right")
    return {g: exact_sum(xs[a:b]) for g, a, b in zip(pick, lo, hi)}


# --------------------------------------------------------------------------
# filter + group-by, full size
# --------------------------------------------------------------------------

def test_filter_group_full_size_vs_oracle():
    from vectra_gb300.plan import col, tbl
    n = 10_000_000
    rng = np.random.default_rng(0)
    station = rng.integers(0, 1000, n)
    temp = rng.normal(20.0, 10.0, n)
    tv = rng.random(n) >= 0.01
    temp[~tv] = 0.0
    year = rng.integers(2000, 2026, n)
    t = {"station": station, "temperature": (temp, tv), "year": year}

    def q(E, temp_dir):
        return (tbl(E, t, batch_rows=100_000).filter((col("temperature") > 30.0) & (col("year") >= 2020.0))
                .group_by("station").summarise(temp_dir=temp_dir, avg=("mean", "temperature"), n=("n",))
                .batches())

    G, O = _gpu(), OracleEngine()
    for td in (O.tmp, None):                              # R's sort path (key order), the hash path
        got, want = q(G, td), q(O, td)
        cases.same_batches(got, want, rtol=TOL, tol_cols=("avg",))
    # the means: the exactly rounded group sum / n, rounded once
    keep = tv & (temp > 30.0) & (year >= 2020)
    b = got[0] if len(got) == 1 else None
    out = {k: np.concatenate([bb[k][0] for bb in got]) for k in got[0]}
    ex = _exact_group_sums(station[keep], temp[keep], out["station"])
    for s, m, c in zip(out["station"], out["avg"], out["n"]):
        assert m == ex[s] / c, (s, m, ex[s] / c)
    assert b is None or len(out["station"]) == 1000


# --------------------------------------------------------------------------
# hash join + aggregate, 1/20 sample
# --------------------------------------------------------------------------

def _join_tables(n_fact, n_dim, seed, zipf_s=1.1):
    rng = np.random.default_rng(seed)
    ranks = np.arange(1, n_dim + 1, dtype=np.float64)
    cdf = np.cumsum(ranks ** -zipf_s)
    cdf /= cdf[-1]
    keys = np.minimum(np.searchsorted(cdf, rng.random(n_fact)), n_dim - 1) + 1
    vals = rng.lognormal(0, 1, n_fact)
    valid = rng.random(n_fact) >= 0.02
    vals[~valid] = 0.0
    fact = {"key": keys.astype(np.int64), "value": (vals, valid)}
    dim = {"id": (rng.permutation(n_dim) + 1).astype(np.int64),
           "category": rng.integers(0, 256, n_dim).astype(np.int64),
           "weight": rng.random(n_dim)}
    return fact, dim


def test_join_aggregate_sample_vs_oracle_and_exact():
    from vectra_gb300.plan import col, tbl
    fact, dim = _join_tables(5_000_000, 500_000, seed=0)

    def q(E, temp_dir):
        return (tbl(E, fact, batch_rows=1_000_000).left_join(tbl(E, dim, batch_rows=500_000), {"key": "id"})
                .group_by("category")
                .summarise(temp_dir=temp_dir, s=("sum", col("value") * col("weight")),
                           sr=("sum", col("value") * col("weight"), True), n=("n",))
                .batches())

    G, O = _gpu(), OracleEngine()
    got = q(G, O.tmp)
    cases.same_batches(got, q(O, O.tmp), rtol=TOL, tol_cols=("s", "sr"))
    out = got[0]
    # every group has NA values: s is NA everywhere, sr and n are exact
    assert not out["s"][1].any()
    pos = np.empty(500_001, np.int64)
    pos[dim["id"]] = np.arange(500_000)
    p = pos[fact["key"]]
    cat = dim["category"][p]
    vals, valid = fact["value"]
    for g, sr, n in zip(out["category"][0], out["sr"][0], out["n"][0]):
        rows = cat == g
        assert n == rows.sum()
        m = rows & valid
        assert sr == exact_sum_products(vals[m], dim["weight"][p[m]]), g


# --------------------------------------------------------------------------
# high-cardinality group-by, 1/20 sample (partitioned path)
# --------------------------------------------------------------------------

def test_high_card_sample_vs_oracle():
    from vectra_gb300.plan import tbl
    n, distinct = 10_000_000, 2_500_000
    rng = np.random.default_rng(0)
    raw = rng.integers(0, distinct, n).astype(np.uint64)
    key = (raw * np.uint64(0x9E3779B97F4A7C15)).astype(np.int64)
    kv = rng.random(n) >= 0.05
    key[~kv] = 0
    x = rng.lognormal(0, 2, n)
    y = rng.integers(-1_000_000, 1_000_001, n)
    xv = rng.random(n) >= 0.02
    x2 = np.where(xv, x, 0.0)

    def q(E, tab, extra):
        return (tbl(E, tab, batch_rows=n).group_by("key")
                .summarise(temp_dir=E.tmp if hasattr(E, "tmp") else "tmp", s=("sum", "x"), m=("mean", "x"),
                           lo=("min", "y"), hi=("max", "y"), n=("n",), **extra).batches())

    G, O = _gpu(), OracleEngine()
    runs0 = G.lib.vgpu_pagg_runs()
    for tab, extra in (({"key": (key, kv), "x": x, "y": y}, {}),
                       ({"key": (key, kv), "x": (x2, xv), "y": y}, {"sr": ("sum", "x", True)})):
        got = q(G, tab, extra)
        want = q(O, tab, extra)
        cases.same_batches(got, want, rtol=TOL, tol_cols=("s", "m", "sr"))
    assert G.lib.vgpu_pagg_runs() > runs0, "the partitioned aggregation did not run"
    # exactly rounded sums on a sample of groups (last run: na.rm sums)
    out = {k: np.concatenate([b[k][0] for b in got]) for k in got[0]}
    ok = {k: np.concatenate([b[k][1] for b in got]) for k in got[0]}
    idx = np.random.default_rng(1).choice(np.nonzero(ok["key"])[0], 2000, replace=False)
    pick = out["key"][idx]
    m = kv & xv
    ex = _exact_group_sums(key[m], x2[m], np.sort(pick))
    for i, k in zip(idx, pick):
        assert out["sr"][i] == ex[k], k


# --------------------------------------------------------------------------
# query sets: 256 instances, each through the oracle
# --------------------------------------------------------------------------

def test_query_set_sample_vs_oracle():
    torch = pytest.importorskip("torch")
    import ctypes as C
    from vectra_gb300 import workloads as W
    from vectra_gb300.plan import tbl
    lib = _gpu().lib
    lib.vgpu_queryset_prepare.restype = C.c_int
    lib.vgpu_queryset_prepare.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
    lib.vgpu_queryset_run.restype = C.c_int
    lib.vgpu_queryset_run.argtypes = [C.c_void_p]
    lib.vgpu_queryset_free.argtypes = [C.c_void_p]
    dev = torch.device("cuda", 0)
    qs = W.gen_query_set(torch, 256, 0, dev)            # the workload's distributions, 256 instances
    arr, outs, out_rows, keep = W.query_set_structs(torch, qs, dev)
    torch.cuda.synchronize()
    plan = C.c_void_p()
    assert lib.vgpu_queryset_prepare(arr, len(arr), C.byref(plan)) == 0, lib.vgpu_last_error()
    try:
        assert lib.vgpu_queryset_run(plan) == 0, lib.vgpu_last_error()
    finally:
        lib.vgpu_queryset_free(plan)
    O = OracleEngine()
    off = np.concatenate([[0], np.cumsum(qs["rows"])])
    boff = np.concatenate([[0], np.cumsum(qs["bcard"])])
    key, value, bkey = qs["key"].cpu().numpy(), qs["value"].cpu().numpy(), qs["bkey"].cpu().numpy()
    nrow = out_rows.cpu().numpy()
    for i in range(len(arr)):
        k = key[off[i]:off[i + 1]]
        o = outs[i]
        m = int(nrow[i])
        if qs["kind"][i] == W.SET_GROUP:
            v = value[off[i]:off[i + 1]]
            b = (tbl(O, {"key": k, "value": v}).group_by("key")
                 .summarise(temp_dir=None, s=("sum", "value"), mn=("mean", "value"), n=("n",)).collect())
            order = np.argsort(b["key"][0])
            wk, ws, wn = b["key"][0][order], b["s"][0][order], b["n"][0][order]
            gk, gs, gm, gn = (o["key"][:m].cpu().numpy(), o["sum"][:m].cpu().numpy(),
                              o["mean"][:m].cpu().numpy(), o["n"][:m].cpu().numpy())
            go = np.argsort(gk)
            gk, gs, gm, gn = gk[go], gs[go], gm[go], gn[go]
            assert np.array_equal(gk, wk), i
            assert np.array_equal(gn.astype(np.float64), wn), i
            # the oracle adds in row order: within 1e-12 of the group's sum of magnitudes
            inv = np.searchsorted(wk, k)
            mag = np.bincount(inv, weights=np.abs(v), minlength=len(wk))
            assert np.all(np.abs(gs - ws) <= TOL * mag), i
            # and the GPU sums are the exactly rounded ones (first groups)
            srt = np.argsort(inv, kind="stable")
            bounds = np.searchsorted(inv[srt], np.arange(min(len(wk), 16) + 1))
            for g in range(min(len(wk), 16)):
                ex = exact_sum(v[srt[bounds[g]:bounds[g + 1]]])
                assert gs[g] == ex, (i, g)
                assert gm[g] == ex / gn[g], (i, g)
        else:
            bk = bkey[boff[i]:boff[i + 1]]
            b = (tbl(O, {"key": k, "prow": np.arange(len(k), dtype=np.int64)})
                 .inner_join(tbl(O, {"key": bk, "brow": np.arange(len(bk), dtype=np.int64)}), "key").collect())
            assert m == len(b["prow"][0]), (i, m, len(b["prow"][0]))
            assert np.array_equal(o["probe"][:m].cpu().numpy(), b["prow"][0]), i
            assert np.array_equal(o["build"][:m].cpu().numpy(), b["brow"][0]), i


# --------------------------------------------------------------------------
# serving: 256 requests, each through the oracle
# --------------------------------------------------------------------------

def test_serve_sample_vs_oracle():
    torch = pytest.importorskip("torch")
    import vectra_gb300
    from vectra_gb300 import workloads as W
    from vectra_gb300.plan import col, tbl
    lib = W.bind_server(vectra_gb300.engine(0).lib)
    dev = torch.device("cuda", 0)
    sizes = [5_000, 10_000, 20_000, 40_000, 60_000, 100_000, 160_000, 250_000]   # 1/200 of the workload's
    tables = W.gen_serve_tables(torch, sizes, 0, dev, ids=50_000)
    torch.cuda.synchronize()
    reqs = W.gen_requests(256, len(tables), 0)
    srv = W.server_with_tables(lib, tables, n_streams=4)
    try:
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
        got = []
        for q, rid in zip(reqs, ids):
            got.append(W.fetch_result(lib, srv, rid, q.kind))
            lib.vgpu_server_release(srv, rid)
    finally:
        lib.vgpu_server_free(srv)
    host = [{k: t[k].cpu().numpy() for k in ("key", "kv", "val", "vv")} for t in tables]
    O = OracleEngine()
    for qi, (q, r) in enumerate(zip(reqs, got)):
        t = host[q.table]
        tab = {"key": (t["key"], t["kv"]), "val": (t["val"], t["vv"]),
               "rid": np.arange(len(t["key"]), dtype=np.int64)}
        if q.kind == W.SERVE_FILTER_SUM:
            b = (tbl(O, tab).filter(col("val") > q.threshold)
                 .summarise(temp_dir=None, n=("n",), s=("sum", "val")).collect())
            n = int(b["n"][0][0]) if len(b["n"][0]) else 0
            assert r[0] == n, qi
            if n:
                ws = b["s"][0][0]
                assert abs(r[1] - ws) <= TOL * abs(ws), qi
                assert r[1] == math.fsum(t["val"][t["vv"] & (t["val"] > q.threshold)]), qi
        elif q.kind == W.SERVE_GROUP_SUM:
            b = (tbl(O, tab).group_by("key")
                 .summarise(temp_dir=O.tmp, s=("sum", "val", True), n=("n",)).collect())
            keys, kval, sums, cnt = r
            wk, wkv = b["key"]
            assert np.array_equal(kval.astype(bool), wkv), qi
            assert np.array_equal(keys[wkv], wk[wkv]), qi
            assert np.array_equal(cnt.astype(np.float64), b["n"][0]), qi
            ws = b["s"][0]
            assert np.all(np.abs(sums - ws) <= TOL * np.abs(ws)), qi
            for j in range(min(len(ws), 20)):
                rows = (t["kv"] & (t["key"] == keys[j])) if kval[j] else ~t["kv"]
                assert sums[j] == math.fsum(t["val"][rows & t["vv"]]), (qi, j)
        else:
            bt = host[q.build_table]
            right = tbl(O, {"key": (bt["key"], bt["kv"])})
            left = tbl(O, tab)
            b = (left.semi_join(right, "key") if q.kind == W.SERVE_SEMI else left.anti_join(right, "key")).collect()
            assert np.array_equal(r.astype(np.int64), b["rid"][0]), qi
