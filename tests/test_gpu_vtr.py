""".vtr scans feeding libvgpu nodes on the GPU (row groups read into
page-locked staging and copied to the device), against the CPU oracle over
the same table:

- the fixture written by the reference's own writer
  (tests/golden/ref_weather.vtr; one of its columns is a string column the
  plans do not read) under filter -> group_by on both group paths, with and
  without the predicate pushed into the scan as the reference optimizer
  pushes it (src/optimize.c:356-371): pruned row groups never change a
  result;
- a join whose probe side is a scan;
- a 2M-row table of the filter + group-by workload's shape in 100k-row
  groups, written by vectra_gb300.vtr (byte-identical to the reference's
  writer on the CPU tests);
- the pool of reader threads that reads row groups ahead into page-locked
  staging: every pool size (none, one, several, the default) gives the
  same batches in file order, with and without pruned row groups, and a
  scan freed while its readers still hold groups read ahead releases them.
"""
import ctypes as C
import os

import numpy as np
import pytest

import cases
from engines import OracleEngine

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURE = os.path.join(ROOT, "tests", "golden", "ref_weather.vtr")


class _ScanNode(C.Structure):
    """include/vectra_abi.h ScanNode (src/scan.h:10-17)."""
    from vectra_gb300 import abi as _abi
    _fields_ = [("base", _abi.VecNode), ("file", C.c_void_p), ("col_mask", C.POINTER(C.c_int)),
                ("next_rg", C.c_uint32), ("predicate", C.c_void_p), ("pred_borrowed", C.c_int)]


class _FilterNode(C.Structure):
    from vectra_gb300 import abi as _abi
    _fields_ = [("base", _abi.VecNode), ("child", C.c_void_p), ("predicate", C.c_void_p)]


def _pushdown(scan_ptr, filter_ptr):
    """What vec_optimize does to FilterNode -> ScanNode: the scan borrows
    the filter's predicate."""
    sn = C.cast(scan_ptr, C.POINTER(_ScanNode)).contents
    fn = C.cast(filter_ptr, C.POINTER(_FilterNode)).contents
    sn.predicate = fn.predicate
    sn.pred_borrowed = 1


def _host_table(t):
    return {k: v for k, v in t.items() if k != "city"}


def test_fixture_filter_group_vs_oracle():
    import vectra_gb300
    from vectra_gb300.plan import col, scan, tbl
    G, O = vectra_gb300.engine(0), OracleEngine()
    t = cases.vtr_weather_table()
    pred = lambda: (col("temperature") > 30.0) & (col("year") >= 2020.0)
    for td in (O.tmp, None):
        for push in (False, True):
            s = scan(G, FIXTURE)
            sp = s.node
            f = s.filter(pred())
            if push:
                _pushdown(sp, f.node)
            got = f.group_by("station").summarise(temp_dir=td, avg=("mean", "temperature"), n=("n",),
                                                  hi=("max", "year")).batches()
            want = (tbl(O, _host_table(t), batch_rows=600).filter(pred()).group_by("station")
                    .summarise(temp_dir=td, avg=("mean", "temperature"), n=("n",), hi=("max", "year")).batches())
            cases.same_batches(got, want, rtol=1e-12, tol_cols=("avg",))


def test_fixture_filter_node_vs_oracle():
    """A filter over the scan, pulled directly (selection vectors on host
    batches of the scan's row groups), with the predicate pushed down."""
    import vectra_gb300
    from vectra_gb300.plan import col, scan, tbl
    G, O = vectra_gb300.engine(0), OracleEngine()
    t = cases.vtr_weather_table()
    p = lambda: (col("temperature") > 28.0) | col("flag").eq(True)
    s = scan(G, FIXTURE, [0, 1, 3])
    sp = s.node
    f = s.filter(p())
    _pushdown(sp, f.node)
    got = f.collect()
    want = tbl(O, {k: t[k] for k in ("station", "temperature", "flag")}, batch_rows=600).filter(p()).collect()
    for k in want:
        assert np.array_equal(got[k][1], want[k][1]), k
        assert np.array_equal(got[k][0][got[k][1]], want[k][0][want[k][1]]), k


def test_scan_join_aggregate_vs_oracle(tmp_path):
    import vectra_gb300
    from vectra_gb300 import vtr
    from vectra_gb300.plan import col, scan, tbl
    G, O = vectra_gb300.engine(0), OracleEngine()
    rng = np.random.default_rng(9)
    n, d = 300_000, 20_000
    fact = {"key": rng.integers(1, d + 1, n).astype(np.int64),
            "value": (rng.lognormal(0, 1, n), rng.random(n) > 0.02)}
    dim = {"id": (rng.permutation(d) + 1).astype(np.int64), "category": rng.integers(0, 64, d).astype(np.int64),
           "weight": rng.random(d)}
    path = str(tmp_path / "fact.vtr")
    vtr.write_vtr(path, fact, 50_000)

    def q(left, E):
        return (left.left_join(tbl(E, dim, batch_rows=d), {"key": "id"}).group_by("category")
                .summarise(temp_dir=O.tmp, s=("sum", col("value") * col("weight"), True), n=("n",)).batches())
    cases.same_batches(q(scan(G, path), G), q(tbl(O, fact, batch_rows=50_000), O), rtol=1e-12, tol_cols=("s",))


def test_filter_group_2m_rows_from_vtr(tmp_path):
    import vectra_gb300
    from vectra_gb300 import vtr
    from vectra_gb300.plan import col, scan, tbl
    G, O = vectra_gb300.engine(0), OracleEngine()
    rng = np.random.default_rng(0)
    n = 2_000_000
    temp = rng.normal(20.0, 10.0, n)
    tv = rng.random(n) >= 0.01
    temp[~tv] = 0.0
    t = {"station": rng.integers(0, 1000, n), "temperature": (temp, tv), "year": rng.integers(2000, 2026, n)}
    path = str(tmp_path / "weather.vtr")
    assert vtr.write_vtr(path, t, 100_000) == 20

    def q(src, td):
        return (src.filter((col("temperature") > 30.0) & (col("year") >= 2020.0)).group_by("station")
                .summarise(temp_dir=td, avg=("mean", "temperature"), n=("n",)).batches())
    for td in (O.tmp, None):
        cases.same_batches(q(scan(G, path), td), q(tbl(O, t, batch_rows=100_000), td), rtol=1e-12,
                           tol_cols=("avg",))


def _with_threads(n, fn):
    """fn() with n reader threads (None: the default pool)."""
    prev = os.environ.get("VGPU_SCAN_THREADS")
    if n is None:
        os.environ.pop("VGPU_SCAN_THREADS", None)
    else:
        os.environ["VGPU_SCAN_THREADS"] = str(n)
    try:
        return fn()
    finally:
        if prev is None:
            os.environ.pop("VGPU_SCAN_THREADS", None)
        else:
            os.environ["VGPU_SCAN_THREADS"] = prev


def test_reader_pool_sizes_agree(tmp_path):
    import vectra_gb300
    from vectra_gb300 import vtr
    from vectra_gb300.plan import col, scan, tbl
    G, O = vectra_gb300.engine(0), OracleEngine()
    rng = np.random.default_rng(3)
    n = 1_300_017
    year = np.sort(rng.integers(2000, 2026, n))          # sorted: row groups prune on year
    x = rng.normal(0.0, 1.0, n)
    xv = rng.random(n) >= 0.03
    x[~xv] = 0.0
    t = {"k": rng.integers(0, 500, n), "x": (x, xv), "year": year}
    path = str(tmp_path / "t.vtr")
    vtr.write_vtr(path, t, 37_000)
    pred = lambda: col("year") >= 2019.0

    def q(push):
        s = scan(G, path)
        sp = s.node
        f = s.filter(pred())
        if push:
            _pushdown(sp, f.node)
        return f.group_by("k").summarise(temp_dir=O.tmp, s=("sum", "x", True), n=("n",)).batches()

    want = tbl(O, t, batch_rows=37_000).filter(pred()).group_by("k").summarise(
        temp_dir=O.tmp, s=("sum", "x", True), n=("n",)).batches()
    first = None
    for threads in (0, 1, 3, None):
        for push in (False, True):
            got = _with_threads(threads, lambda: q(push))
            cases.same_batches(got, want, rtol=1e-12, tol_cols=("s",))
            if first is None:
                first = got
            cases.same_batches(got, first)                # bit for bit across pool sizes
    # the scan's own batches through a GPU projection: file order, every pool size
    rows = lambda: scan(G, path, [0, 2]).mutate(y=col("year") + 1).collect()
    base = _with_threads(0, rows)
    for threads in (2, None):
        got = _with_threads(threads, rows)
        for k in base:
            assert np.array_equal(got[k][0], base[k][0]) and np.array_equal(got[k][1], base[k][1]), k


def test_scan_freed_with_groups_read_ahead(tmp_path):
    import vectra_gb300
    from vectra_gb300 import vtr
    from vectra_gb300.plan import col, scan
    G = vectra_gb300.engine(0)
    lib = G.lib
    lib.vgpu_device_bytes_in_use.restype = C.c_longlong
    rng = np.random.default_rng(5)
    n = 800_000
    t = {"a": rng.integers(0, 10, n), "b": rng.normal(0, 1, n)}
    path = str(tmp_path / "t.vtr")
    vtr.write_vtr(path, t, 10_000)
    lib.vgpu_synchronize()
    before = lib.vgpu_device_bytes_in_use()
    for threads in (1, 4):
        def one():
            f = scan(G, path).mutate(c=col("b") * 2.0)
            node = f._take()
            try:
                for _ in range(3):                          # a few batches, then stop
                    b = G.next_batch(node)
                    assert b
                    G.free_batch(b)
            finally:
                G.free_node(node)
        _with_threads(threads, one)
    lib.vgpu_synchronize()
    assert lib.vgpu_device_bytes_in_use() == before
