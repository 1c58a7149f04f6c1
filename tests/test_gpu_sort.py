"""arrange() on the GPU (sort_node_create) against the CPU oracle's sort
node, which restates the reference's (src/sort.c; pinned against it in
tests/test_oracle_vs_ref.py and the golden fixtures): the restated R tests,
NA placement in both directions, ties kept in input order, signed zeros,
bool and extreme int64 keys, selection vectors below, ragged batch sizes, a
2M-row multi-key sort, and a sort over a .vtr scan.  Batches bit for bit."""
import numpy as np
import pytest

import cases
from engines import OracleEngine

pytestmark = pytest.mark.gpu

NA_F = None


def _gpu():
    import vectra_gb300
    return vectra_gb300.engine(0)


@pytest.mark.parametrize("case", cases.SORT_CASES, ids=lambda f: f.__name__)
def test_sort_case(case):
    cases.same_batches(case(_gpu()), case(OracleEngine()))


@pytest.mark.parametrize("n,batch", cases.RAGGED)
def test_random_sort(n, batch):
    cases.same_batches(cases.r_sort(_gpu(), n + 2, n, batch), cases.r_sort(OracleEngine(), n + 2, n, batch))


def test_sort_2m_rows():
    cases.same_batches(cases.r_sort(_gpu(), 7, 2_000_000, 300_000), cases.r_sort(OracleEngine(), 7, 2_000_000, 300_000))


def test_sort_over_scan(tmp_path):
    from vectra_gb300 import vtr
    from vectra_gb300.plan import col, scan, tbl
    rng = np.random.default_rng(3)
    n = 250_000
    t = {"k": (rng.integers(0, 1000, n), rng.random(n) > 0.02), "x": (rng.normal(0, 1, n), rng.random(n) > 0.02),
         "i": np.arange(n)}
    p = str(tmp_path / "t.vtr")
    vtr.write_vtr(p, t, 40_000)
    got = scan(_gpu(), p).filter(col("x") > 0.5).arrange(("k", True), "x").batches()
    want = tbl(OracleEngine(), t, batch_rows=40_000).filter(col("x") > 0.5).arrange(("k", True), "x").batches()
    cases.same_batches(got, want)


def test_string_columns_are_carried():
    """A child with a string column (here the oracle's own source node, as a
    reference scan would deliver it): the strings travel in the sort's order."""
    from vectra_gb300.plan import Tbl
    G, O = _gpu(), OracleEngine()
    t = cases.T(x=[2.0, 1.0, NA_F, 0.5])
    t["s"] = (["b", "a", "c", "d"], np.array([True, True, False, True]))
    cases.same_batches(Tbl(G, O.make_source(t)).arrange("x").batches(), Tbl(O, O.make_source(t)).arrange("x").batches())


def _spill(budget, fn):
    """fn() with the sort's run budget forced to `budget` rows; returns its
    result and the runs / key ranges the spilled sorts took."""
    import ctypes as C
    import os
    import vectra_gb300
    lib = vectra_gb300.load()
    lib.vgpu_sort_spill_stats.restype = C.c_long
    lib.vgpu_sort_spill_stats.argtypes = [C.POINTER(C.c_long)]
    r0 = C.c_long(0)
    runs0 = lib.vgpu_sort_spill_stats(C.byref(r0))
    os.environ["VGPU_SORT_RUN_ROWS"] = str(budget)
    try:
        out = fn()
    finally:
        del os.environ["VGPU_SORT_RUN_ROWS"]
    r1 = C.c_long(0)
    runs1 = lib.vgpu_sort_spill_stats(C.byref(r1))
    return out, runs1 - runs0, r1.value - r0.value


@pytest.mark.parametrize("n,batch,budget", [(200_000, 9_000, 20_000), (50_001, 1_000, 4_096), (7_000, 64, 1_000)])
def test_sort_beyond_the_device_budget(n, batch, budget):
    """Runs sorted into host memory and merged back by key range give the
    in-memory order exactly (multi-key, NA, descending, ties in input
    order)."""
    got, runs, ranges = _spill(budget, lambda: cases.r_sort(_gpu(), n + 2, n, batch))
    assert runs >= n // budget and ranges > 1
    cases.same_batches(got, cases.r_sort(OracleEngine(), n + 2, n, batch))


def test_sort_beyond_the_budget_skewed_keys():
    """One key repeated on most rows (a key range larger than the budget is
    copied in run order), plus strings and a selection vector below."""
    from vectra_gb300.plan import col, tbl
    rng = np.random.default_rng(21)
    n = 60_000
    k = np.where(rng.random(n) < 0.8, 7, rng.integers(0, 50, n))
    t = {"k": (k, rng.random(n) > 0.01), "s": (cases.random_strings(rng, n, 400, maxlen=10), rng.random(n) > 0.05),
         "i": np.arange(n), "x": rng.normal(0, 1, n)}

    from engines import gpu_engine
    G = gpu_engine()                 # strings come from a foreign source node

    def q(E):
        return tbl(E, t, batch_rows=2_500).filter(col("x") > -1.0).arrange("k", ("s", True)).batches()
    got, runs, ranges = _spill(3_000, lambda: q(G))
    assert runs > 5
    cases.same_batches(got, q(OracleEngine()))

    def q2(E):
        return tbl(E, t, batch_rows=2_500).arrange(("k", True)).batches()
    got2, _, _ = _spill(3_000, lambda: q2(G))
    cases.same_batches(got2, q2(OracleEngine()))
