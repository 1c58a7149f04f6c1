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
