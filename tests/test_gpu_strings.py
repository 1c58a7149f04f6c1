"""String columns on the GPU against the CPU oracle (whose string support
is pinned against the reference in tests/test_oracle_vs_ref.py):

- predicates and projections over strings -- comparisons (memcmp order,
  the shorter string first, bytes above 127 unsigned), nchar, substr with
  every kind of bound, grepl with a fixed pattern (src/expr.c:153-273,
  src/scalar_ops.c:78-107) -- on the restated R tests and on seeded random
  strings with NA, ragged batches and selection vectors;
- string group keys, alone and with an int64 key, in first-seen order and
  in key order (NA last), through the device dictionary: the restated
  group-by tests, a table whose keys outgrow the dictionary several times,
  500k rows over 60k distinct keys, and a .vtr scan.

Strings are fed as the reference's scan feeds them: host batches of a
foreign source node.  Results bit for bit, except double sums (1e-12)."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

FP_COLS = ("s", "m", "s1", "x")


@pytest.fixture(scope="module")
def G():
    from engines import gpu_engine
    return gpu_engine()


@pytest.mark.parametrize("case", cases.STRING_FILTER_CASES, ids=lambda f: f.__name__)
def test_string_filter_cases(case, G, oracle):
    cases.same_batches(case(G), case(oracle))


@pytest.mark.parametrize("temp_dir", ["tmp", None], ids=["sorted", "hash"])
@pytest.mark.parametrize("case", cases.STRING_GROUP_CASES, ids=lambda f: f.__name__)
def test_string_group_cases(case, temp_dir, G, oracle):
    td = None if temp_dir is None else oracle.tmp
    cases.same_batches(case(G, td), case(oracle, td), rtol=1e-12, tol_cols=FP_COLS)


@pytest.mark.parametrize("n,batch", [(0, 32), (33, 32), (700, 64), (5000, 1024), (200_000, 65_536)])
@pytest.mark.parametrize("sel_mode", [0, 1])
def test_random_string_filter(n, batch, sel_mode, G, oracle):
    cases.same_batches(cases.r_string_filter(G, n + 5, n, batch, sel_mode),
                       cases.r_string_filter(oracle, n + 5, n, batch, sel_mode))


@pytest.mark.parametrize("n,batch", [(33, 32), (3000, 256), (100_000, 16_384)])
@pytest.mark.parametrize("temp_dir", ["tmp", None], ids=["sorted", "hash"])
def test_random_string_group(n, batch, temp_dir, G, oracle):
    td = None if temp_dir is None else oracle.tmp
    cases.same_batches(cases.r_string_group(G, n + 9, n, batch, 1, td),
                       cases.r_string_group(oracle, n + 9, n, batch, 1, td), rtol=1e-12, tol_cols=FP_COLS)


@pytest.mark.parametrize("temp_dir", ["tmp", None], ids=["sorted", "hash"])
def test_many_string_groups(temp_dir, G, oracle):
    """500k rows, 60k distinct keys of 0-40 bytes sharing long prefixes:
    the dictionary grows from its first size through several doublings and
    the key order sorts over six 8-byte chunks."""
    from vectra_gb300.plan import tbl
    rng = np.random.default_rng(8)
    n, d = 500_000, 60_000
    pool = ["%s%d" % ("p" * int(rng.integers(0, 34)), i) for i in range(d)]
    keys = [pool[i] for i in rng.integers(0, d, n)]
    t = {"g": (keys, rng.random(n) > 0.01), "x": rng.lognormal(0, 1, n), "i": rng.integers(0, 100, n)}

    def q(E):
        td = None if temp_dir is None else oracle.tmp
        return tbl(E, t, batch_rows=100_000).group_by("g").summarise(
            temp_dir=td, s=("sum", "x"), si=("sum", "i"), n=("n",)).batches()
    cases.same_batches(q(G), q(oracle), rtol=1e-12, tol_cols=FP_COLS)


def test_string_key_over_vtr_scan(tmp_path, G, oracle):
    """group_by a string column of a .vtr file read by the GPU scan (the
    string column travels through the host path) and a string filter."""
    from vectra_gb300 import vtr
    from vectra_gb300.plan import col, grepl, scan, tbl
    t = cases.vtr_weather_table()
    p = str(tmp_path / "w.vtr")
    vtr.write_vtr(p, t, 600)
    got = (scan(G, p).filter(~grepl("i", col("city"))).group_by("city")
           .summarise(temp_dir=oracle.tmp, n=("n",), s=("sum", "temperature", True)).batches())
    want = (tbl(oracle, t, batch_rows=600).filter(~grepl("i", col("city"))).group_by("city")
            .summarise(temp_dir=oracle.tmp, n=("n",), s=("sum", "temperature", True)).batches())
    cases.same_batches(got, want, rtol=1e-12, tol_cols=("s",))


def test_string_aggregate_input_is_an_error(G):
    """Aggregating a string column stays an explicit error (no fallback)."""
    from vectra_gb300.plan import EngineError, tbl
    t = cases.T(g=[1, 2], s=["a", "b"])
    with pytest.raises(EngineError):
        tbl(G, t).group_by("g").summarise(m=("min", "s")).batches()
