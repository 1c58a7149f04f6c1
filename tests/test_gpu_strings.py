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


@pytest.mark.parametrize("case", cases.STRING_JOIN_CASES, ids=lambda f: f.__name__)
def test_string_join_cases(case, G, oracle):
    """String join keys (one dictionary: build strings inserted, probe
    strings looked up) and string columns carried on both sides."""
    cases.same_batches(case(G), case(oracle))


@pytest.mark.parametrize("kind", ["inner_join", "left_join", "semi_join", "anti_join", "full_join"])
@pytest.mark.parametrize("n,batch", [(0, 32), (33, 32), (500, 64), (20_000, 4096)])
def test_random_string_join(kind, n, batch, G, oracle):
    cases.same_batches(cases.r_string_join(G, n + 3, n, batch, kind),
                       cases.r_string_join(oracle, n + 3, n, batch, kind))


@pytest.mark.parametrize("temp_dir", ["tmp", None], ids=["sorted", "hash"])
def test_join_then_group_by_strings(temp_dir, G, oracle):
    """group_by a build-side string column after a string-key join (the
    aggregation consumes the join's batches), and group_by a probe-side
    string column above an int64-key join (fused)."""
    from vectra_gb300.plan import tbl
    rng = np.random.default_rng(12)
    n = 40_000
    cats = np.array(["c%02d" % i for i in range(30)], dtype=object)
    fact = {"name": (cases.random_strings(rng, n, 300, maxlen=8), rng.random(n) > 0.02), "v": rng.lognormal(0, 1, n),
            "id": rng.integers(0, 500, n), "city": (cats[rng.integers(0, 30, n)], rng.random(n) > 0.05)}
    names = cases.random_strings(rng, 250, 260, maxlen=8)
    _, first = np.unique(names, return_index=True)
    dim_s = {"name": names[np.sort(first)], "grp": cats[rng.integers(0, 30, len(first))]}
    dim_i = {"id": np.arange(500), "w": rng.random(500)}
    td = None if temp_dir is None else oracle.tmp

    def q1(E):
        return (tbl(E, fact, batch_rows=8192).inner_join(tbl(E, dim_s), "name").group_by("grp")
                .summarise(temp_dir=td, s=("sum", "v"), n=("n",)).batches())

    def q2(E):
        return (tbl(E, fact, batch_rows=8192).left_join(tbl(E, dim_i), "id").group_by("city")
                .summarise(temp_dir=td, s=("sum", "w", True), n=("n",)).batches())
    cases.same_batches(q1(G), q1(oracle), rtol=1e-12, tol_cols=("s",))
    cases.same_batches(q2(G), q2(oracle), rtol=1e-12, tol_cols=("s",))


def test_string_sort_case(G, oracle):
    """arrange() by string keys (dictionary ranks) with string columns
    carried, in both directions."""
    cases.same_batches(cases.ss_string_keys(G), cases.ss_string_keys(oracle))


@pytest.mark.parametrize("n,batch", [(0, 32), (33, 32), (2000, 256), (300_000, 65_536)])
def test_random_string_sort(n, batch, G, oracle):
    cases.same_batches(cases.r_string_sort(G, n + 1, n, batch), cases.r_string_sort(oracle, n + 1, n, batch))


def test_string_order_long_prefixes(G):
    """60k distinct strings of 0-33 'p's and a number, sorted three times:
    the dictionary's 8-byte order words past each string's end must be
    zero (they once picked up an earlier byte of the string, so a string
    could sort after a longer one it prefixes)."""
    from vectra_gb300.plan import tbl
    rng = np.random.default_rng(8)
    pool = sorted({"%s%d" % ("p" * int(rng.integers(0, 34)), i) for i in range(60_000)})
    want = sorted(pool, key=lambda s: s.encode())
    t = {"g": np.array(pool, dtype=object), "i": np.arange(len(pool))}
    for _ in range(3):
        got = tbl(G, t, batch_rows=100_000).arrange("g").batches()[0]["g"][0]
        assert list(got) == want


@pytest.mark.parametrize("master", range(3))
def test_random_string_plans(master, G, oracle):
    """Randomly drawn plans over string columns (the oracle's fuzzing
    against the reference draws the same kinds): sizes at warp and batch
    edges, selection vectors, both group paths, every join kind, sorts."""
    import sys
    sys.path.insert(0, __import__("os").path.dirname(__file__))
    from test_oracle_fuzz import _string_case, FP
    rng = np.random.default_rng(5000 + master)
    for _ in range(25):
        q = _string_case(rng)
        cases.same_batches(q(G), q(oracle), rtol=1e-12, tol_cols=FP + ("s1",))
