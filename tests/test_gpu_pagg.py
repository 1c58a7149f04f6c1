"""The partitioned group aggregation (many groups, one int64 key, key-ordered
output) against the CPU oracle through the node C API.

VGPU_PAGG=1 sends every eligible plan down the partitioned path whatever its
size, so small inputs exercise it: records per key-range bucket, the bucket
reducer, the bucket split (VGPU_PAGG_G / VGPU_PAGG_BUCKETS force buckets
with more groups than a reducer CTA holds), several input batches (one
record region each), filters and joins in front, every accumulator class,
the NA-key group, and exact double sums (values outside a group's digit
window).  Bit-exact except double sums / means (relative 1e-12 against the
oracle's left-to-right sums; test_pagg_exact_sums has no tolerance)."""
import ctypes as C

import numpy as np
import pytest

import cases
from engines import exact_sum

pytestmark = pytest.mark.gpu

FP_COLS = ("s", "m", "sr", "mr", "p", "mx", "lo", "hi")
RTOL = 1e-12
SCRAMBLE = 0x9E3779B97F4A7C15


@pytest.fixture(scope="module")
def G():
    from engines import gpu_engine
    return gpu_engine()


@pytest.fixture
def force(monkeypatch):
    monkeypatch.setenv("VGPU_PAGG", "1")
    return monkeypatch


def runs(G):
    G.lib.vgpu_pagg_runs.restype = C.c_ulonglong
    return G.lib.vgpu_pagg_runs()


def high_card_table(seed, n, distinct, na=0.05):
    rng = np.random.default_rng(seed)
    raw = rng.integers(0, distinct, n).astype(np.uint64)
    key = (raw * np.uint64(SCRAMBLE)).astype(np.int64)          # spread over the whole int64 range
    kv = rng.random(n) >= na
    return {"k": (key, kv), "x": (rng.lognormal(0, 2, n), rng.random(n) > 0.01),
            "y": rng.integers(-1_000_000, 1_000_001, n)}


def five_aggs(E, t, td, batch_rows=None):
    from vectra_gb300.plan import tbl
    return (tbl(E, t, batch_rows=batch_rows or len(t["y"])).group_by("k")
            .summarise(temp_dir=td, s=("sum", "x"), m=("mean", "x"), lo=("min", "y"), hi=("max", "y"),
                       n=("n",)).batches())


def check(G, oracle, fn):
    before = runs(G)
    a = fn(G, oracle.tmp)
    assert runs(G) > before, "the partitioned path did not run"
    b = fn(oracle, oracle.tmp)
    cases.same_batches(a, b, rtol=RTOL, tol_cols=FP_COLS)
    return a


@pytest.mark.parametrize("n,distinct", [(1, 1), (1000, 300), (200_000, 60_000)])
def test_pagg_high_card(n, distinct, G, oracle, force):
    t = high_card_table(n, n, distinct)
    check(G, oracle, lambda E, td: five_aggs(E, t, td))


def test_pagg_bucket_split(G, oracle, force):
    """Two buckets of ~25k groups with room for 256 per reducer CTA: every
    bucket is split by its key range, twice over."""
    force.setenv("VGPU_PAGG_G", "256")
    force.setenv("VGPU_PAGG_BUCKETS", "2")
    t = high_card_table(3, 120_000, 50_000)
    check(G, oracle, lambda E, td: five_aggs(E, t, td))


def test_pagg_batches(G, oracle, force):
    """Seven input batches: seven record regions per bucket."""
    t = high_card_table(4, 200_000, 40_000)
    check(G, oracle, lambda E, td: five_aggs(E, t, td, batch_rows=30_000))


def test_pagg_narrow_keys(G, oracle, force):
    """Keys spanning fewer values than buckets (one key per bucket), all
    keys NA, and negative keys."""
    rng = np.random.default_rng(5)
    n = 50_000
    ts = [{"k": (rng.integers(-40, 60, n), rng.random(n) > 0.1), "x": (rng.normal(0, 1, n), None),
           "y": rng.integers(-5, 5, n)},
          {"k": (np.zeros(n, np.int64), np.zeros(n, bool)), "x": (rng.normal(0, 1, n), None),
           "y": rng.integers(-5, 5, n)},
          {"k": (np.full(n, -(2 ** 63) + 5, np.int64), None), "x": (rng.normal(0, 1, n), None),
           "y": rng.integers(-5, 5, n)}]
    for t in ts:
        check(G, oracle, lambda E, td: five_aggs(E, t, td))


def test_pagg_filter_every_class(G, oracle, force):
    """A filter in front and every accumulator class: int64 sum / mean,
    double min / max with and without na.rm, count of valid values, bool
    min, a projected expression."""
    from vectra_gb300.plan import tbl, col
    rng = np.random.default_rng(6)
    n = 150_000
    key = (rng.integers(0, 30_000, n).astype(np.uint64) * np.uint64(SCRAMBLE)).astype(np.int64)
    t = {"k": (key, rng.random(n) > 0.03), "x": (rng.normal(0, 1, n), rng.random(n) > 0.05),
         "y": (rng.integers(-100, 100, n), rng.random(n) > 0.05),
         "b": (rng.integers(0, 2, n).astype(np.uint8), rng.random(n) > 0.05)}

    def q(E, td):
        return (tbl(E, t, batch_rows=40_000).filter(col("x") > -0.5).group_by("k")
                .summarise(temp_dir=td, si=("sum", "y"), mi=("mean", "y", True), lo=("min", "x", True),
                           hi=("max", "x"), c=("count", "x"), bl=("min", "b"), p=("sum", col("x") * col("x"), True),
                           n=("n",)).batches())
    check(G, oracle, q)


@pytest.mark.parametrize("kind", ["left_join", "inner_join"])
def test_pagg_join_in_front(kind, G, oracle, force):
    """A join to a dimension, then group_by the fact key: the join probe
    runs in the partition pass (an inner join leaves holes in the record
    ranges of the rows it drops)."""
    from vectra_gb300.plan import tbl, col
    rng = np.random.default_rng(7)
    nf, nd = 120_000, 9_000
    ids = rng.permutation(nd) + 1
    fact = {"key": (rng.integers(1, nd + 500, nf), rng.random(nf) > 0.02),
            "value": (rng.lognormal(0, 1, nf), rng.random(nf) > 0.02)}
    dim = {"id": ids, "weight": rng.random(nd)}

    def q(E, td):
        return (getattr(tbl(E, fact, batch_rows=50_000), kind)(tbl(E, dim, batch_rows=4096), {"key": "id"})
                .group_by("key").summarise(temp_dir=td, s=("sum", col("value") * col("weight")),
                                           mx=("max", "weight"), n=("n",)).batches())
    check(G, oracle, q)


def test_pagg_global_cursors(G, oracle, force):
    """Records placed through per-bucket global cursors (the mode for more
    buckets than the partition kernel keeps counters for), with a filter."""
    from vectra_gb300.plan import tbl, col
    force.setenv("VGPU_PAGG_ATOMIC", "1")
    t = high_card_table(9, 100_000, 30_000)

    def q(E, td):
        return (tbl(E, t, batch_rows=60_000).filter(col("y") > -500_000).group_by("k")
                .summarise(temp_dir=td, s=("sum", "x"), m=("mean", "x"), lo=("min", "y"), hi=("max", "y"),
                           n=("n",)).batches())
    check(G, oracle, q)


def test_pagg_exact_sums(G, force):
    """Double sums on the partitioned path are exactly rounded: values far
    outside a group's digit window go to the compensated pair."""
    from vectra_gb300.plan import tbl
    rng = np.random.default_rng(11)
    patterns = [
        rng.normal(0, 1, 500),
        np.concatenate([rng.normal(0, 1e300, 5), rng.normal(0, 1e-300, 5), [1e308, -1e308, 3.0]]),
        np.concatenate([[1e16, 1.0, -1e16] * 20, rng.normal(0, 1, 7)]),
        rng.normal(0, 1, 300) * 10.0 ** rng.integers(-30, 30, 300),
        np.array([5e-324, 5e-324, -1e-320, 2.2250738585072014e-308]),
        np.array([0.1] * 10),
    ]
    keys = np.concatenate([np.full(len(p), 1000 * g - 2500) for g, p in enumerate(patterns)])
    xs = np.concatenate(patterns)
    perm = rng.permutation(len(xs))
    before = runs(G)
    out = tbl(G, {"g": keys[perm], "x": xs[perm]}).group_by("g").summarise(temp_dir="tmp", s=("sum", "x"),
                                                                             m=("mean", "x")).collect()
    assert runs(G) > before
    for g, p in enumerate(patterns):
        assert out["g"][0][g] == 1000 * g - 2500
        want = exact_sum(p)
        assert out["s"][0][g] == want, (g, out["s"][0][g], want)
        assert out["m"][0][g] == want / len(p)


def test_pagg_not_taken_for_hash_order(G, oracle, force):
    """First-seen order (no temp_dir) keeps the hash path."""
    t = high_card_table(8, 20_000, 5_000)
    before = runs(G)
    a = five_aggs(G, t, None)
    assert runs(G) == before
    cases.same_batches(a, five_aggs(oracle, t, None), rtol=RTOL, tol_cols=FP_COLS)


def test_window_rounding_matches_general(G):
    """The reducer's register-only rounding of a six-digit window gives the
    same double as the general digit rounding, on 4M seeded windows."""
    G.lib.vgpu_pagg_window_selftest.restype = C.c_longlong
    assert G.lib.vgpu_pagg_window_selftest(C.c_longlong(4_000_000), C.c_ulonglong(12345)) == 0


def test_fanout_tuning(G, oracle, force, tmp_path):
    """Tuning on: the first seven queries of a new shape class run the
    sketch's bucket count x1, x2, x4 with one reducer CTA per SM, x1, x2
    with two, x1 with four and x1 with eight -- each result equal to the
    oracle's -- the fastest is appended to the tuning file and the eighth
    query runs it."""
    tune = tmp_path / "tune.txt"
    force.setenv("VGPU_TUNE_FILE", str(tune))
    lib = G.lib
    lib.vgpu_pagg_tuned.restype = C.c_int
    lib.vgpu_pagg_tuned.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    lib.vgpu_pagg_tune.argtypes = [C.c_int]
    t = high_card_table(11, 300_007, 90_001)
    want = five_aggs(oracle, t, oracle.tmp)
    shape = C.create_string_buffer(96)
    ctas = C.c_int(0)
    ms = C.c_double(0)
    lib.vgpu_pagg_tune(1)
    try:
        seen = []
        for i in range(8):
            cases.same_batches(five_aggs(G, t, oracle.tmp), want, rtol=RTOL, tol_cols=FP_COLS)
            d = lib.vgpu_pagg_tuned(shape, 96, C.byref(ctas), C.byref(ms))
            seen.append((d, ctas.value))
            assert ms.value > 0.0
        assert seen[:7] == [(0, 1), (1, 1), (2, 1), (0, 2), (1, 2), (0, 4), (0, 8)], seen
        lines = [ln.split() for ln in tune.read_text().splitlines() if ln.startswith("pagg.")]
        assert len(lines) == 1 and lines[0][0] == shape.value.decode(), lines
        assert (int(lines[0][2]), int(lines[0][1])) == seen[7] and lines[0][5] == "7", (lines, seen)
    finally:
        lib.vgpu_pagg_tune(0)
