"""Parity cases for the filter / group-agg / join path.

Each case is a function (engine) -> list of batches ({name: (values,
valid)}), built with the plan verbs, so the same case runs on the reference
engine, the CPU oracle and libvgpu.  The first group restates the
reference's own testthat cases (tests/testthat/test-filter.R,
test-groupby.R, test-agg.R, test-joins.R, test-full-join.R,
test-optimize.R); the rest are seeded random tables with NA, ragged batch
sizes and selection vectors.
"""
import numpy as np

from vectra_gb300.plan import tbl, col, lit, is_na, nchar, substr, grepl

NA = None


def vals(x, dtype=None):
    """(values, valid) from a list with None as NA."""
    valid = np.array([v is not None for v in x], dtype=bool)
    if dtype is None and any(isinstance(v, str) for v in x):
        return np.array(["" if v is None else v for v in x], dtype=object), valid
    if dtype is None:
        dtype = np.float64 if any(isinstance(v, float) for v in x) else np.int64
    fill = [0 if v is None else v for v in x]
    return np.array(fill, dtype=dtype), valid


def T(**cols):
    out = {}
    for k, v in cols.items():
        out[k] = vals(v) if isinstance(v, list) else v
    return out


# ---------------------------------------------------------------------------
# restated reference tests
# ---------------------------------------------------------------------------

def f_simple(E):          # test-filter.R:1-11
    t = T(x=[1.0, 2.0, 3.0, 4.0, 5.0], y=[10, 20, 30, 40, 50])
    return tbl(E, t).filter(col("x") > 2.0).batches()


def f_equality(E):        # test-filter.R:13-20
    t = T(x=[1, 2, 3, 2, 1])
    return tbl(E, t).filter(col("x").eq(2.0)).batches()


def f_and_or_not(E):      # test-filter.R:22-47
    t = T(x=[1.0, 2.0, 3.0, 4.0, 5.0], y=[5.0, 4.0, 3.0, 2.0, 1.0])
    a = tbl(E, t).filter((col("x") > 1.0) & (col("y") > 1.0)).batches()
    b = tbl(E, t).filter((col("x") < 2.0) | (col("y") < 2.0)).batches()
    c = tbl(E, t).filter(~(col("x") > 3.0)).batches()
    return a + b + c


def f_na_dropped(E):      # test-filter.R:58-69
    t = T(x=[1.0, NA, 3.0, NA, 5.0])
    return tbl(E, t).filter(col("x") > 2.0).batches()


def f_is_na(E):           # test-filter.R:49-56
    t = T(x=[1.0, NA, 3.0], y=[1, 2, 3])
    return tbl(E, t).filter(is_na(col("x"))).batches() + tbl(E, t).filter(~is_na(col("x"))).batches()


def f_kleene(E):          # NA & FALSE = FALSE, NA | TRUE = TRUE (src/scalar_ops.c:168-181)
    t = T(a=[1.0, NA, 3.0, NA, 0.0, 2.0], b=[NA, 1.0, NA, 0.0, NA, 2.0])
    x = tbl(E, t).filter((col("a") > 1.0) | (col("b") > 0.5)).batches()
    y = tbl(E, t).filter(~((col("a") > 1.0) & (col("b") > 0.5))).batches()
    return x + y


def f_double_filter(E):   # test-filter.R:89-97
    t = T(x=list(range(1, 21)), y=[float(i % 7) for i in range(20)])
    return tbl(E, t, batch_rows=8).filter(col("x") > 5).filter(col("y") < 4.0).batches()


def f_empty(E):           # test-filter.R:163-173
    t = T(x=[1.0, 2.0, 3.0])
    return tbl(E, t).filter(col("x") > 100.0).batches()


def f_general_expr(E):    # column-vs-column and arithmetic predicates
    t = T(x=[1.0, 5.0, NA, 7.0, 2.0, 9.0], y=[2, 3, 4, NA, 1, 9])
    a = tbl(E, t).filter(col("x") > col("y")).batches()
    b = tbl(E, t).filter((col("x") + col("y")) >= 8.0).batches()
    c = tbl(E, t).filter((col("y") % 2).eq(1) | is_na(col("x"))).batches()
    return a + b + c


def f_int_vs_double_literal(E):   # int64 column compared with a double (src/scalar_ops.c:110-142)
    big = 2 ** 53
    t = T(v=[big - 2, big - 1, big, big + 1, big + 2, big + 3, -5, 0, 7])
    out = []
    for op in (">", ">=", "<", "<=", "==", "!="):
        e = col("v")._cmp(op, float(big + 1))
        out += tbl(E, t).filter(e).batches()
    out += tbl(E, t).filter(col("v") > 2.5).batches()
    out += tbl(E, t).filter(col("v") <= -4.5).batches()
    return out


def g_basic(E, temp_dir):          # test-groupby.R:1-46
    t = T(g=[1, 2, 1, 2, 1], x=[1.0, 2.0, 3.0, 4.0, 5.0])
    return tbl(E, t).group_by("g").summarise(temp_dir=temp_dir, n=("n",), s=("sum", "x"), m=("mean", "x"),
                                            lo=("min", "x"), hi=("max", "x")).batches()


def g_na_key(E, temp_dir):         # test-groupby.R:48-59
    t = T(g=[1, NA, 1, NA, 2], x=[1.0, 2.0, 3.0, 4.0, 5.0])
    return tbl(E, t).group_by("g").summarise(temp_dir=temp_dir, s=("sum", "x"), n=("n",)).batches()


def g_multi_key(E, temp_dir):      # test-groupby.R:61-72
    t = T(a=[1, 1, 2, 2, 1, NA], b=[1.0, 2.0, 1.0, 1.0, 1.0, 2.0], x=[1, 2, 3, 4, 5, 6])
    return tbl(E, t).group_by("a", "b").summarise(temp_dir=temp_dir, s=("sum", "x"), n=("n",)).batches()


def g_na_semantics(E, temp_dir):   # test-agg.R:3-127, test-groupby.R:74-99
    t = T(g=[1, 1, 2, 2, 3, 3], x=[1.0, NA, NA, NA, 4.0, 5.0], y=[1, NA, NA, NA, 7, 9])
    return tbl(E, t).group_by("g").summarise(
        temp_dir=temp_dir, s=("sum", "x"), m=("mean", "x"), lo=("min", "x"), hi=("max", "x"),
        sr=("sum", "x", True), mr=("mean", "x", True), lor=("min", "x", True), hir=("max", "x", True),
        si=("sum", "y"), sir=("sum", "y", True), mir=("mean", "y", True), loi=("min", "y", True),
        hii=("max", "y", True), n=("n",), c=("count", "x")).batches()


def g_int_sum_double(E, temp_dir):  # test-agg.R:131-139
    t = T(g=[1, 1, 2], y=[2 ** 40, 3, -7])
    return tbl(E, t).group_by("g").summarise(temp_dir=temp_dir, s=("sum", "y"), m=("mean", "y")).batches()


def g_resize_200(E, temp_dir):      # test-groupby.R:101-131 (200 groups over 2000 rows)
    rng = np.random.default_rng(101)
    g = rng.integers(0, 200, 2000)
    x = rng.normal(0, 1, 2000)
    t = {"g": g, "x": x}
    return tbl(E, t, batch_rows=256).group_by("g").summarise(temp_dir=temp_dir, s=("sum", "x"),
                                                              m=("mean", "x"), n=("n",)).batches()


def g_filter_then_group(E, temp_dir):   # test-groupby.R:133-149, test-filter.R:247-284
    t = T(g=[1, 2, 1, 2, 3, 3, 1], x=[1.0, 5.0, 3.0, 7.0, 2.0, 9.0, NA])
    return (tbl(E, t, batch_rows=32).filter(col("x") > 2.0).group_by("g")
            .summarise(temp_dir=temp_dir, s=("sum", "x"), n=("n",)).batches())


def g_program_filter_then_group(E, temp_dir):   # a predicate that does not fold into ranges
    rng = np.random.default_rng(31)
    n = 3000
    x = np.where(np.arange(n) // 500 == 2, -1.0, rng.normal(0, 3, n))   # rows 1000-1499: none pass
    t = {"g": (rng.integers(0, 40, n), rng.random(n) > 0.05), "x": (x, rng.random(n) > 0.05),
         "y": (rng.integers(-5, 5, n), rng.random(n) > 0.1)}
    pred = ((col("x") * 2.0) > col("y")) | (is_na(col("y")) & (col("x") > 0.0))
    return (tbl(E, t, batch_rows=500).filter(pred).group_by("g")
            .summarise(temp_dir=temp_dir, s=("sum", "x", True), n=("n",), c=("count", "y")).batches())


def g_program_filter_join_group(E, temp_dir):   # the same below a fused join
    rng = np.random.default_rng(32)
    n, d = 4000, 300
    fact = {"k": (rng.integers(0, d + 20, n), rng.random(n) > 0.03), "v": rng.lognormal(0, 1, n),
            "z": rng.integers(0, 10, n)}
    dim = {"k": np.arange(d), "cat": rng.integers(0, 12, d), "w": rng.random(d)}
    pred = (col("z") % 3).eq(0) | (col("v") > 2.5)
    return (tbl(E, fact, batch_rows=700).filter(pred).left_join(tbl(E, dim, batch_rows=128), "k").group_by("cat")
            .summarise(temp_dir=temp_dir, s=("sum", col("v") * col("w"), True), n=("n",)).batches())


def g_ungrouped(E, temp_dir):       # summarise without group_by (hash path, one group)
    t = T(x=[1.0, 2.0, NA, 4.0])
    a = tbl(E, t).group_by().summarise(temp_dir=temp_dir, s=("sum", "x", True), n=("n",)).batches()
    b = tbl(E, T(x=[1.0])).filter(col("x") > 5.0).group_by().summarise(temp_dir=temp_dir, n=("n",)).batches()
    return a + b


def g_nested_expr(E, temp_dir):     # test-optimize.R:73-96: sum(x + y) via a hidden projection
    t = T(g=[1, 1, 2, 2], x=[1.0, 2.0, 3.0, NA], y=[10.0, 20.0, 30.0, 40.0])
    return tbl(E, t).group_by("g").summarise(temp_dir=temp_dir, s=("sum", col("x") + col("y")),
                                            p=("sum", col("x") * col("y"), True)).batches()


def g_bool_and_double_keys(E, temp_dir):
    t = T(b=vals([1, 0, 1, None, 0, 1], np.uint8), d=[0.5, -0.0, 0.0, 2.5, NA, 0.5], x=[1, 2, 3, 4, 5, 6])
    a = tbl(E, t).group_by("b").summarise(temp_dir=temp_dir, s=("sum", "x"), lo=("min", "b"), n=("n",)).batches()
    return a


def j_inner_left_semi_anti(E):      # test-joins.R:12-56
    l = T(id=[1, 2, 3, 4], x=[10.0, 20.0, 30.0, 40.0])
    r = T(id=[2, 3, 5], y=[200.0, 300.0, 500.0])
    out = []
    out += tbl(E, l).inner_join(tbl(E, r), "id").batches()
    out += tbl(E, l).left_join(tbl(E, r), "id").batches()
    out += tbl(E, l).semi_join(tbl(E, r), "id").batches()
    out += tbl(E, l).anti_join(tbl(E, r), "id").batches()
    return out


def j_duplicates(E):                # test-joins.R:84-95 (fan-out, descending build order)
    l = T(k=[1, 2, 1, 3], x=[1.0, 2.0, 3.0, 4.0])
    r = T(k=[1, 1, 2, 1, 4], y=[10.0, 11.0, 20.0, 12.0, 40.0])
    return (tbl(E, l).inner_join(tbl(E, r), "k").batches() +
            tbl(E, l).left_join(tbl(E, r), "k").batches())


def j_na_keys(E):                   # test-joins.R:97-120
    l = T(k=[1, NA, 3, NA], x=[1.0, 2.0, 3.0, 4.0])
    r = T(k=[NA, 1, 3, NA], y=[10.0, 11.0, 13.0, 14.0])
    out = []
    for kind in ("inner_join", "left_join", "semi_join", "anti_join"):
        out += getattr(tbl(E, l), kind)(tbl(E, r), "k").batches()
    return out


def j_suffix(E):                    # test-joins.R:122-133
    l = T(id=[1, 2], v=[1.0, 2.0])
    r = T(id=[1, 2], v=[10.0, 20.0])
    return tbl(E, l).inner_join(tbl(E, r), "id").batches()


def j_coerce(E):                    # test-joins.R:220-272
    l = T(id=[1, 2, 3], x=[10.0, 20.0, 30.0])
    r = T(id=[1.0, 2.0, 4.0], y=[100.0, 200.0, 400.0])
    a = tbl(E, l).inner_join(tbl(E, r), "id").batches()
    l2 = T(a=[1.0, 2.0], b=[10, 20], x=[1.0, 2.0])
    r2 = T(a=[1.0, 2.0], b=[10.0, 20.0], y=[3.0, 4.0])
    b = tbl(E, l2).inner_join(tbl(E, r2), ["a", "b"]).batches()
    return a + b


def j_streaming(E):                 # test-joins.R:314-409 (batch_size = 10)
    rng = np.random.default_rng(314)
    l = {"k": rng.integers(0, 30, 95), "x": rng.normal(0, 1, 95)}
    r = {"k": rng.integers(0, 40, 50), "y": rng.normal(0, 1, 50)}
    out = []
    for kind in ("inner_join", "left_join", "semi_join", "anti_join"):
        out += getattr(tbl(E, l, batch_rows=10), kind)(tbl(E, r, batch_rows=10), "k").batches()
    return out


def j_after_filter(E):              # test-joins.R:411-423
    l = T(id=[1, 2, 3, 4, 5], x=[1.0, 2.0, 3.0, 4.0, 5.0])
    r = T(id=[2, 4, 5], y=[20.0, 40.0, 50.0])
    return tbl(E, l).filter(col("x") > 2.0).inner_join(tbl(E, r), "id").batches()


def j_full(E):                      # test-full-join.R:3-72
    l = T(id=[1, 2, 3], x=[1.0, 2.0, 3.0])
    r = T(id=[2, 3, 4, 5], y=[20.0, 30.0, 40.0, 50.0])
    return tbl(E, l).full_join(tbl(E, r), "id").batches()


def ja_join_agg(E, temp_dir):       # the benchmark plan, small: left_join then sum(value * weight)
    rng = np.random.default_rng(7)
    nf, nd = 5000, 300
    ids = rng.permutation(nd) + 1
    fact = {"key": (rng.integers(1, nd + 40, nf), rng.random(nf) > 0.01),
            "value": (rng.lognormal(0, 1, nf), rng.random(nf) > 0.02)}
    dim = {"id": ids, "category": rng.integers(0, 16, nd), "weight": rng.random(nd)}
    a = (tbl(E, fact, batch_rows=1024).left_join(tbl(E, dim, batch_rows=128), {"key": "id"})
         .group_by("category").summarise(temp_dir=temp_dir, s=("sum", col("value") * col("weight")),
                                          sr=("sum", col("value") * col("weight"), True), n=("n",)).batches())
    return a


def ja_join_agg_sparse(E, temp_dir):   # the benchmark plan with scattered ids (hashed join table)
    rng = np.random.default_rng(8)
    nf, nd = 4000, 250
    ids = (rng.permutation(nd) + 1) * 7_000_003 - 2_000_000_000
    fk = ids[rng.integers(0, nd, nf)]
    fk[rng.random(nf) < 0.05] += 1                      # some probe keys match nothing
    fact = {"key": (fk, rng.random(nf) > 0.01), "value": (rng.lognormal(0, 1, nf), rng.random(nf) > 0.02)}
    dim = {"id": ids, "category": rng.integers(0, 16, nd), "weight": rng.random(nd)}
    out = []
    for kind in ("left_join", "inner_join"):
        out += (getattr(tbl(E, fact, batch_rows=1024), kind)(tbl(E, dim, batch_rows=128), {"key": "id"})
                .group_by("category").summarise(temp_dir=temp_dir, s=("sum", col("value") * col("weight")),
                                                n=("n",)).batches())
    return out


def ja_dup_build_keys(E, temp_dir):  # join + aggregate where some build keys repeat (many matches per row)
    rng = np.random.default_rng(9)
    nf, nd = 3000, 400
    ids = rng.integers(1, 300, nd)                      # ~100 repeated ids
    fact = {"key": (rng.integers(1, 320, nf), rng.random(nf) > 0.02), "value": rng.lognormal(0, 1, nf)}
    dim = {"id": ids, "category": rng.integers(0, 12, nd), "weight": (rng.random(nd), rng.random(nd) > 0.05)}
    out = []
    for kind in ("left_join", "inner_join"):
        out += (getattr(tbl(E, fact, batch_rows=1024), kind)(tbl(E, dim, batch_rows=128), {"key": "id"})
                .group_by("category").summarise(temp_dir=temp_dir, s=("sum", col("value") * col("weight")),
                                                n=("n",)).batches())
    return out


def ja_dense_keys(E, temp_dir):     # join + aggregate keyed on a small-range build-side column
    rng = np.random.default_rng(17)
    nf, nd = 7001, 257
    ids = rng.permutation(nd) + 1
    fact = {"key": (rng.integers(1, nd + 30, nf), rng.random(nf) > 0.02),
            "value": (rng.normal(0, 10, nf), rng.random(nf) > 0.03),
            "q": rng.integers(-5, 5, nf)}
    dims = [{"id": ids, "grp": (rng.integers(-40, -20, nd), rng.random(nd) > 0.1), "weight": rng.random(nd)},
            {"id": ids, "grp": (rng.integers(0, 3, nd), np.zeros(nd, bool)), "weight": rng.random(nd)}]
    out = []
    for dim in dims:
        for kind in ("left_join", "inner_join"):
            out += (getattr(tbl(E, fact, batch_rows=2000).filter(col("q") > -3), kind)(
                        tbl(E, dim, batch_rows=100), {"key": "id"})
                    .group_by("grp").summarise(temp_dir=temp_dir, s=("sum", "value"),
                                               m=("mean", col("value") * col("weight"), True),
                                               lo=("min", "q"), n=("n",)).batches())
    return out


def ja_payload_edges(E, temp_dir):  # join + aggregate: NA build keys, a bool build column, NA payload values
    rng = np.random.default_rng(23)
    nf, nd = 6000, 333
    ids = rng.permutation(nd) + 1
    fact = {"key": (rng.integers(1, nd + 20, nf), rng.random(nf) > 0.02),
            "value": (rng.normal(0, 5, nf), rng.random(nf) > 0.03)}
    dim = {"id": (ids, rng.random(nd) > 0.07),
           "flag": (rng.integers(0, 2, nd).astype(np.uint8), rng.random(nd) > 0.1),
           "weight": (rng.random(nd), rng.random(nd) > 0.05)}
    out = []
    for kind in ("left_join", "inner_join"):
        out += (getattr(tbl(E, fact, batch_rows=1500), kind)(tbl(E, dim, batch_rows=100), {"key": "id"})
                .group_by("flag").summarise(temp_dir=temp_dir, s=("sum", col("value") * col("weight")),
                                            sr=("sum", col("value") * col("weight"), True), n=("n",)).batches())
    return out


# ---------------------------------------------------------------------------
# seeded random cases
# ---------------------------------------------------------------------------

def random_table(seed, n, n_groups=50, na=0.05):
    rng = np.random.default_rng(seed)
    return {
        "k": (rng.integers(0, n_groups, n), rng.random(n) > na),
        "d": (rng.normal(0, 100, n), rng.random(n) > na),
        "i": (rng.integers(-1000, 1000, n), rng.random(n) > na),
        "b": (rng.integers(0, 2, n).astype(np.uint8), rng.random(n) > na),
    }


def r_filter(E, seed, n, batch_rows, sel_mode):
    t = random_table(seed, n)
    pred = (col("d") > -20.0) & (col("i") <= 500) & ~(col("b").eq(True))
    return tbl(E, t, batch_rows=batch_rows, sel_mode=sel_mode).filter(pred).batches()


def r_group(E, seed, n, batch_rows, sel_mode, temp_dir):
    t = random_table(seed, n)
    return (tbl(E, t, batch_rows=batch_rows, sel_mode=sel_mode).filter(col("d") > -150.0)
            .group_by("k").summarise(temp_dir=temp_dir, n=("n",), si=("sum", "i"), mi=("mean", "i", True),
                                     lo=("min", "i"), hi=("max", "d", True), c=("count", "d"),
                                     sd=("sum", "d", True)).batches())


def r_join(E, seed, n, batch_rows, kind, spread=1):
    """spread > 1 scatters the key values far apart (a hashed join table
    instead of the direct-addressed one small key ranges get)."""
    rng = np.random.default_rng(seed)
    l = {"k": (rng.integers(0, 60, n) * spread, rng.random(n) > 0.05), "x": rng.normal(0, 1, n)}
    r = {"k": (rng.integers(0, 80, 70) * spread, rng.random(70) > 0.05), "y": rng.normal(0, 1, 70),
         "z": rng.integers(0, 5, 70)}
    return getattr(tbl(E, l, batch_rows=batch_rows), kind)(tbl(E, r, batch_rows=32), "k").batches()


# --- strings (test-optimize.R:95-148, test-groupby.R:1-150) ---

def sf_nchar(E):                    # test-optimize.R:98-116
    t = T(s=["abc", NA, "de", "f", "hello", "", "h\u00e9"])
    return tbl(E, t).mutate(n=nchar(col("s"))).batches()


def sf_substr(E):                   # test-optimize.R:118-126
    t = T(s=["hello", "world", NA, "ab", ""])
    return tbl(E, t).mutate(sub=substr(col("s"), 1, 3)).batches()


def sf_grepl(E):                    # test-optimize.R:128-148
    t = T(s=["apple", "banana", "grape", "pineapple", NA, "abc", "abcdef", "", "ap"])
    a = tbl(E, t).filter(grepl("app", col("s"))).batches()
    b = tbl(E, t).filter(grepl("abc", col("s"))).batches()
    c = tbl(E, t).filter(grepl("", col("s"))).batches()          # an empty pattern matches
    return a + b + c


def sf_compare_literal(E):          # memcmp, then the shorter first; bytes above 127 unsigned
    w = ["b", "a", "ab", "abc", "", NA, "B", "\u00e9", "ba", "abd", "b", "aa"]
    t = T(s=w, i=list(range(len(w))))
    out = []
    for op in ("==", "!=", "<", "<=", ">", ">="):
        out += tbl(E, t).filter(col("s")._cmp(op, "ab")).batches()
        out += tbl(E, t).filter(lit("b")._cmp(op, col("s"))).batches()
    return out


def sf_compare_columns(E):
    t = T(a=["x", "ab", NA, "abc", "", "zz", "q"], b=["x", "abc", "q", NA, "a", "z", "q"])
    return (tbl(E, t).filter(col("a") < col("b")).batches() + tbl(E, t).filter(col("a").eq(col("b"))).batches()
            + tbl(E, t).filter(~(col("a") >= col("b")) | is_na(col("b"))).batches())


def sf_substr_bounds(E):            # start below 1, stop past the end or before start, double bounds
    t = T(s=["hello", "world", "a", "", NA, "abcdef"], st=[0, 2, 1, 1, 1, -4], sp=[10, 4, 0, 3, 2, 3],
          x=[2.7, 1.2, -3.5, 1.0, 1.0, 3.99])
    return tbl(E, t).mutate(a=substr(col("s"), col("st"), col("sp")), b=substr(col("s"), col("x"), 3.9),
                            c=substr(col("s"), 2, 2), n=nchar(substr(col("s"), 2, 100))).batches()


def sf_substr_filter(E):
    t = T(s=["hello", "help", "shell", "he", NA, "yellow", "ell"])
    return tbl(E, t).filter(substr(col("s"), 2, 4).eq("ell")).batches()


def sf_nchar_filter(E):
    t = T(s=["abc", "", NA, "hello", "ab"], v=[1, 2, 3, 4, 5])
    return (tbl(E, t).filter((nchar(col("s")) > 2) | is_na(col("s"))).batches()
            + tbl(E, t).filter(nchar(col("s")).eq(col("v"))).batches())


def sf_passthrough(E):              # string columns carried through filter and select
    t = T(s=["a", NA, "bb", "ccc", ""], x=[1.0, 2.0, 3.0, 4.0, 5.0], u=["p", "q", NA, "r", "s"])
    return (tbl(E, t).filter(col("x") > 1.5).select("u", "x", "s").batches()
            + tbl(E, t).filter(col("u").ne("q")).mutate(y=col("x") * 2.0).batches())


def sg_string_key(E, temp_dir):     # test-groupby.R:1-60: first-seen order, NA key group
    t = T(g=["a", "b", "a", "b", "a", NA, "", NA, "ab"], x=[1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0])
    return tbl(E, t).group_by("g").summarise(temp_dir=temp_dir, n=("n",), s=("sum", "x"), m=("mean", "x"),
                                            lo=("min", "x"), hi=("max", "x")).batches()


def sg_string_and_int_keys(E, temp_dir):   # test-groupby.R:61-72 with a string key
    t = T(a=["x", "x", "y", "y", "x", NA, "y"], b=[1, 2, 1, 1, 1, 2, NA], v=[10, 20, 30, 40, 50, 60, 70])
    return tbl(E, t).group_by("a", "b").summarise(temp_dir=temp_dir, s=("sum", "v"), n=("n",)).batches()


def sg_string_arena_resizes(E, temp_dir):  # test-groupby.R:101-131: many keys, ragged batches
    rng = np.random.default_rng(55)
    n, d = 6000, 900
    base = ["k%04d" % i + "x" * (i % 37) for i in range(d)]
    pick = rng.integers(0, d, n)
    g = [base[i] for i in pick]
    gv = rng.random(n) > 0.03
    t = {"g": (g, gv), "x": rng.normal(0, 1, n), "i": rng.integers(-50, 50, n)}
    return (tbl(E, t, batch_rows=700).filter(col("i") > -40).group_by("g")
            .summarise(temp_dir=temp_dir, s=("sum", "x"), si=("sum", "i"), n=("n",)).batches())


def sg_zero_bytes(E, temp_dir):    # keys that differ only past a zero byte, or only in length
    t = T(g=["ab", "ab\x00", "ab\x00\x00", "ab", "a\x00b", "", "\x00", "ab\x00", NA, "\x00\x00"],
          x=[1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0, 10.0])
    a = tbl(E, t).group_by("g").summarise(temp_dir=temp_dir, s=("sum", "x"), n=("n",)).batches()
    b = tbl(E, t).filter(col("g") > "ab").batches() + tbl(E, t).filter(nchar(col("g")) >= 3).batches()
    return a + b


def sg_filter_on_string(E, temp_dir):      # a string predicate below a string key
    t = T(g=["apple", "pear", "apple", "fig", NA, "pear", "fig"], x=[1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0])
    return (tbl(E, t).filter(grepl("p", col("g")) | is_na(col("g"))).group_by("g")
            .summarise(temp_dir=temp_dir, s=("sum", "x"), n=("n",)).batches())


def random_strings(rng, n, d, maxlen=24):
    """n strings drawn from d distinct ones with shared prefixes, empty
    strings and bytes above 127."""
    alphabet = list("ab\u00e9z") + ["aa", "\u00ff"]
    pool = []
    for i in range(d):
        k = int(rng.integers(0, maxlen))
        pool.append("".join(alphabet[j] for j in rng.integers(0, len(alphabet), k)))
    return np.array([pool[i] for i in rng.integers(0, d, n)], dtype=object)


def r_string_filter(E, seed, n, batch_rows, sel_mode):
    rng = np.random.default_rng(seed)
    t = {"s": (random_strings(rng, n, 60), rng.random(n) > 0.05), "x": rng.normal(0, 1, n)}
    pred = ((col("s") > "ab") & (nchar(col("s")) <= 9)) | grepl("\u00e9z", col("s")) | substr(col("s"), 2, 3).eq("aa")
    return tbl(E, t, batch_rows=batch_rows, sel_mode=sel_mode).filter(pred).batches()


def r_string_group(E, seed, n, batch_rows, sel_mode, temp_dir):
    rng = np.random.default_rng(seed)
    t = {"s": (random_strings(rng, n, max(n // 7, 3)), rng.random(n) > 0.04), "x": rng.normal(0, 1, n),
         "k": rng.integers(0, 3, n)}
    return (tbl(E, t, batch_rows=batch_rows, sel_mode=sel_mode).filter(col("x") > -1.5)
            .group_by("s", "k").summarise(temp_dir=temp_dir, n=("n",), s1=("sum", "x"), c=("count", "x")).batches())


def sj_string_keys(E):              # test-joins.R:133-147
    l = T(name=["alice", "bob"], x=[1.0, 2.0])
    r = T(name=["bob", "carol"], y=[20.0, 30.0])
    out = []
    for kind in ("inner_join", "left_join", "semi_join", "anti_join", "full_join"):
        out += getattr(tbl(E, l), kind)(tbl(E, r), "name").batches()
    return out


def sj_composite_string_key(E):     # test-joins.R:149-160
    l = T(a=[1.0, 1.0, 2.0], b=["x", "y", "x"], v1=[10.0, 20.0, 30.0])
    r = T(a=[1.0, 2.0], b=["x", "x"], v2=[100.0, 300.0])
    return (tbl(E, l).inner_join(tbl(E, r), ["a", "b"]).batches()
            + tbl(E, l).full_join(tbl(E, r), ["a", "b"]).batches())


def sj_many_string_keys(E):         # test-joins.R:164-190: 200 keys, duplicates, string payloads
    rng = np.random.default_rng(42)
    keys = ["key_%d" % i for i in range(1, 201)]
    l = {"id": np.array([k for k in keys for _ in range(3)], dtype=object), "x": rng.normal(0, 1, 600)}
    r = {"id": np.array(keys[::2] + ["key_x%d" % i for i in range(20)], dtype=object),
         "tag": np.array(["t%d" % (i % 7) for i in range(120)], dtype=object), "y": rng.normal(0, 1, 120)}
    return (tbl(E, l, batch_rows=128).left_join(tbl(E, r, batch_rows=50), "id").batches()
            + tbl(E, l, batch_rows=128).full_join(tbl(E, r, batch_rows=50), "id").batches())


def sj_na_and_empty_string_keys(E):  # NA never matches; "" is a key like any other
    l = T(k=["", NA, "a", "b", NA, ""], x=[1, 2, 3, 4, 5, 6])
    r = T(k=[NA, "", "a", "a", "c"], y=["p", "q", NA, "s", "t"])
    out = []
    for kind in ("inner_join", "left_join", "semi_join", "anti_join", "full_join"):
        out += getattr(tbl(E, l), kind)(tbl(E, r), "k").batches()
    return out


def r_string_join(E, seed, n, batch_rows, kind):
    rng = np.random.default_rng(seed)
    lk = random_strings(rng, n, 40, maxlen=6)
    rk = random_strings(rng, 70, 50, maxlen=6)
    l = {"k": (lk, rng.random(n) > 0.05), "x": rng.normal(0, 1, n), "s": (random_strings(rng, n, 9), rng.random(n) > 0.1)}
    r = {"k": (rk, rng.random(70) > 0.05), "y": rng.normal(0, 1, 70), "t": (random_strings(rng, 70, 5), rng.random(70) > 0.1)}
    return getattr(tbl(E, l, batch_rows=batch_rows), kind)(tbl(E, r, batch_rows=32), "k").batches()


STRING_JOIN_CASES = [sj_string_keys, sj_composite_string_key, sj_many_string_keys, sj_na_and_empty_string_keys]


def ss_string_keys(E):              # arrange by strings: NA last ascending, first descending
    t = T(s=["b", NA, "a", "", "ab", "b", "\u00e9", "aa", NA, "B"], i=[1, 2, 3, 4, 5, 6, 7, 8, 9, 10],
          u=["x", "y", NA, "z", "w", "v", "u", "t", "s", "r"])
    return (tbl(E, t).arrange("s").batches() + tbl(E, t).arrange(("s", True)).batches()
            + tbl(E, t).arrange("u", ("i", True)).batches())


def r_string_sort(E, seed, n, batch_rows):
    rng = np.random.default_rng(seed)
    t = {"s": (random_strings(rng, n, max(n // 5, 2), maxlen=14), rng.random(n) > 0.05),
         "k": rng.integers(0, 4, n), "x": rng.normal(0, 1, n), "p": (random_strings(rng, n, 50), rng.random(n) > 0.1)}
    return tbl(E, t, batch_rows=batch_rows).arrange("k", ("s", True), "x").batches()


STRING_FILTER_CASES = [sf_nchar, sf_substr, sf_grepl, sf_compare_literal, sf_compare_columns, sf_substr_bounds,
                       sf_substr_filter, sf_nchar_filter, sf_passthrough]
STRING_GROUP_CASES = [sg_string_key, sg_string_and_int_keys, sg_string_arena_resizes, sg_filter_on_string,
                      sg_zero_bytes]


FILTER_CASES = [f_simple, f_equality, f_and_or_not, f_na_dropped, f_is_na, f_kleene, f_double_filter,
                f_empty, f_general_expr, f_int_vs_double_literal]
GROUP_CASES = [g_basic, g_na_key, g_multi_key, g_na_semantics, g_int_sum_double, g_resize_200,
               g_filter_then_group, g_ungrouped, g_nested_expr, g_bool_and_double_keys, ja_join_agg,
               ja_dense_keys, ja_join_agg_sparse, ja_dup_build_keys, ja_payload_edges,
               g_program_filter_then_group, g_program_filter_join_group]
JOIN_CASES = [j_inner_left_semi_anti, j_duplicates, j_na_keys, j_suffix, j_coerce, j_streaming,
              j_after_filter, j_full]

# sizes chosen to hit warp / block edges: empty, 1, 31, 32, 33, 65, multi-block
RAGGED = [(0, 32), (1, 32), (31, 32), (32, 32), (33, 32), (65, 64), (1000, 96), (20000, 4096)]


# ---------------------------------------------------------------------------
# comparison
# ---------------------------------------------------------------------------

def same_batches(a, b, rtol=0.0, tol_cols=()):
    """Batch lists equal: names, row counts, validity, and values where
    valid (bit-exact unless the column is listed in tol_cols)."""
    assert len(a) == len(b), "batch count %d != %d" % (len(a), len(b))
    for bi, (x, y) in enumerate(zip(a, b)):
        assert list(x.keys()) == list(y.keys()), (bi, list(x.keys()), list(y.keys()))
        for name in x:
            va, ma = x[name]
            vb, mb = y[name]
            assert len(va) == len(vb), (bi, name, len(va), len(vb))
            assert np.array_equal(ma, mb), (bi, name, "validity", ma, mb)
            va, vb = va[ma], vb[mb]
            if va.dtype == object:
                assert list(va) == list(vb), (bi, name)
            elif name in tol_cols and va.dtype == np.float64:
                both_nan = np.isnan(va) & np.isnan(vb)
                close = np.isclose(va, vb, rtol=rtol, atol=0) | both_nan | (va == vb)
                assert close.all(), (bi, name, va[~close], vb[~close])
            else:
                eq = (va == vb) | (np.isnan(va) & np.isnan(vb) if va.dtype == np.float64 else False)
                assert np.all(eq), (bi, name, va[~eq], vb[~eq])


def vtr_weather_table():
    """The table of tests/golden/ref_weather.vtr (written there by the
    reference's own writer, 7 row groups of 600 rows, the last 234):
    station int64 U{0..99}; temperature double N(20, 10) with 2% NA and
    every even row group below 25; year int64 U{2000..2025}; flag bool with
    5% NA; city string with 3% NA."""
    rng = np.random.default_rng(77)
    n = 6 * 600 + 234
    station = rng.integers(0, 100, n).astype(np.int64)
    temp = rng.normal(20.0, 10.0, n)
    g = np.arange(n) // 600
    temp = np.where(g % 2 == 0, np.minimum(temp, 24.0), temp)
    tv = rng.random(n) >= 0.02
    temp[~tv] = 0.0
    year = rng.integers(2000, 2026, n).astype(np.int64)
    flag = rng.random(n) < 0.4
    fv = rng.random(n) >= 0.05
    flag[~fv] = False
    cities = np.array(["oslo", "lima", "quito", "", "kyiv", "perth"], dtype=object)
    city = list(cities[rng.integers(0, len(cities), n)])
    cv = rng.random(n) >= 0.03
    city = [c if ok else "" for c, ok in zip(city, cv)]
    return {"station": station, "temperature": (temp, tv), "year": year, "flag": (flag, fv),
            "city": (city, cv)}


# --- arrange (SortNode, src/sort.c; tests/testthat/test-verbs.R:174-222) ---

def s_ascending(E):          # test-verbs.R:176-183
    return tbl(E, T(x=[3.0, 1.0, 2.0])).arrange("x").batches()


def s_descending(E):         # test-verbs.R:185-192
    return tbl(E, T(x=[3.0, 1.0, 2.0])).arrange(("x", True)).batches()


def s_multi(E):              # test-verbs.R:194-203 (the grouping key as int64)
    return tbl(E, T(g=[1, 2, 1, 2], x=[2.0, 1.0, 1.0, 2.0])).arrange("g", "x").batches()


def s_na_last(E):            # test-verbs.R:205-213
    return tbl(E, T(x=[2.0, None, 1.0, 3.0])).arrange("x").batches()


def s_na_desc(E):            # NA before the values when descending (src/sort.c:38-40)
    return tbl(E, T(x=[2.0, None, 1.0, None, 3.0], i=[1, 2, 3, 4, 5])).arrange(("x", True)).batches()


def s_ties_stable(E):        # equal keys keep their input order (src/sort.c:97-116)
    return tbl(E, T(k=[2, 1, 2, 1, 2, 1, None, 2], i=[1, 2, 3, 4, 5, 6, 7, 8]), batch_rows=3).arrange("k").batches()


def s_signed_zero_bool(E):   # -0 equals +0; bool keys; int64 extremes
    b = (np.array([True, False, False, True, False]), np.array([True, True, False, True, True]))
    return tbl(E, T(z=[0.0, -0.0, -1.5, 0.0, -0.0], b=b,
                    w=[-(2 ** 63), 2 ** 63 - 1, 0, -1, 1])).arrange(("b", True), "z", ("w", True)).batches()


def s_empty(E):              # no rows: one empty batch
    return tbl(E, T(x=[1.0, 2.0])).filter(col("x") > 5.0).arrange("x").batches()


def s_after_filter(E):       # a selection vector below the sort
    rng = np.random.default_rng(11)
    n = 3000
    t = {"k": (rng.integers(0, 40, n), rng.random(n) > 0.1), "v": (np.round(rng.normal(0, 2, n), 1), rng.random(n) > 0.1),
         "i": np.arange(n)}
    return tbl(E, t, batch_rows=500).filter(col("v") > -1.0).arrange(("k", True), "v").batches()


def r_sort(E, seed, n, batch_rows):
    rng = np.random.default_rng(seed)
    t = {"a": (rng.integers(0, 50, n), rng.random(n) > 0.05), "b": (np.round(rng.normal(0, 3, n), 2), rng.random(n) > 0.05),
         "c": (rng.random(n) < 0.5, rng.random(n) > 0.1), "d": rng.integers(-(2 ** 62), 2 ** 62, n), "i": np.arange(n)}
    return tbl(E, t, batch_rows=batch_rows).arrange(("c", True), "a", ("b", True), "d").batches()


SORT_CASES = [s_ascending, s_descending, s_multi, s_na_last, s_na_desc, s_ties_stable, s_signed_zero_bool, s_empty,
              s_after_filter]
