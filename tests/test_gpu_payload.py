"""Join + aggregate plans whose join build carries a payload copy of the
build columns the fused kernel reads, in each of its entry forms, against
the CPU oracle:

- compact 16-byte entries of two columns (an int64 group key narrowed to its
  range, a double) -- the headline plan's shape -- and the same plan with the
  full 32-byte entries (VGPU_PAY32=1), which must agree bit for bit;
- compact entries of one column;
- full 32-byte entries: two double payload columns, and an int64 column
  whose values span more than 2^32 (too wide to narrow);
- the ahead-of-time kernels after a compact build (the join's slot table is
  then derived from the key column).
"""
import os

import numpy as np
import pytest

import cases
from engines import OracleEngine

pytestmark = pytest.mark.gpu


def _tables(seed, n=200_000, d=30_000, cat=None, w2=False):
    rng = np.random.default_rng(seed)
    ranks = np.arange(1, d + 1, dtype=np.float64)
    cdf = np.cumsum(ranks ** -1.1)
    cdf /= cdf[-1]
    keys = np.minimum(np.searchsorted(cdf, rng.random(n)), d - 1) + 1
    vals = rng.lognormal(0, 1, n)
    vv = rng.random(n) >= 0.02
    vals[~vv] = 0.0
    fact = {"key": keys.astype(np.int64), "value": (vals, vv)}
    c = rng.integers(0, 256, d).astype(np.int64) if cat is None else cat(rng, d)
    cv = rng.random(d) >= 0.01
    c[~cv] = 0
    dim = {"id": (rng.permutation(d) + 1).astype(np.int64), "category": (c, cv), "weight": rng.random(d)}
    if w2:
        dim["weight2"] = (rng.normal(0, 1, d), rng.random(d) >= 0.03)
    return fact, dim


def _q(E, fact, dim, summ, by="category", temp_dir="tmp"):
    from vectra_gb300.plan import tbl
    return (tbl(E, fact, batch_rows=len(fact["key"])).left_join(tbl(E, dim, batch_rows=len(dim["id"])),
                                                                {"key": "id"})
            .group_by(by).summarise(temp_dir=temp_dir, **summ).batches())


def _with_env(name, value, fn):
    prev = os.environ.get(name)
    os.environ[name] = value
    try:
        return fn()
    finally:
        if prev is None:
            del os.environ[name]
        else:
            os.environ[name] = prev


def test_compact_two_columns_and_full_entries_agree():
    import vectra_gb300
    from vectra_gb300.plan import col
    G, O = vectra_gb300.engine(0), OracleEngine()
    fact, dim = _tables(1)
    summ = {"s": ("sum", col("value") * col("weight")), "sr": ("sum", col("value") * col("weight"), True),
            "n": ("n",)}
    for td in (O.tmp, None):
        compact = _q(G, fact, dim, summ, temp_dir=td)
        full = _with_env("VGPU_PAY32", "1", lambda: _q(G, fact, dim, summ, temp_dir=td))
        cases.same_batches(compact, full)                 # bit for bit
        cases.same_batches(compact, _q(O, fact, dim, summ, temp_dir=td), rtol=1e-12, tol_cols=("s", "sr"))


def test_compact_one_column():
    import vectra_gb300
    G, O = vectra_gb300.engine(0), OracleEngine()
    fact, dim = _tables(2)
    summ = {"s": ("sum", "value", True), "m": ("mean", "value", True), "n": ("n",)}
    cases.same_batches(_q(G, fact, dim, summ), _q(O, fact, dim, summ), rtol=1e-12, tol_cols=("s", "m"))


def test_full_entries_two_doubles():
    import vectra_gb300
    from vectra_gb300.plan import col
    G, O = vectra_gb300.engine(0), OracleEngine()
    fact, dim = _tables(3, w2=True)
    fact["g"] = (fact["key"] % 97).astype(np.int64)
    summ = {"s": ("sum", col("weight") * col("weight2")), "mx": ("max", "weight2", True), "n": ("n",)}
    cases.same_batches(_q(G, fact, dim, summ, by="g"), _q(O, fact, dim, summ, by="g"), rtol=1e-12,
                       tol_cols=("s",))


def test_full_entries_wide_int_column():
    import vectra_gb300
    from vectra_gb300.plan import col
    G, O = vectra_gb300.engine(0), OracleEngine()
    fact, dim = _tables(4, cat=lambda rng, d: rng.integers(0, 200, d).astype(np.int64) * (1 << 34))
    summ = {"s": ("sum", col("value") * col("weight"), True), "n": ("n",)}
    cases.same_batches(_q(G, fact, dim, summ), _q(O, fact, dim, summ), rtol=1e-12, tol_cols=("s",))


def test_slots_from_keys_after_compact_build():
    """With the run-time compiler switched off (VGPU_NO_JIT=1) the join is
    still built with compact entries, then the ahead-of-time kernels need
    its slot table, derived from the key column."""
    import vectra_gb300
    from vectra_gb300.plan import col
    G, O = vectra_gb300.engine(0), OracleEngine()
    fact, dim = _tables(5, n=60_000, d=9_000)
    summ = {"s": ("sum", col("value") * col("weight"), True), "n": ("n",)}
    got = _with_env("VGPU_NO_JIT", "1", lambda: _q(G, fact, dim, summ))
    cases.same_batches(got, _q(O, fact, dim, summ), rtol=1e-12, tol_cols=("s",))
