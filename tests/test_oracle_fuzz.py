"""The CPU oracle against the reference engine compiled from its own
sources on randomly drawn plans: sizes (empty, one row, warp and batch
edges), batch sizes, selection vectors, hash and sorted group paths, every
join kind on direct-range and scattered keys, join -> group_by plans
with NA and repeated build keys, and plans over string columns (filters,
group keys, join keys, sorts).  Bit-exact, except double sums and means
(relative 1e-12: the reference sums in row order).  Runs where the
reference checkout exists, like test_oracle_vs_ref.py."""
import numpy as np
import pytest

import cases
from vectra_gb300.plan import col, tbl

FP = ("mi", "hi", "s", "m", "sr", "mr")


def _basic_case(rng):
    seed = int(rng.integers(0, 1 << 30))
    n = int(rng.choice([0, 1, 2, 7, 31, 64, 100, 333, 1000, 4097]))
    batch = int(rng.choice([1, 3, 32, 100, 1024]))
    kind = int(rng.integers(0, 3))
    if kind == 0:
        sm = int(rng.integers(0, 2))
        return lambda E: cases.r_filter(E, seed, n, batch, sm)
    if kind == 1:
        sm, td = int(rng.integers(0, 2)), bool(rng.integers(0, 2))
        return lambda E: cases.r_group(E, seed, n, batch, sm, E.tmp if td else None)
    jk = ["inner_join", "left_join", "semi_join", "anti_join", "full_join"][int(rng.integers(0, 5))]
    sp = int(rng.choice([1, 1000003]))
    return lambda E: cases.r_join(E, seed, n, batch, jk, sp)


@pytest.mark.parametrize("master", range(8))
def test_random_plans(master, oracle, ref):
    rng = np.random.default_rng(1000 + master)
    for _ in range(50):
        q = _basic_case(rng)
        cases.same_batches(q(oracle), q(ref), rtol=1e-12, tol_cols=FP)


def _join_agg_case(rng):
    nf = int(rng.choice([0, 1, 5, 100, 1000, 5000]))
    nd = int(rng.choice([1, 3, 50, 300]))
    dup, sparse = bool(rng.integers(0, 2)), bool(rng.integers(0, 2))
    ids = rng.integers(1, nd + 1, nd) if dup else rng.permutation(nd) + 1
    if sparse:
        ids = ids * 7_000_003 - 2_000_000_000
    idv = rng.random(nd) > (0.1 if rng.integers(0, 2) else 0.0)
    fk = (ids[rng.integers(0, nd, nf)] if nf else np.zeros(0, np.int64)) + (rng.random(nf) < 0.1)
    fact = {"key": (fk, rng.random(nf) > 0.05), "value": (rng.lognormal(0, 1, nf), rng.random(nf) > 0.05),
            "q": rng.integers(-5, 5, nf)}
    dim = {"id": (ids, idv), "cat": (rng.integers(0, int(rng.choice([2, 16, 300])), nd), rng.random(nd) > 0.05),
           "w": (rng.random(nd), rng.random(nd) > 0.05)}
    kind = ["left_join", "inner_join"][int(rng.integers(0, 2))]
    sorted_out, filt = bool(rng.integers(0, 2)), bool(rng.integers(0, 2))
    fb, db = int(rng.choice([1, 7, 100, 1024])), int(rng.choice([1, 13, 128]))

    def q(E):
        t = tbl(E, fact, batch_rows=fb)
        if filt:
            t = t.filter(col("q") > -3)
        return (getattr(t, kind)(tbl(E, dim, batch_rows=db), {"key": "id"}).group_by("cat")
                .summarise(temp_dir=E.tmp if sorted_out else None, s=("sum", col("value") * col("w")),
                           sr=("sum", col("value") * col("w"), True), m=("mean", "value", True),
                           lo=("min", "q"), n=("n",)).batches())
    return q


@pytest.mark.parametrize("master", range(4))
def test_random_join_then_group(master, oracle, ref):
    rng = np.random.default_rng(2000 + master)
    for _ in range(50):
        q = _join_agg_case(rng)
        cases.same_batches(q(oracle), q(ref), rtol=1e-12, tol_cols=FP)


def _string_case(rng):
    """Random plans over string columns: string filters, string group keys
    (both paths), string join keys of every kind, sorts by strings."""
    seed = int(rng.integers(0, 1 << 30))
    n = int(rng.choice([0, 1, 2, 31, 64, 333, 1000, 3000]))
    batch = int(rng.choice([1, 7, 32, 100, 1024]))
    kind = int(rng.integers(0, 4))
    if kind == 0:
        sm = int(rng.integers(0, 2))
        return lambda E: cases.r_string_filter(E, seed, n, batch, sm)
    if kind == 1:
        sm, td = int(rng.integers(0, 2)), bool(rng.integers(0, 2))
        return lambda E: cases.r_string_group(E, seed, n, batch, sm, getattr(E, "tmp", "tmp") if td else None)
    if kind == 2:
        jk = ["inner_join", "left_join", "semi_join", "anti_join", "full_join"][int(rng.integers(0, 5))]
        return lambda E: cases.r_string_join(E, seed, n, batch, jk)
    return lambda E: cases.r_string_sort(E, seed, n, batch)


@pytest.mark.parametrize("master", range(4))
def test_random_string_plans(master, oracle, ref):
    rng = np.random.default_rng(3000 + master)
    for _ in range(40):
        q = _string_case(rng)
        cases.same_batches(q(oracle), q(ref), rtol=1e-12, tol_cols=FP + ("s1",))
