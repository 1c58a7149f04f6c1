"""The CPU oracle (this repository's restatement) against the reference
engine compiled from its own sources, on the restated reference tests and
seeded random plans.  Bit-exact: the oracle accumulates in the same order.
Runs where the reference checkout exists (skipped elsewhere; the golden
fixtures in test_golden.py pin the oracle there)."""
import pytest

import cases


@pytest.mark.parametrize("case", cases.FILTER_CASES + cases.JOIN_CASES + cases.SORT_CASES, ids=lambda f: f.__name__)
def test_filter_join_cases(case, oracle, ref):
    cases.same_batches(case(oracle), case(ref))


@pytest.mark.parametrize("temp_dir", ["tmp", None], ids=["sorted", "hash"])
@pytest.mark.parametrize("case", cases.GROUP_CASES, ids=lambda f: f.__name__)
def test_group_cases(case, temp_dir, oracle, ref):
    td = None if temp_dir is None else ref.tmp
    cases.same_batches(case(oracle, td), case(ref, td))


@pytest.mark.parametrize("n,batch", cases.RAGGED)
@pytest.mark.parametrize("sel_mode", [0, 1])
def test_random_filter(n, batch, sel_mode, oracle, ref):
    cases.same_batches(cases.r_filter(oracle, n, n, batch, sel_mode),
                       cases.r_filter(ref, n, n, batch, sel_mode))


@pytest.mark.parametrize("n,batch", cases.RAGGED)
@pytest.mark.parametrize("temp_dir", ["tmp", None], ids=["sorted", "hash"])
def test_random_group(n, batch, temp_dir, oracle, ref):
    td = None if temp_dir is None else ref.tmp
    cases.same_batches(cases.r_group(oracle, n + 1, n, batch, 1, td),
                       cases.r_group(ref, n + 1, n, batch, 1, td))


@pytest.mark.parametrize("kind", ["inner_join", "left_join", "semi_join", "anti_join", "full_join"])
@pytest.mark.parametrize("n,batch", [(0, 32), (33, 32), (500, 64)])
def test_random_join(kind, n, batch, oracle, ref):
    cases.same_batches(cases.r_join(oracle, n + 3, n, batch, kind), cases.r_join(ref, n + 3, n, batch, kind))


def test_join_chain_quirk(oracle, ref):
    """LEFT join, int64 probe keys against double build keys with duplicate
    build rows: the reference's chain walk compares the uncoerced probe
    column (src/join.c:408-410), so only the first match survives (except
    key 0).  The oracle reproduces it by default."""
    from cases import T, tbl
    l = T(k=[0, 1, 2, 3])
    r = T(k=[0.0, 0.0, 1.0, 1.0, 2.0], y=[1.0, 2.0, 3.0, 4.0, 5.0])
    a = tbl(oracle, l).left_join(tbl(oracle, r), "k").batches()
    b = tbl(ref, l).left_join(tbl(ref, r), "k").batches()
    cases.same_batches(a, b)
    # key 0 keeps both matches, key 1 only the first (highest build row)
    assert len(a[0]["k"][0]) == 5
    from engines import port_lib
    port_lib().orc_set_join_quirk(0)
    try:
        c = tbl(oracle, l).left_join(tbl(oracle, r), "k").batches()
    finally:
        port_lib().orc_set_join_quirk(1)
    assert len(c[0]["k"][0]) == 6


@pytest.mark.parametrize("n,batch", cases.RAGGED)
def test_random_sort(n, batch, oracle, ref):
    cases.same_batches(cases.r_sort(oracle, n + 2, n, batch), cases.r_sort(ref, n + 2, n, batch))


@pytest.mark.parametrize("case", cases.STRING_FILTER_CASES, ids=lambda f: f.__name__)
def test_string_filter_cases(case, oracle, ref):
    """String predicates and projections: nchar, substr, grepl, string
    comparisons (src/expr.c:153-273, src/scalar_ops.c:78-107)."""
    cases.same_batches(case(oracle), case(ref))


@pytest.mark.parametrize("temp_dir", ["tmp", None], ids=["sorted", "hash"])
@pytest.mark.parametrize("case", cases.STRING_GROUP_CASES, ids=lambda f: f.__name__)
def test_string_group_cases(case, temp_dir, oracle, ref):
    td = None if temp_dir is None else ref.tmp
    cases.same_batches(case(oracle, td), case(ref, td))


@pytest.mark.parametrize("n,batch", [(0, 32), (33, 32), (700, 64), (5000, 1024)])
@pytest.mark.parametrize("sel_mode", [0, 1])
def test_random_string_filter(n, batch, sel_mode, oracle, ref):
    cases.same_batches(cases.r_string_filter(oracle, n + 5, n, batch, sel_mode),
                       cases.r_string_filter(ref, n + 5, n, batch, sel_mode))


@pytest.mark.parametrize("n,batch", [(33, 32), (3000, 256)])
@pytest.mark.parametrize("temp_dir", ["tmp", None], ids=["sorted", "hash"])
def test_random_string_group(n, batch, temp_dir, oracle, ref):
    td = None if temp_dir is None else ref.tmp
    cases.same_batches(cases.r_string_group(oracle, n + 9, n, batch, 1, td),
                       cases.r_string_group(ref, n + 9, n, batch, 1, td))


@pytest.mark.parametrize("case", cases.STRING_JOIN_CASES, ids=lambda f: f.__name__)
def test_string_join_cases(case, oracle, ref):
    cases.same_batches(case(oracle), case(ref))


@pytest.mark.parametrize("kind", ["inner_join", "left_join", "semi_join", "anti_join", "full_join"])
@pytest.mark.parametrize("n,batch", [(0, 32), (33, 32), (500, 64)])
def test_random_string_join(kind, n, batch, oracle, ref):
    cases.same_batches(cases.r_string_join(oracle, n + 3, n, batch, kind),
                       cases.r_string_join(ref, n + 3, n, batch, kind))


def test_string_sort_case(oracle, ref):
    cases.same_batches(cases.ss_string_keys(oracle), cases.ss_string_keys(ref))


@pytest.mark.parametrize("n,batch", [(0, 32), (33, 32), (2000, 256)])
def test_random_string_sort(n, batch, oracle, ref):
    cases.same_batches(cases.r_string_sort(oracle, n + 1, n, batch), cases.r_string_sort(ref, n + 1, n, batch))
