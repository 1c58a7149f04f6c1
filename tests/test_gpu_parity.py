"""libvgpu against the CPU oracle through the node C API, on the restated
reference tests, seeded random plans with ragged batch sizes and selection
vectors, and exactness checks of the double sums.

Bit-exact for filters, joins, keys, counts, integer sums, min/max and NA
semantics.  Double sums and means: libvgpu returns the correctly rounded
sum, the oracle (like the reference) a left-to-right sum, so those columns
are compared with a relative tolerance of 1e-12; test_exact_sums checks the
GPU against an exactly rounded oracle with no tolerance at all."""
import ctypes as C

import numpy as np
import pytest

import cases
from engines import exact_sum, exact_sum_products

pytestmark = pytest.mark.gpu

FP_COLS = ("s", "m", "sr", "mr", "sd", "p", "avg")
RTOL = 1e-12


@pytest.fixture(scope="module")
def G():
    from engines import gpu_engine
    return gpu_engine()


@pytest.mark.parametrize("case", cases.FILTER_CASES + cases.JOIN_CASES, ids=lambda f: f.__name__)
def test_filter_join_cases(case, G, oracle):
    cases.same_batches(case(G), case(oracle))


@pytest.mark.parametrize("temp_dir", ["tmp", None], ids=["sorted", "hash"])
@pytest.mark.parametrize("case", cases.GROUP_CASES, ids=lambda f: f.__name__)
def test_group_cases(case, temp_dir, G, oracle):
    td = None if temp_dir is None else oracle.tmp
    cases.same_batches(case(G, td), case(oracle, td), rtol=RTOL, tol_cols=FP_COLS)


@pytest.mark.parametrize("n,batch", cases.RAGGED)
@pytest.mark.parametrize("sel_mode", [0, 1])
def test_random_filter(n, batch, sel_mode, G, oracle):
    cases.same_batches(cases.r_filter(G, n, n, batch, sel_mode), cases.r_filter(oracle, n, n, batch, sel_mode))


@pytest.mark.parametrize("n,batch", cases.RAGGED)
@pytest.mark.parametrize("sel_mode", [0, 1])
@pytest.mark.parametrize("temp_dir", ["tmp", None], ids=["sorted", "hash"])
def test_random_group(n, batch, sel_mode, temp_dir, G, oracle):
    td = None if temp_dir is None else oracle.tmp
    cases.same_batches(cases.r_group(G, n + 1, n, batch, sel_mode, td),
                       cases.r_group(oracle, n + 1, n, batch, sel_mode, td), rtol=RTOL, tol_cols=FP_COLS)


@pytest.mark.parametrize("kind", ["inner_join", "left_join", "semi_join", "anti_join", "full_join"])
@pytest.mark.parametrize("n,batch", [(0, 32), (33, 32), (500, 64), (5000, 1024)])
def test_random_join(kind, n, batch, G, oracle):
    cases.same_batches(cases.r_join(G, n + 3, n, batch, kind), cases.r_join(oracle, n + 3, n, batch, kind))


@pytest.mark.parametrize("kind", ["inner_join", "left_join", "semi_join", "anti_join", "full_join"])
@pytest.mark.parametrize("n,batch", [(33, 32), (5000, 1024)])
def test_random_join_sparse_keys(kind, n, batch, G, oracle):
    """Keys spread over a wide range: hashed join tables."""
    sp = 1_000_003
    cases.same_batches(cases.r_join(G, n + 5, n, batch, kind, sp), cases.r_join(oracle, n + 5, n, batch, kind, sp))


def test_high_cardinality_groups(G, oracle):
    """More groups than any shared-memory cache: exercises the global table,
    spill and growth (rehash) paths."""
    rng = np.random.default_rng(5)
    n = 300_000
    t = {"k": rng.integers(0, 120_000, n), "x": rng.normal(0, 1, n), "y": rng.integers(-50, 50, n)}
    from vectra_gb300.plan import tbl
    a = tbl(G, t, batch_rows=65536).group_by("k").summarise(temp_dir=oracle.tmp, s=("sum", "x"), n=("n",),
                                                               lo=("min", "y"), hi=("max", "y")).batches()
    b = tbl(oracle, t, batch_rows=65536).group_by("k").summarise(temp_dir=oracle.tmp, s=("sum", "x"), n=("n",),
                                                                    lo=("min", "y"), hi=("max", "y")).batches()
    cases.same_batches(a, b, rtol=RTOL, tol_cols=FP_COLS)


def test_exact_sums(G):
    """Every double sum is the exactly rounded sum (no tolerance): wide
    exponent range, cancellation, subnormals, one group per pattern."""
    from vectra_gb300.plan import tbl
    rng = np.random.default_rng(11)
    groups, xs = [], []
    patterns = [
        rng.normal(0, 1, 5000),
        rng.lognormal(0, 2, 5000),
        np.concatenate([rng.normal(0, 1e300, 10), rng.normal(0, 1e-300, 10), [1e308, -1e308, 3.0]]),
        np.concatenate([[1e16, 1.0, -1e16] * 50, rng.normal(0, 1, 7)]),
        rng.normal(0, 1, 3000) * 10.0 ** rng.integers(-30, 30, 3000),
        np.array([5e-324, 5e-324, -1e-320, 2.2250738585072014e-308]),
        np.array([0.1] * 10),
    ]
    for g, p in enumerate(patterns):
        groups.append(np.full(len(p), g))
        xs.append(p)
    t = {"g": np.concatenate(groups), "x": np.concatenate(xs)}
    out = tbl(G, t, batch_rows=1024).group_by("g").summarise(temp_dir="tmp", s=("sum", "x"),
                                                             m=("mean", "x")).collect()
    for g, p in enumerate(patterns):
        want = exact_sum(p)
        got = out["s"][0][g]
        assert got == want, (g, got, want)
        assert out["m"][0][g] == want / len(p)


def test_join_agg_exact(G):
    """sum(value * weight) through left_join -> projection -> group_agg is
    the exactly rounded sum of the rounded products."""
    from vectra_gb300.plan import tbl, col
    rng = np.random.default_rng(3)
    nf, nd = 200_000, 5000
    ids = rng.permutation(nd) + 1
    fk = rng.integers(1, nd + 1, nf)
    fv = rng.lognormal(0, 1, nf)
    cat = rng.integers(0, 8, nd)
    w = rng.random(nd)
    out = (tbl(G, {"key": fk, "value": fv}, batch_rows=1 << 16)
           .left_join(tbl(G, {"id": ids, "category": cat, "weight": w}), {"key": "id"})
           .group_by("category").summarise(temp_dir="tmp", s=("sum", col("value") * col("weight")),
                                           n=("n",)).collect())
    pos = np.empty(nd + 1, np.int64)
    pos[ids] = np.arange(nd)
    c = cat[pos[fk]]
    ww = w[pos[fk]]
    for g in range(8):
        m = c == g
        assert out["category"][0][g] == g
        assert out["n"][0][g] == m.sum()
        assert out["s"][0][g] == exact_sum_products(fv[m], ww[m])


def test_join_agg_exact_wide_range(G):
    """The same plan with values spread over 600 decimal orders: most rows
    fall outside their CTA's digit window, are marked for the replay kernel
    and reach the global table there.  Every sum is still the exactly
    rounded sum of the rounded products, every mean that sum over the
    valid rows, every n() exact -- with and without na.rm."""
    from vectra_gb300.plan import tbl, col
    rng = np.random.default_rng(17)
    nf, nd = 300_000, 7000
    ids = rng.permutation(nd) + 1
    fk = rng.integers(1, nd + 1, nf)
    fv = rng.normal(0, 1, nf) * 10.0 ** rng.integers(-300, 300, nf)
    cat = rng.integers(0, 12, nd)
    w = rng.uniform(0.5, 2.0, nd)
    pos = np.empty(nd + 1, np.int64)
    pos[ids] = np.arange(nd)
    c = cat[pos[fk]]
    ww = w[pos[fk]]
    fvv = ~((c < 6) & (rng.random(nf) < 0.02))        # NA values in half of the groups
    fv[~fvv] = 0.0
    fact = {"key": fk, "value": (fv, fvv)}
    dim = {"id": ids, "category": cat, "weight": w}
    for na_rm in (True, False):
        out = (tbl(G, fact, batch_rows=1 << 17)
               .left_join(tbl(G, dim), {"key": "id"})
               .group_by("category").summarise(temp_dir="tmp", s=("sum", col("value") * col("weight"), na_rm),
                                               m=("mean", col("value") * col("weight"), na_rm),
                                               n=("n",)).collect())
        for g in range(12):
            m = c == g
            assert out["category"][0][g] == g
            assert out["n"][0][g] == m.sum()
            ok = m & fvv
            if not na_rm and (m & ~fvv).any():
                assert not out["s"][1][g] and not out["m"][1][g]
                continue
            want = exact_sum_products(fv[ok], ww[ok])
            assert out["s"][0][g] == want, (g, out["s"][0][g], want)
            assert out["m"][0][g] == want / ok.sum()


def test_specialised_kernel_ran(G):
    """The group cases above ran through the run-time specialised kernel."""
    import vectra_gb300
    lib = vectra_gb300.load()
    lib.vgk_jit_compiles.restype = C.c_ulonglong
    cases.ja_join_agg(G, "tmp")
    assert lib.vgk_jit_compiles() > 0


def test_unsupported_is_an_error(G):
    """No silent CPU fallback: a sum over a string column is rejected
    explicitly."""
    from vectra_gb300.plan import EngineError
    from engines import make_oracle_source
    from vectra_gb300.plan import Tbl
    src = make_oracle_source({"s": np.array(["a", "b"], dtype=object), "x": np.array([1.0, 2.0])})
    with pytest.raises(EngineError):
        Tbl(G, src).group_by("x").summarise(t=("sum", "s")).batches()


def test_mapped_host_source(G, oracle):
    """VGPU_SRC_MAPPED: page-locked host columns read in place by the
    kernels give the same result as the copied path; unpinned memory is
    refused at creation."""
    torch = pytest.importorskip("torch")
    from vectra_gb300 import abi
    from vectra_gb300.plan import Tbl, tbl, col
    rng = np.random.default_rng(21)
    nf, nd = 50_000, 700
    ids = rng.permutation(nd) + 1
    fact = {"key": rng.integers(1, nd + 20, nf), "value": rng.lognormal(0, 1, nf)}
    dim = {"id": ids, "category": rng.integers(0, 9, nd), "weight": rng.random(nd)}
    fvalid = rng.random(nf) > 0.03

    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        return t

    def padded_bits(mask):
        bits = abi.validity_from_mask(mask)
        out = np.zeros(((len(bits) + 3) // 4) * 4, np.uint8)
        out[:len(bits)] = bits
        return out

    keep = []

    def mapped(table, n, valid=None):
        cols = {}
        for name, v in table.items():
            tv = pinned(v)
            tm = pinned(padded_bits(valid)) if (valid is not None and name == "value") else None
            keep.extend([tv, tm])
            cols[name] = (tv.data_ptr(), tm.data_ptr() if tm is not None else 0,
                          abi.VEC_DOUBLE if v.dtype == np.float64 else abi.VEC_INT64, n)
        names = list(cols)
        data = (C.c_void_p * len(names))(*[cols[k][0] for k in names])
        val = (C.c_void_p * len(names))(*[cols[k][1] or None for k in names])
        types = (C.c_int * len(names))(*[cols[k][2] for k in names])
        cn = (C.c_char_p * len(names))(*[k.encode() for k in names])
        p = G.lib.vgpu_table_source_create(len(names), cn, types, data, val, n, 8192, 4)
        return G.check(p, "mapped source")

    def query(fsrc, dsrc):
        return (Tbl(G, fsrc).left_join(Tbl(G, dsrc), {"key": "id"}).group_by("category")
                .summarise(temp_dir="tmp", s=("sum", col("value") * col("weight")), n=("n",)).collect())

    got = query(mapped(fact, nf, fvalid), mapped(dim, nd))
    f2 = dict(fact)
    f2["value"] = (fact["value"], fvalid)
    want = (tbl(oracle, f2, batch_rows=8192).left_join(tbl(oracle, dim), {"key": "id"}).group_by("category")
            .summarise(temp_dir=oracle.tmp, s=("sum", col("value") * col("weight")), n=("n",)).collect())
    for k in want:
        assert np.array_equal(got[k][1], want[k][1]), k
        m = want[k][1]
        if k == "s":
            np.testing.assert_allclose(got[k][0][m], want[k][0][m], rtol=RTOL)
        else:
            assert np.array_equal(got[k][0][m], want[k][0][m]), k
    # ordinary (pageable) host memory is refused for in-place reads
    plain = np.arange(10, dtype=np.int64)
    cn = (C.c_char_p * 1)(b"k")
    p = G.lib.vgpu_table_source_create(1, cn, (C.c_int * 1)(abi.VEC_INT64), (C.c_void_p * 1)(plain.ctypes.data),
                                       None, 10, 32, 4)
    assert not p
    assert b"page-locked" in G.lib.vgpu_last_error()
