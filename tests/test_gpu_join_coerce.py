"""LEFT joins of an int64 key against a double key with repeated build keys:
the one place where libvgpu keeps the intended join semantics instead of
the reference's result.

The reference walks a key's chain of build rows comparing the probe column
before its coercion to double (src/join.c:137-150, called at 408-410), so
for an int64 probe value v only the first (highest) matching build row is
emitted -- except v = 0, whose bits equal those of +0.0.  libvgpu emits
every matching build row, as an inner join and a join on equal key types
both do.  The oracle reproduces the reference by default and gives the
intended rows with its quirk switched off; both are checked here, on the
join node itself and under a fused group-by.
"""
import numpy as np
import pytest

import cases
from engines import OracleEngine, port_lib

pytestmark = pytest.mark.gpu


def _tables(seed):
    rng = np.random.default_rng(seed)
    n, d = 5000, 300
    left = {"k": rng.integers(-3, d + 3, n).astype(np.int64), "x": rng.normal(0, 1, n)}
    kb = rng.integers(-2, d, d * 2).astype(np.float64)
    kb[:5] = [0.0, -0.0, 0.0, 7.0, 7.0]           # signed zeros and repeated keys
    right = {"k": (kb, rng.random(len(kb)) > 0.05), "y": rng.normal(0, 1, len(kb))}
    return left, right


def _join(E, left, right):
    from cases import tbl
    return tbl(E, left, batch_rows=1024).left_join(tbl(E, right, batch_rows=2 * 300), "k").batches()


def _agg(E, left, right):
    from cases import tbl
    from vectra_gb300.plan import col
    return (tbl(E, left, batch_rows=1024).left_join(tbl(E, right, batch_rows=600), "k").group_by("k")
            .summarise(temp_dir="tmp", s=("sum", col("x") * col("y"), True), n=("n",)).batches())


def _oracle(fn, left, right, quirk):
    port_lib().orc_set_join_quirk(1 if quirk else 0)
    try:
        return fn(OracleEngine(), left, right)
    finally:
        port_lib().orc_set_join_quirk(1)


@pytest.mark.parametrize("seed", [1, 2])
def test_coerced_left_join_keeps_every_match(seed):
    import vectra_gb300
    G = vectra_gb300.engine(0)
    left, right = _tables(seed)
    got = _join(G, left, right)
    cases.same_batches(got, _oracle(_join, left, right, quirk=False))
    ref_rows = sum(len(b["k"][0]) for b in _oracle(_join, left, right, quirk=True))
    assert sum(len(b["k"][0]) for b in got) > ref_rows       # the reference drops repeated matches
    gagg = _agg(G, left, right)
    cases.same_batches(gagg, _oracle(_agg, left, right, quirk=False), rtol=1e-12, tol_cols=("s",))
