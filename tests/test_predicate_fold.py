"""The predicate compiler (compile.c, vg_compile_pred) on the CPU: random
conjunctions of comparisons, negations and is.na over int64, double and
bool columns with boundary values (int64 extremes, 2^53 +- 1, fractional
and out-of-range double literals, +-0, +-Inf, NaN, NA) are folded into
range terms; the terms, evaluated row by row as the kernels evaluate them
(term_keep in k_groupby_dev.cuh, term_mask in k_jit_lib.cuh), must keep
exactly the rows the CPU oracle's filter keeps (the reference's Kleene
semantics, src/expr.c:91-281, src/scalar_ops.c:70-203)."""
import ctypes as C
import struct

import numpy as np
import pytest

from vectra_gb300 import abi
from vectra_gb300.plan import col, is_na, lit, tbl

MAX_TERMS = 12
RANGE, NOT_RANGE, IS_NA, NOT_NA, NONE = 0, 1, 2, 3, 4
DOM_DOUBLE = 1


class Term(C.Structure):
    _fields_ = [("col", C.c_int32), ("kind", C.c_int32), ("domain", C.c_int32), ("nan_keep", C.c_int32),
                ("lo", C.c_int64), ("hi", C.c_int64)]


class Pred(C.Structure):
    _fields_ = [("n_terms", C.c_int32), ("pad", C.c_int32), ("term", Term * MAX_TERMS)]


MAPFN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_char_p, C.POINTER(C.c_int))

I64_EDGES = [0, 1, -1, 2 ** 53 - 1, 2 ** 53, 2 ** 53 + 1, -(2 ** 53) - 1, 2 ** 63 - 1, -(2 ** 63), 2019, 2020, 2021]
F64_EDGES = [0.0, -0.0, 1.5, -1.5, 2019.5, 2020.0, 2 ** 53 + 0.0, 2.0 ** 63, -(2.0 ** 63), 1e300, -1e300,
             float("inf"), float("-inf"), float("nan"), 5e-324]


def ord_image(x):
    """The kernels' ordered image of a double (vg_ord in k_common.cuh)."""
    s = struct.unpack("<q", struct.pack("<d", x))[0]
    return s if s >= 0 else s ^ 0x7FFFFFFFFFFFFFFF


def keep_rows(pred, cols):
    """Rows the folded terms keep; cols: per column (values, valid, type)."""
    n = len(cols[0][0])
    out = []
    for r in range(n):
        keep = True
        for t in pred.term[:pred.n_terms]:
            v, valid, ty = cols[t.col]
            if t.kind == NONE:
                ok = False
            elif t.kind == IS_NA:
                ok = not valid[r]
            elif t.kind == NOT_NA:
                ok = bool(valid[r])
            elif not valid[r]:
                ok = False
            else:
                if t.domain == DOM_DOUBLE:
                    x = float(v[r])
                    if x != x:
                        ok = bool(t.nan_keep)
                        keep = keep and ok
                        continue
                    x = ord_image(x)
                else:
                    x = int(v[r])
                inside = t.lo <= x <= t.hi
                ok = inside if t.kind == RANGE else not inside
            keep = keep and ok
        if keep:
            out.append(r)
    return out


def random_table(rng, n):
    i = rng.choice(I64_EDGES, n) + rng.integers(-2, 3, n) * (rng.random(n) < 0.3)
    d = np.array(rng.choice(F64_EDGES, n), dtype=np.float64)
    mix = rng.random(n) < 0.4
    d[mix] = rng.normal(2020, 3, int(mix.sum())).round(1)
    b = rng.integers(0, 2, n).astype(np.uint8)
    return {"i": (i.astype(np.int64), rng.random(n) > 0.15), "d": (d, rng.random(n) > 0.15),
            "b": (b, rng.random(n) > 0.15), "rid": np.arange(n, dtype=np.int64)}


def random_literal(rng, ty):
    r = rng.random()
    if r < 0.05:
        return lit(None)
    if ty == abi.VEC_BOOL or r < 0.15:
        return lit(bool(rng.integers(0, 2))) if ty == abi.VEC_BOOL else lit(int(rng.choice(I64_EDGES)))
    if r < 0.55:
        v = int(rng.choice(I64_EDGES)) + int(rng.integers(-1, 2))
        return lit(min(max(v, -(2 ** 63)), 2 ** 63 - 1))
    return lit(float(rng.choice(F64_EDGES)) if rng.random() < 0.6 else float(rng.normal(2020, 5)))


def random_term(rng):
    name = ["i", "d", "b"][int(rng.integers(0, 3))]
    ty = {"i": abi.VEC_INT64, "d": abi.VEC_DOUBLE, "b": abi.VEC_BOOL}[name]
    c = col(name)
    k = rng.random()
    if k < 0.1:
        e = is_na(c)
    elif k < 0.2 and name == "b":
        e = c
    else:
        L = random_literal(rng, ty)
        op = ["<", "<=", ">", ">=", "==", "!="][int(rng.integers(0, 6))]
        e = {"<": c.__lt__, "<=": c.__le__, ">": c.__gt__, ">=": c.__ge__, "==": c.eq, "!=": c.ne}[op](L)
    return ~e if rng.random() < 0.25 else e


@pytest.mark.parametrize("seed", range(6))
def test_folded_terms_keep_the_oracles_rows(seed, oracle):
    import vectra_gb300
    lib = vectra_gb300.load()
    lib.vg_compile_pred.argtypes = [C.c_void_p, MAPFN, C.c_void_p, C.POINTER(Pred)]
    lib.vg_compile_pred.restype = C.c_int
    rng = np.random.default_rng(seed)
    t = random_table(rng, 400)
    names = ["i", "d", "b"]
    types = [abi.VEC_INT64, abi.VEC_DOUBLE, abi.VEC_BOOL]
    schema = list(zip(names, types))

    def colmap(ctx, name, ty):
        k = names.index(name.decode())
        ty[0] = types[k]
        return k
    cmap = MAPFN(colmap)
    cols = [(t[n][0], t[n][1], ty) for n, ty in zip(names, types)]
    folded = 0
    for _ in range(120):
        e = random_term(rng)
        for _ in range(int(rng.integers(0, 3))):
            e = e & random_term(rng)
        p = Pred()
        rc = lib.vg_compile_pred(C.cast(e.to_c(schema), C.c_void_p), cmap, None, C.byref(p))
        if rc <= 0:
            continue                     # not a conjunction of range terms: a program instead
        folded += 1
        got = tbl(oracle, t).filter(e).collect()          # {} when no row passes
        want = got["rid"][0].tolist() if got else []
        assert keep_rows(p, cols) == want, (repr(e.kw), [(x.col, x.kind, x.domain, x.nan_keep, x.lo, x.hi)
                                                        for x in p.term[:p.n_terms]])
    assert folded > 60
