"""The postfix programs of general predicates (compile.c, vg_compile_prog)
on the CPU: random predicates that do not fold into range terms (OR,
arithmetic on columns, negated disjunctions, is.na of an expression) are
compiled, the program is run row by row as the filter kernel runs it
(run_prog in k_filter.cu: int64 arithmetic wrapping with C division, NA on
an integer division by zero, IEEE double arithmetic with fmod, a NaN
comparing equal, R's three-valued AND / OR), and the rows it keeps must be
exactly the rows the CPU oracle's filter keeps (src/expr.c:91-281,
src/scalar_ops.c:11-203).  Likewise the values the fused kernels compute
(vg_compile_value: one operand, or two with one arithmetic operator, after
the reference's type promotion) against the oracle's projection."""
import ctypes as C
import struct

import numpy as np
import pytest

from vectra_gb300 import abi
from vectra_gb300.plan import col, is_na, lit, tbl

MAX_INSNS = 48
(COL_I64, COL_F64, COL_BOOL, LIT_I64, LIT_F64, LIT_BOOL, LIT_NA, I2F, ARITH_I64, ARITH_F64, CMP_I64, CMP_F64,
 AND, OR, NOT, IS_NA, NEG_I64, NEG_F64) = range(1, 19)


class Insn(C.Structure):
    _fields_ = [("op", C.c_int32), ("a", C.c_int32), ("imm", C.c_int64)]


class Prog(C.Structure):
    _fields_ = [("n", C.c_int32), ("result_type", C.c_int32), ("max_depth", C.c_int32), ("pad", C.c_int32),
                ("insn", Insn * MAX_INSNS)]


MAPFN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_char_p, C.POINTER(C.c_int))
M64 = (1 << 64) - 1


def s64(u):
    u &= M64
    return u - (1 << 64) if u >> 63 else u


def f2b(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def b2f(b):
    return struct.unpack("<d", struct.pack("<Q", b & M64))[0]


def arith_i64(a, b, op):
    if op == "+": return s64(a + b), True
    if op == "-": return s64(a - b), True
    if op == "*": return s64(a * b), True
    if b == 0: return 0, False
    if b == -1: return (s64(-a), True) if op == "/" else (0, True)
    q = abs(a) // abs(b) * (1 if (a < 0) == (b < 0) else -1)          # C: truncation toward zero
    return (q, True) if op == "/" else (a - q * b, True)


def arith_f64(a, b, op):
    with np.errstate(all="ignore"):
        x, y = np.float64(a), np.float64(b)
        r = {"+": x + y, "-": x - y, "*": x * y, "/": x / y}.get(op)
        return float(np.fmod(x, y) if r is None else r)


def cmp(c, code):
    return [c == 0, c != 0, c < 0, c <= 0, c > 0, c >= 0][code]


def run(prog, cols, r):
    st = []
    for ins in prog.insn[:prog.n]:
        op = ins.op
        if op in (COL_I64, COL_F64, COL_BOOL):
            v, valid, ty = cols[ins.a]
            x = f2b(float(v[r])) if ty == abi.VEC_DOUBLE else int(v[r]) & M64   # the column's 64-bit payload
            if op == COL_F64 and ty != abi.VEC_DOUBLE:
                x = f2b(float(s64(x)))
            elif op == COL_BOOL:
                x = 1 if x else 0
            st.append([x, bool(valid[r])])
        elif op in (LIT_I64, LIT_F64, LIT_BOOL):
            st.append([ins.imm & M64 if op == LIT_F64 else ins.imm, True])
        elif op == LIT_NA:
            st.append([0, False])
        elif op == I2F:
            st[-1][0] = f2b(float(s64(st[-1][0])))
        elif op in (ARITH_I64, ARITH_F64, CMP_I64, CMP_F64, AND, OR):
            b, a = st.pop(), st.pop()
            ok = a[1] and b[1]
            if op == ARITH_I64:
                v, ok2 = arith_i64(s64(a[0]), s64(b[0]), chr(ins.a)) if ok else (0, ok)
                st.append([v, ok and ok2])
            elif op == ARITH_F64:
                st.append([f2b(arith_f64(b2f(a[0]), b2f(b[0]), chr(ins.a))) if ok else 0, ok])
            elif op == CMP_I64:
                x, y = s64(a[0]), s64(b[0])
                st.append([int(cmp((x > y) - (x < y), ins.a)), ok])
            elif op == CMP_F64:
                x, y = b2f(a[0]), b2f(b[0])
                st.append([int(cmp((x > y) - (x < y), ins.a)), ok])
            elif op == AND:
                if (a[1] and not a[0]) or (b[1] and not b[0]): st.append([0, True])
                elif ok: st.append([1, True])
                else: st.append([0, False])
            else:
                if (a[1] and a[0]) or (b[1] and b[0]): st.append([1, True])
                elif ok: st.append([0, True])
                else: st.append([0, False])
        elif op == NOT:
            st[-1][0] = 0 if st[-1][0] else 1
        elif op == IS_NA:
            st[-1] = [0 if st[-1][1] else 1, True]
        elif op == NEG_I64:
            st[-1][0] = s64(-s64(st[-1][0]))
        elif op == NEG_F64:
            st[-1][0] ^= 1 << 63
        else:
            raise AssertionError("unknown instruction %d" % op)
    assert len(st) == 1
    return st[0]


def random_table(rng, n):
    i = rng.integers(-1000, 1000, n)
    i[rng.random(n) < 0.1] = 0
    d = rng.normal(0, 50, n).round(1)
    special = rng.random(n) < 0.1
    d[special] = rng.choice([0.0, -0.0, np.inf, -np.inf, np.nan, 7.0], int(special.sum()))
    return {"i": (i.astype(np.int64), rng.random(n) > 0.1), "d": (d, rng.random(n) > 0.1),
            "b": (rng.integers(0, 2, n).astype(np.uint8), rng.random(n) > 0.1), "rid": np.arange(n, dtype=np.int64)}


def random_value(rng, depth=0):
    r = rng.random()
    if depth > 1 or r < 0.45:
        k = rng.random()
        if k < 0.4: return col("i")
        if k < 0.7: return col("d")
        if k < 0.8: return lit(None)
        return lit(int(rng.integers(-5, 6))) if rng.random() < 0.5 else lit(float(rng.choice([0.0, 2.5, -7.0, 3.0])))
    op = ["+", "-", "*", "/", "%"][int(rng.integers(0, 5))]
    a, b = random_value(rng, depth + 1), random_value(rng, depth + 1)
    return {"+": a + b, "-": a - b, "*": a * b, "/": a / b, "%": a % b}[op] if rng.random() < 0.9 else -a


def random_bool(rng, depth=0):
    r = rng.random()
    if depth > 1 or r < 0.5:
        if rng.random() < 0.1:
            return col("b")
        if rng.random() < 0.1:
            return is_na(random_value(rng, 1))
        a, b = random_value(rng), random_value(rng)
        return [a.__lt__, a.__le__, a.__gt__, a.__ge__, a.eq, a.ne][int(rng.integers(0, 6))](b)
    a, b = random_bool(rng, depth + 1), random_bool(rng, depth + 1)
    e = (a | b) if rng.random() < 0.6 else (a & b)
    return ~e if rng.random() < 0.3 else e


@pytest.mark.parametrize("seed", range(6))
def test_programs_keep_the_oracles_rows(seed, oracle):
    import vectra_gb300
    lib = vectra_gb300.load()
    lib.vg_compile_prog.argtypes = [C.c_void_p, MAPFN, C.c_void_p, C.POINTER(Prog)]
    lib.vg_compile_prog.restype = C.c_int
    rng = np.random.default_rng(seed)
    t = random_table(rng, 300)
    names = ["i", "d", "b"]
    types = [abi.VEC_INT64, abi.VEC_DOUBLE, abi.VEC_BOOL]

    def colmap(ctx, name, ty):
        k = names.index(name.decode())
        ty[0] = types[k]
        return k
    cmap = MAPFN(colmap)
    cols = [(t[n][0], t[n][1], ty) for n, ty in zip(names, types)]
    ran = 0
    for _ in range(80):
        e = random_bool(rng)
        p = Prog()
        if lib.vg_compile_prog(C.cast(e.to_c(list(zip(names, types))), C.c_void_p), cmap, None,
                               C.byref(p)) != 0:
            continue
        ran += 1
        got = tbl(oracle, t).filter(e).collect()          # {} when no row passes
        want = got["rid"][0].tolist() if got else []
        keep = []
        for r in range(300):
            value, valid = run(p, cols, r)
            if valid and value:                 # TRUE keeps the row; FALSE and NA drop it
                keep.append(r)
        assert keep == want, repr(e.kw)
    assert ran > 60


# ---------------------------------------------------------------------------
# values the fused kernels compute (aggregate inputs, keys): vg_compile_value
# ---------------------------------------------------------------------------

SIDE_PROBE, SIDE_BUILD, SIDE_LIT, SIDE_NA = 0, 1, 2, 3


class Operand(C.Structure):
    _fields_ = [("side", C.c_int32), ("col", C.c_int32), ("type", C.c_int32), ("pad", C.c_int32),
                ("lit", C.c_int64)]


class Value(C.Structure):
    _fields_ = [("op", C.c_int32), ("type", C.c_int32), ("a", Operand), ("b", Operand)]


def operand(o, cols, r, want):
    """The operand's (payload, valid) for row r, coerced to type `want`."""
    if o.side == SIDE_NA:
        return 0, False
    if o.side == SIDE_LIT:
        x, ok, ty = o.lit & M64, True, o.type
    else:
        v, valid, ty = cols[o.col]
        x = f2b(float(v[r])) if ty == abi.VEC_DOUBLE else int(v[r]) & M64
        ok = bool(valid[r])
    if want == abi.VEC_DOUBLE and ty != abi.VEC_DOUBLE:
        x = f2b(float(s64(x)))
    return x, ok


def value_of(val, cols, r):
    a, oka = operand(val.a, cols, r, val.type)
    if val.op == 0:
        return a, oka
    b, okb = operand(val.b, cols, r, val.type)
    if not (oka and okb):
        return 0, False
    if val.type == abi.VEC_DOUBLE:
        return f2b(arith_f64(b2f(a), b2f(b), chr(val.op))), True
    v, ok = arith_i64(s64(a), s64(b), chr(val.op))
    return v & M64, ok


def random_operand(rng):
    k = rng.random()
    if k < 0.3: return col("i")
    if k < 0.6: return col("d")
    if k < 0.7: return col("b")
    if k < 0.75: return lit(None)
    return lit(int(rng.integers(-3, 4))) if rng.random() < 0.5 else lit(float(rng.choice([0.0, -0.0, 2.5, 1e300])))


@pytest.mark.parametrize("seed", range(4))
def test_values_match_the_oracles_projection(seed, oracle):
    import vectra_gb300
    lib = vectra_gb300.load()
    lib.vg_compile_value.argtypes = [C.c_void_p, MAPFN, C.c_void_p, C.c_int, C.POINTER(Value)]
    lib.vg_compile_value.restype = C.c_int
    rng = np.random.default_rng(50 + seed)
    t = random_table(rng, 200)
    names = ["i", "d", "b"]
    types = [abi.VEC_INT64, abi.VEC_DOUBLE, abi.VEC_BOOL]

    def colmap(ctx, name, ty):
        k = names.index(name.decode())
        ty[0] = types[k]
        return k
    cmap = MAPFN(colmap)
    cols = [(t[n][0], t[n][1], ty) for n, ty in zip(names, types)]
    done = 0
    for _ in range(60):
        a, b = random_operand(rng), random_operand(rng)
        op = ["+", "-", "*", "/", "%"][int(rng.integers(0, 5))]
        e = {"+": a + b, "-": a - b, "*": a * b, "/": a / b, "%": a % b}[op]
        v = Value()
        if lib.vg_compile_value(C.cast(e.to_c(list(zip(names, types))), C.c_void_p), cmap, None, SIDE_PROBE,
                                C.byref(v)) <= 0:
            continue
        done += 1
        got = tbl(oracle, {k: t[k] for k in names}).mutate(v=e).collect()["v"]
        for r in range(200):
            x, ok = value_of(v, cols, r)
            assert ok == bool(got[1][r]), (repr(e.kw), r)
            if not ok:
                continue
            want = float(got[0][r]) if v.type == abi.VEC_DOUBLE else int(got[0][r])
            if v.type == abi.VEC_DOUBLE:
                y = b2f(x)
                assert (y != y and want != want) or f2b(y) == f2b(want), (repr(e.kw), r, y, want)
            else:
                assert s64(x) == want, (repr(e.kw), r, s64(x), want)
    assert done > 40
