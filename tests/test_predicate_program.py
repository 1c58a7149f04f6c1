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
 AND, OR, NOT, IS_NA, NEG_I64, NEG_F64, COL_STR, LIT_STR, CMP_STR, NCHAR, SUBSTR, GREPL, F2I) = range(1, 26)
PROG_POOL = 512


class Insn(C.Structure):
    _fields_ = [("op", C.c_int32), ("a", C.c_int32), ("imm", C.c_int64)]


class Prog(C.Structure):
    _fields_ = [("n", C.c_int32), ("result_type", C.c_int32), ("max_depth", C.c_int32), ("pool_n", C.c_int32),
                ("insn", Insn * MAX_INSNS), ("pool", C.c_char * PROG_POOL)]


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


def f2i(x):
    """double -> int64 toward zero; NaN 0, out of range saturated."""
    if x != x: return 0
    if x >= 2.0 ** 63: return (1 << 63) - 1
    if x < -2.0 ** 63: return -(1 << 63)
    return int(x)


def run(prog, cols, r):
    st = []
    pool = bytes(prog.pool)
    for ins in prog.insn[:prog.n]:
        op = ins.op
        if op == COL_STR:                       # a string cell holds its bytes
            v, valid, ty = cols[ins.a]
            st.append([v[r].encode("utf-8", "surrogateescape"), bool(valid[r])])
        elif op == LIT_STR:
            st.append([pool[ins.imm:ins.imm + ins.a], True])
        elif op == CMP_STR:                     # memcmp, then the shorter first: bytes order
            b, a = st.pop(), st.pop()
            ok = a[1] and b[1]
            st.append([int(cmp((a[0] > b[0]) - (a[0] < b[0]), ins.a)) if ok else 0, ok])
        elif op == NCHAR:
            st[-1][0] = len(st[-1][0])
        elif op == SUBSTR:
            stop, start = st.pop(), st.pop()
            s = st[-1]
            ok = s[1] and start[1] and stop[1]
            b0 = max(s64(start[0] - 1), 0)
            e0 = min(s64(stop[0]), len(s[0]))
            st[-1] = [s[0][b0:e0] if ok and e0 > b0 else b"", ok]
        elif op == GREPL:
            st[-1][0] = int(st[-1][1] and pool[ins.imm:ins.imm + ins.a] in st[-1][0])
        elif op == F2I:
            st[-1][0] = f2i(b2f(st[-1][0])) & M64
        elif op in (COL_I64, COL_F64, COL_BOOL):
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


def random_string_bool(rng, depth=0):
    """Predicates over the string column s, the int64 column i and the
    double column d: comparisons with literals and between expressions,
    nchar, substr with column, literal and double bounds, grepl."""
    from vectra_gb300.plan import grepl, nchar, substr
    words = ["", "a", "ab", "abc", "b", "\u00e9", "ba", "zz"]

    def sval(k=0):
        r = rng.random()
        if k > 1 or r < 0.5:
            return col("s") if rng.random() < 0.8 else lit(words[int(rng.integers(0, len(words)))])
        lo = [col("i"), lit(int(rng.integers(-2, 4))), col("d"), lit(float(rng.choice([0.5, 2.9, -1.5])))]
        return substr(sval(k + 1), lo[int(rng.integers(0, 4))], lo[int(rng.integers(0, 4))])
    r = rng.random()
    if depth > 1 or r < 0.55:
        k = rng.random()
        if k < 0.45:
            a, b = sval(), sval()
            return [a.__lt__, a.__le__, a.__gt__, a.__ge__, a.eq, a.ne][int(rng.integers(0, 6))](b)
        if k < 0.65:
            return grepl(words[int(rng.integers(0, len(words)))], sval())
        if k < 0.85:
            return nchar(sval()) > lit(int(rng.integers(0, 4)))
        return is_na(sval())
    a, b = random_string_bool(rng, depth + 1), random_string_bool(rng, depth + 1)
    e = (a | b) if rng.random() < 0.6 else (a & b)
    return ~e if rng.random() < 0.3 else e


@pytest.mark.parametrize("seed", range(4))
def test_string_programs_keep_the_oracles_rows(seed, oracle):
    """String instructions (column views, pool literals, comparison, nchar,
    substr, grepl, double -> int64 bounds) as run_prog runs them, against
    the oracle's filter."""
    import vectra_gb300
    lib = vectra_gb300.load()
    lib.vg_compile_prog.argtypes = [C.c_void_p, MAPFN, C.c_void_p, C.POINTER(Prog)]
    lib.vg_compile_prog.restype = C.c_int
    rng = np.random.default_rng(70 + seed)
    n = 250
    words = ["", "a", "ab", "abc", "abcd", "b", "ba", "\u00e9t\u00e9", "zz", "azb", "bab"]
    t = {"s": ([words[k] for k in rng.integers(0, len(words), n)], rng.random(n) > 0.1),
         "i": (rng.integers(-1, 5, n).astype(np.int64), rng.random(n) > 0.1),
         "d": (rng.choice([0.5, 1.0, 2.7, -3.2, 4.0], n), rng.random(n) > 0.1),
         "rid": np.arange(n, dtype=np.int64)}
    names = ["s", "i", "d"]
    types = [abi.VEC_STRING, abi.VEC_INT64, abi.VEC_DOUBLE]

    def colmap(ctx, name, ty):
        k = names.index(name.decode())
        ty[0] = types[k]
        return k
    cmap = MAPFN(colmap)
    cols = [(t[nm][0], t[nm][1], ty) for nm, ty in zip(names, types)]
    ran = 0
    for _ in range(60):
        e = random_string_bool(rng)
        p = Prog()
        if lib.vg_compile_prog(C.cast(e.to_c(list(zip(names, types))), C.c_void_p), cmap, None,
                               C.byref(p)) != 0:
            continue
        ran += 1
        got = tbl(oracle, t).filter(e).collect()
        want = got["rid"][0].tolist() if got else []
        keep = [r for r in range(n) if (lambda v: v[1] and v[0])(run(p, cols, r))]
        assert keep == want, repr(e.kw)
    assert ran > 50


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


def test_string_program_limits_and_errors():
    """String literals go into the program's 512-byte pool (one that does
    not fit is an error, not a truncation); strings mixed with numbers in
    arithmetic or comparisons are the reference's coercion error
    (src/coerce.c:7-16)."""
    import vectra_gb300
    from vectra_gb300.plan import grepl, nchar, substr
    lib = vectra_gb300.load()
    lib.vg_compile_prog.argtypes = [C.c_void_p, MAPFN, C.c_void_p, C.POINTER(Prog)]
    lib.vg_compile_prog.restype = C.c_int
    lib.vg_compile_error.restype = C.c_char_p
    names = ["s", "i"]
    types = [abi.VEC_STRING, abi.VEC_INT64]

    def colmap(ctx, name, ty):
        k = names.index(name.decode())
        ty[0] = types[k]
        return k
    cmap = MAPFN(colmap)
    schema = list(zip(names, types))

    def compile_(e):
        p = Prog()
        rc = lib.vg_compile_prog(C.cast(e.to_c(schema), C.c_void_p), cmap, None, C.byref(p))
        return rc, p, lib.vg_compile_error().decode()
    rc, p, _ = compile_(col("s").eq("x" * 300) | grepl("y" * 200, col("s")))
    assert rc == 0 and p.pool_n == 500
    rc, _, msg = compile_(col("s").eq("x" * 300) | grepl("y" * 300, col("s")))
    assert rc != 0 and "too long" in msg
    for bad in (col("s") > col("i"), (col("s") + 1) > 0, col("s").eq(1)):
        rc, _, msg = compile_(bad)
        assert rc != 0 and "coerce" in msg, msg
    rc, _, msg = compile_(nchar(col("i")) > 1)
    assert rc != 0 and "nchar" in msg
    rc, _, msg = compile_(substr(col("s"), col("s"), 2).eq("a"))
    assert rc != 0 and "substr" in msg
