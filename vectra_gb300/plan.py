"""Plan building through the node C API, in the shape of vectra's R verbs.

    t = tbl(engine, {"station": ..., "temperature": ..., "year": ...}, batch_rows=100_000)
    out = (t.filter((col("temperature") > 30.0) & (col("year") >= 2020.0))
            .group_by("station")
            .summarise(avg=("mean", "temperature"), n=("n",))
            .collect())

Each verb calls the same C constructor the R bridge calls (src/r_bridge.c:
C_filter_node 880-888, C_project_node, C_group_agg_node 956-992,
C_join_node 1055-1093) and builds its arguments the same way:
- R numbers are doubles, so comparisons with Python floats use lit_double
  literals (R/expr.R:17-21); Python ints give lit_integer (int64) literals;
- summarise(s = sum(x * y)) inserts the hidden projection the R front end
  inserts (R/verbs.R:255-283, 741-747): every existing column passed
  through, then `.vectra_tmp_<name>` for each nested expression;
- group_by + summarise passes a temp_dir like the R bridge always does
  (src/r_bridge.c:990) unless temp_dir=None is given.

An Engine binds the verbs to one library: libvgpu here; the test suite binds
the same verbs to the reference engine and to the CPU oracle.
"""
import ctypes as C

import numpy as np

from . import abi
from .abi import (VecExpr, AggSpec, JoinKey, ProjEntry, VecBatch, VecNode,
                  c_strdup, c_array, c_string_array, libc)

# ---------------------------------------------------------------------------
# expressions
# ---------------------------------------------------------------------------


class Expr:
    def __init__(self, kind, **kw):
        self.kind = kind
        self.kw = kw

    # comparisons
    def _cmp(self, op, other):
        return Expr(abi.EXPR_CMP, op=op, left=self, right=wrap(other))

    def __gt__(self, o): return self._cmp(">", o)
    def __ge__(self, o): return self._cmp(">=", o)
    def __lt__(self, o): return self._cmp("<", o)
    def __le__(self, o): return self._cmp("<=", o)
    def eq(self, o): return self._cmp("==", o)
    def ne(self, o): return self._cmp("!=", o)

    # boolean
    def __and__(self, o): return Expr(abi.EXPR_BOOL, op="&", left=self, right=wrap(o))
    def __or__(self, o): return Expr(abi.EXPR_BOOL, op="|", left=self, right=wrap(o))
    def __invert__(self): return Expr(abi.EXPR_BOOL, op="!", operand=self)

    # arithmetic
    def _ar(self, op, o, rev=False):
        a, b = (wrap(o), self) if rev else (self, wrap(o))
        return Expr(abi.EXPR_ARITH, op=op, left=a, right=b)

    def __add__(self, o): return self._ar("+", o)
    def __sub__(self, o): return self._ar("-", o)
    def __mul__(self, o): return self._ar("*", o)
    def __truediv__(self, o): return self._ar("/", o)
    def __mod__(self, o): return self._ar("%", o)
    def __radd__(self, o): return self._ar("+", o, True)
    def __rsub__(self, o): return self._ar("-", o, True)
    def __rmul__(self, o): return self._ar("*", o, True)
    def __neg__(self): return Expr(abi.EXPR_NEGATE, operand=self)

    def cols(self):
        out = []
        if self.kind == abi.EXPR_COL_REF:
            out.append(self.kw["name"])
        for k in ("left", "right", "operand"):
            if k in self.kw:
                out += self.kw[k].cols()
        return out

    def result_type(self, schema):
        """Result type as the R bridge infers it (src/r_bridge.c:744-876)."""
        k = self.kind
        if k == abi.EXPR_COL_REF:
            return dict(schema).get(self.kw["name"], abi.VEC_DOUBLE)
        if k == abi.EXPR_LIT_INT64: return abi.VEC_INT64
        if k == abi.EXPR_LIT_DOUBLE: return abi.VEC_DOUBLE
        if k == abi.EXPR_LIT_BOOL: return abi.VEC_BOOL
        if k == abi.EXPR_LIT_NA: return self.kw.get("type", abi.VEC_DOUBLE)
        if k == abi.EXPR_ARITH:
            lt, rt = self.kw["left"].result_type(schema), self.kw["right"].result_type(schema)
            return abi.VEC_DOUBLE if abi.VEC_DOUBLE in (lt, rt) else abi.VEC_INT64
        if k in (abi.EXPR_CMP, abi.EXPR_BOOL, abi.EXPR_IS_NA, abi.EXPR_GREPL): return abi.VEC_BOOL
        if k == abi.EXPR_NEGATE: return self.kw["operand"].result_type(schema)
        if k == abi.EXPR_LIT_STRING or k == abi.EXPR_SUBSTR: return abi.VEC_STRING
        if k == abi.EXPR_NCHAR: return abi.VEC_INT64
        return abi.VEC_DOUBLE

    def to_c(self, schema):
        """A malloc'd VecExpr tree (the node takes ownership)."""
        p = libc.calloc(1, C.sizeof(VecExpr))
        e = C.cast(p, C.POINTER(VecExpr))
        x = e.contents
        x.kind = self.kind
        x.result_type = self.result_type(schema)
        kw = self.kw
        if self.kind == abi.EXPR_COL_REF:
            x.col_name = c_strdup(kw["name"])
        elif self.kind == abi.EXPR_LIT_INT64:
            x.lit_i64 = int(kw["value"])
        elif self.kind == abi.EXPR_LIT_DOUBLE:
            x.lit_dbl = float(kw["value"])
        elif self.kind == abi.EXPR_LIT_BOOL:
            x.lit_bln = 1 if kw["value"] else 0
        if "text" in kw:                       # string literal / grepl pattern
            x.lit_str = c_strdup(kw["text"])
        if "op" in kw:
            op = kw["op"]
            x.op = op[0].encode()
            x.op2 = (op[1] if len(op) > 1 else " ").encode()
        for k in ("left", "right", "operand"):
            if k in kw:
                setattr(x, k, kw[k].to_c(schema))
        return e


def col(name):
    return Expr(abi.EXPR_COL_REF, name=name)


def lit(v, na_type=abi.VEC_DOUBLE):
    if v is None:
        return Expr(abi.EXPR_LIT_NA, type=na_type)
    if isinstance(v, str):
        return Expr(abi.EXPR_LIT_STRING, text=v)
    if isinstance(v, (bool, np.bool_)):
        return Expr(abi.EXPR_LIT_BOOL, value=bool(v))
    if isinstance(v, (int, np.integer)):
        return Expr(abi.EXPR_LIT_INT64, value=int(v))
    return Expr(abi.EXPR_LIT_DOUBLE, value=float(v))


def wrap(v):
    return v if isinstance(v, Expr) else lit(v)


def is_na(e):
    return Expr(abi.EXPR_IS_NA, operand=wrap(e))


def nchar(e):
    """nchar(x): bytes of a string (src/expr.c:153-170)."""
    return Expr(abi.EXPR_NCHAR, operand=wrap(e))


def substr(e, start, stop):
    """substr(x, start, stop), 1-based, stop inclusive (src/expr.c:172-235)."""
    return Expr(abi.EXPR_SUBSTR, operand=wrap(e), left=wrap(start), right=wrap(stop))


def grepl(pattern, e):
    """grepl(pattern, x, fixed = TRUE) (src/expr.c:237-268)."""
    return Expr(abi.EXPR_GREPL, operand=wrap(e), text=pattern)


# ---------------------------------------------------------------------------
# engines
# ---------------------------------------------------------------------------


class EngineError(RuntimeError):
    pass


class Engine:
    """Binds the verbs to a library exporting the node constructors."""

    def __init__(self, lib, filter_fn, project_fn, group_agg_fn, join_fn, next_fn,
                 batch_free_fn, last_error_fn):
        self.lib = lib
        P = C.c_void_p
        self._filter = getattr(lib, filter_fn)
        self._filter.restype, self._filter.argtypes = P, [P, P]
        self._project = getattr(lib, project_fn)
        self._project.restype, self._project.argtypes = P, [P, C.c_int, P]
        self._agg = getattr(lib, group_agg_fn)
        self._agg.restype, self._agg.argtypes = P, [P, C.c_int, P, C.c_int, P, C.c_char_p]
        self._join = getattr(lib, join_fn)
        self._join.restype, self._join.argtypes = P, [P, P, C.c_int, C.c_int, P, C.c_char_p, C.c_char_p]
        self._next = getattr(lib, next_fn)
        self._next.restype, self._next.argtypes = C.POINTER(VecBatch), [P]
        self._bfree = getattr(lib, batch_free_fn)
        self._bfree.restype, self._bfree.argtypes = None, [C.POINTER(VecBatch)]
        self._err = getattr(lib, last_error_fn)
        self._err.restype, self._err.argtypes = C.c_char_p, []

    def error(self):
        m = self._err()
        return m.decode() if m else ""

    def check(self, p, what):
        if not p:
            raise EngineError("%s: %s" % (what, self.error()))
        return p

    # subclasses provide make_source(table, batch_rows, **opts) -> node pointer

    def sort(self, node, keys, temp_dir):
        """A sort node (arrange): keys = [(column index, descending)]."""
        f = getattr(self.lib, self.sort_fn)
        f.restype, f.argtypes = C.c_void_p, [C.c_void_p, C.c_int, C.c_void_p, C.c_char_p]
        ka = c_array(abi.SortKey, [abi.SortKey(c, 1 if d else 0) for c, d in keys])
        td = temp_dir.encode() if temp_dir is not None else None
        return self.check(f(node, len(keys), C.cast(ka, C.c_void_p), td), "sort")

    def make_scan(self, path, cols=None, scan_fn=None):
        """A .vtr scan node (scan_node_create through the library's guard);
        cols: file column indices, None = all."""
        f = getattr(self.lib, scan_fn or self.scan_fn)
        f.restype, f.argtypes = C.c_void_p, [C.c_char_p, C.c_void_p, C.c_int]
        idx = (C.c_int * len(cols))(*cols) if cols else None
        return self.check(f(path.encode(), idx, len(cols) if cols else 0), "scan")

    def filter(self, node, expr_ptr):
        return self.check(self._filter(node, C.cast(expr_ptr, C.c_void_p)), "filter")

    def project(self, node, entries):
        arr = c_array(ProjEntry, entries)
        return self.check(self._project(node, len(entries), C.cast(arr, C.c_void_p)), "project")

    def group_agg(self, node, keys, specs, temp_dir):
        kn = c_string_array(keys)
        sa = c_array(AggSpec, specs)
        td = temp_dir.encode() if temp_dir is not None else None
        return self.check(self._agg(node, len(keys), C.cast(kn, C.c_void_p), len(specs),
                                    C.cast(sa, C.c_void_p), td), "group_agg")

    def join(self, left, right, kind, keys, sx, sy):
        ka = c_array(JoinKey, [JoinKey(l, r) for l, r in keys])
        return self.check(self._join(left, right, kind, len(keys), C.cast(ka, C.c_void_p),
                                     sx.encode(), sy.encode()), "join")

    def next_batch(self, node):
        b = self._next(node)
        if not b:
            msg = self.error()
            if msg:
                raise EngineError("next_batch: " + msg)
            return None
        return b

    def free_batch(self, b):
        self._bfree(b)

    def free_node(self, node):
        n = C.cast(node, C.POINTER(VecNode))
        n.contents.free_node(n)


def _table_types(table):
    names, types, datas, valids = [], [], [], []
    n = None
    for name, v in table.items():
        if isinstance(v, tuple):
            vals, valid = v
        else:
            vals, valid = v, None
        vals = np.asarray(vals)
        if vals.dtype == np.float64:
            t = abi.VEC_DOUBLE
        elif vals.dtype == np.bool_ or vals.dtype == np.uint8:
            t, vals = abi.VEC_BOOL, vals.astype(np.uint8)
        elif vals.dtype.kind in "iu":
            t, vals = abi.VEC_INT64, vals.astype(np.int64)
        else:
            t = abi.VEC_STRING
        if n is None:
            n = len(vals)
        assert len(vals) == n, "columns must have equal length"
        names.append(name)
        types.append(t)
        datas.append(vals)
        valids.append(None if valid is None else np.asarray(valid, dtype=bool))
    return names, types, datas, valids, (n or 0)


class GpuEngine(Engine):
    """libvgpu."""

    def __init__(self, lib):
        super().__init__(lib, "vgpu_guard_filter", "vgpu_guard_project", "vgpu_guard_group_agg",
                         "vgpu_guard_join", "vgpu_guard_next_batch", "vgpu_batch_free",
                         "vgpu_last_error")
        self.scan_fn = "vgpu_guard_scan"
        self.sort_fn = "vgpu_guard_sort"
        lib.vgpu_table_source_create.restype = C.c_void_p
        lib.vgpu_table_source_create.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                 C.c_void_p, C.c_int64, C.c_int64, C.c_int]
        self._keep = []

    def make_source(self, table, batch_rows=None, device=False, borrow=False):
        """A table source node.  device=True: `table` maps names to
        (device_ptr, valid_device_ptr_or_0, type, n_rows) tuples."""
        if device:
            names = list(table.keys())
            n = None
            data = (C.c_void_p * len(names))()
            val = (C.c_void_p * len(names))()
            types = (C.c_int * len(names))()
            for i, nm in enumerate(names):
                dp, vp, t, rows = table[nm]
                data[i], val[i], types[i] = dp, (vp or None), t
                n = rows
            cn = (C.c_char_p * len(names))(*[s.encode() for s in names])
            p = self.lib.vgpu_table_source_create(len(names), cn, types, data, val, n,
                                                  batch_rows or n, 2)
            return self.check(p, "table source")
        names, types, datas, valids, n = _table_types(table)
        bufs = []
        data = (C.c_void_p * len(names))()
        val = (C.c_void_p * len(names))()
        for i, (d, v) in enumerate(zip(datas, valids)):
            d = np.ascontiguousarray(d)
            bufs.append(d)
            data[i] = d.ctypes.data
            if v is not None:
                bits = abi.validity_from_mask(v)
                bufs.append(bits)
                val[i] = bits.ctypes.data
        cn = (C.c_char_p * len(names))(*[s.encode() for s in names])
        ct = (C.c_int * len(names))(*types)
        br = batch_rows or max(32, ((n + 31) // 32) * 32)
        p = self.lib.vgpu_table_source_create(len(names), cn, ct, data, val, n, br, 1 if borrow else 0)
        if borrow:
            self._keep.append(bufs)
        return self.check(p, "table source")


# ---------------------------------------------------------------------------
# verbs
# ---------------------------------------------------------------------------


def tbl(engine, table, batch_rows=None, **opts):
    return Tbl(engine, engine.make_source(table, batch_rows, **opts))


def scan(engine, path, cols=None):
    """tbl(path) over a .vtr file: the engine's scan node."""
    return Tbl(engine, engine.make_scan(path, cols))


class Tbl:
    def __init__(self, engine, node):
        self.engine = engine
        self.node = node
        self.groups = None

    @property
    def schema(self):
        return abi.schema_of(C.cast(self.node, C.POINTER(VecNode)))

    def _take(self):
        n, self.node = self.node, None
        if n is None:
            raise RuntimeError("this plan was already consumed")
        return n

    def filter(self, expr):
        schema = self.schema
        return Tbl(self.engine, self.engine.filter(self._take(), expr.to_c(schema)))

    def arrange(self, *keys, temp_dir="<tempdir>"):
        """arrange(): keys are column names, or (name, True) for descending."""
        schema = [n for n, _ in self.schema]
        ks = []
        for k in keys:
            name, desc = (k, False) if isinstance(k, str) else k
            ks.append((schema.index(name), bool(desc)))
        return Tbl(self.engine, self.engine.sort(self._take(), ks, temp_dir))

    def select(self, *names):
        entries = [ProjEntry(c_strdup(n), None) for n in names]
        return Tbl(self.engine, self.engine.project(self._take(), entries))

    def mutate(self, **exprs):
        schema = self.schema
        entries = [ProjEntry(c_strdup(n), None) for n, _ in schema if n not in exprs]
        for name, e in exprs.items():
            entries.append(ProjEntry(c_strdup(name), wrap(e).to_c(schema)))
        return Tbl(self.engine, self.engine.project(self._take(), entries))

    def group_by(self, *keys):
        t = Tbl(self.engine, self._take())
        t.groups = list(keys)
        return t

    def summarise(self, temp_dir="<tempdir>", **aggs):
        """aggs: name=(fn, input[, na_rm]) with fn in n/count/sum/mean/min/max;
        input is a column name or an Expr (nested expressions get the hidden
        projection the R front end adds)."""
        kinds = {"n": abi.AGG_COUNT_STAR, "count": abi.AGG_COUNT, "sum": abi.AGG_SUM,
                 "mean": abi.AGG_MEAN, "min": abi.AGG_MIN, "max": abi.AGG_MAX}
        schema = self.schema
        specs, nested = [], {}
        for name, spec in aggs.items():
            fn = spec[0]
            kind = kinds[fn]
            if kind == abi.AGG_COUNT_STAR:
                specs.append((name, kind, None, 0))
                continue
            inp = spec[1]
            na_rm = int(bool(spec[2])) if len(spec) > 2 else 0
            if isinstance(inp, Expr) and inp.kind != abi.EXPR_COL_REF:
                tmp = ".vectra_tmp_" + name
                nested[tmp] = inp
                inp = tmp
            elif isinstance(inp, Expr):
                inp = inp.kw["name"]
            specs.append((name, kind, inp, na_rm))
        node = self._take()
        if nested:
            entries = [ProjEntry(c_strdup(n), None) for n, _ in schema]
            for tmp, e in nested.items():
                entries.append(ProjEntry(c_strdup(tmp), e.to_c(schema)))
            node = self.engine.project(node, entries)
        cspecs = [AggSpec(c_strdup(n), k, c_strdup(i) if i else None, r) for n, k, i, r in specs]
        keys = self.groups or []
        return Tbl(self.engine, self.engine.group_agg(node, keys, cspecs, temp_dir))

    def _join(self, other, kind, by, suffix):
        ls, rs = self.schema, other.schema
        if isinstance(by, str):
            by = {by: by}
        elif isinstance(by, (list, tuple)):
            by = {b: b for b in by}
        lnames = [n for n, _ in ls]
        rnames = [n for n, _ in rs]
        keys = [(lnames.index(l), rnames.index(r)) for l, r in by.items()]
        node = self.engine.join(self._take(), other._take(), kind, keys, suffix[0], suffix[1])
        return Tbl(self.engine, node)

    def inner_join(self, other, by, suffix=(".x", ".y")):
        return self._join(other, abi.JOIN_INNER, by, suffix)

    def left_join(self, other, by, suffix=(".x", ".y")):
        return self._join(other, abi.JOIN_LEFT, by, suffix)

    def full_join(self, other, by, suffix=(".x", ".y")):
        return self._join(other, abi.JOIN_FULL, by, suffix)

    def semi_join(self, other, by):
        return self._join(other, abi.JOIN_SEMI, by, (".x", ".y"))

    def anti_join(self, other, by):
        return self._join(other, abi.JOIN_ANTI, by, (".x", ".y"))

    def batches(self):
        """Pulls every batch: a list of {name: (values, valid)} over logical rows."""
        node = self._take()
        out = []
        try:
            while True:
                b = self.engine.next_batch(node)
                if not b:
                    break
                d, _ = abi.batch_to_numpy(b)
                out.append(d)
                self.engine.free_batch(b)
            # a finished node keeps answering NULL (src/group_agg.c:593-594)
            assert not self.engine.next_batch(node)
        finally:
            self.engine.free_node(node)
        return out

    def run(self):
        """Pulls every batch through the node API and frees it (the host
        batches a C caller receives), without converting to numpy: the
        number of logical rows produced."""
        node = self._take()
        rows = 0
        try:
            while True:
                b = self.engine.next_batch(node)
                if not b:
                    break
                bb = C.cast(b, C.POINTER(abi.VecBatch)).contents
                rows += bb.sel_n if bb.sel else bb.n_rows
                self.engine.free_batch(b)
        finally:
            self.engine.free_node(node)
        return rows

    def collect(self):
        """All logical rows: {name: (values, valid)}."""
        bs = self.batches()
        if not bs:
            return {}
        out = {}
        for name in bs[0]:
            vals = np.concatenate([b[name][0] for b in bs])
            valid = np.concatenate([b[name][1] for b in bs])
            out[name] = (vals, valid)
        return out
