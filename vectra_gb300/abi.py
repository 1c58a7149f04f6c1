"""ctypes mirror of vectra's node contract (include/vectra_abi.h).

Structures here are layout-identical to the reference's src/types.h,
src/expr.h, src/group_agg.h and src/join.h.  Everything a node takes
ownership of (expression trees, name arrays, AggSpec / JoinKey arrays) is
allocated with the C library's malloc, because the nodes release it with
free(), exactly as the reference does.
"""
import ctypes as C
import ctypes.util

import numpy as np

VEC_INT64, VEC_DOUBLE, VEC_BOOL, VEC_STRING = 0, 1, 2, 3

(EXPR_COL_REF, EXPR_LIT_INT64, EXPR_LIT_DOUBLE, EXPR_LIT_BOOL, EXPR_LIT_STRING,
 EXPR_LIT_NA, EXPR_ARITH, EXPR_CMP, EXPR_BOOL, EXPR_IS_NA, EXPR_IF_ELSE,
 EXPR_CAST, EXPR_NEGATE, EXPR_NCHAR, EXPR_SUBSTR, EXPR_GREPL) = range(16)

AGG_COUNT, AGG_COUNT_STAR, AGG_SUM, AGG_MEAN, AGG_MIN, AGG_MAX = range(6)
JOIN_INNER, JOIN_LEFT, JOIN_FULL, JOIN_SEMI, JOIN_ANTI = range(5)

NP_OF = {VEC_INT64: np.int64, VEC_DOUBLE: np.float64, VEC_BOOL: np.uint8}


class StrBuf(C.Structure):
    # data is not NUL-terminated: a plain pointer (a c_char_p field would be
    # read up to a NUL, past the end of the buffer)
    _fields_ = [("offsets", C.POINTER(C.c_int64)), ("data", C.c_void_p), ("data_len", C.c_int64)]


class ArrBuf(C.Union):
    _fields_ = [("i64", C.POINTER(C.c_int64)), ("dbl", C.POINTER(C.c_double)),
                ("bln", C.POINTER(C.c_uint8)), ("str", StrBuf)]


class VecArray(C.Structure):
    _fields_ = [("type", C.c_int), ("length", C.c_int64), ("validity", C.POINTER(C.c_uint8)),
                ("owns_data", C.c_uint8), ("buf", ArrBuf)]


class VecBatch(C.Structure):
    _fields_ = [("n_rows", C.c_int64), ("n_cols", C.c_int), ("col_names", C.POINTER(C.c_char_p)),
                ("columns", C.POINTER(VecArray)), ("sel", C.POINTER(C.c_int32)), ("sel_n", C.c_int32)]


class VecSchema(C.Structure):
    _fields_ = [("n_cols", C.c_int), ("col_names", C.POINTER(C.c_char_p)),
                ("col_types", C.POINTER(C.c_int)), ("col_annotations", C.POINTER(C.c_char_p))]


class VecNode(C.Structure):
    pass


NEXT_FN = C.CFUNCTYPE(C.POINTER(VecBatch), C.POINTER(VecNode))
FREE_FN = C.CFUNCTYPE(None, C.POINTER(VecNode))
VecNode._fields_ = [("next_batch", NEXT_FN), ("free_node", FREE_FN),
                    ("output_schema", VecSchema), ("kind", C.c_char_p)]


class VecExpr(C.Structure):
    pass


VecExpr._fields_ = [("kind", C.c_int), ("result_type", C.c_int), ("col_name", C.c_void_p),
                    ("lit_i64", C.c_int64), ("lit_dbl", C.c_double), ("lit_bln", C.c_uint8),
                    ("lit_str", C.c_void_p), ("op", C.c_char), ("op2", C.c_char),
                    ("left", C.POINTER(VecExpr)), ("right", C.POINTER(VecExpr)),
                    ("operand", C.POINTER(VecExpr)), ("cond", C.POINTER(VecExpr)),
                    ("then_expr", C.POINTER(VecExpr)), ("else_expr", C.POINTER(VecExpr)),
                    ("cast_to", C.c_int)]


class AggSpec(C.Structure):
    _fields_ = [("output_name", C.c_void_p), ("kind", C.c_int), ("input_col", C.c_void_p),
                ("na_rm", C.c_int)]


class JoinKey(C.Structure):
    _fields_ = [("left_col", C.c_int), ("right_col", C.c_int)]


class ProjEntry(C.Structure):
    _fields_ = [("output_name", C.c_void_p), ("expr", C.POINTER(VecExpr))]


libc = C.CDLL(ctypes.util.find_library("c"))
libc.malloc.restype = C.c_void_p
libc.malloc.argtypes = [C.c_size_t]
libc.calloc.restype = C.c_void_p
libc.calloc.argtypes = [C.c_size_t, C.c_size_t]
libc.free.argtypes = [C.c_void_p]
libc.free.restype = None


def c_strdup(s):
    """A malloc'd copy of s (released with free() by whoever owns it)."""
    b = s.encode() if isinstance(s, str) else s
    p = libc.malloc(len(b) + 1)
    C.memmove(p, b + b"\0", len(b) + 1)
    return p


def c_array(ctype, items):
    """A malloc'd array of ctype filled from items."""
    n = max(len(items), 1)
    p = libc.calloc(n, C.sizeof(ctype))
    arr = C.cast(p, C.POINTER(ctype))
    for i, it in enumerate(items):
        arr[i] = it
    return arr


def c_string_array(names):
    p = libc.calloc(max(len(names), 1), C.sizeof(C.c_void_p))
    arr = C.cast(p, C.POINTER(C.c_void_p))
    for i, n in enumerate(names):
        arr[i] = c_strdup(n)
    return arr


def schema_of(node):
    s = node.contents.output_schema
    return [(s.col_names[i].decode(), s.col_types[i]) for i in range(s.n_cols)]


def validity_from_mask(valid):
    """Reference bitmap (bit i%8 of byte i/8) from a boolean numpy mask."""
    return np.packbits(np.asarray(valid, dtype=bool), bitorder="little")


def mask_from_validity(ptr, n):
    if not ptr or n == 0:
        return np.ones(n, dtype=bool)
    nb = (n + 7) // 8
    raw = np.ctypeslib.as_array(ptr, shape=(nb,)).copy()
    return np.unpackbits(raw, bitorder="little")[:n].astype(bool)


def batch_to_numpy(bp, logical=True):
    """{name: (values, valid)} for a VecBatch pointer; with logical=True the
    selection vector is applied (logical rows), else physical rows."""
    b = bp.contents
    n = b.n_rows
    sel = None
    if b.sel:
        sel = np.ctypeslib.as_array(b.sel, shape=(b.sel_n,)).copy() if b.sel_n > 0 else np.zeros(0, np.int32)
    out = {}
    for c in range(b.n_cols):
        a = b.columns[c]
        name = b.col_names[c].decode()
        if a.type == VEC_STRING:
            offs = np.ctypeslib.as_array(a.buf.str.offsets, shape=(n + 1,)).copy() if n else np.zeros(1, np.int64)
            data = C.string_at(a.buf.str.data, int(offs[-1])) if offs[-1] else b""
            vals = np.array([data[offs[i]:offs[i + 1]].decode("utf-8", "surrogateescape") for i in range(n)],
                            dtype=object)
        elif n == 0:
            vals = np.zeros(0, NP_OF[a.type])
        elif a.type == VEC_BOOL:
            vals = np.ctypeslib.as_array(a.buf.bln, shape=(n,)).copy()
        elif a.type == VEC_DOUBLE:
            vals = np.ctypeslib.as_array(a.buf.dbl, shape=(n,)).copy()
        else:
            vals = np.ctypeslib.as_array(a.buf.i64, shape=(n,)).copy()
        valid = mask_from_validity(a.validity, n)
        if logical and sel is not None:
            vals, valid = vals[sel], valid[sel]
        out[name] = (vals, valid)
    return out, sel


class SortKey(C.Structure):
    """src/sort.h:6-9"""
    _fields_ = [("col_index", C.c_int), ("descending", C.c_int)]
