""".vtr files: a writer of the format the reference's engine reads and
writes (src/vtr1.c:39-153, always version 3 with per-row-group statistics),
so that tables made in Python can be scanned by scan_node_create.

Layout (little-endian): "VTR1", u16 version (3), u16 n_cols, per column
{u16 name length, name, u8 type, u16 annotation length (0)}, u32 row
groups; per row group: u64 n_rows, per column {u8 has_stats, u64 min,
u64 max}, then per column the validity bitmap (bit i%8 of byte i/8) and
the values (int64 / double: 8 bytes each; bool: 1 byte; string: n+1 int64
offsets, u64 data length, data).

Statistics follow the reference writer's loop (src/vtr1.c:69-114): min and
max over the valid values in row order, replaced only by a strictly smaller
(larger) value, so a double NaN that comes first sticks and +-0 keep the
first zero's sign; int64 and double columns without a valid value have no
statistics; bool columns always have them (min = any false, max = any
true); string columns and empty row groups never.
"""
import struct

import numpy as np

from . import abi


def _col(v):
    """(values, valid mask or None, type) of a table column given as an
    array or (array, mask)."""
    if isinstance(v, tuple):
        vals, mask = v
    else:
        vals, mask = v, None
    if isinstance(vals, np.ndarray) and vals.dtype == np.float64:
        t = abi.VEC_DOUBLE
    elif isinstance(vals, np.ndarray) and vals.dtype == np.bool_:
        t = abi.VEC_BOOL
    elif isinstance(vals, np.ndarray) and vals.dtype.kind in "iu":
        t = abi.VEC_INT64
        vals = vals.astype(np.int64)
    else:
        t = abi.VEC_STRING
        vals = list(vals)
    n = len(vals)
    mask = np.ones(n, dtype=bool) if mask is None else np.asarray(mask, dtype=bool)
    return vals, mask, t


def _first_extreme(x, fn):
    """The reference writer's min (fn = np.min) / max over x in order."""
    if np.isnan(x[0]):
        return x[0]
    xs = x[~np.isnan(x)]
    m = fn(xs)
    return xs[np.argmax(xs == m)]


def _stats(vals, mask, t):
    n = len(mask)
    if t == abi.VEC_STRING or n == 0:
        return struct.pack("<BQQ", 0, 0, 0)
    if t == abi.VEC_BOOL:
        v = vals[mask]
        return struct.pack("<BQQ", 1, int((~v).any()), int(v.any()))
    v = vals[mask]
    if len(v) == 0:
        return struct.pack("<BQQ", 0, 0, 0)
    if t == abi.VEC_INT64:
        return struct.pack("<Bqq", 1, int(v.min()), int(v.max()))
    return struct.pack("<Bdd", 1, float(_first_extreme(v, np.min)), float(_first_extreme(v, np.max)))


def _column_bytes(vals, mask, t):
    out = [np.packbits(mask, bitorder="little").tobytes()]
    if t == abi.VEC_INT64:
        out.append(np.ascontiguousarray(vals, dtype="<i8").tobytes())
    elif t == abi.VEC_DOUBLE:
        out.append(np.ascontiguousarray(vals, dtype="<f8").tobytes())
    elif t == abi.VEC_BOOL:
        out.append(np.ascontiguousarray(vals, dtype=np.uint8).tobytes())
    else:
        enc = [b"" if s is None else str(s).encode() for s in vals]
        offs = np.zeros(len(enc) + 1, dtype="<i8")
        offs[1:] = np.cumsum([len(e) for e in enc])
        data = b"".join(enc)
        out += [offs.tobytes(), struct.pack("<Q", len(data)), data]
    return b"".join(out)


def write_vtr(path, table, batch_rows=100_000):
    """Writes `table` ({name: array or (array, valid mask)}; int64 / float64
    / bool arrays or lists of str) as one row group per batch_rows rows."""
    names = list(table)
    cols = [_col(table[n]) for n in names]
    n_rows = len(cols[0][1]) if cols else 0
    groups = [(lo, min(n_rows, lo + batch_rows)) for lo in range(0, n_rows, batch_rows)] if n_rows else []
    with open(path, "wb") as f:
        f.write(b"VTR1" + struct.pack("<HH", 3, len(names)))
        for name, (_, _, t) in zip(names, cols):
            nb = name.encode()
            f.write(struct.pack("<H", len(nb)) + nb + struct.pack("<BH", t, 0))
        f.write(struct.pack("<I", len(groups)))
        for lo, hi in groups:
            f.write(struct.pack("<Q", hi - lo))
            parts = []
            for vals, mask, t in cols:
                v = vals[lo:hi]
                m = mask[lo:hi]
                f.write(_stats(np.asarray(v) if t != abi.VEC_STRING else v, m, t))
                parts.append(_column_bytes(v, m, t))
            for p in parts:
                f.write(p)
    return len(groups)
