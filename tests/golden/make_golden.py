"""Generates tests/golden/ref_cases.npz: the reference engine's own output
(oracle/_ref/libvectra_ref.so, compiled from the reference's C sources) for
every parity case in tests/cases.py.  tests/test_golden.py checks the CPU
oracle against these fixtures wherever the reference checkout is absent.
Also tests/golden/ref_weather.vtr: cases.vtr_weather_table() written by the
reference's own .vtr writer (read by the scan tests).

    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import cases  # noqa: E402
from engines import RefEngine  # noqa: E402


def all_cases():
    for f in cases.FILTER_CASES + cases.JOIN_CASES + cases.SORT_CASES:
        yield f.__name__, (lambda E, f=f: f(E))
    for f in cases.GROUP_CASES:
        for mode in ("sorted", "hash"):
            yield "%s[%s]" % (f.__name__, mode), (lambda E, f=f, m=mode: f(E, None if m == "hash" else E.tmp))
    for n, batch in cases.RAGGED:
        for sel in (0, 1):
            yield "r_filter[%d,%d,%d]" % (n, batch, sel), (lambda E, n=n, b=batch, s=sel: cases.r_filter(E, n, n, b, s))
        for mode in ("sorted", "hash"):
            yield "r_group[%d,%d,%s]" % (n, batch, mode), (
                lambda E, n=n, b=batch, m=mode: cases.r_group(E, n + 1, n, b, 1, None if m == "hash" else E.tmp))
        yield "r_sort[%d,%d]" % (n, batch), (lambda E, n=n, b=batch: cases.r_sort(E, n + 2, n, b))
    # string columns (filters, joins, sorts, group keys on both paths)
    for f in cases.STRING_FILTER_CASES + cases.STRING_JOIN_CASES + [cases.ss_string_keys]:
        yield f.__name__, (lambda E, f=f: f(E))
    for f in cases.STRING_GROUP_CASES:
        for mode in ("sorted", "hash"):
            yield "%s[%s]" % (f.__name__, mode), (lambda E, f=f, m=mode: f(E, None if m == "hash" else E.tmp))
    for n, batch in [(33, 32), (700, 64)]:
        yield "r_string_filter[%d,%d]" % (n, batch), (lambda E, n=n, b=batch: cases.r_string_filter(E, n, n, b, 1))
        for mode in ("sorted", "hash"):
            yield "r_string_group[%d,%d,%s]" % (n, batch, mode), (
                lambda E, n=n, b=batch, m=mode: cases.r_string_group(E, n, n, b, 1, None if m == "hash" else E.tmp))
        for kind in ("left_join", "full_join"):
            yield "r_string_join[%d,%d,%s]" % (n, batch, kind), (
                lambda E, n=n, b=batch, k=kind: cases.r_string_join(E, n, n, b, k))
        yield "r_string_sort[%d,%d]" % (n, batch), (lambda E, n=n, b=batch: cases.r_string_sort(E, n, n, b))


def pack_strings(v):
    """A string column as (offsets int64, bytes uint8): object arrays do
    not go into the fixture file."""
    enc = [str(x).encode("utf-8", "surrogateescape") for x in v]
    offs = np.zeros(len(enc) + 1, np.int64)
    offs[1:] = np.cumsum([len(e) for e in enc])
    return offs, np.frombuffer(b"".join(enc), dtype=np.uint8).copy()


def unpack_strings(offs, data):
    b = data.tobytes()
    return np.array([b[offs[i]:offs[i + 1]].decode("utf-8", "surrogateescape") for i in range(len(offs) - 1)],
                    dtype=object)


def write_vtr_ref(path, table, batch_rows):
    """Writes `table` with the reference's own .vtr writer
    (vtr1_write_header / vtr1_write_rowgroup, src/vtr1.c:39-153)."""
    import ctypes as C
    from engines import ref_lib
    from vectra_gb300 import abi, vtr
    R = ref_lib()
    libc = C.CDLL(None)
    libc.fopen.restype, libc.fopen.argtypes = C.c_void_p, [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    R.vtr1_write_header.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
    R.vtr1_write_rowgroup.argtypes = [C.c_void_p, C.c_void_p]
    names = list(table)
    cols = [vtr._col(table[n]) for n in names]
    n = len(cols[0][1])
    keep = []
    cnames = (C.c_char_p * len(names))(*[x.encode() for x in names])
    ctypes_ = (C.c_int * len(names))(*[t for _, _, t in cols])
    schema = abi.VecSchema(len(names), cnames, ctypes_, None)
    groups = [(lo, min(n, lo + batch_rows)) for lo in range(0, n, batch_rows)] if n else []
    fp = libc.fopen(path.encode(), b"wb")
    R.vtr1_write_header(fp, C.byref(schema), len(groups))
    for lo, hi in groups:
        arrs = (abi.VecArray * len(names))()
        for c, (vals, mask, t) in enumerate(cols):
            a = arrs[c]
            a.type, a.length, a.owns_data = t, hi - lo, 1
            bits = np.packbits(mask[lo:hi], bitorder="little")
            bits = np.concatenate([bits, np.zeros(1, np.uint8)])
            keep.append(bits)
            a.validity = bits.ctypes.data_as(C.POINTER(C.c_uint8))
            if t == abi.VEC_STRING:
                enc = [str(s).encode() for s in vals[lo:hi]]
                offs = np.zeros(len(enc) + 1, np.int64)
                offs[1:] = np.cumsum([len(e) for e in enc])
                data = C.create_string_buffer(b"".join(enc) or b"\0")
                keep += [offs, data]
                a.buf.str.offsets = offs.ctypes.data_as(C.POINTER(C.c_int64))
                a.buf.str.data = C.cast(data, C.c_void_p)
                a.buf.str.data_len = int(offs[-1])
            else:
                v = np.ascontiguousarray(vals[lo:hi], dtype=np.uint8 if t == abi.VEC_BOOL else None)
                keep.append(v)
                a.buf.i64 = v.ctypes.data_as(C.POINTER(C.c_int64))
        b = abi.VecBatch(hi - lo, len(names), cnames, arrs, None, 0)
        keep.append(arrs)
        R.vtr1_write_rowgroup(fp, C.byref(b))
    libc.fclose(fp)
    return len(groups)


def main():
    write_vtr_ref(os.path.join(HERE, "ref_weather.vtr"), cases.vtr_weather_table(), 600)
    R = RefEngine()
    arrays, manifest = {}, {}
    for name, fn in all_cases():
        batches = fn(R)
        manifest[name] = [list(b.keys()) for b in batches]
        for bi, b in enumerate(batches):
            for col, (v, m) in b.items():
                if v.dtype == object:
                    offs, data = pack_strings(v)
                    arrays["%s|%d|%s|o" % (name, bi, col)] = offs
                    arrays["%s|%d|%s|s" % (name, bi, col)] = data
                else:
                    arrays["%s|%d|%s|v" % (name, bi, col)] = v
                arrays["%s|%d|%s|m" % (name, bi, col)] = m
    np.savez_compressed(os.path.join(HERE, "ref_cases.npz"), **arrays)
    with open(os.path.join(HERE, "ref_cases.json"), "w") as f:
        json.dump(manifest, f, indent=0, sort_keys=True)
    print("wrote %d cases" % len(manifest))


if __name__ == "__main__":
    main()
