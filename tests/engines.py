"""Engines for the test suite: the same plan verbs (vectra_gb300.plan) bound
to the CPU oracle (oracle/liboracle_port.so, this repository's restatement
of the reference path) and to the reference engine itself
(oracle/_ref/libvectra_ref.so, compiled from the reference's own C sources
where that checkout exists).  TEST INFRASTRUCTURE: only tests, smoke() and
bench.py's CPU-baseline leg use the oracle.
"""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

from vectra_gb300 import abi
from vectra_gb300.plan import Engine, _table_types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
PORT_LIB = os.path.join(ORACLE_DIR, "liboracle_port.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "libvectra_ref.so")
# the reference checkout's C sources (build recipe input; absent on machines without it)
REF_SRC = os.environ.get("VECTRA_REF_SRC", "/root/reference/src")

_port = None
_ref = None


def build_port():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "port"], check=True)


def port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB):
            build_port()
        _port = C.CDLL(PORT_LIB)
        _port.orc_table_source_create.restype = C.c_void_p
        _port.orc_table_source_create.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                  C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                                                  C.c_int]
        _port.orc_exact_sum.restype = C.c_double
        _port.orc_exact_sum.argtypes = [C.c_void_p, C.c_int64]
        _port.orc_exact_sum_products.restype = C.c_double
        _port.orc_exact_sum_products.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        _port.orc_set_join_quirk.argtypes = [C.c_int]
        _port.orc_warning_count.restype = C.c_long
    return _port


def ref_available():
    if os.path.exists(REF_LIB):
        return True
    if os.path.isdir(REF_SRC):
        r = subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref", "REF=" + REF_SRC], capture_output=True)
        return r.returncode == 0 and os.path.exists(REF_LIB)
    return False


def ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference engine not built (needs the reference checkout)")
        _ref = C.CDLL(REF_LIB)
        _ref.vref_warning_count.restype = C.c_long
    return _ref


def make_oracle_source(table, batch_rows=None, sel_mode=0):
    lib = port_lib()
    names, types, datas, valids, n = _table_types(table)
    keep = []
    data = (C.c_void_p * len(names))()
    strd = (C.c_void_p * len(names))()
    val = (C.c_void_p * len(names))()
    for i, (t, d, v) in enumerate(zip(types, datas, valids)):
        if t == abi.VEC_STRING:
            enc = [("" if s is None else str(s)).encode("utf-8", "surrogateescape") for s in d]
            offs = np.zeros(len(enc) + 1, np.int64)
            offs[1:] = np.cumsum([len(e) for e in enc])
            blob = np.frombuffer(b"".join(enc) + b"\0", dtype=np.uint8).copy()
            keep += [offs, blob]
            data[i] = offs.ctypes.data
            strd[i] = blob.ctypes.data
        else:
            d = np.ascontiguousarray(d)
            keep.append(d)
            data[i] = d.ctypes.data
        if v is not None:
            bits = abi.validity_from_mask(v)
            keep.append(bits)
            val[i] = bits.ctypes.data
    cn = (C.c_char_p * len(names))(*[s.encode() for s in names])
    ct = (C.c_int * len(names))(*types)
    br = batch_rows or max(n, 1)
    p = lib.orc_table_source_create(len(names), cn, ct, data, strd, val, n, br, sel_mode)
    if not p:
        raise RuntimeError("oracle source creation failed")
    return p   # the source copied everything; `keep` may go


class OracleEngine(Engine):
    def __init__(self):
        lib = port_lib()
        super().__init__(lib, "orc_guard_filter", "orc_guard_project", "orc_guard_group_agg",
                         "orc_guard_join", "orc_guard_next_batch", "orc_batch_free", "orc_last_error")
        self.tmp = tempfile.mkdtemp(prefix="vgpu_oracle_")
        self.sort_fn = "orc_guard_sort"

    def make_source(self, table, batch_rows=None, sel_mode=0, **_):
        return make_oracle_source(table, batch_rows, sel_mode)


class RefEngine(Engine):
    def __init__(self):
        lib = ref_lib()
        super().__init__(lib, "vref_guard_filter", "vref_guard_project", "vref_guard_group_agg",
                         "vref_guard_join", "vref_guard_next_batch", "vec_batch_free", "vref_last_error")
        self.tmp = tempfile.mkdtemp(prefix="vgpu_ref_")
        self.scan_fn = "vref_guard_scan"
        self.sort_fn = "vref_guard_sort"

    def make_source(self, table, batch_rows=None, sel_mode=0, **_):
        return make_oracle_source(table, batch_rows, sel_mode)


def exact_sum(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    return port_lib().orc_exact_sum(x.ctypes.data, len(x))


def exact_sum_products(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return port_lib().orc_exact_sum_products(a.ctypes.data, b.ctypes.data, len(a))


def _has_strings(table):
    from vectra_gb300.plan import _table_types
    return abi.VEC_STRING in _table_types(table)[1]


def gpu_engine():
    """libvgpu, fed by its own table source, or -- for batches that carry a
    selection vector (sel_mode=1) -- by the oracle's source node, which is
    how a foreign child (the reference's ScanNode, FilterNode ...) feeds it."""
    import vectra_gb300
    from vectra_gb300.plan import GpuEngine

    class GpuTestEngine(GpuEngine):
        def make_source(self, table, batch_rows=None, sel_mode=0, **opts):
            # string columns come as the reference's scan delivers them:
            # host batches of a foreign source node
            if sel_mode or _has_strings(table):
                return make_oracle_source(table, batch_rows, sel_mode)
            return super().make_source(table, batch_rows, **opts)

    lib = vectra_gb300.load()
    if lib.vgpu_init(0) != 0:
        raise RuntimeError(lib.vgpu_last_error().decode())
    return GpuTestEngine(lib)
