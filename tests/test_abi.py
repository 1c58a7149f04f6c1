"""The C-ABI boundary, without a GPU: libvgpu loads, exports every function
include/*.h declares, and its structs are laid out exactly like the
reference's (so the reference engine, its optimizer and explain() can hold
libvgpu nodes)."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("vgpu.h",):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\(", src, flags=re.M):
            name = m.group(1)
            if name not in ("if", "while", "for", "return", "sizeof"):
                names.add(name)
    return sorted(names)


def test_library_exports_every_declared_symbol():
    import vectra_gb300
    lib = vectra_gb300.load()
    names = declared_functions()
    assert "filter_node_create" in names and "join_node_create" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_no_device_needed_to_load():
    import vectra_gb300
    lib = vectra_gb300.load()
    assert lib.vgpu_kernel_launches() >= 0


def test_struct_layout_matches_reference():
    golden = open(os.path.join(ROOT, "tests", "golden", "abi_layout.txt")).read()
    out = os.path.join(ROOT, "oracle", "_ref")
    os.makedirs(out, exist_ok=True)
    exe = os.path.join(out, "abi_mine")
    subprocess.run(["gcc", "-std=gnu11", "-I", os.path.join(ROOT, "include"), "-o", exe,
                    os.path.join(ROOT, "oracle", "abi_check.c")], check=True)
    mine = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    assert mine == golden


def test_ctypes_mirror_matches_header():
    from vectra_gb300 import abi
    golden = open(os.path.join(ROOT, "tests", "golden", "abi_layout.txt")).read()
    sizes = dict(re.findall(r"sizeof (\w+) (\d+)", golden))
    assert C.sizeof(abi.VecArray) == int(sizes["VecArray"])
    assert C.sizeof(abi.VecBatch) == int(sizes["VecBatch"])
    assert C.sizeof(abi.VecSchema) == int(sizes["VecSchema"])
    assert C.sizeof(abi.VecNode) == int(sizes["VecNode"])
    assert C.sizeof(abi.VecExpr) == int(sizes["VecExpr"])
    assert C.sizeof(abi.AggSpec) == int(sizes["AggSpec"])
    assert C.sizeof(abi.JoinKey) == int(sizes["JoinKey"])
    assert C.sizeof(abi.ProjEntry) == int(sizes["ProjEntry"])


def test_table_source_batch_bounds_and_kind():
    """batch_rows above the int32 row-id range is rejected; the default
    (whole table) is clamped to it; the node's kind is not "ScanNode" (the
    reference optimizer reads a .vtr header through every ScanNode).  Host
    work only: no device is touched."""
    import numpy as np
    import vectra_gb300
    from vectra_gb300 import abi
    lib = vectra_gb300.load()
    f = lib.vgpu_table_source_create
    f.restype = C.c_void_p
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int]
    vals = np.arange(100, dtype=np.int64)
    names = (C.c_char_p * 1)(b"k")
    types = (C.c_int * 1)(abi.VEC_INT64)
    data = (C.c_void_p * 1)(vals.ctypes.data)
    assert f(1, names, types, data, None, 100, 2 ** 31, 0) is None
    assert b"batch_rows 2147483648 is above the largest batch" in lib.vgpu_last_error()
    for br in (0, 7, 2 ** 31 - 1):
        p = f(1, names, types, data, None, 100, br, 0)
        assert p
        node = C.cast(p, C.POINTER(abi.VecNode)).contents
        assert node.kind == b"VgpuTableSource"
        node.free_node(C.cast(p, C.POINTER(abi.VecNode)))
