"""vgpu_filter_select_static, the allocation-free filter.

- against the filter node (filter_node_create over a device table source) on
  the same device columns: three calls in a row on one fixed scratch array (a
  conjunction of ranges, a general expression program, the first predicate
  again), each compared with the node's selected rows;
- at exactly VGPU_STATIC_MAX_ROWS rows, where the keep words fill the
  scratch's 1 MiB part, against the CPU oracle's filter node, twice in a row;
- in a fresh process that never initialises the library (no libvgpu stream:
  the legacy default stream), against a numpy mask.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 100_003


def _padded_bits(mask):
    from vectra_gb300 import abi
    bits = abi.validity_from_mask(mask)
    out = np.zeros(((len(bits) + 3) // 4) * 4, np.uint8)
    out[:len(bits)] = bits
    return out


def _bind(lib):
    fn = lib.vgpu_filter_select_static
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                   C.c_void_p, C.POINTER(C.c_int64)]
    return fn


def test_static_filter_matches_filter_node():
    torch = pytest.importorskip("torch")
    import vectra_gb300
    from vectra_gb300 import abi
    from vectra_gb300.plan import Tbl, col

    lib = vectra_gb300.load()
    fn = _bind(lib)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(23)
    x = rng.normal(0, 1, N)
    x[rng.random(N) < 0.01] = np.nan
    host = {
        "rid": (np.arange(N, dtype=np.int64), None, abi.VEC_INT64),
        "x": (x, rng.random(N) > 0.05, abi.VEC_DOUBLE),
        "k": (rng.integers(-50, 50, N), rng.random(N) > 0.1, abi.VEC_INT64),
        "b": (rng.integers(0, 2, N).astype(np.uint8), rng.random(N) > 0.02, abi.VEC_BOOL),
    }
    d = {}
    for name, (v, m, t) in host.items():
        tv = torch.from_numpy(np.ascontiguousarray(v)).to(dev)
        tm = torch.from_numpy(_padded_bits(m)).to(dev) if m is not None else None
        d[name] = (tv, tm, t)
    torch.cuda.synchronize()
    names = list(d)
    schema = [(n, d[n][2]) for n in names]
    c_names = (C.c_char_p * len(names))(*[n.encode() for n in names])
    c_types = (C.c_int * len(names))(*[d[n][2] for n in names])
    c_data = (C.c_void_p * len(names))(*[d[n][0].data_ptr() for n in names])
    c_valid = (C.c_void_p * len(names))(*[(d[n][1].data_ptr() if d[n][1] is not None else None)
                                           for n in names])
    sel = torch.full((N,), -1, dtype=torch.int32, device=dev)

    preds = [
        (col("x") > -0.5) & (col("k") <= 30) & ~col("b").eq(True),   # conjunction of ranges
        (col("x") * 2.0 + col("k")) > 10.0,                            # general expression program
        (col("x") > -0.5) & (col("k") <= 30) & ~col("b").eq(True),   # the first one again
    ]
    got = []
    launches = lib.vgpu_kernel_launches()
    for p in preds:
        n_sel = C.c_int64(-1)
        rc = fn(len(names), c_names, c_types, c_data, c_valid, N, p.to_c(schema), sel.data_ptr(),
                C.byref(n_sel))
        assert rc == 0, lib.vgpu_last_error().decode()
        assert 0 < n_sel.value < N
        got.append(sel[:n_sel.value].cpu().numpy().astype(np.int64))
    assert lib.vgpu_kernel_launches() > launches
    np.testing.assert_array_equal(got[0], got[2])

    G = vectra_gb300.engine(0)
    for p, g in zip(preds, got):
        src = G.make_source({n: (d[n][0].data_ptr(), d[n][1].data_ptr() if d[n][1] is not None else 0,
                                 d[n][2], N) for n in names}, batch_rows=1 << 17, device=True)
        want = Tbl(G, src).filter(p).collect()
        np.testing.assert_array_equal(g, want["rid"][0])


def test_static_filter_rejects_oversize_input():
    pytest.importorskip("torch")
    import vectra_gb300
    from vectra_gb300 import abi
    from vectra_gb300.plan import col

    lib = vectra_gb300.load()
    fn = _bind(lib)
    limit = 8388608
    c_names = (C.c_char_p * 1)(b"k")
    c_types = (C.c_int * 1)(abi.VEC_INT64)
    c_data = (C.c_void_p * 1)(16)      # never read: the row count is rejected first
    n_sel = C.c_int64(-1)
    rc = fn(1, c_names, c_types, c_data, None, limit + 1, (col("k") > 0).to_c([("k", abi.VEC_INT64)]),
            C.c_void_p(16), C.byref(n_sel))
    assert rc == -1
    assert b"at most 8388608 rows" in lib.vgpu_last_error()
    assert n_sel.value == 0


def _device_cols(torch, dev, host):
    d = {}
    for name, (v, m, t) in host.items():
        tv = torch.from_numpy(np.ascontiguousarray(v)).to(dev)
        tm = torch.from_numpy(_padded_bits(m)).to(dev) if m is not None else None
        d[name] = (tv, tm, t)
    torch.cuda.synchronize()
    names = list(d)
    c_names = (C.c_char_p * len(names))(*[n.encode() for n in names])
    c_types = (C.c_int * len(names))(*[d[n][2] for n in names])
    c_data = (C.c_void_p * len(names))(*[d[n][0].data_ptr() for n in names])
    c_valid = (C.c_void_p * len(names))(*[(d[n][1].data_ptr() if d[n][1] is not None else None)
                                           for n in names])
    return d, names, (c_names, c_types, c_data, c_valid)


def test_static_filter_at_row_limit_matches_oracle():
    """8,388,608 rows (the limit): the selection equals the oracle's filter
    node's on the same rows, on two calls in a row."""
    torch = pytest.importorskip("torch")
    import vectra_gb300
    from vectra_gb300 import abi
    from vectra_gb300.plan import col, tbl
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from engines import OracleEngine

    lib = vectra_gb300.load()
    fn = _bind(lib)
    n = 8388608
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(31)
    host = {
        "rid": (np.arange(n, dtype=np.int64), None, abi.VEC_INT64),
        "t": (rng.normal(20, 10, n), rng.random(n) > 0.01, abi.VEC_DOUBLE),
        "y": (rng.integers(2000, 2026, n), None, abi.VEC_INT64),
    }
    d, names, (c_names, c_types, c_data, c_valid) = _device_cols(torch, dev, host)
    schema = [(nm, host[nm][2]) for nm in names]
    sel = torch.full((n,), -1, dtype=torch.int32, device=dev)
    preds = [(col("t") > 30.0) & (col("y") >= 2020.0),
             ((col("t") - 20.0) * (col("y") - 2000) > 100.0) | col("t").eq(lit_na())]
    O = OracleEngine()
    table = {nm: (host[nm][0], host[nm][1]) if host[nm][1] is not None else host[nm][0] for nm in names}
    for p in preds:
        want = tbl(O, table, batch_rows=100_000).filter(p).collect()["rid"][0]
        for _ in range(2):
            n_sel = C.c_int64(-1)
            rc = fn(len(names), c_names, c_types, c_data, c_valid, n, p.to_c(schema), sel.data_ptr(),
                    C.byref(n_sel))
            assert rc == 0, lib.vgpu_last_error().decode()
            assert n_sel.value == len(want)
            np.testing.assert_array_equal(sel[:n_sel.value].cpu().numpy().astype(np.int64), want)
            sel.fill_(-1)


def lit_na():
    from vectra_gb300.plan import lit
    return lit(None)


_FRESH = r"""
import ctypes as C, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
import vectra_gb300
from vectra_gb300 import abi
from vectra_gb300.plan import col
lib = vectra_gb300.load()          # opens the library; vgpu_init is never called
fn = lib.vgpu_filter_select_static
fn.restype = C.c_int
fn.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
               C.c_void_p, C.POINTER(C.c_int64)]
n = 300_007
rng = np.random.default_rng(5)
x = rng.normal(0, 1, n)
k = rng.integers(-100, 100, n)
ok = rng.random(n) > 0.03
bits = abi.validity_from_mask(ok)
pad = np.zeros(((len(bits) + 3) // 4) * 4, np.uint8)
pad[:len(bits)] = bits
dev = torch.device("cuda", 0)
tx, tk, tv = (torch.from_numpy(a).to(dev) for a in (x, k, pad))
sel = torch.full((n,), -1, dtype=torch.int32, device=dev)
torch.cuda.synchronize()
names = (C.c_char_p * 2)(b"x", b"k")
types = (C.c_int * 2)(abi.VEC_DOUBLE, abi.VEC_INT64)
data = (C.c_void_p * 2)(tx.data_ptr(), tk.data_ptr())
valid = (C.c_void_p * 2)(tv.data_ptr(), None)
pred = ((col("x") > 0.25) & (col("k") < 40)).to_c([("x", abi.VEC_DOUBLE), ("k", abi.VEC_INT64)])
want = np.nonzero(ok & (x > 0.25) & (k < 40))[0]
for _ in range(2):
    m = C.c_int64(-1)
    rc = fn(2, names, types, data, valid, n, pred, sel.data_ptr(), C.byref(m))
    assert rc == 0, lib.vgpu_last_error().decode()
    assert m.value == len(want), (m.value, len(want))
    assert np.array_equal(sel[:m.value].cpu().numpy(), want)
print("fresh ok", m.value)
"""


def test_static_filter_in_fresh_process_without_init():
    """The allocation-free filter in a process where libvgpu was never
    initialised (so it runs on the legacy default stream), against numpy."""
    pytest.importorskip("torch")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _FRESH, root], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fresh ok" in r.stdout
