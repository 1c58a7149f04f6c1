"""vgpu_filter_select_static, the allocation-free filter, against the
filter node (filter_node_create over a device table source) on the same
device columns: three calls in a row on one fixed scratch array (a
conjunction of ranges, a general expression program, the first predicate
again), each compared with the node's selected rows.  The static calls run
first, so in a fresh process they also run before the library is
initialised."""
import ctypes as C

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
