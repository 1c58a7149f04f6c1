"""Synthetic workloads of the reference's benchmark configurations beyond
the join + aggregate headline, generated on the device with torch (seeded),
with the queries built through the node C API and property checks of the
results at full size.

  filter_group  10M rows: station int64 U{0..999}, temperature f64
                N(20, 10) with 1% NA, year int64 U{2000..2025};
                filter(temperature > 30, year >= 2020) |> group_by(station)
                |> summarise(avg = mean(temperature), n = n())
  high_card     200M rows: key int64 over 50M distinct values (a bijective
                scramble of U{0..50M-1}) with 5% NA, x f64 LogNormal(0, 2),
                y int64 U{-1e6..1e6}; group_by(key) |> summarise(sum(x),
                mean(x), min(y), max(y), n())
"""
import ctypes as C

import numpy as np

from .plan import Tbl, col


def _validity(torch, mask):
    n = mask.numel()
    nb = ((n + 31) // 32) * 4
    m = torch.zeros(nb * 8, dtype=torch.uint8, device=mask.device)
    m[:n] = mask.to(torch.uint8)
    w = torch.tensor([1, 2, 4, 8, 16, 32, 64, 128], dtype=torch.uint8, device=mask.device)
    return (m.view(-1, 8) * w).sum(dim=1, dtype=torch.uint8)


def pack_columns(torch, cols):
    """{name: (values, valid_mask or None)} with each mask packed once into
    the validity bitmap the table source reads (for device_source(...,
    packed=True): the queries then start from device-resident columns and
    bitmaps, as a host keeps them)."""
    return {k: (v, _validity(torch, m) if m is not None else None) for k, (v, m) in cols.items()}


def device_source(lib, cols, n_rows, batch_rows=None, packed=False):
    """A VGPU_SRC_DEVICE table source over {name: (values, valid_mask or
    None)}, or over already packed bitmaps (packed=True, pack_columns)."""
    names = list(cols)
    keep = []
    data = (C.c_void_p * len(names))()
    val = (C.c_void_p * len(names))()
    types = (C.c_int * len(names))()
    for i, n in enumerate(names):
        v, m = cols[n]
        data[i] = v.data_ptr()
        types[i] = 1 if v.dtype.is_floating_point else 0
        if m is not None:
            if packed:
                bits = m
            else:
                import torch
                bits = _validity(torch, m)
            keep.append(bits)
            val[i] = bits.data_ptr()
        else:
            val[i] = None
    cn = (C.c_char_p * len(names))(*[n.encode() for n in names])
    lib.vgpu_table_source_create.restype = C.c_void_p
    p = lib.vgpu_table_source_create(len(names), cn, types, data, val, n_rows, batch_rows or n_rows, 2)
    if not p:
        raise RuntimeError(lib.vgpu_last_error().decode())
    return p, keep


# --------------------------------------------------------------------------
# filter + group-by (10M rows)
# --------------------------------------------------------------------------

def gen_filter_group(torch, n, seed, device):
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    station = torch.randint(0, 1000, (n,), device=device, generator=g, dtype=torch.int64)
    temp = torch.randn(n, dtype=torch.float64, device=device, generator=g) * 10.0 + 20.0
    tvalid = torch.rand(n, device=device, generator=g) >= 0.01
    temp[~tvalid] = 0.0
    year = torch.randint(2000, 2026, (n,), device=device, generator=g, dtype=torch.int64)
    return {"station": (station, None), "temperature": (temp, tvalid), "year": (year, None)}


def run_filter_group(eng, src, temp_dir="tmp", numpy=True):
    q = (Tbl(eng, src).filter((col("temperature") > 30.0) & (col("year") >= 2020.0))
         .group_by("station").summarise(temp_dir=temp_dir, avg=("mean", "temperature"), n=("n",)))
    return q.collect() if numpy else q.run()


def check_filter_group(torch, out, cols):
    st, _ = cols["station"]
    t, tv = cols["temperature"]
    y, _ = cols["year"]
    keep = tv & (t > 30.0) & (y >= 2020)
    cnt = torch.bincount(st[keep], minlength=1000)
    s = torch.zeros(1000, dtype=torch.float64, device=st.device).index_add_(0, st[keep], t[keep])
    present = (cnt > 0).cpu().numpy()
    assert list(out["station"][0]) == list(np.nonzero(present)[0]), "groups"
    assert np.array_equal(out["n"][0], cnt.cpu().numpy()[present].astype(np.float64)), "n()"
    want = (s / cnt.clamp(min=1)).cpu().numpy()[present]
    got = out["avg"][0]
    assert np.all(np.abs(got - want) <= 1e-12 * np.abs(want)), "mean"
    return int(keep.sum().item())


def filter_group_bytes(n):
    """Every referenced column once in the reference layout (3 columns)."""
    return 3 * (8 * n + (n + 7) // 8)


# --------------------------------------------------------------------------
# high-cardinality group-by (200M rows, 50M distinct keys)
# --------------------------------------------------------------------------

SCRAMBLE = 0x9E3779B97F4A7C15 - (1 << 64)    # odd: multiplication is a bijection mod 2^64


def gen_high_card(torch, n, distinct, seed, device):
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    raw = torch.randint(0, distinct, (n,), device=device, generator=g, dtype=torch.int64)
    key = raw * SCRAMBLE                                  # wraps: distinct raw -> distinct key
    kvalid = torch.rand(n, device=device, generator=g) >= 0.05
    key[~kvalid] = 0
    x = (torch.randn(n, dtype=torch.float64, device=device, generator=g) * 2.0).exp_()
    y = torch.randint(-1_000_000, 1_000_001, (n,), device=device, generator=g, dtype=torch.int64)
    return {"key": (key, kvalid), "x": (x, None), "y": (y, None)}, raw


def run_high_card(eng, src, temp_dir="tmp", numpy=True):
    q = (Tbl(eng, src).group_by("key")
         .summarise(temp_dir=temp_dir, s=("sum", "x"), m=("mean", "x"), lo=("min", "y"), hi=("max", "y"),
                    n=("n",)))
    return q.collect() if numpy else q.run()


def _signed64(u):
    return u - (1 << 64) if u >= (1 << 63) else u


def check_high_card(torch, out, cols, raw, distinct):
    """Every group against torch: the group count, ascending key order with
    the NA group last, n(), sum and mean (relative 1e-12), min and max."""
    key, kv = cols["key"]
    x, _ = cols["x"]
    y, _ = cols["y"]
    dev = key.device
    keys, kvalid = out["key"]
    r = raw[kv]
    cnt = torch.bincount(r, minlength=distinct)
    n_na = int((~kv).sum().item())
    n_groups = int((cnt > 0).sum().item())
    assert len(keys) == n_groups + (1 if n_na else 0), ("groups", len(keys), n_groups)
    if n_na:
        assert not kvalid[-1] and out["n"][0][-1] == n_na, "NA group last"
    tk = torch.from_numpy(np.ascontiguousarray(keys[:n_groups])).to(dev)
    assert bool((tk[1:] > tk[:-1]).all()), "key order"
    inv = tk * _signed64(pow(SCRAMBLE % (1 << 64), -1, 1 << 64))   # raw id of each output key
    s = torch.zeros(distinct, dtype=torch.float64, device=dev).index_add_(0, r, x[kv])
    big = torch.iinfo(torch.int64)
    lo = torch.full((distinct,), big.max, dtype=torch.int64, device=dev).scatter_reduce_(0, r, y[kv], "amin")
    hi = torch.full((distinct,), big.min, dtype=torch.int64, device=dev).scatter_reduce_(0, r, y[kv], "amax")
    g = lambda name: torch.from_numpy(np.ascontiguousarray(out[name][0][:n_groups])).to(dev)
    assert bool((cnt[inv].to(torch.float64) == g("n")).all()), "n()"
    want = s[inv]
    assert bool(((g("s") - want).abs() <= 1e-12 * want.abs()).all()), "sum"
    wm = want / cnt[inv].to(torch.float64)
    assert bool(((g("m") - wm).abs() <= 1e-12 * wm.abs()).all()), "mean"
    assert bool((g("lo") == lo[inv].to(torch.float64)).all()), "min"
    assert bool((g("hi") == hi[inv].to(torch.float64)).all()), "max"
    return n_groups


def high_card_bytes(n, n_groups):
    """Inputs (3 columns) and outputs (key + 5 aggregates) once each."""
    vb = lambda k: (k + 7) // 8
    return 3 * 8 * n + vb(n) + 6 * (8 * n_groups + vb(n_groups))


# --------------------------------------------------------------------------
# query sets: many small group-by / join instances (vgpu_queryset_*)
# --------------------------------------------------------------------------

SET_GROUP, SET_JOIN = 0, 1


class SetQuery(C.Structure):
    """Mirror of VgpuSetQuery (include/vgpu.h)."""
    _fields_ = [("kind", C.c_int32), ("pad", C.c_int32), ("n", C.c_int64), ("key", C.c_void_p),
                ("value", C.c_void_p), ("n_build", C.c_int64), ("build_key", C.c_void_p),
                ("max_groups", C.c_int64), ("out_key", C.c_void_p), ("out_sum", C.c_void_p),
                ("out_mean", C.c_void_p), ("out_n", C.c_void_p), ("out_probe", C.c_void_p),
                ("out_build", C.c_void_p), ("out_rows", C.c_void_p)]


class SetTuning(C.Structure):
    """Mirror of VgpuSetTuning (include/vgpu.h)."""
    _fields_ = [("threads", C.c_int32), ("table_mult", C.c_int32), ("chunk_rows", C.c_int64), ("ms", C.c_double),
                ("candidates", C.c_int32), ("shape", C.c_char * 60)]

    def as_dict(self):
        return {"threads": self.threads, "table_mult": self.table_mult, "chunk_rows": self.chunk_rows,
                "ms": round(self.ms, 4), "candidates": self.candidates, "shape": self.shape.decode()}


def gen_query_set(torch, n_inst, seed, device, median_rows=20_000, sigma=1.5, cap_rows=5_000_000,
                  max_card=100_000):
    """n_inst instances: rows ~ LogNormal(ln median_rows, sigma) capped,
    group cardinality log-uniform [1, max_card], half group_by + summarise
    (sum, mean, n), half inner joins against `card` unique build keys with
    probe keys uniform over [0, 2 card) (about half match); keys in the
    int32 range for half the instances, scrambled over int64 for the rest;
    values N(0, 1)."""
    rng = np.random.default_rng(seed)
    rows = np.clip(np.round(rng.lognormal(np.log(median_rows), sigma, n_inst)), 1, cap_rows).astype(np.int64)
    card = np.clip(np.round(np.exp(rng.uniform(0.0, np.log(max_card), n_inst))), 1, max_card).astype(np.int64)
    kind = rng.integers(0, 2, n_inst)
    wide = rng.integers(0, 2, n_inst).astype(bool)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    total = int(rows.sum())
    # probe / group keys: uniform over [0, card) or [0, 2 card) per instance
    span = np.where(kind == SET_GROUP, card, 2 * card)
    span_t = torch.from_numpy(np.repeat(span, rows)).to(device)
    key = (torch.rand(total, dtype=torch.float64, device=device, generator=g) * span_t).to(torch.int64)
    key = torch.minimum(key, span_t - 1)
    wide_t = torch.from_numpy(np.repeat(wide, rows)).to(device)
    key = torch.where(wide_t, key * SCRAMBLE, key)
    value = torch.randn(total, dtype=torch.float64, device=device, generator=g)
    bcard = np.where(kind == SET_JOIN, card, 0)
    btotal = int(bcard.sum())
    bkey = torch.cat([torch.arange(int(c), device=device, dtype=torch.int64) for c in bcard if c > 0]) \
        if btotal else torch.empty(0, dtype=torch.int64, device=device)
    bwide = torch.from_numpy(np.repeat(wide, bcard)).to(device)
    bkey = torch.where(bwide, bkey * SCRAMBLE, bkey)
    return {"rows": rows, "card": card, "kind": kind, "wide": wide, "key": key, "value": value, "bkey": bkey,
            "bcard": bcard}


def query_set_structs(torch, qs, device):
    """VgpuSetQuery array over the generated instances, with output buffers."""
    n = len(qs["rows"])
    arr = (SetQuery * n)()
    keep = []
    off = np.concatenate([[0], np.cumsum(qs["rows"])])
    boff = np.concatenate([[0], np.cumsum(qs["bcard"])])
    kp, vp, bp = qs["key"].data_ptr(), qs["value"].data_ptr(), qs["bkey"].data_ptr()
    out_rows = torch.zeros(n, dtype=torch.int64, device=device)
    keep.append(out_rows)
    outs = []
    for i in range(n):
        q = arr[i]
        q.kind = int(qs["kind"][i])
        q.n = int(qs["rows"][i])
        q.key = kp + 8 * int(off[i])
        q.out_rows = out_rows.data_ptr() + 8 * i
        if q.kind == SET_GROUP:
            q.value = vp + 8 * int(off[i])
            mg = int(min(qs["card"][i], qs["rows"][i]))
            q.max_groups = mg
            o = {"key": torch.empty(mg, dtype=torch.int64, device=device),
                 "sum": torch.empty(mg, dtype=torch.float64, device=device),
                 "mean": torch.empty(mg, dtype=torch.float64, device=device),
                 "n": torch.empty(mg, dtype=torch.int64, device=device)}
            q.out_key, q.out_sum = o["key"].data_ptr(), o["sum"].data_ptr()
            q.out_mean, q.out_n = o["mean"].data_ptr(), o["n"].data_ptr()
        else:
            q.n_build = int(qs["bcard"][i])
            q.build_key = bp + 8 * int(boff[i])
            o = {"probe": torch.empty(max(1, q.n), dtype=torch.int32, device=device),
                 "build": torch.empty(max(1, q.n), dtype=torch.int32, device=device)}
            q.out_probe, q.out_build = o["probe"].data_ptr(), o["build"].data_ptr()
        outs.append(o)
    return arr, outs, out_rows, keep


def check_query_set(torch, qs, outs, out_rows, idx):
    """Instances idx against torch: group keys and n exactly, sums within
    1e-12 of the sum of magnitudes (torch adds in arbitrary order), mean =
    sum / n, as sets sorted by key; join pairs exactly, in probe order."""
    off = np.concatenate([[0], np.cumsum(qs["rows"])])
    boff = np.concatenate([[0], np.cumsum(qs["bcard"])])
    nrow = out_rows.cpu().numpy()
    for i in idx:
        k = qs["key"][off[i]:off[i + 1]]
        o = outs[i]
        if qs["kind"][i] == SET_GROUP:
            v = qs["value"][off[i]:off[i + 1]]
            uk, inv = torch.unique(k, return_inverse=True)
            cnt = torch.bincount(inv, minlength=len(uk))
            s = torch.zeros(len(uk), dtype=torch.float64, device=k.device).index_add_(0, inv, v)
            m = int(nrow[i])
            assert m == len(uk), (i, m, len(uk))
            order = torch.argsort(o["key"][:m])
            assert bool((o["key"][:m][order] == uk).all()), i
            assert bool((o["n"][:m][order] == cnt).all()), i
            got = o["sum"][:m][order]
            # torch sums in arbitrary order: bound by the sum of magnitudes
            sa = torch.zeros(len(uk), dtype=torch.float64, device=k.device).index_add_(0, inv, v.abs())
            assert bool(((got - s).abs() <= 1e-12 * sa).all()), i
            mean = o["mean"][:m][order]
            assert bool(((mean - got / cnt.double()).abs() <= 1e-15 * (got / cnt.double()).abs() + 1e-300).all()), i
        else:
            b = qs["bkey"][boff[i]:boff[i + 1]]
            sb, perm = torch.sort(b)
            pos = torch.searchsorted(sb, k).clamp(max=max(0, len(sb) - 1))
            hit = (sb[pos] == k) if len(sb) else torch.zeros_like(k, dtype=torch.bool)
            prow = torch.nonzero(hit).flatten().to(torch.int32)
            brow = perm[pos[hit]].to(torch.int32)
            m = int(nrow[i])
            assert m == len(prow), (i, m, len(prow))
            assert bool((o["probe"][:m] == prow).all()) and bool((o["build"][:m] == brow).all()), i


# --------------------------------------------------------------------------
# serving: resident tables, a stream of filter / group / semi-anti requests
# --------------------------------------------------------------------------

SERVE_FILTER_SUM, SERVE_GROUP_SUM, SERVE_SEMI, SERVE_ANTI = 0, 1, 2, 3


class ServeQuery(C.Structure):
    """Mirror of VgpuServeQuery (include/vgpu.h)."""
    _fields_ = [("kind", C.c_int32), ("table", C.c_int32), ("build_table", C.c_int32), ("pad", C.c_int32),
                ("threshold", C.c_double)]


class ServeResult(C.Structure):
    """Mirror of VgpuServeResult (include/vgpu.h)."""
    _fields_ = [("rows", C.c_int64), ("sum", C.c_double), ("key", C.c_void_p), ("key_valid", C.c_void_p),
                ("group_sum", C.c_void_p), ("group_n", C.c_void_p), ("sel", C.c_void_p)]


def bind_server(lib):
    lib.vgpu_server_create.restype = C.c_void_p
    lib.vgpu_server_create.argtypes = [C.c_int, C.c_int64]
    lib.vgpu_server_add_table.restype = C.c_int
    lib.vgpu_server_add_table.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
    lib.vgpu_server_submit.restype = C.c_int64
    lib.vgpu_server_submit.argtypes = [C.c_void_p, C.POINTER(ServeQuery)]
    lib.vgpu_server_poll.restype = C.c_int
    lib.vgpu_server_poll.argtypes = [C.c_void_p]
    lib.vgpu_server_done.restype = C.c_int
    lib.vgpu_server_done.argtypes = [C.c_void_p, C.c_int64]
    lib.vgpu_server_result.restype = C.c_int
    lib.vgpu_server_result.argtypes = [C.c_void_p, C.c_int64, C.POINTER(ServeResult)]
    lib.vgpu_server_release.argtypes = [C.c_void_p, C.c_int64]
    lib.vgpu_server_free.argtypes = [C.c_void_p]
    lib.vgpu_server_warm.restype = C.c_int
    lib.vgpu_server_warm.argtypes = [C.c_void_p, C.c_int]
    lib.vgpu_copy_to_host.restype = C.c_int
    lib.vgpu_copy_to_host.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
    return lib


def gen_serve_tables(torch, sizes, seed, device, ids=10_000_000, zipf_s=1.0, na=0.03):
    """Tables of the given row counts: key int64 Zipf(s) over 1..ids, val f64
    LogNormal(0, 1), each with `na` NA in both columns (validity masks)."""
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    ranks = torch.arange(1, ids + 1, device=device, dtype=torch.float64)
    cdf = torch.cumsum(ranks.pow(-zipf_s), 0)
    cdf /= cdf[-1].clone()
    tables = []
    for n in sizes:
        key = torch.searchsorted(cdf, torch.rand(n, dtype=torch.float64, device=device, generator=g)) + 1
        key = key.clamp_(max=ids).to(torch.int64)
        kv = torch.rand(n, device=device, generator=g) >= na
        val = torch.randn(n, dtype=torch.float64, device=device, generator=g).exp_()
        vv = torch.rand(n, device=device, generator=g) >= na
        key[~kv] = 0
        val[~vv] = 0.0
        tables.append({"key": key, "kv": kv, "val": val, "vv": vv, "kbits": _validity(torch, kv),
                       "vbits": _validity(torch, vv)})
    return tables


def server_with_tables(lib, tables, n_streams=4, budget=120 << 30):
    srv = lib.vgpu_server_create(n_streams, budget)
    if not srv:
        raise RuntimeError(lib.vgpu_last_error().decode())
    for t in tables:
        r = lib.vgpu_server_add_table(srv, t["key"].data_ptr(), t["kbits"].data_ptr(), t["val"].data_ptr(),
                                      t["vbits"].data_ptr(), t["key"].numel())
        if r < 0:
            raise RuntimeError(lib.vgpu_last_error().decode())
    return srv


def gen_requests(n, n_tables, seed):
    """Equal thirds of filter (val > t, t ~ LogNormal quantiles), group-by
    and semi / anti joins of table i against table j."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        q = ServeQuery()
        third = rng.integers(0, 3)
        q.table = int(rng.integers(0, n_tables))
        if third == 0:
            q.kind = SERVE_FILTER_SUM
            q.threshold = float(np.exp(rng.normal(0, 1)))
        elif third == 1:
            q.kind = SERVE_GROUP_SUM
        else:
            q.kind = SERVE_SEMI if rng.integers(0, 2) == 0 else SERVE_ANTI
            q.build_table = int(rng.integers(0, n_tables))
        out.append(q)
    return out


def fetch_result(lib, srv, rid, kind):
    """A finished request's result on the host (group rows sorted by key,
    the NA group last)."""
    r = ServeResult()
    if lib.vgpu_server_result(srv, rid, C.byref(r)) != 0:
        raise RuntimeError(lib.vgpu_last_error().decode())
    if kind == SERVE_FILTER_SUM:
        return (r.rows, r.sum)
    n = r.rows

    def col(ptr, dt):
        a = np.empty(max(1, n), dt)
        if n and lib.vgpu_copy_to_host(a.ctypes.data, ptr, n * a.itemsize) != 0:
            raise RuntimeError(lib.vgpu_last_error().decode())
        return a[:n]
    if kind == SERVE_GROUP_SUM:
        keys, kval = col(r.key, np.int64), col(r.key_valid, np.uint8)
        sums, cnt = col(r.group_sum, np.float64), col(r.group_n, np.int64)
        order = np.lexsort((keys, kval == 0))
        return (keys[order], kval[order], sums[order], cnt[order])
    return col(r.sel, np.int32)
