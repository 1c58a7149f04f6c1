""".vtr files on the CPU: the writer (vectra_gb300.vtr) against the
reference's own writer, and libvgpu's scan node (scan_node_create) read
through its host path (next_batch, no device) against the reference's
ScanNode.

- the fixture tests/golden/ref_weather.vtr was written by the reference's
  writer (tests/golden/make_golden.py); the writer reproduces it byte for
  byte and the scan reads back its table;
- where the reference checkout exists, both writers also agree on tables
  with edge cases (NaN first, signed zeros, all-NA groups, strings, empty
  and ragged row groups), and libvgpu's scan and the reference's scan return
  identical batches for every column subset.
"""
import ctypes as C
import os

import numpy as np
import pytest

import cases
from engines import RefEngine, ref_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURE = os.path.join(ROOT, "tests", "golden", "ref_weather.vtr")


def _gpu_host_engine():
    """libvgpu bound without initialising a device (scan construction and
    next_batch to a host consumer are host work only)."""
    import vectra_gb300
    from vectra_gb300.plan import GpuEngine
    return GpuEngine(vectra_gb300.load())


def _same(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert list(x) == list(y)
        for k in x:
            assert np.array_equal(x[k][1], y[k][1]), k
            va, vb = x[k][0][x[k][1]], y[k][0][y[k][1]]
            if va.dtype == object:
                assert list(va) == list(vb), k
            else:
                assert np.array_equal(va.view(np.uint8), vb.view(np.uint8)), k   # bit for bit


def _edge_tables():
    rng = np.random.default_rng(3)
    n = 1000
    x = rng.normal(0, 1, n)
    x[0] = np.nan                      # NaN first in the first row group: its statistics stay NaN
    x[1:4] = [-0.0, 0.0, -0.0]
    x[500:505] = np.nan
    xv = rng.random(n) > 0.1
    xv[200:300] = False                # an all-NA stretch (a whole row group at 100-row groups)
    k = rng.integers(-(1 << 62), 1 << 62, n)
    kv = rng.random(n) > 0.2
    b = rng.random(n) < 0.5
    bv = rng.random(n) > 0.5
    bv[200:300] = False
    s = [str(i % 7) * (i % 4) for i in range(n)]
    sv = rng.random(n) > 0.1
    s = [c if ok else "" for c, ok in zip(s, sv)]
    yield {"x": (x, xv), "k": (k, kv), "b": (b, bv), "s": (s, sv)}, 100
    yield {"x": (x, xv), "k": k}, 333                  # ragged last group
    yield {"z": (np.zeros(0), np.zeros(0, bool))}, 10  # no rows, no row groups
    zeros = np.array([0.0, -0.0, 0.0, -0.0])
    yield {"z": zeros}, 2
    yield {"z": -zeros}, 3


def test_writer_reproduces_reference_fixture(tmp_path):
    from vectra_gb300 import vtr
    p = tmp_path / "w.vtr"
    vtr.write_vtr(str(p), cases.vtr_weather_table(), 600)
    assert p.read_bytes() == open(FIXTURE, "rb").read()


def test_writer_matches_reference_writer(tmp_path):
    if not ref_available():
        pytest.skip("reference checkout absent")
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import write_vtr_ref
    from vectra_gb300 import vtr
    for i, (table, br) in enumerate(_edge_tables()):
        a, b = tmp_path / ("m%d.vtr" % i), tmp_path / ("r%d.vtr" % i)
        vtr.write_vtr(str(a), table, br)
        write_vtr_ref(str(b), table, br)
        assert a.read_bytes() == b.read_bytes(), i


def test_scan_reads_fixture_table():
    from vectra_gb300.plan import scan
    G = _gpu_host_engine()
    t = cases.vtr_weather_table()
    got = scan(G, FIXTURE).collect()
    assert list(got) == list(t)
    for name, col in t.items():
        vals, mask = col if isinstance(col, tuple) else (col, np.ones(len(col), bool))
        assert np.array_equal(got[name][1], mask), name
        if name == "city":
            assert list(got[name][0][mask]) == [v for v, m in zip(vals, mask) if m]
        else:
            assert np.array_equal(got[name][0][mask], np.asarray(vals)[mask].astype(got[name][0].dtype)), name
    # every batch is one row group, in file order
    sizes = [len(b["station"][0]) for b in scan(G, FIXTURE).batches()]
    assert sizes == [600] * 6 + [234]


def test_scan_matches_reference_scan(tmp_path):
    if not ref_available():
        pytest.skip("reference checkout absent")
    from vectra_gb300 import vtr
    from vectra_gb300.plan import scan
    G, R = _gpu_host_engine(), RefEngine()
    paths = [FIXTURE]
    for i, (table, br) in enumerate(_edge_tables()):
        p = str(tmp_path / ("e%d.vtr" % i))
        vtr.write_vtr(p, table, br)
        paths.append(p)
    for p in paths:
        _same(scan(G, p).batches(), scan(R, p).batches())
    for cols in ([1], [0, 2], [4, 1]):
        _same(scan(G, FIXTURE, cols).batches(), scan(R, FIXTURE, cols).batches())


def test_scan_errors_are_the_references():
    G = _gpu_host_engine()
    from vectra_gb300.plan import EngineError
    with pytest.raises(EngineError, match="cannot open file"):
        G.make_scan("/nonexistent/x.vtr")
    with pytest.raises(EngineError, match="bad magic"):
        G.make_scan(os.path.join(ROOT, "tests", "golden", "ref_cases.json"))
    with pytest.raises(EngineError, match="column index out of range: 9"):
        G.make_scan(FIXTURE, [0, 9])
