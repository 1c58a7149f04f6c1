"""The query-set autotuner's records on the CPU: a set's shape signature
(instance counts, total and largest rows, group cardinality, each as a
power of two) and the record file named by VGPU_TUNE_FILE, one line per
measurement, the last valid line of a shape winning and malformed lines
(threads other than 256 / 512 / 1024, work items under 1024 rows, a table
multiple other than 2 / 4) ignored.  Each lookup runs in a fresh process:
the records are read once per process."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

LOOKUP = r"""
import ctypes as C, json, sys
sys.path.insert(0, %r)
import vectra_gb300
from vectra_gb300.workloads import SetQuery, SetTuning
lib = vectra_gb300.load()
qs = (SetQuery * 3)()
for i, (kind, n, nb, g) in enumerate([(0, 5000, 0, 100), (0, 70000, 0, 900), (1, 20000, 3000, 0)]):
    qs[i].kind, qs[i].n, qs[i].n_build, qs[i].max_groups = kind, n, nb, g
t = SetTuning()
lib.vgpu_queryset_tuning.argtypes = [C.c_void_p, C.c_int, C.POINTER(SetTuning)]
rc = lib.vgpu_queryset_tuning(qs, 3, C.byref(t))
print(json.dumps(dict(t.as_dict(), rc=rc)))
""" % ROOT


def lookup(tune_file=None):
    env = dict(os.environ)
    env.pop("VGPU_TUNE_FILE", None)
    if tune_file:
        env["VGPU_TUNE_FILE"] = str(tune_file)
    out = subprocess.run([sys.executable, "-c", LOOKUP], env=env, capture_output=True, text=True, timeout=120,
                         check=True)
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_no_record_gives_the_defaults_and_the_shape():
    d = lookup()
    assert d["rc"] == 0
    assert (d["threads"], d["chunk_rows"], d["table_mult"]) == (512, 65536, 2)
    # two group-by instances (2^1), one join (2^0), 98000 rows (2^16), largest 70000 (2^16),
    # mean group bound (100 + 900) / 2 = 500 (2^8)
    assert d["shape"] == "g1.j0.r16.m16.c8"


def test_last_valid_line_of_a_shape_wins(tmp_path):
    shape = lookup()["shape"]
    f = tmp_path / "tune.txt"
    f.write_text("\n".join([
        "%s 256 16384 4 30.0 18" % shape,
        "other.shape 1024 262144 2 1.0 18",
        "%s 1024 262144 2 19.25 18" % shape,
        "%s 333 65536 2 1.0 18" % shape,       # threads not a candidate: ignored
        "%s 512 512 2 1.0 18" % shape,         # work item below 1024 rows: ignored
        "%s 512 65536 3 1.0 18" % shape,       # table multiple not 2 or 4: ignored
    ]) + "\n")
    d = lookup(f)
    assert d["rc"] == 1
    assert (d["threads"], d["chunk_rows"], d["table_mult"], d["candidates"]) == (1024, 262144, 2, 18)
    assert abs(d["ms"] - 19.25) < 1e-9


def test_records_of_other_shapes_do_not_apply(tmp_path):
    f = tmp_path / "tune.txt"
    f.write_text("g9.j9.r9.m9.c9 1024 262144 4 1.0 18\n")
    d = lookup(f)
    assert d["rc"] == 0 and (d["threads"], d["chunk_rows"], d["table_mult"]) == (512, 65536, 2)
