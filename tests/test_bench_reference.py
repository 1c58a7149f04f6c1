"""bench.py --impl reference on the other workloads: the CPU restatement of
the reference path (single-threaded, like the reference engine) timed on a
sample of the filter + group-by, high-cardinality and query-set workloads,
here at a very small scale."""
import argparse
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("workload", ["filter_group", "high_card", "query_set"])
def test_cpu_reference_sample_of_a_workload(workload):
    sys.path.insert(0, ROOT)
    import bench
    args = argparse.Namespace(workload=workload, steps=1, warmup=0, scale=1000)
    line = bench.reference_arm(args, 0, 1)
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_headline_reference_on_every_core(monkeypatch):
    """The headline reference arm runs one copy of the sampled query per
    host core, steps synchronised by a barrier; two copies of a tiny sample
    here."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(bench, "N_FACT", 40_000)
    monkeypatch.setattr(bench, "N_DIM", 4_000)
    v, secs, n = bench.cpu_baseline_all_cores(0, 2, n_copies=2)
    assert n == 2 and secs > 0
    assert v == 2 * (40_000 // bench.SAMPLE_DIV + 4_000 // bench.SAMPLE_DIV) / secs
