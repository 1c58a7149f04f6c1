"""Generates tests/golden/ref_cases.npz: the reference engine's own output
(oracle/_ref/libvectra_ref.so, compiled from the reference's C sources) for
every parity case in tests/cases.py.  tests/test_golden.py checks the CPU
oracle against these fixtures wherever the reference checkout is absent.

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
    for f in cases.FILTER_CASES + cases.JOIN_CASES:
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


def main():
    R = RefEngine()
    arrays, manifest = {}, {}
    for name, fn in all_cases():
        batches = fn(R)
        manifest[name] = [list(b.keys()) for b in batches]
        for bi, b in enumerate(batches):
            for col, (v, m) in b.items():
                arrays["%s|%d|%s|v" % (name, bi, col)] = v
                arrays["%s|%d|%s|m" % (name, bi, col)] = m
    np.savez_compressed(os.path.join(HERE, "ref_cases.npz"), **arrays)
    with open(os.path.join(HERE, "ref_cases.json"), "w") as f:
        json.dump(manifest, f, indent=0, sort_keys=True)
    print("wrote %d cases" % len(manifest))


if __name__ == "__main__":
    main()
