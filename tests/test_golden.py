"""The CPU oracle against golden outputs of the reference engine
(tests/golden/ref_cases.npz, written by tests/golden/make_golden.py from the
reference's own C sources).  Runs anywhere, GPU or not: this is what pins
the oracle where the reference checkout is absent."""
import json
import os

import numpy as np
import pytest

import cases
from golden.make_golden import all_cases

HERE = os.path.dirname(os.path.abspath(__file__))
NPZ = os.path.join(HERE, "golden", "ref_cases.npz")
MANIFEST = os.path.join(HERE, "golden", "ref_cases.json")

CASES = dict(all_cases())


def load_golden(name):
    manifest = json.load(open(MANIFEST))
    z = np.load(NPZ, allow_pickle=False)
    out = []
    for bi, cols in enumerate(manifest[name]):
        out.append({c: (z["%s|%d|%s|v" % (name, bi, c)], z["%s|%d|%s|m" % (name, bi, c)]) for c in cols})
    return out


@pytest.mark.parametrize("name", sorted(json.load(open(MANIFEST)).keys()) if os.path.exists(MANIFEST) else [])
def test_oracle_matches_reference_golden(name, oracle):
    cases.same_batches(CASES[name](oracle), load_golden(name))
