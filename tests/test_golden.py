"""The CPU oracle against golden outputs of the reference engine
(tests/golden/ref_cases.npz, written by tests/golden/make_golden.py from the
reference's own C sources).  Runs anywhere, GPU or not: this is what pins
the oracle where the reference checkout is absent."""
import json
import os

import numpy as np
import pytest

import cases
from golden.make_golden import all_cases, unpack_strings

HERE = os.path.dirname(os.path.abspath(__file__))
NPZ = os.path.join(HERE, "golden", "ref_cases.npz")
MANIFEST = os.path.join(HERE, "golden", "ref_cases.json")

CASES = dict(all_cases())


def load_golden(name):
    manifest = json.load(open(MANIFEST))
    z = np.load(NPZ, allow_pickle=False)
    out = []
    for bi, cols in enumerate(manifest[name]):
        b = {}
        for c in cols:
            key = "%s|%d|%s|" % (name, bi, c)
            v = unpack_strings(z[key + "o"], z[key + "s"]) if key + "o" in z.files else z[key + "v"]
            b[c] = (v, z[key + "m"])
        out.append(b)
    return out


@pytest.mark.parametrize("name", sorted(json.load(open(MANIFEST)).keys()) if os.path.exists(MANIFEST) else [])
def test_oracle_matches_reference_golden(name, oracle):
    cases.same_batches(CASES[name](oracle), load_golden(name))
