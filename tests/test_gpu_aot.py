"""The ahead-of-time compiled aggregation kernels (agg_fast_kernel,
agg_kernel) stay correct on their own: the group and join+aggregate cases
with the run-time specialised kernel switched off (VGPU_NO_JIT)."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

FP_COLS = ("s", "m", "sr", "mr", "sd", "p", "avg")
RTOL = 1e-12


@pytest.fixture(scope="module")
def G():
    from engines import gpu_engine
    return gpu_engine()


@pytest.fixture
def no_jit(monkeypatch):
    monkeypatch.setenv("VGPU_NO_JIT", "1")


@pytest.mark.parametrize("temp_dir", ["tmp", None], ids=["sorted", "hash"])
@pytest.mark.parametrize("case", cases.GROUP_CASES, ids=lambda f: f.__name__)
def test_group_cases_aot(case, temp_dir, G, oracle, no_jit):
    td = None if temp_dir is None else oracle.tmp
    cases.same_batches(case(G, td), case(oracle, td), rtol=RTOL, tol_cols=FP_COLS)


@pytest.mark.parametrize("n,batch", [(1000, 96), (20000, 4096)])
@pytest.mark.parametrize("sel_mode", [0, 1])
def test_random_group_aot(n, batch, sel_mode, G, oracle, no_jit):
    cases.same_batches(cases.r_group(G, n + 1, n, batch, sel_mode, oracle.tmp),
                       cases.r_group(oracle, n + 1, n, batch, sel_mode, oracle.tmp), rtol=RTOL, tol_cols=FP_COLS)
