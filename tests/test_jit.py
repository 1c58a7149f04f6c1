"""The run-time specialised aggregation kernel: representative plan shapes
are generated and compiled for sm_103a with NVRTC (no device needed), with
no register spills (a plan that would spill at 1024 threads per CTA is
compiled for fewer threads), except a few words in the two-CTA shape of a
dense group key behind a direct join's payload copy."""
import ctypes as C
import re

import pytest


@pytest.mark.parametrize("shape", [0, 1, 2, 3, 4, 5, 6, 7, 8, 11],
                         ids=["join_direct_payload", "filter_sel_mean", "two_keys_all_accs", "inner_join_gather",
                              "join_hashed_payload", "partition_cta_ranges", "partition_filter_holes",
                              "partition_global_cursors", "filter_queued_mean", "join_direct_compact_payload"])
def test_generated_kernel_compiles(shape):
    import vectra_gb300
    lib = vectra_gb300.load()
    lib.vgk_jit_error.restype = C.c_char_p
    regs = C.c_int(-1)
    rc = lib.vgpu_jit_selftest(shape, C.byref(regs))
    log = lib.vgk_jit_error().decode()
    assert rc == 0, log
    assert 0 < regs.value <= 128, log
    spills = re.findall(r"(\d+) bytes spill stores", log)
    # the two-CTA shape of dense payload joins accepts up to 64 spilled bytes
    limit = 64 if "threads per CTA: 768" in log else 0
    assert spills and all(int(x) <= limit for x in spills), log


def test_digit_split_32bit_matches_64bit():
    """The specialised kernel's 32-bit digit split of a double equals the
    64-bit split every other path uses (edge patterns + 4M random ones)."""
    import vectra_gb300
    lib = vectra_gb300.load()
    lib.vgk_digits_selftest.restype = C.c_longlong
    assert lib.vgk_digits_selftest(C.c_longlong(4_000_000), C.c_ulonglong(0x9E3779B97F4A7C15)) == 0


@pytest.mark.parametrize("shape", [0, 1, 2, 3, 4, 5, 6, 7],
                         ids=["high_card_5_aggs", "every_acc_class", "high_card_5_aggs_two_ctas",
                              "every_acc_class_two_ctas", "high_card_5_aggs_four_ctas", "every_acc_class_four_ctas",
                              "high_card_5_aggs_eight_ctas", "every_acc_class_eight_ctas"])
def test_partition_reducer_compiles(shape):
    """The partitioned aggregation's bucket reducer for representative
    plans: compiles for one CTA of 1024 threads per SM, or two of 512 /
    four of 256 / eight of 128 with that share of the groups each, within
    64 registers (the exact-sum finish keeps
    its 66-digit array on the stack; the per-record path does not spill
    more than a few words)."""
    import vectra_gb300
    lib = vectra_gb300.load()
    lib.vgk_jit_error.restype = C.c_char_p
    regs = C.c_int(-1)
    rc = lib.vgpu_pagg_selftest(shape, C.byref(regs))
    log = lib.vgk_jit_error().decode()
    assert rc == 0, log
    assert 0 < regs.value <= 64, log
    kernel = re.search(r"Function properties for vg_jit_pagg\s*\n.*?(\d+) bytes spill stores", log)
    assert kernel and int(kernel.group(1)) <= 256, log


@pytest.mark.parametrize("shape,queued", [(8, 1), (1, 0), (9, 0), (10, 0), (6, 0), (0, 0)],
                         ids=["filter_whole_batches", "filter_sel", "filter_first_seen_order", "filter_join",
                              "filter_partition", "no_filter"])
def test_queue_only_behind_a_filter(shape, queued, tmp_path, monkeypatch):
    """Passing rows are queued per warp only for a filter over whole batches
    with no join, no partition mode and no first-seen order."""
    import vectra_gb300
    dump = tmp_path / "src.cu"
    monkeypatch.setenv("VGPU_JIT_DUMP", str(dump))
    lib = vectra_gb300.load()
    lib.vgk_jit_error.restype = C.c_char_p
    regs = C.c_int(-1)
    assert lib.vgpu_jit_selftest(shape, C.byref(regs)) == 0, lib.vgk_jit_error().decode()
    src = dump.read_text() if dump.exists() else ""
    assert src, "the compiled source was not written (already compiled in this process?)"
    assert ("#define VGJ_COMPACT %d\n" % queued) in src


@pytest.mark.parametrize("shape", range(12))
def test_launch_signature_premise(shape):
    """The specialised kernel is looked up by a launch signature that
    reduces pointers to set / unset and clears per-batch numbers; on every
    self-test plan, changing all of those fields leaves the signature and
    the generated source unchanged (vgpu_jit_sigcheck)."""
    import ctypes as C
    import vectra_gb300
    lib = vectra_gb300.load()
    lib.vgpu_jit_sigcheck.restype = C.c_int
    assert lib.vgpu_jit_sigcheck(shape) == 0
