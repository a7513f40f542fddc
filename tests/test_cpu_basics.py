"""CPU tests: the C-ABI library loads and exports every declared symbol, the report writer's format, the
synthetic generator's invariants, and the oracle's independence from thread count and batching."""
import re
from pathlib import Path

import numpy as np
import pytest

from tests.conftest import make_dataset

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"^\w[\w\s\*]*?\b(fp_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol(native):
    import ctypes
    from firepony_gb300.engine import library_path
    lib = ctypes.CDLL(str(library_path()))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert declared_functions(), "no declarations found"
    assert not missing, f"missing exports: {missing}"


def test_bam_library_exports_every_declared_symbol(native):
    """libfpbam exports every fpb_ function include/firepony_gb300_bam.h declares."""
    import ctypes
    from firepony_gb300 import bam
    try:
        lib = bam.lib()
    except RuntimeError as ex:
        pytest.skip(str(ex))
    text = (ROOT / "include" / "firepony_gb300_bam.h").read_text()
    names = sorted(set(re.findall(r"^\w[\w\s\*]*?\b(fpb_\w+)\s*\(", text, flags=re.M)))
    assert "fpb_next_batch_device" in names and "fpb_get_stats" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"


def test_sort_entries_rejects_sizes_beyond_32_bit_offsets(native):
    """fp_sort_entries refuses n above FP_SORT_MAX_ENTRIES before it touches the device (its digit counts and
    offsets are 32-bit), and fp_sort_entries_static refuses n above its fixed scratch."""
    from firepony_gb300.abi import FP_BAD_INPUT
    from firepony_gb300.engine import lib
    L = lib()
    assert L.fp_sort_entries(16, 32, (1 << 32) - 1, 29, None) == FP_BAD_INPUT
    assert L.fp_sort_entries(16, 32, 1 << 33, 29, None) == FP_BAD_INPUT
    assert L.fp_sort_entries(16, 32, 100, 33, None) == FP_BAD_INPUT
    assert L.fp_sort_entries_static(16, 32, (1 << 20) + 1, 29, None) == FP_BAD_INPUT
    text = (ROOT / "include" / "firepony_gb300.h").read_text()
    assert re.search(r"#define FP_SORT_MAX_ENTRIES 0xFFFFFFFEull", text)


def test_report_format_small_table(native, tmp_path):
    from firepony_gb300.engine import write_report
    t = {}
    f64 = lambda *v: np.array(v, np.float64)
    # RecalTable0: one read group, M and I rows
    t[0] = dict(keys=np.array([0, 1], np.uint32), observations=np.array([1000, 1000], np.uint64),
                mismatches=f64(10.004, 0.5), expected_errors=f64(1.0, 0.03), estimated_quality=f64(30.0, 45.0),
                empirical_quality=f64(20.0, 33.0))
    # RecalTable1: Q30 M, Q45 I
    t[1] = dict(keys=np.array([(30 << 2) | 0, (45 << 2) | 1], np.uint32), observations=np.array([1000, 1000], np.uint64),
                mismatches=f64(10.004, 0.5), expected_errors=f64(1.0, 0.03), estimated_quality=f64(30.0, 45.0),
                empirical_quality=f64(20.0, 33.0))
    # cycle: Q30 cycle -3 (raw (3<<1)|1 = 7) M; context: Q30 "AC" 2-mer M
    t[2] = dict(keys=np.array([(30 << 12) | (7 << 2)], np.uint32), observations=np.array([5], np.uint64),
                mismatches=f64(0.125), expected_errors=f64(0.005), estimated_quality=f64(30.0),
                empirical_quality=f64(22.0))
    ctx = (((0 << 2) | 1) << 4) | 2  # context bits: j=0 -> 'C' (low bits), j=1 -> 'A'
    t[3] = dict(keys=np.array([(30 << 13) | (ctx << 2)], np.uint32), observations=np.array([7], np.uint64),
                mismatches=f64(1.0), expected_errors=f64(0.007), estimated_quality=f64(30.0),
                empirical_quality=f64(25.0))
    out = tmp_path / "r.txt"
    write_report(out, t, ["grp1"])
    text = out.read_text()
    golden = (ROOT / "tests" / "golden" / "report_small.txt").read_text()
    assert text == golden


def test_synth_batches_are_consistent_and_deterministic():
    from firepony_gb300 import synth
    p, ref, batches = make_dataset("batched_uneven", 3000, 1000, 300_000)
    _, _, again = make_dataset("batched_uneven", 3000, 1000, 300_000)
    for b, c in zip(batches, again):
        for k in b.arrays:
            np.testing.assert_array_equal(b[k], c[k])
    b = batches[0]
    # reads padded to 8 symbols; CIGAR covers the read
    assert np.all(b["read_start"] % 8 == 0)
    for r in range(0, b.num_reads, 97):
        ops = b["cigars"][b["cigar_start"][r]:b["cigar_start"][r] + b["cigar_len"][r]]
        covered = sum(int(o & 0xFFFFFF) for o in ops if (o >> 24) in (0, 1, 4, 7, 8))
        assert covered == b["read_len"][r]
    assert set(np.unique(b["read_len"])) <= {36, 76, 101, 151, 250}


@pytest.mark.parametrize("threads", [4, 7])
def test_oracle_independent_of_threads_and_batching(threads):
    """The oracle's parallel sort/merge/fold (chunk runs merged pairwise, the running table merged in key
    ranges) gives the tables of one sequential pass, for any thread count and batch size."""
    from oracle.oracle import Oracle
    p, ref, batches = make_dataset("precision_20M_151bp_pe", 3000, 3000, 300_000)
    whole = batches[0]
    o1 = Oracle(p.num_read_groups)
    o1.load_reference(ref)
    o1.process(whole, threads=1)
    t1 = o1.finalize()
    o2 = Oracle(p.num_read_groups)
    o2.load_reference(ref)
    for i in range(0, whole.num_reads, 700):
        o2.process(whole.range(i, min(i + 700, whole.num_reads)), threads=threads)
    t2 = o2.finalize()
    for t in range(4):
        for k in t1[t]:
            np.testing.assert_array_equal(t1[t][k], t2[t][k])


def test_oracle_matches_golden_fixture():
    """Regression pin: the oracle's tables on a small seeded data set and on the edge-case batch."""
    from tests.golden.make_golden import compute
    data = np.load(ROOT / "tests" / "golden" / "oracle_tables.npz")
    now = compute()
    assert set(now) == set(data.files)
    for k in data.files:
        np.testing.assert_array_equal(now[k], data[k], err_msg=k)
