"""Host-side pieces of the job server: zero-copy read ranges, the arrival schedule, job slicing."""
import numpy as np

from firepony_gb300 import synth
from firepony_gb300.serve import jobs_from_pool, poisson_schedule


def _batch():
    p = synth.PRESETS["precision_20M_151bp_pe"].scaled(num_reads=3000, total_reference_bp=300_000,
                                                       batch_reads=3000)
    return synth.Reference(p).batch(0, 3000)


def test_range_equals_subset():
    b = _batch()
    rng = np.random.default_rng(5)
    for first, last in [(0, 3000), (0, 1), (17, 18), (100, 2345), (2999, 3000), (40, 40)]:
        r = b.range(first, last)
        s = b.subset(np.arange(first, last))
        assert r.num_reads == s.num_reads == last - first
        assert (r.num_cigar_ops, r.num_read_symbols, r.num_qualities) == \
               (s.num_cigar_ops, s.num_read_symbols, s.num_qualities)
        for name in r.arrays:
            np.testing.assert_array_equal(r[name], s[name], err_msg=name)
    # the bulk arrays are views of the parent's memory
    r = b.range(10, 20)
    assert np.shares_memory(r["qualities"], b["qualities"]) and np.shares_memory(r["reads"], b["reads"])
    assert rng is not None


def test_poisson_schedule_seeded():
    a1, s1 = poisson_schedule(64, 20.0, 1000, 5_000_000, seed=9)
    a2, s2 = poisson_schedule(64, 20.0, 1000, 5_000_000, seed=9)
    np.testing.assert_array_equal(a1, a2)
    np.testing.assert_array_equal(s1, s2)
    assert a1[0] == 0 and np.all(np.diff(a1) >= 0)
    assert s1.min() >= 1000 and s1.max() <= 5_000_000


def test_jobs_cover_requested_reads():
    b = _batch()
    pool = [b.range(0, 1500), b.range(1500, 3000)]
    jobs = jobs_from_pool(pool, [1, 700, 1500, 2200, 9999], batch_reads=500)
    for job, want in zip(jobs, [1, 700, 1500, 2200, 3000]):
        parts = list(job.batches())
        assert job.num_reads == want
        assert sum(p.num_reads for p in parts) == want
        assert all(p.num_reads <= 500 for p in parts)
