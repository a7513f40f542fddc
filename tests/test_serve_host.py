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


def test_threaded_submit_never_reuses_a_live_buffer_set():
    """submit_threaded over a decoder that rotates three buffer sets (as the BAM reader does): every batch is
    still intact when its copy is queued and when its submit runs, whatever the relative speeds."""
    import random
    import threading
    import time
    from firepony_gb300.engine import Engine

    sets = [None] * 3
    lock = threading.Lock()
    seen = []

    class Decoded:
        def __init__(self, n):
            self.n = n

        def view(self, _cls=None):
            return self

    def decoder(count):
        for n in range(count):
            time.sleep(random.uniform(0, 0.003))
            with lock:
                sets[n % 3] = n  # overwrites the set of batch n - 3
            yield Decoded(n)

    class FakeEngine(Engine):
        def __init__(self):  # no device: only the host-side pipelining is exercised
            pass

        def prefetch_view(self, v):
            with lock:
                assert sets[v.n % 3] == v.n, f"batch {v.n} overwritten before its copy was queued"

        def submit_view(self, v):
            time.sleep(random.uniform(0, 0.003))
            with lock:
                assert sets[v.n % 3] == v.n, f"batch {v.n} overwritten while submitted"
            seen.append(v.n)

        def __del__(self):
            pass

    random.seed(3)
    for count in (0, 1, 2, 3, 7, 40):
        seen.clear()
        FakeEngine().submit_threaded(decoder(count), buffers=3)
        assert seen == list(range(count))


def test_threaded_submit_error_does_not_hang():
    """A failing submit ends submit_threaded with that error; the decoder thread is stopped, not left blocked."""
    import pytest
    from firepony_gb300.engine import Engine

    class FailingEngine(Engine):
        def __init__(self):
            pass

        def prefetch_view(self, v):
            pass

        def submit_view(self, v):
            raise RuntimeError("submit failed")

        def __del__(self):
            pass

    class B:
        def view(self, _cls=None):
            return self

    def endless():
        while True:
            yield B()

    with pytest.raises(RuntimeError, match="submit failed"):
        FailingEngine().submit_threaded(endless(), buffers=3)
