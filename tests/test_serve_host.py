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


def test_admission_by_hbm_footprint():
    """Jobs start in arrival order once a slot is free and the running jobs' estimated device memory plus their
    own fits the budget; a job larger than the budget runs alone."""
    import time
    from firepony_gb300.serve import Job, JobServer, run_schedule

    class FakeEngine:  # host-only stand-in: a job takes one short sleep per batch
        def reset(self):
            pass

        def submit_pipelined(self, batches):
            for _ in batches:
                time.sleep(0.01)

        def finalize(self):
            return {}

        def close(self):
            pass

    footprints = [60, 50, 30, 10, 80, 150, 5, 45, 55, 20]
    jobs = [Job(i, 100, (lambda: iter(range(4))), footprint=f) for i, f in enumerate(footprints)]
    server = JobServer(None, 1, slots=3, hbm_budget_bytes=100, engine_factory=FakeEngine)
    try:
        results = run_schedule(server, jobs, [0.0] * len(jobs))
    finally:
        server.close()
    assert all(r.error is None for r in results)
    # arrival order of the starts (no job passes an earlier one)
    starts = [r.start for r in results]
    assert starts == sorted(starts)
    # at every start, the jobs running together fit the budget (or one job runs alone)
    for r in results:
        live = [f for q, f in zip(results, footprints) if q.start <= r.start < q.done]
        assert len(live) <= 3
        assert len(live) == 1 or sum(live) <= 100, (r.job_id, live)
    assert server.peak_running >= 2  # the budget still lets jobs run side by side
    assert server.in_use == 0 and server.running == 0
