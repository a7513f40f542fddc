"""The job server on the GPU: concurrent jobs on resident engines give each job its own exact tables."""
import numpy as np
import pytest

from tests.test_gpu_parity import assert_tables_equal, run_oracle

pytestmark = pytest.mark.gpu


def test_job_server_tables_match_oracle(native):
    from firepony_gb300 import synth
    from firepony_gb300.serve import JobServer, jobs_from_pool, run_schedule
    p = synth.PRESETS["serving_mixed"].scaled(num_reads=6000, total_reference_bp=600_000, batch_reads=6000)
    ref = synth.Reference(p)
    pool = [ref.batch(0, 6000)]
    sizes = [900, 6000, 1, 2500, 4000, 300]
    jobs = jobs_from_pool(pool, sizes, batch_reads=1000)
    server = JobServer(ref, p.num_read_groups, slots=2, keep_tables=True)
    try:
        results = run_schedule(server, jobs, np.zeros(len(jobs)))
    finally:
        server.close()
    for res, size in zip(results, sizes):
        assert res.error is None, res.error
        assert res.num_reads == size and res.done >= res.start >= res.arrival
        batch = pool[0].range(0, size)
        to, _, _ = run_oracle(ref, [batch], p.num_read_groups)
        assert_tables_equal(res.tables, to)


def test_job_results_same_alone_and_in_the_mix(native):
    """Each job's tables are the same when it runs alone on the server and when it runs beside others (three
    slots, every job arriving at once, an HBM budget admitting at most two at a time)."""
    from firepony_gb300 import synth
    from firepony_gb300.serve import JobServer, estimate_job_bytes, jobs_from_pool, run_schedule
    p = synth.PRESETS["serving_mixed"].scaled(num_reads=8000, total_reference_bp=600_000, batch_reads=8000)
    ref = synth.Reference(p)
    pool = [ref.batch(0, 8000)]
    sizes = [5000, 700, 8000, 1200, 3000, 40]
    alone = {}
    server = JobServer(ref, p.num_read_groups, slots=1, keep_tables=True)
    try:
        for job in jobs_from_pool(pool, sizes, batch_reads=1500):
            res = run_schedule(server, [job], [0.0])[0]
            assert res.error is None, res.error
            alone[job.job_id] = res.tables
    finally:
        server.close()
    budget = 2 * estimate_job_bytes(1500) + 1  # the largest batches of two jobs
    server = JobServer(ref, p.num_read_groups, slots=3, keep_tables=True, hbm_budget_bytes=budget)
    try:
        mix = run_schedule(server, jobs_from_pool(pool, sizes, batch_reads=1500), np.zeros(len(sizes)))
        peak = server.peak_running
    finally:
        server.close()
    assert 1 <= peak <= 2
    for r in mix:
        assert r.error is None, r.error
        assert_tables_equal(r.tables, alone[r.job_id])
