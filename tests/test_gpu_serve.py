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
