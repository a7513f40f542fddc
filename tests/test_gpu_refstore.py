"""Reference store on the GPU: engines attached to one device copy (from a published shared-memory segment)
give the oracle's tables, share the copy, and keep the store alive while attached."""
import os

import numpy as np
import pytest

from tests.conftest import make_dataset
from tests.test_gpu_parity import assert_tables_equal, run_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dataset():
    return make_dataset("precision_20M_151bp_pe", 12000, 6000, 600_000)


@pytest.fixture
def shm_name(request):
    name = f"/fpgb_gtest_{os.getpid()}_{request.node.name[:40]}"
    yield name
    from firepony_gb300.refstore import RefStore
    RefStore.unlink(name)


def run(engine, batches):
    for b in batches:
        engine.submit(b)
    return engine.finalize()


def test_engine_on_published_store_matches_oracle(native, dataset, shm_name):
    from firepony_gb300.engine import Engine
    from firepony_gb300.refstore import RefStore
    p, ref, batches = dataset
    RefStore.build(ref).publish(shm_name)
    store = RefStore.open(shm_name)
    e = Engine(num_read_groups=p.num_read_groups)
    try:
        e.attach_refstore(store)
        info = store.info()
        assert info["device"] == 0 and info["attached_engines"] == 1 and info["mapped"] == 1
        got = run(e, batches)
    finally:
        e.close()
    assert store.info()["attached_engines"] == 0
    store.close()
    want, _, _ = run_oracle(ref, batches, p.num_read_groups)
    assert_tables_equal(got, want)


def test_engines_share_one_copy_and_keep_it_alive(native, dataset):
    from firepony_gb300.engine import Engine, EngineError
    from firepony_gb300.refstore import RefStore, RefStoreError
    p, ref, batches = dataset
    store = RefStore.build(ref)
    store.upload(0)
    with pytest.raises(RefStoreError, match="device copy"):
        store.set_contig(0, np.zeros(1, np.uint32), 8)
    e1 = Engine(num_read_groups=p.num_read_groups)
    e2 = Engine(num_read_groups=p.num_read_groups)
    try:
        e1.attach_refstore(store)
        e2.attach_refstore(store)
        assert store.info()["attached_engines"] == 2
        with pytest.raises(RefStoreError, match="still read"):
            store.close()
        with pytest.raises(EngineError, match="attached reference store"):
            e1.set_contig(0, np.zeros(1, np.uint32), 8)
        # the two engines run interleaved batches on the shared copy
        for b in batches:
            e1.submit(b)
            e2.submit(b)
        t1, t2 = e1.finalize(), e2.finalize()
        assert_tables_equal(t1, t2)
        # detached, an engine takes its own reference again
        e1.attach_refstore(None)
        assert store.info()["attached_engines"] == 1
        e1.reset()
        e1.load_reference(ref)
        assert_tables_equal(run(e1, batches), t1)
    finally:
        e1.close()
        e2.close()
    assert store.info()["attached_engines"] == 0
    store.close()
    want, _, _ = run_oracle(ref, batches, p.num_read_groups)
    assert_tables_equal(t1, want)


def test_job_server_engines_share_the_store(native, dataset):
    from firepony_gb300.serve import JobServer, jobs_from_pool, run_schedule
    p, ref, batches = dataset
    server = JobServer(ref, p.num_read_groups, slots=3, keep_tables=True)
    try:
        assert server.store.info()["attached_engines"] == 3
        res = run_schedule(server, jobs_from_pool(batches, [5000, 12000, 700], batch_reads=2000), [0.0, 0.0, 0.0])
    finally:
        server.close()
    for r, size in zip(res, [5000, 12000, 700]):
        assert r.error is None, r.error
        sub = []
        left = size
        for b in batches:
            n = min(left, b.num_reads)
            if n:
                sub.append(b.range(0, n))
            left -= n
        want, _, _ = run_oracle(ref, sub, p.num_read_groups)
        assert_tables_equal(r.tables, want)
