"""Coalescing of small host batches (fp_options.coalesce_reads): many small batches of uneven read lengths are
gathered into device batches; the tables equal those of per-batch processing and the oracle's."""
import numpy as np
import pytest

from tests.test_gpu_parity import assert_tables_equal, run_oracle

pytestmark = pytest.mark.gpu


def uneven_dataset(num_batches, lo, hi, seed=11):
    """The uneven-batch workload (reads of 36-250 bp, indels, wide deletions, 16 read groups) cut into batches
    of uniformly drawn sizes in [lo, hi]."""
    from firepony_gb300 import synth
    sizes = synth.uneven_batch_sizes(num_batches, lo, hi, seed)
    p = synth.PRESETS["batched_uneven"].scaled(num_reads=int(sizes.sum()), total_reference_bp=2_000_000)
    ref = synth.Reference(p)
    return p, ref, [ref.batch(i, int(n)) for i, n in enumerate(sizes)]


def to_device(batch):
    import torch
    from firepony_gb300.abi import FpBatchView
    from firepony_gb300.synth import BATCH_FIELDS
    keep, v = [], FpBatchView()
    v.num_reads, v.num_cigar_ops = batch.num_reads, batch.num_cigar_ops
    v.num_read_symbols, v.num_qualities = batch.num_read_symbols, batch.num_qualities
    for name, _, _ in BATCH_FIELDS:
        a = batch.arrays[name]
        t = torch.from_numpy(a.view("uint8").copy()).to("cuda") if a.nbytes else torch.zeros(8, dtype=torch.uint8,
                                                                                                   device="cuda")
        keep.append(t)
        setattr(v, name, t.data_ptr())
    return keep, v


def engine_tables(p, ref, batches, coalesce, device_batches=()):
    from firepony_gb300.engine import Engine
    e = Engine(num_read_groups=p.num_read_groups, coalesce_reads=coalesce)
    e.load_reference(ref)
    for i, b in enumerate(batches):
        if i in device_batches:
            keep, v = to_device(b)
            e.submit_device_view(v)
            del keep
        else:
            e.submit(b)
    t = e.finalize()
    st = e.stats()
    e.close()
    return t, st


def test_coalesced_tables_equal_per_batch_and_oracle(native):
    p, ref, batches = uneven_dataset(40, 100, 1500)
    t1, s1 = engine_tables(p, ref, batches, 0)
    t2, s2 = engine_tables(p, ref, batches, 5000)
    assert_tables_equal(t2, t1)
    to, _, _ = run_oracle(ref, batches, p.num_read_groups)
    assert_tables_equal(t2, to)
    assert s2["num_batches"] == s1["num_batches"] == len(batches)
    assert s2["total_reads"] == s1["total_reads"] == sum(b.num_reads for b in batches)


def test_coalescing_with_device_and_large_batches(native):
    """Device batches and batches above the target are processed after the staged reads (stream order)."""
    from firepony_gb300 import synth
    p, ref, batches = uneven_dataset(24, 50, 900)
    big = ref.batch(100, 3000)
    seq = batches[:10] + [big] + batches[10:]
    t1, _ = engine_tables(p, ref, seq, 0)
    t2, _ = engine_tables(p, ref, seq, 2500, device_batches={4, 17})
    assert_tables_equal(t2, t1)


def test_coalescing_rejects_a_bad_batch_at_its_submit(native):
    from firepony_gb300.engine import Engine, EngineError
    p, ref, batches = uneven_dataset(12, 200, 600)
    e = Engine(num_read_groups=p.num_read_groups, coalesce_reads=3000)
    e.load_reference(ref)
    good = []
    for i, b in enumerate(batches):
        if i == 5:
            bad = b.subset(np.arange(b.num_reads))
            bad.arrays["read_group"][2] = p.num_read_groups  # >= num_read_groups
            with pytest.raises(EngineError, match="BAD_INPUT"):
                e.submit(bad)
            bad2 = b.subset(np.arange(b.num_reads))
            bad2.arrays["qual_start"][1] = 10**9
            with pytest.raises(EngineError, match="BAD_INPUT"):
                e.submit(bad2)
            continue
        e.submit(b)
        good.append(b)
    t = e.finalize()
    e.close()
    to, _, _ = run_oracle(ref, good, p.num_read_groups)
    assert_tables_equal(t, to)


def test_coalescing_reset_drops_staged_reads(native):
    from firepony_gb300.engine import Engine
    p, ref, batches = uneven_dataset(10, 100, 400)
    e = Engine(num_read_groups=p.num_read_groups, coalesce_reads=100000)
    e.load_reference(ref)
    for b in batches[:5]:
        e.submit(b)  # staged, not processed
    e.reset()
    for b in batches[5:]:
        e.submit(b)
    t = e.finalize()
    e.close()
    to, _, _ = run_oracle(ref, batches[5:], p.num_read_groups)
    assert_tables_equal(t, to)
