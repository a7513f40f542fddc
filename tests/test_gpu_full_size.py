"""GPU parity at the benchmark configurations' full sizes: the engine against the oracle on a full-size batch
of each configuration's reference (all contigs and known sites), with the per-stage intermediates and all four
tables compared, plus the FP32 precision trace.

* precision configuration: one whole 1M-read batch of 151 bp pairs over 5 contigs / 50 Mbp with 50k SNP and
  5k indel sites (the timed batch shape);
* large single run: 500k reads over 3 contigs / 250 Mbp with 3M SNP and 300k indel sites, 32 read groups,
  duplicates and unmapped / MAPQ-0 reads (the known-site search over a large VCF, many read groups);
* uneven batches: 96 of the configuration's input batches (2k-40k reads, 36-250 bp, wide deletions, 16 read
  groups) coalesced by the engine;
* serving configuration: 200k reads over its shared 250 Mbp reference with 500k sites."""
import numpy as np
import pytest

from tests.test_gpu_parity import assert_stages_equal, assert_tables_equal, run_engine, run_oracle

pytestmark = pytest.mark.gpu


def full_reference(preset_name, num_reads, batch_reads):
    from firepony_gb300 import synth
    p = synth.PRESETS[preset_name].scaled(num_reads=num_reads, batch_reads=batch_reads)
    return p, synth.Reference(p)


def test_precision_config_full_batch(native):
    p, ref = full_reference("precision_20M_151bp_pe", 1_000_000, 1_000_000)
    assert p.total_reference_bp == 50_000_000 and sum(len(s[0]) for s in ref.sites) > 50_000
    batch = ref.batch(0, 1_000_000)
    te, se, ge = run_engine(ref, [batch], p.num_read_groups, "fp32")
    to, so, go = run_oracle(ref, [batch], p.num_read_groups)
    assert se["total_reads"] == so["total_reads"] == 1_000_000
    assert se["filtered_reads"] == so["filtered_reads"]
    assert se["baq_reads"] == so["baq_reads"]
    assert_stages_equal(batch, ge, go)
    assert_tables_equal(te, to)


def test_large_config_500k_reads(native):
    p, ref = full_reference("large_100M_151bp_pe", 500_000, 500_000)
    assert p.total_reference_bp == 250_000_000 and p.num_read_groups == 32
    assert sum(len(s[0]) for s in ref.sites) > 3_000_000
    batch = ref.batch(0, 500_000)
    te, se, ge = run_engine(ref, [batch], p.num_read_groups, "fp32")
    to, so, go = run_oracle(ref, [batch], p.num_read_groups)
    # duplicates (5%) and unmapped / MAPQ-0 reads (1%) are filtered alike
    assert se["filtered_reads"] == so["filtered_reads"] > 0.05 * 500_000
    assert se["baq_reads"] == so["baq_reads"]
    assert_stages_equal(batch, ge, go)
    assert_tables_equal(te, to)


def test_uneven_config_96_batches_coalesced(native):
    from firepony_gb300 import synth
    from firepony_gb300.engine import Engine
    sizes = synth.uneven_batch_sizes(96, 2000, 40000, seed=2)
    p = synth.PRESETS["batched_uneven"].scaled(num_reads=int(sizes.sum()))
    assert p.total_reference_bp == 100_000_000
    ref = synth.Reference(p)
    batches = [ref.batch(i, int(n)) for i, n in enumerate(sizes)]
    e = Engine(num_read_groups=p.num_read_groups, coalesce_reads=1_000_000)
    try:
        e.load_reference(ref)
        for b in batches:
            e.submit(b)
        te = e.finalize()
        se = e.stats()
    finally:
        e.close()
    to, so, _ = run_oracle(ref, batches, p.num_read_groups)
    assert se["total_reads"] == so["total_reads"] == int(sizes.sum())
    assert se["baq_reads_by_band"][2] > 0
    assert_tables_equal(te, to)


def test_serving_config_reference(native):
    p, ref = full_reference("serving_mixed", 200_000, 200_000)
    assert p.total_reference_bp == 250_000_000
    batch = ref.batch(0, 200_000)
    te, se, ge = run_engine(ref, [batch], p.num_read_groups, "fp32")
    to, so, go = run_oracle(ref, [batch], p.num_read_groups)
    assert_stages_equal(batch, ge, go)
    assert_tables_equal(te, to)


def test_precision_trace_certificate_holds(native):
    """The FP32 certified interval holds the FP64 value for every compared base, over a 300k-read sample of
    the precision configuration; the trace leaves the results unchanged."""
    from firepony_gb300.abi import FP_FLAG_PRECISION_TRACE
    from firepony_gb300.engine import Engine
    p, ref = full_reference("precision_20M_151bp_pe", 300_000, 150_000)
    batches = [ref.batch(i, 150_000) for i in range(2)]
    e = Engine(num_read_groups=p.num_read_groups, flags=FP_FLAG_PRECISION_TRACE)
    try:
        e.load_reference(ref)
        for b in batches:
            e.submit(b)
        t = e.finalize()
        ps = e.precision_stats()
        st = e.stats()
    finally:
        e.close()
    t_plain, _, _ = run_engine(ref, batches, p.num_read_groups, "fp32")
    assert_tables_equal(t, t_plain)
    assert ps["bound_violations"] == 0
    assert ps["reads"] + ps["reads_without_fp32"] == st["baq_reads"]
    assert ps["reads"] > 0.95 * st["baq_reads"]
    # about half of a read's bases have an FP64 t below 101 (the rest saturate at 99 either way)
    assert ps["bases"] > 20 * ps["reads"]
    assert sum(ps["err_hist"]) == ps["reads"] == sum(ps["width_hist"])
    # FP32 against FP64: far inside a quality unit
    assert 0 < ps["max_abs_error"] < 0.05
