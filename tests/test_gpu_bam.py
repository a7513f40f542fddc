"""BAM file -> decoder -> engine: the tables equal the oracle's on the decoded batches."""
import numpy as np
import pytest

from tests.test_gpu_parity import assert_tables_equal, run_oracle

pytestmark = pytest.mark.gpu


def test_bam_to_tables(native, tmp_path):
    from firepony_gb300 import bam, synth
    from firepony_gb300.engine import Engine
    try:
        bam.lib()
    except RuntimeError as ex:
        pytest.skip(str(ex))
    p = synth.PRESETS["precision_20M_151bp_pe"].scaled(num_reads=6000, total_reference_bp=400_000, batch_reads=3000)
    ref = synth.Reference(p)
    batches = list(ref.batches())
    path = tmp_path / "in.bam"
    targets = [(f"chr{i}", int(n)) for i, (_, n) in enumerate(ref.contigs)]
    bam.write_bam(str(path), targets, [f"rg{i}" for i in range(p.num_read_groups)], batches)
    reader = bam.BamReader(str(path))
    e = Engine(num_read_groups=p.num_read_groups)
    e.load_reference(ref)
    decoded = []
    # decoded on a producer thread like a loader: batch n+1 is decoded and its copy queued while batch n runs
    def gen():
        for b in reader.batches(2000):
            decoded.append(b.to_batch())
            yield b
    e.submit_threaded(gen())
    tables = e.finalize()
    e.close()
    reader.close()
    assert sum(b.num_reads for b in decoded) == 6000
    to, _, _ = run_oracle(ref, decoded, p.num_read_groups)
    assert_tables_equal(tables, to)
    assert np.all(np.concatenate([b["read_group"] for b in decoded]) < p.num_read_groups)
