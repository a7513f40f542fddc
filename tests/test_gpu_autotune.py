"""The autotuner: every candidate shape gives the same tables, the best one is a candidate."""
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_small_sample(native):
    from firepony_gb300 import synth
    from firepony_gb300.autotune import autotune
    sizes = synth.uneven_batch_sizes(6, 200, 900, seed=7)
    p = synth.PRESETS["batched_uneven"].scaled(num_reads=int(sizes.sum()), total_reference_bp=1_000_000)
    ref = synth.Reference(p)
    batches = [ref.batch(i, int(n)) for i, n in enumerate(sizes)]
    res = autotune(ref, batches, p.num_read_groups, replay_choices=(0, 4), coalesce_choices=(0, 2000))
    assert len(res["results"]) == 4
    assert res["best"]["replay_reads_per_warp"] in (0, 4) and res["best"]["coalesce_reads"] in (0, 2000)
    assert all(r["reads_per_s"] > 0 for r in res["results"])
