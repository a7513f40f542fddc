"""CPU tests of bench.py's helpers: the measured peak it divides by, and that a failing side measurement is
reported in its own field instead of ending the run."""
import json
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_measured_peak_is_read_from_the_peaks_file():
    import bench
    peaks = ROOT / "MEASURED_PEAKS.json"
    got = bench._measured_peak_gbs()
    if peaks.exists():
        assert got == float(json.loads(peaks.read_text()).get("hbm_gbs", 6800.0))
    else:
        assert got == 6800.0


def test_failing_leg_is_reported_not_raised():
    import bench

    def boom(x):
        raise RuntimeError(f"no {x}")

    out = bench._leg(boom, "gpu")
    assert out == {"error": "RuntimeError: no gpu"}
    assert bench._leg(lambda a, b: a + b, 2, 3) == 5


def test_cpu_baseline_times_the_oracle_on_prebuilt_ranges():
    """The CPU leg's 1000-read sub-batches are zero-copy ranges that cover the batch in order, and the leg
    reports the per-stage CPU breakdown in the reference's exit-statistics categories."""
    import numpy as np
    import bench
    from oracle.oracle import STAGES
    from tests.conftest import make_dataset
    p, ref, batches = make_dataset("precision_20M_151bp_pe", 2500, 2500, 300_000)
    subs = bench.cpu_sub_batches(batches[0])
    assert [s.num_reads for s in subs] == [1000, 1000, 500]
    # views, not copies: the qualities of the second range are the batch's own memory
    assert np.shares_memory(subs[1]["qualities"], batches[0]["qualities"])
    out = bench.cpu_baseline(ref, batches, 0.2)
    assert out["value"] > 0 and out["kind"] == "port"
    assert set(out["stages"]["share"]) == set(STAGES)
    assert abs(sum(out["stages"]["share"].values()) - 1.0) < 1e-3
    assert out["stages"]["thread_s"]["baq_hmm"] > 0


def test_autotune_takes_the_largest_target_the_sample_cannot_tell_apart(monkeypatch):
    """Coalescing targets at or above the sample's read count all make one device batch of the sample; when the
    fastest candidate is one of them, the largest is returned."""
    import numpy as np
    from firepony_gb300 import autotune as at

    class B:
        num_reads = 1000

    tables = {0: {"keys": np.arange(3)}}
    times = {(0, 0): 3.0, (0, 500): 2.0, (0, 2000): 1.0, (0, 8000): 1.1, (4, 0): 5.0, (4, 500): 5.0,
             (4, 2000): 5.0, (4, 8000): 5.0}
    monkeypatch.setattr(at, "time_config", lambda ref, batches, n_rg, rpw, co, device=0: (times[(rpw, co)], tables))
    res = at.autotune(None, [B(), B()], 1, replay_choices=(0, 4), coalesce_choices=(0, 500, 2000, 8000))
    assert res["reads"] == 2000
    assert res["best"] == {"replay_reads_per_warp": 0, "coalesce_reads": 8000}
    times[(0, 500)] = 0.5  # a target below the sample's size that wins is kept as is
    res = at.autotune(None, [B(), B()], 1, replay_choices=(0, 4), coalesce_choices=(0, 500, 2000, 8000))
    assert res["best"]["coalesce_reads"] == 500
