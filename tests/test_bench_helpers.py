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
