"""The GATKReport writer (fp_report_write) against an independent restatement of the reference's formatter
(tests/report_restatement.py, written from table_formatter.cu, round_n and the packers' dump loops), byte for
byte, on the oracle's tables of real multi-read-group runs, with and without output rounding."""
import pytest

from tests.conftest import make_dataset


@pytest.mark.parametrize("preset,n,refbp", [("precision_20M_151bp_pe", 6000, 300_000),
                                            ("large_100M_151bp_pe", 8000, 400_000)])
@pytest.mark.parametrize("disable_rounding", [False, True])
def test_report_matches_restatement(native, tmp_path, preset, n, refbp, disable_rounding):
    from firepony_gb300.engine import write_report
    from oracle.oracle import Oracle
    from tests.report_restatement import report
    p, ref, batches = make_dataset(preset, n, n // 2, refbp)
    o = Oracle(p.num_read_groups)
    o.load_reference(ref)
    for b in batches:
        o.process(b)
    tables = o.finalize()
    names = [f"RG{i}.lane{i % 3}" for i in range(p.num_read_groups)]
    path = tmp_path / "report.txt"
    write_report(path, tables, names, disable_rounding=disable_rounding, version=(1, 1, 1))
    got = path.read_text()
    want = report(tables, names, disable_rounding=disable_rounding, version=(1, 1, 1))
    assert len(tables[2]["keys"]) > 100 and len(tables[3]["keys"]) > 100
    assert got == want
