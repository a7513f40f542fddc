"""An independent restatement of the reference's GATKReport output, for checking fp_report_write — TEST CODE.

Written from the reference's sources, not from this project's writer:
  * table_formatter (table_formatter.cu:34-231): columns take the width of their name, widened in a first pass
    over the rows; string/char columns align left and numbers right unless given; the header line lists the
    printf conversions; a data cell is padded to the column width, cells are joined by two spaces, every row
    ends in a newline and every table in an empty line.
  * round_n (device/util.cu:107-116): value * 10^n, C round() (half away from zero), / 10^n, before %.2f / %.4f.
  * output_header (device/pipeline.cu:150-204): the fixed Arguments table, then a Quantized table of 94 rows.
  * RecalTable0 (device/read_group_table.cu:96-143), RecalTable1 (device/covariates/packer_quality_score.h:65-117),
    RecalTable2 with the context rows then the cycle rows (device/covariates.cu:285-311,
    device/covariates/packer_context.h:82-130, device/covariates/packer_cycle_illumina.h:68-110); rows with no
    observations are skipped in tables 1 and 2.
Key layouts: quality (rg << 10 | q << 2 | event), cycle (rg << 20 | q << 12 | cycle << 2 | event),
context (rg << 21 | q << 13 | context << 2 | event), read-group table keys with the quality bits zero.
"""
from __future__ import annotations

import math

STRING, CHAR, UINT64, FLOAT_2, FLOAT_4 = range(5)
LEFT, RIGHT, DEFAULT = range(3)
EVENT_CHAR = {0: "M", 1: "I", 2: "D", 3: "S"}  # cigar_event::ascii (device/cigar.h:58-65)
DNA_CHAR = "ACGT"                                # from_nvbio::dna_to_char (device/from_nvbio/dna.h:38-45)


def c_round(x: float) -> float:
    """C round(): halfway cases away from zero (modf is exact, so no double rounding)."""
    frac, whole = math.modf(x)
    if abs(frac) >= 0.5:
        return whole + math.copysign(1.0, x)
    return whole


def round_n(val: float, n: int) -> float:
    val = val * math.pow(10.0, n)
    val = c_round(val)
    return val / math.pow(10.0, n)


class Table:
    def __init__(self, name: str, description: str = "", disable_rounding: bool = False):
        self.name, self.description, self.disable = name, description, disable_rounding
        self.cols = []  # [name, fmt, align, header_align, width]
        self.rows = []

    def add_column(self, name, fmt, align=DEFAULT, header_align=DEFAULT):
        if align == DEFAULT:
            align = LEFT if fmt in (STRING, CHAR) else RIGHT
        if header_align == DEFAULT:
            header_align = align
        self.cols.append([name, fmt, align, header_align, len(name)])

    def cell(self, i, val) -> str:
        fmt = self.cols[i][1]
        if isinstance(val, str) and fmt in (STRING, CHAR):
            return val
        if fmt == UINT64:
            return "%d" % val
        if fmt in (FLOAT_2, FLOAT_4):
            if self.disable:
                return "%.64f" % val
            n = 2 if fmt == FLOAT_2 else 4
            return ("%%.%df" % n) % round_n(val, n)
        return str(val)

    def row(self, *vals):
        cells = [self.cell(i, v) for i, v in enumerate(vals)]
        for i, c in enumerate(cells):
            self.cols[i][4] = max(self.cols[i][4], len(c))
        self.rows.append(cells)

    def render(self) -> str:
        conv = {STRING: "%s:", CHAR: "%s:", UINT64: "%d:",
                FLOAT_2: "%.64f:" if self.disable else "%.2f:", FLOAT_4: "%.64f:" if self.disable else "%.4f:"}
        out = ["#:GATKTable:%d:%d:" % (len(self.cols), len(self.rows)) + "".join(conv[c[1]] for c in self.cols) + ";\n",
               "#:GATKTable:%s:%s\n" % (self.name, self.description)]

        def pad(s, width, align):
            return s.rjust(width) if align == RIGHT else s.ljust(width)
        out.append("  ".join(pad(c[0], c[4], c[3]) for c in self.cols) + "\n")
        for r in self.rows:
            out.append("  ".join(pad(s, self.cols[i][4], self.cols[i][2]) for i, s in enumerate(r)) + "\n")
        out.append("\n")
        return "".join(out)


ARGUMENTS = [
    ("binary_tag_name", "null"), ("covariate", "ReadGroupCovariate,QualityScoreCovariate,ContextCovariate,CycleCovariate"),
    ("default_platform", "null"), ("deletions_default_quality", "45"), ("force_platform", "null"),
    ("indels_context_size", "3"), ("insertions_default_quality", "45"), ("low_quality_tail", "2"),
    ("maximum_cycle_value", "500"), ("mismatches_context_size", "2"), ("mismatches_default_quality", "-1"),
    ("no_standard_covs", "false"), ("quantizing_levels", "16"), ("recalibration_report", "null"),
    ("run_without_dbsnp", "false"), ("solid_nocall_strategy", "THROW_EXCEPTION"), ("solid_recal_mode", "SET_Q_ZERO"),
]


def header(version=(1, 1, 1)) -> str:
    # output_header prints these lines with fixed padding: argument names to 28 characters, values to 72
    lines = ["#:GATKReport.v1.1:5\n", "#:GATKTable:2:18:%s:%s:;\n",
             "#:GATKTable:Arguments:Recalibration argument collection values used in this run\n",
             "Argument".ljust(28) + "Value".ljust(72) + "\n"]
    for k, v in ARGUMENTS:
        lines.append(k.ljust(28) + v.ljust(72) + "\n")
    # the software line is a fixed format string: 'Firepony_%d.%d.%d' followed by 55 spaces
    lines.append("software".ljust(28) + "Firepony_%d.%d.%d" % version + " " * 55 + "\n")
    lines.append("\n")
    q = Table("Quantized", "Quality quantization map")
    for name in ("QualityScore", "Count", "QuantizedScore"):
        q.add_column(name, STRING, RIGHT)
    for i in range(94):
        q.row(str(i), "0", str(i))
    return "".join(lines) + q.render()


def report(tables: dict, rg_names, disable_rounding=False, version=(1, 1, 1)) -> str:
    """The whole report from the four finalized tables (fp_table_id order: read group, quality, cycle, context),
    each a dict of arrays keys / observations / mismatches / estimated_quality / empirical_quality."""
    out = [header(version)]
    t0 = Table("RecalTable0", disable_rounding=disable_rounding)
    t0.add_column("ReadGroup", STRING)
    t0.add_column("EventType", CHAR)
    t0.add_column("EmpiricalQuality", FLOAT_4)
    t0.add_column("EstimatedQReported", FLOAT_4)
    t0.add_column("Observations", UINT64)
    t0.add_column("Errors", FLOAT_2, RIGHT, LEFT)
    d = tables[0]
    for i in range(len(d["keys"])):
        k = int(d["keys"][i])
        t0.row(rg_names[k >> 10], EVENT_CHAR[k & 3], float(d["empirical_quality"][i]),
               float(d["estimated_quality"][i]), int(d["observations"][i]), float(d["mismatches"][i]))
    out.append(t0.render())

    t1 = Table("RecalTable1", disable_rounding=disable_rounding)
    t1.add_column("ReadGroup", STRING)
    t1.add_column("QualityScore", STRING)
    t1.add_column("EventType", CHAR)
    t1.add_column("EmpiricalQuality", FLOAT_4)
    t1.add_column("Observations", UINT64)
    t1.add_column("Errors", FLOAT_2, RIGHT, LEFT)
    d = tables[1]
    for i in range(len(d["keys"])):
        if int(d["observations"][i]) == 0:
            continue
        k = int(d["keys"][i])
        t1.row(rg_names[k >> 10], "%d" % ((k >> 2) & 0xFF), EVENT_CHAR[k & 3], float(d["empirical_quality"][i]),
               int(d["observations"][i]), float(d["mismatches"][i]))
    out.append(t1.render())

    t2 = Table("RecalTable2", disable_rounding=disable_rounding)
    t2.add_column("ReadGroup", STRING)
    t2.add_column("QualityScore", STRING)
    t2.add_column("CovariateValue", STRING)
    t2.add_column("CovariateName", STRING)
    t2.add_column("EventType", CHAR)
    t2.add_column("EmpiricalQuality", FLOAT_4)
    t2.add_column("Observations", UINT64)
    t2.add_column("Errors", FLOAT_2, RIGHT, LEFT)
    d = tables[3]  # context rows first
    for i in range(len(d["keys"])):
        if int(d["observations"][i]) == 0:
            continue
        k = int(d["keys"][i])
        raw = (k >> 2) & 0x7FF
        size, ctx = raw & 0xF, raw >> 4
        seq = "".join(DNA_CHAR[(ctx >> (2 * j)) & 3] for j in range(size))
        t2.row(rg_names[k >> 21], "%d" % ((k >> 13) & 0xFF), seq, "Context", EVENT_CHAR[k & 3],
               float(d["empirical_quality"][i]), int(d["observations"][i]), float(d["mismatches"][i]))
    d = tables[2]  # then the cycle rows
    for i in range(len(d["keys"])):
        if int(d["observations"][i]) == 0:
            continue
        k = int(d["keys"][i])
        raw = (k >> 2) & 0x3FF
        group = -(raw >> 1) if raw & 1 else raw >> 1
        t2.row(rg_names[k >> 20], "%d" % ((k >> 12) & 0xFF), "%d" % group, "Cycle", EVENT_CHAR[k & 3],
               float(d["empirical_quality"][i]), int(d["observations"][i]), float(d["mismatches"][i]))
    out.append(t2.render())
    return "".join(out)
