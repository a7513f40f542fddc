"""Hand-built alignment batch covering the reference's special cases: every read filter, clip layouts,
leading/trailing insertions, deletions, '=' and X ops, N bases, low-quality tails, qualities above 93, reads at
both contig ends, adapter clipping of short fragments, wide bands, known sites under reads, and malformed
input."""
from __future__ import annotations

import re

import numpy as np

from firepony_gb300.synth import Batch, pack4

OPS = {"M": 0, "I": 1, "D": 2, "N": 3, "S": 4, "H": 5, "P": 6, "=": 7, "X": 8}
IUPAC = {"A": 1, "C": 2, "G": 4, "T": 8, "N": 15}
DNA = "ACGT"


def make_reference(n=3000, seed=7):
    rng = np.random.default_rng(seed)
    seq = "".join(rng.choice(list(DNA), size=n))
    return seq


def parse_cigar(c):
    return [(int(n), op) for n, op in re.findall(r"(\d+)([MIDNSHP=X])", c)]


def read_from_cigar(ref, pos, cigar, rng, sub_positions=(), qual=30, n_at=()):
    """Read bases following the CIGAR over ref[pos:], with substitutions at the given read offsets."""
    seq = []
    rp = pos
    for n, op in parse_cigar(cigar):
        for _ in range(n):
            if op in "M=X":
                seq.append(ref[rp] if rp < len(ref) else "A")
                rp += 1
            elif op in "IS":
                seq.append(DNA[rng.integers(4)])
            elif op in "DNHP":
                if op in "DN":
                    rp += 1
    seq = list(seq)
    for i in sub_positions:
        if i < len(seq):
            seq[i] = {"A": "C", "C": "G", "G": "T", "T": "A"}[seq[i]]
    for i in n_at:
        if i < len(seq):
            seq[i] = "N"
    quals = np.full(len(seq), qual, np.uint8)
    span = sum(n for n, op in parse_cigar(cigar) if op in "M=XDN")
    return "".join(seq), quals, span


def build_batch(records):
    """records: dicts with keys pos, cigar, seq, quals, flags, mapq, rg, chrom, mate_pos, isize."""
    R = len(records)
    chrom = np.array([r.get("chrom", 0) for r in records], np.uint16)
    astart = np.array([r["pos"] for r in records], np.uint32)
    astop = np.array([r["pos"] + max(r.get("span", 1), 1) - 1 for r in records], np.uint32)
    mstart = np.array([r.get("mate_pos", 0) for r in records], np.uint32)
    isize = np.array([r.get("isize", 0) for r in records], np.int32)
    cig, cstart, clen = [], [], []
    syms, rstart, rlen = [], [], []
    quals, qstart, qlen = [], [], []
    for r in records:
        ops = parse_cigar(r["cigar"])
        cstart.append(len(cig))
        clen.append(len(ops))
        cig.extend((n & 0xFFFFFF) | (OPS[op] << 24) for n, op in ops)
        s = [IUPAC[c] for c in r["seq"]]
        pad = (len(s) + 7) // 8 * 8
        rstart.append(len(syms))
        rlen.append(len(s))
        syms.extend(s + [0] * (pad - len(s)))
        q = list(r["quals"])
        qstart.append(len(quals))
        qlen.append(r.get("qual_len", len(q)))
        quals.extend(q)
    arrays = {
        "chromosome": chrom, "alignment_start": astart, "alignment_stop": astop, "mate_alignment_start": mstart,
        "inferred_insert_size": isize, "cigars": np.array(cig, np.uint32), "cigar_start": np.array(cstart, np.uint32),
        "cigar_len": np.array(clen, np.uint32), "reads": pack4(np.array(syms, np.uint8)),
        "read_start": np.array(rstart, np.uint32), "read_len": np.array(rlen, np.uint32),
        "qualities": np.array(quals, np.uint8), "qual_start": np.array(qstart, np.uint32),
        "qual_len": np.array(qlen, np.uint32), "flags": np.array([r.get("flags", 0) for r in records], np.uint16),
        "mapq": np.array([r.get("mapq", 60) for r in records], np.uint8),
        "read_group": np.array([r.get("rg", 0) for r in records], np.uint32),
    }
    return Batch(arrays, R, len(cig), len(syms), len(quals))


def edge_case_dataset(seed=11):
    """Returns (contigs, sites, batch): contigs as [(words, n)], sites as [(start, stop)]."""
    rng = np.random.default_rng(seed)
    ref = make_reference(3000, seed)
    L = len(ref)
    recs = []

    def add(pos, cigar, subs=(), flags=0, mapq=60, rg=0, qual=30, quals=None, n_at=(), chrom=0, mate_pos=0,
            isize=0, qual_len=None):
        seq, q, span = read_from_cigar(ref, pos, cigar, rng, subs, qual, n_at)
        if quals is not None:
            q = np.array(quals, np.uint8)[:len(seq)]
        rec = dict(pos=pos, cigar=cigar, seq=seq, quals=q, flags=flags, mapq=mapq, rg=rg, chrom=chrom,
                   mate_pos=mate_pos, isize=isize, span=span)
        if qual_len is not None:
            rec["qual_len"] = qual_len
        recs.append(rec)

    REV, PAIRED, READ2, MREV = 16, 1, 128, 32
    add(100, "50M", subs=(10, 30))
    add(120, "50M", subs=(5,), flags=REV)
    add(140, "5S40M5S", subs=(20,))
    add(160, "3H47M", subs=(12,))
    add(180, "47M3H", subs=(40,), flags=REV)
    add(200, "10M2I38M", subs=(25,))
    add(220, "10M2I38M", subs=(25,), flags=REV)
    add(240, "10M3D40M", subs=(35,))
    add(260, "10M3D40M", subs=(35,), flags=REV)
    add(280, "2I48M", subs=(30,))
    add(300, "48M2I", subs=(20,), flags=REV)
    add(320, "5S2I43M", subs=(15,))
    add(340, "2D48M", subs=(22,))
    add(360, "20M1D1I29M", subs=(3,))
    add(380, "20=5X25M", subs=(21, 40))
    add(400, "50M", subs=(12,), n_at=(25,))
    add(420, "50M", subs=(12,), quals=[30] * 10 + [4] * 5 + [30] * 33 + [2, 2])
    add(440, "50M", subs=(12,), quals=[2, 2, 2] + [25] * 47)
    add(460, "50M", mapq=0)
    add(480, "50M", mapq=255)
    add(500, "50M", flags=1024)
    add(520, "50M", flags=512)
    add(540, "50M", flags=256)
    add(560, "50M", flags=4)
    add(580, "20M5N30M")
    add(600, "10M5S10M")
    add(620, "5H5S40M", subs=(10,))
    add(640, "5S5H40M")
    add(0, "50M", subs=(10,))
    add(1, "50M", subs=(10,), flags=REV)
    add(2, "3S47M", subs=(10,))
    add(L - 50, "50M", subs=(10,))
    add(L - 48, "48M", subs=(10,), flags=REV)
    add(L - 20, "40M", subs=(5,))
    add(L - 60, "50M", subs=(10,))
    add(700, "50M", subs=(10, 45), flags=PAIRED | MREV, mate_pos=705, isize=40)
    add(705, "50M", subs=(3, 44), flags=PAIRED | REV | READ2, mate_pos=700, isize=-40)
    add(740, "5S45M", subs=(10,), flags=PAIRED | MREV, mate_pos=760, isize=60)
    add(760, "45M5S", subs=(30,), flags=PAIRED | REV | READ2, mate_pos=740, isize=-60)
    add(800, "50M", rg=0xFFFFFFFF)
    add(820, "30M15D20M", subs=(10, 40))
    add(860, "25M10D25M", subs=(5, 30), flags=REV)
    add(900, "1M")
    add(910, "50M", chrom=5)
    add(920, "50M", qual_len=40)
    add(1000, "150M", subs=(20, 70, 140))
    add(1200, "60M", subs=(0, 59))
    add(1300, "30M4I30M", subs=(31, 32))
    add(1400, "40M", quals=[40] * 40)
    add(1500, "100M", subs=tuple(range(0, 100, 7)), flags=PAIRED | READ2)
    add(1650, "511M", subs=(100, 300, 500)) if L > 2200 else None
    add(1800, "70M", subs=(35,), rg=1)
    add(1850, "70M", subs=(35,), rg=2, flags=REV)
    # base qualities above 93 (emissions below the FP32 kernels' range arguments; 0xFF = missing qualities):
    # band classes 0, 1 and 2
    add(2250, "50M", subs=(10, 30), quals=[255] * 50)
    add(2320, "30M3D20M", subs=(5,), quals=[120] * 50)
    add(2400, "25M20D25M", subs=(3, 40), quals=[93] * 20 + [200] * 30)

    # known sites: SNPs under reads 0, 5, 9; an indel site; a site at the read edge
    sites = sorted([(110, 110), (130, 130), (215, 215), (245, 247), (289, 289), (1010, 1012), (1220, 1220),
                    (1259, 1259), (1815, 1815)])
    batch = build_batch(recs)
    seq_syms = np.array([IUPAC[c] for c in ref], np.uint8)
    contigs = [(pack4(seq_syms), L)]
    st = np.array([s for s, _ in sites], np.uint32)
    sp = np.array([e for _, e in sites], np.uint32)
    return contigs, [(st, sp)], batch, 3


def _flank(rng, n, avoid_first=None, avoid_last=None):
    """Random bases with no two equal neighbours, so that no homopolymer run other than the planted one sits
    near a junction; avoid_first / avoid_last keep the ends off the run's base."""
    out = []
    for i in range(n):
        while True:
            c = DNA[rng.integers(4)]
            if out and c == out[-1]:
                continue
            if i == 0 and c == avoid_first:
                continue
            if i == n - 1 and c == avoid_last:
                continue
            break
        out.append(c)
    return "".join(out)


def tied_indel_dataset(seed=21, tie_quals=(2, 3, 4, 30)):
    """Reads whose BAQ posterior at one base splits evenly between two states: a one-base deletion from a
    two-base homopolymer run (the remaining copy aligns to either reference base with the same path weight,
    so the two posteriors agree to about 1e-6 or closer), and a one-base insertion into a single-base run (either
    read copy can be the inserted one; those posteriors split about 0.50 / 0.44). The reference's MAP quality
    there is MIN_BASE_QUAL whichever state wins (device/baq.cu:673), and the capped quality
    (device/baq.cu:895-909) is min(bq, oq) at the expected match and MIN_BASE_QUAL elsewhere, so the winner
    only matters when the tied base's quality is below MIN_BASE_QUAL. Each placement comes with the tied-base
    qualities tie_quals, both CIGAR placements, on both strands, at band widths 7, 14-16, 25-27 and 45-47 (a
    second deletion of 0, 9, 20 or 40 bases later in the read).

    Returns (contigs, sites, batch, num_read_groups, low_quality_tie) where low_quality_tie marks the reads
    whose tied base has quality below MIN_BASE_QUAL."""
    rng = np.random.default_rng(seed)
    parts, motifs = [], []
    pos = 0

    def put(s):
        nonlocal pos
        parts.append(s)
        pos += len(s)

    REV = 16
    combos = [(kind, q, flags, extra) for extra in (0, 9, 20, 40) for q in tie_quals for flags in (0, REV)
              for kind in ("del", "ins")]
    put(_flank(rng, 40))
    for kind, _, _, _ in combos:
        x = DNA[rng.integers(4)]
        left = _flank(rng, 30, avoid_first=parts[-1][-1], avoid_last=x)
        right = _flank(rng, 100, avoid_first=x)
        put(left)
        run_at = pos
        put(x * (2 if kind == "del" else 1))
        put(right)
        motifs.append(run_at)
        put(_flank(rng, 20, avoid_first=right[-1]))
    ref = "".join(parts)
    recs, low = [], []
    for run_at, (kind, q, flags, extra) in zip(motifs, combos):
        x = ref[run_at]
        for variant in (0, 1):
            start = run_at - 20
            # del: variant 0 deletes the run's second copy (the read's copy is expected at the first), variant 1
            # the first copy; ins: variant 0 inserts the read's second copy, variant 1 its first. Both variants
            # of a placement are the same read; the second deletion follows read offset 30.
            head = f"{21 - variant}M1{'D' if kind == 'del' else 'I'}"
            rest = 50 - (22 if kind == "ins" else 21) + variant
            cigar = f"{head}{rest - 19}M{extra}D19M" if extra else f"{head}{rest}M"
            seq, quals, span = read_from_cigar(ref, start, cigar, rng)
            if kind == "ins":
                seq = seq[:20] + x + x + seq[22:]
            quals = quals.copy()
            quals[20:22 if kind == "ins" else 21] = q
            recs.append(dict(pos=start, cigar=cigar, seq=seq, quals=quals, flags=flags, mapq=60, rg=0, span=span))
            low.append(q < 4)
    batch = build_batch(recs)
    seq_syms = np.array([IUPAC[c] for c in ref], np.uint8)
    contigs = [(pack4(seq_syms), len(ref))]
    st = np.zeros(0, np.uint32)
    return contigs, [(st, st.copy())], batch, 1, np.array(low, bool)
