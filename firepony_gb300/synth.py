"""Seeded synthetic inputs shaped like the benchmark configurations (see csrc/synth.cpp).

The presets reproduce the configurations' shapes and distributions; sizes can be scaled down for tests.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from .build import build_synth


class SynthConfig(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64), ("num_contigs", C.c_uint32), ("total_reference_bp", C.c_uint64), ("gc", C.c_double),
        ("read_lengths", C.c_uint32 * 8), ("num_read_lengths", C.c_uint32), ("paired", C.c_int32),
        ("sub_rate", C.c_double), ("indel_read_frac", C.c_double), ("indel_mode", C.c_int32),
        ("geometric_p", C.c_double), ("wide_deletion_frac", C.c_double), ("softclip_frac", C.c_double),
        ("short_fragment_frac", C.c_double), ("qual_mean", C.c_double), ("qual_sd", C.c_double),
        ("qual_min", C.c_int32), ("qual_max", C.c_int32), ("num_read_groups", C.c_uint32),
        ("rg_qual_offset_span", C.c_int32), ("dup_frac", C.c_double), ("unmapped_frac", C.c_double),
        ("num_snps", C.c_uint32), ("num_indel_sites", C.c_uint32), ("alt_frac", C.c_double),
    ]


class SynthReference(C.Structure):
    _fields_ = [
        ("num_contigs", C.c_uint32), ("contig_len", C.POINTER(C.c_uint64)),
        ("contig_words", C.POINTER(C.POINTER(C.c_uint32))), ("num_sites", C.POINTER(C.c_uint32)),
        ("site_start", C.POINTER(C.POINTER(C.c_uint32))), ("site_stop", C.POINTER(C.POINTER(C.c_uint32))),
        ("site_alt", C.POINTER(C.POINTER(C.c_uint8))),
    ]


class SynthBatch(C.Structure):
    _fields_ = [
        ("num_reads", C.c_uint32), ("num_cigar_ops", C.c_uint32), ("num_read_symbols", C.c_uint64),
        ("num_qualities", C.c_uint64), ("chromosome", C.POINTER(C.c_uint16)),
        ("alignment_start", C.POINTER(C.c_uint32)), ("alignment_stop", C.POINTER(C.c_uint32)),
        ("mate_alignment_start", C.POINTER(C.c_uint32)), ("inferred_insert_size", C.POINTER(C.c_int32)),
        ("cigars", C.POINTER(C.c_uint32)), ("cigar_start", C.POINTER(C.c_uint32)),
        ("cigar_len", C.POINTER(C.c_uint32)), ("reads", C.POINTER(C.c_uint32)),
        ("read_start", C.POINTER(C.c_uint32)), ("read_len", C.POINTER(C.c_uint32)),
        ("qualities", C.POINTER(C.c_uint8)), ("qual_start", C.POINTER(C.c_uint32)),
        ("qual_len", C.POINTER(C.c_uint32)), ("flags", C.POINTER(C.c_uint16)), ("mapq", C.POINTER(C.c_uint8)),
        ("read_group", C.POINTER(C.c_uint32)),
    ]


# field name -> (numpy dtype, length attribute)
BATCH_FIELDS = [
    ("chromosome", np.uint16, "num_reads"), ("alignment_start", np.uint32, "num_reads"),
    ("alignment_stop", np.uint32, "num_reads"), ("mate_alignment_start", np.uint32, "num_reads"),
    ("inferred_insert_size", np.int32, "num_reads"), ("cigars", np.uint32, "num_cigar_ops"),
    ("cigar_start", np.uint32, "num_reads"), ("cigar_len", np.uint32, "num_reads"),
    ("reads", np.uint32, "num_read_words"), ("read_start", np.uint32, "num_reads"),
    ("read_len", np.uint32, "num_reads"), ("qualities", np.uint8, "num_qualities"),
    ("qual_start", np.uint32, "num_reads"), ("qual_len", np.uint32, "num_reads"),
    ("flags", np.uint16, "num_reads"), ("mapq", np.uint8, "num_reads"), ("read_group", np.uint32, "num_reads"),
]

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build_synth()))
        _lib.synth_generate_reference.argtypes = [C.POINTER(SynthConfig), C.POINTER(SynthReference)]
        _lib.synth_free_reference.argtypes = [C.POINTER(SynthReference)]
        _lib.synth_generate_batch.argtypes = [C.POINTER(SynthConfig), C.POINTER(SynthReference), C.c_uint64,
                                              C.c_uint32, C.POINTER(SynthBatch)]
        _lib.synth_free_batch.argtypes = [C.POINTER(SynthBatch)]
    return _lib


@dataclass
class Preset:
    name: str
    seed: int = 0
    num_contigs: int = 1
    total_reference_bp: int = 1_000_000
    gc: float = 0.41
    read_lengths: tuple = (101,)
    paired: bool = False
    sub_rate: float = 0.01
    indel_read_frac: float = 0.01
    indel_mode: int = 0
    geometric_p: float = 0.6
    wide_deletion_frac: float = 0.0
    softclip_frac: float = 0.05
    short_fragment_frac: float = 0.02
    qual_mean: float = 32.0
    qual_sd: float = 6.0
    qual_min: int = 2
    qual_max: int = 41
    num_read_groups: int = 1
    rg_qual_offset_span: int = 0
    dup_frac: float = 0.0
    unmapped_frac: float = 0.0
    num_snps: int = 1000
    num_indel_sites: int = 0
    alt_frac: float = 0.3
    num_reads: int = 100_000
    batch_reads: int = 100_000
    extra: dict = field(default_factory=dict)

    def ctype(self) -> SynthConfig:
        c = SynthConfig()
        for f, _ in SynthConfig._fields_:
            if f == "read_lengths":
                arr = (C.c_uint32 * 8)(*list(self.read_lengths)[:8])
                c.read_lengths = arr
            elif f == "num_read_lengths":
                c.num_read_lengths = len(self.read_lengths)
            elif f == "paired":
                c.paired = int(self.paired)
            else:
                setattr(c, f, getattr(self, f))
        return c

    def scaled(self, num_reads: int | None = None, total_reference_bp: int | None = None,
               batch_reads: int | None = None, **kw) -> "Preset":
        d = dict(self.__dict__)
        if num_reads is not None:
            d["num_reads"] = num_reads
        if total_reference_bp is not None:
            ratio = total_reference_bp / self.total_reference_bp
            d["total_reference_bp"] = total_reference_bp
            d["num_snps"] = max(1, int(self.num_snps * ratio))
            d["num_indel_sites"] = int(self.num_indel_sites * ratio)
        if batch_reads is not None:
            d["batch_reads"] = batch_reads
        d.update(kw)
        return Preset(**d)


# The five benchmark configurations (synthetic stand-ins with their shapes and distributions).
PRESETS = {
    "plain_100k_101bp": Preset("plain_100k_101bp", seed=0, num_contigs=1, total_reference_bp=1_000_000,
                               read_lengths=(101,), num_reads=100_000, batch_reads=100_000, num_snps=1000),
    "precision_20M_151bp_pe": Preset("precision_20M_151bp_pe", seed=1, num_contigs=5, total_reference_bp=50_000_000,
                                     read_lengths=(151,), paired=True, indel_read_frac=0.02, num_read_groups=8,
                                     rg_qual_offset_span=3, num_snps=50_000, num_indel_sites=5_000,
                                     num_reads=20_000_000, batch_reads=1_000_000),
    "batched_uneven": Preset("batched_uneven", seed=2, num_contigs=4, total_reference_bp=100_000_000,
                             read_lengths=(36, 76, 101, 151, 250), indel_mode=1, geometric_p=0.6,
                             wide_deletion_frac=0.10, num_read_groups=16, num_snps=100_000, num_indel_sites=10_000,
                             num_reads=4096 * 21_000, batch_reads=21_000),
    "serving_mixed": Preset("serving_mixed", seed=3, num_contigs=3, total_reference_bp=250_000_000,
                            read_lengths=(101, 151), num_read_groups=8, num_snps=450_000, num_indel_sites=50_000,
                            num_reads=1_000_000, batch_reads=1_000_000),
    "large_100M_151bp_pe": Preset("large_100M_151bp_pe", seed=4, num_contigs=3, total_reference_bp=250_000_000,
                                  read_lengths=(151,), paired=True, indel_read_frac=0.02, dup_frac=0.05,
                                  unmapped_frac=0.01, num_read_groups=32, num_snps=3_000_000,
                                  num_indel_sites=300_000, num_reads=100_000_000, batch_reads=2_000_000),
}


class Batch:
    """One alignment batch held in numpy arrays (the engine's input layout)."""

    def __init__(self, arrays: dict, num_reads: int, num_cigar_ops: int, num_read_symbols: int, num_qualities: int):
        self.arrays = arrays
        self.num_reads = num_reads
        self.num_cigar_ops = num_cigar_ops
        self.num_read_symbols = num_read_symbols
        self.num_qualities = num_qualities

    def __getitem__(self, k):
        return self.arrays[k]

    def nbytes(self) -> int:
        return sum(a.nbytes for a in self.arrays.values())

    def view(self, view_cls):
        """Fills an fp_batch_view-compatible ctypes struct with pointers to the arrays."""
        v = view_cls()
        v.num_reads = self.num_reads
        v.num_cigar_ops = self.num_cigar_ops
        v.num_read_symbols = self.num_read_symbols
        v.num_qualities = self.num_qualities
        for name, _, _ in BATCH_FIELDS:
            a = self.arrays[name]
            setattr(v, name, a.ctypes.data_as(C.c_void_p))
        return v

    def range(self, first: int, last: int) -> "Batch":
        """Reads [first, last) as a batch that shares this batch's arrays (no copy of bases, qualities or
        CIGARs): per-read arrays are views and the three start arrays are rebased. Reads of a generated batch
        are stored in order, so their CIGARs, packed bases and qualities are contiguous ranges."""
        a = self.arrays
        if not 0 <= first <= last <= self.num_reads:
            raise ValueError("read range outside the batch")
        n = last - first
        out = {}
        for name in ("chromosome", "alignment_start", "alignment_stop", "mate_alignment_start",
                     "inferred_insert_size", "flags", "mapq", "read_group", "read_len", "qual_len", "cigar_len"):
            out[name] = a[name][first:last]
        if n == 0:
            for name, dt in (("cigars", np.uint32), ("reads", np.uint32), ("qualities", np.uint8)):
                out[name] = np.zeros(0, dt)
            for name in ("cigar_start", "read_start", "qual_start"):
                out[name] = np.zeros(0, np.uint32)
            return Batch(out, 0, 0, 0, 0)
        c0 = int(a["cigar_start"][first])
        c1 = int(a["cigar_start"][last - 1]) + int(a["cigar_len"][last - 1])
        r0 = int(a["read_start"][first])
        r1 = int(a["read_start"][last - 1]) + (int(a["read_len"][last - 1]) + 7) // 8 * 8
        q0 = int(a["qual_start"][first])
        q1 = int(a["qual_start"][last - 1]) + int(a["qual_len"][last - 1])
        if r0 % 8:
            raise ValueError("read start not on a packed-word boundary")
        out["cigars"] = a["cigars"][c0:c1]
        out["reads"] = a["reads"][r0 // 8:(r1 + 7) // 8]
        out["qualities"] = a["qualities"][q0:q1]
        out["cigar_start"] = (a["cigar_start"][first:last] - np.uint32(c0)).astype(np.uint32)
        out["read_start"] = (a["read_start"][first:last] - np.uint32(r0)).astype(np.uint32)
        out["qual_start"] = (a["qual_start"][first:last] - np.uint32(q0)).astype(np.uint32)
        return Batch(out, n, c1 - c0, r1 - r0, q1 - q0)

    def subset(self, read_ids) -> "Batch":
        """A new self-contained batch holding the given reads (in the given order)."""
        read_ids = np.asarray(read_ids, dtype=np.int64)
        a = self.arrays
        out = {}
        for name in ("chromosome", "alignment_start", "alignment_stop", "mate_alignment_start",
                     "inferred_insert_size", "flags", "mapq", "read_group", "read_len", "qual_len", "cigar_len"):
            out[name] = np.ascontiguousarray(a[name][read_ids])
        cig, cs = [], []
        syms, rs = [], []
        quals, qs = [], []
        ncig = nsym = nq = 0
        allsyms = unpack4(a["reads"], self.num_read_symbols)
        for r in read_ids:
            c0, cl = int(a["cigar_start"][r]), int(a["cigar_len"][r])
            cs.append(ncig); cig.append(a["cigars"][c0:c0 + cl]); ncig += cl
            r0, rl = int(a["read_start"][r]), int(a["read_len"][r])
            pad = (rl + 7) // 8 * 8
            s = np.zeros(pad, np.uint8); s[:rl] = allsyms[r0:r0 + rl]
            rs.append(nsym); syms.append(s); nsym += pad
            q0, ql = int(a["qual_start"][r]), int(a["qual_len"][r])
            qs.append(nq); quals.append(a["qualities"][q0:q0 + ql]); nq += ql
        out["cigars"] = np.concatenate(cig).astype(np.uint32) if cig else np.zeros(0, np.uint32)
        out["cigar_start"] = np.array(cs, np.uint32)
        out["reads"] = pack4(np.concatenate(syms) if syms else np.zeros(0, np.uint8))
        out["read_start"] = np.array(rs, np.uint32)
        out["qualities"] = np.concatenate(quals).astype(np.uint8) if quals else np.zeros(0, np.uint8)
        out["qual_start"] = np.array(qs, np.uint32)
        return Batch(out, len(read_ids), ncig, nsym, nq)


def uneven_batch_sizes(num_batches: int, lo: int = 2000, hi: int = 40000, seed: int = 2) -> np.ndarray:
    """Batch sizes drawn uniformly from [lo, hi] (the uneven-batch workload: many input batches of 2k-40k reads)."""
    return np.random.default_rng(seed).integers(lo, hi + 1, size=num_batches)


def unpack4(words: np.ndarray, n: int) -> np.ndarray:
    w = np.asarray(words, dtype=np.uint32)
    sh = (np.arange(8, dtype=np.uint32) * 4)
    s = ((w[:, None] >> sh[None, :]) & 0xF).astype(np.uint8).reshape(-1)
    return s[:n]


def pack4(syms: np.ndarray) -> np.ndarray:
    s = np.asarray(syms, dtype=np.uint32)
    n = (len(s) + 7) // 8 * 8
    if n != len(s):
        s = np.concatenate([s, np.zeros(n - len(s), np.uint32)])
    s = s.reshape(-1, 8)
    sh = (np.arange(8, dtype=np.uint32) * 4)
    return np.bitwise_or.reduce(s << sh[None, :], axis=1).astype(np.uint32)


class Reference:
    """Contigs (4-bit packed) and known sites of one synthetic data set."""

    def __init__(self, preset: Preset):
        self.preset = preset
        self._c = SynthReference()
        self._cfg = preset.ctype()
        lib().synth_generate_reference(C.byref(self._cfg), C.byref(self._c))
        self.contigs = []
        self.sites = []
        for c in range(self._c.num_contigs):
            n = self._c.contig_len[c]
            words = np.ctypeslib.as_array(self._c.contig_words[c], shape=((n + 7) // 8,))
            self.contigs.append((words, n))
            ns = self._c.num_sites[c]
            if ns:
                st = np.ctypeslib.as_array(self._c.site_start[c], shape=(ns,))
                sp = np.ctypeslib.as_array(self._c.site_stop[c], shape=(ns,))
            else:
                st = np.zeros(0, np.uint32)
                sp = np.zeros(0, np.uint32)
            self.sites.append((st, sp))

    def batch(self, batch_index: int, num_reads: int) -> Batch:
        b = SynthBatch()
        lib().synth_generate_batch(C.byref(self._cfg), C.byref(self._c), batch_index, num_reads, C.byref(b))
        lens = {"num_reads": b.num_reads, "num_cigar_ops": b.num_cigar_ops,
                "num_read_words": (b.num_read_symbols + 7) // 8, "num_qualities": b.num_qualities}
        arrays = {}
        for name, dt, ln in BATCH_FIELDS:
            n = lens[ln]
            p = getattr(b, name)
            if n:
                arrays[name] = np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True)
            else:
                arrays[name] = np.zeros(0, dt)
        out = Batch(arrays, b.num_reads, b.num_cigar_ops, b.num_read_symbols, b.num_qualities)
        lib().synth_free_batch(C.byref(b))
        return out

    def batches(self):
        p = self.preset
        done = 0
        i = 0
        while done < p.num_reads:
            n = min(p.batch_reads, p.num_reads - done)
            yield self.batch(i, n)
            done += n
            i += 1

    def __del__(self):
        try:
            lib().synth_free_reference(C.byref(self._c))
        except Exception:
            pass
