"""ctypes wrapper of the BQSR oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use this module, as the checker or as
the timed CPU baseline. The engine never imports it.

Parity status: unpinned against the reference itself (no reference tests, fixtures or runnable build exist);
pinned stage by stage by the hand-derived known-answer tests in tests/test_oracle_kat.py.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from firepony_gb300.abi import FpBatchView, FpTableView, table_to_numpy

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SRC = HERE / "bqsr_oracle.cpp"
LIB = BUILD / "liboracle.so"

_lib = None

# FPO_STAGE_* order (bqsr_oracle.h)
STAGES = ("read_filtering", "cigar_expansion", "bp_filtering", "snp_filtering", "baq_setup", "baq_hmm", "baq_post",
          "fractional_error", "covariates_gather", "covariates_sort_pack", "post_processing")


def build() -> Path:
    """Compiles the oracle (glibc libm, no fast-math, no FMA contraction, OpenMP over reads)."""
    BUILD.mkdir(exist_ok=True)
    deps = [SRC, HERE / "bqsr_oracle.h", HERE.parent / "include" / "firepony_gb300.h"]
    if not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", str(LIB),
               str(SRC)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed\n" + r.stderr)
    return LIB


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        L.fpo_create.restype = C.c_void_p
        L.fpo_create.argtypes = [C.c_uint32]
        L.fpo_destroy.argtypes = [C.c_void_p]
        L.fpo_set_contig.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64]
        L.fpo_set_known_sites.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32]
        L.fpo_process_batch.argtypes = [C.c_void_p, C.POINTER(FpBatchView), C.c_int]
        L.fpo_finalize.argtypes = [C.c_void_p]
        L.fpo_get_table.argtypes = [C.c_void_p, C.c_int32, C.POINTER(FpTableView)]
        L.fpo_get_stats.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
        L.fpo_debug_last_batch.argtypes = [C.c_void_p] + [C.c_void_p] * 6
        L.fpo_kat_hmm.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                  C.c_void_p, C.c_void_p]
        L.fpo_kat_empirical_quality.restype = C.c_double
        L.fpo_kat_empirical_quality.argtypes = [C.c_uint64, C.c_double, C.c_double, C.c_int]
        L.fpo_get_stage_seconds.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.fpo_kat_baq_quality_from_max.restype = C.c_int
        L.fpo_kat_baq_quality_from_max.argtypes = [C.c_double]
        _lib = L
    return _lib


class Oracle:
    def __init__(self, num_read_groups: int = 1):
        self.h = lib().fpo_create(num_read_groups)

    def close(self):
        if self.h:
            lib().fpo_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def load_reference(self, ref) -> None:
        for cid, (words, n) in enumerate(ref.contigs):
            w = np.ascontiguousarray(words, dtype=np.uint32)
            lib().fpo_set_contig(self.h, cid, w.ctypes.data, n)
            st, sp = ref.sites[cid]
            st = np.ascontiguousarray(st, dtype=np.uint32)
            sp = np.ascontiguousarray(sp, dtype=np.uint32)
            lib().fpo_set_known_sites(self.h, cid, st.ctypes.data, sp.ctypes.data, len(st))

    def process(self, batch, threads: int = 0) -> None:
        v = batch.view(FpBatchView)
        rc = lib().fpo_process_batch(self.h, C.byref(v), threads)
        if rc != 0:
            raise ValueError(f"oracle rejected batch (rc={rc})")

    def finalize(self) -> dict:
        lib().fpo_finalize(self.h)
        out = {}
        for t in range(4):
            tv = FpTableView()
            lib().fpo_get_table(self.h, t, C.byref(tv))
            out[t] = table_to_numpy(tv)
        return out

    def stats(self) -> dict:
        a = (C.c_uint64 * 4)()
        lib().fpo_get_stats(self.h, a)
        return {"total_reads": a[0], "filtered_reads": a[1], "baq_reads": a[2], "num_batches": a[3]}

    def stage_seconds(self) -> dict:
        """CPU thread-seconds per stage since creation, in the reference's exit-statistics categories
        (firepony.cu:195-223)."""
        a = (C.c_double * len(STAGES))()
        lib().fpo_get_stage_seconds(self.h, a)
        return {name: a[i] for i, name in enumerate(STAGES)}

    def debug_last_batch(self, batch) -> dict:
        R, Q = batch.num_reads, batch.num_qualities
        d = {"read_status": np.zeros(R, np.uint8), "windows": np.zeros((R, 8), np.uint16),
             "hmm": np.zeros((R, 4), np.int16), "base_flags": np.zeros(Q, np.uint8),
             "baq_tag": np.zeros(Q, np.uint8), "frac_errors": np.zeros((Q, 3), np.float64)}
        lib().fpo_debug_last_batch(self.h, *(d[k].ctypes.data for k in
                                             ("read_status", "windows", "hmm", "base_flags", "baq_tag",
                                              "frac_errors")))
        return d


def hmm(ref, query, qual, band_width, bm_ref_len=None):
    ref = np.ascontiguousarray(ref, np.uint8)
    query = np.ascontiguousarray(query, np.uint8)
    qual = np.ascontiguousarray(qual, np.uint8)
    oq = np.zeros(len(query), np.uint8)
    st = np.zeros(len(query), np.uint32)
    lib().fpo_kat_hmm(ref.ctypes.data, len(ref), bm_ref_len if bm_ref_len is not None else len(ref),
                      query.ctypes.data, qual.ctypes.data, len(query), band_width, oq.ctypes.data, st.ctypes.data)
    return oq, st


def empirical_quality(observations, mismatches, estimated_quality, need_rounding=True):
    return lib().fpo_kat_empirical_quality(observations, mismatches, estimated_quality, int(need_rounding))


def baq_quality_from_max(mx: float) -> int:
    return lib().fpo_kat_baq_quality_from_max(mx)
