"""ctypes mirrors of the C ABI structs in include/firepony_gb300.h and include/firepony_gb300_store.h."""
from __future__ import annotations

import ctypes as C

FP_OK, FP_BAD_INPUT, FP_OOM, FP_DEVICE_ERROR, FP_TIMEOUT, FP_NOT_READY = range(6)
STATUS_NAMES = {0: "FP_OK", 1: "FP_BAD_INPUT", 2: "FP_OOM", 3: "FP_DEVICE_ERROR", 4: "FP_TIMEOUT", 5: "FP_NOT_READY"}

FP_BAQ_FP32, FP_BAQ_FP64 = 0, 1
FP_TABLE_READ_GROUP, FP_TABLE_QUALITY, FP_TABLE_CYCLE, FP_TABLE_CONTEXT = range(4)
TABLE_NAMES = {0: "read_group", 1: "quality", 2: "cycle", 3: "context"}


class FpOptions(C.Structure):
    _fields_ = [("device", C.c_int32), ("baq_mode", C.c_int32), ("num_read_groups", C.c_uint32),
                ("max_batch_reads", C.c_uint32), ("max_batch_bases", C.c_uint64),
                ("max_batch_cigar_ops", C.c_uint64), ("replay_reads_per_warp", C.c_uint32),
                ("flags", C.c_uint32), ("coalesce_reads", C.c_uint32), ("reserved", C.c_uint32)]
FP_FLAG_REPLAY_ALL = 1
FP_FLAG_PRECISION_TRACE = 2
FP_FLAG_EXACT_BAQ_TAGS = 4


class FpBatchView(C.Structure):
    _fields_ = [
        ("num_reads", C.c_uint32), ("num_cigar_ops", C.c_uint32), ("num_read_symbols", C.c_uint64),
        ("num_qualities", C.c_uint64),
        ("chromosome", C.c_void_p), ("alignment_start", C.c_void_p), ("alignment_stop", C.c_void_p),
        ("mate_alignment_start", C.c_void_p), ("inferred_insert_size", C.c_void_p), ("cigars", C.c_void_p),
        ("cigar_start", C.c_void_p), ("cigar_len", C.c_void_p), ("reads", C.c_void_p), ("read_start", C.c_void_p),
        ("read_len", C.c_void_p), ("qualities", C.c_void_p), ("qual_start", C.c_void_p), ("qual_len", C.c_void_p),
        ("flags", C.c_void_p), ("mapq", C.c_void_p), ("read_group", C.c_void_p),
    ]


class FpTableView(C.Structure):
    _fields_ = [("num_rows", C.c_uint32), ("keys", C.POINTER(C.c_uint32)),
                ("observations", C.POINTER(C.c_uint64)), ("mismatches", C.POINTER(C.c_double)),
                ("expected_errors", C.POINTER(C.c_double)), ("estimated_quality", C.POINTER(C.c_double)),
                ("empirical_quality", C.POINTER(C.c_double))]


class FpStats(C.Structure):
    _fields_ = [("total_reads", C.c_uint64), ("filtered_reads", C.c_uint64), ("baq_reads", C.c_uint64),
                ("num_batches", C.c_uint64), ("baq_fp64_escalated_reads", C.c_uint64),
                ("gpu_kernel_launches", C.c_uint64), ("gpu_ms_per_stage", C.c_double * 8),
                ("baq_reads_by_band", C.c_uint64 * 3), ("baq_escalated_by_band", C.c_uint64 * 2),
                ("baq_escalated_by_cause", C.c_uint64 * 2),
                ("baq_band_cells", C.c_uint64 * 3), ("baq_main_launches", C.c_uint64),
                ("baq_main_ms", C.c_double), ("baq_path_ms", C.c_double * 4),
                ("baq_escalated_undecided_rows", C.c_uint64)]


class FpPrecisionStats(C.Structure):
    _fields_ = [("reads", C.c_uint64), ("reads_without_fp32", C.c_uint64), ("bases", C.c_uint64),
                ("bound_violations", C.c_uint64), ("max_abs_error", C.c_double), ("max_half_width", C.c_double),
                ("err_hist", C.c_uint64 * 42), ("width_hist", C.c_uint64 * 42)]


# lower edge of precision-histogram bin i (bin 0 holds exactly 0; bin 1 + k starts at 10^(-10 + k/4))
def precision_bin_lower(i: int) -> float:
    return 0.0 if i == 0 else 10.0 ** (-10.0 + (i - 1) / 4.0)


def precision_percentile(hist, q: float) -> float:
    """Upper edge of the histogram bin that holds the q-quantile (0 < q <= 1) of the per-read values."""
    total = sum(hist)
    if not total:
        return 0.0
    need = q * total
    acc = 0
    for i, c in enumerate(hist):
        acc += c
        if acc >= need:
            return 0.0 if i == 0 else (float("inf") if i == len(hist) - 1 else precision_bin_lower(i + 1))
    return float("inf")


class FpRefstoreInfo(C.Structure):
    _fields_ = [("num_contigs", C.c_uint32), ("attached_engines", C.c_uint32), ("total_bases", C.c_uint64),
                ("total_sites", C.c_uint64), ("image_bytes", C.c_uint64), ("mapped", C.c_int32),
                ("device", C.c_int32)]


def table_to_numpy(tv: FpTableView) -> dict:
    import numpy as np
    n = tv.num_rows
    out = {}
    for name, dt in (("keys", np.uint32), ("observations", np.uint64), ("mismatches", np.float64),
                     ("expected_errors", np.float64), ("estimated_quality", np.float64),
                     ("empirical_quality", np.float64)):
        p = getattr(tv, name)
        out[name] = np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True) if n else np.zeros(0, dt)
    return out
