"""Python binding of the C ABI in include/firepony_gb300.h (ctypes over the in-tree libfpengine.so).

The compute path is the CUDA engine only: if the native library cannot be loaded, or no GPU is present, the
calls raise. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .abi import (FP_OK, STATUS_NAMES, FpBatchView, FpOptions, FpPrecisionStats, FpRefstoreInfo, FpStats,
                  FpTableView, FP_BAQ_FP32, FP_BAQ_FP64, table_to_numpy)

_BUILD = Path(__file__).resolve().parent / "_build"
_lib = None

EXPORTED = [
    "fp_engine_create", "fp_engine_destroy", "fp_last_error", "fp_engine_set_contig", "fp_engine_set_known_sites",
    "fp_engine_submit_batch", "fp_engine_finalize", "fp_engine_get_table", "fp_engine_write_report",
    "fp_engine_reset", "fp_engine_get_stats", "fp_engine_debug_last_batch", "fp_report_write", "fp_host_alloc",
    "fp_host_free", "fp_engine_submit_batch_device", "fp_engine_cuda_stream", "fp_sort_entries",
    "fp_sort_entries_static", "fp_engine_prefetch_batch", "fp_engine_get_precision_stats", "fp_measure_fp32_peak",
]


class EngineError(RuntimeError):
    pass


def library_path() -> Path:
    return _BUILD / "libfpengine.so"


def lib():
    """Loads libfpengine.so (building it first if it is missing)."""
    global _lib
    if _lib is None:
        p = library_path()
        if not p.exists():
            from .build import build_engine
            build_engine()
        L = C.CDLL(str(p))
        L.fp_engine_create.argtypes = [C.POINTER(FpOptions), C.POINTER(C.c_void_p)]
        L.fp_engine_destroy.argtypes = [C.c_void_p]
        L.fp_last_error.restype = C.c_char_p
        L.fp_last_error.argtypes = [C.c_void_p]
        L.fp_engine_set_contig.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64]
        L.fp_engine_set_known_sites.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32]
        L.fp_engine_submit_batch.argtypes = [C.c_void_p, C.POINTER(FpBatchView)]
        L.fp_engine_finalize.argtypes = [C.c_void_p]
        L.fp_engine_get_table.argtypes = [C.c_void_p, C.c_int32, C.POINTER(FpTableView)]
        L.fp_engine_write_report.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_char_p), C.c_uint32, C.c_int,
                                             C.c_int, C.c_int, C.c_int]
        L.fp_engine_reset.argtypes = [C.c_void_p]
        L.fp_engine_get_stats.argtypes = [C.c_void_p, C.POINTER(FpStats)]
        L.fp_engine_get_precision_stats.argtypes = [C.c_void_p, C.POINTER(FpPrecisionStats)]
        L.fp_engine_debug_last_batch.argtypes = [C.c_void_p] + [C.c_void_p] * 6
        L.fp_report_write.argtypes = [C.c_char_p, C.POINTER(FpTableView), C.POINTER(C.c_char_p), C.c_uint32, C.c_int,
                                      C.c_int, C.c_int, C.c_int]
        L.fp_engine_submit_batch_device.argtypes = [C.c_void_p, C.POINTER(FpBatchView)]
        L.fp_engine_prefetch_batch.argtypes = [C.c_void_p, C.POINTER(FpBatchView)]
        L.fp_engine_cuda_stream.restype = C.c_void_p
        L.fp_engine_cuda_stream.argtypes = [C.c_void_p]
        L.fp_sort_entries.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_void_p]
        L.fp_sort_entries_static.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_void_p]
        L.fp_host_alloc.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
        L.fp_measure_fp32_peak.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.fp_host_free.argtypes = [C.c_void_p]
        # reference store (include/firepony_gb300_store.h)
        L.fp_refstore_create.argtypes = [C.c_uint32, C.POINTER(C.c_void_p)]
        L.fp_refstore_set_contig.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64]
        L.fp_refstore_set_known_sites.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32]
        L.fp_refstore_shm_name.argtypes = [C.c_char_p, C.c_char_p, C.c_size_t]
        L.fp_refstore_publish.argtypes = [C.c_void_p, C.c_char_p]
        L.fp_refstore_open.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
        L.fp_refstore_unlink.argtypes = [C.c_char_p]
        L.fp_refstore_get_info.argtypes = [C.c_void_p, C.POINTER(FpRefstoreInfo)]
        L.fp_refstore_get_contig.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.POINTER(C.c_uint32)),
                                             C.POINTER(C.c_uint64)]
        L.fp_refstore_get_known_sites.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.POINTER(C.c_uint32)),
                                                  C.POINTER(C.POINTER(C.c_uint32)), C.POINTER(C.c_uint32)]
        L.fp_refstore_upload.argtypes = [C.c_void_p, C.c_int]
        L.fp_engine_attach_refstore.argtypes = [C.c_void_p, C.c_void_p]
        L.fp_refstore_destroy.argtypes = [C.c_void_p]
        L.fp_refstore_last_error.restype = C.c_char_p
        L.fp_refstore_last_error.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _names(rg_names):
    arr = (C.c_char_p * max(1, len(rg_names)))(*[n.encode() for n in rg_names])
    return arr


def write_report(path, tables: dict, rg_names, disable_rounding=False, version=(1, 1, 1)):
    """Writes a GATKReport from numpy tables (the layout returned by Engine.finalize / Oracle.finalize)."""
    keep = []
    views = (FpTableView * 4)()
    for t in range(4):
        d = tables[t]
        arrs = [np.ascontiguousarray(d[k]) for k in ("keys", "observations", "mismatches", "expected_errors",
                                                     "estimated_quality", "empirical_quality")]
        keep.append(arrs)
        v = views[t]
        v.num_rows = len(arrs[0])
        v.keys = arrs[0].ctypes.data_as(C.POINTER(C.c_uint32))
        v.observations = arrs[1].ctypes.data_as(C.POINTER(C.c_uint64))
        v.mismatches = arrs[2].ctypes.data_as(C.POINTER(C.c_double))
        v.expected_errors = arrs[3].ctypes.data_as(C.POINTER(C.c_double))
        v.estimated_quality = arrs[4].ctypes.data_as(C.POINTER(C.c_double))
        v.empirical_quality = arrs[5].ctypes.data_as(C.POINTER(C.c_double))
    rc = lib().fp_report_write(str(path).encode(), views, _names(rg_names), len(rg_names), int(disable_rounding),
                               *version)
    if rc != FP_OK:
        raise EngineError(f"fp_report_write: {STATUS_NAMES.get(rc, rc)}")


def sort_entries(d_in: int, d_out: int, n: int, key_bits: int, stream: int = 0) -> None:
    """fp_sort_entries on device pointers (stable radix sort of packed 64-bit entries by bits 32..)."""
    rc = lib().fp_sort_entries(d_in, d_out, n, key_bits, stream or None)
    if rc != FP_OK:
        raise EngineError(f"fp_sort_entries: {STATUS_NAMES.get(rc, rc)}")



def measure_fp32_peak(device: int = 0, packed: bool = False) -> float:
    """fp_measure_fp32_peak: the device's FP32 multiply-add throughput in TFLOP/s."""
    v = C.c_double()
    rc = lib().fp_measure_fp32_peak(device, int(packed), C.byref(v))
    if rc != FP_OK:
        raise EngineError(f"fp_measure_fp32_peak: {STATUS_NAMES.get(rc, rc)}")
    return v.value


class Engine:
    """One GB300 BQSR engine (fp_engine handle)."""

    def __init__(self, num_read_groups: int = 1, baq_mode: str = "fp32", device: int = 0,
                 replay_reads_per_warp: int = 0, flags: int = 0, coalesce_reads: int = 0):
        o = FpOptions()
        o.device = device
        o.replay_reads_per_warp = replay_reads_per_warp
        o.flags = flags
        o.coalesce_reads = coalesce_reads
        o.baq_mode = FP_BAQ_FP64 if baq_mode == "fp64" else FP_BAQ_FP32
        o.num_read_groups = num_read_groups
        h = C.c_void_p()
        rc = lib().fp_engine_create(C.byref(o), C.byref(h))
        if rc != FP_OK:
            raise EngineError(f"fp_engine_create failed: {STATUS_NAMES.get(rc, rc)}")
        self.h = h
        self.num_read_groups = num_read_groups

    def _check(self, rc, what):
        if rc != FP_OK:
            msg = lib().fp_last_error(self.h)
            raise EngineError(f"{what}: {STATUS_NAMES.get(rc, rc)}: {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "h", None):
            lib().fp_engine_destroy(self.h)
            self.h = None
        self._store = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_contig(self, cid: int, words: np.ndarray, n: int):
        w = np.ascontiguousarray(words, dtype=np.uint32)
        self._check(lib().fp_engine_set_contig(self.h, cid, w.ctypes.data, n), "set_contig")

    def attach_refstore(self, store):
        """Reads contigs and known sites from `store`'s device copy (fp_engine_attach_refstore; uploaded to this
        engine's GPU first if needed). None detaches. The store stays referenced while attached."""
        self._check(lib().fp_engine_attach_refstore(self.h, store.h if store is not None else None),
                    "attach_refstore")
        self._store = store

    def set_known_sites(self, cid: int, start: np.ndarray, stop: np.ndarray):
        st = np.ascontiguousarray(start, dtype=np.uint32)
        sp = np.ascontiguousarray(stop, dtype=np.uint32)
        self._check(lib().fp_engine_set_known_sites(self.h, cid, st.ctypes.data, sp.ctypes.data, len(st)),
                    "set_known_sites")

    def load_reference(self, ref):
        for cid, (words, n) in enumerate(ref.contigs):
            self.set_contig(cid, words, n)
            st, sp = ref.sites[cid]
            self.set_known_sites(cid, st, sp)

    def submit(self, batch):
        v = batch.view(FpBatchView)
        self._check(lib().fp_engine_submit_batch(self.h, C.byref(v)), "submit_batch")

    def submit_view(self, view: FpBatchView):
        self._check(lib().fp_engine_submit_batch(self.h, C.byref(view)), "submit_batch")

    def prefetch_view(self, view: FpBatchView):
        """Queues the batch's host-to-device copy (fp_engine_prefetch_batch); submit the same view next."""
        self._check(lib().fp_engine_prefetch_batch(self.h, C.byref(view)), "prefetch_batch")

    def submit_threaded(self, batches, buffers: int = 3, device: bool = False):
        """submit_pipelined with the batches produced on a separate thread (a decoder): producing batch n+2
        overlaps the processing of batch n (batch n+1's copy is queued meanwhile). At most `buffers` produced
        batches are alive at a time: the producer starts batch n+buffers only after batch n's submit has
        returned, so a decoder that rotates `buffers` buffer sets (the BAM reader) never overwrites a batch
        whose copy or processing is still pending. Needs buffers >= 2; 3 lets decoding overlap the engine.
        device: the batches' arrays are device pointers (the BAM reader's GPU decoding); each is submitted
        with fp_engine_submit_batch_device, with no copy."""
        import queue
        import threading
        if buffers < 2:
            raise ValueError("submit_threaded needs at least two buffers")
        q = queue.Queue()
        tokens = threading.Semaphore(buffers)
        stop = threading.Event()
        done = object()
        err = []

        def produce():
            try:
                it = iter(batches)
                while True:
                    while not tokens.acquire(timeout=0.1):
                        if stop.is_set():
                            return
                    if stop.is_set():
                        return
                    b = next(it, done)
                    if b is done:
                        break
                    q.put(b)
            except Exception as ex:  # re-raised on the submitting thread
                err.append(ex)
            q.put(done)

        t = threading.Thread(target=produce, daemon=True)
        t.start()

        def consume():
            while True:
                b = q.get()
                if b is done:
                    return
                yield b

        try:
            if device:
                for b in consume():
                    self.submit_device_view(b.view(FpBatchView))
                    tokens.release()
            else:
                self.submit_pipelined(consume(), on_submitted=tokens.release)
        finally:
            stop.set()
            t.join()
        if err:
            raise err[0]

    def submit_pipelined(self, batches, on_submitted=None):
        """Submits a sequence of batches (objects with `.view(FpBatchView)`, or views whose arrays the caller
        keeps alive), prefetching each next batch while the current one runs. A batch object is held until
        its submit returns, so the arrays its view points at stay valid while their copy is queued.
        `on_submitted()` is called after each batch's submit has returned (its arrays are no longer read)."""
        def as_pair(x):
            return (x, x.view(FpBatchView)) if hasattr(x, "view") else (x, x)

        def submit(pair):
            self.submit_view(pair[1])
            if on_submitted is not None:
                on_submitted()
        it = iter(batches)
        first = next(it, None)
        if first is None:
            return
        cur = as_pair(first)
        self.prefetch_view(cur[1])
        for x in it:
            nxt = as_pair(x)
            self.prefetch_view(nxt[1])
            submit(cur)
            cur = nxt
        submit(cur)

    def submit_device_view(self, view: FpBatchView):
        """Submits a batch whose arrays are device pointers (already resident in HBM)."""
        self._check(lib().fp_engine_submit_batch_device(self.h, C.byref(view)), "submit_batch_device")

    @property
    def stream(self) -> int:
        return lib().fp_engine_cuda_stream(self.h) or 0

    def finalize(self) -> dict:
        self._check(lib().fp_engine_finalize(self.h), "finalize")
        out = {}
        for t in range(4):
            tv = FpTableView()
            self._check(lib().fp_engine_get_table(self.h, t, C.byref(tv)), "get_table")
            out[t] = table_to_numpy(tv)
        return out

    def write_report(self, path, rg_names, disable_rounding=False, version=(1, 1, 1)):
        self._check(lib().fp_engine_write_report(self.h, str(path).encode(), _names(rg_names), len(rg_names),
                                                 int(disable_rounding), *version), "write_report")

    def reset(self):
        self._check(lib().fp_engine_reset(self.h), "reset")

    def stats(self) -> dict:
        s = FpStats()
        self._check(lib().fp_engine_get_stats(self.h, C.byref(s)), "get_stats")
        d = {}
        for f, _ in FpStats._fields_:
            v = getattr(s, f)
            d[f] = list(v) if hasattr(v, "__len__") else v
        return d

    def precision_stats(self) -> dict:
        """FP32 vs FP64 pre-floor MAP quality per BAQ read (engine created with FP_FLAG_PRECISION_TRACE)."""
        s = FpPrecisionStats()
        self._check(lib().fp_engine_get_precision_stats(self.h, C.byref(s)), "get_precision_stats")
        d = {}
        for f, _ in FpPrecisionStats._fields_:
            v = getattr(s, f)
            d[f] = list(v) if hasattr(v, "__len__") else v
        return d

    def debug_last_batch(self, batch) -> dict:
        R, Q = batch.num_reads, batch.num_qualities
        d = {"read_status": np.zeros(R, np.uint8), "windows": np.zeros((R, 8), np.uint16),
             "hmm": np.zeros((R, 4), np.int16), "base_flags": np.zeros(Q, np.uint8),
             "baq_tag": np.zeros(Q, np.uint8), "frac_errors": np.zeros((Q, 3), np.float64)}
        self._check(lib().fp_engine_debug_last_batch(self.h, *(d[k].ctypes.data for k in (
            "read_status", "windows", "hmm", "base_flags", "baq_tag", "frac_errors"))), "debug_last_batch")
        return d


class PinnedBatch:
    """A batch copied into page-locked host memory (fp_host_alloc) for full-speed H2D copies."""

    def __init__(self, batch):
        from .synth import BATCH_FIELDS, Batch
        self._ptrs = []
        arrays = {}
        for name, dt, _ in BATCH_FIELDS:
            a = batch.arrays[name]
            p = C.c_void_p()
            rc = lib().fp_host_alloc(max(1, a.nbytes), C.byref(p))
            if rc != FP_OK:
                raise EngineError("fp_host_alloc failed")
            self._ptrs.append(p)
            buf = (C.c_uint8 * max(1, a.nbytes)).from_address(p.value)
            dst = np.frombuffer(buf, dtype=dt, count=len(a))
            dst[:] = a
            arrays[name] = dst
        self.batch = Batch(arrays, batch.num_reads, batch.num_cigar_ops, batch.num_read_symbols, batch.num_qualities)
        self.view = self.batch.view(FpBatchView)

    def close(self):
        for p in self._ptrs:
            lib().fp_host_free(p)
        self._ptrs = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedPool:
    """Page-locked host memory for many batches, taken from a few large fp_host_alloc chunks (one allocation
    per batch array would cost thousands of page-locking calls for a workload of thousands of batches)."""

    def __init__(self, chunk_bytes: int = 1 << 30):
        self.chunk_bytes = chunk_bytes
        self._chunks = []  # (pointer, size)
        self._cur = None
        self._off = 0
        self._size = 0

    def _take(self, nbytes: int) -> int:
        nbytes = max(1, nbytes)
        off = (self._off + 255) // 256 * 256
        if self._cur is None or off + nbytes > self._size:
            size = max(self.chunk_bytes, nbytes)
            p = C.c_void_p()
            if lib().fp_host_alloc(size, C.byref(p)) != FP_OK:
                raise EngineError("fp_host_alloc failed")
            self._chunks.append(p)
            self._cur, self._size, off = p.value, size, 0
        self._off = off + nbytes
        return self._cur + off

    def add(self, batch):
        """Copies a batch into the pool; returns a Batch whose arrays are the pinned copies."""
        from .synth import BATCH_FIELDS, Batch
        arrays = {}
        for name, dt, _ in BATCH_FIELDS:
            a = batch.arrays[name]
            addr = self._take(a.nbytes)
            buf = (C.c_uint8 * max(1, a.nbytes)).from_address(addr)
            dst = np.frombuffer(buf, dtype=dt, count=len(a))
            dst[:] = a
            arrays[name] = dst
        return Batch(arrays, batch.num_reads, batch.num_cigar_ops, batch.num_read_symbols, batch.num_qualities)

    def close(self):
        for p in self._chunks:
            lib().fp_host_free(p)
        self._chunks = []
        self._cur = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
