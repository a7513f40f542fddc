"""BAM input for the engine (libfpbam.so, include/firepony_gb300_bam.h): a reader yielding batches in the
engine's layout and a writer for synthetic BAM files."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .abi import FpBatchView

_lib = None
BUFFER_SETS = 3  # FPB_BUFFER_SETS


class FpbStats(C.Structure):
    """fpb_stats (include/firepony_gb300_bam.h)."""
    _fields_ = [("batches", C.c_uint64), ("records", C.c_uint64), ("compressed_bytes", C.c_uint64),
                ("blocks", C.c_uint64), ("extra_rounds", C.c_uint64), ("serial_walks", C.c_uint64),
                ("seconds_read", C.c_double), ("seconds_decode", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        path = Path(__file__).resolve().parent / "_build" / "libfpbam.so"
        if not path.exists():
            raise RuntimeError(f"{path} missing: build first (python -c 'import __graft_entry__ as g; g.build()'); "
                               "the BAM library needs zlib")
        L = C.CDLL(str(path))
        L.fpb_open.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]
        L.fpb_close.argtypes = [C.c_void_p]
        L.fpb_last_error.restype = C.c_char_p
        L.fpb_last_error.argtypes = [C.c_void_p]
        L.fpb_num_targets.restype = C.c_uint32
        L.fpb_num_targets.argtypes = [C.c_void_p]
        L.fpb_target_name.restype = C.c_char_p
        L.fpb_target_name.argtypes = [C.c_void_p, C.c_uint32]
        L.fpb_target_length.restype = C.c_uint32
        L.fpb_target_length.argtypes = [C.c_void_p, C.c_uint32]
        L.fpb_set_target_map.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
        L.fpb_next_batch.restype = C.c_int64
        L.fpb_next_batch.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(FpBatchView)]
        L.fpb_next_batch_device.restype = C.c_int64
        L.fpb_next_batch_device.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(FpBatchView)]
        L.fpb_num_read_groups.restype = C.c_uint32
        L.fpb_num_read_groups.argtypes = [C.c_void_p]
        L.fpb_read_group_name.restype = C.c_char_p
        L.fpb_read_group_name.argtypes = [C.c_void_p, C.c_uint32]
        L.fpb_get_stats.argtypes = [C.c_void_p, C.POINTER(FpbStats)]
        L.cudaMemcpy.restype = C.c_int  # (from the library's CUDA runtime; device batches are read back with it)
        L.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        L.fpb_write_bam.argtypes = [C.c_char_p, C.c_uint32, C.POINTER(C.c_char_p), C.POINTER(C.c_uint32),
                                    C.c_uint32, C.POINTER(C.c_char_p), C.POINTER(FpBatchView), C.c_uint32,
                                    C.c_int, C.c_int]
        _lib = L
    return _lib


def view_arrays(v: FpBatchView, device: bool = False) -> dict:
    """Copies the arrays of a batch view into numpy arrays (the synth.Batch layout). device: the view holds
    device pointers (fpb_next_batch_device); the arrays are copied with cudaMemcpy."""
    from .synth import BATCH_FIELDS
    lens = {"num_reads": v.num_reads, "num_cigar_ops": v.num_cigar_ops,
            "num_read_words": (v.num_read_symbols + 7) // 8, "num_qualities": v.num_qualities}
    out = {}
    for name, dt, ln in BATCH_FIELDS:
        n = int(lens[ln])
        p = getattr(v, name)
        addr = p if isinstance(p, int) else C.cast(p, C.c_void_p).value
        if n == 0 or not addr:
            out[name] = np.zeros(0, dt)
            continue
        if device:
            a = np.empty(n, dt)
            if lib().cudaMemcpy(C.c_void_p(a.ctypes.data), C.c_void_p(addr), C.c_size_t(a.nbytes), 2) != 0:
                raise RuntimeError(f"copying {name} from the device failed")
            out[name] = a
            continue
        buf = (C.c_uint8 * (n * np.dtype(dt).itemsize)).from_address(addr)
        out[name] = np.frombuffer(buf, dtype=dt, count=n).copy()
    return out


class BamBatch:
    """A decoded batch: its view (reader-owned memory; the reader rotates BUFFER_SETS buffer sets, so the
    batch stays valid until the call that decodes the batch BUFFER_SETS after it). on_device: the view's
    arrays are device pointers (submit with Engine.submit_device_view)."""

    def __init__(self, view: FpBatchView, on_device: bool = False):
        self._view = view
        self.num_reads = view.num_reads
        self.on_device = on_device

    def view(self, view_cls=FpBatchView):
        return self._view

    def to_batch(self):
        from .synth import Batch
        v = self._view
        return Batch(view_arrays(v, self.on_device), v.num_reads, v.num_cigar_ops, v.num_read_symbols,
                     v.num_qualities)


class BamReader:
    def __init__(self, path: str, threads: int = 0):
        h = C.c_void_p()
        if lib().fpb_open(str(path).encode(), threads, C.byref(h)) != 0:
            raise RuntimeError(f"cannot open BAM file {path}")
        self.h = h

    @property
    def targets(self) -> list[tuple[str, int]]:
        n = lib().fpb_num_targets(self.h)
        return [(lib().fpb_target_name(self.h, i).decode(), lib().fpb_target_length(self.h, i)) for i in range(n)]

    def set_target_map(self, contig_of_target):
        a = np.ascontiguousarray(contig_of_target, dtype=np.uint16)
        if lib().fpb_set_target_map(self.h, a.ctypes.data, len(a)) != 0:
            raise RuntimeError("fpb_set_target_map failed")

    def next_batch(self, max_reads: int, device: bool = False) -> BamBatch | None:
        """The next batch of up to max_reads records, None at the end. device: decode on the GPU
        (fpb_next_batch_device; the batch's arrays are device pointers). A reader decodes all its batches one
        way."""
        v = FpBatchView()
        fn = lib().fpb_next_batch_device if device else lib().fpb_next_batch
        n = fn(self.h, max_reads, C.byref(v))
        if n < 0:
            raise RuntimeError("BAM decode failed: " + lib().fpb_last_error(self.h).decode())
        return BamBatch(v, device) if n > 0 else None

    def batches(self, max_reads: int, device: bool = False):
        while True:
            b = self.next_batch(max_reads, device)
            if b is None:
                return
            yield b

    @property
    def stats(self) -> dict:
        st = FpbStats()
        if lib().fpb_get_stats(self.h, C.byref(st)) != 0:
            raise RuntimeError("fpb_get_stats failed")
        return {k: getattr(st, k) for k, _ in FpbStats._fields_}

    @property
    def read_group_names(self) -> list[str]:
        return [lib().fpb_read_group_name(self.h, i).decode() for i in range(lib().fpb_num_read_groups(self.h))]

    def close(self):
        if getattr(self, "h", None):
            lib().fpb_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_bam(path: str, targets, read_group_ids, batches, level: int = 1, threads: int = 0) -> None:
    """targets: [(name, length)]; read_group_ids: names written for read-group indices 0..n-1; batches: objects
    with .view(FpBatchView) (synth.Batch)."""
    names = (C.c_char_p * max(1, len(targets)))(*[t[0].encode() for t in targets])
    lens = (C.c_uint32 * max(1, len(targets)))(*[t[1] for t in targets])
    rgs = (C.c_char_p * max(1, len(read_group_ids)))(*[g.encode() for g in read_group_ids])
    keep = list(batches)
    views = (FpBatchView * max(1, len(keep)))(*[b.view(FpBatchView) for b in keep])
    rc = lib().fpb_write_bam(str(path).encode(), len(targets), names, lens, len(read_group_ids), rgs, views,
                             len(keep), level, threads)
    if rc != 0:
        raise RuntimeError(f"writing {path} failed")
