"""Reference store (include/firepony_gb300_store.h): contigs and known sites as one image, published in POSIX
shared memory by a preloader and attached by engines with one host-to-device copy.

The reference's preloader (firepony-loader.cu:54-93) parses the FASTA and VCF files once and leaves both
databases in shared-memory segments named after the files (mmap.cu:57-89); later runs with `--mmap` read the
segments instead of the files (loader/reference.cu:133-143, loader/variants.cu:48-58). The same flow here:

    store = RefStore.build(reference)                 # contigs + known sites (any object with .contigs/.sites)
    store.publish(RefStore.shm_name("ref.fa"))        # the preloader
    ...
    store = RefStore.open(RefStore.shm_name("ref.fa"))  # a later process: a read-only mapping, no parsing
    engine.attach_refstore(store)                     # one device copy per GPU, shared by engines

A RefStore has `contigs` [(packed words, num_bases)] and `sites` [(start, stop)] like a synthetic Reference, so
it can also be given to Engine.load_reference and to the oracle.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .abi import FP_OK, STATUS_NAMES, FpRefstoreInfo
from .engine import EngineError, lib


class RefStoreError(EngineError):
    pass


class RefStore:
    """One fp_refstore handle."""

    def __init__(self, handle: C.c_void_p):
        self.h = handle

    def _check(self, rc, what):
        if rc != FP_OK:
            msg = lib().fp_refstore_last_error(self.h)
            raise RefStoreError(f"{what}: {STATUS_NAMES.get(rc, rc)}: {msg.decode() if msg else ''}")

    @staticmethod
    def _check_open(rc, what):
        if rc != FP_OK:
            msg = lib().fp_refstore_last_error(None)
            raise RefStoreError(f"{what}: {STATUS_NAMES.get(rc, rc)}: {msg.decode() if msg else ''}")

    # ---- construction ----
    @classmethod
    def create(cls, num_contigs: int) -> "RefStore":
        h = C.c_void_p()
        cls._check_open(lib().fp_refstore_create(num_contigs, C.byref(h)), "fp_refstore_create")
        return cls(h)

    @classmethod
    def build(cls, reference) -> "RefStore":
        """A store holding `reference`'s contigs and known sites."""
        s = cls.create(len(reference.contigs))
        for cid, (words, n) in enumerate(reference.contigs):
            s.set_contig(cid, words, n)
        for cid, (st, sp) in enumerate(reference.sites):
            s.set_known_sites(cid, st, sp)
        return s

    @classmethod
    def open(cls, name: str) -> "RefStore":
        """Maps the published segment `name` read-only."""
        h = C.c_void_p()
        cls._check_open(lib().fp_refstore_open(name.encode(), C.byref(h)), f"fp_refstore_open {name}")
        return cls(h)

    @staticmethod
    def shm_name(path: str) -> str:
        """The segment name of a file, as the reference derives it ("/firepony_" + absolute path, '/' -> '_')."""
        buf = C.create_string_buffer(4096 + 16)
        rc = lib().fp_refstore_shm_name(str(path).encode(), buf, len(buf))
        if rc != FP_OK:
            raise RefStoreError(f"fp_refstore_shm_name {path}: {STATUS_NAMES.get(rc, rc)}")
        return buf.value.decode()

    @staticmethod
    def unlink(name: str) -> bool:
        """Removes the segment name; False when there was none."""
        return lib().fp_refstore_unlink(name.encode()) == FP_OK

    # ---- contents ----
    def set_contig(self, cid: int, words: np.ndarray, n: int):
        w = np.ascontiguousarray(words, dtype=np.uint32)
        self._check(lib().fp_refstore_set_contig(self.h, cid, w.ctypes.data, n), "fp_refstore_set_contig")

    def set_known_sites(self, cid: int, start: np.ndarray, stop: np.ndarray):
        st = np.ascontiguousarray(start, dtype=np.uint32)
        sp = np.ascontiguousarray(stop, dtype=np.uint32)
        self._check(lib().fp_refstore_set_known_sites(self.h, cid, st.ctypes.data, sp.ctypes.data, len(st)),
                    "fp_refstore_set_known_sites")

    def info(self) -> dict:
        i = FpRefstoreInfo()
        self._check(lib().fp_refstore_get_info(self.h, C.byref(i)), "fp_refstore_get_info")
        return {f: getattr(i, f) for f, _ in FpRefstoreInfo._fields_}

    @property
    def num_contigs(self) -> int:
        return self.info()["num_contigs"]

    @property
    def contigs(self) -> list:
        """[(packed words, num_bases)]: views of the store's memory, valid until close()."""
        out = []
        for cid in range(self.num_contigs):
            p = C.POINTER(C.c_uint32)()
            n = C.c_uint64()
            self._check(lib().fp_refstore_get_contig(self.h, cid, C.byref(p), C.byref(n)), "fp_refstore_get_contig")
            words = (n.value + 7) // 8
            out.append((np.ctypeslib.as_array(p, shape=(words,)) if words else np.zeros(0, np.uint32), n.value))
        return out

    @property
    def sites(self) -> list:
        """[(start, stop)] per contig: views of the store's memory, valid until close()."""
        out = []
        for cid in range(self.num_contigs):
            a, b = C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint32)()
            n = C.c_uint32()
            self._check(lib().fp_refstore_get_known_sites(self.h, cid, C.byref(a), C.byref(b), C.byref(n)),
                        "fp_refstore_get_known_sites")
            if n.value:
                out.append((np.ctypeslib.as_array(a, shape=(n.value,)), np.ctypeslib.as_array(b, shape=(n.value,))))
            else:
                out.append((np.zeros(0, np.uint32), np.zeros(0, np.uint32)))
        return out

    # ---- publication and residency ----
    def publish(self, name: str):
        self._check(lib().fp_refstore_publish(self.h, name.encode()), f"fp_refstore_publish {name}")

    def upload(self, device: int = 0):
        self._check(lib().fp_refstore_upload(self.h, device), "fp_refstore_upload")

    def close(self):
        if getattr(self, "h", None):
            self._check(lib().fp_refstore_destroy(self.h), "fp_refstore_destroy")
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
