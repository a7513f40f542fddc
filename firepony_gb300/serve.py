"""Job server over the C ABI: recalibration jobs arriving over time, each turned into its own tables.

The reference runs one job per process (firepony.cu:300-420): it loads the reference and known sites,
streams the job's batches through its pipelines and writes the report. A service answering many jobs
keeps that state resident instead. `JobServer` holds `slots` engines (`fp_engine`) that all read one device
copy of the reference contigs and known sites (a reference store, include/firepony_gb300_store.h: given as
a `RefStore`, e.g. one a preloader published in shared memory, or built from `reference`), and a worker
thread per engine that takes jobs from one
FIFO queue: `fp_engine_reset` (tables to zero, residency kept), the job's batches through
`fp_engine_submit_batch` (host buffers, copies included; each next batch's copy is queued with
`fp_engine_prefetch_batch` while the current one runs), `fp_engine_finalize`. Engines run on their own
CUDA streams, so two jobs share the GPU when more than one is in flight. A job's latency is the time from
its arrival (submission) to its finished tables.

The ctypes calls release the GIL, so worker threads overlap host work (batch packing, result copies) with
the device work of other jobs.

Admission by HBM footprint: with `hbm_budget_bytes` set, a job starts (in arrival order) only when a slot is
free and the estimated device memory of the running jobs plus its own fits the budget; a job larger than
the whole budget runs alone. A job's estimate is `Job.footprint` when given, else `estimate_job_bytes` of its
largest batch.
"""
from __future__ import annotations

import threading
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Callable, Iterable

import numpy as np

from .engine import Engine
from .refstore import RefStore


def estimate_job_bytes(max_batch_reads: int, mean_read_len: float = 151.0) -> int:
    """Device memory a job's batches take in an engine beyond its resident reference, tables and fixed BAQ
    scratch: the input arrays, expanded CIGAR events, per-read and per-base work arrays and covariate
    entries of its largest batch (about 4.5 GB per 1M reads of 151 bp)."""
    return int(max_batch_reads * (600 + 26 * mean_read_len))


@dataclass
class Job:
    """One recalibration job: its batches (host `synth.Batch`-like objects with `.view()`), produced lazily
    by `batches()` so that packing happens on the worker thread, as an io thread would do it. `footprint`:
    its estimated device memory in bytes (0: estimated from num_reads and max_batch_reads)."""
    job_id: int
    num_reads: int
    batches: Callable[[], Iterable]
    arrival: float = 0.0
    footprint: int = 0
    max_batch_reads: int = 1_000_000

    def device_bytes(self) -> int:
        return self.footprint or estimate_job_bytes(min(self.num_reads, self.max_batch_reads))


@dataclass
class JobResult:
    job_id: int
    num_reads: int
    arrival: float
    start: float
    done: float
    tables: dict | None = None
    error: str | None = None

    @property
    def latency(self) -> float:
        return self.done - self.arrival


@dataclass
class _Pending:
    job: Job
    event: threading.Event = field(default_factory=threading.Event)
    result: JobResult | None = None


class JobServer:
    def __init__(self, reference, num_read_groups: int, slots: int = 2, baq_mode: str = "fp32", device: int = 0,
                 keep_tables: bool = False, hbm_budget_bytes: int | None = None, engine_factory=None,
                 share_reference: bool = True):
        """reference: a RefStore (attached by every engine), or contigs/sites (a synth.Reference) from which
        the server builds one store (share_reference) or which every engine uploads for itself."""
        self.keep_tables = keep_tables
        self.hbm_budget = hbm_budget_bytes
        self.engines = []
        self._own_store = None
        store = reference if isinstance(reference, RefStore) else None
        if store is None and share_reference and engine_factory is None:
            store = self._own_store = RefStore.build(reference)
        for _ in range(slots):
            if engine_factory is not None:
                e = engine_factory()
            else:
                e = Engine(num_read_groups=num_read_groups, baq_mode=baq_mode, device=device)
                if store is not None:
                    e.attach_refstore(store)
                else:
                    e.load_reference(reference)
            self.engines.append(e)
        self.store = store
        self._cv = threading.Condition()
        self._queue: deque = deque()
        self._closing = False
        self.in_use = 0           # estimated device bytes of the running jobs
        self.peak_in_use = 0
        self.running = 0
        self.peak_running = 0
        self._threads = [threading.Thread(target=self._worker, args=(e,), daemon=True) for e in self.engines]
        for t in self._threads:
            t.start()

    def submit(self, job: Job) -> _Pending:
        job.arrival = time.perf_counter()
        p = _Pending(job)
        with self._cv:
            self._queue.append(p)
            self._cv.notify_all()
        return p

    def _admissible(self, p: _Pending) -> bool:
        if self.hbm_budget is None or self.running == 0:
            return True
        return self.in_use + p.job.device_bytes() <= self.hbm_budget

    def _next(self):
        """The first queued job once it fits (arrival order: a later job never passes it), or None to stop."""
        with self._cv:
            while True:
                if self._closing and not self._queue:
                    return None
                if self._queue and self._admissible(self._queue[0]):
                    p = self._queue.popleft()
                    self.in_use += p.job.device_bytes()
                    self.running += 1
                    self.peak_in_use = max(self.peak_in_use, self.in_use)
                    self.peak_running = max(self.peak_running, self.running)
                    self._cv.notify_all()
                    return p
                self._cv.wait()

    def _release(self, p: _Pending):
        with self._cv:
            self.in_use -= p.job.device_bytes()
            self.running -= 1
            self._cv.notify_all()

    def _worker(self, eng: Engine):
        while True:
            p = self._next()
            if p is None:
                return
            job = p.job
            start = time.perf_counter()
            try:
                eng.reset()
                # each next batch's copy is queued while the current one runs
                eng.submit_pipelined(job.batches())
                tables = eng.finalize()
                p.result = JobResult(job.job_id, job.num_reads, job.arrival, start, time.perf_counter(),
                                     tables if self.keep_tables else None)
            except Exception as ex:  # the job fails, the server keeps running
                p.result = JobResult(job.job_id, job.num_reads, job.arrival, start, time.perf_counter(),
                                     error=str(ex))
            self._release(p)
            p.event.set()

    def close(self):
        with self._cv:
            self._closing = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()
        for e in self.engines:
            e.close()
        self.engines = []
        if self._own_store is not None:
            self._own_store.close()
            self._own_store = None


def poisson_schedule(num_jobs: int, rate_per_s: float, min_reads: int, max_reads: int, seed: int):
    """Arrival offsets (s) of a Poisson process and log-uniform job sizes (reads), seeded."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, size=num_jobs)
    arrivals = np.cumsum(gaps) - gaps[0]
    sizes = np.exp(rng.uniform(np.log(min_reads), np.log(max_reads), size=num_jobs)).astype(np.int64)
    return arrivals, sizes


def jobs_from_pool(pool: list, sizes, batch_reads: int) -> list[Job]:
    """Jobs made of the first `size` reads of a pool of batches (read ranges of the pool's batches, at most
    `batch_reads` reads per submitted batch)."""
    cap = sum(b.num_reads for b in pool)
    jobs = []
    for j, size in enumerate(sizes):
        size = int(min(size, cap))

        def make(size=size):
            left = size
            for b in pool:
                first = 0
                while left > 0 and first < b.num_reads:
                    n = min(left, batch_reads, b.num_reads - first)
                    yield b.range(first, first + n)
                    first += n
                    left -= n
                if left <= 0:
                    return

        jobs.append(Job(j, size, make, max_batch_reads=batch_reads))
    return jobs


def run_schedule(server: JobServer, jobs: list[Job], arrivals) -> list[JobResult]:
    """Submits each job at its arrival offset (real time) and waits for all results."""
    t0 = time.perf_counter()
    pending = []
    for job, at in zip(jobs, arrivals):
        delay = t0 + float(at) - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        pending.append(server.submit(job))
    out = []
    for p in pending:
        p.event.wait()
        out.append(p.result)
    return out
