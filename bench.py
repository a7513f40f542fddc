#!/usr/bin/env python
"""BQSR throughput benchmark (reads/s) of the GB300 engine on the paired-end precision workload:
20M paired-end 151 bp reads, 8 read groups with quality offsets -3..+3, 5 contigs / 50 Mbp, 50k known SNPs
and 5k known indels, 2% indel reads (seeded synthetic data with those shapes and distributions).

A step is one batch of --batch-reads reads through the whole per-batch hot path (filters, CIGAR expansion,
known sites, BAQ, fractional errors, covariate keys, radix sort and ordered fold into the resident tables);
the job ends with finalize (table compaction, read-group table, empirical qualities). `value` times K steps
+ finalize with the batches already resident in HBM; `e2e` times the same job through the C ABI from pinned
host buffers, host->device copies and the table read-back included.

--impl reference times the reference's CPU path (the oracle port: the reference cannot be built) on all
host cores over bounded samples of the same workload.

Multi-GPU: replicas only (each rank runs its own job on its own GPU; no data exchange).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# dram__bytes_read.sum + dram__bytes_write.sum of one k_baq_seg launch per band-class-0 read, from an ncu capture
# of a 100k-read batch of the workload (78,770 class-0 reads, 921.6 MB; `--batch-reads 100000 ... ncu --set full
# -k regex:k_baq_seg -s 1 -c 1`); the checkpoint scratch traffic is per read, so a launch's traffic scales with
# its reads
TRAFFIC_BYTES_PER_READ = 11700.0
METRIC = "reads/s on 1 GB300, batched vs plain, bit-exact recal table; p50/p99 job latency"
WORKLOAD = ("precision_20M_151bp_pe: paired-end 151 bp reads, 8 read groups (quality offsets -3..+3), "
            "5 contigs / 50 Mbp, 50k known SNPs + 5k known indels, 2% indel reads, 1% substitutions rising to 3'")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch-reads", type=int, default=1_000_000)
    ap.add_argument("--baq", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--cpu-sample-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--replay-rpw", type=int, default=0, help="reads per warp of the FP64 replay kernels (0: default)")
    ap.add_argument("--plain-steps", type=int, default=-1,
                    help="batches through the plain FP64 path, tables compared with the timed run (-1: all, 0: skip)")
    ap.add_argument("--no-precision", action="store_true", help="skip the FP32 vs FP64 per-read precision trace")
    ap.add_argument("--engine-flags", type=int, default=0, help="fp_options.flags (FP_FLAG_*) for the timed engine")
    ap.add_argument("--bam-batches", type=int, default=8, help="workload batches for the BAM input measurement (0: skip)")
    ap.add_argument("--no-config-legs", action="store_true",
                    help="skip the plain 100k-read configuration and the large single run")
    ap.add_argument("--large-reads", type=int, default=100_000_000, help="reads of the large single run")
    ap.add_argument("--large-batch-reads", type=int, default=2_000_000, help="batch size of the large single run")
    ap.add_argument("--large-fp64-batches", type=int, default=3,
                    help="batches of the large run also run through the plain FP64 path (tables compared)")
    ap.add_argument("--batched-batches", type=int, default=4096,
                    help="input batches of the uneven-batch measurement (0: skip)")
    ap.add_argument("--batched-sample", type=int, default=96,
                    help="batches of its per-batch / plain FP64 comparison runs")
    ap.add_argument("--coalesce-reads", type=int, default=1_000_000, help="fp_options.coalesce_reads of the sample's coalesced run")
    ap.add_argument("--no-autotune", action="store_true", help="run the uneven batches with the default shapes")
    ap.add_argument("--serve-jobs", type=int, default=256, help="jobs of the serving measurement (0: skip)")
    ap.add_argument("--no-refstore", action="store_true", help="skip the reference store start-up measurement")
    ap.add_argument("--sort-entries", type=int, default=64_000_000, help="entries of the radix sort measurement (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=20.0, help="job arrivals per second (Poisson)")
    ap.add_argument("--serve-slots", type=int, default=3, help="engines of the job server")
    ap.add_argument("--serve-max-reads", type=int, default=5_000_000, help="largest job (log-uniform from 1000)")
    ap.add_argument("--only", default="", choices=["", "batched", "serving", "configs", "refstore", "sort"],
                    help="run one independent leg alone and print its result (for profiling that leg)")
    ap.add_argument("--serve-hbm-gb", type=float, default=10.0,
                    help="job server admission budget: estimated device memory of the jobs running together "
                         "(0: slots only)")
    return ap.parse_args()


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                f = [x.strip() for x in out.stdout.strip().split(",")]
                if len(f) >= 7:
                    self.samples.append(f)
            except Exception:
                pass
            self._stop.wait(0.2)

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit())
        mx = max((float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].strip() == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def make_workload(num_batches, batch_reads):
    from firepony_gb300 import synth
    p = synth.PRESETS["precision_20M_151bp_pe"].scaled(batch_reads=batch_reads, num_reads=num_batches * batch_reads)
    ref = synth.Reference(p)
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        batches = list(ex.map(lambda i: ref.batch(i, batch_reads), range(num_batches)))
    return p, ref, batches


def tables_identical(a: dict, b: dict) -> bool:
    import numpy as np
    return all(np.array_equal(a[t][k], b[t][k]) for t in a for k in a[t])


def run_plain(args, res):
    """The plain path (every BAQ read in exact FP64, FP_BAQ_FP64) on the same device-resident batches as the
    timed run (all of them by default), CUDA events on the engine's stream; its tables are compared with the
    timed FP32 run's."""
    import torch
    from firepony_gb300.engine import Engine
    n = len(res["dev"]) if args.plain_steps < 0 else min(args.plain_steps, len(res["dev"]))
    p = res["ref"].preset
    eng = Engine(num_read_groups=p.num_read_groups, baq_mode="fp64")
    eng.load_reference(res["ref"])
    stream = torch.cuda.ExternalStream(eng.stream)
    dev = res["dev"][:n]
    eng.submit_device_view(dev[0][1])  # warm-up
    eng.finalize()
    eng.reset()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _, v in dev:
        eng.submit_device_view(v)
    tables = eng.finalize()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    eng.close()
    reads = n * args.batch_reads
    out = {"value": reads / (ms / 1e3), "unit": "reads/s", "baq": "fp64 (every BAQ read exact FP64)",
           "steps": n, "ms_per_step": ms / n}
    if n == len(res["dev"]):
        out["fp32_fp64_tables_identical"] = tables_identical(tables, res["tables"])
        out["compared"] = f"all four tables of the timed FP32 job ({reads} reads) against this FP64 job"
    return out


def run_precision(args, res):
    """FP32 vs FP64 error per read on the timed job's batches: an FP32 engine with the precision trace
    (FP_FLAG_PRECISION_TRACE) also runs every BAQ read through the plain FP64 HMM and compares the pre-floor
    MAP quality t = -4.343 ln(1 - p_max) + 0.499 base by base (bases with FP64 t below 101; above it every
    capped quality is 99). Per read: the largest |t32 - t64| and the widest certified half-interval, as
    percentiles over reads; bound violations count bases whose FP64 t lies outside the FP32 interval."""
    from firepony_gb300.abi import FP_FLAG_PRECISION_TRACE, precision_percentile
    from firepony_gb300.engine import Engine
    p = res["ref"].preset
    eng = Engine(num_read_groups=p.num_read_groups, baq_mode="fp32", flags=FP_FLAG_PRECISION_TRACE)
    eng.load_reference(res["ref"])
    for _, v in res["dev"]:
        eng.submit_device_view(v)
    tables = eng.finalize()
    ps = eng.precision_stats()
    st = eng.stats()
    eng.close()
    qs = (0.5, 0.9, 0.99, 0.999, 1.0)
    return {"reads_compared": ps["reads"], "reads_without_fp32_values": ps["reads_without_fp32"],
            "bases_compared": ps["bases"], "bound_violations": ps["bound_violations"],
            "max_abs_error": ps["max_abs_error"], "max_certified_half_width": ps["max_half_width"],
            "per_read_max_abs_error_upper_edge": {f"p{q * 100:g}": precision_percentile(ps["err_hist"], q) for q in qs},
            "per_read_certified_half_width_upper_edge": {f"p{q * 100:g}": precision_percentile(ps["width_hist"], q)
                                                         for q in qs},
            "err_hist": ps["err_hist"], "width_hist": ps["width_hist"],
            "hist_bins": "bin 0 = exactly 0; bin 1+k = [10^(-10+k/4), 10^(-10+(k+1)/4)); bin 41 = >= 1",
            "baq_reads": st["baq_reads"], "escalated_to_fp64": st["baq_fp64_escalated_reads"],
            "escalated_fraction": st["baq_fp64_escalated_reads"] / max(1, st["baq_reads"]),
            "tables_identical_to_timed_run": tables_identical(tables, res["tables"]),
            "quantity": "t = -4.343 ln(1 - p_max) + 0.499 before flooring (device/baq.cu:673), per base"}


def generate_into(ref, sizes, sink, first_index=0):
    """Generates batch i (i = 0..len(sizes)-1, batch index first_index + i) on host threads and hands each to
    sink(i, batch) in order; generated batches not yet handed over are bounded by the pool's width."""
    from concurrent.futures import ThreadPoolExecutor
    workers = min(16, os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=workers) as ex:
        pending = {}
        nxt = 0
        for i in range(len(sizes)):
            while len(pending) < 2 * workers and nxt < len(sizes):
                pending[nxt] = ex.submit(ref.batch, first_index + nxt, int(sizes[nxt]))
                nxt += 1
            sink(i, pending.pop(i).result())


def run_batched(args):
    """The uneven-batch workload (4 contigs / 100 Mbp, reads of 36-250 bp mixed, 0-8 indels per read, 10% wide
    deletions, 16 read groups) as its 4,096 input batches of 2k-40k reads, from page-locked host buffers
    through the C ABI. The autotuner picks the engine's runtime shapes (FP64 replay layout, device batch size)
    on a separate 16-batch sample; the whole workload then runs with them (wall clock from the first submit to
    the finished tables). On a bounded sample of the same batches: each batch processed alone, the engine
    coalescing them into device batches, and the plain FP64 path on the coalesced batches, which must all give
    identical tables."""
    from firepony_gb300 import synth
    from firepony_gb300.autotune import autotune
    from firepony_gb300.engine import Engine, PinnedPool
    sizes = synth.uneven_batch_sizes(args.batched_batches, 2000, 40000, seed=2)
    p = synth.PRESETS["batched_uneven"].scaled(num_reads=int(sizes.sum()))
    ref = synth.Reference(p)
    out = {}
    best = {"replay_reads_per_warp": 0, "coalesce_reads": args.coalesce_reads}
    if not args.no_autotune:
        tsz = synth.uneven_batch_sizes(16, 2000, 40000, seed=5)
        tune = [ref.batch(1_000_000 + i, int(n)) for i, n in enumerate(tsz)]  # batches not in the workload
        t0 = time.perf_counter()
        tuned = autotune(ref, tune, p.num_read_groups)
        best = tuned["best"]
        out["autotune"] = {"sample_reads": tuned["reads"], "best": best, "seconds": time.perf_counter() - t0,
                           "candidates": len(tuned["results"])}
    pool = PinnedPool()
    pinned = [None] * len(sizes)
    t0 = time.perf_counter()
    generate_into(ref, sizes, lambda i, b: pinned.__setitem__(i, pool.add(b)))
    out["generate_s"] = time.perf_counter() - t0
    reads = int(sizes.sum())
    try:
        # the whole workload with the tuned shapes
        eng = Engine(num_read_groups=p.num_read_groups, coalesce_reads=best["coalesce_reads"],
                     replay_reads_per_warp=best["replay_reads_per_warp"])
        eng.load_reference(ref)
        eng.submit_pipelined(pinned[:64])  # warm-up (device buffers grown), not timed
        eng.finalize()
        eng.reset()
        t0 = time.perf_counter()
        eng.submit_pipelined(pinned)
        eng.finalize()
        dt = time.perf_counter() - t0
        st = eng.stats()
        eng.close()
        out["reads_per_s"] = reads / dt
        out["seconds"] = dt
        out["stage_ms"] = [round(x, 2) for x in st["gpu_ms_per_stage"]]
        out["device_batches"] = st["num_batches"]
        out["baq_reads_by_band"] = st["baq_reads_by_band"]
        out["baq_escalated_by_band"] = st["baq_escalated_by_band"]
        out["baq_fp64_escalated_reads"] = st["baq_fp64_escalated_reads"]
        out["baq_escalated_by_cause"] = st["baq_escalated_by_cause"]
        out["baq_escalated_undecided_rows"] = st["baq_escalated_undecided_rows"]
        # device time from each BAQ stage's start to the end of the class-0 FP32 path, the class-0 replay (which
        # follows the class-2 FP32 kernels on the same stream), the class-1 FP32 path and the class-1 replay,
        # summed over the device batches
        out["baq_path_ms"] = [round(v, 2) for v in st["baq_path_ms"]]
        # bounded sample: per batch / coalesced / plain FP64 coalesced, identical tables
        sample = pinned[:args.batched_sample]
        sreads = int(sum(b.num_reads for b in sample))
        tables = {}
        for name, coalesce, mode in (("per_batch", 0, "fp32"), ("coalesced", args.coalesce_reads, "fp32"),
                                     ("plain_fp64_coalesced", args.coalesce_reads, "fp64")):
            eng = Engine(num_read_groups=p.num_read_groups, coalesce_reads=coalesce, baq_mode=mode)
            eng.load_reference(ref)
            eng.submit_pipelined(sample)  # warm-up pass over the same batches
            eng.finalize()
            eng.reset()
            t0 = time.perf_counter()
            eng.submit_pipelined(sample)
            tables[name] = eng.finalize()
            out["sample_" + name + "_reads_per_s"] = sreads / (time.perf_counter() - t0)
            eng.close()
        out["sample_tables_identical"] = all(tables_identical(tables["per_batch"], tables[o])
                                             for o in ("coalesced", "plain_fp64_coalesced"))
        out["sample"] = f"first {len(sample)} batches, {sreads} reads"
        if not args.no_cpu_baseline:
            out["cpu_oracle"] = cpu_baseline(ref, [pinned[0]], args.cpu_sample_seconds / 3)
    finally:
        del pinned
        pool.close()
    return {"workload": "batched_uneven: 4 contigs / 100 Mbp, reads of 36/76/101/151/250 bp, 0-8 indels per read, "
                        "10% wide deletions, 16 read groups",
            "batches": len(sizes), "reads": reads, "batch_reads": "uniform 2000-40000", "tuned_shapes": best,
            **out,
            "vs_sample_per_batch": out["reads_per_s"] / out["sample_per_batch_reads_per_s"],
            "sample_vs_plain_fp64": out["sample_coalesced_reads_per_s"] / out["sample_plain_fp64_coalesced_reads_per_s"],
            "inputs": "page-locked host buffers through fp_engine_submit_batch (copies in the timed region)"}


def run_config_legs(args):
    """The plain configuration (1 Mbp contig, 100k single-end 101 bp reads, one read group) from page-locked host
    buffers through the C ABI, FP32 and plain FP64; and the large single run (3 contigs / 250 Mbp, 151 bp pairs,
    32 read groups, 5% duplicates and 1% unmapped or MAPQ-0 reads filtered, 3.3M known sites) at its full 100M
    reads: batches generated on host threads and moved to HBM as they come, then one job over all of them
    with the inputs resident (CUDA events on the engine's stream), the full covariate tables resident and
    folded batch by batch. Its first batches also run through the plain FP64 path and an FP32 engine, whose
    tables must be equal. The CPU oracle runs on a bounded sample of each."""
    import torch
    from firepony_gb300 import synth
    from firepony_gb300.engine import Engine, PinnedBatch
    out = {}
    # plain configuration
    p = synth.PRESETS["plain_100k_101bp"]
    ref = synth.Reference(p)
    b0 = ref.batch(0, 100_000)
    pb = PinnedBatch(b0)
    row = {"reads": 100_000}
    tables = {}
    for mode in ("fp32", "fp64"):
        eng = Engine(num_read_groups=p.num_read_groups, baq_mode=mode)
        eng.load_reference(ref)
        eng.submit_pipelined([pb.batch])  # warm-up
        eng.finalize()
        eng.reset()
        t0 = time.perf_counter()
        eng.submit_pipelined([pb.batch])
        tables[mode] = eng.finalize()
        row[mode + "_reads_per_s"] = 100_000 / (time.perf_counter() - t0)
        eng.close()
    pb.close()
    row["fp32_fp64_tables_identical"] = tables_identical(tables["fp32"], tables["fp64"])
    if not args.no_cpu_baseline:
        row["cpu_oracle"] = cpu_baseline(ref, [b0], args.cpu_sample_seconds / 3)
    out["plain_100k_101bp"] = row
    # large single run
    p = synth.PRESETS["large_100M_151bp_pe"]
    ref = synth.Reference(p)
    per = args.large_batch_reads
    nb = (args.large_reads + per - 1) // per
    sizes = [min(per, args.large_reads - i * per) for i in range(nb)]
    dev = [None] * nb
    first = {}

    def sink(i, b):
        dev[i] = to_device(b)
        if i == 0:
            first["batch"] = b
    t0 = time.perf_counter()
    generate_into(ref, sizes, sink)
    row = {"reads": int(sum(sizes)), "batches": nb, "batch_reads": per, "generate_and_upload_s": time.perf_counter() - t0}
    try:
        eng = Engine(num_read_groups=p.num_read_groups)
        eng.load_reference(ref)
        stream = torch.cuda.ExternalStream(eng.stream)
        eng.submit_device_view(dev[0][1])  # warm-up
        eng.finalize()
        eng.reset()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _, v in dev:
            eng.submit_device_view(v)
        eng.finalize()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        st = eng.stats()
        eng.close()
        row["fp32_reads_per_s"] = row["reads"] / (ms / 1e3)
        row["ms_per_batch"] = ms / nb
        row["filtered_reads"] = st["filtered_reads"]
        row["baq_fp64_escalated_reads"] = st["baq_fp64_escalated_reads"]
        k = min(args.large_fp64_batches, nb)
        if k:
            tabs = {}
            for mode in ("fp32", "fp64"):
                eng = Engine(num_read_groups=p.num_read_groups, baq_mode=mode)
                eng.load_reference(ref)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for _, v in dev[:k]:
                    eng.submit_device_view(v)
                tabs[mode] = eng.finalize()
                row[f"first_{k}_batches_{mode}_reads_per_s"] = sum(sizes[:k]) / (time.perf_counter() - t0)
                eng.close()
            row[f"first_{k}_batches_fp32_fp64_tables_identical"] = tables_identical(tabs["fp32"], tabs["fp64"])
        if not args.no_cpu_baseline:
            row["cpu_oracle"] = cpu_baseline(ref, [first["batch"]], args.cpu_sample_seconds / 3)
    finally:
        del dev
        torch.cuda.empty_cache()
    out["large_100M_151bp_pe"] = row
    return out


def run_serving(args):
    """Recalibration jobs arriving as a Poisson process (the serving configuration: 3 contigs / 250 Mbp,
    500k known sites, reads of 101 or 151 bp, 8 read groups) on the job server; each job is the first `size`
    reads of a pinned pool, submitted through the C ABI from host memory. Latency = arrival to finished
    tables."""
    import numpy as np
    from firepony_gb300 import synth
    from firepony_gb300.engine import PinnedBatch
    from firepony_gb300.serve import JobServer, jobs_from_pool, poisson_schedule, run_schedule
    p = synth.PRESETS["serving_mixed"]
    ref = synth.Reference(p)
    per = 1_000_000
    nb = (args.serve_max_reads + per - 1) // per
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        host = list(ex.map(lambda i: ref.batch(i, per), range(nb)))
    pinned = [PinnedBatch(b) for b in host]
    del host
    pool = [pb.batch for pb in pinned]
    arrivals, sizes = poisson_schedule(args.serve_jobs, args.serve_rate, 1000, args.serve_max_reads, seed=3)
    budget = int(args.serve_hbm_gb * 1e9) if args.serve_hbm_gb > 0 else None
    server = JobServer(ref, p.num_read_groups, slots=args.serve_slots, hbm_budget_bytes=budget)
    try:
        run_schedule(server, jobs_from_pool(pool, [20_000] * (2 * args.serve_slots), per), [0.0] * (2 * args.serve_slots))
        server.peak_running = 0
        res = run_schedule(server, jobs_from_pool(pool, sizes, per), arrivals)
        peak = server.peak_running
    finally:
        server.close()
        for pb in pinned:
            pb.close()
    lat = np.array([r.latency for r in res]) * 1e3
    span = max(r.done for r in res) - min(r.arrival for r in res)
    reads = int(sum(r.num_reads for r in res))
    return {"workload": "serving_mixed: 3 contigs / 250 Mbp, 450k SNP + 50k indel sites, 101/151 bp reads, 8 read groups",
            "jobs": len(res), "arrivals": f"Poisson {args.serve_rate:g}/s", "sizes": f"log-uniform 1000-{args.serve_max_reads} reads",
            "slots": args.serve_slots, "hbm_budget_gb": args.serve_hbm_gb or None, "peak_concurrent_jobs": peak,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max()), "reads": reads, "reads_per_s": reads / span,
            "errors": sum(1 for r in res if r.error)}


def _measured_peak_gbs() -> float:
    """The measured HBM copy bandwidth (MEASURED_PEAKS.json), else the fallback 6800 GB/s."""
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs", 6800.0))
    except Exception:
        return 6800.0


def run_sort(args):
    """The radix sort primitive (fp_sort_entries: stable LSD passes of digits of at most 10 bits over packed
    64-bit entries, dense key in the high 32 bits; 29-bit keys take 3 passes) on `--sort-entries` random entries
    with 29-bit keys (the context table's key width), inputs in HBM and larger than L2. Algorithmic bytes follow
    the 8-bit-digit model whatever digit width the kernels use: entries x 8 B x 2 (read + write) x ceil(29 / 8)
    passes, against the measured HBM copy bandwidth. The kernels move entries x 8 B x 3 per pass they run (a
    counting read, then a read and a write). CUDA events on the stream the sort is launched on; the result is
    checked for sortedness and for being a permutation."""
    import numpy as np
    import torch
    from firepony_gb300.engine import sort_entries
    n, key_bits = args.sort_entries, 29
    g = torch.Generator(device="cuda").manual_seed(7)
    keys = torch.randint(0, 1 << key_bits, (n,), device="cuda", dtype=torch.int64, generator=g)
    vals = torch.randint(0, 1 << 31, (n,), device="cuda", dtype=torch.int64, generator=g)
    src = (keys << 32) | vals
    dst = torch.empty_like(src)
    stream = torch.cuda.current_stream()
    for _ in range(3):
        sort_entries(src.data_ptr(), dst.data_ptr(), n, key_bits, stream.cuda_stream)
    reps = 10
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        sort_entries(src.data_ptr(), dst.data_ptr(), n, key_bits, stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    passes = (key_bits + 7) // 8
    kernel_passes = (key_bits + 9) // 10
    algo = n * 8 * 2 * passes
    k = (dst >> 32)
    ok = bool((k[1:] >= k[:-1]).all().item()) and int(dst.sum().item()) == int(src.sum().item())
    peak = _measured_peak_gbs()
    gbs = algo / (ms * 1e-3) / 1e9
    return {"entries": n, "key_bits": key_bits, "passes": passes, "kernel_passes": kernel_passes,
            "kernel_gb": n * 8 * 3 * kernel_passes / 1e9, "ms": ms, "algorithmic_gb": algo / 1e9,
            "achieved_gbs": gbs, "peak_gbs": peak, "frac": gbs / peak if peak else None, "sorted": ok,
            "entries_per_s": n / (ms * 1e-3)}


def run_refstore(args):
    """Start-up of the resident reference (the serving configuration's 3 contigs / 250 Mbp and 500k known
    sites): building the store image, publishing it in POSIX shared memory (the preloader), mapping it in a
    reader, and attaching it to engines (the first attach uploads the image with one copy, later ones share
    it), against an engine uploading the same contigs and sites for itself (fp_engine_set_contig /
    fp_engine_set_known_sites). One 20k-read batch through an attached and a self-loaded engine checks that
    the tables are identical."""
    import numpy as np
    import torch
    from firepony_gb300 import synth
    from firepony_gb300.engine import Engine
    from firepony_gb300.refstore import RefStore
    p = synth.PRESETS["serving_mixed"]
    t0 = time.perf_counter()
    ref = synth.Reference(p)
    gen_s = time.perf_counter() - t0
    name = f"/fpgb_bench_{os.getpid()}"
    out = {"reference": "serving_mixed: 3 contigs / 250 Mbp, 450k SNP + 50k indel sites",
           "generate_ms": gen_s * 1e3}

    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, (time.perf_counter() - t) * 1e3

    engines = []
    store = mapped = None
    try:
        store, out["build_ms"] = timed(lambda: RefStore.build(ref))
        out["image_mb"] = store.info()["image_bytes"] / 1e6
        _, out["publish_ms"] = timed(lambda: store.publish(name))
        mapped, out["open_ms"] = timed(lambda: RefStore.open(name))
        for i in range(3):
            engines.append(Engine(num_read_groups=p.num_read_groups))
        _, out["attach_first_ms"] = timed(lambda: engines[0].attach_refstore(mapped))
        _, out["attach_next_ms"] = timed(lambda: engines[1].attach_refstore(mapped))
        _, out["engine_upload_ms"] = timed(lambda: engines[2].load_reference(ref))
        b = ref.batch(0, 20_000)
        tabs = []
        for e in (engines[0], engines[2]):
            e.submit(b)
            tabs.append(e.finalize())
        out["tables_identical"] = all(np.array_equal(tabs[0][t][k], tabs[1][t][k]) for t in tabs[0] for k in tabs[0][t])
    except Exception as ex:  # e.g. a shared-memory mount too small for the image
        out["error"] = str(ex)
    finally:
        for e in engines:
            e.close()
        for st in (mapped, store):
            if st is not None:
                st.close()
        RefStore.unlink(name)
    return out


def run_bam(args, res):
    """BAM input (libfpbam): the first batches of the workload written as a BGZF-compressed BAM file, then
    (1) decoded alone on all host threads and (2) decoded and recalibrated end to end: BAM file to finished
    tables, the decode of batch n+1 and its copy overlapping the processing of batch n."""
    import tempfile
    import numpy as np
    from firepony_gb300 import bam
    from firepony_gb300.engine import Engine
    try:
        bam.lib()
    except RuntimeError as ex:
        return {"unavailable": str(ex)}
    batches = res["batches"][:args.bam_batches]
    ref = res["ref"]
    p = ref.preset
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "workload.bam")
        targets = [(f"chr{i}", int(n)) for i, (_, n) in enumerate(ref.contigs)]
        bam.write_bam(path, targets, [f"rg{i}" for i in range(p.num_read_groups)], batches, level=1)
        size = os.path.getsize(path)
        reads = sum(b.num_reads for b in batches)
        r = bam.BamReader(path)
        t0 = time.perf_counter()
        n = sum(b.num_reads for b in r.batches(args.batch_reads))
        t_dec = time.perf_counter() - t0
        r.close()
        eng = Engine(num_read_groups=p.num_read_groups)
        eng.load_reference(ref)
        r = bam.BamReader(path)
        eng.submit_threaded(r.batches(args.batch_reads))  # warm-up pass
        eng.finalize()
        eng.reset()
        r.close()
        r = bam.BamReader(path)
        t0 = time.perf_counter()
        eng.submit_threaded(r.batches(args.batch_reads))  # decode on its own thread, overlapping the engine
        tables_host = eng.finalize()
        t_all = time.perf_counter() - t0
        r.close()
        eng.reset()
        # GPU decoding (fpb_next_batch_device): BGZF inflate and record conversion on the device
        gpu = {}
        try:
            r = bam.BamReader(path)
            eng.submit_threaded(r.batches(args.batch_reads, device=True), device=True)  # warm-up pass
            eng.finalize()
            eng.reset()
            r.close()
            r = bam.BamReader(path)
            t0 = time.perf_counter()
            n_dev = sum(b.num_reads for b in r.batches(args.batch_reads, device=True))
            t_dec_dev = time.perf_counter() - t0
            r.close()
            r = bam.BamReader(path)
            t0 = time.perf_counter()
            eng.submit_threaded(r.batches(args.batch_reads, device=True), device=True)
            tables_dev = eng.finalize()
            t_all_dev = time.perf_counter() - t0
            r.close()
            same = all(np.array_equal(tables_host[t][k], tables_dev[t][k]) for t in tables_host for k in tables_host[t])
            gpu = {"gpu_decode_reads_per_s": n_dev / t_dec_dev, "gpu_decode_mb_per_s": size / t_dec_dev / 1e6,
                   "gpu_bam_to_tables_reads_per_s": reads / t_all_dev, "gpu_tables_identical": bool(same)}
        except RuntimeError as ex:
            gpu = {"gpu_decode_unavailable": str(ex)}
        eng.close()
    return {"reads": reads, "bam_bytes": size, "decode_reads_per_s": n / t_dec, "decode_mb_per_s": size / t_dec / 1e6,
            "bam_to_tables_reads_per_s": reads / t_all, "host_threads": os.cpu_count(), **gpu,
            "note": "BGZF level 1 written from the workload batches; decode = inflate + record conversion, on the "
                    "host threads (decode_*, bam_to_tables_*) or on the GPU (gpu_*); the file is read from the page cache"}


def cpu_sub_batches(batch, reads_per_batch=1000):
    """The reference's CPU batch size (1000 reads, firepony.cu:185-190) as zero-copy read ranges of a generated
    batch, built before any timer starts."""
    return [batch.range(i, min(i + reads_per_batch, batch.num_reads))
            for i in range(0, batch.num_reads, reads_per_batch)]


def stage_breakdown(before: dict, after: dict) -> dict:
    """Per-stage CPU thread-seconds between two oracle readings and each stage's share, in the categories the
    reference prints at exit (firepony.cu:195-223)."""
    d = {k: after[k] - before[k] for k in after}
    tot = sum(d.values()) or 1.0
    return {"thread_s": {k: round(v, 4) for k, v in d.items()}, "share": {k: round(v / tot, 4) for k, v in d.items()}}


def cpu_baseline(ref, batches, seconds):
    """The oracle (the reference's CPU path restated) on all host threads, over as many 1000-read batches
    (the reference's CPU batch size) of the same workload as fit in the sample time. The sub-batches are
    zero-copy ranges of a generated batch made before the timer starts, so only the oracle is timed."""
    from oracle.oracle import Oracle
    o = Oracle(ref.preset.num_read_groups)
    o.load_reference(ref)
    subs = cpu_sub_batches(batches[0])
    o.process(subs[-1], threads=0)  # warm-up (thread pool, first-touch of the buffers), not counted
    s0 = o.stage_seconds()
    done = 0
    k = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        o.process(subs[k % len(subs)], threads=0)
        done += subs[k % len(subs)].num_reads
        k += 1
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "reads/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{done} reads of the workload in {k} 1000-read batches ({dt:.1f} s, OpenMP over reads)",
            "stages": stage_breakdown(s0, o.stage_seconds())}


def to_device(batch):
    """Copies a batch's arrays to HBM (torch tensors) and returns (keepalive, device view)."""
    import torch
    from firepony_gb300.abi import FpBatchView
    from firepony_gb300.synth import BATCH_FIELDS
    keep = []
    v = FpBatchView()
    v.num_reads = batch.num_reads
    v.num_cigar_ops = batch.num_cigar_ops
    v.num_read_symbols = batch.num_read_symbols
    v.num_qualities = batch.num_qualities
    for name, _, _ in BATCH_FIELDS:
        a = batch.arrays[name]
        t = torch.from_numpy(a.view("uint8").copy()).to("cuda") if a.nbytes else torch.zeros(8, dtype=torch.uint8,
                                                                                                   device="cuda")
        keep.append(t)
        setattr(v, name, t.data_ptr())
    return keep, v


def run_gb300(args, rank, world):
    import torch
    from firepony_gb300.engine import Engine, PinnedBatch
    torch.cuda.set_device(rank)
    K, W = args.steps, args.warmup
    p, ref, batches = make_workload(K, args.batch_reads)
    eng = Engine(num_read_groups=p.num_read_groups, baq_mode=args.baq, device=rank,
                 replay_reads_per_warp=args.replay_rpw, flags=args.engine_flags)
    eng.load_reference(ref)
    stream = torch.cuda.ExternalStream(eng.stream)

    # ---- value: inputs resident in HBM ----
    dev = [to_device(b) for b in batches]
    torch.cuda.synchronize()
    for i in range(W):
        eng.submit_device_view(dev[i % K][1])
    eng.finalize()
    eng.reset()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(rank)
    clocks.start()
    launches0 = eng.stats()["gpu_kernel_launches"]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(K):
        eng.submit_device_view(dev[i][1])
    tables = eng.finalize()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms_value = e0.elapsed_time(e1)
    st = eng.stats()
    launches = st["gpu_kernel_launches"] - launches0

    # ---- e2e: pinned host buffers through the C ABI ----
    eng.reset()
    pinned = [PinnedBatch(b) for b in batches]
    h2d = sum(pb.batch.nbytes() for pb in pinned) / K
    eng.submit_pipelined([pinned[i % K].batch for i in range(W)])
    eng.finalize()
    eng.reset()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    # the copy of batch i+1 overlaps the processing of batch i (fp_engine_prefetch_batch)
    eng.submit_pipelined([pinned[i].batch for i in range(K)])
    tables_e2e = eng.finalize()
    t_e2e = time.perf_counter() - t0
    rows = sum(len(t["keys"]) for t in tables_e2e.values())
    d2h = (4 * 8 + 16 * 4 + 2 * 4) + rows * (4 + 8 + 4 * 8) / K  # per-batch status words + table read-back
    same = all((tables[t]["keys"] == tables_e2e[t]["keys"]).all() and
               (tables[t]["mismatches"] == tables_e2e[t]["mismatches"]).all() for t in range(4))
    for pb in pinned:
        pb.close()
    stage_ms = st["gpu_ms_per_stage"]
    eng.close()
    return dict(ms_value=ms_value, t_e2e=t_e2e, reads=K * args.batch_reads, h2d=h2d, d2h=d2h, launches=launches,
                clocks=clk, stats=st, stage_ms=stage_ms, same=same, ref=ref, batches=batches, dev=dev, tables=tables)


def fp32_peak():
    """The FP32 SIMT roofline denominator: measured on this GPU (fp_measure_fp32_peak: scalar and packed
    multiply-add chains over one resident grid), beside the nominal SMs x 128 lanes x 2 flops x max clock
    from the device's own SM count."""
    import torch
    from firepony_gb300.engine import measure_fp32_peak
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    out = {"sms": props.multi_processor_count}
    try:
        out["scalar_fma_tflops"] = measure_fp32_peak(torch.cuda.current_device(), packed=False)
        out["packed_fma2_tflops"] = measure_fp32_peak(torch.cuda.current_device(), packed=True)
    except Exception as ex:  # noqa: BLE001 - reported, the nominal figure stays
        out["error"] = str(ex)
    return out


def roofline(res, args, peak32):
    """Roofline of the dominant kernel, the band-class-0 BAQ HMM (k_baq_seg: bandwidth 7, FP32 with certified
    bounds), timed by the engine with CUDA events around each of its launches inside the timed region. Algorithmic bytes per read of that class (L = mean HMM query length): L/2 packed bases + L
    qualities + (L + 6)/2 packed reference window + L BAQ qualities + 4 L MAP states written. Algorithmic
    work: 41 FP32 operations per band cell (forward 19, backward 16, MAP 6), band cells counted exactly per
    read by the engine. The HMM is an FP32 SIMT recurrence, so the compute figure is the binding one; the
    HBM figure is the contract's algorithmic-bytes roofline."""
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    st = res["stats"]
    n = st["baq_main_launches"]
    if not n:
        return None
    ms = st["baq_main_ms"] / n
    reads = st["baq_reads_by_band"][0] / n
    cells = st["baq_band_cells"][0] / n
    L = 151.0
    bytes_ = reads * (L / 2 + L + (L + 6) / 2 + L + 4 * L)
    achieved_gbs = bytes_ / (ms / 1e3) / 1e9
    tops = cells * 41 / (ms / 1e3) / 1e12
    sm_mhz = res["clocks"].get("sm_max_mhz") or peaks.get("sm_max_mhz") or 2070.0
    nominal = peak32["sms"] * 128 * 2 * sm_mhz * 1e6 / 1e12
    measured = max(peak32.get("scalar_fma_tflops", 0.0), peak32.get("packed_fma2_tflops", 0.0))
    f32 = measured if measured > 0 else nominal
    return {"bound": "hbm", "achieved": round(achieved_gbs, 2), "peak": hbm, "unit": "GB/s",
            "frac": round(achieved_gbs / hbm, 5), "traffic": round(TRAFFIC_BYTES_PER_READ * reads),
            "kernel": "k_baq_seg (BAQ HMM, band class 0)",
            "launch_ms": round(ms, 3), "reads_per_launch": int(reads), "band_cells_per_launch": int(cells),
            "peak_source": "measured" if peaks else "fallback",
            "compute": {"unit": "TFLOP/s", "achieved": round(tops, 3), "peak": round(f32, 2),
                        "peak_source": "measured" if measured > 0 else "nominal",
                        "peak_measured": peak32, "peak_nominal": round(nominal, 2),
                        "frac": round(tops / f32, 4),
                        "note": "binding roofline: FP32 SIMT issue"}}


def _leg(fn, *a):
    """An auxiliary measurement: its failure is reported in its own field (traceback on stderr) instead of
    ending the run before the headline line is printed."""
    try:
        return fn(*a)
    except Exception as ex:  # noqa: BLE001 - any failure of a side measurement
        import traceback
        traceback.print_exc()
        return {"error": f"{type(ex).__name__}: {ex}"}


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        from firepony_gb300 import synth
        p = synth.PRESETS["precision_20M_151bp_pe"]
        ref = synth.Reference(p)
        sample = ref.batch(0, 20_000)
        from oracle.oracle import Oracle
        o = Oracle(p.num_read_groups)
        o.load_reference(ref)
        subs = cpu_sub_batches(sample)  # zero-copy 1000-read ranges, made before the timer

        def step():
            for sub in subs:
                o.process(sub, threads=0)
        for _ in range(args.warmup):
            step()
        s0 = o.stage_seconds()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        dt = time.perf_counter() - t0
        stages = stage_breakdown(s0, o.stage_seconds())
        v = args.steps * sample.num_reads / dt
        line = {"metric": METRIC, "value": v, "unit": "reads/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": WORKLOAD, "step": "20000 reads in 1000-read batches",
                           "parallelism": "replicas"},
                "cpu_baseline": {"value": v, "unit": "reads/s", "cores": os.cpu_count(), "kind": "port",
                                 "sample": "20000 reads per step, 1000-read batches, OpenMP over reads",
                                 "stages": stages},
                "e2e": {"value": v, "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    if args.only:
        if rank != 0:
            return 0
        legs = {"batched": run_batched, "serving": run_serving, "configs": run_config_legs, "refstore": run_refstore,
                "sort": run_sort}
        print(json.dumps({"leg": args.only, "result": legs[args.only](args)}))
        return 0
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    res = run_gb300(args, local_rank, world)
    from firepony_gb300.replicas import job_throughput
    value, e2e, ms, t_e2e = job_throughput(res["ms_value"], res["t_e2e"], res["reads"], world, device="cuda")
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline and world == 1:
            cpu = _leg(cpu_baseline, res["ref"], res["batches"], args.cpu_sample_seconds)
        plain = _leg(run_plain, args, res) if args.plain_steps != 0 and world == 1 and args.baq == "fp32" else None
        precision = (_leg(run_precision, args, res) if not args.no_precision and world == 1 and args.baq == "fp32"
                     else None)
        res["dev"] = None  # the device-resident batches of the timed job are not needed past this point
        import torch
        torch.cuda.empty_cache()
        peak32 = _leg(fp32_peak) if world == 1 else {"sms": torch.cuda.get_device_properties(0).multi_processor_count}
        if "sms" not in peak32:
            peak32["sms"] = torch.cuda.get_device_properties(0).multi_processor_count
        serving = _leg(run_serving, args) if args.serve_jobs > 0 and world == 1 else None
        bam_in = _leg(run_bam, args, res) if args.bam_batches > 0 and world == 1 else None
        batched = _leg(run_batched, args) if args.batched_batches > 0 and world == 1 else None
        configs = _leg(run_config_legs, args) if not args.no_config_legs and world == 1 else None
        refstore = _leg(run_refstore, args) if not args.no_refstore and world == 1 else None
        sort = _leg(run_sort, args) if args.sort_entries > 0 and world == 1 else None
        line = {"metric": METRIC, "value": value, "unit": "reads/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "batch_reads": args.batch_reads, "baq": args.baq,
                           "l2": "inputs larger than L2 (about 0.28 GB per 1M-read batch)",
                           "parallelism": "replicas" if world > 1 else "single"},
                "e2e": {"value": e2e, "unit": "reads/s", "h2d_bytes_per_step": int(res["h2d"]),
                        "d2h_bytes_per_step": int(res["d2h"])},
                "gpu_launches": res["launches"],
                "roofline": roofline(res, args, peak32),
                "cpu_baseline": cpu,
                "plain": plain,
                "precision": precision,
                "serving": serving,
                "bam": bam_in,
                "batched": batched,
                "configs": configs,
                "refstore": refstore,
                "sort": sort,
                "clocks": res["clocks"],
                "stage_ms": [round(x, 3) for x in res["stage_ms"]],
                "baq_reads": res["stats"]["baq_reads"],
                "baq_fp64_escalated_reads": res["stats"]["baq_fp64_escalated_reads"],
                "baq_reads_by_band": res["stats"]["baq_reads_by_band"],
                "baq_escalated_by_band": res["stats"]["baq_escalated_by_band"],
                "baq_escalated_by_cause": res["stats"]["baq_escalated_by_cause"],
                "baq_escalated_undecided_rows": res["stats"]["baq_escalated_undecided_rows"],
                "baq_path_ms": [round(v, 3) for v in res["stats"]["baq_path_ms"]],
                "e2e_tables_identical": bool(res["same"])}
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
