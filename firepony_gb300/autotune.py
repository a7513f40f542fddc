"""Autotuner for the engine's runtime shapes on a sample of a workload.

Two shapes of the per-batch path are chosen at run time (fp_options):

* the FP64 replay of reads the FP32 pass cannot certify: `replay_reads_per_warp` = 0 runs the band across a
  group of lanes (k_baq_exact: 8/16/32 lanes x 2-4 slots by band class), 1..32 runs one read per thread with
  that many reads per warp (k_baq_tpr<double>; fewer reads per warp spread a small replay set over more of
  the GPU's FP64 units);
* the device batch: `coalesce_reads` gathers host batches smaller than that many reads into one device batch
  (0: every host batch alone).

`autotune` times every combination on the sample batches (a warm-up pass, then one timed pass from the first
submit to the finished tables) and requires every candidate's tables to equal the first one's: a shape never
changes results, so a difference is an error, not a trade-off. The fastest combination is returned as
Engine keyword arguments. Coalescing targets at or above the sample's read count all gather the whole sample
into one device batch, so the sample cannot tell them apart; when the fastest is one of them, the largest such
target is returned, which on the full workload makes the fewest and largest device batches.

    python -m firepony_gb300.autotune --workload batched_uneven --batches 16 --out tuned.json
    Engine(num_read_groups=16, **json.load(open("tuned.json"))["best"])
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from .engine import Engine

REPLAY_CHOICES = (0, 1, 4, 16, 32)
COALESCE_CHOICES = (0, 250_000, 1_000_000, 4_000_000)


def _tables_equal(a: dict, b: dict) -> bool:
    return all(np.array_equal(a[t][k], b[t][k]) for t in a for k in a[t])


def time_config(reference, batches, num_read_groups: int, replay_reads_per_warp: int, coalesce_reads: int,
                device: int = 0):
    """(seconds of one pass from the first submit to the finished tables, the tables)."""
    e = Engine(num_read_groups=num_read_groups, device=device, replay_reads_per_warp=replay_reads_per_warp,
               coalesce_reads=coalesce_reads)
    try:
        e.load_reference(reference)
        for b in batches[:2]:  # warm-up: buffers grown, kernels loaded
            e.submit(b)
        e.finalize()
        e.reset()
        t0 = time.perf_counter()
        for b in batches:
            e.submit(b)
        tables = e.finalize()
        return time.perf_counter() - t0, tables
    finally:
        e.close()


def autotune(reference, batches, num_read_groups: int, replay_choices=REPLAY_CHOICES,
             coalesce_choices=COALESCE_CHOICES, device: int = 0) -> dict:
    """Times every (replay_reads_per_warp, coalesce_reads) combination on `batches`; returns
    {"best": Engine kwargs, "results": [{config, seconds, reads_per_s}], "reads": n}."""
    reads = int(sum(b.num_reads for b in batches))
    results, ref_tables, best = [], None, None
    for rpw in replay_choices:
        for co in coalesce_choices:
            dt, tables = time_config(reference, batches, num_read_groups, rpw, co, device)
            if ref_tables is None:
                ref_tables = tables
            elif not _tables_equal(tables, ref_tables):
                raise RuntimeError(f"replay_reads_per_warp={rpw}, coalesce_reads={co} changed the tables")
            row = {"replay_reads_per_warp": rpw, "coalesce_reads": co, "seconds": dt, "reads_per_s": reads / dt}
            results.append(row)
            if best is None or dt < best["seconds"]:
                best = row
    co_best = best["coalesce_reads"]
    if co_best >= reads:
        co_best = max(co for co in coalesce_choices if co >= reads)
    return {"best": {"replay_reads_per_warp": best["replay_reads_per_warp"], "coalesce_reads": co_best},
            "results": results, "reads": reads}


def main(argv=None) -> int:
    from . import synth
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--workload", default="batched_uneven", choices=sorted(synth.PRESETS))
    ap.add_argument("--batches", type=int, default=16, help="sample batches (sizes 2k-40k reads)")
    ap.add_argument("--out", default=None, help="write the result as JSON")
    args = ap.parse_args(argv)
    p = synth.PRESETS[args.workload]
    sizes = synth.uneven_batch_sizes(args.batches, 2000, 40000, seed=5)
    p = p.scaled(num_reads=int(sizes.sum()))
    ref = synth.Reference(p)
    batches = [ref.batch(i, int(n)) for i, n in enumerate(sizes)]
    res = autotune(ref, batches, p.num_read_groups)
    res["workload"] = args.workload
    text = json.dumps(res, indent=1)
    if args.out:
        with open(args.out, "w") as f:
            f.write(text)
    print(text)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
