"""Generates tests/golden/oracle_tables.npz: the oracle's four tables on (a) a small seeded data set shaped
like the paired-end configuration and (b) the hand-built edge-case batch. Regenerate with
``python -m tests.golden.make_golden`` after an intentional oracle change, and review the diff."""
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def compute() -> dict:
    from oracle.oracle import Oracle, lib
    from tests.conftest import make_dataset
    from tests.edge_cases import edge_case_dataset
    out = {}
    p, ref, batches = make_dataset("precision_20M_151bp_pe", 2000, 1000, 200_000)
    o = Oracle(p.num_read_groups)
    o.load_reference(ref)
    for b in batches:
        o.process(b, threads=2)
    for t, tab in o.finalize().items():
        for k, v in tab.items():
            out[f"pe/{t}/{k}"] = v
    contigs, sites, batch, n_rg = edge_case_dataset()
    o = Oracle(n_rg)
    for cid, (w, n) in enumerate(contigs):
        w = np.ascontiguousarray(w, np.uint32)
        lib().fpo_set_contig(o.h, cid, w.ctypes.data, n)
    for cid, (st, sp) in enumerate(sites):
        st = np.ascontiguousarray(st, np.uint32)
        sp = np.ascontiguousarray(sp, np.uint32)
        lib().fpo_set_known_sites(o.h, cid, st.ctypes.data, sp.ctypes.data, len(st))
    o.process(batch, threads=1)
    for t, tab in o.finalize().items():
        for k, v in tab.items():
            out[f"edge/{t}/{k}"] = v
    return out


if __name__ == "__main__":
    np.savez_compressed(HERE / "oracle_tables.npz", **compute())
    print("wrote", HERE / "oracle_tables.npz")
