"""GPU parity: the CUDA engine (through the C ABI) against the oracle on the same seeded inputs.

Bar: covariate keys, observation counts, float mismatch sums and empirical qualities bit-exact; expected
errors and estimated qualities within 1e-9 relative (CUDA log10 vs libm on the rounded-prior tables);
per-stage intermediates (read status, windows, HMM window/band width, error and mask bits, BQ tags,
fractional errors) identical for every active read. In FP32 mode without FP_FLAG_EXACT_BAQ_TAGS the engine
certifies of each BQ tag only whether it is NO_BAQ_UNCERTAINTY (64), the one property the tables depend on;
those runs compare that property per base, and the fractional errors it drives, instead of the tag."""
import numpy as np
import pytest

from tests.conftest import make_dataset

pytestmark = pytest.mark.gpu

REL_TOL = 1e-9


def run_engine(ref_or_contigs, batches, n_rg, mode, sites=None, replay_reads_per_warp=0, flags=0):
    """mode: "fp32", "fp64", or "fp32_exact_tags" (FP32 with FP_FLAG_EXACT_BAQ_TAGS)."""
    from firepony_gb300.abi import FP_FLAG_EXACT_BAQ_TAGS
    from firepony_gb300.engine import Engine
    if mode == "fp32_exact_tags":
        mode, flags = "fp32", flags | FP_FLAG_EXACT_BAQ_TAGS
    e = Engine(num_read_groups=n_rg, baq_mode=mode, replay_reads_per_warp=replay_reads_per_warp, flags=flags)
    if sites is None:
        e.load_reference(ref_or_contigs)
    else:
        for cid, (w, n) in enumerate(ref_or_contigs):
            e.set_contig(cid, w, n)
        for cid, (st, sp) in enumerate(sites):
            e.set_known_sites(cid, st, sp)
    dbg = None
    for b in batches:
        e.submit(b)
        dbg = e.debug_last_batch(b)
    dbg["exact_tags"] = mode == "fp64" or bool(flags & FP_FLAG_EXACT_BAQ_TAGS)
    tables = e.finalize()
    stats = e.stats()
    e.close()
    return tables, stats, dbg


def run_oracle(ref_or_contigs, batches, n_rg, sites=None):
    from oracle.oracle import Oracle
    o = Oracle(n_rg)
    if sites is None:
        o.load_reference(ref_or_contigs)
    else:
        from oracle.oracle import lib
        for cid, (w, n) in enumerate(ref_or_contigs):
            w = np.ascontiguousarray(w, np.uint32)
            lib().fpo_set_contig(o.h, cid, w.ctypes.data, n)
        for cid, (st, sp) in enumerate(sites):
            st = np.ascontiguousarray(st, np.uint32)
            sp = np.ascontiguousarray(sp, np.uint32)
            lib().fpo_set_known_sites(o.h, cid, st.ctypes.data, sp.ctypes.data, len(st))
    dbg = None
    for b in batches:
        o.process(b)
        dbg = o.debug_last_batch(b)
    tables = o.finalize()
    return tables, o.stats(), dbg


def assert_tables_equal(a, b):
    for t in range(4):
        ta, tb = a[t], b[t]
        assert len(ta["keys"]) == len(tb["keys"]), f"table {t}: {len(ta['keys'])} vs {len(tb['keys'])} rows"
        np.testing.assert_array_equal(ta["keys"], tb["keys"], err_msg=f"table {t} keys")
        np.testing.assert_array_equal(ta["observations"], tb["observations"], err_msg=f"table {t} observations")
        np.testing.assert_array_equal(ta["mismatches"], tb["mismatches"], err_msg=f"table {t} mismatches")
        np.testing.assert_array_equal(ta["empirical_quality"], tb["empirical_quality"],
                                      err_msg=f"table {t} empirical quality")
        np.testing.assert_allclose(ta["expected_errors"], tb["expected_errors"], rtol=REL_TOL, atol=0)
        np.testing.assert_allclose(ta["estimated_quality"], tb["estimated_quality"], rtol=REL_TOL, atol=0)


def ranges_mask(n, starts, ends):
    """Boolean mask of length n set on the disjoint half-open ranges [starts[i], ends[i])."""
    d = np.zeros(n + 1, np.int64)
    keep = ends > starts
    np.add.at(d, starts[keep], 1)
    np.add.at(d, ends[keep], -1)
    return np.cumsum(d[:n]) > 0


def tag_class(tags):
    """What the tables see of a BQ tag: NO_BAQ_UNCERTAINTY (64), none (0xFF), or another value."""
    return np.where(tags == 64, 1, np.where(tags == 0xFF, 2, 0)).astype(np.uint8)


def assert_stages_equal(batch, ge, go):
    st_e, st_o = ge["read_status"], go["read_status"]
    np.testing.assert_array_equal(st_e, st_o, err_msg="read status")
    act = st_o == 1
    np.testing.assert_array_equal(ge["windows"][act][:, :6], go["windows"][act][:, :6], err_msg="windows")
    np.testing.assert_array_equal(ge["windows"][act][:, 6:], go["windows"][act][:, 6:], err_msg="hq windows")
    np.testing.assert_array_equal(ge["hmm"][act], go["hmm"][act], err_msg="hmm window / band / errors")
    qs, ql = batch["qual_start"].astype(np.int64), batch["qual_len"].astype(np.int64)
    mask = ranges_mask(batch.num_qualities, qs[act], qs[act] + ql[act])
    np.testing.assert_array_equal(ge["base_flags"][mask], go["base_flags"][mask], err_msg="base flags")
    if ge.get("exact_tags", True):
        np.testing.assert_array_equal(ge["baq_tag"][mask], go["baq_tag"][mask], err_msg="BQ tags")
    else:
        np.testing.assert_array_equal(tag_class(ge["baq_tag"][mask]), tag_class(go["baq_tag"][mask]),
                                      err_msg="BQ tags (NO_BAQ_UNCERTAINTY or not)")
    # fractional errors inside the clipped windows (the engine stores them as the table's float values)
    x = go["windows"][act][:, 0].astype(np.int64)
    y = go["windows"][act][:, 1].astype(np.int64)
    win = ranges_mask(batch.num_qualities, qs[act] + x, qs[act] + y + 1)
    fo = go["frac_errors"][win].astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(ge["frac_errors"][win], fo, err_msg="fractional errors")


@pytest.mark.parametrize("mode", ["fp32", "fp32_exact_tags", "fp64"])
@pytest.mark.parametrize("preset,n,batch,refbp", [
    ("plain_100k_101bp", 6000, 2000, 200_000),
    ("precision_20M_151bp_pe", 6000, 3000, 400_000),
    ("batched_uneven", 6000, 1500, 400_000),
])
def test_tables_match_oracle(native, preset, n, batch, refbp, mode):
    p, ref, batches = make_dataset(preset, n, batch, refbp)
    te, se, ge = run_engine(ref, batches, p.num_read_groups, mode)
    to, so, go = run_oracle(ref, batches, p.num_read_groups)
    assert se["total_reads"] == so["total_reads"]
    assert se["filtered_reads"] == so["filtered_reads"]
    assert se["baq_reads"] == so["baq_reads"]
    if preset == "batched_uneven":
        assert se["baq_reads_by_band"][2] > 0  # bands wider than 15 (the exact FP64 kernel across a warp's lanes)
    assert_stages_equal(batches[-1], ge, go)
    assert_tables_equal(te, to)


@pytest.mark.parametrize("mode", ["fp32", "fp32_exact_tags", "fp64"])
def test_edge_cases_match_oracle(native, mode):
    from tests.edge_cases import edge_case_dataset
    contigs, sites, batch, n_rg = edge_case_dataset()
    te, se, ge = run_engine(contigs, [batch], n_rg, mode, sites)
    to, so, go = run_oracle(contigs, [batch], n_rg, sites)
    assert se["filtered_reads"] == so["filtered_reads"]
    assert_stages_equal(batch, ge, go)
    assert_tables_equal(te, to)


@pytest.mark.parametrize("mode", ["fp32", "fp32_exact_tags", "fp64"])
def test_tied_indel_placements_match_oracle(native, mode):
    """One-base indels in homopolymer runs, whose tied base carries quality 2, 3, 4 or 30, in every band
    class: stages and tables equal the oracle's."""
    from tests.edge_cases import tied_indel_dataset
    contigs, sites, batch, n_rg, _ = tied_indel_dataset()
    te, se, ge = run_engine(contigs, [batch], n_rg, mode, sites)
    to, so, go = run_oracle(contigs, [batch], n_rg, sites)
    assert se["baq_reads"] == so["baq_reads"] == batch.num_reads
    assert_stages_equal(batch, ge, go)
    assert_tables_equal(te, to)


def test_tied_states_replay_only_below_min_base_qual(native):
    """A tied deletion placement is a state the FP32 pass cannot order. With the tied base's quality below
    MIN_BASE_QUAL the winner changes the capped quality, so those reads replay in FP64; at quality 30 both
    candidates cap to MIN_BASE_QUAL and the FP32 result stands."""
    from tests.edge_cases import tied_indel_dataset
    contigs, sites, low_batch, n_rg, _ = tied_indel_dataset(tie_quals=(2, 3))
    t_low, s_low, _ = run_engine(contigs, [low_batch], n_rg, "fp32", sites)
    to, _, _ = run_oracle(contigs, [low_batch], n_rg, sites)
    assert_tables_equal(t_low, to)
    # 32 of the 64 reads are deletion placements tied to about 1e-6 or closer
    assert s_low["baq_fp64_escalated_reads"] >= 16, s_low
    contigs, sites, high_batch, n_rg, _ = tied_indel_dataset(tie_quals=(30,))
    t_high, s_high, _ = run_engine(contigs, [high_batch], n_rg, "fp32", sites)
    to, _, _ = run_oracle(contigs, [high_batch], n_rg, sites)
    assert_tables_equal(t_high, to)
    # 16 tied deletion placements; without the tied-state rule every one of them would replay
    assert s_high["baq_fp64_escalated_reads"] < 8, s_high


def test_fp32_and_fp64_paths_agree(native):
    p, ref, batches = make_dataset("precision_20M_151bp_pe", 20000, 10000, 1_000_000)
    t32, s32, _ = run_engine(ref, batches, p.num_read_groups, "fp32")
    t64, s64, _ = run_engine(ref, batches, p.num_read_groups, "fp64")
    assert_tables_equal(t32, t64)
    # escalation is the exception, not the rule
    assert s32["baq_fp64_escalated_reads"] < 0.02 * s32["baq_reads"]


@pytest.mark.parametrize("rpw", [1, 5])
def test_replay_reads_per_warp(native, rpw):
    """The FP64 replay kernels give the same results whatever the number of reads per warp (with exact BQ
    tags, which leave more reads to the replay on this small sample)."""
    p, ref, batches = make_dataset("precision_20M_151bp_pe", 6000, 3000, 400_000)
    te, se, ge = run_engine(ref, batches, p.num_read_groups, "fp32_exact_tags", replay_reads_per_warp=rpw)
    to, so, go = run_oracle(ref, batches, p.num_read_groups)
    assert se["baq_fp64_escalated_reads"] > 0
    assert_stages_equal(batches[-1], ge, go)
    assert_tables_equal(te, to)


def test_batch_size_independent(native):
    """The canonical summation order makes the tables independent of how reads are batched."""
    p, ref, batches = make_dataset("plain_100k_101bp", 8000, 8000, 200_000)
    whole = batches[0]
    parts = [whole.subset(np.arange(i, min(i + 1500, whole.num_reads))) for i in range(0, whole.num_reads, 1500)]
    t1, _, _ = run_engine(ref, [whole], p.num_read_groups, "fp32")
    t2, _, _ = run_engine(ref, parts, p.num_read_groups, "fp32")
    assert_tables_equal(t1, t2)


def test_growing_and_shrinking_batches_with_overlapped_folds(native):
    """Each batch's sort + fold runs on the fold stream while the next batch starts: batches whose entry
    buffers must grow (the previous fold is waited for first), shrink again, and a reset in the middle of a
    stream (the pending fold is joined) give the oracle's tables."""
    from firepony_gb300.engine import Engine
    p, ref, batches = make_dataset("precision_20M_151bp_pe", 24000, 24000, 600_000)
    whole = batches[0]
    cuts = [0, 300, 1300, 9300, 23300, 23800, 24000]  # 300, 1000, 8000, 14000, 500, 200 reads
    parts = [whole.subset(np.arange(a, b)) for a, b in zip(cuts, cuts[1:])]
    e = Engine(num_read_groups=p.num_read_groups)
    try:
        e.load_reference(ref)
        for b in parts[:4]:
            e.submit(b)
        e.reset()  # drops those batches; their folds are joined first
        for b in parts:
            e.submit(b)
        got = e.finalize()
    finally:
        e.close()
    want, _, _ = run_oracle(ref, [whole], p.num_read_groups)
    assert_tables_equal(got, want)


def test_report_identical(native, tmp_path):
    from firepony_gb300.engine import Engine, write_report
    p, ref, batches = make_dataset("precision_20M_151bp_pe", 4000, 2000, 300_000)
    e = Engine(num_read_groups=p.num_read_groups)
    e.load_reference(ref)
    for b in batches:
        e.submit(b)
    e.finalize()
    names = [f"rg{i}" for i in range(p.num_read_groups)]
    e.write_report(tmp_path / "gpu.txt", names)
    e.close()
    to, _, _ = run_oracle(ref, batches, p.num_read_groups)
    write_report(tmp_path / "oracle.txt", to, names)
    assert (tmp_path / "gpu.txt").read_bytes() == (tmp_path / "oracle.txt").read_bytes()


def test_bad_input_rejected_and_engine_usable(native):
    from firepony_gb300.engine import Engine, EngineError
    p, ref, batches = make_dataset("plain_100k_101bp", 500, 500, 100_000)
    e = Engine(num_read_groups=1)
    e.load_reference(ref)
    bad = batches[0].subset(np.arange(500))
    bad.arrays["read_group"][3] = 7  # >= num_read_groups
    with pytest.raises(EngineError, match="BAD_INPUT"):
        e.submit(bad)
    bad2 = batches[0].subset(np.arange(500))
    bad2.arrays["read_start"][5] = 10**9  # outside the batch arrays
    with pytest.raises(EngineError, match="BAD_INPUT"):
        e.submit(bad2)
    e.submit(batches[0])
    t = e.finalize()
    e.close()
    to, _, _ = run_oracle(ref, batches, 1)
    assert_tables_equal(t, to)


def test_large_batch_properties(native):
    """Size-independent properties at a full-size batch (1M reads of 151 bp)."""
    from firepony_gb300.engine import Engine
    p, ref, batches = make_dataset("precision_20M_151bp_pe", 1_000_000, 1_000_000, 50_000_000)
    e = Engine(num_read_groups=p.num_read_groups)
    e.load_reference(ref)
    e.submit(batches[0])
    t = e.finalize()
    s = e.stats()
    e.close()
    q = t[1]
    ev = q["keys"] & 3
    # every gathered base adds one observation to its M, I and D quality keys
    m, i, d = (q["observations"][ev == k].sum() for k in range(3))
    assert m == i == d > 0
    # read-group rows sum the quality rows
    assert t[0]["observations"].sum() == q["observations"].sum()
    # keys ascend
    for k in range(4):
        assert np.all(np.diff(t[k]["keys"].astype(np.int64)) > 0)
    assert s["total_reads"] == 1_000_000


@pytest.mark.parametrize("rpw", [0, 32])
def test_replay_all_reads_exact(native, rpw):
    """Every BAQ read through the exact FP64 replay (warp-cooperative kernel, or thread-per-read with rpw)."""
    from firepony_gb300.abi import FP_FLAG_REPLAY_ALL
    p, ref, batches = make_dataset("precision_20M_151bp_pe", 6000, 3000, 400_000)
    te, se, ge = run_engine(ref, batches, p.num_read_groups, "fp32", replay_reads_per_warp=rpw,
                            flags=FP_FLAG_REPLAY_ALL)
    to, so, go = run_oracle(ref, batches, p.num_read_groups)
    assert_stages_equal(batches[-1], ge, go)
    assert_tables_equal(te, to)


def test_replay_all_wide_bands(native):
    """The uneven-batch workload (bands 16..37) with every BAQ read replayed: the exact FP64 kernels across a
    warp's lanes (16x3, 32x2 and 32x4 lanes x slots) replace the certified FP32 results of every band class."""
    from firepony_gb300.abi import FP_FLAG_REPLAY_ALL
    p, ref, batches = make_dataset("batched_uneven", 6000, 1500, 400_000)
    te, se, ge = run_engine(ref, batches, p.num_read_groups, "fp32", flags=FP_FLAG_REPLAY_ALL)
    to, so, go = run_oracle(ref, batches, p.num_read_groups)
    assert se["baq_reads_by_band"][2] > 0
    assert_stages_equal(batches[-1], ge, go)
    assert_tables_equal(te, to)


@pytest.mark.parametrize("exact_tags", [True, False])
def test_wide_band_fp32_decisions_match_fp64(native, exact_tags):
    """The certified FP32 kernels for bands wider than 15 flush far cells to zero and widen their decision
    margins by the bound on the error that introduces. Over an uneven-batch workload, every BQ tag of the FP32
    path (decided in FP32, or replayed in FP64 where undecided) equals the plain FP64 path's, batch by batch
    (with FP_FLAG_EXACT_BAQ_TAGS; without it, whether each tag is NO_BAQ_UNCERTAINTY), and most wide-band
    reads are decided without a replay."""
    from firepony_gb300.abi import FP_FLAG_EXACT_BAQ_TAGS
    from firepony_gb300.engine import Engine
    p, ref, batches = make_dataset("batched_uneven", 48000, 6000, 800_000)
    e32 = Engine(num_read_groups=p.num_read_groups, baq_mode="fp32",
                 flags=FP_FLAG_EXACT_BAQ_TAGS if exact_tags else 0)
    e64 = Engine(num_read_groups=p.num_read_groups, baq_mode="fp64")
    try:
        for e in (e32, e64):
            e.load_reference(ref)
        for b in batches:
            e32.submit(b)
            d32 = e32.debug_last_batch(b)
            e64.submit(b)
            d64 = e64.debug_last_batch(b)
            np.testing.assert_array_equal(d32["read_status"], d64["read_status"])
            if exact_tags:
                np.testing.assert_array_equal(d32["baq_tag"], d64["baq_tag"], err_msg="BQ tags")
            else:
                np.testing.assert_array_equal(tag_class(d32["baq_tag"]), tag_class(d64["baq_tag"]),
                                              err_msg="BQ tags (NO_BAQ_UNCERTAINTY or not)")
        t32, t64 = e32.finalize(), e64.finalize()
        s32 = e32.stats()
    finally:
        e32.close()
        e64.close()
    assert_tables_equal(t32, t64)
    wide = s32["baq_reads_by_band"][2]
    assert wide > 1000
    # escalations of the wider classes (1 and 2 together) stay well below the wide-band read count
    assert s32["baq_escalated_by_band"][1] < 0.5 * wide, (s32["baq_escalated_by_band"], wide)


def test_replay_all_edge_cases(native):
    from firepony_gb300.abi import FP_FLAG_REPLAY_ALL
    from tests.edge_cases import edge_case_dataset
    contigs, sites, batch, n_rg = edge_case_dataset()
    te, se, ge = run_engine(contigs, [batch], n_rg, "fp32", sites, flags=FP_FLAG_REPLAY_ALL)
    to, so, go = run_oracle(contigs, [batch], n_rg, sites)
    assert_stages_equal(batch, ge, go)
    assert_tables_equal(te, to)


def test_prefetched_submits(native):
    """Batches whose copies were queued ahead (fp_engine_prefetch_batch) give the same tables; a view that was
    not prefetched, a prefetch that is never submitted and a third prefetch ahead are handled."""
    from firepony_gb300.engine import Engine, EngineError, PinnedBatch
    from firepony_gb300.abi import FpBatchView
    p, ref, batches = make_dataset("precision_20M_151bp_pe", 6000, 1500, 400_000)
    pinned = [PinnedBatch(b) for b in batches]
    try:
        e = Engine(num_read_groups=p.num_read_groups)
        e.load_reference(ref)
        e.submit_pipelined([pb.batch for pb in pinned])
        t1 = e.finalize()
        e.reset()
        e.prefetch_view(pinned[3].view)           # submitted last, after other batches
        e.submit_view(pinned[0].view)             # not prefetched: copied into the other buffer
        e.prefetch_view(pinned[1].view)
        with pytest.raises(EngineError):
            e.prefetch_view(pinned[2].view)       # both input buffers hold unsubmitted batches
        e.submit_view(pinned[1].view)
        e.submit_view(pinned[2].view)             # not prefetched
        e.submit_view(pinned[3].view)             # the copy queued first
        t2 = e.finalize()
        e.close()
    finally:
        for pb in pinned:
            pb.close()
    to, _, _ = run_oracle(ref, batches, p.num_read_groups)
    assert_tables_equal(t1, to)
    assert_tables_equal(t2, to)
    assert FpBatchView is not None


def test_reference_n_in_hmm_windows(native):
    """Reads whose HMM reference window holds an N (emission 1 whatever the query base) next to reads without
    one, over runs of N in the reference: the band-class-0 reads with an N go to the general FP32 kernel, the
    others to the class-0 kernel; tables and per-stage intermediates equal the oracle's, in FP32 and FP64."""
    from tests.edge_cases import IUPAC, build_batch, make_reference, read_from_cigar
    from firepony_gb300.synth import pack4
    rng = np.random.default_rng(5)
    ref = list(make_reference(6000, seed=11))
    for a, n in ((1000, 1), (1500, 3), (2000, 12), (3000, 2)):
        ref[a:a + n] = ["N"] * n
    ref = "".join(ref)
    read_src = ref.replace("N", "A")  # the reads carry a base where the reference has N
    recs = []
    for pos in list(range(900, 1100, 9)) + list(range(1400, 1560, 7)) + list(range(1900, 2060, 11)) + \
            list(range(2900, 3050, 13)) + [4000, 4100, 4200]:
        for cigar, subs in (("60M", (10, 40)), ("30M2D30M", (5,)), ("25M1I34M", (50,))):
            seq, q, span = read_from_cigar(read_src, pos, cigar, rng, subs, 30)
            recs.append(dict(pos=pos, cigar=cigar, seq=seq, quals=q, flags=0, mapq=60, rg=0, chrom=0, span=span))
    batch = build_batch(recs)
    syms = np.array([IUPAC[c] for c in ref], np.uint8)
    contigs = [(pack4(syms), len(ref))]
    sites = [(np.zeros(0, np.uint32), np.zeros(0, np.uint32))]
    to, so, go = run_oracle(contigs, [batch], 1, sites)
    for mode in ("fp32", "fp64"):
        te, se, ge = run_engine(contigs, [batch], 1, mode, sites)
        assert se["baq_reads"] == so["baq_reads"] > 100
        if mode == "fp32":
            assert se["baq_reads_by_band"][1] > 0  # the reads with an N in their window
        assert_stages_equal(batch, ge, go)
        assert_tables_equal(te, to)
