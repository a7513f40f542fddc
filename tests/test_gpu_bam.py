"""BAM file -> decoder -> engine: the tables equal the oracle's on the decoded batches."""
import numpy as np
import pytest

from tests.test_gpu_parity import assert_tables_equal, run_oracle

pytestmark = pytest.mark.gpu


def test_bam_to_tables(native, tmp_path):
    from firepony_gb300 import bam, synth
    from firepony_gb300.engine import Engine
    try:
        bam.lib()
    except RuntimeError as ex:
        pytest.skip(str(ex))
    p = synth.PRESETS["precision_20M_151bp_pe"].scaled(num_reads=6000, total_reference_bp=400_000, batch_reads=3000)
    ref = synth.Reference(p)
    batches = list(ref.batches())
    path = tmp_path / "in.bam"
    targets = [(f"chr{i}", int(n)) for i, (_, n) in enumerate(ref.contigs)]
    bam.write_bam(str(path), targets, [f"rg{i}" for i in range(p.num_read_groups)], batches)
    reader = bam.BamReader(str(path))
    e = Engine(num_read_groups=p.num_read_groups)
    e.load_reference(ref)
    decoded = []
    # decoded on a producer thread like a loader: batch n+1 is decoded and its copy queued while batch n runs
    def gen():
        for b in reader.batches(2000):
            decoded.append(b.to_batch())
            yield b
    e.submit_threaded(gen())
    tables = e.finalize()
    e.close()
    reader.close()
    assert sum(b.num_reads for b in decoded) == 6000
    to, _, _ = run_oracle(ref, decoded, p.num_read_groups)
    assert_tables_equal(tables, to)
    assert np.all(np.concatenate([b["read_group"] for b in decoded]) < p.num_read_groups)


BATCH_KEYS = ("chromosome", "alignment_start", "alignment_stop", "mate_alignment_start", "inferred_insert_size",
              "cigars", "cigar_start", "cigar_len", "reads", "read_start", "read_len", "qualities", "qual_start",
              "qual_len", "flags", "mapq", "read_group")


@pytest.fixture(scope="module")
def bam_files(native, tmp_path_factory):
    """A synthetic BAM file per compression level (0: stored blocks) with records crossing block boundaries."""
    from firepony_gb300 import bam, synth
    try:
        bam.lib()
    except RuntimeError as ex:
        pytest.skip(str(ex))
    p = synth.PRESETS["batched_uneven"].scaled(num_reads=9000, total_reference_bp=400_000, batch_reads=3000)
    ref = synth.Reference(p)
    batches = list(ref.batches())
    d = tmp_path_factory.mktemp("bamgpu")
    targets = [(f"chr{i}", int(n)) for i, (_, n) in enumerate(ref.contigs)]
    rg_ids = [f"rg{i}" for i in range(p.num_read_groups)]
    files = {}
    for level in (0, 1, 6):
        path = d / f"l{level}.bam"
        bam.write_bam(str(path), targets, rg_ids, batches, level=level, threads=4)
        files[level] = path
    return p, ref, batches, files


def _decode_all(path, max_reads, device):
    from firepony_gb300 import bam
    r = bam.BamReader(str(path), threads=4)
    got = [b.to_batch() for b in r.batches(max_reads, device=device)]
    names = r.read_group_names
    st = r.stats
    r.close()
    assert st["records"] == sum(b.num_reads for b in got) and st["batches"] == len(got)
    if device:
        # the GPU inflated the blocks after the header, and every batch's record starts were found in parallel
        # (the one-thread walk is only the fallback for a candidate chain that does not verify)
        assert st["blocks"] > 0 and st["serial_walks"] == 0, st
    return got, names


@pytest.mark.parametrize("level,max_reads", [(1, 100000), (1, 1000), (1, 777), (0, 2048), (6, 1500)])
def test_device_decode_equals_host(bam_files, level, max_reads):
    """fpb_next_batch_device gives the host decoder's batches array for array (same batch boundaries,
    read-group ids in order of first occurrence, padded base words)."""
    p, ref, batches, files = bam_files
    host, hn = _decode_all(files[level], max_reads, False)
    dev, dn = _decode_all(files[level], max_reads, True)
    assert [b.num_reads for b in dev] == [b.num_reads for b in host]
    assert sum(b.num_reads for b in dev) == 9000
    assert dn == hn
    for bh, bd in zip(host, dev):
        assert (bd.num_cigar_ops, bd.num_read_symbols, bd.num_qualities) == \
               (bh.num_cigar_ops, bh.num_read_symbols, bh.num_qualities)
        for k in BATCH_KEYS:
            np.testing.assert_array_equal(bd[k], bh[k], err_msg=k)


def test_device_decode_tiny_batches(bam_files):
    """Batches of a few records: every batch carries most of the inflated stream into the next one."""
    p, ref, batches, files = bam_files
    from firepony_gb300 import bam
    r = bam.BamReader(str(files[1]), threads=2)
    got = []
    for _ in range(40):
        b = r.next_batch(7, device=True)
        got.append(b.to_batch())
    r.close()
    whole = {k: np.concatenate([b[k] for b in batches]) for k in ("alignment_start", "flags", "qual_len")}
    for k in whole:
        np.testing.assert_array_equal(np.concatenate([b[k] for b in got]), whole[k][:280], err_msg=k)


def test_bam_to_tables_device_decode(native, tmp_path):
    """BAM file -> GPU decoding -> engine (device batches, decoded on a producer thread): the tables equal the
    oracle's on the decoded batches."""
    from firepony_gb300 import bam, synth
    from firepony_gb300.engine import Engine
    p = synth.PRESETS["precision_20M_151bp_pe"].scaled(num_reads=6000, total_reference_bp=400_000, batch_reads=3000)
    ref = synth.Reference(p)
    path = tmp_path / "in.bam"
    targets = [(f"chr{i}", int(n)) for i, (_, n) in enumerate(ref.contigs)]
    bam.write_bam(str(path), targets, [f"rg{i}" for i in range(p.num_read_groups)], list(ref.batches()))
    reader = bam.BamReader(str(path))
    e = Engine(num_read_groups=p.num_read_groups)
    e.load_reference(ref)
    decoded = []

    def gen():
        for b in reader.batches(2000, device=True):
            decoded.append(b.to_batch())
            yield b
    e.submit_threaded(gen(), device=True)
    tables = e.finalize()
    e.close()
    reader.close()
    assert sum(b.num_reads for b in decoded) == 6000
    to, _, _ = run_oracle(ref, decoded, p.num_read_groups)
    assert_tables_equal(tables, to)


def _blocks(data: bytes):
    """(offset, size) of each BGZF block."""
    out, o = [], 0
    while o + 18 <= len(data):
        bsize = int.from_bytes(data[o + 16:o + 18], "little") + 1
        out.append((o, bsize))
        o += bsize
    return out


@pytest.mark.parametrize("where", ["crc", "deflate", "isize_small"])
def test_device_decode_corrupt_block(bam_files, tmp_path, where):
    """A damaged BGZF block in the middle of the file ends GPU decoding with an error, not with wrong batches."""
    p, ref, batches, files = bam_files
    from firepony_gb300 import bam
    data = bytearray(files[1].read_bytes())
    blks = _blocks(bytes(data))
    o, n = blks[len(blks) // 2]
    if where == "crc":
        data[o + n - 8] ^= 0x5A
    elif where == "deflate":
        data[o + 18 + (n - 26) // 2] ^= 0x10
    else:
        data[o + n - 4:o + n] = (int.from_bytes(data[o + n - 4:o + n], "little") - 100).to_bytes(4, "little")
    path = tmp_path / "bad.bam"
    path.write_bytes(bytes(data))
    r = bam.BamReader(str(path))
    with pytest.raises(RuntimeError, match="BGZF"):
        for _ in r.batches(100000, device=True):
            pass
    with pytest.raises(RuntimeError, match="failed earlier"):  # the reader stays failed
        r.next_batch(100000, device=True)
    r.close()
