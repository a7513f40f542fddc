"""BAM input: BGZF + record decoding into the engine's batch layout (CPU; no GPU needed)."""
import numpy as np
import pytest

from firepony_gb300 import synth


def _remap_first_occurrence(rg):
    """read-group ids in order of first occurrence (the reference loader's read_groups_db.insert)."""
    out = np.empty_like(rg)
    seen = {}
    for i, g in enumerate(rg):
        if g not in seen:
            seen[g] = len(seen)
        out[i] = seen[g]
    return out, seen


@pytest.fixture(scope="module")
def data(tmp_path_factory):
    pytest.importorskip("zlib")
    from firepony_gb300 import bam
    try:
        bam.lib()
    except RuntimeError as ex:
        pytest.skip(str(ex))
    p = synth.PRESETS["batched_uneven"].scaled(num_reads=5000, total_reference_bp=400_000, batch_reads=2500)
    ref = synth.Reference(p)
    batches = [ref.batch(0, 2500), ref.batch(1, 2500)]
    path = tmp_path_factory.mktemp("bam") / "x.bam"
    targets = [(f"chr{i}", int(n)) for i, (_, n) in enumerate(ref.contigs)]
    rg_ids = [f"rg{i}" for i in range(p.num_read_groups)]
    bam.write_bam(str(path), targets, rg_ids, batches, level=1, threads=4)
    return p, ref, batches, path, targets, rg_ids


@pytest.mark.parametrize("max_reads", [5000, 1000, 777])
def test_decode_equals_written(data, max_reads):
    from firepony_gb300 import bam
    p, ref, batches, path, targets, rg_ids = data
    r = bam.BamReader(str(path), threads=3)
    assert r.targets == targets
    got = [b.to_batch() for b in r.batches(max_reads)]
    names = r.read_group_names
    st = r.stats
    r.close()
    assert st["records"] == 5000 and st["batches"] == len(got) and st["compressed_bytes"] == path.stat().st_size
    assert sum(b.num_reads for b in got) == 5000
    assert all(b.num_reads <= max_reads for b in got)
    whole = {k: np.concatenate([b[k] for b in batches]) for k in batches[0].arrays}
    dec = {k: np.concatenate([b[k] for b in got]) for k in got[0].arrays}
    for k in ("chromosome", "alignment_start", "alignment_stop", "mate_alignment_start", "inferred_insert_size",
              "cigar_len", "read_len", "qual_len", "flags", "mapq", "cigars", "qualities"):
        np.testing.assert_array_equal(dec[k], whole[k], err_msg=k)
    want_rg, seen = _remap_first_occurrence(whole["read_group"])
    np.testing.assert_array_equal(dec["read_group"], want_rg)
    assert names == [rg_ids[g] for g in sorted(seen, key=seen.get)]
    # bases (each read padded to 8 symbols in both layouts)
    syms_w = np.concatenate([synth.unpack4(b["reads"], b.num_read_symbols) for b in batches])
    syms_d = np.concatenate([synth.unpack4(b["reads"], b.num_read_symbols) for b in got])
    assert len(syms_w) == len(syms_d)
    np.testing.assert_array_equal(syms_d, syms_w)


def test_target_map_and_bad_file(data, tmp_path):
    from firepony_gb300 import bam
    p, ref, batches, path, targets, rg_ids = data
    r = bam.BamReader(str(path), threads=2)
    r.set_target_map([3, 2, 1, 0][:len(targets)])
    b = r.next_batch(100000).to_batch()
    r.close()
    m = np.array([3, 2, 1, 0][:len(targets)], np.uint16)
    orig = np.concatenate([x["chromosome"] for x in batches])
    want = np.where(orig == 0xFFFF, 0xFFFF, m[np.minimum(orig, len(m) - 1)])
    np.testing.assert_array_equal(b["chromosome"], want)
    bad = tmp_path / "bad.bam"
    bad.write_bytes(b"not a bam file at all")
    with pytest.raises(RuntimeError):
        bam.BamReader(str(bad))


def test_bgzf_block_decoder_against_zlib():
    """The GPU's DEFLATE block decoder (csrc/bgzf_inflate.cuh), built for the host with the address and
    undefined-behaviour sanitizers: round trips of zlib streams at every level and strategy, CRC-32 and CRC
    concatenation against zlib, and corrupt or truncated streams that must end in an error status inside
    the buffers."""
    import subprocess
    from firepony_gb300 import build
    if not build.zlib_available():
        pytest.skip("zlib headers missing")
    try:
        exe = build.build_inflate_check(sanitize=True)
    except RuntimeError as ex:
        if "sanitize" not in str(ex) and "asan" not in str(ex):
            raise
        exe = build.build_inflate_check(sanitize=False)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")


def test_corrupt_block_fails_and_stays_failed(data, tmp_path):
    """A BGZF block with a wrong CRC-32 ends decoding with an error; the reader then refuses further batches
    (its undecoded stream is undefined after the error) instead of returning later records."""
    from firepony_gb300 import bam
    p, ref, batches, path, targets, rg_ids = data
    raw = bytearray(path.read_bytes())
    o, blocks = 0, []
    while o + 18 <= len(raw):
        n = int.from_bytes(raw[o + 16:o + 18], "little") + 1
        blocks.append((o, n))
        o += n
    o, n = blocks[len(blocks) // 2]
    raw[o + n - 8] ^= 0x5A  # CRC-32 field of a middle block
    bad = tmp_path / "crc.bam"
    bad.write_bytes(bytes(raw))
    r = bam.BamReader(str(bad), threads=2)
    with pytest.raises(RuntimeError, match="BGZF"):
        for _ in r.batches(500):
            pass
    with pytest.raises(RuntimeError, match="failed earlier"):
        r.next_batch(500)
    r.close()
