"""Reference store on the CPU: shared-memory publication and mapping (the preloader), the segment name of a
file, validation of segments and inputs. No GPU call is made (no upload, no engine)."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]

pytestmark = pytest.mark.skipif(not os.path.isdir("/dev/shm"), reason="POSIX shared memory not mounted")


@pytest.fixture(scope="module")
def reference():
    from firepony_gb300 import synth
    p = synth.PRESETS["precision_20M_151bp_pe"].scaled(num_reads=1000, total_reference_bp=400_003)
    return synth.Reference(p)


@pytest.fixture
def shm_name(request):
    name = f"/fpgb_test_{os.getpid()}_{request.node.name[:40]}"
    yield name
    from firepony_gb300.refstore import RefStore
    RefStore.unlink(name)


def masked(words, n):
    w = np.array(words, dtype=np.uint32, copy=True)
    if n % 8:
        w[-1] &= (1 << ((n % 8) * 4)) - 1
    return w


def assert_same_contents(ref, store):
    assert len(store.contigs) == len(ref.contigs)
    for (w1, n1), (w2, n2) in zip(ref.contigs, store.contigs):
        assert n1 == n2
        assert np.array_equal(masked(w1, n1), w2)
    for (a, b), (c, d) in zip(ref.sites, store.sites):
        assert np.array_equal(a, c) and np.array_equal(b, d)


def test_publish_open_round_trip(reference, shm_name):
    from firepony_gb300.refstore import RefStore
    with RefStore.build(reference) as s:
        info = s.info()
        assert info["num_contigs"] == len(reference.contigs) and info["mapped"] == 0 and info["device"] == -1
        assert info["total_bases"] == sum(n for _, n in reference.contigs)
        assert info["total_sites"] == sum(len(a) for a, _ in reference.sites)
        assert_same_contents(reference, s)
        s.publish(shm_name)
        built_bytes = info["image_bytes"]
    with RefStore.open(shm_name) as m:
        info = m.info()
        assert info["mapped"] == 1 and info["image_bytes"] == built_bytes
        assert os.path.getsize("/dev/shm" + shm_name) == built_bytes
        assert_same_contents(reference, m)
        # a mapped store republishes the same image under another name
        other = shm_name + "_b"
        try:
            m.publish(other)
            with RefStore.open(other) as m2:
                assert_same_contents(reference, m2)
        finally:
            RefStore.unlink(other)


def test_image_layout_prefix_max_and_padding(reference, shm_name):
    """The segment holds the device layout: 256-byte aligned arrays, the last word's unused symbols zeroed, a
    zero word after each contig, and the prefix maximum of the stops after start and stop."""
    from firepony_gb300.refstore import RefStore
    with RefStore.build(reference) as s:
        s.publish(shm_name)
    raw = np.fromfile("/dev/shm" + shm_name, dtype=np.uint8)
    hdr = raw[:64]
    assert bytes(hdr[:8]) == b"FPGBREFS"
    nc = int(hdr[12:16].view(np.uint32)[0])
    dir_ = raw[64:64 + 48 * nc].view(np.uint64).reshape(nc, 6)
    for cid, (words, n) in enumerate(reference.contigs):
        num_bases, coff, cwords, soff = (int(x) for x in dir_[cid, :4])
        nsites = int(dir_[cid, 4] & 0xFFFFFFFF)
        assert num_bases == n and cwords == (n + 7) // 8 + 1 and coff % 256 == 0
        img_words = raw[coff:coff + 4 * cwords].view(np.uint32)
        assert np.array_equal(img_words[:-1], masked(words, n)) and img_words[-1] == 0
        st, sp = reference.sites[cid]
        assert nsites == len(st)
        if nsites:
            assert soff % 256 == 0
            arr = raw[soff:soff + 12 * nsites].view(np.uint32)
            assert np.array_equal(arr[:nsites], st) and np.array_equal(arr[nsites:2 * nsites], sp)
            assert np.array_equal(arr[2 * nsites:], np.maximum.accumulate(sp))


def test_shm_name_follows_the_reference(tmp_path):
    """compute_shmem_path (mmap.cu:57-89): "/firepony_" + realpath with every '/' replaced by '_'."""
    from firepony_gb300.refstore import RefStore, RefStoreError
    f = tmp_path / "sub" / "ref.fa"
    f.parent.mkdir()
    f.write_text(">c\nACGT\n")
    link = tmp_path / "link.fa"
    link.symlink_to(f)
    want = "/firepony_" + os.path.realpath(f).replace("/", "_")
    assert RefStore.shm_name(str(f)) == want
    assert RefStore.shm_name(str(link)) == want  # the absolute path resolves links
    with pytest.raises(RefStoreError):
        RefStore.shm_name(str(tmp_path / "missing.fa"))


def test_input_validation(reference, shm_name):
    from firepony_gb300.refstore import RefStore, RefStoreError
    with RefStore.create(2) as s:
        with pytest.raises(RefStoreError, match="out of range"):
            s.set_contig(2, np.zeros(1, np.uint32), 8)
        with pytest.raises(RefStoreError, match="sorted"):
            s.set_known_sites(0, np.array([5, 3], np.uint32), np.array([6, 4], np.uint32))
        s.set_contig(0, np.array([0x12481248], np.uint32), 8)  # contig 1 stays empty
        for bad in ("noslash", "/a/b", "/", "/" + "x" * 300):
            with pytest.raises(RefStoreError):
                s.publish(bad)
        s.publish(shm_name)
        info = s.info()
        assert info["total_bases"] == 8 and info["total_sites"] == 0
    with RefStore.open(shm_name) as m:
        (w0, n0), (w1, n1) = m.contigs
        assert n0 == 8 and w0.tolist() == [0x12481248] and n1 == 0 and len(w1) == 0
        with pytest.raises(RefStoreError, match="read-only"):
            m.set_contig(0, np.zeros(1, np.uint32), 8)
    with pytest.raises(RefStoreError, match="No such file"):
        RefStore.open(shm_name + "_missing")


def _corrupt(name, offset, data: bytes):
    with open("/dev/shm" + name, "r+b") as f:
        f.seek(offset)
        f.write(data)


@pytest.mark.parametrize("case", ["incomplete", "magic", "directory", "truncated", "version"])
def test_damaged_segments_are_refused(reference, shm_name, case):
    from firepony_gb300.refstore import RefStore, RefStoreError
    with RefStore.build(reference) as s:
        s.publish(shm_name)
    path = "/dev/shm" + shm_name
    if case == "incomplete":       # the writer's completion mark
        _corrupt(shm_name, 48, b"\0\0\0\0")
        msg = "incomplete"
    elif case == "magic":
        _corrupt(shm_name, 0, b"XXXXXXXX")
        msg = "not a reference store"
    elif case == "directory":      # a contig's length in the directory
        _corrupt(shm_name, 64, b"\x01")
        msg = "checksum"
    elif case == "truncated":
        os.truncate(path, os.path.getsize(path) - 256)
        msg = "size"
    else:
        _corrupt(shm_name, 8, b"\x63\0\0\0")
        msg = "version"
    with pytest.raises(RefStoreError, match=msg):
        RefStore.open(shm_name)


def test_republish_keeps_existing_mappings_valid(reference, shm_name):
    """Publishing replaces the name, not the object: a process still mapping the old segment reads the old
    image, and a new open sees the new one."""
    from firepony_gb300.refstore import RefStore
    with RefStore.create(1) as a:
        a.set_contig(0, np.array([0x11111111], np.uint32), 8)
        a.publish(shm_name)
    old = RefStore.open(shm_name)
    with RefStore.create(1) as b:
        b.set_contig(0, np.array([0x22222222, 0x4], np.uint32), 9)
        b.publish(shm_name)
    try:
        assert old.contigs[0][1] == 8 and old.contigs[0][0].tolist() == [0x11111111]
        with RefStore.open(shm_name) as new:
            assert new.contigs[0][1] == 9 and new.contigs[0][0].tolist() == [0x22222222, 0x4]
    finally:
        old.close()


def test_preloader_in_another_process(reference, shm_name):
    """One process publishes (the preloader), a later one maps the segment: the same contents."""
    from firepony_gb300.refstore import RefStore
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "from firepony_gb300 import synth\n"
        "from firepony_gb300.refstore import RefStore\n"
        "p = synth.PRESETS['precision_20M_151bp_pe'].scaled(num_reads=1000, total_reference_bp=400_003)\n"
        "RefStore.build(synth.Reference(p)).publish(%r)\n" % (str(ROOT), shm_name))
    subprocess.run([sys.executable, "-c", code], check=True, timeout=300)
    with RefStore.open(shm_name) as m:
        assert_same_contents(reference, m)
