"""GPU tests of the stable radix sort exposed as fp_sort_entries (the engine's K4 sort)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def reference_sort(a, key_bits):
    key = (a >> np.uint64(32)) & np.uint64((1 << key_bits) - 1)
    return a[np.argsort(key, kind="stable")]


@pytest.mark.parametrize("n,key_bits", [(1, 8), (1000, 8), (4097, 12), (70_001, 20), (1 << 20, 28), (3_000_017, 24),
                                        (2_000_003, 32)])
def test_sort_entries_stable(native, n, key_bits):
    import torch
    from firepony_gb300.engine import sort_entries
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 1 << key_bits, n, dtype=np.uint64)
    payload = np.arange(n, dtype=np.uint64)  # stream position, so stability is visible
    a = (keys << np.uint64(32)) | payload
    d_in = torch.from_numpy(a.view(np.int64).copy()).cuda()
    d_out = torch.empty_like(d_in)
    sort_entries(d_in.data_ptr(), d_out.data_ptr(), n, key_bits)
    torch.cuda.synchronize()
    got = d_out.cpu().numpy().view(np.uint64)
    np.testing.assert_array_equal(got, reference_sort(a, key_bits))
    # the input is left untouched
    np.testing.assert_array_equal(d_in.cpu().numpy().view(np.uint64), a)


def test_sort_entries_skewed_digits(native):
    """Covariate keys are dense and skewed: long runs share their high digits and a few keys take most
    entries. Runs of one digit across whole warps and tiles, and tiles of a single key, keep the order."""
    import torch
    from firepony_gb300.engine import sort_entries
    rng = np.random.default_rng(11)
    n = 1_500_000
    hot = rng.integers(0, 40, n // 2, dtype=np.uint64)            # a few hot keys
    cold = rng.integers(0, 1 << 21, n - n // 2, dtype=np.uint64)  # spread over 21 bits
    keys = np.concatenate([np.sort(hot)[: n // 4], hot[n // 4:], cold])
    keys[:300_000] = 7                                             # one key over many whole tiles
    payload = np.arange(n, dtype=np.uint64)
    a = (keys << np.uint64(32)) | payload
    d_in = torch.from_numpy(a.view(np.int64).copy()).cuda()
    d_out = torch.empty_like(d_in)
    sort_entries(d_in.data_ptr(), d_out.data_ptr(), n, 29)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_out.cpu().numpy().view(np.uint64), reference_sort(a, 29))


@pytest.mark.parametrize("key_bits", [20, 13])
def test_sort_entries_ignores_bits_above_key_bits(native, key_bits):
    """Only key bits below key_bits decide the order: entries whose keys differ only above it (the last
    digit of a width that is not a multiple of the digit size) keep their input order."""
    import torch
    from firepony_gb300.engine import sort_entries
    rng = np.random.default_rng(key_bits)
    n = 300_001
    low = rng.integers(0, 1 << key_bits, n, dtype=np.uint64)
    high = rng.integers(0, 1 << (32 - key_bits), n, dtype=np.uint64) << np.uint64(key_bits)  # noise above key_bits
    payload = np.arange(n, dtype=np.uint64)
    a = ((low | high) << np.uint64(32)) | payload
    d_in = torch.from_numpy(a.view(np.int64).copy()).cuda()
    d_out = torch.empty_like(d_in)
    sort_entries(d_in.data_ptr(), d_out.data_ptr(), n, key_bits)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_out.cpu().numpy().view(np.uint64), reference_sort(a, key_bits))
