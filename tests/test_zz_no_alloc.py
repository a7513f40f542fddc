"""GPU test of fp_sort_entries_static, the sort entry point that allocates no device memory (for callers
that must not allocate while they run, such as a job loop admitting work against a fixed HBM budget).
It is called through the C ABI twice in a row and must match fp_sort_entries (the allocating entry point)
bit for bit; sizes above its fixed scratch capacity are rejected. Kept in its own file, collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP_OK, FP_BAD_INPUT = 0, 1
MAX = 1 << 20


def _lib():
    from firepony_gb300.engine import lib
    L = lib()
    L.fp_sort_entries_static.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                                         ctypes.c_void_p]
    L.fp_sort_entries.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p]
    return L


def _entries(n, key_bits, seed):
    rng = np.random.default_rng(seed)
    keys = rng.integers(0, 1 << key_bits, n, dtype=np.uint64)
    return (keys << np.uint64(32)) | rng.integers(0, 1 << 32, n, dtype=np.uint64)


def test_static_sort_matches_allocating_sort_twice():
    import torch
    L = _lib()
    for call, (n, bits) in enumerate([(MAX, 24), (300_001, 28)]):
        a = _entries(n, bits, seed=call)
        d_in = torch.from_numpy(a.view(np.int64).copy()).cuda()
        want = torch.empty_like(d_in)
        got = torch.empty_like(d_in)
        torch.cuda.synchronize()
        assert L.fp_sort_entries(d_in.data_ptr(), want.data_ptr(), n, bits, None) == FP_OK
        torch.cuda.synchronize()
        assert L.fp_sort_entries_static(d_in.data_ptr(), got.data_ptr(), n, bits, None) == FP_OK
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"call {call}: static sort differs"
        assert torch.equal(d_in.cpu(), torch.from_numpy(a.view(np.int64)))


def test_static_sort_rejects_sizes_above_capacity():
    import torch
    L = _lib()
    d = torch.zeros(8, dtype=torch.int64, device="cuda")
    assert L.fp_sort_entries_static(d.data_ptr(), d.data_ptr(), MAX + 1, 20, None) == FP_BAD_INPUT
