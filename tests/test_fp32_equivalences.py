"""Exactness arguments the kernels rely on, checked exhaustively on the host."""
import numpy as np


def test_fractional_error_division_single_rounding():
    """float(double(n) / double(len)) (the reference's fractional error) equals one correctly rounded FP32
    division for every count and window length the engine can meet (reads of at most 511 bases)."""
    n = np.arange(0, 512, dtype=np.float64)[:, None]
    ln = np.arange(1, 513, dtype=np.float64)[None, :]
    via_double = (n / ln).astype(np.float32)
    direct = n.astype(np.float32) / ln.astype(np.float32)
    assert int((via_double != direct).sum()) == 0
