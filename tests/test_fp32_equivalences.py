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


def test_fp32_baq_range_arguments():
    """The FP32 BAQ kernels' range arguments, in float32 arithmetic: with base qualities <= 93 (higher ones go
    to the exact replay) every emission is >= 1.67e-10, and
    - band class 0: a stored value >= 1e-22 times any factor chain of the next row (emission, gap-open
      transition, 0.1 extension, insertion emission 0.25) stays a normal float;
    - flush-and-bound (classes 1 and 2): operands >= 2^-78 keep every product and sum of a row normal, and a
      flushed value's absolute error, carried through the row scaling, stays far below the 2^-24 slack."""
    tiny = np.float32(np.finfo(np.float32).tiny)  # 2^-126
    q = np.arange(0, 94)
    p = 10.0 ** (-np.maximum(q, 4) / 10.0)
    e_mis = (p * 0.33333333333).astype(np.float32)
    e_match = (1 - p).astype(np.float32)
    e_min = min(e_mis.min(), e_match.min())
    assert e_min >= np.float32(1.6e-10)
    gop = 10.0 ** (-4.0)
    ds_max = 1.0 / (2 * 1 + 2)  # qL >= 1
    m2_min = np.float32(gop * (1 - ds_max))  # gap open (and m1)
    # class 0: one row of products from a stored value >= 1e-22 (the D chain of the same row adds m2 then 0.1 steps
    # whose values are stored or rescaled within the row sum)
    v = np.float32(1e-22) * e_min * np.float32(0.9) * m2_min
    assert v >= tiny
    # flush-and-bound: every operand is 0 or >= 2^-78, and a computed cell is flushed before it feeds another
    # cell, so the products of a row are at most two factors deep on a kept operand: emission x transition
    # (M, and the backward e = emission x B_M then x m0 / m3 / m6), EI x m1 or m4 (I), m2 x M and m8 x D (the D
    # chains)
    flush = np.float32(2.0 ** -78)
    m_min = min(np.float32((1 - 2 * gop) * (1 - ds_max)), np.float32(0.9 * (1 - ds_max)), np.float32(0.9))
    chains = [flush * e_min * m_min, flush * np.float32(0.25) * m2_min, flush * m2_min, flush * np.float32(0.1)]
    assert min(chains) >= tiny
    assert min(chains) >= np.float32(2.0 ** -112)
    assert float(flush) == 3.3087224502121107e-24
    # posterior terms of two kept values may underflow: 2^-150 each at most, far below a row sum >= 2^0
    assert 2 * 63 * 2.0 ** -150 < 2.0 ** -24


def test_tied_map_states_cap_at_min_base_qual():
    """A base whose MAP state is undecided (a rival term within the certified bound of the maximum) keeps the
    best posterior at or below about 1/2, so the reference's MAP quality (device/baq.cu:673: (int)(-4.343 *
    log(1 - max) + .499), clamped to [MIN_BASE_QUAL, 99]) is MIN_BASE_QUAL = 4 whichever term wins; the FP32
    kernels additionally require the certified upper end of t below 4.9. The capping step
    (device/baq.cu:895-909) then gives min(4, oq) at the expected match and 4 elsewhere: one value when oq >= 4."""
    min_base_qual = 4

    def map_quality(p_max):
        k = np.trunc(-4.343 * np.log(1.0 - p_max) + 0.499).astype(np.int64)
        return np.where(k > 100, 99, np.where(k < min_base_qual, min_base_qual, k))

    rel_state = 1e-3  # far wider than any kernel's state bound
    # posterior of the best of two terms within rel_state of each other, any remaining mass elsewhere
    p = np.linspace(0.0, 1.0 / (2.0 - rel_state), 200_001)
    assert (map_quality(p) == min_base_qual).all()
    # a candidate's t exceeds the certified upper end by far less than 0.05 (a few relative bounds of about
    # 1e-4); t up to 4.9 + 0.05 still floors to 4
    t_hi = np.float32(4.9)
    p_at = 1.0 - np.exp((0.499 - float(t_hi) - 0.05) / 4.343)
    assert map_quality(np.array([p_at]))[0] == min_base_qual
    oq = np.arange(0, 94)
    at_expected = np.minimum(min_base_qual, oq)
    elsewhere = np.full_like(oq, min_base_qual)
    assert ((at_expected == elsewhere) == (oq >= min_base_qual)).all()


def test_tag_property_is_monotone_in_t():
    """The FP32 kernels decide, per base, whether the capped quality equals the base's quality (the BQ tag is
    NO_BAQ_UNCERTAINTY), the one property of the tag the reference reads (fractional_errors.cu:93). At the
    expected match the capped value is min(capped_q(t), oq) with capped_q the reference's MAP quality
    (device/baq.cu:673: floor, clamped to [MIN_BASE_QUAL, 99], 100 kept); the test capped_q(t) >= oq is
    monotone in t for oq <= 99, so the endpoints of a certified interval decide it (baq_amb bit 16). Elsewhere
    the capped value is MIN_BASE_QUAL, equal to oq exactly when oq == 4."""
    min_base_qual = 4

    def capped_q(t):
        t = np.asarray(t, np.float64)
        k = np.where(np.isnan(t), 0, np.where(t >= 2147483520.0, 2147483647, np.floor(np.nan_to_num(t, neginf=-1e18))))
        k = np.maximum(k, -2.0 ** 31)
        return np.where(k > 100, 99, np.where(k < min_base_qual, min_base_qual, k)).astype(np.int64)

    t = np.concatenate([[-np.inf], np.linspace(-5.0, 130.0, 270_001), [np.inf]])
    for oq in range(0, 100):
        same = np.minimum(capped_q(t), oq) == oq
        # monotone: once true, true for every larger t
        first = np.argmax(same) if same.any() else len(t)
        assert same[first:].all(), oq
        if oq <= min_base_qual:
            assert same.all()
    # qualities above 100 never equal a capped value (the kernels leave such reads to the exact replay)
    assert not (capped_q(t) >= 101).any()
    # elsewhere than the expected match
    oq = np.arange(0, 94)
    assert ((np.full_like(oq, min_base_qual) == oq) == (oq == min_base_qual)).all()
