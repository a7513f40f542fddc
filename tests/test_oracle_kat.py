"""Known-answer and cross-implementation tests that pin the oracle stage by stage.

The reference ships no tests or fixtures and cannot be built here, so the oracle (a C++ restatement) is
checked against values worked out by hand from the cited reference lines, and against independent Python
restatements of the same formulas (which call the platform libm through ctypes, as the reference's host
build does)."""
import ctypes
import math

import numpy as np
import pytest

from oracle import oracle as O

libm = ctypes.CDLL("libm.so.6")
libm.lgammaf.restype = ctypes.c_float
libm.lgammaf.argtypes = [ctypes.c_float]


# ---- MAP quality conversion (device/baq.cu:673-674) ----
@pytest.mark.parametrize("mx,expected", [
    (1.0, 99),              # 1 - max == 0 -> +inf -> saturates to INT_MAX -> capped 99 (CUDA / Arm / Java)
    (0.999, 30),            # -4.343 ln(0.001) + 0.499 = 30.499...
    (0.5, 4),               # 3.51 -> 3 -> raised to MIN_BASE_QUAL
    (1 - 1e-10, 100),       # 100.49...: k == 100 is not > 100, kept
    (1 - 1e-11, 99),        # 110.5 -> > 100 -> 99
    (float("nan"), 4),      # (int)NaN -> 0 -> 4
    (0.0, 4),
])
def test_map_quality_known_answers(mx, expected):
    assert O.baq_quality_from_max(mx) == expected


# ---- empirical quality (device/empirical_quality.cu:35-198), independent restatement ----
def c_round(x):
    """C round(): halves away from zero."""
    return math.copysign(math.floor(abs(x) + 0.5), x)


def py_empirical(obs, mism, est, need_rounding):
    MAXOBS = 2147483647 - 1
    k = int(mism + 0.5) + 1
    n = obs + 2
    if n > MAXOBS:
        frac = MAXOBS / n
        k = int(c_round(k * frac))
        n = MAXOBS

    def lf(x):
        return float(libm.lgammaf(float(x + 1))) * math.log10(math.e)

    coef = lf(n) - lf(k) - lf(n - k)
    best, best_bin = None, 0
    for b in range(61):
        delta = b - est
        if need_rounding:
            delta = c_round(delta)
        diff = min(abs(int(delta)), 40)
        g = 0.0 + 0.9 * math.pow(math.e, -(math.pow(diff - 0.0, 2.0) / (2 * 0.5 * 0.5)))
        prior = math.log10(g) if g > 0 else float("-inf")  # C log10(0) = -inf
        log10p = b / -10.0
        one_m = 1 - math.pow(10.0, log10p)
        l1mp = math.log10(one_m) if one_m > 0 else float("-inf")
        lik = coef + log10p * k + l1mp * (n - k)
        post = prior + lik
        if best is None or post > best:
            best, best_bin = post, b
    return min(float(best_bin), 93.0)


@pytest.mark.parametrize("obs,mism,est,rnd", [
    (1000, 10.0, 20.0, True), (100000, 3.25, 30.0, True), (5, 0.0, 40.0, True), (2, 1.0, 6.0, True),
    (123456, 1234.5, 20.0, True), (10**7, 10**5 + 0.25, 20.0, True), (50, 49.5, 10.0, True),
    (2**32, 4.2e7, 20.0, True), (3 * 10**9, 1.0, 40.0, True),
    (1000, 10.0, 20.37, False), (987654, 4321.0, 27.5, False), (77, 7.0, 30.000000000000004, False),
    (77, 7.0, 29.999999999999996, False), (10, 0.0, 45.0, False),
])
def test_empirical_quality_matches_independent_restatement(obs, mism, est, rnd):
    assert O.empirical_quality(obs, mism, est, rnd) == py_empirical(obs, mism, est, rnd)


def test_empirical_quality_known_answers():
    # 1% observed errors around Q20 with a Q20 report: posterior peaks at 20
    assert O.empirical_quality(100000, 1000.0, 20.0, True) == 20.0
    # no errors at all: the smoothing error (+1) over 10^6 observations -> ~Q60 region, capped by the prior
    assert O.empirical_quality(10**6, 0.0, 40.0, True) == pytest.approx(O.empirical_quality(10**6, 0.4, 40.0, True))


# ---- BAQ HMM (device/baq.cu:214-697), independent Python transcription ----
def py_hmm(ref, query, qual, bw, bm_ref_len=None):
    EM, EI, GEP = 0.33333333333, 0.25, 0.1
    GOP = math.pow(10.0, -40.0 / 10.0)
    lref = len(ref)
    bmL = bm_ref_len if bm_ref_len is not None else lref
    ql = len(query)
    bw2 = bw * 2 + 1
    row = bw2 * 3 + 6
    F = [[0.0] * row for _ in range(ql + 1)]
    B = [[0.0] * row for _ in range(ql + 1)]
    S = [0.0] * (ql + 2)
    sM = 1.0 / (2 * ql + 2)
    sI = sM
    bM = (1 - GOP) / bmL
    bI = GOP / bmL
    m = [(1 - GOP - GOP) * (1 - sM), GOP * (1 - sM), GOP * (1 - sM),
         (1 - GEP) * (1 - sI), GEP * (1 - sI), 0.0, 1 - GEP, 0.0, GEP]

    def su(i, k):
        x = max(i - bw, 0)
        return (k + 1 - x) * 3

    def eps(r, q, qq):
        if r == 15 or q == 15:
            return 1.0
        p = math.pow(10.0, -max(qq, 4) / 10.0)
        return 1 - p if r == q else p * EM

    S[0] = 1.0
    end = min(lref, bw + 1)
    s = 0.0
    for k in range(1, end + 1):
        e = eps(ref[k - 1], query[0], qual[0])
        u = su(1, k)
        F[1][u] = e * bM
        F[1][u + 1] = EI * bI
        s += F[1][u] + F[1][u + 1]
    S[1] = s
    for k in range(su(1, 1), su(1, end) + 3):
        F[1][k] /= s
    for i in range(2, ql + 1):
        beg, end = max(1, i - bw), min(lref, i + bw)
        s = 0.0
        fi, f1 = F[i], F[i - 1]
        for k in range(beg, end + 1):
            e = eps(ref[k - 1], query[i - 1], qual[i - 1])
            u, v11, v10, v01 = su(i, k), su(i - 1, k - 1), su(i - 1, k), su(i, k - 1)
            fi[u] = e * (m[0] * f1[v11] + m[3] * f1[v11 + 1] + m[6] * f1[v11 + 2])
            fi[u + 1] = EI * (m[1] * f1[v10] + m[4] * f1[v10 + 1])
            fi[u + 2] = m[2] * fi[v01] + m[8] * fi[v01 + 2]
            s += fi[u] + fi[u + 1] + fi[u + 2]
        S[i] = s
        inv = 1. / s
        for k in range(su(i, beg), su(i, end) + 3):
            fi[k] *= inv
    s = 0.0
    for k in range(1, lref + 1):
        u = su(ql, k)
        if u < 3 or u >= bw2 * 3 + 3:
            continue
        s += F[ql][u] * sM + F[ql][u + 1] * sI
    S[ql + 1] = s
    for k in range(1, lref + 1):
        u = su(ql, k)
        if u < 3 or u >= bw2 * 3 + 3:
            continue
        B[ql][u] = sM / S[ql] / S[ql + 1]
        B[ql][u + 1] = sI / S[ql] / S[ql + 1]
    for i in range(ql - 1, 0, -1):
        beg, end = max(1, i - bw), min(lref, i + bw)
        y = 1.0 if i > 1 else 0.0
        bi, b1 = B[i], B[i + 1]
        for k in range(end, beg - 1, -1):
            u, v11, v10, v01 = su(i, k), su(i + 1, k + 1), su(i + 1, k), su(i, k + 1)
            e = 0.0 if k >= lref else eps(ref[k], query[i], qual[i]) * b1[v11]
            bi[u] = e * m[0] + EI * m[1] * b1[v10 + 1] + m[2] * bi[v01 + 2]
            bi[u + 1] = e * m[3] + EI * m[4] * b1[v10 + 1]
            bi[u + 2] = (e * m[6] + m[8] * bi[v01 + 2]) * y
        yy = 1.0 / S[i]
        for k in range(su(i, beg), su(i, end) + 3):
            bi[k] *= yy
    quals, states = [], []
    for i in range(1, ql + 1):
        beg, end = max(1, i - bw), min(lref, i + bw)
        s, mx, mk = 0.0, 0.0, -1
        for k in range(beg, end + 1):
            u = su(i, k)
            for st in (0, 1):
                z = F[i][u + st] * B[i][u + st]
                s += z
                if z > mx:
                    mx, mk = z, (k - 1) << 2 | st
        mx /= s
        one_minus = 1.0 - mx
        t = -4.343 * math.log(one_minus) + 0.499 if one_minus > 0 else float("inf")
        kq = 2147483647 if t >= 2147483647 else int(t)
        quals.append(99 if kq > 100 else max(kq, 4))
        states.append(mk & 0xFFFFFFFF)
    return quals, states


@pytest.mark.parametrize("seed", range(6))
def test_hmm_matches_independent_transcription(seed):
    rng = np.random.default_rng(seed)
    ql = int(rng.integers(8, 40))
    lref = ql + 6 + int(rng.integers(0, 4))
    sym = np.array([1, 2, 4, 8], np.uint8)
    ref = sym[rng.integers(0, 4, lref)]
    query = ref[3:3 + ql].copy()
    for i in rng.integers(0, ql, 3):
        query[i] = sym[rng.integers(0, 4)]
    if seed % 3 == 0:
        query[ql // 2] = 15  # an N
    qual = rng.integers(2, 42, ql).astype(np.uint8)
    bw = 7 if seed % 2 == 0 else 9
    oq, ost = O.hmm(ref, query, qual, bw)
    pq, pst = py_hmm([int(x) for x in ref], [int(x) for x in query], [int(x) for x in qual], bw)
    assert list(oq) == pq
    assert list(ost) == pst


def test_hmm_perfect_match_is_confident():
    ref = np.array([1, 2, 4, 8, 1, 4, 2, 8, 8, 1, 2, 2, 4, 1, 8, 4, 2, 1, 1, 8], np.uint8)
    q = ref[3:17].copy()
    qual = np.full(len(q), 35, np.uint8)
    oq, st = O.hmm(ref, q, qual, 7)
    # interior bases align at their own column with (near) certainty
    assert all(x >= 35 for x in oq[3:-3])
    assert [s >> 2 for s in st[3:-3]] == list(range(6, 6 + len(q) - 6))
    assert all((s & 3) == 0 for s in st)


def _unpack4(words, start, n):
    return np.array([(int(words[(start + i) // 8]) >> (4 * ((start + i) % 8))) & 15 for i in range(n)], np.uint8)


def test_tied_indel_dataset_splits_the_posterior():
    """Every one-base deletion placement of tied_indel_dataset leaves its tied base (read offset 20) with MAP
    quality MIN_BASE_QUAL in the oracle's HMM, its MAP state a match at one of the run's two reference copies;
    both CIGAR placements of the same read give the same HMM outputs."""
    from tests.edge_cases import tied_indel_dataset
    contigs, sites, b, n_rg, _ = tied_indel_dataset(tie_quals=(2, 30))
    o = O.Oracle(n_rg)
    O.lib().fpo_set_contig(o.h, 0, np.ascontiguousarray(contigs[0][0], np.uint32).ctypes.data, contigs[0][1])
    o.process(b)
    bw = o.debug_last_batch(b)["hmm"][:, 2]
    words = contigs[0][0]
    prev = None
    for r in range(b.num_reads):
        ops = b["cigars"][b["cigar_start"][r]:b["cigar_start"][r] + b["cigar_len"][r]]
        if (int(ops[1]) >> 24) != 2:  # deletion placements only (the second CIGAR op is the one-base D)
            continue
        start, stop = int(b["alignment_start"][r]), int(b["alignment_stop"][r])
        # HMM window: the aligned span plus MIN_BAND_WIDTH / 2 reference bases on each side
        win = _unpack4(words, start - 3, stop - start + 7)
        rl = int(b["read_len"][r])
        query = _unpack4(b["reads"], int(b["read_start"][r]), rl)
        qual = b["qualities"][b["qual_start"][r]:b["qual_start"][r] + rl]
        oq, st = O.hmm(win, query, qual, int(bw[r]))
        assert oq[20] == 4, (r, oq[18:23])
        assert (st[20] & 3) == 0 and (st[20] >> 2) in (23, 24), (r, st[20] >> 2)
        if prev is not None and prev[0] == start:
            np.testing.assert_array_equal(prev[1], oq)
            np.testing.assert_array_equal(prev[2], st)
        prev = (start, oq, st)
    o.close()
