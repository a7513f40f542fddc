// K2: the banded glocal BAQ HMM (device/baq.cu:214-697), one thread per read with the band row held in
// registers. W = 2*BW+1 band slots are fully unrolled, so every cell of a row is a named register: the
// M/I recurrences from the previous row are register reads, the D chain along the row is the natural
// sequential recurrence, and rows are updated in place. The forward rows (M, I) needed by MAP go to a
// per-warp scratch slot, interleaved by lane so each warp store/load moves 32 consecutive words; backward
// is fused with MAP.
//
// Two arithmetic modes share the code:
//   EXACT (double): the reference's operations in the reference's order, each multiply and add an explicit
//     __dmul_rn/__dadd_rn (never fused), so every intermediate double equals the reference's host value.
//     Used for reads the FP32 bound cannot decide.
//   FP32 (float): fused multiply-adds, with a certified relative error bound. Every HMM value is a sum of
//     products of non-negative terms, so a computed value is the exact one times (1 + theta) with
//     |theta| <= (roundings on the deepest path) * 2^-24, and the per-row scalings cancel in the posterior.
//     Per row a path takes at most 7 roundings (M or I entry: 5 including the emission, 1 for the row
//     scaling, 1 spare) plus 2 per D step, and a path makes at most refLen D steps, so forward and backward
//     values carry eps <= (7 qlen + 2 refLen + 8) 2^-24 each and a posterior term eps_z = 2 eps + 2^-24; a
//     sum of at most 2W terms adds 2W 2^-24, so the ratio (sum of the other terms)/(total) is within
//     rel = 2 (eps_z + 2W u) + u. A base's MAP quality is undecided when min(q_orig, clamp(floor(t'))) is not
//     constant for t' within dt = 4.343 rel / (1 - rel) + 1e-4 of the computed t (1e-4 covers logf and the
//     reference's own double rounding), and its MAP state is undecided when the runner-up term is within
//     2 eps_z + 2u (relative) of the best; such a base also records its rival state when there is exactly
//     one. Rows are rescaled by powers of two (forward sum 2^64, backward factor 2^32) so that band cells far
//     from the alignment stay normal numbers; a read with a stored M value below 1e-22 (where a product of the
//     next row could leave the normal range) is undecided throughout. Posterior terms of such far cells can
//     still round to subnormals; their absolute error (< 2W 2^-149) is ~1e-70 of the row's total and is
//     covered by the 2^-24 slack terms above.
#include "kernels.h"

namespace fpg {

__constant__ double ct_qual2prob[256];
__constant__ double ct_gap_open;

namespace {

constexpr u32 FULL = 0xffffffffu;
constexpr int TPR_THREADS = 128;

template <typename T, bool EXACT> struct Ar;
template <> struct Ar<double, true> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double mad(double a, double b, double c) { return __dadd_rn(__dmul_rn(a, b), c); }
};
template <> struct Ar<float, false> {
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float div(float a, float b) { return a / b; }
    static __device__ __forceinline__ float mad(float a, float b, float c) { return fmaf(a, b, c); }
};

// FP32 row scaling: forward rows are normalised to sum 2^64 (the reference: 1) and backward values carry a
// factor 2^32, so band cells down to ~1e-41 of their row stay normal numbers. Per-row constants cancel in the
// MAP ratios; every value, sum and posterior term stays below ~1e34.
constexpr float FWD_SCALE = 18446744073709551616.0f;    // 2^64
constexpr float BWD_INIT = 79228162514264337593543950336.0f;  // 2^96 = 2^64 (sLast) x 2^32 (backward factor)
__device__ __forceinline__ bool tiny_positive(float v) {
    // 0 < v < 1e-22 on the bit pattern (v >= 0 here). A stored M value (forward or backward) at or above 1e-22
    // keeps every product of the next row above 2^-126 (smallest emission 1.7e-10, gap transitions >= 1e-4,
    // insertion emission 0.25), so no operation of a read without a flag leaves the normal range.
    return (__float_as_uint(v) - 1u) < (0x1AF1C901u - 1u);
}
__device__ __forceinline__ bool tiny_positive(double) { return false; }

// Band class 1 (FP32, 31 slots) replaces the read-level guard above by flushing: a computed value below
// FLUSH_T becomes zero, so every operand is zero or at least 2^-78 and every kept product and sum stays at
// or above 2^-112 (normal), and each flush's absolute error (below 2^-78 in the units of its row) is bounded
// and added to the decision margins. The bound: a forward error e in row j reaches the posterior terms
// through backward values of at most 1 (reference units), i.e. at most e * prod(inv of the rows after j) /
// sLast of the posterior total; a backward error e in row i through forward values of at most the row sum
// 2^64, i.e. at most e * 2^64 / (row i's posterior sum); an underflowed posterior product adds at most 2^-150.
constexpr float FLUSH_T = 3.3087224502121107e-24f;  // 2^-78
template <typename T> __device__ __forceinline__ void flush_t(T &v, float &c) {
    if (v < T(FLUSH_T)) {
        c += v > T(0) ? 1.0f : 0.0f;
        v = T(0);
    }
}

template <typename T>
__device__ __forceinline__ T emission(const T *em_tab, const T *mis_tab, u8 ref, u8 rd, u8 q) {
    if (ref == IUPAC_N || rd == IUPAC_N) return T(1);
    return ref == rd ? em_tab[q] : mis_tab[q];
}

// calcEpsilon for one query base against any reference symbol: the match and mismatch values of the row,
// with a query N giving 1 for both; a reference N gives 1 (row_emission)
template <typename T>
__device__ __forceinline__ void row_emission(const T *em_tab, const T *mis_tab, u8 rd, u8 q, T &e_match, T &e_mis) {
    const bool n = rd == IUPAC_N;
    e_match = n ? T(1) : em_tab[q];
    e_mis = n ? T(1) : mis_tab[q];
}
template <typename T>
__device__ __forceinline__ T cell_emission(u8 ref, u8 rd, T e_match, T e_mis) {
    return ref == rd ? e_match : (ref == IUPAC_N ? T(1) : e_mis);
}

template <typename T, int W, bool EXACT>
__global__ void __launch_bounds__(TPR_THREADS) k_baq_tpr(DevBatch b, DevRef dref, BatchWork w, const u32 *list,
                                                         const u32 *count, u32 *work_ctr, T *scratch, u32 max_q,
                                                         u32 rpw) {
    using A = Ar<T, EXACT>;
    constexpr bool FL = !EXACT && W == 31;  // flush-and-bound instead of the read-level guard
    __shared__ T s_em[256], s_mis[256];
    for (int q = threadIdx.x; q < 256; q += blockDim.x) {
        const double p = ct_qual2prob[q < MIN_BASE_QUAL ? MIN_BASE_QUAL : q];
        // calcEpsilon (device/baq.cu:361-372): 1 - p for a match, p * EM for a mismatch
        s_em[q] = T(1 - p);
        s_mis[q] = T(p * 0.33333333333);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const u32 gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    // per-warp scratch: rows 0..max_q, per row W slots x (M, I) then the row's scaling factor; x32 lanes
    const u64 row_words = u64(W) * 2 + 1;
    // rpw reads per warp (lanes 0..rpw-1): 32 for the FP32 kernels; the FP64 replays of a few reads spread
    // them over more warps (their time is the FP64 latency of one read). Scratch is interleaved by rpw.
    const u32 stride = EXACT ? rpw : 32u;
    T *slot_base = scratch + u64(gwarp) * (u64(max_q) + 2) * row_words * stride + lane;
    auto FS = [&](int row, int s, int st) -> T & { return slot_base[((u64(row) * row_words) + s * 2 + st) * stride]; };
    auto SC = [&](int row) -> T & { return slot_base[((u64(row) * row_words) + W * 2) * stride]; };
    const u32 n_list = *count;
    const T EI = T(0.25);
    const double GOP = ct_gap_open;

    for (;;) {
        u32 base = 0;
        if (lane == 0) base = atomicAdd(work_ctr, EXACT ? rpw : 32u);
        base = __shfl_sync(FULL, base, 0);
        if (base >= n_list) break;
        const u32 li = base + lane;
        if ((EXACT && u32(lane) >= rpw) || li >= n_list) continue;
        const u32 r = list[li];

        // ---- setup (device/baq.cu:247-334) ----
        const u16 *win = w.win + size_t(r) * 8;
        const int qx = win[0], qy = win[1];
        const int hx = w.hmm[size_t(r) * 2], hy = w.hmm[size_t(r) * 2 + 1];
        const int bw = w.bw[r];
        int refLen = hy - hx + 1;
        const int bmLen = refLen;
        const int qL = qy - qx + 1;
        const u32 astart = b.astart[r];
        u64 ref_off;
        const u32 ahx = hx < 0 ? u32(-hx) : u32(hx);
        if (hx < 0 && astart < ahx) { ref_off = 0; refLen--; }
        else ref_off = u64(u32(astart + u32(hx)));
        const DevContig g = dref.contigs[b.chromosome[r]];
        const u64 qsym = u64(b.read_start[r]) + qx;
        const u32 qual0 = b.qual_start[r] + qx;
        auto REF = [&](int k) -> u8 { return k >= 0 ? contig_at(g, ref_off + u64(k)) : u8(0); };
        auto QRY = [&](int i) -> u8 { return sym4(b.reads, qsym + u64(i)); };
        auto QUL = [&](int i) -> u8 { return b.quals[qual0 + i]; };

        const double dsM = 1.0 / (2 * qL + 2);
        const T sM = T(dsM), sI = sM;
        const T bM = T((1 - GOP) / bmLen), bI = T(GOP / bmLen);
        const T m0 = T((1 - GOP - GOP) * (1 - dsM)), m1 = T(GOP * (1 - dsM)), m2 = m1;
        const T m3 = T((1 - 0.1) * (1 - dsM)), m4 = T(0.1 * (1 - dsM));
        const T m6 = T(1 - 0.1), m8 = T(0.1);
        bool under = false;
        // the range arguments take emissions >= 1.7e-10 (base qualities <= 93); a read with a higher quality
        // (up to 255: 0xFF marks a missing quality string) is left undecided for the exact replay
        int qmax = QUL(0);
        float kf = 0.0f;  // FL: forward flush errors (units of FLUSH_T) carried to row qL's scale
        // interior rows (every slot in the band, no cell at the reference end) take the branch-free path
        const bool full = 2 * bw + 1 == W;
        const T EIm1 = A::mul(EI, m1), EIm4 = A::mul(EI, m4);

        T M[W], I[W], D[W];
        u8 rw[W];  // reference symbol used by slot s in the current row
#pragma unroll
        for (int s = 0; s < W; s++) { M[s] = T(0); I[s] = T(0); D[s] = T(0); rw[s] = s >= 1 ? REF(s - 1) : 0; }

        // ---- forward, row 1: k = s, band [1, min(refLen, bw+1)] ----
        {
            const u8 q0 = QRY(0), qq0 = QUL(0);
            const int end = refLen < bw + 1 ? refLen : bw + 1;
            T sum = T(0);
#pragma unroll
            for (int s = 0; s < W; s++) {
                const bool inb = s >= 1 && s <= end;
                if (inb) {
                    const T e = emission<T>(s_em, s_mis, rw[s], q0, qq0);
                    M[s] = A::mul(e, bM);
                    I[s] = A::mul(EI, bI);
                    sum = A::add(sum, A::add(M[s], I[s]));
                }
            }
            SC(1) = sum;
            T inv1 = T(0);
            if constexpr (!EXACT) inv1 = FWD_SCALE / sum;
#pragma unroll
            for (int s = 0; s < W; s++) {
                if constexpr (EXACT) {
                    M[s] = A::div(M[s], sum);
                    I[s] = A::div(I[s], sum);
                } else {
                    M[s] = M[s] * inv1;
                    I[s] = I[s] * inv1;
                }
                if constexpr (FL) {
                    flush_t(M[s], kf);
                    flush_t(I[s], kf);
                }
                FS(1, s, 0) = M[s];
                FS(1, s, 1) = I[s];
                if (!FL && tiny_positive(M[s])) under = true;
            }
        }
        // ---- forward, rows 2..qL ----
        // the symbols a row needs are loaded one row ahead so their latency overlaps the previous row
        u8 nq = qL >= 2 ? QRY(1) : 0, nqq = qL >= 2 ? QUL(1) : 0;
        u8 nref = REF(W - 1 + (2 - bw > 0 ? 2 - bw : 0) - 1);
        for (int i = 2; i <= qL; i++) {
            const u8 qyi = nq, qq = nqq, top = nref;
            qmax = qmax > qq ? qmax : qq;
            if (i < qL) {
                nq = QRY(i);
                nqq = QUL(i);
                nref = REF(W - 1 + (i + 1 - bw > 0 ? i + 1 - bw : 0) - 1);
            }
            const int beg = 1 > i - bw ? 1 : i - bw;
            const int end = refLen < i + bw ? refLen : i + bw;
            const int x = i - bw > 0 ? i - bw : 0;  // slot s holds cell k = s + x
            T sum = T(0);
            float cpre = 0.0f;  // FL: flushes of the row before its scaling
            if (full && i > bw && i + bw < refLen) {
#pragma unroll
                for (int s = 0; s < W - 1; s++) rw[s] = rw[s + 1];
                rw[W - 1] = top;
                T eq, ex;
                row_emission<T>(s_em, s_mis, qyi, qq, eq, ex);
                T dprev = T(0), mprev = T(0);
#pragma unroll
                for (int s = 0; s < W; s++) {
                    const T oM = M[s], oI = I[s], oD = D[s];
                    const T nM1 = s + 1 < W ? M[s + 1] : T(0), nI1 = s + 1 < W ? I[s + 1] : T(0);
                    const T e = cell_emission<T>(rw[s], qyi, eq, ex);
                    T m = A::mul(e, A::add(A::add(A::mul(m0, oM), A::mul(m3, oI)), A::mul(m6, oD)));
                    T ii = A::mul(EI, A::add(A::mul(m1, nM1), A::mul(m4, nI1)));
                    if constexpr (FL) {
                        flush_t(m, cpre);
                        flush_t(ii, cpre);
                    }
                    T d = A::add(A::mul(m2, mprev), A::mul(m8, dprev));
                    if constexpr (FL) flush_t(d, cpre);
                    sum = A::add(sum, A::add(A::add(m, ii), d));
                    M[s] = m; I[s] = ii; D[s] = d;
                    mprev = m; dprev = d;
                }
            } else if (i > bw) {
                // the band slides one cell: slot s now holds k = s + x, whose reference base is REF(s + x - 1)
#pragma unroll
                for (int s = 0; s < W - 1; s++) rw[s] = rw[s + 1];
                rw[W - 1] = top;
                // M(i,k) reads slot s of row i-1 (cell k-1), I(i,k) reads slot s+1 (cell k): ascending in place
                T dprev = T(0), mprev = T(0);
#pragma unroll
                for (int s = 0; s < W; s++) {
                    const int k = s + x;
                    const bool inb = k >= beg && k <= end;
                    const T oM = M[s], oI = I[s], oD = D[s];
                    const T nM1 = s + 1 < W ? M[s + 1] : T(0), nI1 = s + 1 < W ? I[s + 1] : T(0);
                    T m = T(0), ii = T(0), d = T(0);
                    if (inb) {
                        const T e = emission<T>(s_em, s_mis, rw[s], qyi, qq);
                        m = A::mul(e, A::add(A::add(A::mul(m0, oM), A::mul(m3, oI)), A::mul(m6, oD)));
                        ii = A::mul(EI, A::add(A::mul(m1, nM1), A::mul(m4, nI1)));
                        if constexpr (FL) {
                            flush_t(m, cpre);
                            flush_t(ii, cpre);
                        }
                        d = A::add(A::mul(m2, mprev), A::mul(m8, dprev));
                        if constexpr (FL) flush_t(d, cpre);
                        sum = A::add(sum, A::add(A::add(m, ii), d));
                    }
                    M[s] = m; I[s] = ii; D[s] = d;
                    mprev = m; dprev = d;
                }
            } else {
                // growing band (x = 0, slot s = cell k): M(i,k) reads slot s-1, I(i,k) reads slot s
#pragma unroll
                for (int s = W - 1; s >= 0; s--) {
                    const int k = s;
                    const bool inb = k >= beg && k <= end;
                    T m = T(0), ii = T(0);
                    if (inb) {
                        const T e = emission<T>(s_em, s_mis, rw[s], qyi, qq);
                        const T pM = s >= 1 ? M[s - 1] : T(0), pI = s >= 1 ? I[s - 1] : T(0),
                                pD = s >= 1 ? D[s - 1] : T(0);
                        m = A::mul(e, A::add(A::add(A::mul(m0, pM), A::mul(m3, pI)), A::mul(m6, pD)));
                        ii = A::mul(EI, A::add(A::mul(m1, M[s]), A::mul(m4, I[s])));
                        if constexpr (FL) {
                            flush_t(m, cpre);
                            flush_t(ii, cpre);
                        }
                    }
                    M[s] = m; I[s] = ii;
                }
                T dprev = T(0), mprev = T(0);
#pragma unroll
                for (int s = 0; s < W; s++) {
                    const int k = s;
                    const bool inb = k >= beg && k <= end;
                    T d = T(0);
                    if (inb) {
                        d = A::add(A::mul(m2, mprev), A::mul(m8, dprev));
                        if constexpr (FL) flush_t(d, cpre);
                        sum = A::add(sum, A::add(A::add(M[s], I[s]), d));
                    }
                    D[s] = d;
                    mprev = M[s]; dprev = d;
                }
            }
            SC(i) = sum;
            const T inv = A::div(EXACT ? T(1) : T(FWD_SCALE), sum);
            float cpost = 0.0f;
#pragma unroll
            for (int s = 0; s < W; s++) {
                M[s] = A::mul(M[s], inv);
                I[s] = A::mul(I[s], inv);
                D[s] = A::mul(D[s], inv);
                if constexpr (FL) {
                    flush_t(M[s], cpost);
                    flush_t(I[s], cpost);
                    flush_t(D[s], cpost);
                }
                FS(i, s, 0) = M[s];
                FS(i, s, 1) = I[s];
                if (!FL && tiny_positive(M[s])) under = true;
            }
            if constexpr (FL) kf = (kf + cpre) * float(inv) + cpost;
        }
        // s[qL+1]: band cells of row qL (slots 0..2bw with k in [1, refLen])
        T sLast = T(0);
        {
            const int x = qL - bw > 0 ? qL - bw : 0;
#pragma unroll
            for (int s = 0; s < W; s++) {
                const int k = s + x;
                if (s <= 2 * bw && k >= 1 && k <= refLen) sLast = A::add(sLast, A::add(A::mul(M[s], sM), A::mul(I[s], sI)));
            }
        }
        const T sQ = SC(qL);
        // FL: forward flush errors relative to the posterior total (1.01 covers the rounding of the bound)
        float ef = 0.0f;
        if constexpr (FL) {
            ef = kf > 0.0f ? 1.01f * FLUSH_T * kf / float(sLast) : 0.0f;
            if (!(ef < 1.0f)) ef = __int_as_float(0x7f800000);
        }
        float eb = 0.0f;  // FL: backward flush errors of the rows done so far, relative to the posterior total

        // ---- backward fused with MAP ----
        // slot s of row i holds cell k = s + x(i); the reference symbol it needs is REF(k)
        T bMv[W], bIv[W], bDv[W];
        {
            const int x = qL - bw > 0 ? qL - bw : 0;
            T v;
            if constexpr (EXACT) {
                v = A::div(A::div(sM, sQ), sLast);
            } else {
                // sM / s(qL) / sLast in reference units, times 2^32: sQ carries 2^64 unless qL == 1, sLast 2^64
                v = ((sM / sQ) * (qL >= 2 ? FWD_SCALE : 1.0f) / sLast) * BWD_INIT;
            }
#pragma unroll
            for (int s = 0; s < W; s++) {
                const int k = s + x;
                const bool cell = s <= 2 * bw && k >= 1 && k <= refLen;
                bMv[s] = cell ? v : T(0);
                bIv[s] = cell ? v : T(0);
                bDv[s] = T(0);
                rw[s] = REF(k);
            }
        }
        // certified FP32 bounds (see the file comment): per-direction eps, posterior term eps_z, sums of up to
        // 2W terms, ratio excl/total and runner-up test
        const float u = 5.9604644775390625e-8f;
        const float eps = float((7.0 * qL + 2.0 * refLen + 8.0) * 5.9604644775390625e-8);
        const float eps_z = 2.0f * eps + u;
        const float rel = 2.0f * (eps_z + 2.0f * W * u) + u;
        const float rel_state = 2.0f * eps_z + 2.0f * u;
        const float dt = 4.343f * rel / (1.0f - rel) + 1e-4f;
        // the row inputs of the next backward step are loaded one step ahead
        nq = 0; nqq = 0; nref = 0;
        if (qL >= 2) {
            nq = QRY(qL - 1);
            nqq = QUL(qL - 1);
            nref = REF(qL - 1 - bw > 0 ? qL - 1 - bw : 0);
        }
        // the MAP step of row i compares with the base's own quality QUL(i - 1): for 1 < i it is nqq (loaded a
        // row ahead for the next backward step), for row 1 this value (a global load right before its use would
        // stall the row)
        const u8 q_first = QUL(0);
        // the forward scaling factor of the row below (used after that row's backward arithmetic), loaded a row
        // ahead for the same reason
        T next_scale = qL >= 2 ? SC(qL - 1) : T(1);
        for (int i = qL; i >= 1; i--) {
            const int beg = 1 > i - bw ? 1 : i - bw;
            const int end = refLen < i + bw ? refLen : i + bw;
            const int x = i - bw > 0 ? i - bw : 0;
            // forward row i (for MAP) is loaded first: the backward arithmetic of the row runs while the loads
            // are in flight. FP32: the warp's row i - 3 (contiguous, all lanes) is pulled into L2 ahead of use
            // by one bulk prefetch (the lists are ordered by query length, so a warp's lanes share rows)
            if constexpr (!EXACT) {
                const u32 am = __activemask();
                if (i > 3 && lane == __ffs(am) - 1) {
                    const T *wrow = scratch + (u64(gwarp) * (u64(max_q) + 2) + u64(i - 3)) * row_words * 32;
                    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(wrow),
                                 "r"(u32(row_words * 32 * sizeof(T)))
                                 : "memory");
                }
            }
            T fM[W], fI[W];
#pragma unroll
            for (int s = 0; s < W; s++) {
                fM[s] = FS(i, s, 0);
                fI[s] = FS(i, s, 1);
            }
            float rowflush = 0.0f;  // FL: this row's backward flush errors (its scaled units, in FLUSH_T)
            if (i < qL) {
                float cbpre = 0.0f;
                const u8 qyi1 = nq, qq1 = nqq, ref0 = nref;
                if (i > 1) {
                    nq = QRY(i - 1);
                    nqq = QUL(i - 1);
                    nref = REF(i - 1 - bw > 0 ? i - 1 - bw : 0);
                }
                const T scale_i = next_scale;
                if (i > 1) next_scale = SC(i - 1);
                const T y = (i > 1) ? T(1) : T(0);
                const bool grow = i < bw;  // row i+1 still in the growing band
                if (!grow) {
                    // x(i) = x(i+1) - 1: slots move up one cell; slot 0 takes cell x
#pragma unroll
                    for (int s = W - 1; s >= 1; s--) rw[s] = rw[s - 1];
                    rw[0] = ref0;
                }
                if (full && i > bw && i + bw < refLen) {
                    // interior row below a sliding row: every slot in band and k < refLen
                    T eq, ex;
                    row_emission<T>(s_em, s_mis, qyi1, qq1, eq, ex);
                    T dnext = T(0);
#pragma unroll
                    for (int s = W - 1; s >= 0; s--) {
                        const T bi1 = s >= 1 ? bIv[s - 1] : T(0);
                        const T e = A::mul(cell_emission<T>(rw[s], qyi1, eq, ex), bMv[s]);
                        const T bm = A::add(A::add(A::mul(e, m0), A::mul(EIm1, bi1)), A::mul(m2, dnext));
                        const T bi = A::add(A::mul(e, m3), A::mul(EIm4, bi1));
                        T bd = A::mul(A::add(A::mul(e, m6), A::mul(m8, dnext)), y);
                        if constexpr (FL) flush_t(bd, cbpre);
                        bMv[s] = bm; bIv[s] = bi; bDv[s] = bd;
                        dnext = bd;
                    }
                } else {
                // descending in place. B_M(i+1, k+1) is slot s of row i+1 (sliding) or slot s+1 (growing, carried
                // from the previous iteration); B_I(i+1, k) is slot s-1 (sliding, not yet overwritten) or slot s.
                T dnext = T(0), carryM = T(0);
#pragma unroll
                for (int s = W - 1; s >= 0; s--) {
                    const int k = s + x;
                    const bool inb = k >= beg && k <= end;
                    const T oldM = bMv[s], oldI = bIv[s];
                    const T nbm = grow ? carryM : oldM;
                    const T bi1 = grow ? oldI : (s >= 1 ? bIv[s - 1] : T(0));
                    T bm = T(0), bi = T(0), bd = T(0);
                    if (inb) {
                        T e = T(0);
                        if (k < refLen) e = A::mul(emission<T>(s_em, s_mis, rw[s], qyi1, qq1), nbm);
                        bm = A::add(A::add(A::mul(e, m0), A::mul(EIm1, bi1)), A::mul(m2, dnext));
                        bi = A::add(A::mul(e, m3), A::mul(EIm4, bi1));
                        bd = A::mul(A::add(A::mul(e, m6), A::mul(m8, dnext)), y);
                        if constexpr (FL) flush_t(bd, cbpre);
                    }
                    bMv[s] = bm; bIv[s] = bi; bDv[s] = bd;
                    dnext = bd;
                    carryM = oldM;
                }
                }
                // 1 / s(i) in reference units: SC(i) carries 2^64 for rows after the first
                const T yy = A::div(EXACT || i == 1 ? T(1) : T(FWD_SCALE), scale_i);
                // the cells of column refLen (no emission; they only feed a diagonal neighbour, scaled by their
                // own tiny value) may decay through the subnormal range: their absolute error (< 2^-149 per
                // operation) is below 1e-23 of any cell they feed and is not flagged
                const int last_ok = refLen - 1 - x;
                float cbpost = 0.0f;
#pragma unroll
                for (int s = 0; s < W; s++) {
                    bMv[s] = A::mul(bMv[s], yy);
                    bIv[s] = A::mul(bIv[s], yy);
                    bDv[s] = A::mul(bDv[s], yy);
                    if constexpr (FL) {
                        flush_t(bMv[s], cbpost);
                        flush_t(bIv[s], cbpost);
                    }
                    if (!FL && tiny_positive(bMv[s]) && s <= last_ok) under = true;
                }
                if constexpr (FL) rowflush = cbpre * float(yy) + cbpost;
            }
            // ---- MAP for row i (device/baq.cu:619-681): first maximum in (k, M before I) order ----
            T sum = T(0), mx = T(0), second = T(0), excl = T(0);
            int max_k = -1;
            if (!EXACT && full && i > bw && i + bw < refLen) {
                // the old maximum (or z itself) joins the sum of the other terms: excl += min(z, mx) and the
                // runner-up is max(second, min(z, mx)); ties keep the first maximum
                const int k0 = (x - 1) << 2;
#pragma unroll
                for (int s = 0; s < W; s++) {
#pragma unroll
                    for (int st = 0; st < 2; st++) {
                        const T z = A::mul(st == 0 ? fM[s] : fI[s], st == 0 ? bMv[s] : bIv[s]);
                        sum = A::add(sum, z);
                        const T lo = fminf(z, mx);
                        excl = A::add(excl, lo);
                        second = fmaxf(second, lo);
                        max_k = z > mx ? k0 + (s << 2) + st : max_k;
                        mx = fmaxf(z, mx);
                    }
                }
            } else {
#pragma unroll
            for (int s = 0; s < W; s++) {
                const int k = s + x;
                if (k >= beg && k <= end) {
#pragma unroll
                    for (int st = 0; st < 2; st++) {
                        const T z = A::mul(st == 0 ? fM[s] : fI[s], st == 0 ? bMv[s] : bIv[s]);
                        sum = A::add(sum, z);
                        if (z > mx) {
                            if (!EXACT) { excl = A::add(excl, mx); second = mx; }
                            mx = z;
                            max_k = (k - 1) << 2 | st;
                        } else if (!EXACT) {
                            excl = A::add(excl, z);
                            if (z > second) second = z;
                        }
                    }
                }
            }
            }
            const u32 qi = qual0 + u32(i - 1);
            if constexpr (FL) {
                // this row's backward flushes join the bound before its decisions (a row without a usable sum
                // leaves every later row undecided)
                if (rowflush > 0.0f)
                    eb = (float(sum) > 0.0f && float(sum) <= 3.0e38f)
                             ? eb + 2.02f * FLUSH_T * rowflush * FWD_SCALE / float(sum)
                             : __int_as_float(0x7f800000);
            }
            if (EXACT) {
                const double p = double(A::div(mx, sum));
                // -4.343 * log(1 - max) + .499 with no fused operation; (int) saturates like the reference's
                // CUDA build (+inf -> INT_MAX, NaN -> 0)
                const double t = __dadd_rn(__dmul_rn(-4.343, log(__dsub_rn(1.0, p))), 0.499);
                const int kq = int(t);
                w.baq_q[qi] = u8(kq > 100 ? 99 : (kq < MIN_BASE_QUAL ? MIN_BASE_QUAL : kq));
                w.baq_state[qi] = u32(max_k);
                w.baq_amb[qi] = 0;
            } else {
                const int qo = i == 1 ? q_first : nqq;
                u8 amb = 0;
                int qv = MIN_BASE_QUAL;
                u32 state = U32_NONE;
                float tq_trace = 0.0f, lo_trace = 0.0f, hi_trace = 0.0f;  // (precision trace only)
                if (!(sum > T(0)) || !(sum <= T(3.0e38f)) || max_k < 0) {
                    amb = 7;
                } else {
                    state = u32(max_k);
                    float abs_err = 0.0f;  // FL: absolute error of the posterior terms, in the row's units
                    if constexpr (FL) {
                        abs_err = (ef + eb) * float(sum) + 2.0f * W * __int_as_float(4);
                        if (!(abs_err < 3.0e38f)) abs_err = __int_as_float(0x7f800000);
                    }
                    const float thr = float(mx) * (1.0f - rel_state) - 2.0f * abs_err;
                    if (float(second) >= thr) {
                        // undecided state: the rivals are the other cells whose term is within the bound of the
                        // maximum; with exactly one, the capping step can still decide when neither state is the
                        // match at the base's expected position
                        amb |= 2;
                        int rivals = 0;
                        u32 alt = 0;
#pragma unroll
                        for (int s = 0; s < W; s++) {
                            const int k = s + x;
                            if (k >= beg && k <= end) {
#pragma unroll
                                for (int st = 0; st < 2; st++) {
                                    const T z = A::mul(st == 0 ? fM[s] : fI[s], st == 0 ? bMv[s] : bIv[s]);
                                    const u32 idx = u32((k - 1) << 2 | st);
                                    if (idx != state && float(z) >= thr) {
                                        if (!rivals) alt = idx;
                                        rivals++;
                                    }
                                }
                            }
                        }
                        if (rivals == 1) w.baq_alt[qi] = u16(alt);
                        else amb |= 4;
                    }
                    const float ratio = float(excl) / float(sum);
                    const float tq = ratio > 0.f ? -4.343f * logf(ratio) + 0.499f : __int_as_float(0x7f800000);
                    float lo = tq - dt, hi = tq + dt;
                    if (FL && abs_err > 0.0f) {
                        // the other terms' sum moves by at most abs_err: t by 4.343 ln(1 + abs_err / excl)
                        const float extra = float(excl) > 0.0f ? abs_err / float(excl) : __int_as_float(0x7f800000);
                        if (extra < 0.25f) {
                            const float dta = 4.343f * extra / (1.0f - extra);
                            lo -= dta;
                            hi += dta;
                        } else {
                            const float rhi = (float(excl) * (1.0f + rel) + abs_err) / (float(sum) * (1.0f - rel));
                            lo = -4.343f * logf(rhi) + 0.499f - 1e-4f;
                            hi = __int_as_float(0x7f800000);
                        }
                    }
                    auto capped = [&](float tt) {
                        int k;
                        if (!(tt == tt)) k = 0;
                        else if (tt >= 2147483520.0f) k = 2147483647;
                        else k = int(floorf(tt));
                        return k > 100 ? 99 : (k < MIN_BASE_QUAL ? MIN_BASE_QUAL : k);
                    };
                    qv = capped(tq);
                    tq_trace = tq;
                    lo_trace = lo;
                    hi_trace = hi;
                    const int flo = capped(lo), fhi = capped(hi);
                    if (qo <= 99) {
                        if ((flo < qo ? flo : qo) != (fhi < qo ? fhi : qo)) amb |= 1;
                        // whether min(capped, qo) == qo, i.e. capped >= qo: monotone in t for qo <= 99
                        if ((flo >= qo) != (fhi >= qo)) amb |= 16;
                    } else if (!(hi < 100.f && flo == fhi) && !(lo >= 101.5f)) {
                        amb |= 1 | 16;
                    }
                    // bit 8: undecided state, every candidate's MAP quality MIN_BASE_QUAL (t < 5 for all)
                    if ((amb & 2) && hi < 4.9f) amb |= 8;
                }
                w.baq_q[qi] = u8(qv);
                w.baq_state[qi] = state;
                w.baq_amb[qi] = amb;
                if (w.trace32) {
                    const float nan = __int_as_float(0x7fc00000);
                    w.trace32[3 * size_t(qi)] = amb == 7 ? nan : tq_trace;
                    w.trace32[3 * size_t(qi) + 1] = lo_trace;
                    w.trace32[3 * size_t(qi) + 2] = hi_trace;
                }
            }
        }
        if (!EXACT && (under || qmax > 93)) {
            for (int i = 0; i < qL; i++) w.baq_amb[qual0 + i] = 7;
            if (w.trace32)
                for (int i = 0; i < qL; i++) w.trace32[3 * size_t(qual0 + i)] = __int_as_float(0x7fc00000);
        }
    }
}

template <typename T, int W, bool EXACT>
void launch_one(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                u32 max_reads, u32 *ctr, T *scratch, u64 scratch_elems, u32 max_q, u32 rpw, cudaStream_t s) {
    const u32 stride = EXACT ? rpw : 32u;
    const u64 per_warp = (u64(max_q) + 2) * (u64(W) * 2 + 1) * stride;
    u64 warps = scratch_elems / per_warp;
    u64 blocks = warps / (TPR_THREADS / 32);
    const u64 reads_per_block = u64(TPR_THREADS / 32) * (EXACT ? rpw : 32u);
    const u64 need = (u64(max_reads) + reads_per_block - 1) / reads_per_block;
    if (blocks > need) blocks = need;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks == 0) return;
    cudaMemsetAsync(ctr, 0, sizeof(u32), s);
    k_baq_tpr<T, W, EXACT><<<u32(blocks), TPR_THREADS, 0, s>>>(b, ref, w, list, count, ctr, scratch, max_q, rpw);
    g_kernel_launches++;
}

}  // namespace

void baq_tpr_set_constants(const HmmConst &c) {
    cudaMemcpyToSymbol(ct_qual2prob, c.qual2prob, sizeof(c.qual2prob));
    cudaMemcpyToSymbol(ct_gap_open, &c.gap_open, sizeof(double));
}

u64 baq_tpr_scratch_bytes(int band_class, bool exact, u32 max_q) {
    const int W = band_class == 0 ? 15 : 31;
    const u64 per_warp = (u64(max_q) + 2) * (u64(W) * 2 + 1) * 32 * (exact ? 8 : 4);
    return per_warp * (152 * 8) * (TPR_THREADS / 32);
}

void launch_baq_tpr(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                    u32 max_reads, int band_class, bool exact, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q,
                    u32 rpw, cudaStream_t s) {
    if (!max_reads) return;
    if (exact) {
        if (band_class == 0)
            launch_one<double, 15, true>(b, ref, w, list, count, max_reads, ctr, (double *)scratch, scratch_bytes / 8, max_q, rpw, s);
        else
            launch_one<double, 31, true>(b, ref, w, list, count, max_reads, ctr, (double *)scratch, scratch_bytes / 8, max_q, rpw, s);
    } else {
        if (band_class == 0)
            launch_one<float, 15, false>(b, ref, w, list, count, max_reads, ctr, (float *)scratch, scratch_bytes / 4, max_q, 32u, s);
        else
            launch_one<float, 31, false>(b, ref, w, list, count, max_reads, ctr, (float *)scratch, scratch_bytes / 4, max_q, 32u, s);
    }
}

}  // namespace fpg
