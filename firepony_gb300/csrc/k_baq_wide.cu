// K2 for bands wider than 15 (bw <= 31): the banded glocal BAQ HMM (device/baq.cu:214-697) in FP32 with the
// certified decisions of k_baq_tpr.cu, the band spread over a group of G lanes as in k_baq_exact.cu (G lanes x
// NS slots, WC = G*NS >= 2*bw+1; 32/G reads per warp). A thread-per-read kernel cannot hold a band this wide in
// registers, and the exact FP64 kernel costs ~64 cycles per FP64 warp instruction on this GPU.
//
// Every M and I cell takes the operations of k_baq_tpr<float> (the same products and sums in the same
// grouping). The D recurrence along a row, D(k) = c(k) + m8 * D(k-1), is a linear scan: D(k) =
// sum_n m8^n c(k-n), computed per segment of G slots in log2(G) shuffle steps over the group's lanes plus a
// carry from the segment below, instead of a serial chain on one lane. A path's D run within a row then takes
// a fixed number of roundings (2 to enter, 2 per scan level, 2 per carry) instead of 2 per D step, so forward
// and backward values carry eps <= (7 qL + D_RUN min(qL, refLen) + 8) 2^-24 (at most one D run per row), a
// posterior term eps_z = 2 eps + 2^-24, a sum of at most 2 WC terms adds 2 WC 2^-24 (in any order: the row
// and posterior sums here are lane partial sums combined by shuffles), and the decisions (MAP quality within
// dt of a rounding boundary, runner-up state within the bound) are taken as in k_baq_tpr<float>. The forward
// row sums only set the row scaling, a common factor that cancels in every posterior ratio.
//
// Cells far from the alignment decay by many orders of magnitude across a wide band. Instead of giving up on
// a read with such a cell, a computed cell value below FLUSH is replaced by zero. Every operand of the
// recurrences is then zero or at least FLUSH; the smallest factors are a mismatch emission (1.7e-10), the
// gap-open transition (>= 7.5e-5) and 0.1, so every product and sum of kept values stays at or above
// FLUSH * 2^-34 > 2^-126 and the relative error analysis above holds for them. Each flushed value carries an
// absolute error below FLUSH, whose effect on the posterior terms is bounded separately (backward values are
// at most 1 and forward values at most the row sum in the scaled units; see the error terms below) and added
// to the decision margins as an absolute error. Posterior products of kept values may still underflow: each
// adds at most 2^-150. In the D scans a partial sum times a high power of m8 may fall below the normal range;
// it enters a fused add, and a kept D value (at least FLUSH) then carries at most 2^-150 per scan step from
// it, below 2^-70 of the value, inside the 8 spare roundings of eps.
//
// Slot s of row i holds cell k = s + x(i), x(i) = max(i - bw, 0); rows are exchanged through per-group shared
// buffers indexed by slot + 1 with zero sentinels. A group whose read has a band wider than WC takes no read
// (the thread-per-read FP64 kernel computes those). Per group scratch (global): rows 0..max_q+1 of 2*WC+1
// floats: forward M (WC), forward I (WC) and the row sum before scaling.
#include "kernels.h"

namespace fpg {

__constant__ double cw_qual2prob[256];
__constant__ double cw_gap_open;

namespace {

constexpr u32 FULL = 0xffffffffu;
constexpr int WD_THREADS = 128;
// Forward rows sum to 2^110 and backward values carry 2^-14 (their posterior products 2^96): a row's
// unscaled sum stays below 1.25 * 2^110, and a forward cell is flushed only below 2^-188 of its row, so the
// forward flush bound (which grows by 1/s(i) per row) stays small even for reads whose rows drop sharply
constexpr float FWD_SCALE = 1298074214633706907132624082305024.0f;  // 2^110
constexpr float BWD_INIT = 79228162514264337593543950336.0f;         // 2^96 = 2^110 (sLast) x 2^-14

constexpr float FLUSH = 3.3087224502121107e-24f;  // 2^-78

// v < FLUSH -> 0, counting the values that were not zero already
__device__ __forceinline__ void flush(float &v, float &c) {
    if (v < FLUSH) {
        c += v > 0.0f ? 1.0f : 0.0f;
        v = 0.0f;
    }
}

// sums / maxima over the G lanes of a group (every lane gets the result; every lane of the warp must call them)
template <int G> __device__ __forceinline__ float gsum(float v) {
#pragma unroll
    for (int o = G / 2; o >= 1; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}
template <int G> __device__ __forceinline__ float gmax(float v) {
#pragma unroll
    for (int o = G / 2; o >= 1; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
template <int G> __device__ __forceinline__ u32 gsumu(u32 v) {
#pragma unroll
    for (int o = G / 2; o >= 1; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}
template <int G> __device__ __forceinline__ u32 gminu(u32 v) {
#pragma unroll
    for (int o = G / 2; o >= 1; o >>= 1) v = min(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

// MAP quality bounds as in k_baq_tpr: the capped quality of t, saturating like the reference's CUDA build
__device__ __forceinline__ int capped_q(float tt) {
    int k;
    if (!(tt == tt)) k = 0;
    else if (tt >= 2147483520.0f) k = 2147483647;
    else k = int(floorf(tt));
    return k > 100 ? 99 : (k < MIN_BASE_QUAL ? MIN_BASE_QUAL : k);
}

template <int G, int NS>
__global__ void __launch_bounds__(WD_THREADS) k_baq_wide(DevBatch b, DevRef dref, BatchWork w, const u32 *list,
                                                         const u32 *count, u32 *work_ctr, float *scratch,
                                                         u32 max_q, int min_bw) {
    constexpr int WC = G * NS;          // band slots per read
    constexpr int GPW = 32 / G;         // reads (groups) per warp
    constexpr int WPB = WD_THREADS / 32;
    constexpr int ROWF = 2 * WC + 1;    // scratch floats per row
    constexpr int XB = 2 * WC + 2;      // exchange buffer length
    constexpr int LOG2G = G == 32 ? 5 : (G == 16 ? 4 : (G == 8 ? 3 : (G == 4 ? 2 : 1)));
    static_assert((1 << LOG2G) == G, "G is a power of two");
    __shared__ float s_em[256], s_mis[256];
    // per group: forward previous row (M, I, D), backward next row (M, I), three exchange buffers
    __shared__ float s_buf[WPB][GPW][8][XB];
    for (int q = threadIdx.x; q < 256; q += blockDim.x) {
        const double p = cw_qual2prob[q < MIN_BASE_QUAL ? MIN_BASE_QUAL : q];
        // calcEpsilon (device/baq.cu:361-372): 1 - p for a match, p * EM for a mismatch
        s_em[q] = float(1 - p);
        s_mis[q] = float(p * 0.33333333333);
    }
    for (int i = threadIdx.x; i < WPB * GPW * 8 * XB; i += blockDim.x) (&s_buf[0][0][0][0])[i] = 0.0f;
    __syncthreads();

    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int g = lane / G, l = lane % G;
    // powers of m8 = 0.1 for the D scans, each rounded once to float from a double product (relative error
    // of the double below 2^-48): m8^(2^lv) per scan level, m8^(l+1) and m8^(G-l) for the segment carries
    float m8p[LOG2G], m8up, m8dn;
    {
        double p = 1.0, pu = 0.0, pd = 0.0;
#pragma unroll
        for (int n = 1; n <= G; n++) {
            p *= 0.1;
            for (int lv = 0; lv < LOG2G; lv++)
                if (n == (1 << lv)) m8p[lv] = float(p);
            if (n == l + 1) pu = p;
            if (n == G - l) pd = p;
        }
        m8up = float(pu);
        m8dn = float(pd);
    }
    float *PM = s_buf[wib][g][0], *PI = s_buf[wib][g][1], *PD = s_buf[wib][g][2];
    float *QM = s_buf[wib][g][3], *QI = s_buf[wib][g][4];
    float *X0 = s_buf[wib][g][5], *X1 = s_buf[wib][g][6];
    const u32 gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    float *gs = scratch + (u64(gwarp) * GPW + g) * (u64(max_q) + 2) * ROWF;
    auto FROW = [&](int row) -> float * { return gs + u64(row) * ROWF; };
    const u32 n_list = *count;
    const float EI = 0.25f;
    const double GOP = cw_gap_open;

    for (;;) {
        u32 base = 0;
        if (lane == 0) base = atomicAdd(work_ctr, u32(GPW));
        base = __shfl_sync(FULL, base, 0);
        if (base >= n_list) break;
        const u32 li = base + g;
        bool has = li < n_list;
        const u32 r = has ? list[li] : 0;
        if (has && 2 * int(w.bw[r]) + 1 > WC) has = false;  // left to the thread-per-read FP64 kernel
        if (has && int(w.bw[r]) < min_bw) has = false;       // a narrower kernel of the same class takes it

        // ---- setup (device/baq.cu:247-334), identical for the lanes of a group ----
        int qL = 0, refLen = 0, bmLen = 1, bw = 0;
        u64 ref_off = 0;
        u32 qsym = 0, qual0 = 0, contig = 0;
        if (has) {
            const u16 *win = w.win + size_t(r) * 8;
            const int qx = win[0], qy = win[1];
            const int hx = w.hmm[size_t(r) * 2], hy = w.hmm[size_t(r) * 2 + 1];
            bw = w.bw[r];
            refLen = hy - hx + 1;
            bmLen = refLen;
            qL = qy - qx + 1;
            const u32 astart = b.astart[r];
            const u32 ahx = hx < 0 ? u32(-hx) : u32(hx);
            if (hx < 0 && astart < ahx) { ref_off = 0; refLen--; }
            else ref_off = u64(u32(astart + u32(hx)));
            contig = b.chromosome[r];
            qsym = b.read_start[r] + u32(qx);
            qual0 = b.qual_start[r] + u32(qx);
        }
        const DevContig gc = has ? dref.contigs[contig] : DevContig{nullptr, 0};
        auto REF = [&](int k) -> u8 { return (has && k >= 0) ? contig_at(gc, ref_off + u64(k)) : u8(0); };
        auto QRY = [&](int i) -> u8 { return sym4(b.reads, u64(qsym) + u64(i)); };
        auto QUL = [&](int i) -> u8 { return b.quals[qual0 + u32(i)]; };
        auto EMI = [&](u8 ref, u8 rd, u8 q) -> float {
            if (ref == IUPAC_N || rd == IUPAC_N) return 1.0f;
            return ref == rd ? s_em[q] : s_mis[q];
        };
        const int Qmax = int(__reduce_max_sync(FULL, u32(qL)));

        // the constants of k_baq_tpr<float> (device/baq.cu:247-334 in double, rounded once)
        const double dsM = 1.0 / (2 * (qL > 0 ? qL : 1) + 2);
        const float sM = float(dsM), sI = sM;
        const float bM = float((1 - GOP) / bmLen), bI = float(GOP / bmLen);
        const float m0 = float((1 - GOP - GOP) * (1 - dsM)), m1 = float(GOP * (1 - dsM)), m2 = m1;
        const float m3 = float((1 - 0.1) * (1 - dsM)), m4 = float(0.1 * (1 - dsM));
        const float m6 = float(1 - 0.1), m8 = float(0.1);
        (void)m8;
        const float EIm1 = EI * m1, EIm4 = EI * m4;
        // forward flush errors in units of FLUSH, carried to row qL's scale: K = (K + before-scaling flushes)
        // * inv + after-scaling flushes, row by row (each lane its own flushes; the terms add up)
        float kf = 0.0f;
        // the range arguments take emissions >= 1.7e-10 (base qualities <= 93); a read with a higher quality
        // (up to 255: 0xFF marks a missing quality string) is left undecided for the exact replay
        int qmax = 0;

        // ---- forward, row 1: slot s = cell k, band [1, min(refLen, bw + 1)] ----
        float fM[NS], fI[NS], fD[NS];
        {
            const int end = refLen < bw + 1 ? refLen : bw + 1;
            const bool act = qL >= 1;
            const u8 q0 = act ? QRY(0) : 0, qq0 = act ? QUL(0) : 0;
            qmax = qq0;
            float part = 0.0f;
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G;
                const bool inb = act && s >= 1 && s <= end;
                fM[j] = inb ? EMI(REF(s - 1), q0, qq0) * bM : 0.0f;
                fI[j] = inb ? EI * bI : 0.0f;
                fD[j] = 0.0f;
                part += inb ? fM[j] + fI[j] : 0.0f;
            }
            const float sum = gsum<G>(part);
            const float inv1 = act ? FWD_SCALE / sum : 0.0f;
            if (act && l == 0) FROW(1)[2 * WC] = sum;
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G;
                fM[j] *= inv1;
                fI[j] *= inv1;
                float c = 0.0f;
                flush(fM[j], c);
                flush(fI[j], c);
                if (act) kf += c;
                if (act) {
                    FROW(1)[s] = fM[j];
                    FROW(1)[WC + s] = fI[j];
                }
                PM[s + 1] = fM[j];
                PI[s + 1] = fI[j];
                PD[s + 1] = 0.0f;
            }
            __syncwarp();
        }

        // ---- forward, rows 2..qL ----
        for (int i = 2; i <= Qmax; i++) {
            const bool act = i <= qL;
            const int beg = 1 > i - bw ? 1 : i - bw;
            const int end = refLen < i + bw ? refLen : i + bw;
            const int x = i - bw > 0 ? i - bw : 0;
            const bool slide = i > bw;
            const u8 qy = act ? QRY(i - 1) : 0, qq = act ? QUL(i - 1) : 0;
            qmax = qmax > qq ? qmax : qq;
            // M and I of every slot from the previous row; m2 * M feeds the D chain of the next slot
            float mI[NS];
            float cpre = 0.0f;  // this lane's flushes of the row before its scaling
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G, k = s + x;
                const bool inb = act && k >= beg && k <= end;
                const float oM = slide ? PM[s + 1] : PM[s], oI = slide ? PI[s + 1] : PI[s];
                const float oD = slide ? PD[s + 1] : PD[s];
                const float nM1 = slide ? PM[s + 2] : PM[s + 1], nI1 = slide ? PI[s + 2] : PI[s + 1];
                float m = 0.0f, ii = 0.0f;
                if (inb) {
                    const float e = EMI(REF(k - 1), qy, qq);
                    m = e * ((m0 * oM + m3 * oI) + m6 * oD);
                    ii = EI * (m1 * nM1 + m4 * nI1);
                    flush(m, cpre);
                    flush(ii, cpre);
                }
                fM[j] = m;
                fI[j] = ii;
                mI[j] = m + ii;
                X0[s + 1] = m2 * m;
            }
            __syncwarp();
            // D(k) = m2 * M(k-1) + m8 * D(k-1) along the row, as D(k) = sum_n m8^n * m2 * M(k-1-n): per segment
            // of G slots a scan over the group's lanes, then the carry m8^(l+1) * D(top slot of the segment
            // below). Zero below the band; values past it are discarded (only in-band flushes count)
            {
                float carry = 0.0f;
#pragma unroll
                for (int j = 0; j < NS; j++) {
                    const int s = l + j * G, k = s + x;
                    float d = s == 0 ? 0.0f : X0[s];
#pragma unroll
                    for (int lv = 0; lv < LOG2G; lv++) {
                        const float up = __shfl_up_sync(FULL, d, 1 << lv, G);
                        if (l >= (1 << lv)) d = fmaf(m8p[lv], up, d);
                    }
                    if (j > 0) d = fmaf(m8up, carry, d);
                    if (act && k >= beg && k <= end) flush(d, cpre);
                    else if (d < FLUSH) d = 0.0f;
                    X1[s] = d;
                    carry = __shfl_sync(FULL, d, G - 1, G);
                }
            }
            __syncwarp();
            float part = 0.0f;
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G, k = s + x;
                const bool inb = act && k >= beg && k <= end;
                fD[j] = inb ? X1[s] : 0.0f;
                part += inb ? mI[j] + fD[j] : 0.0f;
            }
            const float sum = gsum<G>(part);
            const float inv = act ? FWD_SCALE / sum : 0.0f;
            if (act && l == 0) FROW(i)[2 * WC] = sum;
            __syncwarp();  // every lane has read the previous row before it is replaced
            float cpost = 0.0f;
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G;
                fM[j] *= inv;
                fI[j] *= inv;
                fD[j] *= inv;
                flush(fM[j], cpost);
                flush(fI[j], cpost);
                flush(fD[j], cpost);
                PM[s + 1] = fM[j];
                PI[s + 1] = fI[j];
                PD[s + 1] = fD[j];
                if (act) {
                    FROW(i)[s] = fM[j];
                    FROW(i)[WC + s] = fI[j];
                }
            }
            if (act) kf = (kf + cpre) * inv + cpost;
            __syncwarp();
        }

        // ---- s[qL+1] and the backward start (device/baq.cu:520-545), as k_baq_tpr<float> ----
        float bMv[NS], bIv[NS];
        float ef = 0.0f;  // forward flush error bound relative to the posterior total
        {
            const int x = qL - bw > 0 ? qL - bw : 0;
            bool cell[NS];
            float part = 0.0f;
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G, k = s + x;
                cell[j] = qL >= 1 && s <= 2 * bw && k >= 1 && k <= refLen;
                // fM / fI still hold row qL (scaled) for groups whose read has qL == Qmax; the others reload it
                const float lm = qL >= 1 ? FROW(qL)[s] : 0.0f, lI = qL >= 1 ? FROW(qL)[WC + s] : 0.0f;
                part += cell[j] ? lm * sM + lI * sI : 0.0f;
            }
            const float sLast = gsum<G>(part);
            // forward flushes, relative to the posterior total: an error e (row j's scaled units) reaches every
            // posterior sum through backward values <= 1 (reference units), i.e. at most e * prod(inv of the
            // rows after j) / sLast of the total; 1.01 covers the rounding of the bound itself
            const float kf_all = gsum<G>(kf);
            // (a bound below the normal range is kept at 2^-125, above any value that rounds there)
            ef = kf_all > 0.0f ? fmaxf(1.01f * FLUSH * kf_all / sLast, 2.350988701644575e-38f) : 0.0f;
            if (!(ef < 1.0f)) ef = __int_as_float(0x7f800000);
            const float sQ = qL >= 1 ? FROW(qL)[2 * WC] : 1.0f;
            // sM / s(qL) / sLast in reference units, times 2^-14: sQ carries 2^110 unless qL == 1, sLast 2^110
            // (grouped so that no intermediate leaves the normal range)
            const float v = ((sM * (qL >= 2 ? FWD_SCALE : 1.0f)) / sQ) * (BWD_INIT / sLast);
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G;
                bMv[j] = cell[j] ? v : 0.0f;
                bIv[j] = cell[j] ? v : 0.0f;
                QM[s + 1] = bMv[j];
                QI[s + 1] = bIv[j];
            }
            __syncwarp();
        }
        // certified FP32 bounds of k_baq_tpr (2 WC terms at most per posterior sum)
        const float u = 5.9604644775390625e-8f;
        // a path's D run within a row (at most one per row, so at most min(qL, refLen) runs) takes 2 roundings
        // to enter (m2 and its product), 2 per scan level (an m8 power and the fused add) and 2 per segment
        // carry, whatever its length
        constexpr int D_RUN = 2 + 2 * LOG2G + 2 * (NS - 1);
        const float eps = float((7.0 * qL + double(D_RUN) * (qL < refLen ? qL : refLen) + 8.0) * 5.9604644775390625e-8);
        const float eps_z = 2.0f * eps + u;
        const float rel = 2.0f * (eps_z + 2.0f * WC * u) + u;
        const float rel_state = 2.0f * eps_z + 2.0f * u;
        const float dt = 4.343f * rel / (1.0f - rel) + 1e-4f;
        // backward flushes, relative to the posterior total, over the rows done so far (qL down to i): an error
        // e in a backward value of row i' reaches every posterior sum through that cell's forward value, at
        // most the forward row sum 2^110, i.e. at most e * 2^110 / (row i' posterior sum) of the total
        float eb = 0.0f;

        // ---- backward fused with MAP, rows qL..1 of every group (t steps back from its own last row) ----
        for (int t = 0; t < Qmax; t++) {
            const int i = qL - t;
            const bool act = i >= 1;
            float rowflush = 0.0f;  // this lane's backward flush errors of row i (its scaled units, in FLUSH)
            const int beg = 1 > i - bw ? 1 : i - bw;
            const int end = refLen < i + bw ? refLen : i + bw;
            const int x = i - bw > 0 ? i - bw : 0;
            if (t > 0) {
                const bool grow = i < bw;  // row i+1 still in the growing band
                const bool y = i > 1;
                const u8 qy1 = act ? QRY(i) : 0, qq1 = act ? QUL(i) : 0;
                float a1[NS];
                float cbpre = 0.0f;  // this lane's flushes of the row before its scaling
#pragma unroll
                for (int j = 0; j < NS; j++) {
                    const int s = l + j * G, k = s + x;
                    const bool inb = act && k >= beg && k <= end;
                    // B_M(i+1, k+1): slot s+1 (growing) or s (sliding); B_I(i+1, k): slot s or s-1
                    const float nbm = grow ? QM[s + 2] : QM[s + 1];
                    const float bi1 = grow ? QI[s + 1] : QI[s];
                    float e = 0.0f;
                    if (inb && k < refLen) e = EMI(REF(k), qy1, qq1) * nbm;
                    a1[j] = e * m0 + EIm1 * bi1;
                    bIv[j] = inb ? e * m3 + EIm4 * bi1 : 0.0f;
                    X0[s] = inb ? e * m6 : 0.0f;
                }
                __syncwarp();
                // B_D(k) = (e * m6 + m8 * B_D(k+1)) * y, descending along the row: per segment a scan over the
                // group's lanes, then the carry m8^(G-l) * B_D(bottom slot of the segment above)
                {
                    float carry = 0.0f;
#pragma unroll
                    for (int j = NS - 1; j >= 0; j--) {
                        const int s = l + j * G, k = s + x;
                        float d = X0[s];
#pragma unroll
                        for (int lv = 0; lv < LOG2G; lv++) {
                            const float dn = __shfl_down_sync(FULL, d, 1 << lv, G);
                            if (l + (1 << lv) < G) d = fmaf(m8p[lv], dn, d);
                        }
                        if (j < NS - 1) d = fmaf(m8dn, carry, d);
                        if (!y) d = 0.0f;
                        if (act && k >= beg && k <= end) flush(d, cbpre);
                        else if (d < FLUSH) d = 0.0f;
                        X1[s] = d;
                        carry = __shfl_sync(FULL, d, 0, G);
                    }
                    if (l == 0) X1[WC] = 0.0f;  // (above the top slot)
                }
                __syncwarp();
                // 1 / s(i) in reference units: s(i) carries 2^110 for rows after the first
                const float yy = act ? (i == 1 ? 1.0f : FWD_SCALE) / FROW(i)[2 * WC] : 0.0f;
                float cbpost = 0.0f;
#pragma unroll
                for (int j = 0; j < NS; j++) {
                    const int s = l + j * G, k = s + x;
                    const bool inb = act && k >= beg && k <= end;
                    const float bm = inb ? a1[j] + m2 * X1[s + 1] : 0.0f;
                    bMv[j] = bm * yy;
                    bIv[j] = bIv[j] * yy;
                    flush(bMv[j], cbpost);
                    flush(bIv[j], cbpost);
                }
                rowflush = act ? cbpre * yy + cbpost : 0.0f;
                __syncwarp();
#pragma unroll
                for (int j = 0; j < NS; j++) {
                    const int s = l + j * G;
                    QM[s + 1] = bMv[j];
                    QI[s + 1] = bIv[j];
                }
            }
            // ---- MAP for row i (device/baq.cu:619-681) with the certified decisions of k_baq_tpr<float> ----
            // (the flush errors of this row's backward values join the bound once the row's sum is known)
            // posterior terms of the in-band cells; the first maximum in (k, M before I) order: non-negative
            // floats order like their bit patterns, ties keep the smaller index
            float z[2 * NS];
            u32 bbits = 0, bidx = 0xFFFFFFFFu;
            float part = 0.0f;
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G, k = s + x;
                const bool inb = act && k >= beg && k <= end;
                z[2 * j] = inb ? FROW(i)[s] * bMv[j] : 0.0f;
                z[2 * j + 1] = inb ? FROW(i)[WC + s] * bIv[j] : 0.0f;
#pragma unroll
                for (int st = 0; st < 2; st++) {
                    const u32 zb = __float_as_uint(z[2 * j + st]), idx = u32(((k - 1) << 2) | st);
                    part += z[2 * j + st];
                    if (inb && (zb > bbits || (zb == bbits && idx < bidx))) { bbits = zb; bidx = idx; }
                }
            }
#pragma unroll
            for (int o = G / 2; o >= 1; o >>= 1) {
                const u32 ob = __shfl_xor_sync(FULL, bbits, o), oi = __shfl_xor_sync(FULL, bidx, o);
                if (ob > bbits || (ob == bbits && oi < bidx)) { bbits = ob; bidx = oi; }
            }
            const float sum = gsum<G>(part), mx = __uint_as_float(bbits);
            // the sum of the other terms and the runner-up (every term but the first maximum)
            float ex = 0.0f, sec = 0.0f;
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int k = l + j * G + x;
#pragma unroll
                for (int st = 0; st < 2; st++) {
                    const u32 idx = u32(((k - 1) << 2) | st);
                    const float zz = idx == bidx ? 0.0f : z[2 * j + st];
                    ex += zz;
                    sec = fmaxf(sec, zz);
                }
            }
            const float excl = gsum<G>(ex), second = gmax<G>(sec);
            const bool valid = sum > 0.0f && sum <= 3.0e38f && bbits != 0;
            // absolute error of the posterior terms, relative to the row's exact total (the computed sum is
            // within a factor 2 of it): forward flushes, backward flushes of rows qL..i, and underflowed products
            const float rf = gsum<G>(rowflush);
            // (a row without a usable sum leaves every later row undecided)
            if (rf > 0.0f) eb = valid ? eb + 2.02f * FLUSH * rf * FWD_SCALE / sum : __int_as_float(0x7f800000);
            // underflowed products: at most 2^-150 each, 2 WC terms (2^-148 per term, in the row's units)
            const float ez = 2.0f * WC * __int_as_float(4);
            float abs_err = (ef + eb) * sum + ez;  // in the row's units
            if (!(abs_err < 3.0e38f)) abs_err = __int_as_float(0x7f800000);
            const float thr = mx * (1.0f - rel_state) - 2.0f * abs_err;
            // an undecided state records its rival when there is exactly one
            u32 rivals = 0, alt = 0xFFFFFFFFu;
            // (a warp-wide vote: the group sums below are full-warp shuffles, so every lane must take this branch
            // when any group does; a group without a rival counts none)
            if (__any_sync(FULL, act && valid && second >= thr)) {
                u32 c = 0, a = 0xFFFFFFFFu;
#pragma unroll
                for (int j = 0; j < NS; j++) {
                    const int s = l + j * G, k = s + x;
                    const bool inb = act && k >= beg && k <= end;
#pragma unroll
                    for (int st = 0; st < 2; st++) {
                        const u32 idx = u32(((k - 1) << 2) | st);
                        if (inb && idx != bidx && z[2 * j + st] >= thr) {
                            c++;
                            a = min(a, idx);
                        }
                    }
                }
                rivals = gsumu<G>(c);
                alt = gminu<G>(a);
            }
            if (act && l == 0) {
                const u32 qi = qual0 + u32(i - 1);
                const int qo = QUL(i - 1);
                u8 amb = 0;
                int qv = MIN_BASE_QUAL;
                u32 state = U32_NONE;
                float tq_trace = __int_as_float(0x7fc00000), lo_trace = 0.0f, hi_trace = 0.0f;  // (trace only)
                if (!valid) {
                    amb = 7;
                } else {
                    state = bidx;
                    if (second >= thr) {
                        amb |= 2;
                        if (rivals == 1) w.baq_alt[qi] = u16(alt);
                        else amb |= 4;
                    }
                    const float ratio = excl / sum;
                    const float tq = ratio > 0.f ? -4.343f * logf(ratio) + 0.499f : __int_as_float(0x7f800000);
                    float lo = tq - dt, hi = tq + dt;
                    // the absolute error moves the other terms' sum by at most abs_err: t by at most
                    // 4.343 * ln(1 + abs_err / excl); when that is large, only the lower bound of t is kept
                    const float extra = abs_err > 0.0f ? (excl > 0.0f ? abs_err / excl : __int_as_float(0x7f800000)) : 0.0f;
                    if (extra > 0.0f) {
                        if (extra < 0.25f) {
                            const float dta = 4.343f * extra / (1.0f - extra);
                            lo -= dta;
                            hi += dta;
                        } else {
                            const float rhi = (excl * (1.0f + rel) + abs_err) / (sum * (1.0f - rel));
                            lo = -4.343f * logf(rhi) + 0.499f - 1e-4f;
                            hi = __int_as_float(0x7f800000);
                        }
                    }
                    qv = capped_q(tq);
                    tq_trace = tq;
                    lo_trace = lo;
                    hi_trace = hi;
                    const int flo = capped_q(lo), fhi = capped_q(hi);
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
                    w.trace32[3 * size_t(qi)] = tq_trace;
                    w.trace32[3 * size_t(qi) + 1] = lo_trace;
                    w.trace32[3 * size_t(qi) + 2] = hi_trace;
                }
            }
        }
        if (has && qmax > 93) {
            for (int row = l; row < qL; row += G) w.baq_amb[qual0 + u32(row)] = 7;
            if (w.trace32)
                for (int row = l; row < qL; row += G) w.trace32[3 * size_t(qual0 + u32(row))] = __int_as_float(0x7fc00000);
        }
        __syncwarp();
    }
}

template <int G, int NS>
void launch_w(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
              u32 max_reads, u32 *ctr, float *scratch, u64 scratch_elems, u32 max_q, cudaStream_t s, int min_bw = 0) {
    constexpr int WC = G * NS, GPW = 32 / G;
    const u64 per_group = (u64(max_q) + 2) * (2 * WC + 1);
    const u64 groups = scratch_elems / per_group;
    u64 blocks = groups / (u64(GPW) * (WD_THREADS / 32));
    const u64 reads_per_block = u64(GPW) * (WD_THREADS / 32);
    const u64 need = (u64(max_reads) + reads_per_block - 1) / reads_per_block;
    if (blocks > need) blocks = need;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks == 0) return;
    cudaMemsetAsync(ctr, 0, sizeof(u32), s);
    k_baq_wide<G, NS><<<u32(blocks), WD_THREADS, 0, s>>>(b, ref, w, list, count, ctr, scratch, max_q, min_bw);
    g_kernel_launches++;
}

}  // namespace

void baq_wide_set_constants(const HmmConst &c) {
    cudaMemcpyToSymbol(cw_qual2prob, c.qual2prob, sizeof(c.qual2prob));
    cudaMemcpyToSymbol(cw_gap_open, &c.gap_open, sizeof(double));
}

u64 baq_wide_scratch_bytes(u32 reads, u32 max_q) {
    // whole blocks of the 32 x 2 kernel (the launch sizes its grid by the groups the scratch holds; fewer than a
    // block launches none), and at least one block of the 16 x 3 and of the 32 x 4 kernel
    constexpr u64 per_block = WD_THREADS / 32;  // groups per block of the 32 x 2 kernel (one read per warp)
    const u64 rows = u64(max_q) + 2;
    const u64 per_group = rows * (2 * 64 + 1) * sizeof(float);
    u64 groups = std::min<u64>(std::max<u32>(reads, 1), 152ull * 8 * per_block);
    groups = (groups + per_block - 1) / per_block * per_block;
    const u64 block_16x3 = rows * (2 * 48 + 1) * sizeof(float) * (2 * per_block);
    const u64 block_32x4 = rows * (2 * 128 + 1) * sizeof(float) * per_block;
    return std::max<u64>(per_group * groups, std::max(block_16x3, block_32x4));
}

void launch_baq_wide(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                     u32 max_reads, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q, cudaStream_t s) {
    if (!max_reads) return;
    // bands up to bw 23 (47 cells): 16 lanes x 3 slots, two reads per warp; bw 24..31 (63 cells): 32 lanes x 2
    // slots, a read per warp. Each kernel takes its share of the list and skips the other's reads; the two share
    // the scratch and the work counters, so they run one after the other.
    launch_w<16, 3>(b, ref, w, list, count, max_reads, ctr, (float *)scratch, scratch_bytes / 4, max_q, s);
    launch_w<32, 2>(b, ref, w, list, count, max_reads, ctr, (float *)scratch, scratch_bytes / 4, max_q, s, 24);
}

void launch_baq_wide64(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                       u32 max_reads, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q, cudaStream_t s) {
    if (!max_reads) return;
    // bands of bw 32..63 (at most 127 cells) from the class-2 list: 32 lanes x 4 slots, a read per warp
    launch_w<32, 4>(b, ref, w, list, count, max_reads, ctr, (float *)scratch, scratch_bytes / 4, max_q, s, 32);
}

void launch_baq_wide16(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                       u32 max_reads, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q, cudaStream_t s) {
    if (!max_reads) return;
    // band class 1 (bw <= 15, at most 31 cells): 16 lanes x 2 slots, two reads per warp
    launch_w<16, 2>(b, ref, w, list, count, max_reads, ctr, (float *)scratch, scratch_bytes / 4, max_q, s);
}

}  // namespace fpg
