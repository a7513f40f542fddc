// K2 replay: the banded glocal BAQ HMM (device/baq.cu:214-697) in exact FP64 for the reads whose FP32
// result could not be certified, one group of G lanes per read (32/G reads per warp).
//
// Every multiply and add is an explicit __dmul_rn/__dadd_rn in the reference's order, so each intermediate
// double equals the reference's. On this GPU an FP64 warp instruction holds its warp for ~64 cycles whatever
// its active lanes, so a replay's time is its FP64 instruction count per read: the band cells of a row are
// spread over the group's lanes (G lanes x NS slots, WC = G*NS >= 2*bw+1), and only the order-sensitive
// chains run on one lane per group (lane 0): the D recurrence along the row and the running sums (forward
// row sum, MAP posterior sum), each a strict left-to-right sequence as in the reference. The 32/G chain
// lanes of a warp run their chains in the same instructions.
//
// Slot s of row i holds cell k = s + x(i), x(i) = max(i - bw, 0). Row exchange goes through a per-group
// shared buffer indexed by slot + 1 with zero sentinels at both ends, so out-of-band neighbours read 0 as in
// the reference's zero-initialised rows. All groups of a warp step through the same row loop (the longest
// read of the warp); a group past its own read's rows computes zeros and writes nothing.
//
// A replayed read needs exact results only where the FP32 pass left a base undecided (baq_amb != 0): the
// certified rows keep their FP32 MAP output, which agrees with the reference wherever the capping step
// looks. The forward pass is complete; the backward pass runs from the last row down to the lowest
// undecided row, and MAP runs on the undecided rows only (all rows with the test hook).
//
// Per group scratch (global): rows 0..max_q+1 of ROWD doubles: forward M (WC), forward I (WC), the forward
// row sum (replaced by its reciprocal before the backward pass), and the row's MAP maximum and sum.
#include "kernels.h"

namespace fpg {

__constant__ double cx_qual2prob[256];
__constant__ double cx_gap_open;

namespace {

constexpr u32 FULL = 0xffffffffu;
// 64-thread blocks (80-96 registers a thread): a replay block fits in the registers an SM running three
// blocks of the FP32 band-class-0 kernel leaves free, so a replay on another stream runs beside it
constexpr int EX_THREADS = 64;

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }

template <int G, int NS>
__global__ void __launch_bounds__(EX_THREADS) k_baq_exact(DevBatch b, DevRef dref, BatchWork w, const u32 *list,
                                                          const u32 *count, u32 *work_ctr, double *scratch,
                                                          u32 max_q, int full, int min_wc) {
    constexpr int WC = G * NS;          // band slots per read
    constexpr int GPW = 32 / G;         // reads (groups) per warp
    constexpr int WPB = EX_THREADS / 32;
    constexpr int ROWD = 2 * WC + 3;    // scratch doubles per row
    constexpr int XB = 2 * WC + 2;      // exchange buffer length
    __shared__ double s_em[256], s_mis[256];
    // per group: forward previous row (M, I, D), backward next row (M, I), three exchange buffers
    __shared__ double s_buf[WPB][GPW][8][XB];
    for (int q = threadIdx.x; q < 256; q += blockDim.x) {
        const double p = cx_qual2prob[q < MIN_BASE_QUAL ? MIN_BASE_QUAL : q];
        // calcEpsilon (device/baq.cu:361-372)
        s_em[q] = 1 - p;
        s_mis[q] = p * 0.33333333333;
    }
    for (int i = threadIdx.x; i < WPB * GPW * 8 * XB; i += blockDim.x) (&s_buf[0][0][0][0])[i] = 0.0;
    __syncthreads();

    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int g = lane / G, l = lane % G, gbase = g * G;
    double *PM = s_buf[wib][g][0], *PI = s_buf[wib][g][1], *PD = s_buf[wib][g][2];
    double *QM = s_buf[wib][g][3], *QI = s_buf[wib][g][4];
    double *X0 = s_buf[wib][g][5], *X1 = s_buf[wib][g][6], *X2 = s_buf[wib][g][7];
    const u32 gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    double *gs = scratch + (u64(gwarp) * GPW + g) * (u64(max_q) + 2) * ROWD;
    auto FROW = [&](int row) -> double * { return gs + u64(row) * ROWD; };
    const u32 n_list = *count;
    const double EI = 0.25;
    const double GOP = cx_gap_open;

    for (;;) {
        u32 base = 0;
        if (lane == 0) base = atomicAdd(work_ctr, u32(GPW));
        base = __shfl_sync(FULL, base, 0);
        if (base >= n_list) break;
        const u32 li = base + g;
        bool has = li < n_list;
        const u32 r = has ? list[li] : 0;
        // a read whose band does not fit the group's slots is left to a wider kernel (or the thread-per-read
        // one), a read whose band fits min_wc slots to the narrower kernel that took it
        if (has && (2 * int(w.bw[r]) + 1 > WC || 2 * int(w.bw[r]) + 1 <= min_wc)) has = false;

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
        auto EMI = [&](u8 ref, u8 rd, u8 q) -> double {
            if (ref == IUPAC_N || rd == IUPAC_N) return 1.0;
            return ref == rd ? s_em[q] : s_mis[q];
        };
        const int Qmax = int(__reduce_max_sync(FULL, u32(qL)));
        // rows whose FP32 result was certified keep it (the capping step needs exactly the certified part):
        // only undecided rows get an exact MAP, and the backward pass stops at the lowest of them (full: all)
        int i_min = qL + 1;
        if (has) {
            if (full) {
                i_min = 1;
            } else {
                for (int row = 1 + l; row <= qL; row += G)
                    if (w.baq_amb[qual0 + u32(row - 1)]) { i_min = row; break; }
            }
        }
#pragma unroll
        for (int o = G / 2; o >= 1; o >>= 1) {
            const int v = __shfl_xor_sync(FULL, i_min, o);
            i_min = v < i_min ? v : i_min;
        }
        const int Tmax = int(__reduce_max_sync(FULL, u32(qL - i_min + 1 > 0 ? qL - i_min + 1 : 0)));

        const double dsM = 1.0 / (2 * (qL > 0 ? qL : 1) + 2);
        const double sM = dsM, sI = dsM;
        const double bM = (1 - GOP) / bmLen, bI = GOP / bmLen;
        const double m0 = (1 - GOP - GOP) * (1 - dsM), m1 = GOP * (1 - dsM), m2 = m1;
        const double m3 = (1 - 0.1) * (1 - dsM), m4 = 0.1 * (1 - dsM);
        const double m6 = 1 - 0.1, m8 = 0.1;
        const double EIm1 = dm(EI, m1), EIm4 = dm(EI, m4);

        // ---- forward, row 1: slot s = cell k, band [1, min(refLen, bw + 1)] ----
        double fM[NS], fI[NS], fD[NS];
        {
            const int end = refLen < bw + 1 ? refLen : bw + 1;
            const bool act = qL >= 1;
            const u8 q0 = act ? QRY(0) : 0, qq0 = act ? QUL(0) : 0;
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G;
                const bool inb = act && s >= 1 && s <= end;
                fM[j] = inb ? dm(EMI(REF(s - 1), q0, qq0), bM) : 0.0;
                fI[j] = inb ? dm(EI, bI) : 0.0;
                fD[j] = 0.0;
                X0[s] = inb ? da(fM[j], fI[j]) : 0.0;
            }
            __syncwarp();
            double sum = 0.0;
            if (l == 0) {
#pragma unroll
                for (int s = 0; s < WC; s++) sum = da(sum, X0[s]);
                if (act) FROW(1)[2 * WC] = sum;
            }
            sum = __shfl_sync(FULL, sum, gbase);
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G;
                if (act) {
                    fM[j] = __ddiv_rn(fM[j], sum);
                    fI[j] = __ddiv_rn(fI[j], sum);
                    FROW(1)[s] = fM[j];
                    FROW(1)[WC + s] = fI[j];
                }
                PM[s + 1] = act ? fM[j] : 0.0;
                PI[s + 1] = act ? fI[j] : 0.0;
                PD[s + 1] = 0.0;
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
            // the serial loops below visit only the slots that hold band cells of some group of the warp: every
            // other slot holds zeros, which change neither a sum nor the D chain (bit for bit)
            const int slo = int(__reduce_min_sync(FULL, u32(act ? (beg - x > 0 ? beg - x : 0) : WC)));
            const int shi = int(__reduce_max_sync(FULL, u32(act ? (end - x < WC - 1 ? end - x : WC - 1) : 0)));
            // phase A: M and I of every slot from the previous row; m2 * M feeds the D chain of the next slot
            double mI[NS];
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G, k = s + x;
                const bool inb = act && k >= beg && k <= end;
                const double oM = slide ? PM[s + 1] : PM[s], oI = slide ? PI[s + 1] : PI[s];
                const double oD = slide ? PD[s + 1] : PD[s];
                const double nM1 = slide ? PM[s + 2] : PM[s + 1], nI1 = slide ? PI[s + 2] : PI[s + 1];
                double m = 0.0, ii = 0.0;
                if (inb) {
                    const double e = EMI(REF(k - 1), qy, qq);
                    m = dm(e, da(da(dm(m0, oM), dm(m3, oI)), dm(m6, oD)));
                    ii = dm(EI, da(dm(m1, nM1), dm(m4, nI1)));
                }
                fM[j] = m;
                mI[j] = da(m, ii);
                fI[j] = ii;
                X0[s + 1] = dm(m2, m);
            }
            __syncwarp();
            // phase B1: D(k) = m2 * M(k-1) + m8 * D(k-1) along the row (zero below the band; past it the chain
            // runs on but those slots are discarded)
            if (l == 0) {
                double d = 0.0;  // (zero at and below the lowest band slot: M below the band is zero)
                for (int s = slo; s <= shi; s++) {
                    d = da(s == 0 ? 0.0 : X0[s], dm(m8, d));
                    X1[s] = d;
                }
            }
            __syncwarp();
            // phase B2: the row-sum terms (M + I) + D
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G, k = s + x;
                const bool inb = act && k >= beg && k <= end;
                fD[j] = inb ? X1[s] : 0.0;
                X2[s] = inb ? da(mI[j], fD[j]) : 0.0;
            }
            __syncwarp();
            // phase B3: the row sum in k order, its reciprocal
            double inv = 0.0;
            if (l == 0) {
                double sum = 0.0;
                for (int s = slo; s <= shi; s++) sum = da(sum, X2[s]);
                if (act) {
                    FROW(i)[2 * WC] = sum;
                    inv = __ddiv_rn(1.0, sum);
                }
            }
            inv = __shfl_sync(FULL, inv, gbase);
            // phase C: scale; publish the row for the next one and the scratch copy for MAP
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G;
                fM[j] = dm(fM[j], inv);
                fI[j] = dm(fI[j], inv);
                fD[j] = dm(fD[j], inv);
                PM[s + 1] = fM[j];
                PI[s + 1] = fI[j];
                PD[s + 1] = fD[j];
                if (act) {
                    FROW(i)[s] = fM[j];
                    FROW(i)[WC + s] = fI[j];
                }
            }
            __syncwarp();
        }

        // ---- s[qL+1] and the backward start (device/baq.cu:520-545) ----
        double bMv[NS], bIv[NS];
        {
            const int x = qL - bw > 0 ? qL - bw : 0;
            bool cell[NS];
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G, k = s + x;
                cell[j] = qL >= 1 && s <= 2 * bw && k >= 1 && k <= refLen;
                const double lm = qL >= 1 ? FROW(qL)[s] : 0.0, lI = qL >= 1 ? FROW(qL)[WC + s] : 0.0;
                X0[s] = cell[j] ? da(dm(lm, sM), dm(lI, sI)) : 0.0;
            }
            __syncwarp();
            double sLast = 0.0;
            if (l == 0) {
#pragma unroll
                for (int s = 0; s < WC; s++) sLast = da(sLast, X0[s]);
            }
            sLast = __shfl_sync(FULL, sLast, gbase);
            const double sQ = qL >= 1 ? FROW(qL)[2 * WC] : 1.0;
            const double v = __ddiv_rn(__ddiv_rn(sM, sQ), sLast);
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G;
                bMv[j] = cell[j] ? v : 0.0;
                bIv[j] = cell[j] ? v : 0.0;
                QM[s + 1] = bMv[j];
                QI[s + 1] = bIv[j];
            }
            // 1 / s[i] for the backward rows, in parallel over the rows
            for (int row = i_min + l; row < qL; row += G) FROW(row)[2 * WC] = __ddiv_rn(1.0, FROW(row)[2 * WC]);
            __syncwarp();
        }

        // ---- backward fused with MAP, rows qL..i_min of every group (t steps back from its own last row) ----
        for (int t = 0; t < Tmax; t++) {
            const int i = qL - t;
            const bool act = i >= i_min;
            const int beg = 1 > i - bw ? 1 : i - bw;
            const int end = refLen < i + bw ? refLen : i + bw;
            const int x = i - bw > 0 ? i - bw : 0;
            const bool on = i >= 1 && i <= qL;
            const int slo = int(__reduce_min_sync(FULL, u32(on ? (beg - x > 0 ? beg - x : 0) : WC)));
            const int shi = int(__reduce_max_sync(FULL, u32(on ? (end - x < WC - 1 ? end - x : WC - 1) : 0)));
            if (t > 0) {
                const bool grow = i < bw;  // row i+1 still in the growing band
                const bool y = i > 1;
                const u8 qy1 = act ? QRY(i) : 0, qq1 = act ? QUL(i) : 0;
                double a1[NS], e6[NS];
#pragma unroll
                for (int j = 0; j < NS; j++) {
                    const int s = l + j * G, k = s + x;
                    const bool inb = act && k >= beg && k <= end;
                    // B_M(i+1, k+1): slot s+1 (growing) or s (sliding); B_I(i+1, k): slot s or s-1
                    const double nbm = grow ? QM[s + 2] : QM[s + 1];
                    const double bi1 = grow ? QI[s + 1] : QI[s];
                    double e = 0.0;
                    if (inb && k < refLen) e = dm(EMI(REF(k), qy1, qq1), nbm);
                    a1[j] = da(dm(e, m0), dm(EIm1, bi1));
                    bIv[j] = inb ? da(dm(e, m3), dm(EIm4, bi1)) : 0.0;
                    e6[j] = inb ? dm(e, m6) : 0.0;
                    X0[s] = e6[j];
                }
                __syncwarp();
                // B_D(k) = (e * m6 + m8 * B_D(k+1)) * y, descending along the row
                if (l == 0) {
                    double d = 0.0;  // (zero above the highest band slot)
                    X1[WC] = 0.0;
                    X1[shi + 1] = 0.0;
                    for (int s = shi; s >= slo; s--) {
                        d = y ? da(X0[s], dm(m8, d)) : 0.0;
                        X1[s] = d;
                    }
                }
                __syncwarp();
                const double yy = act ? FROW(i)[2 * WC] : 0.0;
#pragma unroll
                for (int j = 0; j < NS; j++) {
                    const int s = l + j * G, k = s + x;
                    const bool inb = act && k >= beg && k <= end;
                    const double dnext = X1[s + 1];
                    const double bm = inb ? da(a1[j], dm(m2, dnext)) : 0.0;
                    bMv[j] = dm(bm, yy);
                    bIv[j] = dm(bIv[j], yy);
                }
                __syncwarp();
#pragma unroll
                for (int j = 0; j < NS; j++) {
                    const int s = l + j * G;
                    QM[s + 1] = bMv[j];
                    QI[s + 1] = bIv[j];
                }
            }
            // ---- MAP for row i (device/baq.cu:619-681): first maximum in (k, M before I) order ----
            const bool need = act && (full || w.baq_amb[qual0 + u32(i - 1)] != 0);
            if (!__any_sync(FULL, need)) continue;
            unsigned long long best = 0;
            u32 best_k = 0xFFFFFFFFu;
#pragma unroll
            for (int j = 0; j < NS; j++) {
                const int s = l + j * G, k = s + x;
                const bool inb = need && k >= beg && k <= end;
                double zm = 0.0, zi = 0.0;
                if (inb) {
                    zm = dm(FROW(i)[s], bMv[j]);
                    zi = dm(FROW(i)[WC + s], bIv[j]);
                }
                X2[2 * s] = zm;
                X2[2 * s + 1] = zi;
                // non-negative doubles order like their bit patterns; ties keep the smaller (earlier) index
                const unsigned long long bm_ = __double_as_longlong(zm), bi_ = __double_as_longlong(zi);
                const u32 km = u32((k - 1) << 2), ki = km | 1u;
                if (bm_ > best || (bm_ == best && km < best_k)) { best = bm_; best_k = km; }
                if (bi_ > best || (bi_ == best && ki < best_k)) { best = bi_; best_k = ki; }
            }
#pragma unroll
            for (int o = G / 2; o >= 1; o >>= 1) {
                const unsigned long long ob = __shfl_xor_sync(FULL, best, o);
                const u32 ok = __shfl_xor_sync(FULL, best_k, o);
                if (ob > best || (ob == best && ok < best_k)) { best = ob; best_k = ok; }
            }
            __syncwarp();
            if (l == 0 && need) {
                double sum = 0.0;
                for (int q = 2 * slo; q <= 2 * shi + 1; q++) sum = da(sum, X2[q]);
                FROW(i)[2 * WC + 1] = __longlong_as_double((long long)best);
                FROW(i)[2 * WC + 2] = sum;
                // the reference keeps max_k = -1 when no term exceeds 0
                w.baq_state[qual0 + u32(i - 1)] = best == 0 ? U32_NONE : best_k;
            }
            __syncwarp();
        }

        // ---- MAP qualities, in parallel over the rows: (int)(-4.343 * log(1 - max/sum) + .499) ----
        for (int row = 1 + l; row <= qL; row += G) {
            if (!full && !w.baq_amb[qual0 + u32(row - 1)]) continue;
            const double mx = FROW(row)[2 * WC + 1], sum = FROW(row)[2 * WC + 2];
            const double p = __ddiv_rn(mx, sum);
            const double tq = da(dm(-4.343, log(__dsub_rn(1.0, p))), 0.499);
            const int kq = int(tq);
            const u32 qi = qual0 + u32(row - 1);
            w.baq_q[qi] = u8(kq > 100 ? 99 : (kq < MIN_BASE_QUAL ? MIN_BASE_QUAL : kq));
            w.baq_amb[qi] = 0;
        }
        __syncwarp();
    }
}

template <int G, int NS>
void launch_g(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
              u32 max_reads, u32 *ctr, double *scratch, u64 scratch_elems, u32 max_q, int full, cudaStream_t s,
              int min_wc = 0) {
    constexpr int WC = G * NS, GPW = 32 / G;
    const u64 per_group = (u64(max_q) + 2) * (2 * WC + 3);
    const u64 groups = scratch_elems / per_group;
    u64 blocks = groups / (u64(GPW) * (EX_THREADS / 32));
    const u64 reads_per_block = u64(GPW) * (EX_THREADS / 32);
    const u64 need = (u64(max_reads) + reads_per_block - 1) / reads_per_block;
    if (blocks > need) blocks = need;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks == 0) return;
    cudaMemsetAsync(ctr, 0, sizeof(u32), s);
    k_baq_exact<G, NS><<<u32(blocks), EX_THREADS, 0, s>>>(b, ref, w, list, count, ctr, scratch, max_q, full, min_wc);
    g_kernel_launches++;
}

}  // namespace

u64 baq_exact_block_scratch_bytes(int band_class, u32 max_q) {
    // one block of each kernel a band class uses (GPW groups per warp, 2 warps): the launches size their grids
    // by the groups the scratch holds and launch nothing below one block
    auto block = [&](int wc, int gpw) { return u64(gpw) * (EX_THREADS / 32) * (u64(max_q) + 2) * (2 * wc + 3) * 8; };
    if (band_class == 0) return block(16, 4);
    if (band_class == 1) return block(32, 2);
    return std::max(std::max(block(48, 2), block(64, 1)), block(128, 1));
}

void baq_exact_set_constants(const HmmConst &c) {
    cudaMemcpyToSymbol(cx_qual2prob, c.qual2prob, sizeof(c.qual2prob));
    cudaMemcpyToSymbol(cx_gap_open, &c.gap_open, sizeof(double));
}

void launch_baq_exact(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                      u32 max_reads, int band_class, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q,
                      bool all_rows, cudaStream_t s) {
    if (!max_reads) return;
    // band class 0 (bw <= 7, 15 slots): 8 lanes x 2 slots, 4 reads per warp; class 1 (bw <= 15, 31 slots):
    // 16 lanes x 2 slots, 2 reads per warp; wider bands: 16 lanes x 3 slots (bw <= 23, 2 reads per warp), then
    // 32 lanes x 2 slots up to bw 31 and 32 lanes x 4 slots up to bw 63 (a read per warp; each later launch reuses
    // the work counter after the earlier one finishes on the same stream)
    double *d = (double *)scratch;
    const int full = all_rows ? 1 : 0;
    if (band_class == 0) {
        launch_g<8, 2>(b, ref, w, list, count, max_reads, ctr, d, scratch_bytes / 8, max_q, full, s);
    } else if (band_class == 1) {
        launch_g<16, 2>(b, ref, w, list, count, max_reads, ctr, d, scratch_bytes / 8, max_q, full, s);
    } else {
        launch_g<16, 3>(b, ref, w, list, count, max_reads, ctr, d, scratch_bytes / 8, max_q, full, s);
        launch_g<32, 2>(b, ref, w, list, count, max_reads, ctr, d, scratch_bytes / 8, max_q, full, s, 48);
        launch_g<32, 4>(b, ref, w, list, count, max_reads, ctr, d, scratch_bytes / 8, max_q, full, s, 64);
    }
}

}  // namespace fpg
