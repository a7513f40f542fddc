// K2 (plain FP64 path and FP64 escalation path): the banded glocal HMM of device/baq.cu:214-697 replayed
// in IEEE double with the reference's operation order, one thread per read. Compiled with -fmad=false so
// no product is fused into an addition: every intermediate double is bit-identical to the reference's host
// computation. The per-read forward/backward matrices live in a global scratch pool interleaved across the
// 32 lanes of a warp; each row is cleared just before it is written, which reproduces the zero-filled
// matrices of device/baq.cu:1245-1247 for every cell the recurrences read.
#include "kernels.h"

namespace fpg {

__constant__ double c64_qual2prob[256];
__constant__ double c64_gap_open;

namespace {

constexpr u32 THREADS = 128;
constexpr u32 BLOCKS_PER_SM = 4;
constexpr u32 NUM_SM = 152;

struct Strided {
    double *p;
    __device__ __forceinline__ double &operator[](u64 j) const { return p[j * 32]; }
};

__device__ __forceinline__ int set_u(int b, int i, int k) {
    int x = i - b;
    x = x > 0 ? x : 0;
    return (k + 1 - x) * 3;
}

__device__ __forceinline__ double calc_eps(u8 ref, u8 read, u8 q) {
    if (ref == IUPAC_N || read == IUPAC_N) return 1.0;
    const double qual = c64_qual2prob[q < MIN_BASE_QUAL ? MIN_BASE_QUAL : q];
    return ref == read ? 1 - qual : qual * 0.33333333333;
}

__global__ void __launch_bounds__(THREADS) k_baq64(DevBatch b, DevRef ref, BatchWork w, const u32 *list,
                                                   const u32 *count, double *scratch, u64 per_thread, int min_bw,
                                                   bool trace_only) {
    const u32 tid = blockIdx.x * blockDim.x + threadIdx.x;
    const u32 nthreads = gridDim.x * blockDim.x;
    const u32 n = *count;
    double *base = scratch + u64(tid / 32) * 32 * per_thread + (tid % 32);
    const double GOP = c64_gap_open;
    const double EI = 0.25;
    const double GEP = 0.1;

    for (u32 li = tid; li < n; li += nthreads) {
        const u32 r = list[li];
        if (int(w.bw[r]) < min_bw) continue;  // (narrower bands are computed by another kernel)
        const u16 *win = w.win + size_t(r) * 8;
        const int qx = win[0], qy = win[1];
        const int hx = w.hmm[size_t(r) * 2], hy = w.hmm[size_t(r) * 2 + 1];
        const int bandWidth = w.bw[r];
        const int bandWidth2 = bandWidth * 2 + 1;
        const int row = bandWidth2 * 3 + 6;
        int referenceLength = hy - hx + 1;
        const int bmLen = referenceLength;
        const int queryLen = qy - qx + 1;
        const u32 astart = b.astart[r];
        u64 ref_off;
        const u32 ahx = hx < 0 ? u32(-hx) : u32(hx);
        if (hx < 0 && astart < ahx) {
            ref_off = 0;
            referenceLength--;
        } else {
            ref_off = u64(u32(astart + u32(hx)));
        }
        const DevContig g = ref.contigs[b.chromosome[r]];
        const u64 qsym = u64(b.read_start[r]) + qx;
        const u32 qual0 = b.qual_start[r] + qx;
        auto REF = [&](int k) -> u8 { return contig_at(g, ref_off + u64(k)); };
        auto QRY = [&](int i) -> u8 { return sym4(b.reads, qsym + u64(i)); };
        auto QUL = [&](int i) -> u8 { return b.quals[qual0 + i]; };

        Strided F{base};
        Strided B{base + u64(queryLen + 1) * row * 32};
        Strided S{base + u64(queryLen + 1) * row * 2 * 32};
        auto zero_row = [&](const Strided &M, int i) {
            for (int j = 0; j < row; j++) M[u64(i) * row + j] = 0.0;
        };

        const double sM = 1.0 / (2 * queryLen + 2);
        const double sI = sM;
        const double bM = (1 - GOP) / bmLen;
        const double bI = GOP / bmLen;
        double m[9];
        m[0] = (1 - GOP - GOP) * (1 - sM);
        m[1] = GOP * (1 - sM);
        m[2] = m[1];
        m[3] = (1 - GEP) * (1 - sI);
        m[4] = GEP * (1 - sI);
        m[5] = 0.0;
        m[6] = 1 - GEP;
        m[7] = 0.0;
        m[8] = GEP;

        int i, k;
        // forward
        S[0] = 1.0;
        {
            zero_row(F, 1);
            const u64 fo = u64(row);
            double sum = 0.0;
            const int beg = 1;
            const int end = referenceLength < bandWidth + 1 ? referenceLength : bandWidth + 1;
            for (k = beg; k <= end; ++k) {
                const double e = calc_eps(REF(k - 1), QRY(0), QUL(0));
                const int u = set_u(bandWidth, 1, k);
                F[fo + u] = e * bM;
                F[fo + u + 1] = EI * bI;
                sum += F[fo + u] + F[fo + u + 1];
            }
            S[1] = sum;
            const int _beg = set_u(bandWidth, 1, beg);
            const int _end = set_u(bandWidth, 1, end) + 2;
            for (k = _beg; k <= _end; ++k) F[fo + k] /= sum;
        }
        for (i = 2; i <= queryLen; ++i) {
            zero_row(F, i);
            const u64 fo = u64(i) * row, fo1 = u64(i - 1) * row;
            int beg = 1, end = referenceLength, x;
            const u8 qyi = QRY(i - 1);
            const u8 qq = QUL(i - 1);
            x = i - bandWidth;
            beg = beg > x ? beg : x;
            x = i + bandWidth;
            end = end < x ? end : x;
            double sum = 0.0;
            for (k = beg; k <= end; ++k) {
                const double e = calc_eps(REF(k - 1), qyi, qq);
                const int u = set_u(bandWidth, i, k);
                const int v11 = set_u(bandWidth, i - 1, k - 1);
                const int v10 = set_u(bandWidth, i - 1, k);
                const int v01 = set_u(bandWidth, i, k - 1);
                F[fo + u] = e * (m[0] * F[fo1 + v11] + m[3] * F[fo1 + v11 + 1] + m[6] * F[fo1 + v11 + 2]);
                F[fo + u + 1] = EI * (m[1] * F[fo1 + v10] + m[4] * F[fo1 + v10 + 1]);
                F[fo + u + 2] = m[2] * F[fo + v01] + m[8] * F[fo + v01 + 2];
                sum += F[fo + u] + F[fo + u + 1] + F[fo + u + 2];
            }
            S[i] = sum;
            const int _beg = set_u(bandWidth, i, beg);
            const int _end = set_u(bandWidth, i, end) + 2;
            sum = 1. / sum;
            for (k = _beg; k <= _end; ++k) F[fo + k] *= sum;
        }
        {
            double sum = 0.0;
            const u64 fo = u64(queryLen) * row;
            for (k = 1; k <= referenceLength; ++k) {
                const int u = set_u(bandWidth, queryLen, k);
                if (u < 3 || u >= bandWidth2 * 3 + 3) continue;
                sum += F[fo + u] * sM + F[fo + u + 1] * sI;
            }
            S[queryLen + 1] = sum;
        }
        // backward (b[0] is never read by MAP and is not computed)
        {
            zero_row(B, queryLen);
            const u64 bo = u64(queryLen) * row;
            for (k = 1; k <= referenceLength; ++k) {
                const int u = set_u(bandWidth, queryLen, k);
                if (u < 3 || u >= bandWidth2 * 3 + 3) continue;
                B[bo + u] = sM / S[queryLen] / S[queryLen + 1];
                B[bo + u + 1] = sI / S[queryLen] / S[queryLen + 1];
            }
        }
        for (i = queryLen - 1; i >= 1; --i) {
            zero_row(B, i);
            const u64 bo = u64(i) * row, bo1 = u64(i + 1) * row;
            int beg = 1, end = referenceLength, x;
            double y = (i > 1) ? 1. : 0.;
            const u8 qyi1 = QRY(i);
            const u8 qq1 = QUL(i);
            x = i - bandWidth;
            beg = beg > x ? beg : x;
            x = i + bandWidth;
            end = end < x ? end : x;
            for (k = end; k >= beg; --k) {
                const int u = set_u(bandWidth, i, k);
                const int v11 = set_u(bandWidth, i + 1, k + 1);
                const int v10 = set_u(bandWidth, i + 1, k);
                const int v01 = set_u(bandWidth, i, k + 1);
                double e;
                if (k >= referenceLength) e = 0;
                else e = calc_eps(REF(k), qyi1, qq1) * B[bo1 + v11];
                B[bo + u] = e * m[0] + EI * m[1] * B[bo1 + v10 + 1] + m[2] * B[bo + v01 + 2];
                B[bo + u + 1] = e * m[3] + EI * m[4] * B[bo1 + v10 + 1];
                B[bo + u + 2] = (e * m[6] + m[8] * B[bo + v01 + 2]) * y;
            }
            const int _beg = set_u(bandWidth, i, beg);
            const int _end = set_u(bandWidth, i, end) + 2;
            y = 1.0 / S[i];
            for (k = _beg; k <= _end; ++k) B[bo + k] *= y;
        }
        // MAP
        for (i = 1; i <= queryLen; ++i) {
            double sum = 0.0, max = 0.0;
            const u64 o = u64(i) * row;
            int beg = 1, end = referenceLength, x, max_k = -1;
            x = i - bandWidth;
            beg = beg > x ? beg : x;
            x = i + bandWidth;
            end = end < x ? end : x;
            for (k = beg; k <= end; ++k) {
                const int u = set_u(bandWidth, i, k);
                double z = F[o + u] * B[o + u];
                sum += z;
                if (z > max) { max = z; max_k = (k - 1) << 2 | 0; }
                z = F[o + u + 1] * B[o + u + 1];
                sum += z;
                if (z > max) { max = z; max_k = (k - 1) << 2 | 1; }
            }
            max /= sum;
            const u32 qi = qual0 + u32(i - 1);
            const double tt = double(-4.343) * log(double(1.0) - double(max)) + double(.499);
            if (trace_only) {  // precision trace: the pre-floor quality only, the batch's results untouched
                w.trace64[qi] = tt;
                continue;
            }
            w.baq_state[qi] = u32(max_k);
            // (int) conversion saturates (+inf -> INT_MAX, NaN -> 0) like the reference's CUDA build
            const int kq = int(tt);
            w.baq_q[qi] = u8(kq > 100 ? 99 : (kq < MIN_BASE_QUAL ? MIN_BASE_QUAL : kq));
            w.baq_amb[qi] = 0;
        }
    }
}

}  // namespace

u32 baq64_threads() { return THREADS * BLOCKS_PER_SM * NUM_SM; }

u64 baq64_scratch_doubles(u32 threads, u32 max_qlen, u32 max_bw) {
    const u64 row = u64(max_bw * 2 + 1) * 3 + 6;
    const u64 per = u64(max_qlen + 1) * row * 2 + (max_qlen + 2);
    return (u64(threads + THREADS - 1) / THREADS) * THREADS * per;
}

void baq64_set_constants(const HmmConst &c) {
    cudaMemcpyToSymbol(c64_qual2prob, c.qual2prob, sizeof(c.qual2prob));
    cudaMemcpyToSymbol(c64_gap_open, &c.gap_open, sizeof(double));
}

void launch_baq64(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                  u32 max_reads, double *scratch, u64 scratch_doubles, u32 max_qlen, u32 max_bw, cudaStream_t s,
                  u32 min_bw, bool trace_only) {
    if (!max_reads) return;
    const u64 row = u64(max_bw * 2 + 1) * 3 + 6;
    const u64 per = u64(max_qlen + 1) * row * 2 + (max_qlen + 2);
    // every launched thread owns one scratch slot: the grid is sized to the slots that fit
    u64 blocks = scratch_doubles / per / THREADS;
    const u64 max_blocks = baq64_threads() / THREADS;
    if (blocks > max_blocks) blocks = max_blocks;
    const u64 need = (max_reads + THREADS - 1) / THREADS;
    if (need < blocks) blocks = need;
    if (blocks == 0) return;  // caller guarantees room for at least one block
    k_baq64<<<u32(blocks), THREADS, 0, s>>>(b, ref, w, list, count, scratch, per, int(min_bw), trace_only);
    g_kernel_launches++;
}

}  // namespace fpg
