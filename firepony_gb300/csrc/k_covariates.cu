// K3: fractional errors (device/fractional_errors.cu:39-141), high-quality windows
// (device/covariates.cu:215-246) and covariate keys (device/covariates.cu:50-103 with the bit packers of
// device/covariates/bit_packers/*.h) — one thread per read, in two passes over the read's events:
//   count: folds observation counts (order-free integers) into the dense tables with atomics and counts
//          the read's entries with a nonzero mismatch value;
//   emit:  writes those entries as packed 64-bit (dense key << 32 | float bits) in stream order
//          (event, then M/I/D slot) at the read's offset, for the ordered float fold of k_sort.cu.
// Zero mismatch values are not emitted: adding +0.0f to a non-negative float sum is the identity, so the
// ordered sum over nonzero addends equals the reference's fold over all of them.
#include "kernels.h"

namespace fpg {

namespace {

struct us2 { u16 x, y; };

// calculateFractionalErrorArray for one error bit of the per-base flags
__device__ void fractional_errors(const u8 *bf, const u8 *tag, int n, u8 bit, float *out, int stride) {
    bool inBlock = false;
    int bs = -1;
    int iii;
    auto block = [&](int last, int start) {
        const int s0 = start - 1 > 0 ? start - 1 : 0;
        int total = 0;
        for (int j = s0; j <= last; j++) total += (bf[j] & bit) ? 1 : 0;
        const double v = double(total) / double(last - s0 + 1);
        for (int j = s0; j <= last; j++) out[j * stride] = float(v);
    };
    for (iii = 0; iii < n; iii++) {
        if (tag[iii] == NO_BAQ_UNCERTAINTY) {
            if (!inBlock) {
                out[iii * stride] = (bf[iii] & bit) ? 1.0f : 0.0f;
            } else {
                block(iii, bs);
                inBlock = false;
                bs = -1;
            }
        } else {
            inBlock = true;
            if (bs == -1) bs = iii;
        }
    }
    if (inBlock) block(iii - 1, bs);
}

struct ReadKeys {
    u32 rg, qs, rs;
    bool neg, paired_second;
    us2 cw, hq;
    const u32 *reads;
};

// covariate_Cycle_Illumina::encode (cycle_illumina.h:46-95)
__device__ __forceinline__ void cycle_keys(const ReadKeys &k, int off, u32 &sub, u32 &ind) {
    const int readLength = int(k.cw.y) - int(k.cw.x) + 1;
    const int order = k.paired_second ? -1 : 1;
    const int i = off - int(k.cw.x);
    int cycle, inc;
    if (k.neg) { cycle = readLength * order; inc = -order; }
    else { cycle = order; inc = order; }
    cycle += i * inc;
    const int maxc = readLength - 4 - 1;
    u32 res = u32(cycle < 0 ? -cycle : cycle) << 1;
    if (cycle < 0) res++;
    sub = res;
    ind = (i < 4 || i > maxc) ? CYCLE_INVALID : res;
}

// covariate_Context::encode (context.h:106-174)
__device__ __forceinline__ void context_keys(const ReadKeys &k, int off, u32 &cm, u32 &ci) {
    cm = CONTEXT_INVALID;
    ci = CONTEXT_INVALID;
    const int dir = k.neg ? 1 : -1;
    const int avail = k.neg ? int(k.hq.y) - off + 1 : off - int(k.hq.x) + 1;
    const int nb = avail < 3 ? avail : 3;
    if (nb < 2) return;
    u32 ctx = 0;
    int num = 0;
    for (int j = 0, i = off; j < nb; j++, i += dir) {
        const u8 bp = sym4(k.reads, u64(k.rs) + u32(i));
        if (bp != IUPAC_A && bp != IUPAC_C && bp != IUPAC_T && bp != IUPAC_G) break;
        ctx = (ctx << 2) | u32(31 - __clz(u32(bp)));
        num++;
    }
    if (k.neg) ctx = ~ctx & ((1u << (num * 2)) - 1);
    if (num >= 2) cm = ((ctx >> (num - 2) * 2) << 4) | 2;
    if (num >= 3) ci = ((ctx >> (num - 3) * 2) << 4) | 3;
}

template <bool EMIT>
__global__ void __launch_bounds__(128) k_cov(DevBatch b, BatchWork w, Tables t) {
    const u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= b.R) return;
    if (w.status[r] != RS_ACTIVE) {
        if (!EMIT) w.entry_count[r] = 0;
        return;
    }
    const u16 *win = w.win + size_t(r) * 8;
    ReadKeys k;
    k.rg = b.rg[r];
    k.qs = b.qual_start[r];
    k.rs = b.read_start[r];
    const u16 fl = b.flags[r];
    k.neg = fl & F_REVERSE;
    k.paired_second = (fl & F_PAIRED) && (fl & F_READ2);
    k.cw = us2{win[0], win[1]};
    k.reads = b.reads;
    const u8 *q = b.quals + k.qs;
    const u8 *bf = w.bflags + k.qs;
    const int n = int(k.cw.y) - int(k.cw.x) + 1;
    float *frac = w.frac + size_t(k.qs) * 3;

    if (!EMIT) {
        // high-quality window (LOW_QUAL_TAIL = 2)
        us2 h = k.cw;
        while (q[h.x] <= 2 && h.x < h.y) h.x++;
        while (q[h.y] <= 2 && h.y > h.x) h.y--;
        w.win[size_t(r) * 8 + 6] = h.x;
        w.win[size_t(r) * 8 + 7] = h.y;
        k.hq = h;
        const u8 *tg = w.tag + k.qs + k.cw.x;
        fractional_errors(bf + k.cw.x, tg, n, BF_SNP, frac + size_t(k.cw.x) * 3 + 0, 3);
        fractional_errors(bf + k.cw.x, tg, n, BF_INS, frac + size_t(k.cw.x) * 3 + 1, 3);
        fractional_errors(bf + k.cw.x, tg, n, BF_DEL, frac + size_t(k.cw.x) * 3 + 2, 3);
    } else {
        k.hq = us2{win[6], win[7]};
    }

    const u32 cs = w.cigar_offsets[b.cigar_start[r]];
    const u32 ce = w.cigar_offsets[b.cigar_start[r] + b.cigar_len[r]];
    const KeySpace ks = t.ks;
    u32 nnz = 0;
    u64 *out = EMIT ? w.entries + w.entry_offset[r] : nullptr;
    const u32 rgq = k.rg * Q_SPAN;
    for (u32 e = cs; e < ce; e++) {
        const u32 rc = w.ev_rc[e];
        const u16 off = u16(rc & 0xFFFF);
        if (off == U16_NONE) continue;
        if (off < k.cw.x || off > k.cw.y) continue;
        if (!(bf[off] & BF_ACTIVE)) continue;
        if (w.ev_type[e] == EV_S) continue;
        const u32 qm = q[off];
        const float mm[3] = {frac[size_t(off) * 3 + 0], frac[size_t(off) * 3 + 1], frac[size_t(off) * 3 + 2]};
        const u32 qv[3] = {qm, 45, 45};
        u32 sub, ind, cm, ci;
        cycle_keys(k, off, sub, ind);
        context_keys(k, off, cm, ci);
        const u32 cyc[3] = {sub, ind, ind};
        const u32 ctx[3] = {cm, ci, ci};
#pragma unroll
        for (u32 ev = 0; ev < 3; ev++) {
            const u32 rq = rgq + qv[ev];
            const u32 kq = ks.qual_base + rq * 3 + ev;
            const bool vc = cyc[ev] != CYCLE_INVALID;
            const u32 kc = vc ? ks.cycle_base + (rq * CYCLE_SPAN + cyc[ev]) * 3 + ev : 0;
            const bool vx = ctx[ev] != CONTEXT_INVALID;
            const u32 kx = vx ? ks.context_base + (rq * CONTEXT_SPAN + context_rank(ctx[ev])) * 3 + ev : 0;
            if (!EMIT) {
                atomicAdd(&t.obs[kq], 1ull);
                if (vc) atomicAdd(&t.obs[kc], 1ull);
                if (vx) atomicAdd(&t.obs[kx], 1ull);
            }
            if (mm[ev] != 0.0f) {
                const u64 fb = u64(__float_as_uint(mm[ev]));
                if (EMIT) {
                    out[nnz] = (u64(kq) << 32) | fb;
                    if (vc) out[nnz + 1] = (u64(kc) << 32) | fb;
                    if (vx) out[nnz + 1 + (vc ? 1 : 0)] = (u64(kx) << 32) | fb;
                }
                nnz += 1 + (vc ? 1 : 0) + (vx ? 1 : 0);
            }
        }
    }
    if (!EMIT) w.entry_count[r] = nnz;
}

}  // namespace

void launch_cov_count(const DevBatch &b, const BatchWork &w, const Tables &t, cudaStream_t s) {
    if (!b.R) return;
    k_cov<false><<<(b.R + 127) / 128, 128, 0, s>>>(b, w, t);
    g_kernel_launches++;
}

void launch_cov_emit(const DevBatch &b, const BatchWork &w, const Tables &t, cudaStream_t s) {
    if (!b.R) return;
    k_cov<true><<<(b.R + 127) / 128, 128, 0, s>>>(b, w, t);
    g_kernel_launches++;
}

}  // namespace fpg
