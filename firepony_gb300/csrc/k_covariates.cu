// K3: fractional errors (device/fractional_errors.cu:39-141), high-quality windows
// (device/covariates.cu:215-246) and covariate keys (device/covariates.cu:50-103 with the bit packers of
// device/covariates/bit_packers/*.h; the cycle key follows cycle_illumina.h:46-95 and the context key
// context.h:106-174) — one warp per read, in two passes over the read's events:
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

constexpr int COV_WARPS = 8;
constexpr u32 FULL = 0xffffffffu;

struct CovSmem {
    u8 q[512];
    u8 bf[512];
    u8 tag[512];
    u8 sym[512];
};
struct FracSmem {
    u32 pre[512];   // window-relative prefix counts of the SNP / insertion / deletion bits (10 bits each)
    i16 last[512];  // last base before j (window-relative) whose BQ tag is NO_BAQ_UNCERTAINTY, or -1
    u8 nz[512];     // read position -> which of the base's three fractional errors are nonzero (bits M, I, D)
};

// calculateFractionalErrorArray (device/fractional_errors.cu:39-141) for the three error bits at once, in
// parallel over the window. The reference walks the window once: a base whose BQ tag is
// NO_BAQ_UNCERTAINTY outside a block takes its own error bit; a maximal run of other tags (a block) and
// the bases on either side of it (the one before, and the closing one after if any) take the block's
// average, a later block overwriting the shared base of an earlier one. For base j with last64 / next64
// the nearest NO_BAQ_UNCERTAINTY bases before / after it (-1 / n when none):
//   block member:                      range [max(last64, 0), min(next64, n - 1)]
//   base before a block (j+1 member):  range [j, min(next64, n - 1)]
//   closing base (j-1 member):         range [max(last64, 0), j]
//   otherwise:                         its own bit
// with the average double(bits in range) / double(range length) rounded to float, as in the reference.
__device__ void fractional_errors_warp(const CovSmem &sm, FracSmem &fs, u32 wx, int n, float *frac, int lane) {
    const u32 lt = (1u << lane) - 1;
    u32 carry_pre = 0;
    int carry_last = -1;
    for (int c = 0; c < n; c += 32) {
        const int j = c + lane;
        const bool in = j < n;
        const u8 bfv = in ? sm.bf[wx + j] : 0;
        const bool m64 = in && sm.tag[wx + j] == NO_BAQ_UNCERTAINTY;
        const u32 ms = __ballot_sync(FULL, bfv & BF_SNP), mi = __ballot_sync(FULL, bfv & BF_INS);
        const u32 md = __ballot_sync(FULL, bfv & BF_DEL), m6 = __ballot_sync(FULL, m64);
        const u32 pre = carry_pre + u32(__popc(ms & lt)) + (u32(__popc(mi & lt)) << 10) + (u32(__popc(md & lt)) << 20);
        const u32 below = m6 & lt;
        const int last = below ? c + 31 - __clz(below) : carry_last;
        if (in) {
            fs.pre[j] = pre;
            fs.last[j] = i16(last);
        }
        carry_pre += u32(__popc(ms)) + (u32(__popc(mi)) << 10) + (u32(__popc(md)) << 20);
        if (m6) carry_last = c + 31 - __clz(m6);
    }
    if (lane == 0) fs.pre[n] = carry_pre;
    __syncwarp();
    int carry_next = n;
    for (int c = ((n - 1) / 32) * 32; c >= 0; c -= 32) {
        const int j = c + lane;
        const bool in = j < n;
        const bool m64 = in && sm.tag[wx + j] == NO_BAQ_UNCERTAINTY;
        const u32 m6 = __ballot_sync(FULL, m64);
        const u32 above = m6 & ~((2u << lane) - 1u);
        const int next = above ? c + __ffs(above) - 1 : carry_next;
        if (in) {
            int lo = -1, hi = -1;
            if (!m64) {
                lo = fs.last[j] > 0 ? fs.last[j] : 0;
                hi = next < n - 1 ? next : n - 1;
            } else if (j + 1 < n && sm.tag[wx + j + 1] != NO_BAQ_UNCERTAINTY) {
                lo = j;
                hi = next < n - 1 ? next : n - 1;
            } else if (j >= 1 && sm.tag[wx + j - 1] != NO_BAQ_UNCERTAINTY) {
                lo = fs.last[j] > 0 ? fs.last[j] : 0;
                hi = j;
            }
            float *o = frac + size_t(j) * 3;
            if (lo < 0) {
                const u8 bfv = sm.bf[wx + j];
                o[0] = (bfv & BF_SNP) ? 1.0f : 0.0f;
                o[1] = (bfv & BF_INS) ? 1.0f : 0.0f;
                o[2] = (bfv & BF_DEL) ? 1.0f : 0.0f;
                fs.nz[wx + j] = u8(((bfv & BF_SNP) ? 1 : 0) | ((bfv & BF_INS) ? 2 : 0) | ((bfv & BF_DEL) ? 4 : 0));
            } else {
                // float(double(n) / double(len)) as in the reference, computed as one correctly rounded FP32
                // division: with n <= 2^24 and len < 2^28 the exact quotient is at least 2^-25/len away from any
                // float rounding midpoint it does not equal, far more than the 2^-53 the double rounding can
                // move it, so both roundings give the same float
                const u32 d = fs.pre[hi + 1] - fs.pre[lo];
                const float len = float(hi - lo + 1);
                o[0] = __fdiv_rn(float(d & 1023u), len);
                o[1] = __fdiv_rn(float((d >> 10) & 1023u), len);
                o[2] = __fdiv_rn(float(d >> 20), len);
                // a nonzero count over a range of at most 512 bases gives a nonzero float quotient
                fs.nz[wx + j] = u8(((d & 1023u) ? 1 : 0) | (((d >> 10) & 1023u) ? 2 : 0) | ((d >> 20) ? 4 : 0));
            }
        }
        if (m6) carry_next = c + __ffs(m6) - 1;
    }
}

__device__ __forceinline__ void context_keys_smem(const u8 *sym, bool neg, us2 hq, int off, u32 &cm, u32 &ci) {
    cm = CONTEXT_INVALID;
    ci = CONTEXT_INVALID;
    const int dir = neg ? 1 : -1;
    const int avail = neg ? int(hq.y) - off + 1 : off - int(hq.x) + 1;
    const int nb = avail < 3 ? avail : 3;
    if (nb < 2) return;
    u32 ctx = 0;
    int num = 0;
    for (int j = 0, i = off; j < nb; j++, i += dir) {
        const u8 bp = sym[i];
        if (bp != IUPAC_A && bp != IUPAC_C && bp != IUPAC_T && bp != IUPAC_G) break;
        ctx = (ctx << 2) | u32(31 - __clz(u32(bp)));
        num++;
    }
    if (neg) ctx = ~ctx & ((1u << (num * 2)) - 1);
    if (num >= 2) cm = ((ctx >> (num - 2) * 2) << 4) | 2;
    if (num >= 3) ci = ((ctx >> (num - 3) * 2) << 4) | 3;
}

// warp-aggregated increment: lanes holding the same key add their count through one atomic
__device__ __forceinline__ void agg_add(u32 *cnt, u32 key, bool valid, int lane) {
    const u32 k = valid ? key : 0xFFFFFFFFu;
    const u32 peers = __match_any_sync(FULL, k);
    if (valid && (__ffs(peers) - 1) == lane) atomicAdd(&cnt[key], u32(__popc(peers)));
}
// adds n to both counters of the aligned (I, D) pair starting at `key` (slot 2) with one 64-bit atomic
__device__ __forceinline__ void add_pair(u32 *cnt, u32 key, u32 n) {
    atomicAdd(reinterpret_cast<unsigned long long *>(cnt + key), (unsigned long long)n | ((unsigned long long)n << 32));
}

// Count-kernel counters privatised per block (when the read groups are few enough): the quality-table M
// counters (n_rg x 256) and the context-table I/D pair counters (n_rg x 80, the I and D counts of a key are
// equal), in dynamic shared memory, flushed with one global atomic per nonzero counter at the end.
constexpr u32 HIST_MAX_RG = 8;
__host__ __device__ constexpr u32 hist_words(u32 n_rg) { return n_rg <= HIST_MAX_RG ? n_rg * (256 + 80) : 0; }

// One warp per read. Lanes stage the read's qualities, flags, BQ tags and bases in shared memory, then walk
// the read's CIGAR events 32 at a time (lane = event).
// Count passes: the first (LIST false) takes every active read and skips the deferred ones; the second
// (LIST true) takes the reads of a replay list and marks them active again. The emit pass takes every
// active read.
template <bool EMIT, bool LIST = false>
__global__ void __launch_bounds__(COV_WARPS * 32) k_cov(DevBatch b, BatchWork w, Tables t, const u32 *list,
                                                        const u32 *list_count) {
    __shared__ CovSmem smem[COV_WARPS];
    __shared__ FracSmem fsmem[EMIT ? 1 : COV_WARPS];
    extern __shared__ u32 hist[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    CovSmem &sm = smem[warp];
    FracSmem &fs = fsmem[EMIT ? 0 : warp];
    const u32 lt = (1u << lane) - 1;
    const KeySpace ks = t.ks;
    const u32 hw_n = EMIT ? 0 : hist_words(ks.n_rg);
    u32 *hist_q = hist, *hist_x = hist + ks.n_rg * 256;
    if (!EMIT) {
        for (u32 i = threadIdx.x; i < hw_n; i += blockDim.x) hist[i] = 0;
        __syncthreads();
    }
    const u32 n_items = LIST ? *list_count : b.R;
    for (u32 item = blockIdx.x * COV_WARPS + warp; item < n_items; item += gridDim.x * COV_WARPS) {
        const u32 r = LIST ? list[item] : item;
        const u8 status = w.status[r];
        if (!LIST && status != RS_ACTIVE) {
            // deferred reads are counted by the second pass, which also writes their entry counts
            if (!EMIT && lane == 0 && status != RS_DEFERRED) w.entry_count[r] = 0;
            continue;
        }
        if (LIST && lane == 0) w.status[r] = RS_ACTIVE;
        const u16 *win = w.win + size_t(r) * 8;
        const us2 cw = {win[0], win[1]};
        const u32 qs = b.qual_start[r], rs = b.read_start[r], rlen = b.read_len[r];
        const u32 rg = b.rg[r];
        const u16 fl = b.flags[r];
        const bool neg = fl & F_REVERSE;
        const bool second = (fl & F_PAIRED) && (fl & F_READ2);
        __syncwarp();
        for (u32 i = lane; i < rlen; i += 32) {
            sm.q[i] = b.quals[qs + i];
            sm.bf[i] = w.bflags[qs + i];
            sm.tag[i] = w.tag[qs + i];
            sm.sym[i] = sym4(b.reads, u64(rs) + i);
        }
        __syncwarp();
        float *frac = w.frac + size_t(qs) * 3;
        us2 hq;
        if (!EMIT) {
            // high-quality window (device/covariates.cu:215-246): first base in [x, y) with q > 2, else y;
            // then the last base in (x', y] with q > 2, else x'
            u32 hx = cw.y;
            for (u32 c = cw.x; c < cw.y; c += 32) {
                const u32 pos = c + lane;
                const u32 m = __ballot_sync(FULL, pos < cw.y && sm.q[pos < 511 ? pos : 0] > 2);
                if (m) { hx = c + __ffs(m) - 1; break; }
            }
            u32 hy = hx;
            for (int c = int(cw.y); c > int(hx); c -= 32) {
                const int pos = c - lane;
                const u32 m = __ballot_sync(FULL, pos > int(hx) && sm.q[pos > 0 ? pos : 0] > 2);
                if (m) { hy = u32(c - (__ffs(m) - 1)); break; }
            }
            hq = us2{u16(hx), u16(hy)};
            if (lane == 0) {
                w.win[size_t(r) * 8 + 6] = hq.x;
                w.win[size_t(r) * 8 + 7] = hq.y;
            }
            fractional_errors_warp(sm, fs, cw.x, int(cw.y) - int(cw.x) + 1, frac + size_t(cw.x) * 3, lane);
            __syncwarp();
        } else {
            hq = us2{win[6], win[7]};
        }

        const u32 cs = w.cigar_offsets[b.cigar_start[r]];
        const u32 ce = w.cigar_offsets[b.cigar_start[r] + b.cigar_len[r]];
        const u32 rgq = rg * Q_SPAN;
        const int readLength = int(cw.y) - int(cw.x) + 1;
        const int order = second ? -1 : 1;
        u32 gathered_total = 0;
        u32 nnz_total = 0;
        u64 *out = EMIT ? w.entries + w.entry_offset[r] : nullptr;
        for (u32 base = cs; base < ce; base += 32) {
            const u32 e = base + lane;
            bool g = false;
            u16 off = 0;
            if (e < ce) {
                const u32 rc = w.ev_rc[e];
                off = u16(rc & 0xFFFF);
                g = off != U16_NONE && off >= cw.x && off <= cw.y && (sm.bf[off] & BF_ACTIVE) &&
                    w.ev_type[e] != EV_S;
            }
            const u32 gm = __ballot_sync(FULL, g);
            if (!gm) continue;
            gathered_total += __popc(gm);
            // keys (covariate chains of device/covariates/packer_*.h)
            u32 qm = 0, sub = 0, ind = CYCLE_INVALID, cm = CONTEXT_INVALID, ci = CONTEXT_INVALID;
            float mm0 = 0.f, mm1 = 0.f, mm2 = 0.f;
            if (g) {
                qm = sm.q[off];
                const int i = int(off) - int(cw.x);
                int cycle, inc;
                if (neg) { cycle = readLength * order; inc = -order; }
                else { cycle = order; inc = order; }
                cycle += i * inc;
                u32 res = u32(cycle < 0 ? -cycle : cycle) << 1;
                if (cycle < 0) res++;
                sub = res;
                ind = (i < 4 || i > readLength - 5) ? CYCLE_INVALID : res;
                context_keys_smem(sm.sym, neg, hq, off, cm, ci);
                if (EMIT) {
                    mm0 = frac[size_t(off) * 3 + 0];
                    mm1 = frac[size_t(off) * 3 + 1];
                    mm2 = frac[size_t(off) * 3 + 2];
                } else {
                    // the count pass needs only which values are nonzero (the fractional-error step's mask)
                    const u8 z = fs.nz[off];
                    mm0 = (z & 1) ? 1.f : 0.f;
                    mm1 = (z & 2) ? 1.f : 0.f;
                    mm2 = (z & 4) ? 1.f : 0.f;
                }
            }
            const u32 kq0 = ks.qual_base + (rgq + qm) * EV_SLOTS + 0;
            const u32 kq1 = ks.qual_base + (rgq + 45) * EV_SLOTS + 2;
            const u32 kq2 = kq1 + 1;
            const u32 kc0 = ks.cycle_base + ((rgq + qm) * CYCLE_SPAN + sub) * EV_SLOTS + 0;
            const bool vci = ind != CYCLE_INVALID;
            const u32 kc1 = vci ? ks.cycle_base + ((rgq + 45) * CYCLE_SPAN + ind) * EV_SLOTS + 2 : 0;
            const u32 kc2 = kc1 + 1;
            const bool vxm = cm != CONTEXT_INVALID, vxi = ci != CONTEXT_INVALID;
            const u32 kx0 = vxm ? ks.context_base + ((rgq + qm) * CONTEXT_SPAN + context_rank(cm)) * EV_SLOTS + 0 : 0;
            const u32 kx1 = vxi ? ks.context_base + ((rgq + 45) * CONTEXT_SPAN + context_rank(ci)) * EV_SLOTS + 2 : 0;
            const u32 kx2 = kx1 + 1;
            if (!EMIT) {
                if (hw_n) {
                    if (g) atomicAdd(&hist_q[rg * 256 + qm], 1u);
                } else {
                    agg_add(t.stage, kq0, g, lane);
                }
                if (g) atomicAdd(&t.stage[kc0], 1u);
                // cycle I/D pairs: along a run of events on consecutive bases |cycle| moves by one, so a run
                // is one range update of the (read group, cycle sign) difference array
                {
                    const bool gv = g && vci;
                    const u32 gvm = __ballot_sync(FULL, gv);
                    const u32 poff = __shfl_up_sync(FULL, u32(off), 1), noff = __shfl_down_sync(FULL, u32(off), 1);
                    const bool pv = lane > 0 && ((gvm >> (lane - 1)) & 1u);
                    const bool nv = lane < 31 && ((gvm >> (lane + 1)) & 1u);
                    const bool run_start = gv && !(pv && poff + 1 == u32(off));
                    const bool run_end = gv && !(nv && noff == u32(off) + 1);
                    if (run_start || run_end) {
                        const int i = int(off) - int(cw.x);
                        const int a = neg ? readLength - i : 1 + i;  // |cycle|
                        int *d = t.cyc_diff + (size_t(rg) * 2 + (second ? 1 : 0)) * CYC_DIFF_LEN;
                        // forward strand: |cycle| rises along the run, reverse strand: it falls
                        if (run_start) atomicAdd(d + (neg ? a + 1 : a), neg ? -1 : 1);
                        if (run_end) atomicAdd(d + (neg ? a : a + 1), neg ? 1 : -1);
                    }
                }
                // context M keys spread over (read group, quality, 2-mer): one plain atomic per lane costs fewer issue
                // slots than a match-based aggregation (the quality and context I/D keys below collide far more
                // often within a warp and keep theirs)
                if (g && vxm) atomicAdd(&t.stage[kx0], 1u);
                if (hw_n) {
                    if (g && vxi) atomicAdd(&hist_x[rg * 80 + context_rank(ci)], 1u);
                } else {
                    // the I and D context keys of a base share the context value: aggregate once, add the pair
                    const u32 k = (g && vxi) ? kx1 : 0xFFFFFFFFu;
                    const u32 peers = __match_any_sync(FULL, k);
                    if (g && vxi && (__ffs(peers) - 1) == lane) add_pair(t.stage, kx1, u32(__popc(peers)));
                }
            }
            // entries with a nonzero mismatch value, in slot order M, I, D; per slot quality, cycle, context
            u32 cnt = 0;
            if (g) {
                if (mm0 != 0.f) cnt += 1 + 1 + (vxm ? 1 : 0);
                if (mm1 != 0.f) cnt += 1 + (vci ? 1 : 0) + (vxi ? 1 : 0);
                if (mm2 != 0.f) cnt += 1 + (vci ? 1 : 0) + (vxi ? 1 : 0);
            }
            u32 x = cnt;
            u32 chunk_total;
            if (EMIT) {
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const u32 y = __shfl_up_sync(FULL, x, d);
                    if (lane >= d) x += y;
                }
                chunk_total = __shfl_sync(FULL, x, 31);
            } else {
                chunk_total = __reduce_add_sync(FULL, cnt);  // the count pass needs the total only
            }
            if (EMIT && cnt) {
                u64 *o = out + nnz_total + (x - cnt);
                u32 j = 0;
                if (mm0 != 0.f) {
                    const u64 fb = u64(__float_as_uint(mm0));
                    o[j++] = (u64(kq0) << 32) | fb;
                    o[j++] = (u64(kc0) << 32) | fb;
                    if (vxm) o[j++] = (u64(kx0) << 32) | fb;
                }
                if (mm1 != 0.f) {
                    const u64 fb = u64(__float_as_uint(mm1));
                    o[j++] = (u64(kq1) << 32) | fb;
                    if (vci) o[j++] = (u64(kc1) << 32) | fb;
                    if (vxi) o[j++] = (u64(kx1) << 32) | fb;
                }
                if (mm2 != 0.f) {
                    const u64 fb = u64(__float_as_uint(mm2));
                    o[j++] = (u64(kq2) << 32) | fb;
                    if (vci) o[j++] = (u64(kc2) << 32) | fb;
                    if (vxi) o[j++] = (u64(kx2) << 32) | fb;
                }
            }
            nnz_total += chunk_total;
            (void)lt;
        }
        if (!EMIT && lane == 0) {
            w.entry_count[r] = nnz_total;
            if (gathered_total) {
                // every gathered base adds one observation to the read group's I and D quality keys
                add_pair(t.stage, ks.qual_base + (rgq + 45) * EV_SLOTS + 2, gathered_total);
            }
        }
    }
    if (!EMIT && hw_n) {
        __syncthreads();
        for (u32 i = threadIdx.x; i < ks.n_rg * 256; i += blockDim.x) {
            const u32 v = hist_q[i];
            if (v) atomicAdd(&t.stage[ks.qual_base + i * EV_SLOTS + 0], v);
        }
        for (u32 i = threadIdx.x; i < ks.n_rg * 80; i += blockDim.x) {
            const u32 v = hist_x[i];
            if (v) add_pair(t.stage, ks.context_base + (((i / 80) * Q_SPAN + 45) * CONTEXT_SPAN + i % 80) * EV_SLOTS + 2, v);
        }
    }
}

// folds the batch's cycle difference arrays into the cycle I/D counters and clears them: one warp per
// (read group, cycle sign), a running sum over |cycle|
__global__ void k_cycle_pairs(Tables t) {
    const u32 wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (wid >= t.ks.n_rg * 2) return;
    const u32 rg = wid >> 1, sign = wid & 1;
    int *d = t.cyc_diff + size_t(wid) * CYC_DIFF_LEN;
    int carry = 0;
    for (u32 c = 0; c < CYC_DIFF_LEN; c += 32) {
        const u32 a = c + lane;
        int v = a < CYC_DIFF_LEN ? d[a] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, v, o);
            if (int(lane) >= o) v += y;
        }
        const int n = carry + v;
        carry += __shfl_sync(FULL, v, 31);
        if (a < CYC_DIFF_LEN) {
            d[a] = 0;
            if (n > 0) {
                const u32 res = (a << 1) | sign;
                const u32 key = t.ks.cycle_base + ((rg * Q_SPAN + 45) * CYCLE_SPAN + res) * EV_SLOTS + 2;
                t.stage[key] += u32(n);
                t.stage[key + 1] += u32(n);
            }
        }
    }
}


__global__ void k_merge_stage(u32 *stage, unsigned long long *obs, u32 n) {
    const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const u32 v = stage[i];
    if (v) {
        obs[i] += v;
        stage[i] = 0;
    }
}

}  // namespace

void launch_merge_stage(const Tables &t, cudaStream_t s) {
    const u32 n = t.ks.total;
    k_merge_stage<<<(n + 255) / 256, 256, 0, s>>>(t.stage, t.obs, n);
    g_kernel_launches++;
}


void launch_cov_count(const DevBatch &b, const BatchWork &w, const Tables &t, cudaStream_t s) {
    if (!b.R) return;
    u32 blocks = (b.R + COV_WARPS - 1) / COV_WARPS;
    if (blocks > 152 * 16) blocks = 152 * 16;
    const size_t smem = size_t(hist_words(t.ks.n_rg)) * sizeof(u32);
    if (smem) cudaFuncSetAttribute(k_cov<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    k_cov<false, false><<<blocks, COV_WARPS * 32, smem, s>>>(b, w, t, nullptr, nullptr);
    g_kernel_launches++;
}

void launch_cov_count_list(const DevBatch &b, const BatchWork &w, const Tables &t, const u32 *list,
                           const u32 *count, u32 max_items, cudaStream_t s) {
    if (!max_items) return;
    u32 blocks = (max_items + COV_WARPS - 1) / COV_WARPS;
    if (blocks > 152 * 16) blocks = 152 * 16;
    const size_t smem = size_t(hist_words(t.ks.n_rg)) * sizeof(u32);
    if (smem) cudaFuncSetAttribute(k_cov<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    k_cov<false, true><<<blocks, COV_WARPS * 32, smem, s>>>(b, w, t, list, count);
    g_kernel_launches++;
}

void launch_cycle_pairs(const Tables &t, cudaStream_t s) {
    const u32 warps = t.ks.n_rg * 2;
    k_cycle_pairs<<<(warps + 3) / 4, 128, 0, s>>>(t);
    g_kernel_launches++;
}

void launch_cov_emit(const DevBatch &b, const BatchWork &w, const Tables &t, cudaStream_t s) {
    if (!b.R) return;
    u32 blocks = (b.R + COV_WARPS - 1) / COV_WARPS;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_cov<true, false><<<blocks, COV_WARPS * 32, 0, s>>>(b, w, t, nullptr, nullptr);
    g_kernel_launches++;
}

}  // namespace fpg
