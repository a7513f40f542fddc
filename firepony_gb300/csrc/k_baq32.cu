// K2 (fast path): the banded glocal BAQ HMM (device/baq.cu:214-697) in FP32 with per-row scaling, one
// group of G lanes per read (G = 16 for band width <= 7, G = 32 for <= 15); lane l holds band slot l+1 of
// the current row, so the M/I recurrences from the previous row are one register shuffle away and the D
// chain along the row is a log2(G)-step parallel linear-recurrence scan. Forward rows (M, I) are kept for
// the MAP step in a per-group scratch slot (L2-resident); backward is fused with MAP.
//
// Certified decisions. All HMM quantities are sums of products of non-negative terms, so every value
// carries a relative error of at most (rounding depth) * 2^-24, and uniform row scalings cancel in the
// posterior. Per read the bound is eps = (33 (qlen+1) + 10) 2^-24 (33 roundings per row on the deepest
// path: 6 for M, 26 for the scanned D chain, 1 for the row scaling). For each base the kernel reports
//   - the MAP quality clamp(floor(t)) and whether min(original quality, clamp(floor(t'))) is the same for
//     every t' within the bound (else bit0 of baq_amb: quality undecided);
//   - the MAP state and whether the runner-up cell is below the best by more than the bound (else bit1).
// The capping kernel recomputes in FP64 exactly those reads whose capped qualities depend on an undecided
// value. In-band values below 1e-30 (where FP32 loses relative precision) mark the whole read undecided.
#include "kernels.h"

namespace fpg {

__constant__ float c32_e_match[256];
__constant__ float c32_e_mis[256];
__constant__ double c32_gap_open;

namespace {

constexpr u32 FULL = 0xffffffffu;
constexpr int WARPS = 8;
constexpr int MAXQ = 512;
constexpr int MAXREF = 1024;
constexpr float UNDERFLOW_GUARD = 1e-30f;

struct GroupSmem {
    u8 ref[MAXREF];
    u8 qry[MAXQ];
    u8 qul[MAXQ];
    float scale[MAXQ + 2];
};

template <int G> __device__ __forceinline__ float sh_up(float v, int d) { return __shfl_up_sync(FULL, v, d, G); }
template <int G> __device__ __forceinline__ float sh_dn(float v, int d) { return __shfl_down_sync(FULL, v, d, G); }
template <int G> __device__ __forceinline__ float sh_x(float v, int m) { return __shfl_xor_sync(FULL, v, m, G); }
template <int G> __device__ __forceinline__ int sh_xi(int v, int m) { return __shfl_xor_sync(FULL, v, m, G); }

template <int G> __device__ __forceinline__ float reduce_add(float v) {
#pragma unroll
    for (int m = G / 2; m >= 1; m >>= 1) v += sh_x<G>(v, m);
    return v;
}

// inclusive x_l = a_l + c * x_{l-1}
template <int G> __device__ __forceinline__ float scan_fwd(float a, float c, int gl) {
    float x = a, p = c;
#pragma unroll
    for (int d = 1; d < G; d <<= 1) {
        const float y = sh_up<G>(x, d);
        if (gl >= d) x = fmaf(p, y, x);
        p = p * p;
    }
    return x;
}
// inclusive x_l = a_l + c * x_{l+1}
template <int G> __device__ __forceinline__ float scan_bwd(float a, float c, int gl) {
    float x = a, p = c;
#pragma unroll
    for (int d = 1; d < G; d <<= 1) {
        const float y = sh_dn<G>(x, d);
        if (gl + d < G) x = fmaf(p, y, x);
        p = p * p;
    }
    return x;
}

__device__ __forceinline__ float eps32(u8 ref, u8 rd, u8 q) {
    if (ref == IUPAC_N || rd == IUPAC_N) return 1.0f;
    return ref == rd ? c32_e_match[q] : c32_e_mis[q];
}

// min(original, clamp(floor(t))) with clamp of device/baq.cu:673-674 and saturating (int) conversion
__device__ __forceinline__ int capped_value(float t, int qo) {
    int k;
    if (!(t == t)) k = 0;
    else if (t >= 2147483520.0f) k = 2147483647;
    else k = int(floorf(t));
    const int c = k > 100 ? 99 : (k < MIN_BASE_QUAL ? MIN_BASE_QUAL : k);
    return c < qo ? c : qo;
}
__device__ __forceinline__ int clamp_value(float t) {
    int k;
    if (!(t == t)) k = 0;
    else if (t >= 2147483520.0f) k = 2147483647;
    else k = int(floorf(t));
    return k > 100 ? 99 : (k < MIN_BASE_QUAL ? MIN_BASE_QUAL : k);
}

template <int G>
__global__ void __launch_bounds__(WARPS * 32) k_baq32(DevBatch b, DevRef ref, BatchWork w, const u32 *list,
                                                      const u32 *count, u32 *work_ctr, float *scratch) {
    constexpr int GPW = 32 / G;  // groups per warp
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GroupSmem *sm_all = reinterpret_cast<GroupSmem *>(smem_raw);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int g = lane / G;       // group within the warp
    const int gl = lane % G;      // lane within the group
    GroupSmem &sm = sm_all[warp * GPW + g];
    const u32 slot = (blockIdx.x * WARPS + warp) * GPW + g;
    float2 *frow = reinterpret_cast<float2 *>(scratch) + u64(slot) * (MAXQ + 1) * G;
    const u32 n = *count;
    const float EI = 0.25f;
    const double GOP = c32_gap_open;

    for (;;) {
        u32 base = 0;
        if (lane == 0) base = atomicAdd(work_ctr, u32(GPW));
        base = __shfl_sync(FULL, base, 0);
        if (base >= n) break;
        const u32 li = base + g;
        const bool has = li < n;
        const u32 r = has ? list[li] : 0;

        // ---- per-read setup (device/baq.cu:247-334) ----
        int qLen = 0, refLen = 0, bw = 1, qx = 0;
        u32 qual0 = 0;
        float sM = 0, bM = 0, bI = 0, m0 = 0, m1 = 0, m2 = 0, m3 = 0, m4 = 0, m6 = 0, m8 = 0;
        if (has) {
            const u16 *win = w.win + size_t(r) * 8;
            qx = win[0];
            const int qy = win[1];
            const int hx = w.hmm[size_t(r) * 2], hy = w.hmm[size_t(r) * 2 + 1];
            bw = w.bw[r];
            refLen = hy - hx + 1;
            const int bmLen = refLen;
            qLen = qy - qx + 1;
            const u32 astart = b.astart[r];
            u64 ref_off;
            const u32 ahx = hx < 0 ? u32(-hx) : u32(hx);
            if (hx < 0 && astart < ahx) { ref_off = 0; refLen--; }
            else ref_off = u64(u32(astart + u32(hx)));
            const DevContig gc = ref.contigs[b.chromosome[r]];
            const u64 qsym = u64(b.read_start[r]) + qx;
            qual0 = b.qual_start[r] + qx;
            for (int k = gl; k < refLen && k < MAXREF; k += G) sm.ref[k] = contig_at(gc, ref_off + u64(k));
            for (int i = gl; i < qLen; i += G) {
                sm.qry[i] = sym4(b.reads, qsym + u64(i));
                sm.qul[i] = b.quals[qual0 + i];
            }
            const double dsM = 1.0 / (2 * qLen + 2);
            sM = float(dsM);
            bM = float((1 - GOP) / bmLen);
            bI = float(GOP / bmLen);
            m0 = float((1 - GOP - GOP) * (1 - dsM));
            m1 = float(GOP * (1 - dsM));
            m2 = m1;
            m3 = float((1 - 0.1) * (1 - dsM));
            m4 = float(0.1 * (1 - dsM));
            m6 = float(1 - 0.1);
            m8 = 0.1f;
        }
        __syncwarp();
        const int qOther = __shfl_xor_sync(FULL, qLen, 16);  // only meaningful for G == 16
        const int maxQ = (G == 16) ? (qLen > qOther ? qLen : qOther) : qLen;
        const float eps = float((33.0 * (qLen + 1) + 10.0) * 5.9604644775390625e-8);
        const float dt = 4.343f * (2.0f * eps + 6e-8f) / (1.0f - 2.0f * eps) + 1e-4f;
        bool under = false;

        // ---- forward ----
        float pM = 0.f, pI = 0.f, pD = 0.f;
        if (has && 1 <= qLen) {
            const int k = gl;
            const int end = refLen < bw + 1 ? refLen : bw + 1;
            const bool inb = k >= 1 && k <= end;
            const float e = inb ? eps32(sm.ref[k - 1], sm.qry[0], sm.qul[0]) : 0.f;
            pM = e * bM;
            pI = inb ? EI * bI : 0.f;
        }
        float lastM = 0.f, lastI = 0.f;  // row qlen, for s[qlen+1]
        {
            const float s1 = reduce_add<G>(pM + pI);
            if (has && gl == 0) sm.scale[1] = s1;
            const float inv = has ? 1.0f / s1 : 0.f;
            pM *= inv;
            pI *= inv;
            if (has && qLen >= 1) frow[G + gl] = make_float2(pM, pI);
            if ((pM > 0.f && pM < UNDERFLOW_GUARD) || (pI > 0.f && pI < UNDERFLOW_GUARD)) under = true;
            lastM = pM;
            lastI = pI;
        }
        for (int i = 2; i <= maxQ; i++) {
            const bool act = has && i <= qLen;
            const int d = (i <= bw) ? 1 : 0;
            const int k = (i > bw) ? gl + i - bw : gl;
            const int beg = 1 > i - bw ? 1 : i - bw;
            const int end = refLen < i + bw ? refLen : i + bw;
            const bool inb = act && k >= beg && k <= end;
            float Ma = sh_up<G>(pM, d), Ia = sh_up<G>(pI, d), Da = sh_up<G>(pD, d);
            if (d && gl == 0) { Ma = 0.f; Ia = 0.f; Da = 0.f; }
            float Mb = sh_dn<G>(pM, 1 - d), Ib = sh_dn<G>(pI, 1 - d);
            if (!d && gl == G - 1) { Mb = 0.f; Ib = 0.f; }
            const u8 q = act ? sm.qry[i - 1] : 0;
            const u8 qq = act ? sm.qul[i - 1] : 0;
            const float e = inb ? eps32(sm.ref[k - 1], q, qq) : 0.f;
            float M = e * fmaf(m0, Ma, fmaf(m3, Ia, m6 * Da));
            float I = inb ? EI * fmaf(m1, Mb, m4 * Ib) : 0.f;
            float a = m2 * sh_up<G>(M, 1);
            if (gl == 0) a = 0.f;
            float D = scan_fwd<G>(a, m8, gl);
            if (!inb) { M = 0.f; I = 0.f; D = 0.f; }
            const float s = reduce_add<G>(M + I + D);
            if (act && gl == 0) sm.scale[i] = s;
            const float inv = act ? 1.0f / s : 0.f;
            pM = M * inv;
            pI = I * inv;
            pD = D * inv;
            if (act) frow[u64(i) * G + gl] = make_float2(pM, pI);
            if ((pM > 0.f && pM < UNDERFLOW_GUARD) || (pI > 0.f && pI < UNDERFLOW_GUARD) ||
                (pD > 0.f && pD < UNDERFLOW_GUARD))
                under = true;
            if (i == qLen) {
                lastM = pM;
                lastI = pI;
            }
        }
        // s[qlen+1]
        {
            float t = 0.f;
            if (has) {
                const int x = qLen - bw > 0 ? qLen - bw : 0;
                const int k = gl + x;  // slot gl+1
                if (k >= 1 && k <= refLen && gl <= 2 * bw) t = lastM * sM + lastI * sM;
            }
            const float sl = reduce_add<G>(t);
            if (has && gl == 0) sm.scale[qLen + 1] = sl;
        }
        __syncwarp();
        under = __any_sync(FULL, under);  // conservative across the warp's groups

        // ---- backward fused with MAP ----
        float bMv = 0.f, bIv = 0.f, bDv = 0.f;
        for (int t = 0; t < maxQ; t++) {
            const int i = qLen - t;
            const bool act = has && i >= 1;
            const int k = (i > bw) ? gl + i - bw : gl;
            const int beg = 1 > i - bw ? 1 : i - bw;
            const int end = refLen < i + bw ? refLen : i + bw;
            const bool inb = act && k >= beg && k <= end;
            float2 f = make_float2(0.f, 0.f);
            if (act) f = frow[u64(i) * G + gl];
            if (t == 0) {
                // b[l_query] (:533-545)
                const bool cell = act && k >= 1 && k <= refLen && gl <= 2 * bw;
                const float s0 = act ? sm.scale[qLen] : 1.f, s1 = act ? sm.scale[qLen + 1] : 1.f;
                bMv = cell ? sM / s0 / s1 : 0.f;
                bIv = bMv;
                bDv = 0.f;
            } else {
                const int dp = (i < bw) ? 1 : 0;
                float nBM = sh_dn<G>(bMv, dp);
                if (dp && gl == G - 1) nBM = 0.f;
                float nBI = sh_up<G>(bIv, 1 - dp);
                if (!dp && gl == 0) nBI = 0.f;
                const float y = (i > 1) ? 1.f : 0.f;
                float e = 0.f;
                if (inb && k < refLen) e = eps32(sm.ref[k], sm.qry[i], sm.qul[i]) * nBM;
                float Dn = scan_bwd<G>(y * (e * m6), y * m8, gl);
                if (!inb) Dn = 0.f;
                float Dk1 = sh_dn<G>(Dn, 1);
                if (gl == G - 1) Dk1 = 0.f;
                float M = fmaf(e, m0, fmaf(EI * m1, nBI, m2 * Dk1));
                float I = fmaf(e, m3, EI * m4 * nBI);
                if (!inb) { M = 0.f; I = 0.f; }
                const float inv = act ? 1.0f / sm.scale[i] : 0.f;
                bMv = M * inv;
                bIv = I * inv;
                bDv = Dn * inv;
                if ((bMv > 0.f && bMv < UNDERFLOW_GUARD) || (bIv > 0.f && bIv < UNDERFLOW_GUARD) ||
                    (bDv > 0.f && bDv < UNDERFLOW_GUARD))
                    under = true;
            }
            // MAP for row i (:619-681): best cell (first maximum in k order, M before I), runner-up, and the
            // sum of every cell other than the best
            const bool mapcell = act && k >= beg && k <= end;
            const float zM = mapcell ? f.x * bMv : 0.f;
            const float zI = mapcell ? f.y * bIv : 0.f;
            float top, second, excl;
            int idx;
            if (zI > zM) { top = zI; second = zM; idx = (k - 1) * 2 + 1; }
            else { top = zM; second = zI; idx = (k - 1) * 2; }
            if (!mapcell) { top = 0.f; second = 0.f; idx = 0x7fffffff; }
            excl = second;
#pragma unroll
            for (int m = G / 2; m >= 1; m >>= 1) {
                const float ot = sh_x<G>(top, m), os = sh_x<G>(second, m), oe = sh_x<G>(excl, m);
                const int oi = sh_xi<G>(idx, m);
                const bool mine = (top > ot) || (top == ot && idx < oi);
                const float nt = mine ? top : ot;
                const int ni = mine ? idx : oi;
                const float loser = mine ? ot : top;
                second = fmaxf(mine ? second : os, loser);
                excl = excl + oe + loser;
                top = nt;
                idx = ni;
            }
            if (act && gl == 0) {
                const u32 qi = qual0 + u32(i - 1);
                const int qo = sm.qul[i - 1];
                u8 amb = 0;
                u32 state;
                int qv;
                const float total = top + excl;
                if (!(total > 0.f) || top <= 0.f) {
                    amb = 3;
                    state = U32_NONE;
                    qv = MIN_BASE_QUAL;
                } else {
                    const int kk = idx >> 1;  // k - 1
                    state = (u32(kk) << 2) | u32(idx & 1);
                    if (second >= top * (1.0f - 2.0f * eps - 1.2e-7f)) amb |= 2;
                    const float ratio = excl / total;
                    const float tq = (ratio > 0.f) ? -4.343f * __logf(ratio) + 0.499f : __int_as_float(0x7f800000);
                    qv = clamp_value(tq);
                    const float lo = tq - dt, hi = tq + dt;
                    if (qo <= 99) {
                        if (capped_value(lo, qo) != capped_value(hi, qo)) amb |= 1;
                    } else {
                        if (!(hi < 100.f && capped_value(lo, qo) == capped_value(hi, qo)) && !(lo >= 101.5f)) amb |= 1;
                    }
                }
                w.baq_q[qi] = u8(qv);
                w.baq_state[qi] = state;
                w.baq_amb[qi] = amb;
            }
        }
        under = __any_sync(FULL, under);
        if (under && has) {
            __syncwarp();
            for (int i = gl; i < qLen; i += G) w.baq_amb[qual0 + i] = 3;
        }
        __syncwarp();
    }
}

}  // namespace

void baq32_set_constants(const HmmConst &c) {
    float em[256], mi[256];
    for (int q = 0; q < 256; q++) {
        const double p = c.qual2prob[q < MIN_BASE_QUAL ? MIN_BASE_QUAL : q];
        em[q] = float(1 - p);
        mi[q] = float(p * 0.33333333333);
    }
    cudaMemcpyToSymbol(c32_e_match, em, sizeof(em));
    cudaMemcpyToSymbol(c32_e_mis, mi, sizeof(mi));
    cudaMemcpyToSymbol(c32_gap_open, &c.gap_open, sizeof(double));
}

u64 baq32_scratch_floats(int group_lanes, u32 max_qlen) {
    (void)max_qlen;
    const u64 slots = u64(152) * 4 * WARPS * (32 / group_lanes);
    return slots * (MAXQ + 1) * group_lanes * 2;
}

void launch_baq32(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                  u32 max_reads, int group_lanes, float *scratch, u32 max_qlen, cudaStream_t s) {
    (void)max_qlen;
    if (!max_reads) return;
    u32 *ctr = w.counters + 8 + (group_lanes == 16 ? 0 : 1);
    cudaMemsetAsync(ctr, 0, sizeof(u32), s);
    const u32 per_block = WARPS * (32 / group_lanes);
    u32 blocks = u32(152) * 4;
    const u32 need = (max_reads + per_block - 1) / per_block;
    if (need < blocks) blocks = need;
    const size_t smem = sizeof(GroupSmem) * WARPS * (32 / group_lanes);
    if (group_lanes == 16) {
        static bool attr16 = false;
        if (!attr16) {
            cudaFuncSetAttribute(k_baq32<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            attr16 = true;
        }
        k_baq32<16><<<blocks, WARPS * 32, smem, s>>>(b, ref, w, list, count, ctr, scratch);
    } else {
        static bool attr32 = false;
        if (!attr32) {
            cudaFuncSetAttribute(k_baq32<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            attr32 = true;
        }
        k_baq32<32><<<blocks, WARPS * 32, smem, s>>>(b, ref, w, list, count, ctr, scratch);
    }
    g_kernel_launches++;
}

}  // namespace fpg
