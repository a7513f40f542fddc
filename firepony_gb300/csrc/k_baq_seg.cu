// K2, band class 0 (bandwidth <= 7, the bulk of BAQ reads): the banded glocal HMM of device/baq.cu:214-697 in
// FP32 with certified decisions, one thread per read, the band row in registers.
//
// Layout and arithmetic:
//   * Slots. Row i holds cells k = s + i - bw for slots s = 0..15 (15 band slots and one that stays zero), also
//     for the first rows, where some slots fall left of the reference (k < 1): every row slides by one cell, so
//     M(i,k) reads slot s of row i-1, I(i,k) slot s+1 of row i-1 and D(i,k) slot s-1 of row i, with no special
//     case for the growing band. Rows whose band is clipped (k < 1 or k > refLen) zero their outside slots.
//   * Packed pairs. Slots are held as float2 pairs, and every update whose operands are slot-aligned (the M
//     recurrence, the emission products, the row sums, the MAP products) runs as one two-lane FP32 operation
//     (__fmul2_rn / __ffma2_rn / __fadd2_rn: each lane rounds as the scalar operation would).
//   * Scaling. Each row is scaled by a power of two chosen from the previous row's M + I sum (forward: into
//     [2^64, 2^65), backward: [2^32, 2^33)); the factor is folded into the row's emission values and gap
//     coefficients, so it costs no operation per cell and no rounding. The MAP step only uses ratios within a
//     row, where every row factor cancels.
//   * Emissions. The reference window is a 64-bit register of 16 four-bit symbols that slides with the band;
//     one XOR against the query symbol and a zero-nibble test give the row's match bits, and each slot selects
//     its match or mismatch value. Reads whose window holds a reference N go to the general kernel (k_prep
//     assigns them band class 1), so no slot needs the N case here.
//   * Memory. The forward pass keeps every SEG_K-th row (M, I, its scale and reference window) in HBM scratch.
//     The backward pass walks the segments from the last: it recomputes a segment's forward rows from its
//     checkpoint into shared memory (the same instructions, so the same values) and runs the backward rows and
//     the MAP step of the segment against them. Scratch traffic falls to 36 words per SEG_K rows from 30 per row.
//
// Certificate (as for the other FP32 kernels): every HMM value is a sum of products of non-negative terms, so a
// computed value is the exact one times (1 + theta), |theta| <= (roundings on its path) 2^-24. A path takes at
// most 6 roundings per row (the emission's and the transition's own roundings, three multiply-adds, the
// emission product; the row scale is exact) plus 2 per D step, and at most refLen D steps, so forward and
// backward values carry eps <= (7 qL + 2 refLen + 8) 2^-24 (the bound of the other FP32 kernels, kept as is).
// A posterior term carries eps_z = 2 eps + 2^-24; the sum of the terms other than the maximum and the total are
// sums of at most 2W terms in any order (2W 2^-24), so (other terms)/total is within rel = 2 (eps_z + 2W u) + u.
// A base's MAP quality is undecided when min(q_orig, clamp(floor(t'))) is not constant for t' within
// dt = 4.343 rel / (1 - rel) + 1e-4 of the computed t (1e-4 covers logf and the reference's own FP64 rounding);
// its MAP state is undecided when a rival term is within 2 eps_z + 2u (relative) of the maximum (checked only
// when the other terms together reach that threshold); with exactly one rival the rival state is recorded.
// Underflow guard: a read with an in-band M value (forward, or backward below the last reference column) below
// 1e-22 of its normalised row is undecided throughout; above it every product of the next row stays normal.
#include "kernels.h"

namespace fpg {

__constant__ double cs_qual2prob[256];
__constant__ double cs_gap_open;

namespace {

constexpr u32 FULL = 0xffffffffu;
constexpr int SEG_THREADS = 128;
constexpr int SEG_BLOCKS_PER_SM = 3;
constexpr int SEG_K = 4;          // forward rows per checkpoint
constexpr int NS = 16;            // slots per row (15 band slots + one zero slot)
constexpr int NP = NS / 2;        // slot pairs
constexpr int BW = 7;             // band half-width of class 0 (reads with a narrower band clip their slots)
constexpr int CP_WORDS = 36;      // checkpoint: M[16], I[16], scale, reference window (2 words), pad
constexpr int CP_VEC = CP_WORDS / 4;
constexpr float TINY = 1e-22f;

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float &sx(float2 (&a)[NP], int s) { return (s & 1) ? a[s >> 1].y : a[s >> 1].x; }
__device__ __forceinline__ float sxc(const float2 (&a)[NP], int s) { return (s & 1) ? a[s >> 1].y : a[s >> 1].x; }

// A power of two p with S * p in [2^target, 2^(target + 1)); `bad` is set (and 1 returned) when S is not a
// positive normal number or p would not be one.
__device__ __forceinline__ float pow2_scale(float S, int target, bool &bad) {
    const u32 eb = __float_as_uint(S) >> 23;
    const int se = 254 + target - int(eb);
    if (!(S > 0.0f) || eb >= 255u || se < 1 || se > 254) {
        bad = true;
        return 1.0f;
    }
    return __uint_as_float(u32(se) << 23);
}

// Nonzero-nibble mask of x: bit 4n set where nibble n of x is not zero.
__device__ __forceinline__ u64 nz_nibbles(u64 x) {
    x |= x >> 1;
    x |= x >> 2;
    return x & 0x1111111111111111ull;
}

// Per-read constants.
struct Coef {
    float2 m0, m3, m6, m2;  // transition pairs
    float m8, c1, c4;       // D extension, EI * m1, EI * m4 (EI = 0.25: exact products)
};

// One forward row (i >= 2) from row i-1 in place. eqs/exs: the row's match/mismatch emission times the previous
// row's scale; sig: that scale; nz: mismatch nibbles of the row's window; [lo, hi]: band slots (edge: the row is
// clipped, zero the others).
__device__ __forceinline__ void fwd_row(float2 (&M)[NP], float2 (&I)[NP], float2 (&D)[NP], const Coef &c, float sig,
                                        float eqs, float exs, u64 nz, bool edge, int lo, int hi) {
    const float c1 = c.c1 * sig, c4 = c.c4 * sig;
    float nI[NS];
#pragma unroll
    for (int s = 0; s < NS - 2; s++) nI[s] = __fmaf_rn(c4, sxc(I, s + 1), __fmul_rn(c1, sxc(M, s + 1)));
    nI[NS - 2] = 0.0f;
    nI[NS - 1] = 0.0f;
#pragma unroll
    for (int j = 0; j < NP; j++) {
        float2 t = mul2(c.m0, M[j]);
        t = fma2(c.m3, I[j], t);
        t = fma2(c.m6, D[j], t);
        const float2 e = f2(((nz >> (8 * j)) & 1) ? exs : eqs, ((nz >> (8 * j + 4)) & 1) ? exs : eqs);
        M[j] = mul2(e, t);
        I[j] = f2(nI[2 * j], nI[2 * j + 1]);
    }
    if (edge) {
#pragma unroll
        for (int s = 0; s < NS; s++)
            if (s < lo || s > hi) {
                sx(M, s) = 0.0f;
                sx(I, s) = 0.0f;
            }
    }
    float2 P[NP];
#pragma unroll
    for (int j = 0; j < NP; j++) P[j] = mul2(c.m2, M[j]);
    float d = 0.0f;
    sx(D, 0) = 0.0f;
#pragma unroll
    for (int s = 1; s < NS - 1; s++) {
        d = __fmaf_rn(c.m8, d, sxc(P, s - 1));
        sx(D, s) = (edge && s > hi) ? 0.0f : d;
    }
    sx(D, NS - 1) = 0.0f;
}

// D of a forward row from its M (a checkpointed row): the chain of fwd_row.
__device__ __forceinline__ void d_from_m(const float2 (&M)[NP], float2 (&D)[NP], const Coef &c, int hi, bool edge) {
    float2 P[NP];
#pragma unroll
    for (int j = 0; j < NP; j++) P[j] = mul2(c.m2, M[j]);
    float d = 0.0f;
    sx(D, 0) = 0.0f;
#pragma unroll
    for (int s = 1; s < NS - 1; s++) {
        d = __fmaf_rn(c.m8, d, sxc(P, s - 1));
        sx(D, s) = (edge && s > hi) ? 0.0f : d;
    }
    sx(D, NS - 1) = 0.0f;
}

// Sum of M + I over the row (the scale input).
__device__ __forceinline__ float row_sum(const float2 (&A)[NP], const float2 (&B)[NP]) {
    float2 acc = add2(A[0], B[0]);
#pragma unroll
    for (int j = 1; j < NP; j++) acc = add2(acc, add2(A[j], B[j]));
    return __fadd_rn(acc.x, acc.y);
}

// Smallest positive value of slots lo..hi of A (+inf bits when none).
__device__ __forceinline__ u32 min_positive_bits(const float2 (&A)[NP], bool edge, int lo, int hi) {
    u32 m = 0xFFFFFFFFu;
#pragma unroll
    for (int s = 0; s < NS - 1; s += 3) {
        u32 a = __float_as_uint(sxc(A, s)) - 1u;
        u32 b = s + 1 < NS - 1 ? __float_as_uint(sxc(A, s + 1)) - 1u : 0xFFFFFFFFu;
        u32 d = s + 2 < NS - 1 ? __float_as_uint(sxc(A, s + 2)) - 1u : 0xFFFFFFFFu;
        if (edge) {
            if (s < lo || s > hi) a = 0xFFFFFFFFu;
            if (s + 1 < lo || s + 1 > hi) b = 0xFFFFFFFFu;
            if (s + 2 < lo || s + 2 > hi) d = 0xFFFFFFFFu;
        }
        m = __vimin3_u32(m, a < b ? a : b, d);
    }
    return m + 1u;  // (0 when no positive value: 0xFFFFFFFF + 1)
}

__device__ __forceinline__ bool is_tiny(u32 min_bits, float scale) {
    return min_bits != 0u && __fmul_rn(__uint_as_float(min_bits), scale) < TINY;
}

__global__ void __launch_bounds__(SEG_THREADS, SEG_BLOCKS_PER_SM)
    k_baq_seg(DevBatch b, DevRef dref, BatchWork w, const u32 *list, const u32 *count, u32 *work_ctr,
              float4 *scratch, u32 max_q) {
    __shared__ float s_em[256], s_mis[256];
    extern __shared__ float4 s_seg[];  // forward rows of the current segment: SEG_K x 8 float4 per thread
    for (int q = threadIdx.x; q < 256; q += blockDim.x) {
        const double p = cs_qual2prob[q < MIN_BASE_QUAL ? MIN_BASE_QUAL : q];
        // calcEpsilon (device/baq.cu:361-372): 1 - p for a match, p * EM for a mismatch
        s_em[q] = float(1 - p);
        s_mis[q] = float(p * 0.33333333333);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const u32 gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u32 n_cp = (max_q + SEG_K - 1) / SEG_K + 1;
    float4 *cp_base = scratch + u64(gwarp) * n_cp * CP_VEC * 32 + lane;
    auto CP = [&](int cp, int v) -> float4 & { return cp_base[(u64(cp) * CP_VEC + v) * 32]; };
    auto SEG = [&](int r, int v) -> float4 & { return s_seg[(r * (2 * NS / 4) + v) * SEG_THREADS + threadIdx.x]; };
    const u32 n_list = *count;
    const float EI = 0.25f;
    const double GOP = cs_gap_open;
    const u64 REP = 0x1111111111111111ull;

    for (;;) {
        u32 base = 0;
        if (lane == 0) base = atomicAdd(work_ctr, 32u);
        base = __shfl_sync(FULL, base, 0);
        if (base >= n_list) break;
        const u32 li = base + lane;
        if (li >= n_list) continue;
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
        auto REF = [&](int k) -> u64 { return k >= 0 ? u64(contig_at(g, ref_off + u64(k))) : 0ull; };
        auto QRY = [&](int i) -> u32 { return sym4(b.reads, qsym + u64(i)); };
        auto QUL = [&](int i) -> u32 { return b.quals[qual0 + i]; };

        const double dsM = 1.0 / (2 * qL + 2);
        Coef c;
        {
            const float m0 = float((1 - GOP - GOP) * (1 - dsM)), m1 = float(GOP * (1 - dsM));
            const float m3 = float((1 - 0.1) * (1 - dsM)), m4 = float(0.1 * (1 - dsM));
            c.m0 = f2(m0, m0);
            c.m3 = f2(m3, m3);
            c.m6 = f2(float(1 - 0.1), float(1 - 0.1));
            c.m2 = f2(m1, m1);
            c.m8 = float(0.1);
            c.c1 = EI * m1;
            c.c4 = EI * m4;
        }
        const float bMs = float((1 - GOP) / bmLen), bIs = float(GOP / bmLen);
        // band slots of row i: cells k = s + i - bw in [max(1, i - bw), min(refLen, i + bw)]
        auto LO = [&](int i) { return 1 - (i - bw) > 0 ? 1 - (i - bw) : 0; };
        auto HI = [&](int i) { return refLen - (i - bw) < 2 * bw ? refLen - (i - bw) : 2 * bw; };
        auto EDGE = [&](int i) { return LO(i) != 0 || HI(i) != NS - 2; };
        // the row's emission constants (times `scale`) and window mismatch nibbles
        auto emis = [&](u64 wnd, u32 qsy, u32 ql, float scale, float &eqs, float &exs, u64 &nz) {
            if (qsy == IUPAC_N) {
                eqs = scale;
                exs = scale;
                nz = 0;
            } else {
                eqs = __fmul_rn(s_em[ql], scale);
                exs = __fmul_rn(s_mis[ql], scale);
                nz = nz_nibbles(wnd ^ (u64(qsy) * REP));
            }
        };
        bool under = false;
        u32 qmax = 0;

        // ---- forward ----
        float2 M[NP], I[NP], D[NP];
        u64 wf = 0;  // forward window of row i: nibble s = REF(s + i - bw - 1)
#pragma unroll
        for (int s = 0; s < NS; s++) wf |= REF(s - bw) << (4 * s);
        float sig;  // scale applied to the next row
        {
            const u32 q0 = QRY(0), ql0 = QUL(0);
            qmax = ql0;
            float eqs, exs;
            u64 nz;
            emis(wf, q0, ql0, 1.0f, eqs, exs, nz);
            const int lo = LO(1), hi = HI(1);
#pragma unroll
            for (int s = 0; s < NS; s++) {
                const bool in = s >= lo && s <= hi;
                sx(M, s) = in ? __fmul_rn(((nz >> (4 * s)) & 1) ? exs : eqs, bMs) : 0.0f;
                sx(I, s) = in ? __fmul_rn(EI, bIs) : 0.0f;
                sx(D, s) = 0.0f;
            }
            sig = pow2_scale(row_sum(M, I), 64, under);
            if (is_tiny(min_positive_bits(M, true, lo, hi), sig)) under = true;
            // checkpoint 0 = row 1
            CP(0, 0) = make_float4(M[0].x, M[0].y, M[1].x, M[1].y);
            CP(0, 1) = make_float4(M[2].x, M[2].y, M[3].x, M[3].y);
            CP(0, 2) = make_float4(M[4].x, M[4].y, M[5].x, M[5].y);
            CP(0, 3) = make_float4(M[6].x, M[6].y, M[7].x, M[7].y);
            CP(0, 4) = make_float4(I[0].x, I[0].y, I[1].x, I[1].y);
            CP(0, 5) = make_float4(I[2].x, I[2].y, I[3].x, I[3].y);
            CP(0, 6) = make_float4(I[4].x, I[4].y, I[5].x, I[5].y);
            CP(0, 7) = make_float4(I[6].x, I[6].y, I[7].x, I[7].y);
            CP(0, 8) = make_float4(sig, __uint_as_float(u32(wf)), __uint_as_float(u32(wf >> 32)), 0.0f);
        }
        for (int i = 2; i <= qL; i++) {
            wf = (wf >> 4) | (REF(i + NS - 2 - bw) << 60);
            const u32 qs = QRY(i - 1), ql = QUL(i - 1);
            qmax = qmax > ql ? qmax : ql;
            float eqs, exs;
            u64 nz;
            emis(wf, qs, ql, sig, eqs, exs, nz);
            const int lo = LO(i), hi = HI(i);
            const bool edge = EDGE(i);
            fwd_row(M, I, D, c, sig, eqs, exs, nz, edge, lo, hi);
            sig = pow2_scale(row_sum(M, I), 64, under);
            if (is_tiny(min_positive_bits(M, edge, lo, hi), sig)) under = true;
            if ((i - 1) % SEG_K == 0) {
                const int cp = (i - 1) / SEG_K;
                CP(cp, 0) = make_float4(M[0].x, M[0].y, M[1].x, M[1].y);
                CP(cp, 1) = make_float4(M[2].x, M[2].y, M[3].x, M[3].y);
                CP(cp, 2) = make_float4(M[4].x, M[4].y, M[5].x, M[5].y);
                CP(cp, 3) = make_float4(M[6].x, M[6].y, M[7].x, M[7].y);
                CP(cp, 4) = make_float4(I[0].x, I[0].y, I[1].x, I[1].y);
                CP(cp, 5) = make_float4(I[2].x, I[2].y, I[3].x, I[3].y);
                CP(cp, 6) = make_float4(I[4].x, I[4].y, I[5].x, I[5].y);
                CP(cp, 7) = make_float4(I[6].x, I[6].y, I[7].x, I[7].y);
                CP(cp, 8) = make_float4(sig, __uint_as_float(u32(wf)), __uint_as_float(u32(wf >> 32)), 0.0f);
            }
        }

        // ---- backward fused with MAP, segment by segment from the last ----
        // certified FP32 bounds (see the file comment)
        const float u = 5.9604644775390625e-8f;
        const float eps = float((7.0 * qL + 2.0 * refLen + 8.0) * 5.9604644775390625e-8);
        const float eps_z = 2.0f * eps + u;
        const float rel = 2.0f * (eps_z + 2.0f * (2 * BW + 1) * u) + u;
        const float rel_state = 2.0f * eps_z + 2.0f * u;
        const float dt = 4.343f * rel / (1.0f - rel) + 1e-4f;
        float2 bM[NP], bI[NP];
        float tau = 1.0f;  // scale of the next (lower) backward row
        u64 wb = 0;        // backward window of row i: nibble s = REF(s + i - bw)
        const int n_seg = (qL - 1) / SEG_K + 1;
        for (int sg = n_seg - 1; sg >= 0; sg--) {
            const int r0 = 1 + sg * SEG_K;
            const int r1 = r0 + SEG_K - 1 < qL ? r0 + SEG_K - 1 : qL;
            // recompute the segment's forward rows into shared memory
            {
                float4 v;
                v = CP(sg, 0); M[0] = f2(v.x, v.y); M[1] = f2(v.z, v.w);
                v = CP(sg, 1); M[2] = f2(v.x, v.y); M[3] = f2(v.z, v.w);
                v = CP(sg, 2); M[4] = f2(v.x, v.y); M[5] = f2(v.z, v.w);
                v = CP(sg, 3); M[6] = f2(v.x, v.y); M[7] = f2(v.z, v.w);
                v = CP(sg, 4); I[0] = f2(v.x, v.y); I[1] = f2(v.z, v.w);
                v = CP(sg, 5); I[2] = f2(v.x, v.y); I[3] = f2(v.z, v.w);
                v = CP(sg, 6); I[4] = f2(v.x, v.y); I[5] = f2(v.z, v.w);
                v = CP(sg, 7); I[6] = f2(v.x, v.y); I[7] = f2(v.z, v.w);
                v = CP(sg, 8);
                float rs = v.x;
                u64 rw = u64(__float_as_uint(v.y)) | (u64(__float_as_uint(v.z)) << 32);
                if (r0 == 1) {
#pragma unroll
                    for (int j = 0; j < NP; j++) D[j] = f2(0.0f, 0.0f);
                } else {
                    d_from_m(M, D, c, HI(r0), EDGE(r0));
                }
#pragma unroll
                for (int j = 0; j < NP; j += 2) {
                    SEG(0, j / 2) = make_float4(M[j].x, M[j].y, M[j + 1].x, M[j + 1].y);
                    SEG(0, 4 + j / 2) = make_float4(I[j].x, I[j].y, I[j + 1].x, I[j + 1].y);
                }
                for (int i = r0 + 1; i <= r1; i++) {
                    rw = (rw >> 4) | (REF(i + NS - 2 - bw) << 60);
                    const u32 qs = QRY(i - 1), ql = QUL(i - 1);
                    float eqs, exs;
                    u64 nz;
                    emis(rw, qs, ql, rs, eqs, exs, nz);
                    const int lo = LO(i), hi = HI(i);
                    fwd_row(M, I, D, c, rs, eqs, exs, nz, EDGE(i), lo, hi);
                    bool dummy = false;
                    rs = pow2_scale(row_sum(M, I), 64, dummy);
#pragma unroll
                    for (int j = 0; j < NP; j += 2) {
                        SEG(i - r0, j / 2) = make_float4(M[j].x, M[j].y, M[j + 1].x, M[j + 1].y);
                        SEG(i - r0, 4 + j / 2) = make_float4(I[j].x, I[j].y, I[j + 1].x, I[j + 1].y);
                    }
                }
            }
            for (int i = r1; i >= r0; i--) {
                const int lo = LO(i), hi = HI(i);
                const bool edge = EDGE(i);
                if (i == qL) {
                    // B(qL, k) = sM / s(qL) / sLast for every band cell: one constant (only ratios are used)
#pragma unroll
                    for (int s = 0; s < NS; s++) {
                        const bool in = s >= lo && s <= hi;
                        sx(bM, s) = in ? 1.0f : 0.0f;
                        sx(bI, s) = in ? 1.0f : 0.0f;
                    }
#pragma unroll
                    for (int s = 0; s < NS; s++) wb |= REF(s + qL - bw) << (4 * s);
                } else {
                    // row i from row i + 1: the emission of cell (i + 1, k + 1) uses REF(k) and query base i
                    wb = (wb << 4) | REF(i - bw);
                    const u32 qs = QRY(i), ql = QUL(i);
                    float eqs, exs;
                    u64 nz;
                    emis(wb, qs, ql, tau, eqs, exs, nz);
                    const float c1 = c.c1 * tau, c4 = c.c4 * tau;
                    float2 A[NP], Bv[NP], Cv[NP];
#pragma unroll
                    for (int j = 0; j < NP; j++) {
                        const float2 e = f2(((nz >> (8 * j)) & 1) ? exs : eqs, ((nz >> (8 * j + 4)) & 1) ? exs : eqs);
                        const float2 E = mul2(e, bM[j]);  // B_M(i + 1, k + 1) is slot s of row i + 1
                        A[j] = mul2(E, c.m0);
                        Bv[j] = mul2(E, c.m3);
                        Cv[j] = mul2(E, c.m6);
                    }
                    float nbm[NS], nbi[NS];
                    float dn = 0.0f;  // B_D(i, k + 1)
                    const bool y = i > 1;
#pragma unroll
                    for (int s = NS - 2; s >= 0; s--) {
                        const float bi1 = s >= 1 ? sxc(bI, s - 1) : 0.0f;  // B_I(i + 1, k)
                        nbm[s] = __fmaf_rn(c.m2.x, dn, __fmaf_rn(c1, bi1, sxc(A, s)));
                        nbi[s] = __fmaf_rn(c4, bi1, sxc(Bv, s));
                        dn = y ? __fmaf_rn(c.m8, dn, sxc(Cv, s)) : 0.0f;
                    }
                    nbm[NS - 1] = 0.0f;
                    nbi[NS - 1] = 0.0f;
#pragma unroll
                    for (int s = 0; s < NS; s++) {
                        const bool in = !edge || (s >= lo && s <= hi);
                        sx(bM, s) = in ? nbm[s] : 0.0f;
                        sx(bI, s) = in ? nbi[s] : 0.0f;
                    }
                }
                tau = pow2_scale(row_sum(bM, bI), 32, under);
                if (i < qL) {
                    // the cells of column refLen (no emission; they only feed a diagonal neighbour, scaled by
                    // their own tiny value) may decay: the guard covers k < refLen
                    const int last_ok = refLen - 1 - (i - bw);
                    if (is_tiny(min_positive_bits(bM, true, lo, hi < last_ok ? hi : last_ok), tau)) under = true;
                }

                // ---- MAP for row i (device/baq.cu:619-681): first maximum in (k, M before I) order ----
                float2 fM[NP], fI[NP];
#pragma unroll
                for (int j = 0; j < NP; j += 2) {
                    const float4 a = SEG(i - r0, j / 2), q4 = SEG(i - r0, 4 + j / 2);
                    fM[j] = f2(a.x, a.y);
                    fM[j + 1] = f2(a.z, a.w);
                    fI[j] = f2(q4.x, q4.y);
                    fI[j + 1] = f2(q4.z, q4.w);
                }
                // two streams (M terms, I terms), each with its first maximum and the sum of its other terms
                u32 mxM = 0, mxI = 0;
                int iM = -1, iI = -1;
                float2 ex2 = f2(0.0f, 0.0f);
#pragma unroll
                for (int j = 0; j < NP; j++) {
                    const float2 zM = mul2(fM[j], bM[j]), zI = mul2(fI[j], bI[j]);
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int s = 2 * j + h;
                        if (s >= NS - 1) continue;
                        const float zm = h ? zM.y : zM.x, zi = h ? zI.y : zI.x;
                        ex2 = add2(ex2, f2(fminf(zm, __uint_as_float(mxM)), fminf(zi, __uint_as_float(mxI))));
                        bool pm, pi;
                        mxM = __vibmax_u32(mxM, __float_as_uint(zm), &pm);
                        mxI = __vibmax_u32(mxI, __float_as_uint(zi), &pi);
                        iM = pm ? iM : s;
                        iI = pi ? iI : s;
                    }
                }
                const float fmM = __uint_as_float(mxM), fmI = __uint_as_float(mxI);
                // the earlier of two equal maxima: an M term at slot a precedes an I term at slot b when a <= b
                const bool m_wins = mxM > mxI || (mxM == mxI && iM >= 0 && (iI < 0 || iM <= iI));
                const float mx = m_wins ? fmM : fmI;
                const int win_s = m_wins ? iM : iI;
                const float excl = __fadd_rn(__fadd_rn(ex2.x, ex2.y), fminf(fmM, fmI));
                const float sum = __fadd_rn(excl, mx);
                const u32 qi = qual0 + u32(i - 1);
                const int qo = int(QUL(i - 1));
                u8 amb = 0;
                int qv = MIN_BASE_QUAL;
                u32 state = U32_NONE;
                float tq_trace = __int_as_float(0x7fc00000), lo_trace = 0.0f, hi_trace = 0.0f;
                if (!(sum > 0.0f) || !(sum <= 3.0e38f) || win_s < 0) {
                    amb = 7;
                } else {
                    state = u32(((win_s + i - bw - 1) << 2) | (m_wins ? 0 : 1));
                    const float thr = mx * (1.0f - rel_state);
                    if (excl >= thr) {
                        // a rival may be within the bound: the terms other than the maximum at or above it
                        int rivals = 0;
                        u32 alt = 0;
#pragma unroll
                        for (int j = 0; j < NP; j++) {
                            const float2 zM = mul2(fM[j], bM[j]), zI = mul2(fI[j], bI[j]);
#pragma unroll
                            for (int h = 0; h < 2; h++) {
                                const int s = 2 * j + h;
                                if (s >= NS - 1) continue;
#pragma unroll
                                for (int st = 0; st < 2; st++) {
                                    const float z = st == 0 ? (h ? zM.y : zM.x) : (h ? zI.y : zI.x);
                                    const bool is_max = s == win_s && st == (m_wins ? 0 : 1);
                                    if (!is_max && z >= thr && s >= lo && s <= hi) {
                                        if (!rivals) alt = u32(((s + i - bw - 1) << 2) | st);
                                        rivals++;
                                    }
                                }
                            }
                        }
                        if (rivals) {
                            amb |= 2;
                            if (rivals == 1) w.baq_alt[qi] = u16(alt);
                            else amb |= 4;
                        }
                    }
                    const float ratio = excl / sum;
                    const float tq = ratio > 0.f ? -4.343f * logf(ratio) + 0.499f : __int_as_float(0x7f800000);
                    const float tlo = tq - dt, thi = tq + dt;
                    auto capped = [&](float tt) {
                        int k;
                        if (!(tt == tt)) k = 0;
                        else if (tt >= 2147483520.0f) k = 2147483647;
                        else k = int(floorf(tt));
                        return k > 100 ? 99 : (k < MIN_BASE_QUAL ? MIN_BASE_QUAL : k);
                    };
                    qv = capped(tq);
                    tq_trace = tq;
                    lo_trace = tlo;
                    hi_trace = thi;
                    const int flo = capped(tlo), fhi = capped(thi);
                    if (qo <= 99) {
                        if ((flo < qo ? flo : qo) != (fhi < qo ? fhi : qo)) amb |= 1;
                    } else if (!(thi < 100.f && flo == fhi) && !(tlo >= 101.5f)) {
                        amb |= 1;
                    }
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
        if (under || qmax > 93) {
            for (int i = 0; i < qL; i++) w.baq_amb[qual0 + i] = 7;
            if (w.trace32)
                for (int i = 0; i < qL; i++) w.trace32[3 * size_t(qual0 + i)] = __int_as_float(0x7fc00000);
        }
    }
}

}  // namespace

void baq_seg_set_constants(const HmmConst &c) {
    cudaMemcpyToSymbol(cs_qual2prob, c.qual2prob, sizeof(c.qual2prob));
    cudaMemcpyToSymbol(cs_gap_open, &c.gap_open, sizeof(double));
}

u64 baq_seg_scratch_bytes(u32 max_q) {
    const u64 n_cp = (u64(max_q) + SEG_K - 1) / SEG_K + 1;
    return n_cp * CP_VEC * 32 * sizeof(float4) * (u64(152) * SEG_BLOCKS_PER_SM * (SEG_THREADS / 32));
}

void launch_baq_seg(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                    u32 max_reads, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q, cudaStream_t s) {
    if (!max_reads) return;
    const u64 n_cp = (u64(max_q) + SEG_K - 1) / SEG_K + 1;
    const u64 per_warp = n_cp * CP_VEC * 32 * sizeof(float4);
    u64 blocks = scratch_bytes / per_warp / (SEG_THREADS / 32);
    const u64 need = (u64(max_reads) + SEG_THREADS - 1) / SEG_THREADS;
    if (blocks > need) blocks = need;
    if (blocks > u64(152) * SEG_BLOCKS_PER_SM) blocks = u64(152) * SEG_BLOCKS_PER_SM;
    if (blocks == 0) return;
    constexpr int smem = SEG_K * (2 * NS / 4) * SEG_THREADS * int(sizeof(float4));
    static bool attr_set[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr_set[dev]) {
        cudaFuncSetAttribute(k_baq_seg, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr_set[dev] = true;
    }
    cudaMemsetAsync(ctr, 0, sizeof(u32), s);
    k_baq_seg<<<u32(blocks), SEG_THREADS, smem, s>>>(b, ref, w, list, count, ctr, reinterpret_cast<float4 *>(scratch),
                                                     max_q);
    g_kernel_launches++;
}

}  // namespace fpg
