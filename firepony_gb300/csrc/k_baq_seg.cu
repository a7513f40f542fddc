// K2, band class 0 (bandwidth <= 7, the bulk of BAQ reads): the banded glocal HMM of device/baq.cu:214-697 in
// FP32 with certified decisions, one thread per read, the band row in registers.
//
// Layout and arithmetic:
//   * Slots. Row i holds cells k = s + i - bw for slots s = 0..15 (15 band slots and one that stays zero), also
//     for the first rows, where some slots fall left of the reference (k < 1): every row slides by one cell, so
//     M(i,k) reads slot s of row i-1, I(i,k) slot s+1 of row i-1 and D(i,k) slot s-1 of row i, with no special
//     case for the growing band. Rows whose band is clipped (k < 1 or k > refLen) zero their outside slots;
//     interior rows run a copy of the row code without any of that masking.
//   * Packed pairs. Slots are held as float2 pairs, and every update whose operands are slot-aligned (the M
//     recurrence, the emission products, the row sums, the MAP products) runs as one two-lane FP32 operation
//     (__fmul2_rn / __ffma2_rn / __fadd2_rn: each lane rounds as the scalar operation would).
//   * Scaling. Each row is scaled by a power of two chosen from the previous row's M + I sum (forward: into
//     [2^64, 2^65), backward: [2^32, 2^33)); the factor is folded into the row's emission values and gap
//     coefficients, so it costs no operation per cell and no rounding. The MAP step only uses ratios within a
//     row, where every row factor cancels.
//   * Emissions. The reference window is a 64-bit register of four 16-bit one-hot masks (A, C, G, T present at
//     slot s) that slides with the band; the query base selects one of them as the row's 16 match bits, and each
//     slot selects its match or mismatch value. Reads whose window holds a reference N go to the general kernel
//     (k_prep assigns them band class 1), so no slot needs the N case here. The emission of cell (i + 1, k + 1)
//     that the backward row i needs is the forward row i + 1's emission at the same slot, so the backward pass
//     reuses the forward rows' match bits and qualities and loads nothing.
//   * Memory. The forward pass keeps every SEG_K-th row (M, I, its scale, window, match bits, quality) in HBM
//     scratch. The backward pass walks the segments from the last: it recomputes a segment's forward rows from its
//     checkpoint into shared memory (the same instructions, so the same values) and runs the backward rows and the
//     MAP step of the segment against them. Scratch traffic falls to 40 words per SEG_K rows from 30 per row.
//     Query symbols, qualities and reference symbols are read as whole words one word ahead of use.
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
constexpr int CP_VEC = 9;         // checkpoint float4s: M[16], I[16], scale, window (2 words), meta
constexpr int SEG_VEC = 8;        // shared row float4s: M[0..14] + meta in slot 15, I[16]
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

// One-hot lane of a 4-bit IUPAC symbol: A, C, G, T -> 0..3; other symbols -> none
__device__ __forceinline__ int base_lane(u32 sym) {
    return sym == IUPAC_A ? 0 : sym == IUPAC_C ? 1 : sym == IUPAC_G ? 2 : sym == IUPAC_T ? 3 : -1;
}
// window register: bit 16 * lane + s set when slot s holds that base; pushing slides the band by one cell and
// enters the new slot 15
__device__ __forceinline__ u64 window_push(u64 wnd, u32 sym) {
    wnd = (wnd >> 1) & 0x7FFF7FFF7FFF7FFFull;
    const int l = base_lane(sym);
    return l >= 0 ? wnd | (1ull << (16 * l + 15)) : wnd;
}
__device__ __forceinline__ u32 match_bits(u64 wnd, u32 qsym) {
    const int l = base_lane(qsym);
    return l >= 0 ? u32(wnd >> (16 * l)) & 0xFFFFu : 0u;
}

// Successive 4-bit symbols of a packed word array from a start index upward, one word ahead in flight;
// symbols at or past `limit` read as 0.
struct Sym4Up {
    const u32 *w;
    u64 nwords, limit, idx;
    u32 cur, nxt;
    __device__ __forceinline__ void init(const u32 *words, u64 n_words, u64 lim, u64 i0) {
        w = words;
        nwords = n_words;
        limit = lim;
        idx = i0;
        const u64 k = i0 >> 3;
        cur = k < nwords ? w[k] : 0u;
        nxt = k + 1 < nwords ? w[k + 1] : 0u;
    }
    __device__ __forceinline__ u32 next() {
        const u32 s = idx < limit ? (cur >> (4 * (idx & 7))) & 0xFu : 0u;
        idx++;
        if ((idx & 7) == 0) {
            cur = nxt;
            const u64 k = (idx >> 3) + 1;
            nxt = k < nwords ? w[k] : 0u;
        }
        return s;
    }
};

// Successive bytes of [base, base + n) from a start offset upward, read as aligned 32-bit words one word ahead;
// a word that is not wholly inside the array is assembled from its bytes that are.
struct ByteUp {
    const u8 *base;
    u64 n, idx;
    u32 cur, nxt;
    __device__ __forceinline__ u32 word_at(uintptr_t a) const {
        const uintptr_t lo = uintptr_t(base), hi = lo + n;
        if (a >= lo && a + 4 <= hi) return *reinterpret_cast<const u32 *>(a);
        u32 v = 0;
        for (int k = 0; k < 4; k++)
            if (a + k >= lo && a + k < hi) v |= u32(*reinterpret_cast<const u8 *>(a + k)) << (8 * k);
        return v;
    }
    __device__ __forceinline__ void init(const u8 *b, u64 size, u64 i0) {
        base = b;
        n = size;
        idx = i0;
        const uintptr_t a = (uintptr_t(b) + i0) & ~uintptr_t(3);
        cur = word_at(a);
        nxt = word_at(a + 4);
    }
    __device__ __forceinline__ u32 next() {
        const uintptr_t p = uintptr_t(base) + idx;
        const u32 v = (cur >> (8 * (p & 3))) & 0xFFu;
        idx++;
        if (((p + 1) & 3) == 0) {
            cur = nxt;
            nxt = word_at(p + 1 + 4);
        }
        return v;
    }
};

// Per-read constants.
struct Coef {
    float2 m0, m3, m6, m2;  // transition pairs
    float m8, c1, c4;       // D extension, EI * m1, EI * m4 (EI = 0.25: exact products)
};

__device__ __forceinline__ float2 emis_pair(u32 m16, int j, float eqs, float exs) {
    return f2(((m16 >> (2 * j)) & 1u) ? eqs : exs, ((m16 >> (2 * j + 1)) & 1u) ? eqs : exs);
}

// One forward row (i >= 2) from row i-1 in place. eqs/exs: the row's match/mismatch emission times sig, the
// previous row's scale; m16: the row's match bits; [lo, hi]: band slots (EDGE: zero the others).
template <bool EDGE>
__device__ __forceinline__ void fwd_row(float2 (&M)[NP], float2 (&I)[NP], float2 (&D)[NP], const Coef &c, float sig,
                                        float eqs, float exs, u32 m16, int lo, int hi) {
    const float c1 = __fmul_rn(c.c1, sig), c4 = __fmul_rn(c.c4, sig);
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
        M[j] = mul2(emis_pair(m16, j, eqs, exs), t);
        I[j] = f2(nI[2 * j], nI[2 * j + 1]);
    }
    if constexpr (EDGE) {
#pragma unroll
        for (int s = 0; s < NS; s++) {
            const bool in = s >= lo && s <= hi;
            sx(M, s) = in ? sxc(M, s) : 0.0f;
            sx(I, s) = in ? sxc(I, s) : 0.0f;
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
        sx(D, s) = (EDGE && s > hi) ? 0.0f : d;
    }
    sx(D, NS - 1) = 0.0f;
}

// D of a forward row from its M (a checkpointed row): the chain of fwd_row.
template <bool EDGE>
__device__ __forceinline__ void d_from_m(const float2 (&M)[NP], float2 (&D)[NP], const Coef &c, int hi) {
    float2 P[NP];
#pragma unroll
    for (int j = 0; j < NP; j++) P[j] = mul2(c.m2, M[j]);
    float d = 0.0f;
    sx(D, 0) = 0.0f;
#pragma unroll
    for (int s = 1; s < NS - 1; s++) {
        d = __fmaf_rn(c.m8, d, sxc(P, s - 1));
        sx(D, s) = (EDGE && s > hi) ? 0.0f : d;
    }
    sx(D, NS - 1) = 0.0f;
}

// One backward row i (< qL) from row i + 1 in place. eqs/exs/m16: the emission of cells (i + 1, k + 1), i.e. the
// forward row i + 1's match bits and quality, times tau, the row i + 1 scale. FIRST: row 1 (no D states).
template <bool EDGE, bool FIRST>
__device__ __forceinline__ void bwd_row(float2 (&bM)[NP], float2 (&bI)[NP], const Coef &c, float tau, float eqs,
                                        float exs, u32 m16, int lo, int hi) {
    const float c1 = __fmul_rn(c.c1, tau), c4 = __fmul_rn(c.c4, tau);
    float2 A[NP], Bv[NP], Cv[NP];
#pragma unroll
    for (int j = 0; j < NP; j++) {
        const float2 E = mul2(emis_pair(m16, j, eqs, exs), bM[j]);  // B_M(i + 1, k + 1) is slot s of row i + 1
        A[j] = mul2(E, c.m0);
        Bv[j] = mul2(E, c.m3);
        Cv[j] = mul2(E, c.m6);
    }
    float nbm[NS], nbi[NS];
    float dn = 0.0f;  // B_D(i, k + 1)
#pragma unroll
    for (int s = NS - 2; s >= 0; s--) {
        const float bi1 = s >= 1 ? sxc(bI, s - 1) : 0.0f;  // B_I(i + 1, k)
        if constexpr (FIRST) {
            nbm[s] = __fmaf_rn(c1, bi1, sxc(A, s));
        } else {
            nbm[s] = __fmaf_rn(c.m2.x, dn, __fmaf_rn(c1, bi1, sxc(A, s)));
            dn = __fmaf_rn(c.m8, dn, sxc(Cv, s));
        }
        nbi[s] = __fmaf_rn(c4, bi1, sxc(Bv, s));
    }
    nbm[NS - 1] = 0.0f;
    nbi[NS - 1] = 0.0f;
#pragma unroll
    for (int s = 0; s < NS; s++) {
        const bool in = !EDGE || (s >= lo && s <= hi);
        sx(bM, s) = in ? nbm[s] : 0.0f;
        sx(bI, s) = in ? nbi[s] : 0.0f;
    }
}

// Sum of A + B over the row (the scale input).
__device__ __forceinline__ float row_sum(const float2 (&A)[NP], const float2 (&B)[NP]) {
    float2 acc = add2(A[0], B[0]);
#pragma unroll
    for (int j = 1; j < NP; j++) acc = add2(acc, add2(A[j], B[j]));
    return __fadd_rn(acc.x, acc.y);
}

// Smallest positive value among slots lo..hi of A, as float bits (0 when none).
__device__ __forceinline__ u32 min_positive_bits(const float2 (&A)[NP], int lo, int hi) {
    u32 m = 0xFFFFFFFFu;
#pragma unroll
    for (int s = 0; s < NS - 1; s++) {
        const u32 v = __float_as_uint(sxc(A, s)) - 1u;  // 0 -> 0xFFFFFFFF: zeros never count
        m = (s >= lo && s <= hi) ? (v < m ? v : m) : m;
    }
    return m + 1u;
}
// Smallest value of slots 0..14 (an interior row: every slot in band), as float bits.
__device__ __forceinline__ u32 min_bits15(const float2 (&A)[NP]) {
    u32 m = __vimin3_u32(__float_as_uint(A[0].x), __float_as_uint(A[0].y), __float_as_uint(A[1].x));
    m = __vimin3_u32(m, __float_as_uint(A[1].y), __float_as_uint(A[2].x));
    m = __vimin3_u32(m, __float_as_uint(A[2].y), __float_as_uint(A[3].x));
    m = __vimin3_u32(m, __float_as_uint(A[3].y), __float_as_uint(A[4].x));
    m = __vimin3_u32(m, __float_as_uint(A[4].y), __float_as_uint(A[5].x));
    m = __vimin3_u32(m, __float_as_uint(A[5].y), __float_as_uint(A[6].x));
    m = __vimin3_u32(m, __float_as_uint(A[6].y), __float_as_uint(A[7].x));
    return m;
}

__device__ __forceinline__ bool is_tiny(u32 min_bits, float scale) {
    return min_bits != 0u && __fmul_rn(__uint_as_float(min_bits), scale) < TINY;
}

__device__ __forceinline__ void store_cp(float4 *cp, const float2 (&M)[NP], const float2 (&I)[NP], float sg, u64 wnd,
                                         u32 meta) {
    cp[0 * 32] = make_float4(M[0].x, M[0].y, M[1].x, M[1].y);
    cp[1 * 32] = make_float4(M[2].x, M[2].y, M[3].x, M[3].y);
    cp[2 * 32] = make_float4(M[4].x, M[4].y, M[5].x, M[5].y);
    cp[3 * 32] = make_float4(M[6].x, M[6].y, M[7].x, M[7].y);
    cp[4 * 32] = make_float4(I[0].x, I[0].y, I[1].x, I[1].y);
    cp[5 * 32] = make_float4(I[2].x, I[2].y, I[3].x, I[3].y);
    cp[6 * 32] = make_float4(I[4].x, I[4].y, I[5].x, I[5].y);
    cp[7 * 32] = make_float4(I[6].x, I[6].y, I[7].x, I[7].y);
    cp[8 * 32] = make_float4(sg, __uint_as_float(u32(wnd)), __uint_as_float(u32(wnd >> 32)), __uint_as_float(meta));
}

__global__ void __launch_bounds__(SEG_THREADS, SEG_BLOCKS_PER_SM)
    k_baq_seg(DevBatch b, DevRef dref, BatchWork w, const u32 *list, const u32 *count, u32 *work_ctr,
              float4 *scratch, u32 max_q) {
    __shared__ float s_em[256], s_mis[256];
    extern __shared__ float4 s_seg[];  // forward rows of the current segment: SEG_K x SEG_VEC float4 per thread
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
    auto CP = [&](int cp) -> float4 * { return cp_base + u64(cp) * CP_VEC * 32; };
    auto SEG = [&](int r, int v) -> float4 & { return s_seg[(r * SEG_VEC + v) * SEG_THREADS + threadIdx.x]; };
    const u32 n_list = *count;
    const float EI = 0.25f;
    const double GOP = cs_gap_open;
    const u64 read_words = (b.num_syms + 7) >> 3;

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
        const u64 contig_words = (g.size + 7) >> 3;
        const u64 qsym = u64(b.read_start[r]) + qx;
        const u32 qual0 = b.qual_start[r] + qx;

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
        // band slots of row i: cells k = s + i - bw in [max(1, i - bw), min(refLen, i + bw)]; interior rows
        // (bw = 7, 8 <= i <= refLen - 7) have every slot 0..14 in band
        auto LO = [&](int i) { return 1 - (i - bw) > 0 ? 1 - (i - bw) : 0; };
        auto HI = [&](int i) { return refLen - (i - bw) < 2 * bw ? refLen - (i - bw) : 2 * bw; };
        auto EDGE = [&](int i) { return bw != BW || i <= BW || i > refLen - BW; };
        // the row's emission values (times `scale`): a query N gives 1 for every slot
        auto emis = [&](u32 qsy, u32 ql, float scale, float &eqs, float &exs) {
            if (qsy == IUPAC_N) {
                eqs = scale;
                exs = scale;
            } else {
                eqs = __fmul_rn(s_em[ql], scale);
                exs = __fmul_rn(s_mis[ql], scale);
            }
        };
        bool under = false;
        u32 qmax = 0;

        // certified FP32 bounds (see the file comment)
        const float u = 5.9604644775390625e-8f;
        const float eps = float((7.0 * qL + 2.0 * refLen + 8.0) * 5.9604644775390625e-8);
        const float eps_z = 2.0f * eps + u;
        const float rel = 2.0f * (eps_z + 2.0f * (2 * BW + 1) * u) + u;
        const float rel_state = 2.0f * eps_z + 2.0f * u;
        const float dt = 4.343f * rel / (1.0f - rel) + 1e-4f;

        float2 M[NP], I[NP], D[NP], bM[NP], bI[NP];
        float tau = 1.0f;   // scale of the next (lower) backward row
        u32 up_meta = 0;    // match bits | quality << 16 | query symbol << 24 of the forward row above
        const int n_seg = (qL - 1) / SEG_K + 1;
        // phase n_seg: the forward pass over the whole read (checkpoints every SEG_K rows); phases n_seg - 1..0:
        // the segments from the last, each recomputed forward and then run backward with the MAP step
        for (int ph = n_seg; ph >= 0; ph--) {
            const bool fwd_pass = ph == n_seg;
            const int r0 = fwd_pass ? 1 : 1 + ph * SEG_K;
            const int r1 = fwd_pass ? qL : (r0 + SEG_K - 1 < qL ? r0 + SEG_K - 1 : qL);
            u64 wnd;   // window of the current forward row: bit 16 * base + s for slot s (cell s + i - bw)
            float sg;  // scale of the current forward row (applied to the next one)
            u32 meta;  // the current forward row's match bits | quality << 16 | query symbol << 24
            if (fwd_pass) {
                // row 1: cells 1..min(refLen, bw + 1)
                wnd = 0;
#pragma unroll
                for (int s = 0; s < NS; s++) {
                    const int k = s - bw;  // REF(s + 1 - bw - 1)
                    const u32 sym = k >= 0 ? contig_at(g, ref_off + u64(k)) : 0u;
                    const int l = base_lane(sym);
                    if (l >= 0) wnd |= 1ull << (16 * l + s);
                }
                const u32 q0 = sym4(b.reads, qsym), ql0 = b.quals[qual0];
                qmax = ql0;
                float eqs, exs;
                emis(q0, ql0, 1.0f, eqs, exs);
                const u32 m16 = q0 == IUPAC_N ? 0xFFFFu : match_bits(wnd, q0);
                const int lo = LO(1), hi = HI(1);
#pragma unroll
                for (int s = 0; s < NS; s++) {
                    const bool in = s >= lo && s <= hi;
                    sx(M, s) = in ? __fmul_rn(((m16 >> s) & 1u) ? eqs : exs, bMs) : 0.0f;
                    sx(I, s) = in ? __fmul_rn(EI, bIs) : 0.0f;
                    sx(D, s) = 0.0f;
                }
                sg = pow2_scale(row_sum(M, I), 64, under);
                if (is_tiny(min_positive_bits(M, lo, hi), sg)) under = true;
                meta = m16 | (ql0 << 16) | (q0 << 24);
                store_cp(CP(0), M, I, sg, wnd, meta);
            } else {
                const float4 *cp = CP(ph);
                float4 v;
                v = cp[0 * 32]; M[0] = f2(v.x, v.y); M[1] = f2(v.z, v.w);
                v = cp[1 * 32]; M[2] = f2(v.x, v.y); M[3] = f2(v.z, v.w);
                v = cp[2 * 32]; M[4] = f2(v.x, v.y); M[5] = f2(v.z, v.w);
                v = cp[3 * 32]; M[6] = f2(v.x, v.y); M[7] = f2(v.z, v.w);
                v = cp[4 * 32]; I[0] = f2(v.x, v.y); I[1] = f2(v.z, v.w);
                v = cp[5 * 32]; I[2] = f2(v.x, v.y); I[3] = f2(v.z, v.w);
                v = cp[6 * 32]; I[4] = f2(v.x, v.y); I[5] = f2(v.z, v.w);
                v = cp[7 * 32]; I[6] = f2(v.x, v.y); I[7] = f2(v.z, v.w);
                v = cp[8 * 32];
                sg = v.x;
                wnd = u64(__float_as_uint(v.y)) | (u64(__float_as_uint(v.z)) << 32);
                meta = __float_as_uint(v.w);
                if (r0 == 1) {
#pragma unroll
                    for (int j = 0; j < NP; j++) D[j] = f2(0.0f, 0.0f);
                } else if (EDGE(r0)) {
                    d_from_m<true>(M, D, c, HI(r0));
                } else {
                    d_from_m<false>(M, D, c, HI(r0));
                }
#pragma unroll
                for (int j = 0; j < NP; j += 2) {
                    SEG(0, j / 2) = make_float4(M[j].x, M[j].y, M[j + 1].x,
                                                j + 1 == NP - 1 ? __uint_as_float(meta) : M[j + 1].y);
                    SEG(0, 4 + j / 2) = make_float4(I[j].x, I[j].y, I[j + 1].x, I[j + 1].y);
                }
            }
            // forward rows r0 + 1 .. r1 (query base i - 1, quality i - 1, reference symbol of slot 15)
            Sym4Up qs_in, ref_in;
            ByteUp ql_in;
            qs_in.init(b.reads, read_words, b.num_syms, qsym + u64(r0));
            ql_in.init(b.quals, b.num_quals, u64(qual0) + u64(r0));
            ref_in.init(g.words, contig_words, g.size, ref_off + u64(r0 + NS - 1 - bw));
            for (int i = r0 + 1; i <= r1; i++) {
                wnd = window_push(wnd, ref_in.next());
                const u32 qs = qs_in.next(), ql = ql_in.next();
                float eqs, exs;
                emis(qs, ql, sg, eqs, exs);
                const u32 m16 = qs == IUPAC_N ? 0xFFFFu : match_bits(wnd, qs);
                const int lo = LO(i), hi = HI(i);
                const bool edge = EDGE(i);
                if (edge) fwd_row<true>(M, I, D, c, sg, eqs, exs, m16, lo, hi);
                else fwd_row<false>(M, I, D, c, sg, eqs, exs, m16, lo, hi);
                bool bad = false;
                sg = pow2_scale(row_sum(M, I), 64, bad);
                meta = m16 | (ql << 16) | (qs << 24);
                if (fwd_pass) {
                    qmax = qmax > ql ? qmax : ql;
                    under |= bad;
                    if (is_tiny(edge ? min_positive_bits(M, lo, hi) : min_bits15(M), sg)) under = true;
                    if ((i - 1) % SEG_K == 0) store_cp(CP((i - 1) / SEG_K), M, I, sg, wnd, meta);
                } else {
                    const int t = i - r0;
#pragma unroll
                    for (int j = 0; j < NP; j += 2) {
                        SEG(t, j / 2) = make_float4(M[j].x, M[j].y, M[j + 1].x,
                                                    j + 1 == NP - 1 ? __uint_as_float(meta) : M[j + 1].y);
                        SEG(t, 4 + j / 2) = make_float4(I[j].x, I[j].y, I[j + 1].x, I[j + 1].y);
                    }
                }
            }
            if (fwd_pass) continue;

            // ---- backward rows r1 .. r0 with the MAP step ----
            for (int i = r1; i >= r0; i--) {
                const int t = i - r0;
                const int lo = LO(i), hi = HI(i);
                const bool edge = EDGE(i);
                const float4 mrow3 = SEG(t, 3);
                const u32 my_meta = __float_as_uint(mrow3.w);  // the forward row i's match bits and quality
                if (i == qL) {
                    // B(qL, k) = sM / s(qL) / sLast for every band cell: one constant (only ratios are used)
#pragma unroll
                    for (int s = 0; s < NS; s++) {
                        const bool in = s >= lo && s <= hi;
                        sx(bM, s) = in ? 1.0f : 0.0f;
                        sx(bI, s) = in ? 1.0f : 0.0f;
                    }
                } else {
                    // the emission of cell (i + 1, k + 1): the forward row i + 1's match bits and quality
                    const u32 qs1 = up_meta >> 24, ql1 = (up_meta >> 16) & 0xFFu, m16 = up_meta & 0xFFFFu;
                    float eqs, exs;
                    emis(qs1, ql1, tau, eqs, exs);
                    if (i == 1) bwd_row<true, true>(bM, bI, c, tau, eqs, exs, m16, lo, hi);
                    else if (edge) bwd_row<true, false>(bM, bI, c, tau, eqs, exs, m16, lo, hi);
                    else bwd_row<false, false>(bM, bI, c, tau, eqs, exs, m16, lo, hi);
                }
                tau = pow2_scale(row_sum(bM, bI), 32, under);
                if (i < qL) {
                    // the cells of column refLen (no emission; they only feed a diagonal neighbour, scaled by
                    // their own tiny value) may decay: the guard covers k < refLen
                    const int last_ok = refLen - 1 - (i - bw);
                    if (is_tiny(edge ? min_positive_bits(bM, lo, hi < last_ok ? hi : last_ok) : min_bits15(bM), tau))
                        under = true;
                }
                up_meta = my_meta;

                // ---- MAP for row i (device/baq.cu:619-681): first maximum in (k, M before I) order ----
                float2 fM[NP], fI[NP];
#pragma unroll
                for (int j = 0; j < NP; j += 2) {
                    const float4 a = j == NP - 2 ? mrow3 : SEG(t, j / 2), q4 = SEG(t, 4 + j / 2);
                    fM[j] = f2(a.x, a.y);
                    fM[j + 1] = f2(a.z, j + 1 == NP - 1 ? 0.0f : a.w);
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
                const int qo = int((my_meta >> 16) & 0xFFu);
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
                                    if (!is_max && z >= thr) {
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
                        // whether min(capped, qo) == qo, i.e. capped >= qo: monotone in t for qo <= 99
                        if ((flo >= qo) != (fhi >= qo)) amb |= 16;
                    } else if (!(thi < 100.f && flo == fhi) && !(tlo >= 101.5f)) {
                        amb |= 1 | 16;
                    }
                    // bit 8: the state is undecided, but every candidate's MAP quality is MIN_BASE_QUAL (a rival
                    // within the bound keeps the best posterior near 1/2, so t < 5 whichever term the exact
                    // computation picks)
                    if ((amb & 2) && thi < 4.9f) amb |= 8;
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
    constexpr int smem = SEG_K * SEG_VEC * SEG_THREADS * int(sizeof(float4));
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
