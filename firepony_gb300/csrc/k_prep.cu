// K1 read preparation: input validation, read filters, CIGAR expansion, clipping windows, error vectors,
// base and known-site masks and the BAQ work list — one thread per read, every stage of the reference's
// per-read functors fused into one pass over the read's events (which stay in L1/L2 while it runs).
// K2b (BAQ capping and BQ-tag encoding) is also here because it walks the same events.
#include "kernels.h"

namespace fpg {

unsigned long long g_kernel_launches = 0;

namespace {

struct us2 { u16 x, y; };
struct ss2 { i16 x, y; };

typedef long long i64;
template <typename T> __device__ __forceinline__ T tmin(T a, T b) { return a < b ? a : b; }
template <typename T> __device__ __forceinline__ T tmax(T a, T b) { return a > b ? a : b; }
__device__ __forceinline__ u32 baq_abs(i32 v) { return v < 0 ? u32(-v) : u32(v); }  // device/baq.cu:84-87

// ---------------------------------------------------------------------------------------------------
// validation: ranges in bounds, read length <= 511, read group < n_rg (or none)
__global__ void k_validate(DevBatch b, u32 n_rg, u32 *err) {
    const u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= b.R) return;
    u32 e = 0;
    if (u64(b.cigar_start[r]) + b.cigar_len[r] > b.num_cigar_ops) e |= ERR_BAD_READ_RANGE;
    if (u64(b.read_start[r]) + b.read_len[r] > b.num_syms) e |= ERR_BAD_READ_RANGE;
    if (u64(b.qual_start[r]) + b.qual_len[r] > b.num_quals) e |= ERR_BAD_READ_RANGE;
    if (b.read_len[r] > MAX_READ_LEN) e |= ERR_READ_TOO_LONG;
    if (b.rg[r] != U32_NONE && b.rg[r] >= n_rg) e |= ERR_BAD_READ_GROUP;
    if (e) raise_error(err, e);
}

__global__ void k_rebase_starts(u32 *cigar_start, u32 *read_start, u32 *qual_start, u32 n, u32 d_cigar, u32 d_sym,
                                u32 d_qual) {
    const u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    cigar_start[r] += d_cigar;
    read_start[r] += d_sym;
    qual_start[r] += d_qual;
}

__global__ void k_op_lengths(DevBatch b, u32 *out) {
    const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < b.num_cigar_ops) out[i] = op_len(b.cigars[i]);
}

// ---------------------------------------------------------------------------------------------------
struct Read {
    const DevBatch &b;
    const DevRef &ref;
    const BatchWork &w;
    u32 r;
    u32 cs, ce;         // event range (global event indices)
    u32 *rc;            // ev_rc + cs
    u8 *ty;             // ev_type + cs
    u32 n;              // events in the read
    u32 qs, rs, rlen;
    u32 astart;
    u16 flags;

    __device__ Read(const DevBatch &b_, const DevRef &ref_, const BatchWork &w_, u32 r_) : b(b_), ref(ref_), w(w_), r(r_) {
        cs = w.cigar_offsets[b.cigar_start[r]];
        ce = w.cigar_offsets[b.cigar_start[r] + b.cigar_len[r]];
        rc = w.ev_rc + cs;
        ty = w.ev_type + cs;
        n = ce - cs;
        qs = b.qual_start[r];
        rs = b.read_start[r];
        rlen = b.read_len[r];
        astart = b.astart[r];
        flags = b.flags[r];
    }
    __device__ __forceinline__ u16 readc(u32 e) const { return u16(rc[e] & 0xFFFF); }
    __device__ __forceinline__ u16 refc(u32 e) const { return u16(rc[e] >> 16); }
    __device__ __forceinline__ u8 sym(u32 i) const { return sym4(b.reads, u64(rs) + i); }
};

__device__ const DevContig *contig_of(const DevRef &ref, u32 id) {
    if (id < ref.num_contigs && ref.contigs[id].size > 0) return &ref.contigs[id];
    return nullptr;
}

// filter_mapq, filter_if_any_set, filter_if_cigar_malformed (device/read_filters.cu:42-75, :156-258)
__device__ bool passes_invalid_filters(const DevBatch &b, u32 r) {
    if (b.mapq[r] == 0 || b.mapq[r] == 255) return false;
    if (b.flags[r] & (F_DUPLICATE | F_QC_FAIL | F_UNMAP | F_SECONDARY)) return false;
    int st = 0;  // 0 leading hard, 1 leading soft, 2 no clips, 3 trailing soft, 4 trailing hard
    const u32 c0 = b.cigar_start[r], c1 = c0 + b.cigar_len[r];
    for (u32 i = c0; i < c1; i++) {
        const u32 op = op_code(b.cigars[i]);
        if (op == OP_N) return false;
        if (op == OP_H) {
            if (st == 1) return false;
            if (st == 2 || st == 3) st = 4;
        } else if (op == OP_S) {
            if (st == 0) st = 1;
            else if (st == 2) st = 3;
            else if (st == 4) return false;
        } else {
            if (st == 0 || st == 1) st = 2;
            else if (st == 3 || st == 4) return false;
        }
    }
    return true;
}

// compute_read_offset_list + compute_alignment_window (device/snp_filter.cu:42-147): the window ends at the
// reference offset of the last read base that has one. Also returns the number of read bases the CIGAR
// covers and whether an op code above X occurs.
__device__ void alignment_window(const DevBatch &b, u32 r, u32 &wx, u32 &wy, u32 &covered, bool &bad_op) {
    u16 offset = 0;
    u32 pos = 0;
    int last = -1;
    u16 last_off = 0;
    bad_op = false;
    const u32 c0 = b.cigar_start[r], c1 = c0 + b.cigar_len[r];
    const u32 rlen = b.read_len[r];
    for (u32 c = c0; c < c1; c++) {
        const u32 v = b.cigars[c], op = op_code(v), len = op_len(v);
        switch (op) {
        case OP_M: case OP_EQ: case OP_X:
            if (len) {
                // offsets offset .. offset+len-1 at read positions pos .. pos+len-1
                u32 lastpos = pos + len - 1;
                if (pos < rlen) {
                    u32 lp = lastpos < rlen ? lastpos : rlen - 1;
                    last = int(lp);
                    last_off = u16(offset + (lp - pos));
                }
                offset = u16(offset + len);
                pos += len;
            }
            break;
        case OP_I: case OP_N:
            if (len) {
                u32 lastpos = pos + len - 1;
                if (pos < rlen) {
                    u32 lp = lastpos < rlen ? lastpos : rlen - 1;
                    last = int(lp);
                    last_off = offset;
                }
                pos += len;
            }
            break;
        case OP_D: case OP_H: case OP_P:
            offset = u16(offset + len);
            break;
        case OP_S:
            pos += len;
            break;
        default:
            bad_op = true;
            break;
        }
    }
    covered = pos;
    if (last < 0) {
        wx = U32_NONE;
        wy = U32_NONE;
    } else {
        wx = b.astart[r];
        wy = b.astart[r] + last_off;
    }
}

// remove_soft_clips (device/cigar.cu:346-408)
__device__ void remove_soft_clips(const Read &rd, us2 &w) {
    const DevBatch &b = rd.b;
    const u32 c0 = b.cigar_start[rd.r], cl = b.cigar_len[rd.r];
    u32 ci = c0, ro = 0;
    while (ci < c0 + cl && ro < rd.rlen) {
        const u32 v = b.cigars[ci], op = op_code(v), len = op_len(v);
        if (op == OP_H || op == OP_S) {
            if (ro + len > w.x) w.x = tmin<u16>(u16(ro + len), w.y);
            ro += len;
            ci++;
        } else {
            break;
        }
    }
    if (cl > 0) {
        int cj = int(c0 + cl - 1);
        ro = rd.rlen - 1;
        while (cj >= int(c0) && ro > w.x) {
            const u32 v = b.cigars[cj], op = op_code(v), len = op_len(v);
            if (op == OP_H || op == OP_S) {
                if (ro - len < w.y) w.y = tmax<u16>(u16(ro - len), w.x);
                ro -= len;
                cj--;
            } else {
                break;
            }
        }
    }
}

// lower_bound / upper_bound (device/primitives/algorithms.h:39-100) over a non-decreasing array, as a
// 32-ary search by the whole warp: each round the lanes probe 32 evenly spaced positions and a ballot keeps
// the stretch between the last probe below the bound and the first at or past it (3 rounds for 11k sites
// instead of 14 dependent loads). The first index meeting the predicate is unique, so the result equals the
// reference's binary search. Every lane gets the result; all 32 lanes must call it.
template <typename Past>
__device__ __forceinline__ u32 warp_first_past(const u32 *a, u32 n, int lane, Past past) {
    u32 lo = 0, hi = n;  // the answer lies in [lo, hi]
    while (hi - lo >= 32) {
        const u32 step = (hi - lo + 30) / 31;  // lane 31 probes at or past hi
        const u32 p = lo + u32(lane) * step;
        const bool t = p < hi ? past(a[p]) : true;
        const u32 f = u32(__ffs(__ballot_sync(0xffffffffu, t)) - 1);
        const u32 nhi = lo + f * step;
        if (f > 0) lo = lo + (f - 1) * step + 1;
        hi = nhi < hi ? nhi : hi;
    }
    const u32 p = lo + u32(lane);
    const bool t = p < hi ? past(a[p]) : true;  // lane hi - lo (<= 31) always votes true
    return lo + u32(__ffs(__ballot_sync(0xffffffffu, t)) - 1);
}
// first index with a[i] >= x
__device__ __forceinline__ u32 warp_lower_bound(u32 x, const u32 *a, u32 n, int lane) {
    return warp_first_past(a, n, lane, [x](u32 v) { return !(v < x); });
}
// first index with a[i] > x
__device__ __forceinline__ u32 warp_upper_bound(u32 x, const u32 *a, u32 n, int lane) {
    return warp_first_past(a, n, lane, [x](u32 v) { return x < v; });
}

// ---------------------------------------------------------------------------------------------------
// Warp-per-read forms of the event scans and per-base passes used by k_prep. Every lane of the warp holds
// the same read-level scalars (computed redundantly, the loads are broadcasts); event searches are ballots
// over 32 events at a time and per-event / per-base work is lane-strided.
constexpr u32 WFULL = 0xffffffffu;

// first event e in [lo, n) with pred(e), or n
template <typename P> __device__ __forceinline__ u32 first_from(u32 lo, u32 n, int lane, P pred) {
    for (u32 c = lo; c < n; c += 32) {
        const u32 e = c + u32(lane);
        const u32 m = __ballot_sync(WFULL, e < n && pred(e));
        if (m) return c + __ffs(m) - 1;
    }
    return n;
}
// last event e in [0, hi) with pred(e), or -1
template <typename P> __device__ __forceinline__ int last_below(int hi, int lane, P pred) {
    for (int c = hi - 32; c > -32; c -= 32) {
        const int e = c + lane;
        const u32 m = __ballot_sync(WFULL, e >= 0 && e < hi && pred(u32(e)));
        if (m) return c + 31 - __clz(m);
    }
    return -1;
}

// cigar_coordinates_expand (device/cigar.cu:536-614) + cigar_op_expand (:55-95): op by op, the op's events
// lane-strided; read and reference offsets at the op start carried as scalars
__device__ void expand_read_w(Read &rd, int lane) {
    const DevBatch &b = rd.b;
    u32 ro = 0, fo = 0, e = 0;
    const u32 c0 = b.cigar_start[rd.r], c1 = c0 + b.cigar_len[rd.r];
    for (u32 c = c0; c < c1; c++) {
        const u32 v = b.cigars[c], op = op_code(v), len = op_len(v);
        const bool reads_base = op == OP_M || op == OP_EQ || op == OP_X || op == OP_S || op == OP_N || op == OP_I;
        const bool refs_base = op == OP_M || op == OP_EQ || op == OP_X || !reads_base;
        for (u32 i = u32(lane); i < len; i += 32) {
            u32 rcv;
            u8 t;
            if (op == OP_M || op == OP_EQ || op == OP_X) { rcv = u32(u16(ro + i)) | (u32(u16(fo + i)) << 16); t = EV_M; }
            else if (op == OP_S) { rcv = u32(u16(ro + i)) | (u32(U16_NONE) << 16); t = EV_S; }
            else if (op == OP_N || op == OP_I) { rcv = u32(u16(ro + i)) | (u32(U16_NONE) << 16); t = EV_I; }
            else { rcv = u32(U16_NONE) | (u32(u16(fo + i)) << 16); t = EV_D; }  // D, H, P
            rd.rc[e + i] = rcv;
            rd.ty[e + i] = t;
        }
        if (reads_base) ro += len;
        if (refs_base) fo += len;
        e += len;
    }
    __syncwarp();
}

// remove_adapters' read coordinate search (device/cigar.cu:251-344); see read_coord_for_ref
__device__ int read_coord_for_ref_w(const Read &rd, u32 ref_coord, bool right_tail, int lane) {
    const u32 ev = first_from(0, rd.n, lane, [&](u32 e) { return rd.astart + u32(rd.refc(e)) == ref_coord; });
    if (ev == rd.n) return -1;
    u16 read_coord = rd.readc(ev);
    if (read_coord == U16_NONE) {
        if (right_tail) {
            const u32 e2 = first_from(ev, rd.n, lane, [&](u32 e) { return rd.readc(e) != U16_NONE; });
            if (e2 == rd.n) return -1;
            read_coord = rd.readc(e2);
        } else {
            const int e2 = last_below(int(ev), lane, [&](u32 e) { return rd.readc(e) != U16_NONE; });
            if (e2 < 0) return -1;
            read_coord = rd.readc(u32(e2));
        }
    }
    return read_coord;
}

// current_reference_window (device/cigar.cu:165-200, init (0, 0)) and compute_reference_window
// (:473-534, init (0xFFFF, 0xFFFF)): the reference offsets of the first event at read offset a.x (or the
// next event that has one) and of the last event at read offset a.y (or the previous one; reaching the first
// event gives (0xFFFF, 0xFFFF))
__device__ us2 ref_window_w(const Read &rd, us2 a, u16 init, int lane) {
    us2 out = {init, init};
    const u32 i = first_from(0, rd.n, lane, [&](u32 e) { return rd.readc(e) == a.x; });
    if (i < rd.n) {
        const u32 j = first_from(i, rd.n, lane, [&](u32 e) { return rd.refc(e) != U16_NONE; });
        if (j == rd.n) return us2{U16_NONE, U16_NONE};
        out.x = rd.refc(j);
    }
    const int k = last_below(int(rd.n), lane, [&](u32 e) { return rd.readc(e) == a.y; });
    if (k >= 0) {
        const int j = last_below(k + 1, lane, [&](u32 e) { return e >= 1 && rd.refc(e) != U16_NONE; });
        if (j < 1) return us2{U16_NONE, U16_NONE};
        out.y = rd.refc(u32(j));
    }
    return out;
}

// remove_adapters (device/cigar.cu:111-344). The backward walk for a left tail cannot leave the read: a
// matched event without a read coordinate always follows the read's first read-coordinate event, because
// the window check before it rejects boundaries left of the first aligned base.
__device__ void remove_adapters_w(const Read &rd, us2 &w, int lane) {
    const DevBatch &b = rd.b;
    const u32 r = rd.r;
    const u32 flags = rd.flags;
    const i32 isize = b.isize[r];
    // hasWellDefinedFragmentSize (:117-146)
    if (isize == 0) return;
    if (!(flags & F_PAIRED)) return;
    if ((flags & F_UNMAP) || (flags & F_MATE_UNMAP)) return;
    const bool rev = flags & F_REVERSE, mate_rev = flags & F_MATE_REVERSE;
    if (rev == mate_rev) return;
    bool ok = rev ? (b.astop[r] > b.mstart[r]) : (rd.astart <= b.mstart[r] + u32(isize));
    if (!ok) return;
    // getAdaptorBoundary (:150-163)
    u32 boundary;
    if (rev) boundary = u32(b.mstart[r] - 1);
    else boundary = u32(rd.astart + u32(isize < 0 ? -isize : isize) + 1u);
    if (boundary == U32_NONE) return;
    const us2 rw = ref_window_w(rd, w, 0, lane);
    if (boundary < rd.astart + u32(rw.x) || boundary > rd.astart + u32(rw.y)) return;
    if (rev) {
        // hardClipByReferenceCoordinates with refStart = -1 (:251-266)
        const int stop = read_coord_for_ref_w(rd, u32(int(boundary)), false, lane);
        w.x = tmax<u16>(w.x, u16(u16(stop) + 1));
    } else {
        int start;
        if (int(boundary) < 0) start = 0;  // refStart < 0 branch
        else start = read_coord_for_ref_w(rd, u32(int(boundary)), true, lane);
        w.y = tmin<u16>(w.y, u16(u16(start) - 1));
    }
}

// compute_no_insertions_window (device/cigar.cu:410-471); (0xFFFF, 0xFFFF) when nothing qualifies
__device__ us2 no_insertions_window_w(const Read &rd, us2 w, int lane) {
    us2 out = {U16_NONE, U16_NONE};
    const u32 i = first_from(0, rd.n, lane, [&](u32 e) {
        const u16 ro = rd.readc(e);
        return ro != U16_NONE && ro >= w.x && rd.ty[e] != EV_I;
    });
    if (i < rd.n) out.x = rd.readc(i);
    const int k = last_below(int(rd.n), lane, [&](u32 e) {
        const u16 ro = rd.readc(e);
        return ro != U16_NONE && ro <= w.y && rd.ty[e] != EV_I;
    });
    if (k >= 0) out.y = rd.readc(u32(k));
    return out;
}

// compute_error_vectors (device/cigar.cu:616-737) on the warp's staged base flags: the events of an M op
// lane-strided (each base of an M op belongs to one event), I and D ops as scalars written by lane 0
__device__ u16 error_vectors_w(const Read &rd, const DevContig *g, us2 w, us2 rw, u8 *sbf, int lane) {
    const DevBatch &b = rd.b;
    const bool neg = rd.flags & F_REVERSE;
    u32 cur = 0, nerr = 0;
    const u32 c0 = b.cigar_start[rd.r], c1 = c0 + b.cigar_len[rd.r];
    for (u32 c = c0; c < c1; c++) {
        const u32 e0 = rd.w.cigar_offsets[c] - rd.cs, e1 = rd.w.cigar_offsets[c + 1] - rd.cs;
        const u32 op = op_code(b.cigars[c]);
        if (op == OP_M) {
            for (u32 base = e0; base < e1; base += 32) {
                const u32 i = base + u32(lane);
                bool err = false;
                if (i < e1) {
                    const u16 rc = rd.readc(i);
                    const u8 rbp = rd.sym(rc);
                    const u8 fbp = contig_at(*g, u64(rd.astart) + rd.refc(i));
                    if (fbp != rbp) {
                        sbf[rc] |= BF_SNP;
                        err = rc >= w.x && rc <= w.y;
                    }
                }
                nerr += __popc(__ballot_sync(WFULL, err));
            }
            if (e1 > e0) cur = rd.readc(e1 - 1);
        } else if (op == OP_I) {
            cur = rd.readc(e0);
            if (cur >= w.x && cur <= w.y) {
                const int off = neg ? int(cur) + int(op_len(b.cigars[c])) : int(cur) - 1;
                if (off >= 0 && off <= int(w.y)) {
                    __syncwarp();
                    if (lane == 0) sbf[off] |= BF_INS;
                    nerr++;
                }
            }
        } else if (op == OP_D) {
            const u16 cref = rd.refc(e0);
            if (cref >= rw.x && cref <= rw.y) {
                __syncwarp();
                if (!neg) {
                    if (lane == 0) sbf[u16(cur)] |= BF_DEL;
                    nerr++;
                } else {
                    const u16 off = u16(cur + 1);
                    if (off < rd.rlen) {
                        if (lane == 0) sbf[off] |= BF_DEL;
                        nerr++;
                    }
                }
            }
        }
        __syncwarp();
    }
    return u16(nerr);
}

// compute_vcf_ranges + filter_bps (device/snp_filter.cu:162-395): per overlapping feature the start event by
// a ballot search, the short walks around it as scalars, the masked bases lane-strided
__device__ void filter_known_sites_w(const Read &rd, us2 w, us2 rw, u8 *sbf, int lane) {
    const u32 ch = rd.b.chromosome[rd.r];
    if (ch >= rd.ref.num_site_contigs) return;
    const DevSites db = rd.ref.sites[ch];
    const u32 wx = rd.astart + u32(rw.x), wy = rd.astart + u32(rw.y);
    const u32 vx = warp_lower_bound(wx, db.maxend, db.n, lane);
    if (vx >= db.n) return;
    u32 vy = warp_upper_bound(wy, db.start, db.n, lane);
    if (vy <= vx) return;
    if (vy >= db.n) vy = db.n - 1;
    const u32 n = rd.n;
    for (u32 feature = vx; feature <= vy; feature++) {
        const int fstart = int(db.start[feature] - rd.astart);
        const int fend = int(db.stop[feature] - rd.astart);
        u32 ev = first_from(0, n, lane, [&](u32 e) {
            const u16 rc = rd.refc(e);
            return rc != U16_NONE && int(rc) >= fstart;
        });
        if (ev == n) continue;
        const u16 ref_coord = rd.refc(ev);
        int left = int(ref_coord) - fstart;
        u32 evs = ev;
        if (left > 0) {
            while (left && evs > 0) {
                const u8 t = rd.ty[evs];
                if (t == EV_S) break;
                if (t == EV_M || t == EV_D) left--;
                evs--;
            }
            while (evs > 0 && rd.ty[evs - 1] == EV_I) evs--;
            while (evs < n && rd.readc(evs) == U16_NONE) evs++;
        } else {
            if (rd.refc(evs) <= rw.y) {
                while (evs > 0 && rd.ty[evs] == EV_D) evs--;
            }
        }
        int right = fend - int(ref_coord);
        while (right > 0 && ev + 1 < n) {
            ev++;
            const u8 t = rd.ty[ev];
            if (t == EV_S) break;
            if (t == EV_M || t == EV_D) right--;
        }
        while (ev > 0 && rd.readc(ev) == U16_NONE) ev--;
        if (ev < evs) continue;
        u32 a = rd.readc(evs), z = rd.readc(ev);
        if ((a < w.x && z < w.x) || (a > w.y && z > w.y)) continue;
        a = tmin<u32>(tmax<u32>(a, w.x), w.y);
        z = tmin<u32>(tmax<u32>(z, w.x), w.y);
        for (u32 d = a + u32(lane); d <= z; d += 32) sbf[d] &= u8(~BF_ACTIVE);
        __syncwarp();
    }
}

// compute_hmm_windows (device/baq.cu:89-187)
__device__ bool hmm_window(const Read &rd, const DevContig *g, u16 nerr, us2 w, us2 ni, us2 rw, ss2 &hw, u16 &bw) {
    const bool needs = nerr != 0;
    const int offset = MIN_BAND_WIDTH / 2;
    const bool left_clip = w.x != 0;
    const bool right_clip = w.y != u16(rd.rlen - 1);
    const i16 li = i16(left_clip ? 0 : int(ni.x) - int(w.x));
    const i16 ri = i16(right_clip ? 0 : int(w.y) - int(ni.y));
    hw.x = i16(int(rw.x) - li - offset);
    hw.y = i16(int(rw.y) + ri + offset);
    const u64 csize = g ? g->size : 0;
    int shift = 0;
    if (hw.x < 0 && rd.astart < baq_abs(hw.x)) shift = -1;
    if (needs && u32(rd.astart + u32(int(hw.y)) + u32(shift)) >= u32(csize)) {
        hw.x = -1;
        hw.y = -1;
        return false;
    }
    const int refLen = hw.y - hw.x + 1;
    const int qLen = w.y - w.x + 1;
    u16 band = u16(refLen > qLen ? refLen : qLen);
    const u32 d = baq_abs(refLen - qLen);
    if (u32(MIN_BAND_WIDTH) < d) band = u16(d + 3);
    if (band > MIN_BAND_WIDTH) band = MIN_BAND_WIDTH;
    if (band < d) band = u16(d);
    bw = band;
    return true;
}

constexpr int PREP_WARPS = 8;

// K1: one warp per read. Filters and CIGAR-op walks run as identical scalars on every lane; event scans are
// ballots and per-event / per-base work is lane-strided; the read's base flags live in shared memory until
// written out once.
__global__ void __launch_bounds__(PREP_WARPS * 32) k_prep(DevBatch b, DevRef ref, BatchWork w) {
    __shared__ u8 s_bf[PREP_WARPS][512];
    // per warp, over its reads: band cells per class, BAQ reads, longest query, widest band per class; added to
    // the batch counters once, when the warp has no reads left
    __shared__ unsigned long long s_cells[PREP_WARPS][3];
    __shared__ u32 s_agg[PREP_WARPS][5];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    u8 *sbf = s_bf[wib];
    if (lane < 3) s_cells[wib][lane] = 0;
    if (lane < 5) s_agg[wib][lane] = 0;
    __syncwarp();
    for (u32 r = blockIdx.x * PREP_WARPS + wib; r < b.R; r += gridDim.x * PREP_WARPS) {
        const u32 qs = b.qual_start[r];
        const u32 rlen = b.read_len[r];

        // filter_invalid_reads -> alignment windows -> filter_malformed_reads (device/pipeline.cu:66-80)
        bool pass = passes_invalid_filters(b, r);
        if (pass) {
            u32 wx, wy, covered;
            bool bad_op;
            alignment_window(b, r, wx, wy, covered, bad_op);
            // filter_if_read_malformed (device/read_filters.cu:77-154); the uint16 contig id never equals
            // uint32(-1), so those checks are inert. Unknown contigs fail the contig-end check; reads whose
            // CIGAR does not cover read_len bases or holds an op code above X are rejected (undefined in the
            // reference).
            const DevContig *g0 = contig_of(ref, b.chromosome[r]);
            if (!(b.flags[r] & F_UNMAP)) {
                if (b.astart[r] == U32_NONE) pass = false;
                else if (wy <= wx) pass = false;
                else if (wx >= (g0 ? g0->size : 0)) pass = false;
                else if (b.cigar_len[r] == 0) pass = false;
            }
            if (b.rg[r] == U32_NONE) pass = false;
            if (b.qual_len[r] != rlen) pass = false;
            if (rlen == 0) pass = false;
            if (covered != rlen || bad_op) pass = false;
        }
        if (!pass) {
            if (lane == 0) {
                w.status[r] = RS_FILTERED;
                atomicAdd(&w.counters[5], 1u);
            }
            continue;
        }

        Read rd(b, ref, w, r);
        const DevContig *g = contig_of(ref, b.chromosome[r]);
        expand_read_w(rd, lane);
        // start_batch: every base active (device/firepony_context.cu:52-59); error bits cleared
        for (u32 i = u32(lane); i < rlen; i += 32) sbf[i] = BF_ACTIVE;
        __syncwarp();

        us2 wcl = {0, u16(rlen - 1)};  // read_window_init (device/cigar.cu:97-109)
        remove_adapters_w(rd, wcl, lane);
        remove_soft_clips(rd, wcl);
        const us2 ni = no_insertions_window_w(rd, wcl, lane);
        const us2 rw = ref_window_w(rd, ni, U16_NONE, lane);
        const u16 nerr = error_vectors_w(rd, g, wcl, rw, sbf, lane);

        // filter_bases (device/read_filters.cu:375-439)
        for (u32 i = u32(lane); i < rlen; i += 32) {
            const u8 bp = rd.sym(i);
            const bool regular = bp == IUPAC_A || bp == IUPAC_C || bp == IUPAC_G || bp == IUPAC_T;
            if (!regular || b.quals[qs + i] < 6) sbf[i] &= u8(~BF_ACTIVE);
        }
        __syncwarp();
        filter_known_sites_w(rd, wcl, rw, sbf, lane);

        ss2 hw;
        u16 bw = 0;
        const bool hmm_ok = hmm_window(rd, g, nerr, wcl, ni, rw, hw, bw);
        const u8 status = hmm_ok ? RS_ACTIVE : RS_REMOVED;
        if (!hmm_ok) {
            // the read's events lose their read coordinates (device/baq.cu:136-158): it contributes nothing
            for (u32 e = u32(lane); e < rd.n; e += 32) rd.rc[e] = u32(U16_NONE) | (rd.rc[e] & 0xFFFF0000u);
        }
        for (u32 i = u32(lane); i < rlen; i += 32) w.bflags[qs + i] = sbf[i];

        if (lane == 0) {
            u16 *win = w.win + size_t(r) * 8;
            win[0] = wcl.x; win[1] = wcl.y; win[2] = ni.x; win[3] = ni.y; win[4] = rw.x; win[5] = rw.y;
            w.hmm[size_t(r) * 2 + 0] = hw.x;
            w.hmm[size_t(r) * 2 + 1] = hw.y;
            w.bw[r] = bw;
            w.nerr[r] = nerr;
            w.status[r] = status;
        }
        if (status == RS_ACTIVE && nerr == 0) {
            // read_flat_baq (device/baq.cu:842-868)
            for (u32 i = wcl.x + u32(lane); i <= wcl.y; i += 32) w.tag[qs + i] = NO_BAQ_UNCERTAINTY;
        }
        // a reference N inside the HMM window (emission 1 for every query base) takes a read of band class 0 to
        // the general kernel of class 1: the class-0 kernel selects emissions by symbol equality alone
        bool ref_n = false;
        if (status == RS_ACTIVE && nerr != 0 && bw <= 7 && g) {
            int refLen = int(hw.y) - int(hw.x) + 1;
            u64 off;
            if (hw.x < 0 && rd.astart < baq_abs(hw.x)) {
                off = 0;
                refLen--;
            } else {
                off = u64(u32(rd.astart + u32(int(hw.x))));
            }
            bool any = false;
            for (int k = lane; k < refLen; k += 32) any |= contig_at(*g, off + u64(k)) == IUPAC_N;
            ref_n = __any_sync(WFULL, any);
        }
        if (lane == 0 && status == RS_ACTIVE && nerr != 0) {
            // BAQ work list by band class: 0 -> bw <= 7, 1 -> bw <= 15, 2 -> wider
            const u32 cls = bw <= 7 ? (ref_n ? 1 : 0) : (bw <= 15 ? 1 : 2);
            const u32 slot = atomicAdd(&w.counters[cls], 1u);
            w.baq_list[size_t(cls) * b.R + slot] = r;
            // band cells of the read's HMM (rows 1..qL, reference positions max(1, i-bw)..min(refLen, i+bw)),
            // the work unit of the BAQ kernels' throughput figures
            int refLen = int(hw.y) - int(hw.x) + 1;
            if (hw.x < 0 && rd.astart < baq_abs(hw.x)) refLen--;
            // closed form of sum_i (min(refLen, i+bw) - max(1, i-bw) + 1); |refLen - qL| <= bw keeps every
            // term non-negative
            const i64 qL = int(wcl.y) - int(wcl.x) + 1, R = refLen, B = bw;
            auto tri = [](i64 n) -> i64 { return n > 0 ? n * (n + 1) / 2 : 0; };
            i64 sum_hi = tri(qL) + qL * B;
            const i64 t0 = R - B + 1 > 1 ? R - B + 1 : 1;
            if (t0 <= qL) sum_hi -= tri(qL + B - R) - tri(t0 - 1 + B - R);
            const i64 m = qL < B ? qL : B;
            const i64 sum_lo = tri(qL) - qL * B + (m * (B + 1) - tri(m));
            const u64 cells = u64(sum_hi - sum_lo + qL);
            s_cells[wib][cls] += cells;
            s_agg[wib][0] += 1u;
            s_agg[wib][1] = max(s_agg[wib][1], u32(wcl.y - wcl.x + 1));
            s_agg[wib][2 + cls] = max(s_agg[wib][2 + cls], u32(bw));
        }
        __syncwarp();
    }
    __syncwarp();
    if (lane < 3 && s_cells[wib][lane])
        atomicAdd(reinterpret_cast<unsigned long long *>(w.counters + 16) + lane, s_cells[wib][lane]);
    if (lane == 3 && s_agg[wib][0]) atomicAdd(&w.counters[6], s_agg[wib][0]);
    if (lane == 4 && s_agg[wib][1]) atomicMax(&w.counters[7], s_agg[wib][1]);
    if (lane >= 5 && lane < 8 && s_agg[wib][2 + lane - 5]) atomicMax(&w.counters[12 + lane - 5], s_agg[wib][2 + lane - 5]);
}

// ---------------------------------------------------------------------------------------------------
// cap_baq_qualities + recode_baq_qualities (device/baq.cu:870-1081), one warp per BAQ read. The reference
// walks the read's events from the first one inside the clipped window (baq_start) to the first one past it,
// counting reference steps (S, D, M), deletions and read steps (I, M); read coordinates increase along the
// events, so that walk is a contiguous range and the running counts are prefix counts (ballots).
// cap_baq<false> is the read-step total check; cap_baq<true> writes min(bq, baq) or 4 per M base and the
// original quality per I base. In FP32 mode (exact == 0) the HMM outputs can be undecided (baq_amb); if a
// capped value depends on one (an undecided quality of a base whose state is the match at its expected
// position, or an undecided state whose candidates do not all give MIN_BASE_QUAL), the read goes to the
// escalation list and the exact replay's capping rewrites its values. A state left undecided by a rival
// within the bound (baq_amb bit 2) caps at MIN_BASE_QUAL whichever candidate wins whenever the kernel also
// proved every candidate's MAP quality to be MIN_BASE_QUAL (bit 8) and the original quality is at least that.
constexpr int CAP_PF = 4;  // chunks of 32 events whose loads k_cap issues together

__global__ void __launch_bounds__(64) k_cap(DevBatch b, BatchWork w, const u32 *list, const u32 *count, int exact) {
    constexpr u32 FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const u32 lt = (1u << lane) - 1;
    const u32 nwarps = (gridDim.x * blockDim.x) >> 5;
    const u32 n_list = *count;
    for (u32 idx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; idx < n_list; idx += nwarps) {
        const u32 r = list[idx];
        const u32 cs = w.cigar_offsets[b.cigar_start[r]];
        const u32 ce = w.cigar_offsets[b.cigar_start[r] + b.cigar_len[r]];
        const u32 n = ce - cs;
        const u32 *rc = w.ev_rc + cs;
        const u8 *ty = w.ev_type + cs;
        const u16 *win = w.win + size_t(r) * 8;
        const us2 wcl = {win[0], win[1]}, rw = {win[4], win[5]};
        const ss2 hw = {w.hmm[size_t(r) * 2], w.hmm[size_t(r) * 2 + 1]};
        const u32 qs = b.qual_start[r];
        const u32 astart = b.astart[r];
        i16 reference_shift = 0, read_shift = 0;
        if (hw.x < 0 && astart < baq_abs(hw.x)) {
            reference_shift = i16(baq_abs(hw.x));
            read_shift = i16(astart);
        }
        const i16 refOffset = i16(int(hw.x) - int(rw.x) + int(reference_shift));

        // baq_start: first event with a read coordinate >= window.x
        u32 baq_start = 0;
        for (u32 c = 0; c < n; c += 32) {
            const u32 i = c + lane;
            const u16 rb = i < n ? u16(rc[i] & 0xFFFF) : U16_NONE;
            const u32 m = __ballot_sync(FULL, rb != U16_NONE && rb >= wcl.x);
            if (m) { baq_start = c + __ffs(m) - 1; break; }
        }

        // One walk from baq_start to `end`, the first later event past window.y (found in the chunk that holds
        // it, which ends the walk). It makes the read-step total of cap_baq<false>, and writes cap_baq<true>'s
        // values already recoded (recode_baq_qualities: quality + 64 - capped; an I base's capped value is its
        // quality, so its tag is 64). Bases the walk does not write keep the batch's 0xFF, which recoding
        // leaves alone. The writes are speculative in FP32 mode: a read whose capped values depend on an
        // undecided HMM output is deferred, and the exact replay's capping rewrites the same bases (the
        // walk does not depend on the HMM) before anything reads them.
        u32 end = n;
        u32 refI_c = 0, numD_c = 0, readI_c = 0;
        bool escalate = false, by_state = false, unbounded = false;
        // CAP_PF chunks of 32 events at a time: their events and the HMM outputs of their M bases are loaded
        // together (one round of dependent loads per CAP_PF chunks), then the chunks are walked in order. The
        // walk ends inside a group only (the chunk holding `end`), so every group starts with end == n; loads
        // past `end` stay inside the read (its bases and events) and are not used.
        for (u32 c0 = baq_start; c0 < end; c0 += 32 * CAP_PF) {
            u32 rc_v[CAP_PF], st_v[CAP_PF];
            u8 ty_v[CAP_PF], oq_v[CAP_PF], bq_v[CAP_PF], amb_v[CAP_PF];
#pragma unroll
            for (int q = 0; q < CAP_PF; q++) {
                const u32 i = c0 + 32 * q + lane;
                rc_v[q] = i < end ? rc[i] : u32(U16_NONE);
                ty_v[q] = i < end ? ty[i] : u8(EV_S);
            }
#pragma unroll
            for (int q = 0; q < CAP_PF; q++) {
                const u16 rb = u16(rc_v[q] & 0xFFFF);
                const bool m = ty_v[q] == EV_M && rb != U16_NONE;
                st_v[q] = m ? w.baq_state[qs + rb] : 0u;
                oq_v[q] = m ? b.quals[qs + rb] : u8(0);
                bq_v[q] = m ? w.baq_q[qs + rb] : u8(0);
                amb_v[q] = m && !exact ? w.baq_amb[qs + rb] : u8(0);
            }
#pragma unroll
            for (int q = 0; q < CAP_PF; q++) {
                const u32 c = c0 + 32 * q;
                if (c >= end) break;  // (end is the same in every lane)
                const u32 i = c + lane;
                const u32 rcv = i < end ? rc_v[q] : u32(U16_NONE);
                const u16 rb = u16(rcv & 0xFFFF);
                const u32 past = __ballot_sync(FULL, rb != U16_NONE && rb > wcl.y);
                if (past) end = c + __ffs(past) - 1;
                const bool in = i < end;
                const u8 t = in ? ty_v[q] : u8(EV_S);
                const bool isM = in && t == EV_M, isI = in && t == EV_I, isD = in && t == EV_D;
                const bool isRef = in && (t == EV_S || t == EV_D || t == EV_M);
                const u32 mRef = __ballot_sync(FULL, isRef), mD = __ballot_sync(FULL, isD);
                const u32 mRead = __ballot_sync(FULL, isM || isI);
                if (isI) {
                    w.tag[qs + rb] = NO_BAQ_UNCERTAINTY;
                } else if (isM) {
                    const u32 refI = refI_c + __popc(mRef & lt), numD = numD_c + __popc(mD & lt);
                    const u32 readI = readI_c + __popc(mRead & lt);
                    const u32 expectedPos =
                        refI - u32(int(refOffset)) + (i - numD - baq_start - readI) + u32(int(read_shift));
                    const u32 state = st_v[q];
                    const u8 oq = oq_v[q];
                    const u8 bq = bq_v[q];
                    // the capped value uses the HMM quality only when the MAP state is the match at expectedPos
                    const bool at_expected = (state & 3) == 0 && (state >> 2) == expectedPos;
                    if (!exact && !w.exact_tags) {
                        // Only whether the capped value equals oq reaches the tables (the covariate passes test
                        // tag == NO_BAQ_UNCERTAINTY, as device/fractional_errors.cu:93 does): at the expected match
                        // that is bq >= oq (undecided under bit 16), elsewhere oq == MIN_BASE_QUAL
                        const u8 amb = amb_v[q];
                        if (amb == 7) {
                            unbounded = true;  // a row the FP32 pass left wholly undecided
                            escalate = true;
                            by_state = true;
                        } else if (amb & 6) {
                            // undecided state: the candidates are the FP32 winner and its one rival, or (several
                            // rivals) any state
                            bool can_expected = true, can_other = true;
                            if (!(amb & 4)) {
                                const u32 alt = w.baq_alt[qs + rb];
                                const bool alt_expected = (alt & 3) == 0 && (alt >> 2) == expectedPos;
                                can_expected = at_expected || alt_expected;
                                can_other = !at_expected || !alt_expected;
                            }
                            const bool same_at_expected = bq >= oq, same_elsewhere = oq == MIN_BASE_QUAL;
                            if (can_expected && ((amb & 16) || (can_other && same_at_expected != same_elsewhere))) {
                                escalate = true;
                                by_state = true;
                            }
                        } else if ((amb & 16) && at_expected) {
                            escalate = true;
                        }
                    } else if (!exact) {
                        const u8 amb = amb_v[q];
                        unbounded |= amb == 7;  // a row the FP32 pass left wholly undecided
                        if ((amb & 8) && oq >= MIN_BASE_QUAL) {
                            // undecided state whose candidates all have MAP quality MIN_BASE_QUAL: min(bq, oq) at
                            // the expected match and MIN_BASE_QUAL elsewhere are the same value
                        } else if (amb & 4) {
                            escalate = true;
                            by_state = true;
                        } else if (amb & 2) {
                            // one rival state: decided when neither state is the match at expectedPos (the value is
                            // MIN_BASE_QUAL whichever wins)
                            const u32 alt = w.baq_alt[qs + rb];
                            const bool alt_expected = (alt & 3) == 0 && (alt >> 2) == expectedPos;
                            if (at_expected || alt_expected) {
                                escalate = true;
                                by_state = true;
                            }
                        } else if ((amb & 1) && at_expected) {
                            escalate = true;
                        }
                    }
                    const u8 v = at_expected ? (bq < oq ? bq : oq) : u8(MIN_BASE_QUAL);
                    w.tag[qs + rb] = u8(u8(oq + 64) - v);
                }
                refI_c += __popc(mRef);
                numD_c += __popc(mD);
                readI_c += __popc(mRead);
            }
        }
        const bool need_update = readI_c == u32(wcl.y - wcl.x + 1);
        if (!need_update) {
            // cap_baq<true> is skipped: the window keeps its original qualities, recoded to 64
            __syncwarp();
            for (u32 i = wcl.x + lane; i <= wcl.y; i += 32) w.tag[qs + i] = NO_BAQ_UNCERTAINTY;
            continue;
        }
        if (!exact && __any_sync(FULL, escalate)) {
            if (lane == 0) {
                // escalation lists by band class: class 0 (band <= 7), class 1 (band <= 15), class 2 (wider)
                const u32 cls = w.bw[r] <= 7 ? 0 : (w.bw[r] <= 15 ? 1 : 2);
                const u32 slot = atomicAdd(&w.counters[cls == 0 ? 4 : (cls == 1 ? 10 : 27)], 1u);
                w.esc_list[size_t(cls) * b.R + slot] = r;
                w.status[r] = RS_DEFERRED;
            }
            // escalation cause: some MAP state undecided, or only qualities undecided
            const bool st = __any_sync(FULL, by_state);
            if (lane == 0) atomicAdd(&w.counters[st ? 22 : 23], 1u);
            const bool ub = __any_sync(FULL, unbounded);
            if (lane == 0 && ub) atomicAdd(&w.counters[25], 1u);
        }
    }
}

}  // namespace

void launch_validate(const DevBatch &b, u32 n_rg, u32 *err, cudaStream_t s) {
    if (!b.R) return;
    k_validate<<<(b.R + 255) / 256, 256, 0, s>>>(b, n_rg, err);
    g_kernel_launches++;
}

void launch_rebase_starts(u32 *cigar_start, u32 *read_start, u32 *qual_start, u32 n, u32 d_cigar, u32 d_sym,
                          u32 d_qual, cudaStream_t s) {
    if (!n) return;
    k_rebase_starts<<<(n + 255) / 256, 256, 0, s>>>(cigar_start, read_start, qual_start, n, d_cigar, d_sym, d_qual);
    g_kernel_launches++;
}

void launch_op_lengths(const DevBatch &b, u32 *out, cudaStream_t s) {
    if (!b.num_cigar_ops) return;
    k_op_lengths<<<(b.num_cigar_ops + 255) / 256, 256, 0, s>>>(b, out);
    g_kernel_launches++;
}

void launch_prep(const DevBatch &b, const DevRef &ref, const BatchWork &w, cudaStream_t s) {
    if (!b.R) return;
    u32 blocks = (b.R + PREP_WARPS - 1) / PREP_WARPS;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_prep<<<blocks, PREP_WARPS * 32, 0, s>>>(b, ref, w);
    g_kernel_launches++;
}

// ---------------------------------------------------------------------------------------------------
// BAQ work lists ordered by HMM query length (longest first), a counting sort over the two FP32 band
// classes: the 32 reads a warp of the thread-per-read kernels takes then walk the same rows, so their
// scratch rows coalesce and their loops stay converged. Bins: class * 512 + (511 - query length).
namespace {

__device__ __forceinline__ u32 qlen_bin(const BatchWork &w, u32 r, u32 cls) {
    const u16 *win = w.win + size_t(r) * 8;
    return cls * 512u + (511u - u32(win[1] - win[0] + 1));
}

__global__ void k_len_hist(BatchWork w, u32 R, u32 *hist) {
    __shared__ u32 h[1024];
    for (u32 i = threadIdx.x; i < 1024; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (u32 cls = 0; cls < 2; cls++) {
        const u32 n = w.counters[cls];
        const u32 *list = w.baq_list + size_t(cls) * R;
        for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            atomicAdd(&h[qlen_bin(w, list[i], cls)], 1u);
    }
    __syncthreads();
    for (u32 i = threadIdx.x; i < 1024; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// exclusive scan of the 1024 bins in place, restarting at each class (one block of 1024 threads)
__global__ void k_len_scan(u32 *hist) {
    __shared__ u32 v[1024];
    const u32 t = threadIdx.x;
    v[t] = hist[t];
    __syncthreads();
    for (u32 o = 1; o < 512; o <<= 1) {
        const u32 add = (t % 512) >= o ? v[t - o] : 0u;
        __syncthreads();
        v[t] += add;
        __syncthreads();
    }
    hist[t] = v[t] - hist[t];
}

__global__ void k_len_scatter(BatchWork w, u32 R, u32 *offs, u32 *sorted) {
    constexpr u32 FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    for (u32 cls = 0; cls < 2; cls++) {
        const u32 n = w.counters[cls];
        const u32 *list = w.baq_list + size_t(cls) * R;
        u32 *out = sorted + size_t(cls) * R;
        // the grid-stride loop runs the same trip count on every lane of a warp (lanes past n idle)
        const u32 stride = gridDim.x * blockDim.x;
        for (u32 base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
            const u32 i = base + lane;
            const bool in = i < n;
            const u32 r = in ? list[i] : 0;
            const u32 bin = in ? qlen_bin(w, r, cls) : 0xFFFFFFFFu;
            const u32 peers = __match_any_sync(FULL, bin);
            const int leader = __ffs(peers) - 1;
            u32 pos = 0;
            if (in && lane == leader) pos = atomicAdd(&offs[bin], u32(__popc(peers)));
            pos = __shfl_sync(FULL, pos, leader);
            if (in) out[pos + u32(__popc(peers & ((1u << lane) - 1)))] = r;
        }
    }
}

}  // namespace

void launch_sort_baq_lists(const BatchWork &w, u32 R, u32 max_class_reads, u32 *hist, u32 *sorted, cudaStream_t s) {
    if (!max_class_reads) return;
    cudaMemsetAsync(hist, 0, 1024 * sizeof(u32), s);
    u32 blocks = (max_class_reads + 255) / 256;
    if (blocks > 152 * 4) blocks = 152 * 4;
    k_len_hist<<<blocks, 256, 0, s>>>(w, R, hist);
    k_len_scan<<<1, 1024, 0, s>>>(hist);
    k_len_scatter<<<blocks, 256, 0, s>>>(w, R, hist, sorted);
    g_kernel_launches += 3;
}

void launch_cap(const DevBatch &b, const BatchWork &w, const u32 *list, const u32 *count, int exact, cudaStream_t s,
                u32 max_reads) {
    if (!max_reads) return;
    // one warp per read, 2 warps per block: small blocks also fit beside the BAQ kernels of the other band
    // class running on another stream
    u32 blocks = (max_reads + 1) / 2;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_cap<<<blocks, 64, 0, s>>>(b, w, list, count, exact);
    g_kernel_launches++;
}

}  // namespace fpg
