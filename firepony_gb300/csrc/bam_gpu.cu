// GPU decoding of BAM input (fpb_next_batch_device): the same batches as the host decoder, with the BGZF
// inflate and the record conversion on the device.
//
// Per batch, on the decoder's own CUDA stream:
//   1. the host parses BGZF block headers (sizes, CRC, ISIZE) and uploads the compressed bytes of whole blocks;
//   2. k_inflate: one thread per block decodes its DEFLATE stream (literals written, matches listed), the
//      decoders of a warp stepping in lockstep; k_resolve_crc: one warp per block, staged in shared memory,
//      resolves the matches in order and checks the block's CRC-32;
//   3. record location without a serial walk: the stream is cut into segments (one per block, plus the pieces
//      of the bytes carried over from the previous batch, whose record starts are known). k_seg_walk finds in
//      each segment a candidate first record start (a chain of plausible records reaching the segment's end)
//      and walks the chain to its exit (the first record start past the segment). k_seg_verify checks that
//      every exit lands on the next segment's candidate: then, by induction from the known first start, every
//      candidate is a true record start. Otherwise k_walk_serial walks the whole stream on one thread (the
//      slow path: it gives the same records, only later). The counts are scanned and k_seg_offsets lists the
//      record offsets;
//   4. k_rec_sizes, three exclusive scans, k_rec_convert (a warp per record: fixed fields, CIGAR, 4-bit bases,
//      qualities, RG tag), then read-group ids in order of first occurrence (k_rg_assign, k_rg_apply).
// Records past max_reads and a partial record at the end stay in the stream and are carried into the next
// batch's stream buffer (device to device), with their known record starts.
//
// Every device loop is bounded by a buffer length and every access is checked against its buffer: a corrupt
// file ends in an error status.
#include <unistd.h>

#include <thread>

#include "bam_internal.h"
#include "bgzf_inflate.cuh"

namespace fpb_detail {

namespace {

constexpr uint64_t NONE = ~0ull;
constexpr uint32_t NONE32 = 0xFFFFFFFFu;
constexpr int INF_WARPS_PER_SM = 4;  // k_inflate: target warps per SM (one per SM sub-partition)

enum DevError : uint32_t {
    DE_INFLATE = 1,    // index: block, detail: fpinf status
    DE_CRC = 2,        // index: block
    DE_SHORT = 3,      // a record shorter than its fixed fields
    DE_MALFORMED = 4,  // a record whose fields exceed its length (index: record)
    DE_TOO_LARGE = 5,  // a batch whose CIGAR, base or quality count exceeds 2^32
};

struct BlockDesc {
    uint64_t c_off;  // deflate data offset in the chunk's compressed bytes
    uint64_t u_off;  // output offset in the stream buffer
    uint64_t m_off;  // first match slot
    uint32_t c_len;  // deflate data bytes
    uint32_t isize;  // uncompressed bytes
    uint32_t crc;    // CRC-32 of the uncompressed bytes
    uint32_t pad;
};

struct SegDesc {
    uint64_t u;      // first byte of the segment
    uint64_t known;  // a record start known to be the first in the segment (== u), or NONE: search
};

struct Summary {
    uint32_t status, err_index, err_detail, ok;
    uint64_t total;           // complete records in the stream
    uint64_t end_of_records;  // just past the last complete record
    uint64_t carry_start;     // first record not taken (or end_of_records)
    uint64_t tot[3];          // CIGAR ops, padded bases, qualities of the taken records
};

__device__ __forceinline__ void set_error(Summary *s, uint32_t code, uint32_t index, uint32_t detail) {
    if (atomicCAS(&s->status, 0u, code) == 0u) {
        s->err_index = index;
        s->err_detail = detail;
    }
}

__host__ __device__ __forceinline__ uint32_t ld32(const uint8_t *p) {
    return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
}
__host__ __device__ __forceinline__ uint32_t ld16(const uint8_t *p) { return uint32_t(p[0]) | (uint32_t(p[1]) << 8); }

// ---- 2. inflate ----

// A warp of up to 32 block decoders (`dpw` per warp, chosen so that the SMs get several warps each: a decoder's
// steps are latency-bound). Each step decodes one symbol (or one block header) per thread; the vote after every
// step reconverges the warp, whose threads would otherwise drift apart at their first differing branch and run
// one at a time for the rest of their blocks.
__global__ void __launch_bounds__(32) k_inflate(const uint8_t *__restrict__ cin, const BlockDesc *blk, uint32_t nblk,
                                                uint32_t dpw, uint8_t *stream, uint32_t *matches, uint32_t *nmatch,
                                                Summary *sum) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    fpinf::Tables *tab = reinterpret_cast<fpinf::Tables *>(smem_raw);  // dpw tables
    const uint32_t lane = threadIdx.x, b = blockIdx.x * dpw + lane;
    const bool have = lane < dpw && b < nblk;
    fpinf::Work w;
    fpinf::Inflater f;
    if (have) {
        const BlockDesc d = blk[b];
        f.init(cin + d.c_off, d.c_len, stream + d.u_off, d.isize, matches + 2 * d.m_off,
               fpinf::match_capacity(d.isize));
    }
    bool run = have;
    while (__any_sync(0xffffffffu, run))
        if (run) run = f.step(tab[lane], w);
    if (!have) return;
    nmatch[b] = f.status == fpinf::OK ? f.nm : 0u;
    if (f.status != fpinf::OK) set_error(sum, DE_INFLATE, b, uint32_t(f.status));
}

// A warp per block, the block staged in shared memory: the matches are resolved (a lane per match, as many
// matches at a time as their sources allow; a copy reads bytes that earlier matches wrote, so shared memory keeps
// that chain short), then the CRC-32 of the block is taken as 32 lane segments combined by x^(8 * bytes after
// the segment), and the block is written back. Shared and global addresses share their offset mod 16, so the
// bulk moves as 16-byte words.
constexpr uint32_t RES_SMEM = 65536 + 16;

__global__ void __launch_bounds__(32) k_resolve_crc(const BlockDesc *blk, uint32_t nblk, uint8_t *stream,
                                                    const uint32_t *matches, const uint32_t *nmatch, Summary *sum) {
    extern __shared__ __align__(16) unsigned char sbuf[];
    __shared__ uint32_t crc_t[256];
    const uint32_t lane = threadIdx.x, wb = blockIdx.x;
    for (uint32_t k = lane; k < 256; k += 32) {
        uint32_t c = k;
        for (int j = 0; j < 8; j++) c = (c & 1) ? (c >> 1) ^ fpinf::CRC_POLY : c >> 1;
        crc_t[k] = c;
    }
    if (wb >= nblk) return;  // (the grid has one CTA per block)
    const BlockDesc d = blk[wb];
    uint8_t *out = stream + d.u_off;
    const uint32_t n = d.isize;  // at most 65536 (checked when the blocks are gathered)
    const uint32_t shift = uint32_t(reinterpret_cast<uintptr_t>(out) & 15u);
    uint8_t *sb = sbuf + shift;
    const uint32_t head = min(n, (16u - shift) & 15u), nw = (n - head) / 16u, tail0 = head + nw * 16u;
    uint4 *gw = reinterpret_cast<uint4 *>(out + head);
    uint4 *sw = reinterpret_cast<uint4 *>(sb + head);
    if (lane < head) sb[lane] = out[lane];
    for (uint32_t k = lane; k < nw; k += 32) sw[k] = gw[k];
    for (uint32_t k = tail0 + lane; k < n; k += 32) sb[k] = out[k];
    __syncwarp();
    // Matches, 32 at a time, a lane each, in rounds: a lane copies its match once every byte it reads is final,
    // i.e. its source ends at or below the lowest destination of the group's matches still pending before it
    // (destinations ascend with the lane; everything below that point is a literal or already resolved). The
    // lowest pending lane always qualifies, so every round resolves at least one match.
    const uint32_t nm = nmatch[wb];
    const uint32_t *m = matches + 2 * d.m_off;
    for (uint32_t j0 = 0; j0 < nm; j0 += 32) {
        const uint32_t j = j0 + lane;
        bool pending = j < nm;
        const uint32_t mp = pending ? m[2 * j] : 0xFFFFFFFFu, ml = pending ? m[2 * j + 1] : 0u;
        const uint32_t len = ml >> 16, dist = ml & 0xFFFFu;
        // (the decoder guarantees 1 <= dist <= mp and mp + len <= isize)
        const uint32_t src0 = mp - dist, src_end = src0 + (len < dist ? len : dist);
        while (__any_sync(0xffffffffu, pending)) {
            uint32_t lo = pending ? mp : 0xFFFFFFFFu;  // inclusive prefix minimum over the lanes
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, lo, o);
                if (lane >= uint32_t(o)) lo = t < lo ? t : lo;
            }
            uint32_t below = __shfl_up_sync(0xffffffffu, lo, 1);
            if (lane == 0) below = 0xFFFFFFFFu;
            const bool ready = pending && src_end <= below;
            if (ready) {
                uint32_t k = 0;
                for (uint32_t c = 0; c < len; c++) {
                    sb[mp + c] = sb[src0 + k];
                    k = k + 1 == dist ? 0u : k + 1;
                }
            }
            __syncwarp();
            pending = pending && !ready;
        }
    }
    const uint32_t seg = (n + 31) / 32;
    const uint32_t a = lane * seg < n ? lane * seg : n;
    const uint32_t e = a + seg < n ? a + seg : n;
    const uint32_t c = fpinf::crc_bytes(crc_t, sb + a, e - a);
    uint32_t term = fpinf::gf2_mulmod(fpinf::x8n_mod(n - e), c);
    for (int o = 16; o; o >>= 1) term ^= __shfl_xor_sync(0xffffffffu, term, o);
    // (a block that failed to inflate already holds the error: the first error is kept)
    if (lane == 0 && term != d.crc) set_error(sum, DE_CRC, wb, 0);
    if (nm == 0) return;  // literals and stored bytes only: the global copy is already complete
    if (lane < head) out[lane] = sb[lane];
    for (uint32_t k = lane; k < nw; k += 32) gw[k] = sw[k];
    for (uint32_t k = tail0 + lane; k < n; k += 32) out[k] = sb[k];
}

// ---- 3. record location ----

struct StreamView {
    const uint8_t *p;
    uint64_t end;
    int32_t n_targets;
};

__host__ __device__ __forceinline__ bool is_alpha(uint8_t c) { return (c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z'); }
__host__ __device__ __forceinline__ bool is_alnum(uint8_t c) { return is_alpha(c) || (c >= '0' && c <= '9'); }

// A record at o whose length prefix and body lie inside the stream and whose fields are those of a valid BAM
// record: reference ids in range, positions >= -1, a NUL-terminated printable name, CIGAR op codes 0..8 whose
// query length equals l_seq (when both are present), and aux fields that parse exactly to the record's end.
// Offsets inside real records (a few bytes off a record start, where small integer fields still read as
// plausible ones) fail the CIGAR or the aux check.
__host__ __device__ __forceinline__ bool plausible(const StreamView &s, uint64_t o, uint32_t bs) {
    const uint8_t *b = s.p + o + 4;
    const int32_t ref = int32_t(ld32(b)), pos = int32_t(ld32(b + 4)), nref = int32_t(ld32(b + 20)),
                  npos = int32_t(ld32(b + 24)), lseq = int32_t(ld32(b + 16));
    const uint32_t lname = b[8], ncig = ld16(b + 12);
    if (ref < -1 || ref >= s.n_targets || nref < -1 || nref >= s.n_targets || pos < -1 || npos < -1 || lseq < 0)
        return false;
    if (lname < 1) return false;
    const uint64_t need = 32ull + lname + 4ull * ncig + (uint64_t(lseq) + 1) / 2 + uint64_t(lseq);
    if (need > bs) return false;
    const uint8_t *nm = b + 32;
    if (nm[lname - 1] != 0) return false;
    for (uint32_t k = 0; k + 1 < lname; k++)
        if (nm[k] < 33 || nm[k] > 126) return false;
    if (ncig > 0) {
        const uint8_t *cg = nm + lname;
        uint64_t qlen = 0;
        for (uint32_t k = 0; k < ncig; k++) {
            const uint32_t w = ld32(cg + 4 * k), op = w & 15u;
            if (op > 8) return false;
            if (op == 0 || op == 1 || op == 4 || op == 7 || op == 8) qlen += w >> 4;
        }
        if (lseq > 0 && qlen != uint64_t(lseq)) return false;
    }
    const uint8_t *a = b + need, *end = b + bs;
    while (a < end) {
        if (end - a < 4 || !is_alpha(a[0]) || !is_alnum(a[1])) return false;
        const uint8_t type = a[2];
        a += 3;
        uint64_t sz = 0;
        switch (type) {
        case 'A': case 'c': case 'C': sz = 1; break;
        case 's': case 'S': sz = 2; break;
        case 'i': case 'I': case 'f': sz = 4; break;
        case 'Z': case 'H':
            while (a < end && *a) a++;
            if (a == end) return false;  // no terminating NUL
            sz = 1;
            break;
        case 'B': {
            if (end - a < 5) return false;
            const uint8_t sub = a[0];
            const uint64_t es = (sub == 'c' || sub == 'C') ? 1 : (sub == 's' || sub == 'S') ? 2
                                : (sub == 'i' || sub == 'I' || sub == 'f') ? 4 : 0;
            if (es == 0) return false;
            sz = 5 + es * uint64_t(ld32(a + 1));
            break;
        }
        default: return false;
        }
        if (uint64_t(end - a) < sz) return false;
        a += sz;
    }
    return true;
}

// Walks records from o while their start is below limit. exit: the first start at or past limit, or the start
// of a record that does not fit in the stream (terminal). Returns false on a record that is not plausible
// (when check) or shorter than its fixed fields.
__host__ __device__ __forceinline__ bool walk(const StreamView &s, uint64_t o, uint64_t limit, bool check,
                                              uint32_t &count, uint64_t &exit, bool &terminal) {
    count = 0;
    terminal = false;
    while (o < limit) {
        if (s.end - o < 4) { terminal = true; break; }
        const uint32_t bs = ld32(s.p + o);
        if (bs < 32) return false;
        if (s.end - o - 4 < bs) { terminal = true; break; }
        if (check && !plausible(s, o, bs)) return false;
        count++;
        o += 4 + uint64_t(bs);
    }
    if (o >= s.end) terminal = true;
    exit = o;
    return true;
}

constexpr uint32_t SEARCH_HOPS = 1u << 16;  // record hops a candidate search may spend before giving up

// A warp per segment. Candidate search: the lanes test 32 consecutive offsets for a plausible record; for each
// plausible offset in order, the whole warp follows its record chain in lockstep (the same bytes on every lane)
// and takes it when the chain stays plausible to the segment's end. Then the warp walks the chain from the
// candidate (or the known start) to its exit.
__global__ void __launch_bounds__(256) k_seg_walk(StreamView s, const SegDesc *seg, uint32_t nseg, uint64_t *cand,
                                                  uint64_t *exitp, uint32_t *count, uint8_t *term, uint8_t *bad) {
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= nseg) return;  // whole warps leave together
    const uint64_t u = seg[i].u, lim = i + 1 < nseg ? seg[i + 1].u : s.end;
    uint64_t c = seg[i].known;
    if (c == NONE) {
        uint32_t hops = 0;
        for (uint64_t base = u; base < lim && c == NONE && hops < SEARCH_HOPS; base += 32) {
            const uint64_t o = base + lane;
            bool ok = o < lim && s.end - o >= 4;
            if (ok) {
                const uint32_t bs = ld32(s.p + o);
                ok = bs >= 32 && s.end - o - 4 >= bs && plausible(s, o, bs);
            }
            uint32_t mask = __ballot_sync(0xffffffffu, ok);
            while (mask && c == NONE && hops < SEARCH_HOPS) {
                const uint64_t co = base + uint32_t(__ffs(mask) - 1);
                mask &= mask - 1;
                // the chain from co must stay plausible up to the segment's end
                uint64_t q = co;
                bool good = true;
                while (q < lim && hops < SEARCH_HOPS) {
                    hops++;
                    if (s.end - q < 4) break;
                    const uint32_t b2 = ld32(s.p + q);
                    if (b2 < 32) { good = false; break; }
                    if (s.end - q - 4 < b2) break;
                    if (!plausible(s, q, b2)) { good = false; break; }
                    q += 4 + uint64_t(b2);
                }
                if (good && (q >= lim || s.end - q < 4 || s.end - q - 4 < ld32(s.p + q))) c = co;
            }
        }
    }
    uint32_t n = 0;
    uint64_t x = 0;
    bool t = false, okw = true;
    if (c != NONE) okw = walk(s, c, lim, seg[i].known == NONE, n, x, t);
    if (lane == 0) {
        cand[i] = c;
        exitp[i] = x;
        count[i] = n;
        term[i] = t;
        bad[i] = !okw;
    }
}

// one CTA: checks the candidate chain, scans the per-segment counts into record bases
__global__ void __launch_bounds__(1024) k_seg_verify(StreamView s, const SegDesc *seg, uint32_t nseg,
                                                     const uint64_t *cand, const uint64_t *exitp,
                                                     const uint32_t *count, const uint8_t *term,
                                                     const uint8_t *bad, uint64_t *base, Summary *sum) {
    __shared__ int ok;
    __shared__ unsigned long long last_exit;
    __shared__ uint64_t part[1024];
    if (threadIdx.x == 0) {
        ok = nseg > 0 && cand[0] != NONE;
        last_exit = 0;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nseg; i += blockDim.x) {
        if (cand[i] == NONE) continue;
        if (bad[i]) { ok = 0; continue; }
        atomicMax(&last_exit, (unsigned long long)exitp[i]);
        if (term[i]) {
            for (uint32_t v = i + 1; v < nseg; v++)
                if (cand[v] != NONE) { ok = 0; break; }
            continue;
        }
        // the segment holding the exit: every segment before it has no record start, it starts at the exit
        const uint64_t x = exitp[i];
        uint32_t t = i + 1;
        while (t + 1 < nseg && seg[t + 1].u <= x) {
            if (cand[t] != NONE) ok = 0;
            t++;
        }
        if (t >= nseg || cand[t] != x) ok = 0;
    }
    // exclusive scan of the counts (contiguous slices per thread)
    const uint32_t per = (nseg + blockDim.x - 1) / blockDim.x;
    const uint32_t a = threadIdx.x * per, z = a + per < nseg ? a + per : nseg;
    uint64_t sum_local = 0;
    for (uint32_t i = a; i < z; i++) sum_local += cand[i] != NONE ? count[i] : 0u;
    part[threadIdx.x] = sum_local;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t run = 0;
        for (uint32_t k = 0; k < blockDim.x; k++) {
            const uint64_t v = part[k];
            part[k] = run;
            run += v;
        }
        sum->total = run;
        sum->ok = ok;
        sum->end_of_records = last_exit;
        sum->carry_start = last_exit;
    }
    __syncthreads();
    uint64_t run = part[threadIdx.x];
    for (uint32_t i = a; i < z; i++) {
        base[i] = run;
        run += cand[i] != NONE ? count[i] : 0u;
    }
}

__global__ void k_seg_offsets(StreamView s, const SegDesc *seg, uint32_t nseg, const uint64_t *cand,
                              const uint64_t *base, uint64_t take, uint64_t *rec_off, Summary *sum) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nseg || !sum->ok || cand[i] == NONE) return;
    const uint64_t lim = i + 1 < nseg ? seg[i + 1].u : s.end;
    uint64_t o = cand[i], g = base[i];
    while (o < lim && s.end - o >= 4) {
        const uint32_t bs = ld32(s.p + o);
        if (bs < 32 || s.end - o - 4 < bs) break;
        if (g < take) rec_off[g] = o;
        else if (g == take) sum->carry_start = o;
        g++;
        o += 4 + uint64_t(bs);
    }
}

// the slow path: one thread walks every record (used only when the candidate chain did not verify)
__global__ void k_walk_serial(StreamView s, uint64_t take, uint64_t cap, uint64_t *rec_off, Summary *sum) {
    if (sum->ok) return;
    uint64_t o = 0, g = 0, carry = NONE;
    while (s.end - o >= 4) {
        const uint32_t bs = ld32(s.p + o);
        if (bs < 32) {
            set_error(sum, DE_SHORT, uint32_t(g), 0);
            return;
        }
        if (s.end - o - 4 < bs) break;
        if (g < take && g < cap) rec_off[g] = o;
        else if (g == take) carry = o;
        g++;
        o += 4 + uint64_t(bs);
    }
    sum->total = g;
    sum->end_of_records = o;
    sum->carry_start = carry == NONE ? o : carry;
}

// ---- 4. records ----

__global__ void k_rec_sizes(StreamView s, const uint64_t *rec_off, uint32_t n, uint32_t *clen, uint32_t *rlen,
                            uint32_t *qlen, uint32_t *symcnt, Summary *sum) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t o = rec_off[i];
    const uint32_t bs = ld32(s.p + o);
    const uint8_t *b = s.p + o + 4;
    const uint32_t lname = b[8], ncig = ld16(b + 12), lseq = ld32(b + 16);
    const uint64_t need = 32ull + lname + 4ull * ncig + (uint64_t(lseq) + 1) / 2 + uint64_t(lseq);
    const bool good = need <= bs;
    if (!good) set_error(sum, DE_MALFORMED, i, 0);
    clen[i] = good ? ncig : 0u;
    rlen[i] = good ? lseq : 0u;
    qlen[i] = good ? lseq : 0u;
    symcnt[i] = good ? (lseq + 7u) / 8u * 8u : 0u;
}

// exclusive scans of three u32 arrays (blockIdx.y picks the array), 4096 elements per CTA, in three phases
constexpr int SCAN_T = 1024, SCAN_PER = 4, SCAN_TILE = SCAN_T * SCAN_PER;

__device__ __forceinline__ uint64_t block_excl_scan(uint64_t v, uint64_t *sh, uint64_t &total) {
    // Hillis-Steele over the CTA's threads
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < SCAN_T; o <<= 1) {
        const uint64_t add = threadIdx.x >= unsigned(o) ? sh[threadIdx.x - o] : 0ull;
        __syncthreads();
        sh[threadIdx.x] += add;
        __syncthreads();
    }
    total = sh[SCAN_T - 1];
    const uint64_t incl = sh[threadIdx.x];
    __syncthreads();
    return incl - v;
}

struct Scan3 {
    const uint32_t *in[3];
    uint32_t *out[3];
};

__global__ void __launch_bounds__(SCAN_T) k_scan_tiles(Scan3 a, uint32_t n, uint64_t *tile_sum) {
    __shared__ uint64_t sh[SCAN_T];
    const uint32_t y = blockIdx.y, base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER;
    uint64_t v = 0;
    for (int k = 0; k < SCAN_PER; k++)
        if (base + k < n) v += a.in[y][base + k];
    uint64_t tot;
    block_excl_scan(v, sh, tot);
    if (threadIdx.x == 0) tile_sum[size_t(y) * gridDim.x + blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_T) k_scan_top(uint64_t *tile_sum, uint32_t ntiles, Summary *sum) {
    __shared__ uint64_t sh[SCAN_T];
    const uint32_t y = blockIdx.x;
    uint64_t carry = 0;
    for (uint32_t t0 = 0; t0 < ntiles; t0 += SCAN_T) {
        const uint32_t t = t0 + threadIdx.x;
        const uint64_t v = t < ntiles ? tile_sum[size_t(y) * ntiles + t] : 0ull;
        uint64_t tot;
        const uint64_t ex = block_excl_scan(v, sh, tot);
        if (t < ntiles) tile_sum[size_t(y) * ntiles + t] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        sum->tot[y] = carry;
        if (carry > 0xFFFFFFFFull) set_error(sum, DE_TOO_LARGE, y, 0);
    }
}

__global__ void __launch_bounds__(SCAN_T) k_scan_apply(Scan3 a, uint32_t n, const uint64_t *tile_sum) {
    __shared__ uint64_t sh[SCAN_T];
    const uint32_t y = blockIdx.y, base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER;
    uint32_t vals[SCAN_PER];
    uint64_t v = 0;
    for (int k = 0; k < SCAN_PER; k++) {
        vals[k] = base + k < n ? a.in[y][base + k] : 0u;
        v += vals[k];
    }
    uint64_t tot;
    uint64_t run = block_excl_scan(v, sh, tot) + tile_sum[size_t(y) * gridDim.x + blockIdx.x];
    for (int k = 0; k < SCAN_PER; k++) {
        if (base + k < n) a.out[y][base + k] = uint32_t(run);
        run += vals[k];
    }
}

struct OutArrays {
    uint16_t *chrom;
    uint32_t *astart, *astop, *mstart;
    int32_t *isize;
    uint32_t *cigars, *cstart, *clen;
    uint32_t *reads, *rstart, *rlen;
    uint8_t *quals;
    uint32_t *qstart, *qlen;
    uint16_t *flags;
    uint8_t *mapq;
    uint32_t *rg;
};

struct RgTables {
    const uint8_t *id_bytes;    // @RG ID strings, concatenated
    const uint32_t *id_off;     // n_ids + 1 offsets
    const uint32_t *id_name;    // name index of each ID
    uint32_t n_ids;
    uint32_t *id_of_name;       // read-group id of each name, NONE32 until first seen
    uint32_t *first_seen;       // first record (this batch) of each name without an id
    uint32_t n_names;
};

// RG:Z value of a record's aux data, as the host decoder's find_rg: returns its offset (or NONE) and length
__device__ uint64_t find_rg_dev(const uint8_t *p, uint64_t a, uint64_t end, uint32_t &len) {
    while (end >= 3 && a <= end - 3) {
        const uint8_t t0 = p[a], t1 = p[a + 1], type = p[a + 2];
        a += 3;
        uint64_t sz = 0;
        switch (type) {
        case 'A': case 'c': case 'C': sz = 1; break;
        case 's': case 'S': sz = 2; break;
        case 'i': case 'I': case 'f': sz = 4; break;
        case 'Z': case 'H': {
            uint64_t q = a;
            while (q < end && p[q]) q++;
            if (t0 == 'R' && t1 == 'G' && type == 'Z') {
                len = uint32_t(q - a);
                return a;
            }
            a = q + 1;
            continue;
        }
        case 'B': {
            if (a + 5 > end) return NONE;
            const uint8_t sub = p[a];
            const uint64_t n = ld32(p + a + 1);
            const uint64_t es = (sub == 'c' || sub == 'C') ? 1 : (sub == 's' || sub == 'S') ? 2 : 4;
            a += 5 + es * n;
            continue;
        }
        default: return NONE;
        }
        a += sz;
    }
    return NONE;
}

// a warp per record
__global__ void __launch_bounds__(256) k_rec_convert(StreamView s, const uint64_t *rec_off, uint32_t n,
                                                     const uint16_t *contig_of_target, uint32_t ntarg,
                                                     OutArrays out, RgTables rg, uint32_t *rg_name_of_read) {
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= n) return;
    const uint64_t o = rec_off[i];
    const uint8_t *b = s.p + o + 4;
    const uint32_t bs = ld32(s.p + o);
    const uint32_t lname = b[8], ncig = ld16(b + 12), lseq = ld32(b + 16);
    if (32ull + lname + 4ull * ncig + (uint64_t(lseq) + 1) / 2 + uint64_t(lseq) > bs) return;  // flagged by sizes
    const uint8_t *cig = b + 32 + lname;
    const uint8_t *seq = cig + 4 * ncig;
    const uint8_t *qual = seq + (lseq + 1) / 2;
    // CIGAR: op B has no firepony op and becomes X; reference-consuming ops (M, D, N, =, X) give the end
    const uint32_t cs = out.cstart[i];
    uint32_t rref = 0;
    for (uint32_t c = lane; c < ncig; c += 32) {
        const uint32_t w = ld32(cig + 4 * c), op = w & 0xF;
        if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) rref += w >> 4;
        const uint32_t fop = op == 9 ? 8u : op;
        out.cigars[cs + c] = ((w >> 4) & 0xFFFFFFu) | (fop << 24);
    }
    for (int k = 16; k; k >>= 1) rref += __shfl_xor_sync(0xffffffffu, rref, k);
    // bases: a word is four BAM bytes with their nibbles swapped; an odd length leaves the last nibble zero
    const uint32_t nbytes = (lseq + 1) / 2, words = (lseq + 7) / 8;
    uint32_t *dst = out.reads + out.rstart[i] / 8;
    for (uint32_t wd = lane; wd < words; wd += 32) {
        uint32_t word = 0;
        for (uint32_t k = 0; k < 4; k++) {
            const uint32_t j = wd * 4 + k;
            if (j < nbytes) {
                const uint32_t v = seq[j];
                word |= (((v & 15u) << 4) | (v >> 4)) << (8 * k);
            }
        }
        if ((lseq & 1) && wd == (lseq - 1) / 8) word &= ~(0xFu << (4 * (lseq & 7)));
        dst[wd] = word;
    }
    const uint32_t qs = out.qstart[i];
    for (uint32_t j = lane; j < lseq; j += 32) out.quals[qs + j] = qual[j];
    if (lane == 0) {
        const int32_t tid = int32_t(ld32(b)), pos = int32_t(ld32(b + 4));
        const uint32_t flag = ld16(b + 14);
        out.chrom[i] = (tid >= 0 && uint32_t(tid) < ntarg) ? contig_of_target[tid] : uint16_t(0xFFFF);
        out.astart[i] = uint32_t(pos);
        out.astop[i] = (!(flag & 4) && ncig > 0) ? uint32_t(pos) + rref - 1 : uint32_t(pos);
        out.mstart[i] = ld32(b + 24);
        out.isize[i] = int32_t(ld32(b + 28));
        out.flags[i] = uint16_t(flag);
        out.mapq[i] = b[9];
        // read group: the RG:Z value looked up among the header's @RG IDs
        uint32_t len = 0, name = NONE32;
        const uint64_t at = find_rg_dev(s.p, o + 4 + 32 + lname + 4ull * ncig + nbytes + lseq, o + 4 + bs, len);
        if (at != NONE) {
            for (uint32_t h = 0; h < rg.n_ids; h++) {
                const uint32_t a = rg.id_off[h], l = rg.id_off[h + 1] - a;
                if (l != len) continue;
                uint32_t k = 0;
                while (k < l && rg.id_bytes[a + k] == s.p[at + k]) k++;
                if (k == l) {
                    name = rg.id_name[h];
                    break;
                }
            }
        }
        rg_name_of_read[i] = name;
        if (name != NONE32 && rg.id_of_name[name] == NONE32) atomicMin(&rg.first_seen[name], i);
    }
}

// ids for the names first seen in this batch, in order of their first record
__global__ void k_rg_assign(RgTables rg, uint32_t *next_id) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (uint32_t round = 0; round < rg.n_names; round++) {
        uint32_t best = NONE32, bn = NONE32;
        for (uint32_t k = 0; k < rg.n_names; k++)
            if (rg.id_of_name[k] == NONE32 && rg.first_seen[k] < best) {
                best = rg.first_seen[k];
                bn = k;
            }
        if (bn == NONE32) break;
        rg.id_of_name[bn] = (*next_id)++;
    }
    for (uint32_t k = 0; k < rg.n_names; k++) rg.first_seen[k] = NONE32;
}

__global__ void k_rg_apply(const uint32_t *rg_name_of_read, uint32_t n, const uint32_t *id_of_name, uint32_t *rg) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t nm = rg_name_of_read[i];
    rg[i] = nm == NONE32 ? NONE32 : id_of_name[nm];
}

}  // namespace

// ---- host side ----

namespace {

template <typename T> struct DevBuf {
    T *p = nullptr;
    size_t cap = 0;  // elements
    bool ensure(size_t n) {
        if (p && n <= cap) return true;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(n + n / 4, 256);
        if (cudaMalloc(&p, want * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return false;
        }
        cap = want;
        return true;
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

struct OutSet {
    DevBuf<uint16_t> chrom, flags;
    DevBuf<uint32_t> astart, astop, mstart, cigars, cstart, clen, reads, rstart, rlen, qstart, qlen, rg;
    DevBuf<int32_t> isize;
    DevBuf<uint8_t> quals, mapq;
    bool ensure_reads(size_t n) {
        return chrom.ensure(n) && flags.ensure(n) && astart.ensure(n) && astop.ensure(n) && mstart.ensure(n) &&
               cstart.ensure(n) && clen.ensure(n) && rstart.ensure(n) && rlen.ensure(n) && qstart.ensure(n) &&
               qlen.ensure(n) && rg.ensure(n) && isize.ensure(n) && mapq.ensure(n);
    }
};

}  // namespace

struct DeviceDecoder {
    cudaStream_t st = nullptr;
    int num_sms = 0;
    // compressed input, page-locked: [pos, len) not yet used
    uint8_t *slab = nullptr;
    size_t slab_cap = 0, slab_len = 0, slab_pos = 0;
    bool file_eof = false;
    int fd = -1;        // the reader's file, read with pread from foff on
    uint64_t foff = 0;
    DevBuf<uint8_t> cin;
    DevBuf<uint8_t> stream[2];
    int cur = 0;
    uint64_t carry_off = 0, carry_len = 0;  // in stream[cur]
    std::vector<uint64_t> carry_known;      // record starts in the carry (relative to carry_off), ascending
    DevBuf<BlockDesc> blk;
    DevBuf<SegDesc> seg;
    DevBuf<uint32_t> matches, nmatch, count, symcnt, rgname;
    DevBuf<uint64_t> cand, exitp, base, rec_off, tile_sum;
    DevBuf<uint8_t> term, bad;
    DevBuf<Summary> sum;
    DevBuf<uint16_t> ctmap;
    // read groups
    DevBuf<uint8_t> id_bytes;
    DevBuf<uint32_t> id_off, id_name, id_of_name, first_seen, next_id;
    std::vector<std::string> names;
    uint32_t n_ids = 0;
    OutSet sets[FPB_BUFFER_SETS];
    int next_set = 0;
    double est = 512.0;  // stream bytes per record
    std::vector<BlockDesc> hblk;
    std::vector<SegDesc> hseg;
    std::vector<uint64_t> hcand;
    ~DeviceDecoder() {
        if (slab) cudaFreeHost(slab);
        if (st) cudaStreamDestroy(st);
    }
};

void destroy_device_decoder(DeviceDecoder *d) {
    if (d && d->st) cudaStreamSynchronize(d->st);
    delete d;
}

namespace {

int64_t dfail(fpb_reader *r, const std::string &m) {
    r->err = m;
    return -1;
}

bool grow_slab(DeviceDecoder *d, size_t want) {
    if (want <= d->slab_cap) return true;
    const size_t cap = std::max(want, d->slab_cap * 2);
    uint8_t *p = nullptr;
    if (cudaHostAlloc(reinterpret_cast<void **>(&p), cap, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (d->slab_len) memcpy(p, d->slab, d->slab_len);
    if (d->slab) cudaFreeHost(d->slab);
    d->slab = p;
    d->slab_cap = cap;
    return true;
}

// Reads the next READ_CHUNK bytes of the file into the slab (growing it by doubling), split into pieces read by
// parallel pread calls (page-cache copies scale with threads); false at the end of the file or when memory
// runs out. Chunks are modest so that the unused tail moved to the slab's front at the next batch stays small.
constexpr size_t READ_CHUNK = 16u << 20, READ_PIECE_MIN = 2u << 20;

bool read_more_dev(fpb_reader *r, DeviceDecoder *d) {
    if (d->file_eof) return false;
    if (d->slab_cap - d->slab_len < READ_CHUNK && !grow_slab(d, d->slab_len + READ_CHUNK)) return false;
    const size_t want = READ_CHUNK;
    const int np = int(std::max<size_t>(1, std::min<size_t>(size_t(std::max(1, r->threads)), want / READ_PIECE_MIN)));
    const size_t piece = (want + np - 1) / np;
    std::vector<size_t> got(np, 0);
    std::vector<std::thread> th;
    auto read_piece = [&](int k) {
        const size_t a = size_t(k) * piece, z = std::min(want, a + piece);
        size_t done = 0;
        while (a + done < z) {
            const ssize_t n = pread(d->fd, d->slab + d->slab_len + a + done, z - a - done, off_t(d->foff + a + done));
            if (n <= 0) break;  // end of file (or a read error, treated as the end)
            done += size_t(n);
        }
        got[k] = done;
    };
    const double t0 = now_s();
    for (int k = 1; k < np; k++) th.emplace_back(read_piece, k);
    read_piece(0);
    for (auto &t : th) t.join();
    r->stats.seconds_read += now_s() - t0;
    // the bytes read are the pieces up to the first short one
    size_t total = 0;
    for (int k = 0; k < np; k++) {
        total += got[k];
        if (size_t(k) * piece + got[k] < std::min(want, size_t(k + 1) * piece)) {
            d->file_eof = true;
            break;
        }
    }
    d->slab_len += total;
    d->foff += total;
    r->stats.compressed_bytes += total;
    return total > 0;
}

bool setup(fpb_reader *r, DeviceDecoder *d) {
    if (cudaStreamCreateWithFlags(&d->st, cudaStreamNonBlocking) != cudaSuccess) return false;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&d->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || d->num_sms < 1)
        return false;
    if (cudaFuncSetAttribute(k_inflate, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(32 * sizeof(fpinf::Tables))) != cudaSuccess)
        return false;
    if (cudaFuncSetAttribute(k_resolve_crc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(RES_SMEM)) != cudaSuccess)
        return false;
    // compressed bytes the host decoder has read but not inflated
    if (!grow_slab(d, std::max<size_t>(r->cbuf.size() - r->cpos, 64u << 20))) return false;
    memcpy(d->slab, r->cbuf.data() + r->cpos, r->cbuf.size() - r->cpos);
    d->slab_len = r->cbuf.size() - r->cpos;
    d->file_eof = r->eof_in;
    d->fd = fileno(r->f);
    const off_t pos = ftello(r->f);  // past the bytes the host decoder has read (the slab holds the unused ones)
    if (d->fd < 0 || pos < 0) return false;
    d->foff = uint64_t(pos);
    // records the host decoder has inflated (after the header): the first carry. Record starts about every
    // 64 KiB become known segment starts; their mean size is the first estimate
    const uint8_t *u = r->ubuf.data() + r->upos;
    const size_t ul = r->ubuf.size() - r->upos;
    d->carry_off = 0;
    d->carry_len = ul;
    d->carry_known.clear();
    if (ul) {
        if (!d->stream[0].ensure(ul)) return false;
        if (cudaMemcpy(d->stream[0].p, u, ul, cudaMemcpyHostToDevice) != cudaSuccess) return false;
        size_t o = 0, n = 0, last = 0;
        d->carry_known.push_back(0);
        while (ul - o >= 4) {
            const uint32_t bs = rd32(u + o);
            if (bs < 32 || ul - o - 4 < bs) break;
            if (o - last >= (64u << 10)) {
                d->carry_known.push_back(o);
                last = o;
            }
            o += 4 + size_t(bs);
            n++;
        }
        if (n >= 16) d->est = double(o) / double(n);
    }
    d->cur = 0;
    // read groups: the header's @RG IDs and their names (PU if present, else ID)
    std::vector<std::string> ids;
    std::vector<uint32_t> id_name;
    std::unordered_map<std::string, uint32_t> name_idx;
    for (const auto &kv : r->rg_name_of_id) {
        ids.push_back(kv.first);
        auto it = name_idx.find(kv.second);
        if (it == name_idx.end()) {
            it = name_idx.emplace(kv.second, uint32_t(d->names.size())).first;
            d->names.push_back(kv.second);
        }
        id_name.push_back(it->second);
    }
    d->n_ids = uint32_t(ids.size());
    std::vector<uint8_t> bytes;
    std::vector<uint32_t> off{0};
    for (const auto &s : ids) {
        bytes.insert(bytes.end(), s.begin(), s.end());
        off.push_back(uint32_t(bytes.size()));
    }
    const size_t nn = d->names.size();
    std::vector<uint32_t> ion(nn, NONE32), fs(nn, NONE32);
    for (size_t k = 0; k < nn; k++) {  // names that already have an id keep it
        auto it = r->rg_index.find(d->names[k]);
        if (it != r->rg_index.end()) ion[k] = it->second;
    }
    const uint32_t nid = uint32_t(r->rg_names.size());
    if (!d->id_bytes.ensure(bytes.size() + 1) || !d->id_off.ensure(off.size()) || !d->id_name.ensure(id_name.size() + 1) ||
        !d->id_of_name.ensure(nn + 1) || !d->first_seen.ensure(nn + 1) || !d->next_id.ensure(1) || !d->sum.ensure(1))
        return false;
    bool ok = true;
    if (!bytes.empty()) ok &= cudaMemcpy(d->id_bytes.p, bytes.data(), bytes.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    ok &= cudaMemcpy(d->id_off.p, off.data(), off.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    if (!id_name.empty()) ok &= cudaMemcpy(d->id_name.p, id_name.data(), id_name.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    if (nn) {
        ok &= cudaMemcpy(d->id_of_name.p, ion.data(), nn * 4, cudaMemcpyHostToDevice) == cudaSuccess;
        ok &= cudaMemcpy(d->first_seen.p, fs.data(), nn * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    ok &= cudaMemcpy(d->next_id.p, &nid, 4, cudaMemcpyHostToDevice) == cudaSuccess;
    return ok;
}

// Appends whole BGZF blocks after slab_pos until the stream would hold `target` bytes. Returns -1 on a
// malformed block (message set), else the number of blocks; *eof when the file has no more blocks.
int gather(fpb_reader *r, DeviceDecoder *d, uint64_t target, uint64_t &chunk_begin, uint64_t &chunk_bytes,
           uint64_t &u_total, uint64_t &m_total, bool &eof) {
    // keep only the unused bytes, at the front of the slab
    if (d->slab_pos) {
        memmove(d->slab, d->slab + d->slab_pos, d->slab_len - d->slab_pos);
        d->slab_len -= d->slab_pos;
        d->slab_pos = 0;
    }
    chunk_begin = 0;
    d->hblk.clear();
    uint64_t u = d->carry_len, m = 0;
    size_t p = 0;
    eof = false;
    const size_t max_blocks = 1u << 20;
    while (u < target && d->hblk.size() < max_blocks) {
        if (d->slab_len - p < 18) {
            if (read_more_dev(r, d)) continue;
            if (d->slab_len - p == 0) {
                eof = true;
                break;
            }
            r->err = "truncated BGZF block";
            return -1;
        }
        const uint8_t *h = d->slab + p;
        if (h[0] != 31 || h[1] != 139 || h[2] != 8 || !(h[3] & 4)) {
            r->err = "not a BGZF block";
            return -1;
        }
        const uint32_t xlen = rd16(h + 10);
        if (d->slab_len - p < size_t(12) + xlen) {
            if (read_more_dev(r, d)) continue;
            r->err = "truncated BGZF block";
            return -1;
        }
        size_t bsize = 0;
        for (size_t x = 0; x + 4 <= xlen;) {
            const uint8_t *sf = h + 12 + x;
            const uint16_t slen = rd16(sf + 2);
            if (sf[0] == 66 && sf[1] == 67 && slen == 2) bsize = size_t(rd16(sf + 4)) + 1;
            x += 4 + slen;
        }
        if (bsize == 0) {
            r->err = "BGZF block without a BC field";
            return -1;
        }
        if (bsize < size_t(12) + xlen + 8) {
            r->err = "BGZF block shorter than its header";
            return -1;
        }
        if (d->slab_len - p < bsize) {
            if (read_more_dev(r, d)) continue;
            r->err = "truncated BGZF block";
            return -1;
        }
        BlockDesc b;
        b.c_off = p + 12 + xlen;
        b.c_len = uint32_t(bsize - 12 - xlen - 8);
        b.crc = rd32(h + bsize - 8);
        b.isize = rd32(h + bsize - 4);
        b.u_off = u;
        b.m_off = m;
        b.pad = 0;
        if (b.isize > 65536) {
            r->err = "BGZF block larger than 64 KiB";
            return -1;
        }
        d->hblk.push_back(b);
        u += b.isize;
        m += fpinf::match_capacity(b.isize);
        p += bsize;
    }
    if (!eof && d->slab_len - p == 0 && d->file_eof) eof = true;
    d->slab_pos = p;
    chunk_bytes = p;
    u_total = u;
    m_total = m;
    return int(d->hblk.size());
}

template <typename K, typename... A> bool launch(K k, dim3 g, dim3 b, size_t sh, cudaStream_t st, A... a) {
    if (g.x == 0 || g.y == 0) return true;
    k<<<g, b, sh, st>>>(a...);
    return cudaGetLastError() == cudaSuccess;
}

std::string device_error(const Summary &s) {
    switch (s.status) {
    case DE_INFLATE: return "corrupt BGZF block (deflate status " + std::to_string(s.err_detail) + ")";
    case DE_CRC: return "corrupt BGZF block (CRC mismatch)";
    case DE_SHORT: return "BAM record shorter than its fixed fields";
    case DE_MALFORMED: return "malformed BAM record (its fields exceed its length)";
    case DE_TOO_LARGE: return "batch too large";
    default: return "device decoding error " + std::to_string(s.status);
    }
}

}  // namespace

}  // namespace fpb_detail

using namespace fpb_detail;

static int64_t next_batch_device(fpb_reader *r, uint32_t max_reads, fp_batch_view *v);

extern "C" int64_t fpb_next_batch_device(fpb_reader *r, uint32_t max_reads, fp_batch_view *v) {
    if (!r || !v) return -1;
    if (r->failed) {  // after an error the carried stream and the file position are undefined
        memset(v, 0, sizeof(*v));
        r->err = "the reader failed earlier: " + r->failure;
        return -1;
    }
    const double t0 = now_s(), read0 = r->stats.seconds_read;
    int64_t n;
    try {  // (no C++ exception crosses the C ABI)
        n = next_batch_device(r, max_reads, v);
    } catch (...) {
        r->err.assign("host alloc fail");
        n = -1;
    }
    r->stats.seconds_decode += (now_s() - t0) - (r->stats.seconds_read - read0);
    if (n < 0 && r->mode == 2 && !r->failed) {  // (a call in the wrong mode leaves the reader usable)
        r->failed = true;
        r->failure = r->err;
    }
    if (n > 0) {
        r->stats.batches++;
        r->stats.records += uint64_t(n);
    }
    return n;
}

static int64_t next_batch_device(fpb_reader *r, uint32_t max_reads, fp_batch_view *v) {
    memset(v, 0, sizeof(*v));
    if (r->mode == 1) return dfail(r, "the reader decodes on the host (fpb_next_batch)");
    r->mode = 2;
    if (!r->dev) {
        r->dev = new DeviceDecoder();
        if (!setup(r, r->dev)) {
            destroy_device_decoder(r->dev);
            r->dev = nullptr;
            return dfail(r, "GPU decoder setup failed");
        }
    }
    DeviceDecoder *d = r->dev;
    if (max_reads == 0) return 0;
    const cudaStream_t st = d->st;
    const int32_t ntarg = int32_t(std::min<size_t>(r->target_names.size(), 0x7FFFFFFF));
    Summary hs;
    uint64_t u_total = 0, take = 0;
    int nxt = 0;
    StreamView sv{};
    for (;;) {
        // 1. blocks for about 10% more records than asked for
        const uint64_t target = uint64_t(d->est * double(max_reads) * 1.1) + (512u << 10);
        uint64_t chunk_begin = 0, chunk_bytes = 0, m_total = 0;
        bool eof = false;
        const int nblk = gather(r, d, std::max<uint64_t>(target, d->carry_len + 1), chunk_begin, chunk_bytes,
                                u_total, m_total, eof);
        if (nblk < 0) return -1;
        // segments: known record starts in the carry, then the non-empty blocks
        d->hseg.clear();
        for (uint64_t k : d->carry_known) d->hseg.push_back({k, k});
        for (const BlockDesc &b : d->hblk)
            if (b.isize) d->hseg.push_back({b.u_off, d->hseg.empty() ? b.u_off : NONE});
        const uint32_t nseg = uint32_t(d->hseg.size());
        if (u_total == 0) return 0;  // no bytes left
        nxt = d->cur ^ 1;
        const uint64_t rec_cap = std::min<uint64_t>(max_reads, u_total / 36 + 1);
        if (!d->stream[nxt].ensure(u_total) || !d->cin.ensure(chunk_bytes + 1) || !d->blk.ensure(nblk + 1) ||
            !d->seg.ensure(nseg + 1) || !d->matches.ensure(2 * m_total + 2) || !d->nmatch.ensure(nblk + 1) ||
            !d->cand.ensure(nseg + 1) || !d->exitp.ensure(nseg + 1) || !d->count.ensure(nseg + 1) ||
            !d->term.ensure(nseg + 1) || !d->bad.ensure(nseg + 1) || !d->base.ensure(nseg + 1) ||
            !d->rec_off.ensure(rec_cap + 1))
            return dfail(r, "out of device memory");
        bool ok = true;
        if (d->carry_len)
            ok &= cudaMemcpyAsync(d->stream[nxt].p, d->stream[d->cur].p + d->carry_off, d->carry_len,
                                  cudaMemcpyDeviceToDevice, st) == cudaSuccess;
        if (chunk_bytes)
            ok &= cudaMemcpyAsync(d->cin.p, d->slab + chunk_begin, chunk_bytes, cudaMemcpyHostToDevice, st) == cudaSuccess;
        if (nblk)
            ok &= cudaMemcpyAsync(d->blk.p, d->hblk.data(), nblk * sizeof(BlockDesc), cudaMemcpyHostToDevice, st) ==
                  cudaSuccess;
        ok &= cudaMemcpyAsync(d->seg.p, d->hseg.data(), nseg * sizeof(SegDesc), cudaMemcpyHostToDevice, st) == cudaSuccess;
        ok &= cudaMemsetAsync(d->sum.p, 0, sizeof(Summary), st) == cudaSuccess;
        sv = StreamView{d->stream[nxt].p, u_total, ntarg};
        const uint32_t nb = uint32_t(nblk);
        const uint32_t dpw = std::min<uint32_t>(32, std::max<uint32_t>(
                                 1, (nb + INF_WARPS_PER_SM * d->num_sms - 1) / (INF_WARPS_PER_SM * d->num_sms)));
        ok = ok && launch(k_inflate, dim3((nb + dpw - 1) / dpw), dim3(32), dpw * sizeof(fpinf::Tables), st,
                          (const uint8_t *)d->cin.p, (const BlockDesc *)d->blk.p, nb, dpw, d->stream[nxt].p,
                          d->matches.p, d->nmatch.p, d->sum.p);
        ok = ok && launch(k_resolve_crc, dim3(nb), dim3(32), RES_SMEM, st, (const BlockDesc *)d->blk.p, nb,
                          d->stream[nxt].p, (const uint32_t *)d->matches.p, (const uint32_t *)d->nmatch.p, d->sum.p);
        ok = ok && launch(k_seg_walk, dim3((nseg * 32ull + 255) / 256), dim3(256), 0, st, sv, (const SegDesc *)d->seg.p,
                          nseg, d->cand.p, d->exitp.p, d->count.p, d->term.p, d->bad.p);
        ok = ok && launch(k_seg_verify, dim3(1), dim3(1024), 0, st, sv, (const SegDesc *)d->seg.p, nseg,
                          (const uint64_t *)d->cand.p, (const uint64_t *)d->exitp.p, (const uint32_t *)d->count.p,
                          (const uint8_t *)d->term.p, (const uint8_t *)d->bad.p, d->base.p, d->sum.p);
        ok = ok && launch(k_seg_offsets, dim3((nseg + 127) / 128), dim3(128), 0, st, sv, (const SegDesc *)d->seg.p,
                          nseg, (const uint64_t *)d->cand.p, (const uint64_t *)d->base.p, uint64_t(max_reads),
                          d->rec_off.p, d->sum.p);
        ok = ok && launch(k_walk_serial, dim3(1), dim3(1), 0, st, sv, uint64_t(max_reads), rec_cap, d->rec_off.p,
                          d->sum.p);
        d->hcand.resize(nseg);
        ok = ok && cudaMemcpyAsync(&hs, d->sum.p, sizeof(Summary), cudaMemcpyDeviceToHost, st) == cudaSuccess;
        ok = ok && cudaMemcpyAsync(d->hcand.data(), d->cand.p, nseg * 8ull, cudaMemcpyDeviceToHost, st) == cudaSuccess;
        ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
        if (!ok) return dfail(r, std::string("GPU decoding failed: ") + cudaGetErrorString(cudaGetLastError()));
        if (hs.status) return dfail(r, device_error(hs));
        r->stats.blocks += uint64_t(nblk);
        r->stats.serial_walks += hs.ok ? 0u : 1u;
        // the carry for whatever comes next: the stream from `from`, with the chain's record starts
        auto set_carry = [&](uint64_t from) {
            d->cur = nxt;
            d->carry_off = from;
            d->carry_len = u_total - from;
            d->carry_known.clear();
            if (d->carry_len == 0) return;
            d->carry_known.push_back(0);
            if (!hs.ok) return;
            for (uint32_t s = 0; s < nseg; s++)
                if (d->hcand[s] != NONE && d->hcand[s] > from && d->hcand[s] < u_total)
                    d->carry_known.push_back(d->hcand[s] - from);
            std::sort(d->carry_known.begin(), d->carry_known.end());
        };
        if (hs.total < max_reads && !eof) {
            // fewer records than asked for and more input: keep the whole stream and add blocks
            set_carry(0);
            d->est *= 1.25;
            r->stats.extra_rounds++;
            continue;
        }
        take = std::min<uint64_t>(hs.total, max_reads);
        if (take == hs.total && eof && u_total - hs.end_of_records >= 4)
            return dfail(r, "truncated BAM record");
        if (take == 0) {
            set_carry(u_total);
            return 0;
        }
        set_carry(hs.carry_start);
        d->est = double(hs.carry_start) / double(take);
        break;
    }
    // 4. records
    const uint32_t n = uint32_t(take);
    OutSet &o = d->sets[d->next_set];
    if (!o.ensure_reads(n) || !d->symcnt.ensure(n) || !d->rgname.ensure(n))
        return dfail(r, "out of device memory");
    const uint32_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (!d->tile_sum.ensure(3ull * ntiles + 3)) return dfail(r, "out of device memory");
    bool ok = true;
    ok = ok && launch(k_rec_sizes, dim3((n + 255) / 256), dim3(256), 0, st, sv, (const uint64_t *)d->rec_off.p, n,
                      o.clen.p, o.rlen.p, o.qlen.p, d->symcnt.p, d->sum.p);
    Scan3 sc{{o.clen.p, d->symcnt.p, o.qlen.p}, {o.cstart.p, o.rstart.p, o.qstart.p}};
    ok = ok && launch(k_scan_tiles, dim3(ntiles, 3), dim3(SCAN_T), 0, st, sc, n, d->tile_sum.p);
    ok = ok && launch(k_scan_top, dim3(3), dim3(SCAN_T), 0, st, d->tile_sum.p, ntiles, d->sum.p);
    ok = ok && launch(k_scan_apply, dim3(ntiles, 3), dim3(SCAN_T), 0, st, sc, n, (const uint64_t *)d->tile_sum.p);
    ok = ok && cudaMemcpyAsync(&hs, d->sum.p, sizeof(Summary), cudaMemcpyDeviceToHost, st) == cudaSuccess;
    ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) return dfail(r, std::string("GPU decoding failed: ") + cudaGetErrorString(cudaGetLastError()));
    if (hs.status) return dfail(r, device_error(hs));
    if (!o.cigars.ensure(hs.tot[0] + 1) || !o.reads.ensure(hs.tot[1] / 8 + 1) || !o.quals.ensure(hs.tot[2] + 1))
        return dfail(r, "out of device memory");
    const size_t nt = r->contig_of_target.size();
    if (!d->ctmap.ensure(nt + 1)) return dfail(r, "out of device memory");
    if (nt)
        ok = ok && cudaMemcpyAsync(d->ctmap.p, r->contig_of_target.data(), nt * 2, cudaMemcpyHostToDevice, st) ==
                       cudaSuccess;
    OutArrays oa{o.chrom.p, o.astart.p, o.astop.p, o.mstart.p, o.isize.p, o.cigars.p, o.cstart.p, o.clen.p,
                 o.reads.p, o.rstart.p, o.rlen.p, o.quals.p, o.qstart.p, o.qlen.p, o.flags.p, o.mapq.p, o.rg.p};
    RgTables rg{d->id_bytes.p, d->id_off.p, d->id_name.p, d->n_ids, d->id_of_name.p, d->first_seen.p,
                uint32_t(d->names.size())};
    ok = ok && launch(k_rec_convert, dim3((n * 32ull + 255) / 256), dim3(256), 0, st, sv, (const uint64_t *)d->rec_off.p,
                      n, (const uint16_t *)d->ctmap.p, uint32_t(nt), oa, rg, d->rgname.p);
    ok = ok && launch(k_rg_assign, dim3(1), dim3(1), 0, st, rg, d->next_id.p);
    ok = ok && launch(k_rg_apply, dim3((n + 255) / 256), dim3(256), 0, st, (const uint32_t *)d->rgname.p, n,
                      (const uint32_t *)d->id_of_name.p, o.rg.p);
    std::vector<uint32_t> ion(d->names.size());
    if (!ion.empty())
        ok = ok && cudaMemcpyAsync(ion.data(), d->id_of_name.p, ion.size() * 4, cudaMemcpyDeviceToHost, st) ==
                       cudaSuccess;
    ok = ok && cudaMemcpyAsync(&hs, d->sum.p, sizeof(Summary), cudaMemcpyDeviceToHost, st) == cudaSuccess;
    ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) return dfail(r, std::string("GPU decoding failed: ") + cudaGetErrorString(cudaGetLastError()));
    if (hs.status) return dfail(r, device_error(hs));
    // the host's read-group list follows the ids the device assigned
    std::vector<std::pair<uint32_t, uint32_t>> fresh;
    for (size_t k = 0; k < ion.size(); k++)
        if (ion[k] != NONE32 && r->rg_index.find(d->names[k]) == r->rg_index.end()) fresh.push_back({ion[k], uint32_t(k)});
    std::sort(fresh.begin(), fresh.end());
    for (const auto &f : fresh) {
        r->rg_index[d->names[f.second]] = f.first;
        if (r->rg_names.size() <= f.first) r->rg_names.resize(f.first + 1);
        r->rg_names[f.first] = d->names[f.second];
    }
    d->next_set = (d->next_set + 1) % FPB_BUFFER_SETS;
    v->num_reads = n;
    v->num_cigar_ops = uint32_t(hs.tot[0]);
    v->num_read_symbols = hs.tot[1];
    v->num_qualities = hs.tot[2];
    v->chromosome = o.chrom.p; v->alignment_start = o.astart.p; v->alignment_stop = o.astop.p;
    v->mate_alignment_start = o.mstart.p; v->inferred_insert_size = o.isize.p; v->cigars = o.cigars.p;
    v->cigar_start = o.cstart.p; v->cigar_len = o.clen.p; v->reads = o.reads.p; v->read_start = o.rstart.p;
    v->read_len = o.rlen.p; v->qualities = o.quals.p; v->qual_start = o.qstart.p; v->qual_len = o.qlen.p;
    v->flags = o.flags.p; v->mapq = o.mapq.p; v->read_group = o.rg.p;
    return int64_t(n);
}
