// Raw DEFLATE (RFC 1951) decoding of one BGZF block, written for one GPU thread per block (a warp decodes 32
// blocks in lockstep, a step at a time) and compiled for the host as well (the host build is what the decoder's
// unit tests run against zlib).
//
// The decoder is split in two passes so that no pass waits on its own output:
//   1. `Inflater` (`inflate_tokens` on one thread) decodes the Huffman stream, writes literal bytes straight to
//      their output positions and records each back-reference as a match (output position, length, distance)
//      without copying it;
//   2. the matches are resolved in stream order (`resolve_matches_serial` here; a warp per block on the GPU,
//      32 bytes of one match at a time). Byte k of a match at position p with distance d is
//      out[p - d + (k mod d)]: every source byte lies before p, so it is final once the earlier matches are
//      resolved.
//
// Every loop is bounded by the input length or the output size, and every table and output index is checked:
// a corrupt block ends with an error status, never with an access outside its buffers.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define FPI_HD __host__ __device__ __forceinline__
#else
#define FPI_HD inline
#endif

namespace fpinf {

constexpr int MAXBITS = 15;
constexpr int LIT_FAST = 10;  // bits of the literal/length lookup table
constexpr int DIST_FAST = 8;  // bits of the distance lookup table
constexpr int CL_FAST = 7;    // code-length codes are at most 7 bits: a direct table

enum Status : int {
    OK = 0,
    E_INPUT = 1,     // the stream runs past its compressed bytes
    E_BTYPE = 2,     // block type 3
    E_STORED = 3,    // stored block length and its complement differ
    E_CODES = 4,     // invalid code lengths (over-subscribed, incomplete, repeat without a previous length)
    E_SYMBOL = 5,    // a bit pattern that is no code, or symbol 286/287, distance 30/31
    E_DIST = 6,      // a distance reaching before the start of the block
    E_OUTPUT = 7,    // more output than the block's ISIZE
    E_SIZE = 8,      // less output than the block's ISIZE
    E_MATCHES = 9,   // more matches than the match list holds
};

// Canonical Huffman decoding table: a direct table for codes of at most FB bits (entry = symbol | length << 9;
// 0 = a longer code) and the per-length counts and sorted symbols for the longer ones.
template <int FB, int NS> struct Huff {
    uint16_t fast[1 << FB];
    uint16_t count[MAXBITS + 1];
    uint16_t sym[NS];
};

// the tables the symbol loop reads (kept in shared memory on the GPU)
struct Tables {
    Huff<LIT_FAST, 288> lit;
    Huff<DIST_FAST, 32> dist;
};
// what only the block headers need (thread-local on the GPU)
struct Work {
    Huff<CL_FAST, 19> clen;
    uint8_t lens[288 + 32];
};

// Builds h from the code lengths of n symbols. Returns < 0 if the code is over-subscribed, the number of
// unused codes otherwise (0: complete).
template <int FB, int NS> FPI_HD int build(Huff<FB, NS> &h, const uint8_t *len, int n) {
    for (int l = 0; l <= MAXBITS; l++) h.count[l] = 0;
    for (int s = 0; s < n; s++) h.count[len[s] & 15]++;
    for (int k = 0; k < (1 << FB); k++) h.fast[k] = 0;
    if (h.count[0] == n) return 0;  // no codes: decoding any symbol fails
    int left = 1;
    for (int l = 1; l <= MAXBITS; l++) {
        left <<= 1;
        left -= h.count[l];
        if (left < 0) return left;
    }
    uint16_t offs[MAXBITS + 2];
    offs[1] = 0;
    for (int l = 1; l <= MAXBITS; l++) offs[l + 1] = uint16_t(offs[l] + h.count[l]);
    for (int s = 0; s < n; s++)
        if (len[s] & 15) h.sym[offs[len[s] & 15]++] = uint16_t(s);
    // direct entries: the canonical code of each symbol of length l <= FB, bit-reversed (DEFLATE sends codes
    // most significant bit first into an LSB-first bit stream), repeated over the free high bits
    int code = 0, idx = 0;
    for (int l = 1; l <= FB; l++) {
        for (int j = 0; j < h.count[l]; j++, idx++, code++) {
            int rev = 0;
            for (int b = 0; b < l; b++) rev |= ((code >> b) & 1) << (l - 1 - b);
            const uint16_t e = uint16_t(h.sym[idx] | (l << 9));
            for (int k = rev; k < (1 << FB); k += 1 << l) h.fast[k] = e;
        }
        code <<= 1;
    }
    return left;
}

// LSB-first bit reader over n bytes. Bytes past the end read as 0 and are counted; the caller checks
// `overrun()` before trusting a result.
struct Bits {
    const uint8_t *p;
    uint32_t n;
    uint32_t pos;  // next byte to load
    uint32_t cnt;  // bits in buf
    uint64_t buf;
    FPI_HD void init(const uint8_t *in, uint32_t len) {
        p = in; n = len; pos = 0; cnt = 0; buf = 0;
    }
    FPI_HD void refill() {
        while (cnt <= 56) {
            const uint64_t byte = pos < n ? p[pos] : 0u;
            pos++;
            buf |= byte << cnt;
            cnt += 8;
        }
    }
    FPI_HD uint32_t take(uint32_t k) {  // k <= cnt, k <= 32
        const uint32_t v = uint32_t(buf & ((uint64_t(1) << k) - 1));
        buf >>= k;
        cnt -= k;
        return v;
    }
    // consumed more bits than the input holds
    FPI_HD bool overrun() const { return uint64_t(pos) * 8 - cnt > uint64_t(n) * 8; }
};

// Decodes one symbol (needs cnt >= 15). Returns the symbol or -1.
template <int FB, int NS> FPI_HD int decode(Bits &b, const Huff<FB, NS> &h) {
    const uint32_t e = h.fast[b.buf & ((1u << FB) - 1)];
    if (e) {
        b.buf >>= (e >> 9);
        b.cnt -= (e >> 9);
        return int(e & 511);
    }
    int code = 0, first = 0, index = 0;
    uint64_t bb = b.buf;
    for (int l = 1; l <= MAXBITS; l++) {
        code |= int(bb & 1);
        bb >>= 1;
        const int c = h.count[l];
        if (code - c < first) {
            b.buf >>= l;
            b.cnt -= uint32_t(l);
            return h.sym[index + (code - first)];
        }
        index += c;
        first += c;
        first <<= 1;
        code <<= 1;
    }
    return -1;
}

FPI_HD int len_base(int s) {  // s = 0..28 (symbols 257..285)
    return s < 8 ? 3 + s : s == 28 ? 258 : ((4 + (s & 3)) << ((s - 4) >> 2)) + 3;
}
FPI_HD int len_extra(int s) { return s < 8 || s == 28 ? 0 : (s - 4) >> 2; }
FPI_HD int dist_base(int s) {  // s = 0..29
    return s < 4 ? 1 + s : ((2 + (s & 1)) << ((s >> 1) - 1)) + 1;
}
FPI_HD int dist_extra(int s) { return s < 4 ? 0 : (s >> 1) - 1; }

FPI_HD int build_fixed(Tables &t, Work &s) {
    for (int i = 0; i < 144; i++) s.lens[i] = 8;
    for (int i = 144; i < 256; i++) s.lens[i] = 9;
    for (int i = 256; i < 280; i++) s.lens[i] = 7;
    for (int i = 280; i < 288; i++) s.lens[i] = 8;
    build(t.lit, s.lens, 288);
    for (int i = 0; i < 30; i++) s.lens[i] = 5;
    build(t.dist, s.lens, 30);
    return OK;
}

FPI_HD int build_dynamic(Bits &b, Tables &t, Work &s) {
    // code-length code lengths arrive in this order (RFC 1951 3.2.7)
    const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    b.refill();
    const int nlen = int(b.take(5)) + 257, ndist = int(b.take(5)) + 1, ncode = int(b.take(4)) + 4;
    if (nlen > 286 || ndist > 30) return E_CODES;
    uint8_t cl[19];
    for (int i = 0; i < 19; i++) cl[i] = 0;
    for (int i = 0; i < ncode; i++) {
        b.refill();
        cl[order[i]] = uint8_t(b.take(3));
    }
    if (build(s.clen, cl, 19) != 0) return E_CODES;  // must be complete
    int idx = 0;
    while (idx < nlen + ndist) {
        b.refill();
        if (b.overrun()) return E_INPUT;
        int sym = decode(b, s.clen);
        if (sym < 0) return E_SYMBOL;
        if (sym < 16) {
            s.lens[idx++] = uint8_t(sym);
            continue;
        }
        int len = 0, rep;
        if (sym == 16) {
            if (idx == 0) return E_CODES;
            len = s.lens[idx - 1];
            rep = 3 + int(b.take(2));
        } else if (sym == 17) {
            rep = 3 + int(b.take(3));
        } else {
            rep = 11 + int(b.take(7));
        }
        if (idx + rep > nlen + ndist) return E_CODES;
        while (rep--) s.lens[idx++] = uint8_t(len);
    }
    if (s.lens[256] == 0) return E_CODES;  // no end-of-block code
    int err = build(t.lit, s.lens, nlen);
    if (err < 0 || (err > 0 && nlen - t.lit.count[0] != 1)) return E_CODES;  // incomplete only for one code
    err = build(t.dist, s.lens + nlen, ndist);
    if (err < 0 || (err > 0 && ndist - t.dist.count[0] != 1)) return E_CODES;
    return OK;
}

// Pass 1 as a resumable decoder: each `step` does one unit of work, a block header (with the bytes of a stored
// block) or one literal/length symbol, so that the GPU can run the decoders of a warp in lockstep (a warp-wide
// vote after every step reconverges threads whose symbols took different branches). Literals go to out[];
// each match goes to matches[] as {position, length << 16 | distance}.
struct Inflater {
    Bits b;
    uint8_t *out;
    uint32_t out_size, o;
    uint32_t *matches;
    uint32_t match_cap, nm;
    int status;     // OK while running, then the final status
    bool header;    // a block header comes next
    bool last;      // the current block is the stream's last

    FPI_HD void init(const uint8_t *in, uint32_t n_in, uint8_t *out_, uint32_t out_size_, uint32_t *matches_,
                     uint32_t match_cap_) {
        b.init(in, n_in);
        out = out_;
        out_size = out_size_;
        o = 0;
        matches = matches_;
        match_cap = match_cap_;
        nm = 0;
        status = OK;
        header = true;
        last = false;
    }
    FPI_HD bool fail(int st) {
        status = st;
        return false;
    }
    // end of the last block: every input bit accounted for and exactly out_size bytes produced
    FPI_HD bool finish() {
        if (b.overrun()) return fail(E_INPUT);
        return fail(o == out_size ? OK : E_SIZE);
    }
    // 32 more bits (needs cnt <= 32): four independent byte loads instead of a data-dependent loop (checked
    // against the end only near it)
    FPI_HD void refill32() {
        uint32_t w = 0;
        if (b.n - b.pos >= 4 && b.pos <= b.n) {
            const uint8_t *q = b.p + b.pos;
            w = uint32_t(q[0]) | (uint32_t(q[1]) << 8) | (uint32_t(q[2]) << 16) | (uint32_t(q[3]) << 24);
        } else {
            for (uint32_t k = 0; k < 4; k++) w |= uint32_t(b.pos + k < b.n ? b.p[b.pos + k] : 0u) << (8 * k);
        }
        b.buf |= uint64_t(w) << b.cnt;
        b.cnt += 32;
        b.pos += 4;
    }
    // Returns true while more steps remain; `status` holds the result once it returns false.
    FPI_HD bool step(Tables &t, Work &s) {
        if (header) {
            b.refill();
            if (b.overrun()) return fail(E_INPUT);
            last = b.take(1) != 0;
            const uint32_t type = b.take(2);
            if (type == 0) {
                b.take(b.cnt & 7);  // to the byte boundary
                b.refill();
                const uint32_t len = b.take(16), nlen = b.take(16);
                if ((len ^ 0xFFFFu) != nlen) return fail(E_STORED);
                if (len > out_size - o) return fail(E_OUTPUT);
                for (uint32_t k = 0; k < len; k++) {
                    if (b.cnt < 8) b.refill();
                    out[o++] = uint8_t(b.take(8));
                }
                if (b.overrun()) return fail(E_INPUT);
                return last ? finish() : true;
            }
            if (type == 3) return fail(E_BTYPE);
            const int st = type == 1 ? build_fixed(t, s) : build_dynamic(b, t, s);
            if (st != OK) return fail(st);
            header = false;
            return true;
        }
        // a symbol needs at most 15 + 5 bits, its distance 15 + 13
        if (b.cnt <= 32) refill32();
        // each symbol takes at least one bit, so this check bounds the number of steps by the input length
        if (b.overrun()) return fail(E_INPUT);
        const int sym = decode(b, t.lit);
        if (sym < 0) return fail(E_SYMBOL);
        if (sym < 256) {
            if (o >= out_size) return fail(E_OUTPUT);
            out[o++] = uint8_t(sym);
            // up to five more literals with direct-table codes (at most LIT_FAST bits each) from the bits
            // already buffered: most symbols of base and quality data are literals
            for (int k = 0; k < 5 && b.cnt >= uint32_t(LIT_FAST) && o < out_size; k++) {
                const uint32_t e = t.lit.fast[b.buf & ((1u << LIT_FAST) - 1)];
                if (e == 0 || (e & 511u) >= 256u) break;
                b.buf >>= (e >> 9);
                b.cnt -= (e >> 9);
                out[o++] = uint8_t(e & 511u);
            }
            return true;
        }
        if (sym == 256) {
            header = true;
            return last ? finish() : true;
        }
        const int ls = sym - 257;
        if (ls >= 29) return fail(E_SYMBOL);
        const uint32_t len = uint32_t(len_base(ls)) + b.take(uint32_t(len_extra(ls)));
        if (b.cnt <= 32) refill32();
        const int ds = decode(b, t.dist);
        if (ds < 0 || ds >= 30) return fail(E_SYMBOL);
        const uint32_t dist = uint32_t(dist_base(ds)) + b.take(uint32_t(dist_extra(ds)));
        if (dist > o) return fail(E_DIST);
        if (len > out_size - o) return fail(E_OUTPUT);
        if (nm >= match_cap) return fail(E_MATCHES);
        matches[2 * nm] = o;
        matches[2 * nm + 1] = (len << 16) | dist;
        nm++;
        o += len;
        return true;
    }
};

// Pass 1 on one thread: decodes a raw DEFLATE stream of n_in bytes whose output is exactly out_size bytes.
// *n_matches gets the number of matches listed.
FPI_HD int inflate_tokens(const uint8_t *in, uint32_t n_in, uint8_t *out, uint32_t out_size, uint32_t *matches,
                          uint32_t match_cap, uint32_t *n_matches, Tables &t, Work &s) {
    Inflater f;
    f.init(in, n_in, out, out_size, matches, match_cap);
    while (f.step(t, s)) {
    }
    *n_matches = f.status == OK ? f.nm : 0u;
    return f.status;
}

// Pass 2 on one thread (host tests and small blocks): forward byte copies in stream order.
FPI_HD void resolve_matches_serial(uint8_t *out, const uint32_t *matches, uint32_t n) {
    for (uint32_t j = 0; j < n; j++) {
        const uint32_t p = matches[2 * j], len = matches[2 * j + 1] >> 16, d = matches[2 * j + 1] & 0xFFFFu;
        for (uint32_t k = 0; k < len; k++) out[p + k] = out[p + k - d];
    }
}

// Most matches a block of `out_size` bytes can hold (every match is at least 3 bytes).
FPI_HD uint32_t match_capacity(uint32_t out_size) { return out_size / 3 + 1; }

// ---- CRC-32 (the gzip polynomial, reflected: 0xEDB88320) ----
// Polynomials over GF(2) are held reflected: bit 31 is x^0, bit 0 is x^31.
constexpr uint32_t CRC_POLY = 0xEDB88320u;

// a(x) * b(x) mod P(x)
FPI_HD uint32_t gf2_mulmod(uint32_t a, uint32_t b) {
    uint32_t p = 0;
    for (int i = 0; i < 32; i++) {  // coefficient of x^i in a is bit 31 - i
        if (a & (0x80000000u >> i)) p ^= b;
        b = (b & 1) ? (b >> 1) ^ CRC_POLY : b >> 1;  // b *= x
    }
    return p;
}

// x^(8n) mod P(x), by squaring
FPI_HD uint32_t x8n_mod(uint64_t n) {
    uint32_t r = 0x80000000u;       // x^0
    uint32_t sq = 0x80000000u >> 8;  // x^8
    while (n) {
        if (n & 1) r = gf2_mulmod(r, sq);
        sq = gf2_mulmod(sq, sq);
        n >>= 1;
    }
    return r;
}

// CRC of A||B from crc(A), crc(B) and |B|: crc(A) * x^(8|B|) xor crc(B) (the pre- and post-conditioning of
// the standard CRC-32 cancel in this form)
FPI_HD uint32_t crc_concat(uint32_t crc_a, uint32_t crc_b, uint64_t len_b) {
    return gf2_mulmod(x8n_mod(len_b), crc_a) ^ crc_b;
}

// the byte-at-a-time table: t[i] = CRC register after shifting byte i through, from the definition
FPI_HD void crc_table(uint32_t *t) {
    for (uint32_t i = 0; i < 256; i++) {
        uint32_t c = i;
        for (int k = 0; k < 8; k++) c = (c & 1) ? (c >> 1) ^ CRC_POLY : c >> 1;
        t[i] = c;
    }
}

FPI_HD uint32_t crc_bytes(const uint32_t *t, const uint8_t *p, uint32_t n) {
    uint32_t c = 0xFFFFFFFFu;
    for (uint32_t i = 0; i < n; i++) c = t[(c ^ p[i]) & 255] ^ (c >> 8);
    return c ^ 0xFFFFFFFFu;
}

}  // namespace fpinf
