// BAM input: multi-threaded BGZF inflate and record decoding into the engine's batch layout, and a BAM
// writer for synthetic inputs. See include/firepony_gb300_bam.h for the field semantics (those of the
// reference's htslib loader, loader/alignments.cu:136-437).
#include <cuda_runtime.h>
#include <zlib.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bam_internal.h"

using namespace fpb_detail;

namespace {

template <typename F> void parallel_for(int threads, size_t n, F f) {
    if (n == 0) return;
    const int nt = int(std::min<size_t>(size_t(threads), n));
    if (nt <= 1) {
        f(size_t(0), n);
        return;
    }
    std::vector<std::thread> th;
    const size_t chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; t++) {
        const size_t a = t * chunk, z = std::min(n, a + chunk);
        if (a >= z) break;
        th.emplace_back([=, &f]() { f(a, z); });
    }
    for (auto &x : th) x.join();
}

struct NibbleSwapTable {
    uint8_t t[256];
    constexpr NibbleSwapTable() : t() {
        for (int b = 0; b < 256; b++) t[b] = uint8_t(((b & 15) << 4) | (b >> 4));
    }
};
constexpr NibbleSwapTable kNibbleSwapT{};
constexpr const uint8_t *kNibbleSwap = kNibbleSwapT.t;

}  // namespace


namespace {

int fail(fpb_reader *r, const std::string &m) {
    r->err = m;
    return -1;
}

// reads more compressed input (up to `bytes`); false at end of file
bool read_more(fpb_reader *r, size_t bytes) {
    if (r->eof_in) return false;
    if (r->cpos > 0) {
        r->cbuf.erase_prefix(r->cpos);
        r->cpos = 0;
    }
    const size_t old = r->cbuf.size();
    if (!r->cbuf.resize(old + bytes)) return false;
    const double t0 = now_s();
    const size_t got = fread(r->cbuf.data() + old, 1, bytes, r->f);
    r->stats.seconds_read += now_s() - t0;
    r->stats.compressed_bytes += got;
    r->cbuf.resize(old + got);
    if (got < bytes) r->eof_in = true;
    return got > 0;
}

// inflates the next BGZF blocks (at most max_blocks, in parallel) and appends them to the stream; returns the
// number of blocks, 0 at the end, -1 on a malformed block
int inflate_blocks(fpb_reader *r, int max_blocks) {
    struct Blk { size_t off, csize; uint32_t isize; size_t uoff; };
    std::vector<Blk> blks;
    size_t total = 0;
    for (;;) {
        if ((int)blks.size() >= max_blocks) break;
        size_t p = r->cpos;
        for (const Blk &b : blks) p = std::max(p, b.off + b.csize);
        if (r->cbuf.size() - p < 18) {
            if (!blks.empty()) break;
            if (!read_more(r, 16 << 20) && r->cbuf.size() - r->cpos < 18) return 0;
            continue;
        }
        const uint8_t *h = r->cbuf.data() + p;
        if (h[0] != 31 || h[1] != 139 || h[2] != 8 || !(h[3] & 4)) return fail(r, "not a BGZF block"), -1;
        const uint16_t xlen = rd16(h + 10);
        if (r->cbuf.size() - p < size_t(12) + xlen) {
            if (!blks.empty()) break;
            if (!read_more(r, 16 << 20)) return fail(r, "truncated BGZF block"), -1;
            continue;
        }
        size_t bsize = 0;
        for (size_t x = 0; x + 4 <= xlen;) {
            const uint8_t *sf = h + 12 + x;
            const uint16_t slen = rd16(sf + 2);
            if (sf[0] == 66 && sf[1] == 67 && slen == 2) bsize = size_t(rd16(sf + 4)) + 1;
            x += 4 + slen;
        }
        if (bsize == 0) return fail(r, "BGZF block without a BC field"), -1;
        if (r->cbuf.size() - p < bsize) {
            if (!blks.empty()) break;
            if (!read_more(r, 16 << 20)) return fail(r, "truncated BGZF block"), -1;
            continue;
        }
        const uint32_t isize = rd32(h + bsize - 4);
        blks.push_back({p, bsize, isize, total});
        total += isize;
    }
    if (blks.empty()) return 0;
    // compact the decoded stream, then inflate the blocks side by side
    if (r->upos > 0) {
        r->ubuf.erase_prefix(r->upos);
        r->upos = 0;
    }
    const size_t base = r->ubuf.size();
    if (!r->ubuf.resize(base + total)) return fail(r, "out of memory"), -1;
    std::atomic<int> bad{0};
    parallel_for(r->threads, blks.size(), [&](size_t a, size_t z) {
        z_stream zs;
        memset(&zs, 0, sizeof(zs));
        if (inflateInit2(&zs, -15) != Z_OK) { bad = 1; return; }
        for (size_t i = a; i < z; i++) {
            const Blk &b = blks[i];
            const uint8_t *h = r->cbuf.data() + b.off;
            const uint16_t xlen = rd16(h + 10);
            const size_t cstart = 12 + xlen, clen = b.csize - cstart - 8;
            inflateReset(&zs);
            zs.next_in = const_cast<Bytef *>(h + cstart);
            zs.avail_in = uInt(clen);
            zs.next_out = r->ubuf.data() + base + b.uoff;
            zs.avail_out = uInt(b.isize);
            const int rc = inflate(&zs, Z_FINISH);
            if ((rc != Z_STREAM_END && !(rc == Z_BUF_ERROR && b.isize == 0)) || zs.avail_out != 0) { bad = 1; continue; }
            const uint32_t crc = uint32_t(crc32(0L, r->ubuf.data() + base + b.uoff, uInt(b.isize)));
            if (crc != rd32(h + b.csize - 8)) bad = 1;
        }
        inflateEnd(&zs);
    });
    if (bad) return fail(r, "corrupt BGZF block"), -1;
    r->cpos = blks.back().off + blks.back().csize;
    return int(blks.size());
}

// ensures n undecoded bytes are available, inflating up to max_blocks blocks at a time: 1 when they are, 0 if
// the stream ends first, -1 on a malformed block (r->err set)
int need(fpb_reader *r, size_t n, int max_blocks = 512) {
    while (r->ubuf.size() - r->upos < n) {
        const int k = inflate_blocks(r, max_blocks);
        if (k <= 0) return k < 0 ? -1 : 0;
    }
    return 1;
}

}  // namespace

namespace {

// @RG lines: ID -> PU when present, else ID (loader/alignments.cu:164-186)
void parse_read_groups(fpb_reader *r, const std::string &text) {
    size_t pos = 0;
    while ((pos = text.find("@RG", pos)) != std::string::npos) {
        size_t end = text.find('\n', pos);
        if (end == std::string::npos) end = text.size();
        const std::string line = text.substr(pos, end - pos);
        std::string id, pu;
        size_t f = 0;
        while ((f = line.find('\t', f)) != std::string::npos) {
            const size_t g = line.find('\t', f + 1);
            const std::string field = line.substr(f + 1, (g == std::string::npos ? line.size() : g) - f - 1);
            if (field.compare(0, 3, "ID:") == 0) id = field.substr(3);
            if (field.compare(0, 3, "PU:") == 0) pu = field.substr(3);
            f += 1;
        }
        if (!id.empty()) r->rg_name_of_id[id] = pu.empty() ? id : pu;
        pos = end;
    }
}

// RG:Z value of a record's aux data (nullptr if absent); sets len
const char *find_rg(const uint8_t *p, const uint8_t *end, size_t &len) {
    while (p + 3 <= end) {
        const char t0 = char(p[0]), t1 = char(p[1]), type = char(p[2]);
        p += 3;
        size_t sz = 0;
        switch (type) {
        case 'A': case 'c': case 'C': sz = 1; break;
        case 's': case 'S': sz = 2; break;
        case 'i': case 'I': case 'f': sz = 4; break;
        case 'Z': case 'H': {
            const uint8_t *q = p;
            while (q < end && *q) q++;
            if (t0 == 'R' && t1 == 'G' && type == 'Z') {
                len = size_t(q - p);
                return reinterpret_cast<const char *>(p);
            }
            p = q + 1;
            continue;
        }
        case 'B': {
            if (p + 5 > end) return nullptr;
            const char sub = char(p[0]);
            const uint32_t n = rd32(p + 1);
            const size_t es = (sub == 'c' || sub == 'C') ? 1 : (sub == 's' || sub == 'S') ? 2 : 4;
            p += 5 + es * n;
            continue;
        }
        default: return nullptr;
        }
        p += sz;
    }
    return nullptr;
}

}  // namespace

extern "C" {

static int open_impl(const char *path, int threads, fpb_reader **out);

int fpb_open(const char *path, int threads, fpb_reader **out) {
    if (!path || !out) return -1;
    *out = nullptr;
    try {  // (no C++ exception crosses the C ABI)
        return open_impl(path, threads, out);
    } catch (...) {
        return -1;
    }
}

static int open_impl(const char *path, int threads, fpb_reader **out) {
    fpb_reader *r = new fpb_reader();
    r->threads = threads > 0 ? threads : int(std::max(1u, std::thread::hardware_concurrency()));
    r->f = fopen(path, "rb");
    if (!r->f) { delete r; return -1; }
    // magic, text, targets: inflated a block at a time, so that the records after the header stay compressed
    // for whichever decoder (host or GPU) reads them
    if (need(r, 12, 1) <= 0 || memcmp(r->ubuf.data() + r->upos, "BAM\1", 4) != 0) { fpb_close(r); return -1; }
    const uint32_t l_text = rd32(r->ubuf.data() + r->upos + 4);
    if (need(r, 12 + size_t(l_text), 1) <= 0) { fpb_close(r); return -1; }
    const std::string text(reinterpret_cast<const char *>(r->ubuf.data() + r->upos + 8), l_text);
    r->upos += 8 + l_text;
    parse_read_groups(r, text);
    if (need(r, 4, 1) <= 0) { fpb_close(r); return -1; }
    const uint32_t n_ref = rd32(r->ubuf.data() + r->upos);
    r->upos += 4;
    for (uint32_t i = 0; i < n_ref; i++) {
        if (need(r, 4, 1) <= 0) { fpb_close(r); return -1; }
        const uint32_t l_name = rd32(r->ubuf.data() + r->upos);
        if (need(r, 8 + size_t(l_name), 1) <= 0) { fpb_close(r); return -1; }
        const char *nm = reinterpret_cast<const char *>(r->ubuf.data() + r->upos + 4);
        r->target_names.emplace_back(nm, strnlen(nm, l_name));
        r->target_lens.push_back(rd32(r->ubuf.data() + r->upos + 4 + l_name));
        r->upos += 8 + l_name;
        r->contig_of_target.push_back(uint16_t(i < 0xFFFF ? i : 0xFFFF));
    }
    *out = r;
    return 0;
}

void fpb_close(fpb_reader *r) {
    if (!r) return;
    if (r->dev) destroy_device_decoder(r->dev);
    if (r->f) fclose(r->f);
    delete r;
}

const char *fpb_last_error(const fpb_reader *r) { return r ? r->err.c_str() : "null reader"; }
uint32_t fpb_num_targets(const fpb_reader *r) { return r ? uint32_t(r->target_names.size()) : 0; }
const char *fpb_target_name(const fpb_reader *r, uint32_t i) {
    return (r && i < r->target_names.size()) ? r->target_names[i].c_str() : nullptr;
}
uint32_t fpb_target_length(const fpb_reader *r, uint32_t i) {
    return (r && i < r->target_lens.size()) ? r->target_lens[i] : 0;
}
int fpb_set_target_map(fpb_reader *r, const uint16_t *map, uint32_t n) {
    if (!r || (!map && n)) return -1;
    for (size_t i = 0; i < r->contig_of_target.size(); i++) r->contig_of_target[i] = i < n ? map[i] : 0xFFFF;
    return 0;
}
uint32_t fpb_num_read_groups(const fpb_reader *r) { return r ? uint32_t(r->rg_names.size()) : 0; }
const char *fpb_read_group_name(const fpb_reader *r, uint32_t id) {
    return (r && id < r->rg_names.size()) ? r->rg_names[id].c_str() : nullptr;
}

static int64_t next_batch_host(fpb_reader *r, uint32_t max_reads, fp_batch_view *v);

int64_t fpb_next_batch(fpb_reader *r, uint32_t max_reads, fp_batch_view *v) {
    if (!r || !v) return -1;
    if (r->failed) {  // after an error the undecoded stream and the file position are undefined
        memset(v, 0, sizeof(*v));
        r->err = "the reader failed earlier: " + r->failure;
        return -1;
    }
    const double t0 = now_s(), read0 = r->stats.seconds_read;
    int64_t n;
    try {  // (no C++ exception crosses the C ABI)
        n = next_batch_host(r, max_reads, v);
    } catch (...) {
        r->err.assign("host alloc fail");
        n = -1;
    }
    r->stats.seconds_decode += (now_s() - t0) - (r->stats.seconds_read - read0);
    if (n < 0 && r->mode == 1 && !r->failed) {  // (a call in the wrong mode leaves the reader usable)
        r->failed = true;
        r->failure = r->err;
    }
    if (n > 0) {
        r->stats.batches++;
        r->stats.records += uint64_t(n);
    }
    return n;
}

int fpb_get_stats(const fpb_reader *r, fpb_stats *out) {
    if (!r || !out) return -1;
    *out = r->stats;
    return 0;
}

static int64_t next_batch_host(fpb_reader *r, uint32_t max_reads, fp_batch_view *v) {
    memset(v, 0, sizeof(*v));
    if (r->mode == 2) return fail(r, "the reader decodes on the GPU (fpb_next_batch_device)");
    r->mode = 1;
    // locate the records: length prefixes, in stream order
    std::vector<size_t> rec;
    rec.reserve(max_reads);
    size_t p = r->upos;
    while (rec.size() < max_reads) {
        if (r->ubuf.size() - p < 4) {
            const size_t rel = p - r->upos;
            const int k = need(r, rel + 4);
            if (k < 0) return -1;  // (the malformed block's error is kept)
            if (k == 0) break;
            // need() may have compacted or moved the stream: record offsets are kept relative to upos
            p = r->upos + rel;
        }
        const uint32_t bs = rd32(r->ubuf.data() + p);
        if (r->ubuf.size() - p < 4 + size_t(bs)) {
            const size_t rel = p - r->upos;
            const int k = need(r, rel + 4 + bs);
            if (k < 0) return -1;
            if (k == 0) return fail(r, "truncated BAM record");
            p = r->upos + rel;
        }
        if (bs < 32) return fail(r, "BAM record shorter than its fixed fields");
        {
            const uint8_t *b = r->ubuf.data() + p + 4;
            const uint64_t need_bytes = 32ull + b[8] + 4ull * rd16(b + 12) + (uint64_t(rd32(b + 16)) + 1) / 2 +
                                        uint64_t(rd32(b + 16));
            if (need_bytes > bs) return fail(r, "malformed BAM record (its fields exceed its length)");
        }
        rec.push_back(p - r->upos);
        p += 4 + bs;
    }
    const size_t n = rec.size();
    if (n == 0) return 0;
    const uint8_t *ub = r->ubuf.data() + r->upos;
    // sizes and offsets of the variable arrays
    std::vector<uint32_t> cig_off(n + 1), sym_off(n + 1), qual_off(n + 1);
    uint64_t nc = 0, ns = 0, nq = 0;
    for (size_t i = 0; i < n; i++) {
        const uint8_t *b = ub + rec[i] + 4;
        const uint32_t l_seq = rd32(b + 16), n_cig = rd16(b + 12);
        cig_off[i] = uint32_t(nc);
        sym_off[i] = uint32_t(ns);
        qual_off[i] = uint32_t(nq);
        nc += n_cig;
        ns += (uint64_t(l_seq) + 7) / 8 * 8;
        nq += l_seq;
    }
    if (nc > 0xFFFFFFFFull || ns > 0xFFFFFFFFull || nq > 0xFFFFFFFFull) return fail(r, "batch too large");
    // read group names, resolved to ids in order of first occurrence: known names in parallel, names not yet
    // indexed in stream order
    std::vector<uint32_t> rg(n, 0xFFFFFFFFu);
    std::vector<uint8_t> rg_new(n, 0);
    auto rg_of = [&](size_t i, size_t &len) -> const char * {
        const uint8_t *b = ub + rec[i] + 4;
        const uint32_t bs = rd32(ub + rec[i]);
        const uint32_t l_seq = rd32(b + 16), n_cig = rd16(b + 12), l_name = b[8];
        const uint8_t *aux = b + 32 + l_name + 4 * size_t(n_cig) + (l_seq + 1) / 2 + l_seq;
        return find_rg(aux, b + bs, len);
    };
    parallel_for(r->threads, n, [&](size_t a, size_t z) {
        std::string key;
        for (size_t i = a; i < z; i++) {
            size_t len = 0;
            const char *s = rg_of(i, len);
            if (!s) continue;
            key.assign(s, len);
            auto it = r->rg_name_of_id.find(key);
            if (it == r->rg_name_of_id.end()) continue;  // unknown read group id: -1, as the reference
            auto jt = r->rg_index.find(it->second);
            if (jt != r->rg_index.end()) rg[i] = jt->second;
            else rg_new[i] = 1;
        }
    });
    {
        std::string key;
        for (size_t i = 0; i < n; i++) {
            if (!rg_new[i]) continue;
            size_t len = 0;
            const char *s = rg_of(i, len);
            key.assign(s, len);
            const std::string &name = r->rg_name_of_id[key];
            auto jt = r->rg_index.find(name);
            if (jt == r->rg_index.end()) {
                const uint32_t id = uint32_t(r->rg_names.size());
                r->rg_index[name] = id;
                r->rg_names.push_back(name);
                rg[i] = id;
            } else {
                rg[i] = jt->second;
            }
        }
    }
    // output arrays (rotating buffer sets)
    BatchBufs &bb = r->bufs[r->next_set];
    r->next_set = (r->next_set + 1) % FPB_BUFFER_SETS;
    const size_t sizes[17] = {n * 2, n * 4, n * 4, n * 4, n * 4, size_t(nc) * 4, n * 4, n * 4, size_t(ns) / 2,
                              n * 4, n * 4, size_t(nq), n * 4, n * 4, n * 2, n, n * 4};
    for (int k = 0; k < 17; k++)
        if (!bb.a[k].ensure(sizes[k] ? sizes[k] : 1)) return fail(r, "page-locked allocation failed");
    uint16_t *chrom = (uint16_t *)bb.a[0].p;
    uint32_t *astart = (uint32_t *)bb.a[1].p, *astop = (uint32_t *)bb.a[2].p, *mstart = (uint32_t *)bb.a[3].p;
    int32_t *isize = (int32_t *)bb.a[4].p;
    uint32_t *cigars = (uint32_t *)bb.a[5].p, *cstart = (uint32_t *)bb.a[6].p, *clen = (uint32_t *)bb.a[7].p;
    uint32_t *reads = (uint32_t *)bb.a[8].p, *rstart = (uint32_t *)bb.a[9].p, *rlen = (uint32_t *)bb.a[10].p;
    uint8_t *quals = (uint8_t *)bb.a[11].p;
    uint32_t *qstart = (uint32_t *)bb.a[12].p, *qlen = (uint32_t *)bb.a[13].p;
    uint16_t *flags = (uint16_t *)bb.a[14].p;
    uint8_t *mapq = (uint8_t *)bb.a[15].p;
    uint32_t *rgo = (uint32_t *)bb.a[16].p;
    const uint16_t *tmap = r->contig_of_target.data();
    const size_t ntarg = r->contig_of_target.size();
    parallel_for(r->threads, n, [&](size_t a, size_t z) {
        for (size_t i = a; i < z; i++) {
            const uint8_t *b = ub + rec[i] + 4;
            const int32_t tid = int32_t(rd32(b)), pos = int32_t(rd32(b + 4));
            const uint32_t l_name = b[8], mq = b[9], n_cig = rd16(b + 12), flag = rd16(b + 14);
            const uint32_t l_seq = rd32(b + 16);
            const int32_t mpos = int32_t(rd32(b + 24)), tlen = int32_t(rd32(b + 28));
            const uint8_t *cig = b + 32 + l_name;
            const uint8_t *seq = cig + 4 * size_t(n_cig);
            const uint8_t *qual = seq + (l_seq + 1) / 2;
            chrom[i] = (tid >= 0 && size_t(tid) < ntarg) ? tmap[tid] : uint16_t(0xFFFF);
            astart[i] = uint32_t(pos);
            // htslib bam_endpos - 1: reference-consuming ops (M, D, N, =, X) of a mapped read
            uint32_t rlen_ref = 0;
            for (uint32_t c = 0; c < n_cig; c++) {
                const uint32_t w = rd32(cig + 4 * c), op = w & 0xF;
                if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) rlen_ref += w >> 4;
                const uint32_t fop = op == 9 ? 8u : op;  // B has no firepony op: X (alignments.cu:188-200)
                cigars[cig_off[i] + c] = ((w >> 4) & 0xFFFFFFu) | (fop << 24);
            }
            astop[i] = (!(flag & 4) && n_cig > 0) ? uint32_t(pos) + rlen_ref - 1 : uint32_t(pos);
            mstart[i] = uint32_t(mpos);
            isize[i] = tlen;
            cstart[i] = cig_off[i];
            clen[i] = n_cig;
            // 4-bit symbols: BAM holds two per byte, high nibble first; the engine 8 per word, low first. A
            // word is four BAM bytes with their nibbles swapped; the last word is zero-padded
            const uint32_t s0 = sym_off[i];
            const uint32_t nbytes = (l_seq + 1) / 2, words = (l_seq + 7) / 8;
            uint32_t *dst = reads + s0 / 8;
            for (uint32_t wd = 0; wd < words; wd++) {
                uint32_t word = 0;
                for (uint32_t k = 0; k < 4; k++) {
                    const uint32_t j = wd * 4 + k;
                    if (j < nbytes) word |= uint32_t(kNibbleSwap[seq[j]]) << (8 * k);
                }
                dst[wd] = word;
            }
            if (l_seq & 1) dst[(l_seq - 1) / 8] &= ~(0xFu << (4 * (l_seq & 7)));  // odd length: no 2nd nibble
            rstart[i] = s0;
            rlen[i] = l_seq;
            memcpy(quals + qual_off[i], qual, l_seq);
            qstart[i] = qual_off[i];
            qlen[i] = l_seq;
            flags[i] = uint16_t(flag);
            mapq[i] = uint8_t(mq);
            rgo[i] = rg[i];
        }
    });
    r->upos += rec.back() + 4 + rd32(ub + rec.back());
    v->num_reads = uint32_t(n);
    v->num_cigar_ops = uint32_t(nc);
    v->num_read_symbols = ns;
    v->num_qualities = nq;
    v->chromosome = chrom; v->alignment_start = astart; v->alignment_stop = astop; v->mate_alignment_start = mstart;
    v->inferred_insert_size = isize; v->cigars = cigars; v->cigar_start = cstart; v->cigar_len = clen;
    v->reads = reads; v->read_start = rstart; v->read_len = rlen; v->qualities = quals; v->qual_start = qstart;
    v->qual_len = qlen; v->flags = flags; v->mapq = mapq; v->read_group = rgo;
    return int64_t(n);
}

}  // extern "C"

// ---- writer ----
namespace {

// htslib reg2bin (SAM spec 4.2.1): the smallest bin holding [beg, end)
int reg2bin(int beg, int end) {
    --end;
    if (beg >> 14 == end >> 14) return ((1 << 15) - 1) / 7 + (beg >> 14);
    if (beg >> 17 == end >> 17) return ((1 << 12) - 1) / 7 + (beg >> 17);
    if (beg >> 20 == end >> 20) return ((1 << 9) - 1) / 7 + (beg >> 20);
    if (beg >> 23 == end >> 23) return ((1 << 6) - 1) / 7 + (beg >> 23);
    if (beg >> 26 == end >> 26) return ((1 << 3) - 1) / 7 + (beg >> 26);
    return 0;
}

}  // namespace

static int write_bam_impl(const char *path, uint32_t num_targets, const char *const *target_names,
                          const uint32_t *target_lengths, uint32_t num_read_groups,
                          const char *const *read_group_ids, const fp_batch_view *batches, uint32_t num_batches,
                          int level, int threads);

extern "C" int fpb_write_bam(const char *path, uint32_t num_targets, const char *const *target_names,
                             const uint32_t *target_lengths, uint32_t num_read_groups,
                             const char *const *read_group_ids, const fp_batch_view *batches, uint32_t num_batches,
                             int level, int threads) {
    try {  // (no C++ exception crosses the C ABI)
        return write_bam_impl(path, num_targets, target_names, target_lengths, num_read_groups, read_group_ids,
                              batches, num_batches, level, threads);
    } catch (...) {
        return -1;
    }
}

static int write_bam_impl(const char *path, uint32_t num_targets, const char *const *target_names,
                          const uint32_t *target_lengths, uint32_t num_read_groups,
                          const char *const *read_group_ids, const fp_batch_view *batches, uint32_t num_batches,
                          int level, int threads) {
    if (!path || (num_targets && (!target_names || !target_lengths)) || (num_read_groups && !read_group_ids))
        return -1;
    const int nt = threads > 0 ? threads : int(std::max(1u, std::thread::hardware_concurrency()));
    std::vector<uint8_t> u;  // uncompressed stream
    std::string text = "@HD\tVN:1.6\tSO:unsorted\n";
    for (uint32_t t = 0; t < num_targets; t++)
        text += std::string("@SQ\tSN:") + target_names[t] + "\tLN:" + std::to_string(target_lengths[t]) + "\n";
    for (uint32_t g = 0; g < num_read_groups; g++) text += std::string("@RG\tID:") + read_group_ids[g] + "\n";
    u.insert(u.end(), {'B', 'A', 'M', 1});
    wr32(u, uint32_t(text.size()));
    u.insert(u.end(), text.begin(), text.end());
    wr32(u, num_targets);
    for (uint32_t t = 0; t < num_targets; t++) {
        const size_t l = strlen(target_names[t]) + 1;
        wr32(u, uint32_t(l));
        u.insert(u.end(), target_names[t], target_names[t] + l);
        wr32(u, target_lengths[t]);
    }
    uint64_t serial = 0;
    for (uint32_t bi = 0; bi < num_batches; bi++) {
        const fp_batch_view &v = batches[bi];
        for (uint32_t i = 0; i < v.num_reads; i++, serial++) {
            const std::string name = "r" + std::to_string(serial);
            const uint32_t n_cig = v.cigar_len[i], l_seq = v.read_len[i];
            const uint32_t rgi = v.read_group[i];
            const char *rgid = rgi < num_read_groups ? read_group_ids[rgi] : nullptr;
            const uint32_t aux = rgid ? uint32_t(3 + strlen(rgid) + 1) : 0;
            const uint32_t bs = 32 + uint32_t(name.size() + 1) + 4 * n_cig + (l_seq + 1) / 2 + l_seq + aux;
            wr32(u, bs);
            const uint16_t chrom = v.chromosome[i];
            const int32_t tid = chrom == 0xFFFF ? -1 : int32_t(chrom);
            const int32_t pos = int32_t(v.alignment_start[i]);
            uint32_t rref = 0;
            for (uint32_t c = 0; c < n_cig; c++) {
                const uint32_t w = v.cigars[v.cigar_start[i] + c], op = (w >> 24) & 0xF;
                if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) rref += w & 0xFFFFFF;
            }
            wr32(u, uint32_t(tid));
            wr32(u, uint32_t(pos));
            u.push_back(uint8_t(name.size() + 1));
            u.push_back(v.mapq[i]);
            wr16(u, uint16_t(pos >= 0 ? reg2bin(pos, pos + int(std::max<uint32_t>(rref, 1))) : 4680));
            wr16(u, uint16_t(n_cig));
            wr16(u, v.flags[i]);
            wr32(u, l_seq);
            wr32(u, uint32_t(v.mate_alignment_start[i] == 0xFFFFFFFFu ? -1 : tid));
            wr32(u, v.mate_alignment_start[i]);
            wr32(u, uint32_t(v.inferred_insert_size[i]));
            u.insert(u.end(), name.begin(), name.end());
            u.push_back(0);
            for (uint32_t c = 0; c < n_cig; c++) {
                const uint32_t w = v.cigars[v.cigar_start[i] + c];
                wr32(u, ((w & 0xFFFFFF) << 4) | ((w >> 24) & 0xF));
            }
            const uint64_t s0 = v.read_start[i];
            for (uint32_t j = 0; j < l_seq; j += 2) {
                auto sym = [&](uint64_t k) -> uint32_t { return (v.reads[k >> 3] >> ((k & 7) * 4)) & 0xF; };
                const uint32_t hi = sym(s0 + j), lo = j + 1 < l_seq ? sym(s0 + j + 1) : 0;
                u.push_back(uint8_t((hi << 4) | lo));
            }
            u.insert(u.end(), v.qualities + v.qual_start[i], v.qualities + v.qual_start[i] + l_seq);
            if (rgid) {
                u.insert(u.end(), {'R', 'G', 'Z'});
                u.insert(u.end(), rgid, rgid + strlen(rgid) + 1);
            }
        }
    }
    // BGZF: 0xff00-byte pieces deflated side by side, then the end-of-file block
    const size_t piece = 0xff00;
    const size_t nblk = (u.size() + piece - 1) / piece;
    std::vector<std::vector<uint8_t>> out(nblk);
    std::atomic<int> bad{0};
    parallel_for(nt, nblk, [&](size_t a, size_t z) {
        for (size_t k = a; k < z; k++) {
            const size_t off = k * piece, len = std::min(piece, u.size() - off);
            z_stream zs;
            memset(&zs, 0, sizeof(zs));
            if (deflateInit2(&zs, level, Z_DEFLATED, -15, 8, Z_DEFAULT_STRATEGY) != Z_OK) { bad = 1; continue; }
            std::vector<uint8_t> c(deflateBound(&zs, uLong(len)) + 32);
            zs.next_in = u.data() + off;
            zs.avail_in = uInt(len);
            zs.next_out = c.data();
            zs.avail_out = uInt(c.size());
            if (deflate(&zs, Z_FINISH) != Z_STREAM_END) bad = 1;
            const size_t clen = c.size() - zs.avail_out;
            deflateEnd(&zs);
            const size_t bsize = 18 + clen + 8;
            if (bsize > 65536) { bad = 1; continue; }
            std::vector<uint8_t> &o = out[k];
            o = {31, 139, 8, 4, 0, 0, 0, 0, 0, 255, 6, 0, 66, 67, 2, 0};
            wr16(o, uint16_t(bsize - 1));
            o.insert(o.end(), c.begin(), c.begin() + long(clen));
            wr32(o, uint32_t(crc32(0L, u.data() + off, uInt(len))));
            wr32(o, uint32_t(len));
        }
    });
    if (bad) return -1;
    FILE *f = fopen(path, "wb");
    if (!f) return -1;
    bool ok = true;
    for (const auto &o : out) ok = ok && fwrite(o.data(), 1, o.size(), f) == o.size();
    static const uint8_t eof_block[28] = {31, 139, 8, 4, 0, 0, 0, 0, 0, 255, 6, 0, 66, 67, 2, 0, 27, 0, 3, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    ok = ok && fwrite(eof_block, 1, 28, f) == 28;
    ok = (fclose(f) == 0) && ok;
    return ok ? 0 : -1;
}
