/*
 * Seeded synthetic BQSR inputs: a random reference, known sites and alignment batches in the engine's
 * input layout (include/firepony_gb300.h). No public dataset is used; the generator reproduces the shapes,
 * sizes and value distributions of the benchmark configurations (read lengths, substitution profile rising
 * toward the 3' end, indel and soft-clip rates, discretised-normal qualities, read groups with quality
 * offsets, paired-end flags and insert sizes, duplicates and unmapped reads, known SNPs and indels with alt
 * alleles carried by a fraction of covering reads).
 *
 * Every batch is generated from (seed, batch index) alone, so batches can be produced in any order or in
 * parallel and the data set is identical on every machine.
 */
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>
#include <algorithm>

extern "C" {

typedef struct {
    uint64_t seed;
    uint32_t num_contigs;
    uint64_t total_reference_bp;
    double gc;                      /* GC fraction of the reference */
    uint32_t read_lengths[8];       /* read lengths drawn uniformly from this list */
    uint32_t num_read_lengths;
    int32_t paired;                 /* 1: paired-end (read1 forward / read2 reverse pairs) */
    double sub_rate;                /* mean substitution rate, rising linearly toward the 3' end */
    double indel_read_frac;         /* fraction of reads carrying one 1-5 bp indel (indel_mode 0) */
    int32_t indel_mode;             /* 0: single indel; 1: geometric number of indels on 0..8 */
    double geometric_p;             /* indel_mode 1: P(k) ~ (1-p)^k */
    double wide_deletion_frac;      /* reads carrying one extra 15 bp deletion (band width 21) */
    double softclip_frac;
    double short_fragment_frac;     /* paired reads with a fragment shorter than the read (adapter clip) */
    double qual_mean, qual_sd;
    int32_t qual_min, qual_max;
    uint32_t num_read_groups;
    int32_t rg_qual_offset_span;    /* read group g gets quality offset -span..+span spread over groups */
    double dup_frac;
    double unmapped_frac;           /* half flagged unmapped, half MAPQ 0 */
    uint32_t num_snps, num_indel_sites;
    double alt_frac;                /* probability a read covering a known SNP carries its alt allele */
} synth_config;

typedef struct {
    uint32_t num_contigs;
    uint64_t *contig_len;
    uint32_t **contig_words;        /* 4-bit packed */
    uint32_t *num_sites;
    uint32_t **site_start;
    uint32_t **site_stop;
    uint8_t **site_alt;             /* 4-bit alt symbol for SNP sites, 0 for indels */
} synth_reference;

typedef struct {
    uint32_t num_reads, num_cigar_ops;
    uint64_t num_read_symbols, num_qualities;
    uint16_t *chromosome;
    uint32_t *alignment_start, *alignment_stop, *mate_alignment_start;
    int32_t *inferred_insert_size;
    uint32_t *cigars, *cigar_start, *cigar_len;
    uint32_t *reads, *read_start, *read_len;
    uint8_t *qualities;
    uint32_t *qual_start, *qual_len;
    uint16_t *flags;
    uint8_t *mapq;
    uint32_t *read_group;
} synth_batch;

}

namespace {

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t &x) {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (int i = 0; i < 4; i++) s[i] = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {  // xoshiro256**
        const uint64_t result = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return result;
    }
    double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
    uint64_t below(uint64_t n) { return n ? next() % n : 0; }
};

const uint8_t IUPAC[4] = {1, 2, 4, 8};

inline void put4(uint32_t *w, uint64_t i, uint8_t v) {
    w[i >> 3] = (w[i >> 3] & ~(0xFu << ((i & 7) * 4))) | (uint32_t(v & 0xF) << ((i & 7) * 4));
}
inline uint8_t get4(const uint32_t *w, uint64_t i) { return (w[i >> 3] >> ((i & 7) * 4)) & 0xF; }

uint8_t random_base(Rng &r, double gc) {
    double u = r.uniform();
    if (u < gc * 0.5) return IUPAC[1];
    if (u < gc) return IUPAC[2];
    if (u < gc + (1 - gc) * 0.5) return IUPAC[0];
    return IUPAC[3];
}

struct QualTable {
    // cumulative distribution of the clamped, rounded normal
    std::vector<double> cdf;
    // guide[j]: the first index whose cdf value is >= j / GUIDE, where the search for any u in
    // [j / GUIDE, (j + 1) / GUIDE) starts (the result equals a binary search's, without its branch misses)
    static constexpr int GUIDE = 4096;
    std::vector<uint16_t> guide;
    int qmin;
    void build(double mean, double sd, int lo, int hi) {
        qmin = lo;
        cdf.assign(hi - lo + 1, 0.0);
        double acc = 0;
        for (int q = lo; q <= hi; q++) {
            double a = (q == lo) ? -1e300 : (q - 0.5 - mean) / sd;
            double b = (q == hi) ? 1e300 : (q + 0.5 - mean) / sd;
            double pa = (a < -1e299) ? 0.0 : 0.5 * std::erfc(-a / std::sqrt(2.0));
            double pb = (b > 1e299) ? 1.0 : 0.5 * std::erfc(-b / std::sqrt(2.0));
            acc += pb - pa;
            cdf[q - lo] = acc;
        }
        for (auto &c : cdf) c /= acc;
        guide.assign(GUIDE + 1, 0);
        for (int j = 0; j <= GUIDE; j++)
            guide[j] = uint16_t(std::lower_bound(cdf.begin(), cdf.end(), double(j) / GUIDE) - cdf.begin());
    }
    uint8_t draw(Rng &r) const {
        const double u = r.uniform();
        size_t i = guide[size_t(u * GUIDE)];
        while (i < cdf.size() && cdf[i] < u) i++;
        if (i >= cdf.size()) i = cdf.size() - 1;
        return uint8_t(qmin + int(i));
    }
};

struct Op { uint32_t op, len; };

template <typename T> T *alloc_copy(const std::vector<T> &v) {
    T *p = (T *)malloc(std::max<size_t>(v.size(), 1) * sizeof(T));
    if (!v.empty()) memcpy(p, v.data(), v.size() * sizeof(T));
    return p;
}

}  // namespace

extern "C" {

int synth_generate_reference(const synth_config *cfg, synth_reference *out) {
    Rng rng(cfg->seed * 1000003ull + 17);
    const uint32_t nc = cfg->num_contigs;
    out->num_contigs = nc;
    out->contig_len = (uint64_t *)calloc(nc, sizeof(uint64_t));
    out->contig_words = (uint32_t **)calloc(nc, sizeof(uint32_t *));
    out->num_sites = (uint32_t *)calloc(nc, sizeof(uint32_t));
    out->site_start = (uint32_t **)calloc(nc, sizeof(uint32_t *));
    out->site_stop = (uint32_t **)calloc(nc, sizeof(uint32_t *));
    out->site_alt = (uint8_t **)calloc(nc, sizeof(uint8_t *));
    // contig lengths: equal split with +-20% variation, summing to the total
    std::vector<double> w(nc);
    double ws = 0;
    for (uint32_t c = 0; c < nc; c++) { w[c] = 0.8 + 0.4 * rng.uniform(); ws += w[c]; }
    uint64_t assigned = 0;
    for (uint32_t c = 0; c < nc; c++) {
        uint64_t len = (c + 1 == nc) ? cfg->total_reference_bp - assigned : uint64_t(cfg->total_reference_bp * w[c] / ws);
        assigned += len;
        out->contig_len[c] = len;
    }
    // bases, generated in parallel per 1 Mbp block from its own seed
    for (uint32_t c = 0; c < nc; c++) {
        const uint64_t len = out->contig_len[c];
        uint32_t *words = (uint32_t *)calloc((len + 7) / 8 + 1, sizeof(uint32_t));
        const uint64_t block = 1 << 20;  // multiple of 8 symbols
        const uint64_t nblocks = (len + block - 1) / block;
        unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; t++) {
            th.emplace_back([&, t]() {
                for (uint64_t bi = t; bi < nblocks; bi += nt) {
                    Rng br(cfg->seed * 7919ull + c * 1000003ull + bi * 31ull + 5);
                    const uint64_t b0 = bi * block, b1 = std::min(len, b0 + block);
                    for (uint64_t i = b0; i < b1; i++) put4(words, i, random_base(br, cfg->gc));
                }
            });
        }
        for (auto &x : th) x.join();
        out->contig_words[c] = words;
    }
    // known sites, split over contigs by length
    const uint64_t total = cfg->total_reference_bp;
    for (uint32_t c = 0; c < nc; c++) {
        const uint64_t len = out->contig_len[c];
        uint32_t ns = uint32_t(double(cfg->num_snps) * len / total);
        uint32_t ni = uint32_t(double(cfg->num_indel_sites) * len / total);
        std::vector<std::pair<uint32_t, uint32_t>> sites;  // (start, stop)
        std::vector<uint8_t> alts;
        std::vector<uint32_t> pos;
        for (uint32_t i = 0; i < ns + ni; i++) pos.push_back(uint32_t(rng.below(len > 20 ? len - 10 : 1)));
        std::sort(pos.begin(), pos.end());
        pos.erase(std::unique(pos.begin(), pos.end()), pos.end());
        // choose which positions are indels
        std::vector<uint8_t> is_indel(pos.size(), 0);
        for (uint32_t i = 0; i < ni && !pos.empty(); i++) is_indel[rng.below(pos.size())] = 1;
        std::vector<uint32_t> st, sp;
        std::vector<uint8_t> al;
        for (size_t i = 0; i < pos.size(); i++) {
            st.push_back(pos[i]);
            if (is_indel[i]) {
                sp.push_back(pos[i] + 1 + uint32_t(rng.below(5)));
                al.push_back(0);
            } else {
                sp.push_back(pos[i]);
                uint8_t refb = get4(out->contig_words[c], pos[i]);
                uint8_t a;
                do { a = IUPAC[rng.below(4)]; } while (a == refb);
                al.push_back(a);
            }
        }
        out->num_sites[c] = uint32_t(st.size());
        out->site_start[c] = alloc_copy(st);
        out->site_stop[c] = alloc_copy(sp);
        out->site_alt[c] = alloc_copy(al);
    }
    return 0;
}

void synth_free_reference(synth_reference *r) {
    for (uint32_t c = 0; c < r->num_contigs; c++) {
        free(r->contig_words[c]); free(r->site_start[c]); free(r->site_stop[c]); free(r->site_alt[c]);
    }
    free(r->contig_len); free(r->contig_words); free(r->num_sites);
    free(r->site_start); free(r->site_stop); free(r->site_alt);
    memset(r, 0, sizeof(*r));
}

int synth_generate_batch(const synth_config *cfg, const synth_reference *ref, uint64_t batch_index,
                         uint32_t num_reads, synth_batch *out) {
    Rng rng(cfg->seed * 0x9E3779B97F4A7C15ull + batch_index * 0xD1B54A32D192ED03ull + 1);
    std::vector<QualTable> qt(std::max(1u, cfg->num_read_groups));
    for (uint32_t g = 0; g < qt.size(); g++) {
        int off = 0;
        if (cfg->rg_qual_offset_span > 0 && qt.size() > 1)
            off = -cfg->rg_qual_offset_span + int(std::lround(2.0 * cfg->rg_qual_offset_span * g / (qt.size() - 1)));
        qt[g].build(cfg->qual_mean + off, cfg->qual_sd, cfg->qual_min, cfg->qual_max);
    }
    uint64_t total = 0;
    for (uint32_t c = 0; c < ref->num_contigs; c++) total += ref->contig_len[c];

    std::vector<uint16_t> chromosome; std::vector<uint32_t> astart, astop, mstart; std::vector<int32_t> isize;
    std::vector<uint32_t> cigars, cstart, clen, rstart, rlen, qstart, qlen, rg;
    std::vector<uint8_t> quals, mapq; std::vector<uint16_t> flags;
    std::vector<uint8_t> syms;  // unpacked read symbols (padded)
    chromosome.reserve(num_reads);

    // per-read scratch, reused across reads
    struct Ev { uint32_t at; uint32_t op; uint32_t len; };
    std::vector<Op> ops, merged;
    std::vector<Ev> evs;
    uint32_t mate_pending = 0;  // paired mode: second read of a pair
    uint32_t pair_contig = 0, pair_r1_start = 0, pair_frag = 0, pair_len = 0;
    for (uint32_t r = 0; r < num_reads; r++) {
        const uint32_t L = cfg->read_lengths[rng.below(cfg->num_read_lengths ? cfg->num_read_lengths : 1)];
        // ---- alignment layout ----
        ops.clear();
        // indels
        int n_indels = 0;
        if (cfg->indel_mode == 0) {
            n_indels = rng.uniform() < cfg->indel_read_frac ? 1 : 0;
        } else {
            while (n_indels < 8 && rng.uniform() > cfg->geometric_p) n_indels++;
        }
        const bool wide = rng.uniform() < cfg->wide_deletion_frac;
        uint32_t clip_left = 0, clip_right = 0;
        if (rng.uniform() < cfg->softclip_frac) {
            uint32_t s = 1 + uint32_t(rng.below(10));
            if (rng.uniform() < 0.5) clip_left = s; else clip_right = s;
        }
        // read positions (inside the aligned part) that start an indel event
        evs.clear();
        const uint32_t core = L - clip_left - clip_right;
        for (int k = 0; k < n_indels; k++) {
            uint32_t at = 10 + uint32_t(rng.below(core > 20 ? core - 20 : 1));
            uint32_t op = rng.uniform() < 0.5 ? 1u : 2u;
            uint32_t len = 1 + uint32_t(rng.below(5));
            evs.push_back({at, op, len});
        }
        if (wide) evs.push_back({core / 2, 2u, 15u});
        std::sort(evs.begin(), evs.end(), [](const Ev &a, const Ev &b) { return a.at < b.at; });
        // build ops: S? (M [I|D])* M S?
        if (clip_left) ops.push_back({4, clip_left});
        uint32_t consumed = 0;  // read bases consumed by M/I in the core
        for (const Ev &e : evs) {
            if (e.at <= consumed || e.at >= core) continue;
            uint32_t m = e.at - consumed;
            if (e.op == 1 && consumed + m + e.len >= core) continue;  // keep the insertion inside the core
            ops.push_back({0, m});
            consumed += m;
            ops.push_back({e.op, e.len});
            if (e.op == 1) consumed += e.len;
        }
        if (core > consumed) ops.push_back({0, core - consumed});
        if (clip_right) ops.push_back({4, clip_right});
        // merge adjacent same ops
        merged.clear();
        for (auto &o : ops) {
            if (o.len == 0) continue;
            if (!merged.empty() && merged.back().op == o.op) merged.back().len += o.len; else merged.push_back(o);
        }
        uint32_t ref_span = 0;
        for (auto &o : merged) if (o.op == 0 || o.op == 2) ref_span += o.len;

        // ---- placement ----
        uint32_t contig;
        uint32_t pos;
        uint16_t f = 0;
        int32_t isz = 0;
        uint32_t mpos = 0;
        if (cfg->paired && mate_pending) {
            contig = pair_contig;
            // read2: reverse strand, ends at the fragment end
            int64_t p = int64_t(pair_r1_start) + int64_t(pair_frag) - int64_t(ref_span);
            if (p < 0) p = 0;
            pos = uint32_t(p);
            if (uint64_t(pos) + ref_span + 1 >= ref->contig_len[contig]) pos = uint32_t(ref->contig_len[contig] - ref_span - 2);
            f = 1 | 2 | 16 | 128;
            mpos = pair_r1_start;
            isz = -int32_t(pair_frag);
            mate_pending = 0;
        } else {
            uint64_t g = rng.below(total);
            contig = 0;
            while (contig + 1 < ref->num_contigs && g >= ref->contig_len[contig]) g -= ref->contig_len[contig++];
            const uint64_t clen_ = ref->contig_len[contig];
            uint64_t maxstart = clen_ > ref_span + 2 ? clen_ - ref_span - 2 : 0;
            pos = uint32_t(g % (maxstart + 1));
            if (cfg->paired) {
                uint32_t frag;
                if (rng.uniform() < cfg->short_fragment_frac) frag = L / 2 + uint32_t(rng.below(L / 2));
                else frag = 250 + uint32_t(rng.below(150));
                if (uint64_t(pos) + frag + 2 >= clen_) frag = uint32_t(clen_ - pos - 2);
                if (frag < ref_span) frag = ref_span;
                f = 1 | 2 | 32 | 64;
                pair_contig = contig; pair_r1_start = pos; pair_frag = frag; pair_len = L;
                mpos = pos + frag - ref_span;  // approximate mate start (its own span may differ)
                isz = int32_t(frag);
                mate_pending = 1;
            } else {
                if (rng.uniform() < 0.5) f |= 16;
            }
        }
        (void)pair_len;
        uint8_t mq = 60;
        if (rng.uniform() < cfg->dup_frac) f |= 1024;
        if (rng.uniform() < cfg->unmapped_frac) {
            if (rng.uniform() < 0.5) f |= 4; else mq = 0;
        }
        const uint32_t group = cfg->num_read_groups ? uint32_t(rng.below(cfg->num_read_groups)) : 0;

        // ---- bases and qualities ----
        const uint32_t *cw = ref->contig_words[contig];
        const uint32_t ns = ref->num_sites[contig];
        const uint32_t *sst = ref->site_start[contig];
        const uint8_t *salt = ref->site_alt[contig];
        const uint64_t rs = syms.size();
        const uint32_t padded = (L + 7) / 8 * 8;
        syms.resize(rs + padded, 0);
        const uint64_t qs = quals.size();
        quals.resize(qs + L);
        uint32_t rp = 0;       // read position
        uint32_t refp = pos;   // reference position
        size_t site = std::lower_bound(sst, sst + ns, pos) - sst;
        for (auto &o : merged) {
            for (uint32_t i = 0; i < o.len; i++) {
                if (o.op == 0) {
                    uint8_t b = get4(cw, refp);
                    while (site < ns && sst[site] < refp) site++;
                    if (site < ns && sst[site] == refp && salt[site] && rng.uniform() < cfg->alt_frac) b = salt[site];
                    const double pe = 2.0 * cfg->sub_rate * (rp + 0.5) / L;
                    if (rng.uniform() < pe) {
                        uint8_t nb;
                        do { nb = IUPAC[rng.below(4)]; } while (nb == b);
                        b = nb;
                    }
                    syms[rs + rp++] = b;
                    refp++;
                } else if (o.op == 1 || o.op == 4) {
                    syms[rs + rp++] = random_base(rng, cfg->gc);
                } else if (o.op == 2) {
                    refp++;
                }
            }
        }
        for (uint32_t i = 0; i < L; i++) quals[qs + i] = qt[group].draw(rng);

        chromosome.push_back(uint16_t(contig));
        astart.push_back(pos);
        astop.push_back(pos + ref_span - 1);
        mstart.push_back(mpos);
        isize.push_back(isz);
        cstart.push_back(uint32_t(cigars.size()));
        clen.push_back(uint32_t(merged.size()));
        for (auto &o : merged) cigars.push_back((o.len & 0xFFFFFFu) | (o.op << 24));
        rstart.push_back(uint32_t(rs));
        rlen.push_back(L);
        qstart.push_back(uint32_t(qs));
        qlen.push_back(L);
        flags.push_back(f);
        mapq.push_back(mq);
        rg.push_back(group);
    }
    // pack symbols
    std::vector<uint32_t> words((syms.size() + 7) / 8, 0);
    for (uint64_t i = 0; i < syms.size(); i++) put4(words.data(), i, syms[i]);

    out->num_reads = num_reads;
    out->num_cigar_ops = uint32_t(cigars.size());
    out->num_read_symbols = syms.size();
    out->num_qualities = quals.size();
    out->chromosome = alloc_copy(chromosome);
    out->alignment_start = alloc_copy(astart);
    out->alignment_stop = alloc_copy(astop);
    out->mate_alignment_start = alloc_copy(mstart);
    out->inferred_insert_size = alloc_copy(isize);
    out->cigars = alloc_copy(cigars);
    out->cigar_start = alloc_copy(cstart);
    out->cigar_len = alloc_copy(clen);
    out->reads = alloc_copy(words);
    out->read_start = alloc_copy(rstart);
    out->read_len = alloc_copy(rlen);
    out->qualities = alloc_copy(quals);
    out->qual_start = alloc_copy(qstart);
    out->qual_len = alloc_copy(qlen);
    out->flags = alloc_copy(flags);
    out->mapq = alloc_copy(mapq);
    out->read_group = alloc_copy(rg);
    return 0;
}

void synth_free_batch(synth_batch *b) {
    free(b->chromosome); free(b->alignment_start); free(b->alignment_stop); free(b->mate_alignment_start);
    free(b->inferred_insert_size); free(b->cigars); free(b->cigar_start); free(b->cigar_len); free(b->reads);
    free(b->read_start); free(b->read_len); free(b->qualities); free(b->qual_start); free(b->qual_len);
    free(b->flags); free(b->mapq); free(b->read_group);
    memset(b, 0, sizeof(*b));
}

}  // extern "C"
