// Host check of the BGZF block decoder (firepony_gb300/csrc/bgzf_inflate.cuh) against zlib: round trips of
// raw DEFLATE streams made by zlib at every level and strategy from varied data, CRC-32 and CRC concatenation
// against zlib's crc32, the GPU's round-based match resolution against the serial one, and corrupt streams
// (bit flips, truncation), which must end in an error status or in output of the right size, never outside
// the buffers (the test builds this file with the address and undefined-behaviour sanitizers). Prints "ok" and
// exits 0 when every case passes.
#include <zlib.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "bgzf_inflate.cuh"

static int failures = 0;
#define CHECK(c, ...)                                  \
    do {                                               \
        if (!(c)) {                                    \
            if (failures < 20) {                       \
                fprintf(stderr, __VA_ARGS__);          \
                fprintf(stderr, "\n");                 \
            }                                          \
            failures++;                                \
        }                                              \
    } while (0)

static std::vector<uint8_t> deflate_raw(const std::vector<uint8_t> &u, int level, int strategy, int mem) {
    z_stream zs;
    memset(&zs, 0, sizeof(zs));
    deflateInit2(&zs, level, Z_DEFLATED, -15, mem, strategy);
    std::vector<uint8_t> c(deflateBound(&zs, uLong(u.size())) + 64);
    zs.next_in = const_cast<Bytef *>(u.data());
    zs.avail_in = uInt(u.size());
    zs.next_out = c.data();
    zs.avail_out = uInt(c.size());
    deflate(&zs, Z_FINISH);
    c.resize(c.size() - zs.avail_out);
    deflateEnd(&zs);
    return c;
}

// The GPU's match resolution (k_resolve_crc in bam_gpu.cu) restated on one thread: groups of 32 matches, a lane
// each, in rounds; a lane copies its match once its source ends at or below the lowest destination of the
// group's earlier pending matches. Lanes ready in the same round touch disjoint bytes, so copying them in lane
// order gives what the warp writes. Returns false if a round resolves nothing.
static bool resolve_rounds(std::vector<uint8_t> &out, const std::vector<uint32_t> &m, uint32_t nm) {
    for (uint32_t j0 = 0; j0 < nm; j0 += 32) {
        bool pending[32];
        uint32_t mp[32], len[32], dist[32], src0[32], src_end[32];
        for (uint32_t l = 0; l < 32; l++) {
            const uint32_t j = j0 + l;
            pending[l] = j < nm;
            mp[l] = pending[l] ? m[2 * j] : 0xFFFFFFFFu;
            const uint32_t ml = pending[l] ? m[2 * j + 1] : 0u;
            len[l] = ml >> 16;
            dist[l] = ml & 0xFFFFu;
            src0[l] = mp[l] - dist[l];
            src_end[l] = src0[l] + (len[l] < dist[l] ? len[l] : dist[l]);
        }
        for (;;) {
            bool any = false, ready[32];
            uint32_t below = 0xFFFFFFFFu;
            for (uint32_t l = 0; l < 32; l++) {
                ready[l] = pending[l] && src_end[l] <= below;
                if (pending[l] && mp[l] < below) below = mp[l];
                any |= pending[l];
            }
            if (!any) break;
            bool progress = false;
            for (uint32_t l = 0; l < 32; l++) {
                if (!ready[l]) continue;
                progress = true;
                uint32_t k = 0;
                for (uint32_t c = 0; c < len[l]; c++) {
                    out[mp[l] + c] = out[src0[l] + k];
                    k = k + 1 == dist[l] ? 0u : k + 1;
                }
                pending[l] = false;
            }
            if (!progress) return false;
        }
    }
    return true;
}

static int decode(const std::vector<uint8_t> &c, std::vector<uint8_t> &out, uint32_t size) {
    static fpinf::Tables t;
    static fpinf::Work w;
    out.assign(size, 0xA5);
    std::vector<uint32_t> m(2 * fpinf::match_capacity(size));
    uint32_t nm = 0;
    // the input is copied to an exact-size heap buffer so that the sanitizer sees any over-read
    std::vector<uint8_t> in(c);
    const int st = fpinf::inflate_tokens(in.empty() ? nullptr : in.data(), uint32_t(in.size()),
                                         out.empty() ? nullptr : out.data(), size, m.data(),
                                         fpinf::match_capacity(size), &nm, t, w);
    if (st == fpinf::OK) {
        std::vector<uint8_t> lit(out);
        fpinf::resolve_matches_serial(out.data(), m.data(), nm);
        CHECK(resolve_rounds(lit, m, nm) && lit == out, "round-based match resolution differs (%u matches)", nm);
    }
    return st;
}

static std::vector<uint8_t> make_data(std::mt19937_64 &rng, int kind, size_t n) {
    std::vector<uint8_t> u(n);
    switch (kind) {
    case 0:  // random bytes
        for (auto &x : u) x = uint8_t(rng());
        break;
    case 1:  // one byte value
        for (auto &x : u) x = 'A';
        break;
    case 2: {  // short alphabet with runs (qualities, bases)
        for (size_t i = 0; i < n;) {
            const uint8_t v = uint8_t(30 + rng() % 12);
            size_t r = 1 + rng() % 6;
            for (; r && i < n; r--) u[i++] = v;
        }
        break;
    }
    case 3: {  // records with repeated structure at varying distances
        for (size_t i = 0; i < n; i++) {
            const size_t rec = i % 337;
            u[i] = rec < 40 ? uint8_t("r12345\tchr1\t100\t60\t151M\tRG:Z:rg3\t"[rec % 34]) : uint8_t(33 + rng() % 41);
        }
        break;
    }
    default: {  // text-like with long repeats
        const char *words[] = {"alpha ", "beta ", "gamma ", "delta ", "epsilon ", "zeta\n"};
        std::string t;
        while (t.size() < n) t += words[rng() % 6];
        if (n) memcpy(u.data(), t.data(), n);
    }
    }
    return u;
}

int main() {
    std::mt19937_64 rng(12345);
    // round trips
    const size_t sizes[] = {0, 1, 2, 3, 17, 258, 259, 1000, 32768, 32769, 65280, 65536};
    const int strategies[] = {Z_DEFAULT_STRATEGY, Z_FILTERED, Z_HUFFMAN_ONLY, Z_RLE, Z_FIXED};
    int cases = 0;
    for (size_t n : sizes)
        for (int kind = 0; kind < 5; kind++)
            for (int level = 0; level <= 9; level++)
                for (int strategy : strategies) {
                    if (level != 1 && level != 6 && level != 9 && strategy != Z_DEFAULT_STRATEGY) continue;
                    const std::vector<uint8_t> u = make_data(rng, kind, n);
                    const std::vector<uint8_t> c = deflate_raw(u, level, strategy, 8);
                    std::vector<uint8_t> out;
                    const int st = decode(c, out, uint32_t(n));
                    CHECK(st == fpinf::OK, "n=%zu kind=%d level=%d strategy=%d: status %d", n, kind, level, strategy, st);
                    CHECK(st != fpinf::OK || out == u, "n=%zu kind=%d level=%d strategy=%d: output differs", n, kind,
                          level, strategy);
                    cases++;
                }
    // wrong expected size
    {
        const std::vector<uint8_t> u = make_data(rng, 3, 5000);
        const std::vector<uint8_t> c = deflate_raw(u, 6, Z_DEFAULT_STRATEGY, 8);
        std::vector<uint8_t> out;
        CHECK(decode(c, out, 4999) == fpinf::E_OUTPUT, "short output size not detected");
        CHECK(decode(c, out, 5001) == fpinf::E_SIZE, "long output size not detected");
    }
    // corrupt streams: flipped bits and truncation end in a status, inside the buffers
    int errors_seen = 0;
    for (int t = 0; t < 3000; t++) {
        const size_t n = 1 + rng() % 20000;
        const std::vector<uint8_t> u = make_data(rng, int(rng() % 5), n);
        std::vector<uint8_t> c = deflate_raw(u, int(rng() % 10), Z_DEFAULT_STRATEGY, 8);
        if (rng() % 4 == 0) {
            c.resize(rng() % (c.size() + 1));
        } else {
            const int flips = 1 + int(rng() % 8);
            for (int f = 0; f < flips && !c.empty(); f++) c[rng() % c.size()] ^= uint8_t(1u << (rng() % 8));
        }
        std::vector<uint8_t> out;
        const int st = decode(c, out, uint32_t(n));
        errors_seen += st != fpinf::OK;
        CHECK(st >= 0 && st <= fpinf::E_MATCHES, "bad status %d", st);
    }
    CHECK(errors_seen > 1000, "corrupt streams mostly not detected (%d)", errors_seen);
    // random garbage
    for (int t = 0; t < 2000; t++) {
        std::vector<uint8_t> c(rng() % 400);
        for (auto &x : c) x = uint8_t(rng());
        std::vector<uint8_t> out;
        decode(c, out, uint32_t(rng() % 70000));
    }
    // CRC-32
    uint32_t table[256];
    fpinf::crc_table(table);
    for (int t = 0; t < 200; t++) {
        const size_t na = rng() % 3000, nb = rng() % 70000;
        const std::vector<uint8_t> a = make_data(rng, 0, na), b = make_data(rng, 0, nb);
        std::vector<uint8_t> ab(a);
        ab.insert(ab.end(), b.begin(), b.end());
        const uint32_t ca = fpinf::crc_bytes(table, a.data(), uint32_t(na));
        const uint32_t cb = fpinf::crc_bytes(table, b.data(), uint32_t(nb));
        CHECK(ca == uint32_t(crc32(0, a.data(), uInt(na))), "crc of %zu bytes differs from zlib", na);
        CHECK(fpinf::crc_concat(ca, cb, nb) == uint32_t(crc32(0, ab.data(), uInt(ab.size()))),
              "crc concatenation differs (%zu + %zu bytes)", na, nb);
    }
    if (failures) {
        fprintf(stderr, "%d failures\n", failures);
        return 1;
    }
    printf("ok %d round trips, %d corrupt streams detected\n", cases, errors_seen);
    return 0;
}
