// Reference store (include/firepony_gb300_store.h): the contigs and known sites an engine reads, as one image
// that is published as a POSIX shared-memory segment and uploaded to a GPU with one copy.
//
// The reference keeps the same data as host databases, serialises them into one shm segment per input file
// (firepony-loader.cu:33-93, mmap.cu:146-190) and, when a segment of the file's name exists, reads them back
// instead of parsing the file (loader/reference.cu:133-143, loader/variants.cu:48-58). Here the segment holds
// the device layout itself, so a process that maps it attaches the reference with one host-to-device copy.
//
// Image layout (native byte order, all offsets from the image start):
//   ImageHeader (64 B) | DirEntry[num_contigs] (48 B each) | payload
// The payload holds per contig the packed words ((num_bases + 7) / 8 words, the unused symbols of the last
// word zeroed, then one zero word: the engine's kernels may read one word past a contig's end) and, when the
// contig has known sites, start[n], stop[n] and the prefix maximum of the stops maxend[n] as u32. Every
// array starts on a 256-byte boundary of the image, so the device copy keeps the alignment of cudaMalloc.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "firepony_gb300_store.h"
#include "refstore_internal.h"

using namespace fpg;

namespace {

constexpr char MAGIC[8] = {'F', 'P', 'G', 'B', 'R', 'E', 'F', 'S'};
constexpr u32 VERSION = 1;
constexpr u32 READY = 0x52454459u;  // set last by the writer: the segment is complete
constexpr u64 ALIGN = 256;

struct ImageHeader {
    char magic[8];
    u32 version;
    u32 num_contigs;
    u64 image_bytes;
    u64 total_bases;
    u64 total_sites;
    u64 dir_hash;  // FNV-1a over the fields above and the directory
    u32 ready;
    u32 reserved[3];
};
static_assert(sizeof(ImageHeader) == 64, "image header size");

struct DirEntry {
    u64 num_bases;
    u64 contig_off;
    u64 contig_words;  // (num_bases + 7) / 8 + 1
    u64 sites_off;     // 0 when num_sites == 0
    u32 num_sites;
    u32 reserved;
    u64 reserved2;
};
static_assert(sizeof(DirEntry) == 48, "directory entry size");

u64 align_up(u64 x) { return (x + ALIGN - 1) / ALIGN * ALIGN; }

u64 fnv1a(u64 h, const void *p, size_t n) {
    const u8 *b = static_cast<const u8 *>(p);
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

u64 dir_hash(const ImageHeader &h, const DirEntry *dir) {
    u64 x = 0xcbf29ce484222325ull;
    x = fnv1a(x, h.magic, sizeof(h.magic));
    x = fnv1a(x, &h.version, sizeof(h.version));
    x = fnv1a(x, &h.num_contigs, sizeof(h.num_contigs));
    x = fnv1a(x, &h.image_bytes, sizeof(h.image_bytes));
    x = fnv1a(x, &h.total_bases, sizeof(h.total_bases));
    x = fnv1a(x, &h.total_sites, sizeof(h.total_sites));
    return fnv1a(x, dir, sizeof(DirEntry) * h.num_contigs);
}

bool valid_shm_name(const char *name) {
    if (!name || name[0] != '/' || !name[1]) return false;
    const size_t n = strlen(name);
    if (n > NAME_MAX) return false;
    return strchr(name + 1, '/') == nullptr;
}

std::string sys_error(const char *what, const char *name) {
    return std::string(what) + " " + name + ": " + strerror(errno);
}

// why the calling thread's last fp_refstore_open / fp_refstore_create failed
thread_local std::string g_open_error;
fp_status open_fail(fp_status s, std::string m) {
    g_open_error = std::move(m);
    return s;
}

}  // namespace

struct fp_refstore {
    std::string err;
    u32 nc = 0;
    // a built store: host copies (words with the padding word, start/stop/maxend)
    std::vector<std::vector<u32>> words;
    std::vector<u64> bases;
    std::vector<std::vector<u32>> sites;
    // a mapped store
    bool mapped = false;
    const u8 *map = nullptr;
    size_t map_bytes = 0;
    // the device copy
    int device = -1;
    void *d_image = nullptr;
    void *d_tables = nullptr;  // DevContig[nc] then DevSites[nc]
    DevRef ref{};
    std::atomic<u32> attached{0};

    fp_status fail(fp_status s, std::string m) {
        err = std::move(m);
        return s;
    }
    const ImageHeader &header() const { return *reinterpret_cast<const ImageHeader *>(map); }
    const DirEntry *dir() const { return reinterpret_cast<const DirEntry *>(map + sizeof(ImageHeader)); }

    void contig(u32 i, const u32 *&w, u64 &n) const {
        if (mapped) {
            w = reinterpret_cast<const u32 *>(map + dir()[i].contig_off);
            n = dir()[i].num_bases;
        } else {
            w = words[i].data();
            n = bases[i];
        }
    }
    // start[n], stop[n], maxend[n]
    void site_arrays(u32 i, const u32 *&s, u32 &n) const {
        if (mapped) {
            n = dir()[i].num_sites;
            s = n ? reinterpret_cast<const u32 *>(map + dir()[i].sites_off) : nullptr;
        } else {
            n = u32(sites[i].size() / 3);
            s = n ? sites[i].data() : nullptr;
        }
    }
    u64 total_bases() const {
        u64 t = 0;
        for (u32 i = 0; i < nc; i++) {
            const u32 *w;
            u64 n;
            contig(i, w, n);
            t += n;
        }
        return t;
    }
    u64 total_sites() const {
        u64 t = 0;
        for (u32 i = 0; i < nc; i++) {
            const u32 *s;
            u32 n;
            site_arrays(i, s, n);
            t += n;
        }
        return t;
    }

    // directory of a built store's image; returns the image size
    u64 layout(std::vector<DirEntry> &d) const {
        d.assign(nc, DirEntry{});
        u64 off = align_up(sizeof(ImageHeader) + sizeof(DirEntry) * u64(nc));
        for (u32 i = 0; i < nc; i++) {
            d[i].num_bases = bases[i];
            d[i].contig_words = words[i].size();
            d[i].contig_off = off;
            off = align_up(off + d[i].contig_words * 4);
            d[i].num_sites = u32(sites[i].size() / 3);
            if (d[i].num_sites) {
                d[i].sites_off = off;
                off = align_up(off + u64(d[i].num_sites) * 12);
            }
        }
        return off;
    }
    u64 image_bytes() const {  // (allocates nothing)
        if (mapped) return map_bytes;
        u64 off = align_up(sizeof(ImageHeader) + sizeof(DirEntry) * u64(nc));
        for (u32 i = 0; i < nc; i++) {
            off = align_up(off + u64(words[i].size()) * 4);
            if (!sites[i].empty()) off = align_up(off + u64(sites[i].size()) * 4);
        }
        return off;
    }
    // writes a built store's image into `dst` (image_bytes() bytes, zero-filled); the ready mark is left 0
    void write_image(u8 *dst) const {
        std::vector<DirEntry> d;
        ImageHeader h{};
        memcpy(h.magic, MAGIC, sizeof(MAGIC));
        h.version = VERSION;
        h.num_contigs = nc;
        h.image_bytes = layout(d);
        h.total_bases = total_bases();
        h.total_sites = total_sites();
        h.dir_hash = dir_hash(h, d.data());
        h.ready = 0;
        memcpy(dst, &h, sizeof(h));
        memcpy(dst + sizeof(h), d.data(), sizeof(DirEntry) * nc);
        for (u32 i = 0; i < nc; i++) {
            memcpy(dst + d[i].contig_off, words[i].data(), words[i].size() * 4);
            if (d[i].num_sites) memcpy(dst + d[i].sites_off, sites[i].data(), sites[i].size() * 4);
        }
    }

    // checks a mapping of `bytes` bytes; empty string when it is a complete image of this format
    static std::string check_image(const u8 *p, size_t bytes) {
        if (bytes < sizeof(ImageHeader)) return "segment smaller than an image header";
        const ImageHeader &h = *reinterpret_cast<const ImageHeader *>(p);
        if (memcmp(h.magic, MAGIC, sizeof(MAGIC)) != 0) return "not a reference store image";
        if (h.version != VERSION) return "reference store image version " + std::to_string(h.version);
        if (__atomic_load_n(&h.ready, __ATOMIC_ACQUIRE) != READY) return "segment is incomplete (writer not done)";
        if (h.image_bytes != bytes) return "image size does not match the segment size";
        if (sizeof(ImageHeader) + sizeof(DirEntry) * u64(h.num_contigs) > bytes) return "directory out of range";
        const DirEntry *d = reinterpret_cast<const DirEntry *>(p + sizeof(ImageHeader));
        if (dir_hash(h, d) != h.dir_hash) return "directory checksum mismatch";
        u64 tb = 0, ts = 0;
        for (u32 i = 0; i < h.num_contigs; i++) {
            const DirEntry &e = d[i];
            if (e.contig_words != (e.num_bases + 7) / 8 + 1 || e.contig_off % ALIGN ||
                e.contig_off > bytes || e.contig_words * 4 > bytes - e.contig_off)
                return "contig " + std::to_string(i) + " out of range";
            if (e.num_sites && (e.sites_off % ALIGN || e.sites_off > bytes || u64(e.num_sites) * 12 > bytes - e.sites_off))
                return "known sites of contig " + std::to_string(i) + " out of range";
            tb += e.num_bases;
            ts += e.num_sites;
        }
        if (tb != h.total_bases || ts != h.total_sites) return "totals do not match the directory";
        return "";
    }

    void free_device() {
        if (device < 0) return;
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        if (d_image) cudaFree(d_image);
        if (d_tables) cudaFree(d_tables);
        cudaSetDevice(prev);
        d_image = d_tables = nullptr;
        device = -1;
        ref = DevRef{};
    }
};

namespace fpg {

const DevRef *refstore_acquire(fp_refstore *s, int device, std::string &err, int &status) {
    if (s->device >= 0 && s->device != device) {
        err = "the reference store's device copy is on GPU " + std::to_string(s->device);
        status = FP_BAD_INPUT;
        return nullptr;
    }
    if (s->device < 0) {
        const fp_status u = fp_refstore_upload(s, device);
        if (u != FP_OK) {
            err = "reference store upload: " + s->err;
            status = u;
            return nullptr;
        }
    }
    s->attached.fetch_add(1);
    return &s->ref;
}

void refstore_release(fp_refstore *s) { s->attached.fetch_sub(1); }

}  // namespace fpg

extern "C" {

fp_status fp_refstore_create(uint32_t num_contigs, fp_refstore **out) {
    if (!out) return open_fail(FP_BAD_INPUT, "null output pointer");
    *out = nullptr;
    fp_refstore *s = new (std::nothrow) fp_refstore;
    if (!s) return open_fail(FP_OOM, "reference store");
    s->nc = num_contigs;
    try {
        s->words.assign(num_contigs, std::vector<u32>(1, 0u));
        s->bases.assign(num_contigs, 0);
        s->sites.assign(num_contigs, std::vector<u32>());
    } catch (...) {
        delete s;
        return open_fail(FP_OOM, "reference store directory");
    }
    *out = s;
    return FP_OK;
}

fp_status fp_refstore_set_contig(fp_refstore *s, uint32_t id, const uint32_t *packed4, uint64_t n) {
    if (!s) return FP_BAD_INPUT;
    if (s->mapped) return s->fail(FP_BAD_INPUT, "a mapped reference store is read-only");
    if (s->device >= 0) return s->fail(FP_BAD_INPUT, "the reference store has a device copy");
    if (id >= s->nc) return s->fail(FP_BAD_INPUT, "contig id out of range");
    if (!packed4 && n) return s->fail(FP_BAD_INPUT, "null contig words");
    const u64 w = (n + 7) / 8;
    try {
        std::vector<u32> v(w + 1, 0u);
        if (w) memcpy(v.data(), packed4, w * 4);
        if (n % 8) v[w - 1] &= (1u << ((n % 8) * 4)) - 1;  // symbols past the contig's end read as 0
        s->words[id].swap(v);
    } catch (...) {
        return s->fail(FP_OOM, "contig copy");
    }
    s->bases[id] = n;
    return FP_OK;
}

fp_status fp_refstore_set_known_sites(fp_refstore *s, uint32_t id, const uint32_t *start, const uint32_t *stop,
                                      uint32_t n) {
    if (!s) return FP_BAD_INPUT;
    if (s->mapped) return s->fail(FP_BAD_INPUT, "a mapped reference store is read-only");
    if (s->device >= 0) return s->fail(FP_BAD_INPUT, "the reference store has a device copy");
    if (id >= s->nc) return s->fail(FP_BAD_INPUT, "contig id out of range");
    if ((!start || !stop) && n) return s->fail(FP_BAD_INPUT, "null known-site arrays");
    for (u32 i = 1; i < n; i++)
        if (start[i] < start[i - 1]) return s->fail(FP_BAD_INPUT, "known sites must be sorted by start");
    try {
        std::vector<u32> v(size_t(n) * 3);
        for (u32 i = 0; i < n; i++) {
            v[i] = start[i];
            v[size_t(n) + i] = stop[i];
            // prefix maximum of the stops (loader/variants.cu:125-133)
            v[2 * size_t(n) + i] = i ? std::max(v[2 * size_t(n) + i - 1], stop[i]) : stop[0];
        }
        s->sites[id].swap(v);
    } catch (...) {
        return s->fail(FP_OOM, "known-site copy");
    }
    return FP_OK;
}

fp_status fp_refstore_shm_name(const char *path, char *name, size_t cap) {
    if (!path || !name) return FP_BAD_INPUT;
    char *abs = realpath(path, nullptr);
    if (!abs) return FP_BAD_INPUT;
    std::string r = std::string("/firepony_") + abs;
    free(abs);
    for (size_t i = 1; i < r.size(); i++)
        if (r[i] == '/') r[i] = '_';
    if (r.size() + 1 > cap) return FP_BAD_INPUT;
    memcpy(name, r.c_str(), r.size() + 1);
    return FP_OK;
}

fp_status fp_refstore_publish(const fp_refstore *cs, const char *name) {
    if (!cs) return FP_BAD_INPUT;
    fp_refstore *s = const_cast<fp_refstore *>(cs);  // only the error message changes
    if (!valid_shm_name(name)) return s->fail(FP_BAD_INPUT, "shared-memory name must be '/' followed by a name without '/'");
    const u64 bytes = s->image_bytes();
    if (shm_unlink(name) != 0 && errno != ENOENT) return s->fail(FP_BAD_INPUT, sys_error("shm_unlink", name));
    const int fd = shm_open(name, O_RDWR | O_CREAT | O_EXCL, 0600);
    if (fd < 0) return s->fail(FP_BAD_INPUT, sys_error("shm_open", name));
    auto undo = [&](fp_status st, const std::string &m) {
        close(fd);
        shm_unlink(name);
        return s->fail(st, m);
    };
    // reserve the pages: writing to a tmpfs page that cannot be allocated would raise SIGBUS
    const int fe = posix_fallocate(fd, 0, off_t(bytes));
    if (fe != 0) {
        errno = fe;
        return undo(fe == ENOSPC ? FP_OOM : FP_BAD_INPUT, sys_error("posix_fallocate", name));
    }
    void *p = mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_SHARED, fd, 0);
    if (p == MAP_FAILED) return undo(FP_BAD_INPUT, sys_error("mmap", name));
    u8 *dst = static_cast<u8 *>(p);
    if (s->mapped) {
        memcpy(dst, s->map, bytes);
        reinterpret_cast<ImageHeader *>(dst)->ready = 0;
    } else {
        try {
            s->write_image(dst);
        } catch (...) {
            munmap(p, bytes);
            return undo(FP_OOM, "image directory");
        }
    }
    __atomic_store_n(&reinterpret_cast<ImageHeader *>(dst)->ready, READY, __ATOMIC_RELEASE);
    munmap(p, bytes);
    close(fd);
    return FP_OK;
}

fp_status fp_refstore_open(const char *name, fp_refstore **out) {
    if (!out) return open_fail(FP_BAD_INPUT, "null output pointer");
    *out = nullptr;
    if (!valid_shm_name(name)) return open_fail(FP_BAD_INPUT, "shared-memory name must be '/' followed by a name without '/'");
    const int fd = shm_open(name, O_RDONLY, 0);
    if (fd < 0) return open_fail(FP_BAD_INPUT, sys_error("shm_open", name));
    struct stat st;
    if (fstat(fd, &st) != 0 || st.st_size <= 0) {
        close(fd);
        return open_fail(FP_BAD_INPUT, std::string("empty segment ") + name);
    }
    const size_t bytes = size_t(st.st_size);
    void *p = mmap(nullptr, bytes, PROT_READ, MAP_SHARED, fd, 0);
    close(fd);  // the mapping stays valid
    if (p == MAP_FAILED) return open_fail(FP_BAD_INPUT, sys_error("mmap", name));
    const std::string bad = fp_refstore::check_image(static_cast<const u8 *>(p), bytes);
    if (!bad.empty()) {
        munmap(p, bytes);
        return open_fail(FP_BAD_INPUT, std::string(name) + ": " + bad);
    }
    fp_refstore *s = new (std::nothrow) fp_refstore;
    if (!s) {
        munmap(p, bytes);
        return open_fail(FP_OOM, "reference store");
    }
    s->mapped = true;
    s->map = static_cast<const u8 *>(p);
    s->map_bytes = bytes;
    s->nc = s->header().num_contigs;
    *out = s;
    return FP_OK;
}

fp_status fp_refstore_unlink(const char *name) {
    if (!valid_shm_name(name)) return FP_BAD_INPUT;
    return shm_unlink(name) == 0 ? FP_OK : FP_BAD_INPUT;
}

fp_status fp_refstore_get_info(const fp_refstore *s, fp_refstore_info *out) {
    if (!s || !out) return FP_BAD_INPUT;
    out->num_contigs = s->nc;
    out->attached_engines = s->attached.load();
    out->total_bases = s->total_bases();
    out->total_sites = s->total_sites();
    out->image_bytes = s->image_bytes();
    out->mapped = s->mapped ? 1 : 0;
    out->device = s->device;
    return FP_OK;
}

fp_status fp_refstore_get_contig(const fp_refstore *s, uint32_t id, const uint32_t **packed4, uint64_t *n) {
    if (!s || !packed4 || !n || id >= s->nc) return FP_BAD_INPUT;
    const u32 *w;
    u64 nb;
    s->contig(id, w, nb);
    *packed4 = w;
    *n = nb;
    return FP_OK;
}

fp_status fp_refstore_get_known_sites(const fp_refstore *s, uint32_t id, const uint32_t **start,
                                      const uint32_t **stop, uint32_t *n) {
    if (!s || !start || !stop || !n || id >= s->nc) return FP_BAD_INPUT;
    const u32 *a;
    u32 ns;
    s->site_arrays(id, a, ns);
    *start = a;
    *stop = a ? a + ns : nullptr;
    *n = ns;
    return FP_OK;
}

fp_status fp_refstore_upload(fp_refstore *s, int device) {
    if (!s) return FP_BAD_INPUT;
    if (s->device == device) return FP_OK;
    if (s->device >= 0) {
        if (s->attached.load()) return s->fail(FP_BAD_INPUT, "engines read the store's device copy on another GPU");
        s->free_device();
    }
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return s->fail(FP_BAD_INPUT, "no GPU " + std::to_string(device));
    const u64 bytes = s->image_bytes();
    std::vector<u8> built;
    const u8 *img = s->map;
    fp_status st = FP_OK;
    std::string msg;
    try {
        if (!s->mapped) {
            built.assign(bytes, 0);
            s->write_image(built.data());
            img = built.data();
        }
    } catch (...) {
        cudaSetDevice(prev);
        return s->fail(FP_OOM, "image build");
    }
    std::vector<DevContig> hc(s->nc);
    std::vector<DevSites> hs(s->nc);
    const DirEntry *d = reinterpret_cast<const DirEntry *>(img + sizeof(ImageHeader));
    cudaError_t e = cudaMalloc(&s->d_image, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(s->d_image, img, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_tables, std::max<size_t>(1, s->nc) * (sizeof(DevContig) + sizeof(DevSites)));
    if (e == cudaSuccess) {
        const u8 *base = static_cast<const u8 *>(s->d_image);
        for (u32 i = 0; i < s->nc; i++) {
            hc[i] = DevContig{reinterpret_cast<const u32 *>(base + d[i].contig_off), d[i].num_bases};
            const u32 n = d[i].num_sites;
            const u32 *a = n ? reinterpret_cast<const u32 *>(base + d[i].sites_off) : nullptr;
            hs[i] = DevSites{a, a ? a + n : nullptr, a ? a + 2 * size_t(n) : nullptr, n, 0};
        }
        DevContig *tc = static_cast<DevContig *>(s->d_tables);
        DevSites *ts = reinterpret_cast<DevSites *>(tc + std::max<u32>(1, s->nc));
        if (s->nc) e = cudaMemcpy(tc, hc.data(), s->nc * sizeof(DevContig), cudaMemcpyHostToDevice);
        if (e == cudaSuccess && s->nc) e = cudaMemcpy(ts, hs.data(), s->nc * sizeof(DevSites), cudaMemcpyHostToDevice);
        s->ref = DevRef{tc, s->nc, ts, s->nc};
    }
    if (e != cudaSuccess) {
        st = e == cudaErrorMemoryAllocation ? FP_OOM : FP_DEVICE_ERROR;
        msg = std::string("reference store upload: ") + cudaGetErrorString(e);
        s->device = device;  // free_device needs it
        s->free_device();
        cudaSetDevice(prev);
        return s->fail(st, msg);
    }
    s->device = device;
    cudaSetDevice(prev);
    return FP_OK;
}

fp_status fp_refstore_destroy(fp_refstore *s) {
    if (!s) return FP_OK;
    if (s->attached.load())
        return s->fail(FP_BAD_INPUT, std::to_string(s->attached.load()) + " engines still read the reference store");
    s->free_device();
    if (s->mapped && s->map) munmap(const_cast<u8 *>(s->map), s->map_bytes);
    delete s;
    return FP_OK;
}

const char *fp_refstore_last_error(const fp_refstore *s) { return s ? s->err.c_str() : g_open_error.c_str(); }

}  // extern "C"
