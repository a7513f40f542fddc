// Internal to libfpbam: the reader's state, shared by the host decoder (bam.cpp) and the GPU decoder
// (bam_gpu.cu).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "firepony_gb300_bam.h"

namespace fpb_detail {

inline uint16_t rd16(const uint8_t *p) { return uint16_t(p[0] | (p[1] << 8)); }
inline uint32_t rd32(const uint8_t *p) { return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24); }
inline void wr16(std::vector<uint8_t> &v, uint16_t x) { v.push_back(uint8_t(x)); v.push_back(uint8_t(x >> 8)); }
inline void wr32(std::vector<uint8_t> &v, uint32_t x) { for (int i = 0; i < 4; i++) v.push_back(uint8_t(x >> (8 * i))); }

// host buffer for batch arrays (grows; contents not kept): page-locked when a CUDA device is present, so
// the engine's copies run asynchronously; ordinary memory otherwise (decoding needs no GPU)
struct PinnedBuf {
    void *p = nullptr;
    size_t cap = 0;
    bool pinned = false;
    void release() {
        if (p) { if (pinned) cudaFreeHost(p); else free(p); }
        p = nullptr;
        cap = 0;
    }
    bool ensure(size_t bytes) {
        if (bytes <= cap && p) return true;
        release();
        const size_t want = std::max<size_t>(bytes + bytes / 4, 4096);
        if (cudaHostAlloc(&p, want, cudaHostAllocDefault) == cudaSuccess) {
            pinned = true;
        } else {
            cudaGetLastError();  // clear the failed allocation's error
            pinned = false;
            p = malloc(want);
            if (!p) return false;
        }
        cap = want;
        return true;
    }
    ~PinnedBuf() { release(); }
};

// growable byte buffer that, unlike std::vector, does not zero new bytes (the streams are filled by fread
// and inflate right after growing)
struct ByteBuf {
    uint8_t *p = nullptr;
    size_t n = 0, cap = 0;
    size_t size() const { return n; }
    uint8_t *data() { return p; }
    const uint8_t *data() const { return p; }
    bool resize(size_t m) {
        if (m > cap) {
            const size_t c = std::max(m, cap + cap / 2);
            void *q = realloc(p, c);
            if (!q) return false;
            p = static_cast<uint8_t *>(q);
            cap = c;
        }
        n = m;
        return true;
    }
    void erase_prefix(size_t k) {
        if (k == 0) return;
        memmove(p, p + k, n - k);
        n -= k;
    }
    ~ByteBuf() { free(p); }
};

inline double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// one set of batch arrays, in fp_batch_view order
struct BatchBufs {
    PinnedBuf a[17];
};

struct DeviceDecoder;  // bam_gpu.cu
void destroy_device_decoder(DeviceDecoder *d);

}  // namespace fpb_detail

struct fpb_reader {
    FILE *f = nullptr;
    int threads = 1;
    std::string err;
    bool eof_in = false;             // no more compressed input
    fpb_detail::ByteBuf cbuf;        // compressed bytes not yet inflated
    size_t cpos = 0;
    fpb_detail::ByteBuf ubuf;        // uncompressed stream not yet decoded
    size_t upos = 0;
    // header
    std::vector<std::string> target_names;
    std::vector<uint32_t> target_lens;
    std::vector<uint16_t> contig_of_target;
    std::unordered_map<std::string, std::string> rg_name_of_id;  // @RG ID -> name (PU if present, else ID)
    std::unordered_map<std::string, uint32_t> rg_index;         // name -> id, in order of first occurrence
    std::vector<std::string> rg_names;
    fpb_detail::BatchBufs bufs[FPB_BUFFER_SETS];
    int next_set = 0;
    fpb_stats stats{};
    bool failed = false;  // a batch failed: the stream state is undefined, every later call fails
    std::string failure;
    int mode = 0;  // 0: no batch yet, 1: host decoding (fpb_next_batch), 2: GPU decoding (fpb_next_batch_device)
    fpb_detail::DeviceDecoder *dev = nullptr;
};
