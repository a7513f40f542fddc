// K4: exclusive scan, stable LSD radix sort of packed 64-bit covariate entries (dense key in the high 32
// bits, float mismatch bits in the low 32), and the ordered segmented fold into the resident mismatch
// table. Stable sorting keeps each key's entries in stream order, so folding a segment left to right from
// the running total reproduces the reference's append + stable sort + reduce_by_key of every batch
// (device/covariates.cu:172-201, device/covariate_table.cu:43-107) as one sequential float sum per key.
#include <mutex>

#include "kernels.h"
#include "firepony_gb300.h"

namespace fpg {

namespace {

constexpr u32 FULL = 0xffffffffu;
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// block-wide exclusive scan of one value per thread; returns the block total in *total
__device__ u32 block_exclusive_scan(u32 v, u32 *total) {
    __shared__ u32 warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u32 x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const u32 y = __shfl_up_sync(FULL, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        u32 s = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const u32 y = __shfl_up_sync(FULL, s, d);
            if (lane >= d) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    const u32 warp_prefix = warp ? warp_sums[warp - 1] : 0;
    *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const u32 *in, u64 n, u32 *sums) {
    const u64 base = u64(blockIdx.x) * SCAN_TILE + u64(threadIdx.x) * SCAN_ITEMS;
    u32 s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++)
        if (base + j < n) s += in[base + j];
    u32 total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const u32 *in, u64 n, const u32 *offsets, u32 *out) {
    const u64 base = u64(blockIdx.x) * SCAN_TILE + u64(threadIdx.x) * SCAN_ITEMS;
    u32 v[SCAN_ITEMS];
    u32 s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) {
        v[j] = base + j < n ? in[base + j] : 0;
        s += v[j];
    }
    u32 total;
    u32 p = block_exclusive_scan(s, &total) + (offsets ? offsets[blockIdx.x] : 0);
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) {
        if (base + j < n) out[base + j] = p;
        p += v[j];
    }
}

__global__ void k_scan_total(const u32 *in, u64 n, u32 *out) {
    // out[n] = out[n-1] + in[n-1]
    if (n) out[n] = out[n - 1] + in[n - 1];
    else out[0] = 0;
}

void scan_rec(const u32 *in, u32 *out, u64 n, u32 *tmp, cudaStream_t s) {
    const u64 blocks = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (blocks <= 1) {
        k_scan_apply<<<1, SCAN_THREADS, 0, s>>>(in, n, nullptr, out);
        g_kernel_launches++;
    } else {
        u32 *sums = tmp;
        u32 *sums_scan = tmp + blocks + 1;
        k_scan_reduce<<<u32(blocks), SCAN_THREADS, 0, s>>>(in, n, sums);
        scan_rec(sums, sums_scan, blocks, sums_scan + blocks + 1, s);
        k_scan_apply<<<u32(blocks), SCAN_THREADS, 0, s>>>(in, n, sums_scan, out);
        g_kernel_launches += 2;
    }
    k_scan_total<<<1, 1, 0, s>>>(in, n, out);
    g_kernel_launches++;
}

// ---- radix sort ----
// A tile of RS_TILE keys per block; warp w of the block takes the tile's w-th run of RS_WARP_KEYS consecutive
// keys, 32 per round, so tile order is (warp, round, lane). The scatter pass ranks each key among the equal
// digits before it in tile order (warp-private counters, no block barrier per round), reorders the tile by
// digit in shared memory, and writes each digit's run with consecutive threads on consecutive addresses.
constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ROUNDS = 16;
constexpr int RS_WARP_KEYS = 32 * RS_ROUNDS;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;

// The digit of a pass: key bits [shift, shift + 8) of the entry, cut at key_bits so that key bits above the
// sorted width never decide the order (the last pass of a width that is not a multiple of 8 takes fewer bits).
__device__ __forceinline__ u32 digit_mask(int shift, int key_bits) {
    const int w = key_bits - shift;
    return w >= 8 ? 0xFFu : ((1u << w) - 1u);
}
__device__ __forceinline__ u32 digit_of(u64 v, int shift, u32 mask) { return u32(v >> (32 + shift)) & mask; }

// The lanes of the warp holding a key with digit d (the caller's own lane included), from one ballot per digit
// bit; lanes without a key form their own group. Votes run on the integer pipe, where a match instruction
// would queue on the warp-divergence unit (measured: that unit 84-89% busy, the sort issue-bound on it).
__device__ __forceinline__ u32 digit_peers(u32 d, bool valid) {
    const u32 vm = __ballot_sync(FULL, valid);
    u32 peers = valid ? vm : ~vm;
#pragma unroll
    for (int b = 0; b < 8; b++) {
        const bool bit = (d >> b) & 1u;
        const u32 m = __ballot_sync(FULL, bit);
        peers &= bit ? m : ~m;
    }
    return peers;
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const u64 *in, u64 n, int shift, int key_bits, u32 *hist,
                                                        u32 nblocks) {
    const u32 dmask = digit_mask(shift, key_bits);
    __shared__ u32 h[RS_WARPS][256];  // per warp: only its own lanes update it
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int j = threadIdx.x; j < RS_WARPS * 256; j += RS_THREADS) (&h[0][0])[j] = 0;
    __syncthreads();
    const u64 wbase = u64(blockIdx.x) * RS_TILE + u64(warp) * RS_WARP_KEYS;
    u64 v[RS_ROUNDS];
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const u64 i = wbase + u64(r) * 32 + lane;
        v[r] = i < n ? in[i] : 0;
    }
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const bool valid = wbase + u64(r) * 32 + lane < n;
        const u32 d = digit_of(v[r], shift, dmask);
        const u32 peers = digit_peers(d, valid);
        // one update per distinct digit (distinct addresses within the instruction)
        if (valid && int(__ffs(peers)) - 1 == lane) h[warp][d] += u32(__popc(peers));
        __syncwarp();  // the next round's updater of a digit may be another lane
    }
    __syncthreads();
    u32 t = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) t += h[w][threadIdx.x];
    hist[u64(threadIdx.x) * nblocks + blockIdx.x] = t;
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const u64 *in, u64 n, int shift, int key_bits,
                                                           const u32 *offs, u32 nblocks, u64 *out) {
    const u32 dmask = digit_mask(shift, key_bits);
    __shared__ u64 buf[RS_TILE];            // the tile ordered by digit
    __shared__ u32 wcnt[RS_WARPS][256];     // per warp: digit counts, then the warp's first slot per digit
    __shared__ u32 tstart[256];             // first slot of each digit in the ordered tile
    __shared__ u32 gbase[256];              // global position of this tile's first key of each digit
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u32 lt = (1u << lane) - 1;
    for (int j = threadIdx.x; j < RS_WARPS * 256; j += RS_THREADS) (&wcnt[0][0])[j] = 0;
    gbase[threadIdx.x] = offs[u64(threadIdx.x) * nblocks + blockIdx.x];
    __syncthreads();
    const u64 tile0 = u64(blockIdx.x) * RS_TILE;
    const u64 wbase = tile0 + u64(warp) * RS_WARP_KEYS;
    u64 v[RS_ROUNDS];
    u32 rank[RS_ROUNDS / 2];  // per key: the warp's earlier keys with the same digit (< 512), two per word
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const u64 i = wbase + u64(r) * 32 + lane;
        v[r] = i < n ? in[i] : 0;
    }
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const bool valid = wbase + u64(r) * 32 + lane < n;
        const u32 d = digit_of(v[r], shift, dmask);
        const u32 peers = digit_peers(d, valid);
        const u32 before = valid ? wcnt[warp][d] : 0u;  // the digit's peers read one word together
        const u32 rk = before + u32(__popc(peers & lt));
        if (r & 1) rank[r >> 1] |= rk << 16;
        else rank[r >> 1] = rk;
        __syncwarp();
        if (valid && int(__ffs(peers)) - 1 == lane) wcnt[warp][d] = before + u32(__popc(peers));
        __syncwarp();
    }
    __syncthreads();
    {
        // thread d: the digit's count over the warps (warp-major within the digit), then its place in the tile
        const u32 d = threadIdx.x;
        u32 run = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) {
            const u32 c = wcnt[w][d];
            wcnt[w][d] = run;
            run += c;
        }
        u32 total;
        const u32 start = block_exclusive_scan(run, &total);
        tstart[d] = start;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) wcnt[w][d] += start;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const u64 i = wbase + u64(r) * 32 + lane;
        if (i < n) buf[wcnt[warp][digit_of(v[r], shift, dmask)] + ((rank[r >> 1] >> ((r & 1) * 16)) & 0xFFFFu)] = v[r];
    }
    __syncthreads();
    const u32 tile_n = u32(n - tile0 < u64(RS_TILE) ? n - tile0 : u64(RS_TILE));
    for (u32 p = threadIdx.x; p < tile_n; p += RS_THREADS) {
        const u64 key = buf[p];
        const u32 d = digit_of(key, shift, dmask);
        out[gbase[d] + (p - tstart[d])] = key;
    }
}

// ---- ordered fold ----
__global__ void k_heads(const u64 *s, u64 n, u32 *flag) {
    const u64 i = u64(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = (i == 0 || (s[i] >> 32) != (s[i - 1] >> 32)) ? 1u : 0u;
}

__global__ void k_head_list(const u32 *flag, const u32 *pos, u64 n, u32 *heads) {
    const u64 i = u64(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (flag[i]) heads[pos[i]] = u32(i);
}

// one warp per segment (grid-stride over segments): lanes load 32 entries at a time (coalesced) and the
// sum runs through them in order
__global__ void k_fold(const u64 *s, u64 n, const u32 *heads, const u32 *num_heads, float *mism) {
    const u32 nwarps = (gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    const u32 nh = *num_heads;
    for (u32 h = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; h < nh; h += nwarps) {
        const u64 start = heads[h];
        const u64 end = (h + 1 < nh) ? heads[h + 1] : n;
        const u32 key = u32(s[start] >> 32);
        float acc = mism[key];
        for (u64 c = start; c < end; c += 32) {
            const u64 i = c + lane;
            const float v = i < end ? __uint_as_float(u32(s[i])) : 0.0f;
            const int cnt = int(end - c < 32 ? end - c : 32);
            for (int j = 0; j < cnt; j++) {
                const float x = __shfl_sync(FULL, v, j);
                acc = __fadd_rn(acc, x);
            }
        }
        if (lane == 0) mism[key] = acc;
    }
}

}  // namespace

size_t scan_tmp_bytes(u64 n) {
    // sums and scanned sums for every level
    u64 total = 0;
    u64 m = n;
    while (m > u64(SCAN_TILE)) {
        m = (m + SCAN_TILE - 1) / SCAN_TILE;
        total += 2 * (m + 1);
    }
    return size_t(total + 64) * sizeof(u32);
}

void launch_exclusive_scan(const u32 *in, u32 *out, u64 n, void *tmp, cudaStream_t s) {
    scan_rec(in, out, n, reinterpret_cast<u32 *>(tmp), s);
}

size_t radix_tmp_bytes(u64 n) {
    const u64 nblocks = (n + RS_TILE - 1) / RS_TILE + 1;
    const u64 hist = nblocks * 256;
    return size_t(2 * (hist + 1)) * sizeof(u32) + scan_tmp_bytes(hist) + 256;
}

size_t fold_tmp_bytes(u64 n) { return size_t(3 * (n + 1)) * sizeof(u32) + scan_tmp_bytes(n) + 256; }

void launch_radix_sort(u64 *keys, u64 *alt, u64 n, int key_bits, void *tmp, size_t tmp_bytes, u64 **result,
                       cudaStream_t s) {
    (void)tmp_bytes;
    u64 *src = keys, *dst = alt;
    if (n > 1) {
        const u32 nblocks = u32((n + RS_TILE - 1) / RS_TILE);
        const u64 hist_n = u64(nblocks) * 256;
        u32 *hist = reinterpret_cast<u32 *>(tmp);
        u32 *offs = hist + hist_n + 1;
        void *stmp = offs + hist_n + 1;
        for (int shift = 0; shift < key_bits; shift += 8) {
            k_rs_hist<<<nblocks, RS_THREADS, 0, s>>>(src, n, shift, key_bits, hist, nblocks);
            scan_rec(hist, offs, hist_n, reinterpret_cast<u32 *>(stmp), s);
            k_rs_scatter<<<nblocks, RS_THREADS, 0, s>>>(src, n, shift, key_bits, offs, nblocks, dst);
            g_kernel_launches += 2;
            u64 *t = src;
            src = dst;
            dst = t;
        }
    }
    *result = src;
}

void launch_fold(const u64 *sorted, u64 n, float *mism, void *tmp, cudaStream_t s) {
    if (!n) return;
    u32 *flag = reinterpret_cast<u32 *>(tmp);
    u32 *pos = flag + n + 1;
    u32 *heads = pos + n + 1;
    void *stmp = heads + n + 1;
    const u32 blocks = u32((n + 255) / 256);
    k_heads<<<blocks, 256, 0, s>>>(sorted, n, flag);
    scan_rec(flag, pos, n, reinterpret_cast<u32 *>(stmp), s);
    k_head_list<<<blocks, 256, 0, s>>>(flag, pos, n, heads);
    // number of segments = pos[n]; a fixed grid of warps strides over them
    u64 fold_blocks = (n * 32 + 255) / 256;
    if (fold_blocks > 152 * 16) fold_blocks = 152 * 16;
    k_fold<<<u32(fold_blocks), 256, 0, s>>>(sorted, n, heads, pos + n, mism);
    g_kernel_launches += 3;
}

// ---- C ABI: the radix sort as a standalone primitive ----
namespace {

// Runs the LSD passes so that the last pass lands in `out`; the first pass reads `in` and never writes it.
void sort_into(const u64 *in, u64 *out, u64 *alt, u64 n, int key_bits, void *tmp, cudaStream_t s) {
    int passes = 0;
    for (int shift = 0; shift < key_bits; shift += 8) passes++;
    if (n <= 1 || passes == 0) {
        if (n) cudaMemcpyAsync(out, in, n * sizeof(u64), cudaMemcpyDeviceToDevice, s);
        return;
    }
    const u32 nblocks = u32((n + RS_TILE - 1) / RS_TILE);
    const u64 hist_n = u64(nblocks) * 256;
    u32 *hist = reinterpret_cast<u32 *>(tmp);
    u32 *offs = hist + hist_n + 1;
    void *stmp = offs + hist_n + 1;
    const u64 *src = in;
    int p = 0;
    for (int shift = 0; shift < key_bits; shift += 8, p++) {
        // pass p writes `out` when the number of passes left (passes - p) is odd
        u64 *dst = ((passes - p) % 2 == 1) ? out : alt;
        k_rs_hist<<<nblocks, RS_THREADS, 0, s>>>(src, n, shift, key_bits, hist, nblocks);
        scan_rec(hist, offs, hist_n, reinterpret_cast<u32 *>(stmp), s);
        k_rs_scatter<<<nblocks, RS_THREADS, 0, s>>>(src, n, shift, key_bits, offs, nblocks, dst);
        g_kernel_launches += 2;
        src = dst;
    }
}

}  // namespace

}  // namespace fpg

extern "C" fp_status fp_sort_entries(const uint64_t *d_in, uint64_t *d_out, uint64_t n, int key_bits, void *stream) {
    using namespace fpg;
    if ((!d_in || !d_out) && n) return FP_BAD_INPUT;
    if (key_bits < 0 || key_bits > 32) return FP_BAD_INPUT;
    if (n > FP_SORT_MAX_ENTRIES) return FP_BAD_INPUT;  // digit counts and offsets are 32-bit
    if (n == 0) return FP_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t tmp_bytes = radix_tmp_bytes(n);
    void *tmp = nullptr, *alt = nullptr;
    if (cudaMallocAsync(&tmp, tmp_bytes, s) != cudaSuccess) return FP_OOM;
    if (cudaMallocAsync(&alt, n * sizeof(u64), s) != cudaSuccess) {
        cudaFreeAsync(tmp, s);
        return FP_OOM;
    }
    sort_into(reinterpret_cast<const u64 *>(d_in), reinterpret_cast<u64 *>(d_out), reinterpret_cast<u64 *>(alt), n,
              key_bits, tmp, s);
    cudaFreeAsync(alt, s);
    cudaFreeAsync(tmp, s);
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_DEVICE_ERROR;
}

// ---- allocation-free variant ----
// Some callers cannot allocate device memory while they run: a serving loop that admits jobs against a
// fixed HBM budget (an allocation mid-job would break its accounting), or a host framework that owns all
// device memory through its own pool and forbids driver allocations. fp_sort_entries_static serves them
// from a fixed scratch array that lives in the library image, sized for at most FP_STATIC_SORT_MAX entries.
namespace fpg {
namespace {

constexpr u64 STATIC_SORT_MAX = u64(1) << 20;
constexpr size_t STATIC_ALT_BYTES = size_t(STATIC_SORT_MAX) * sizeof(u64);
constexpr size_t STATIC_TMP_BYTES = size_t(5) << 18;  // 1.25 MiB: histograms, offsets and scan sums

// Every GPU that loads the library holds this array (about 9.25 MiB) until the process exits. All calls
// share it: calls whose work overlaps on the GPU (different streams, or different host threads) race on it.
static __device__ __align__(256) unsigned char g_static_sort_scratch[STATIC_ALT_BYTES + STATIC_TMP_BYTES];

std::mutex g_static_mu;
void *g_static_addr[64] = {};

// Device address of the scratch array on the current device, looked up once per device (host code only
// sees a stand-in for the symbol; the kernels must be given this address).
cudaError_t static_scratch(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_sort_scratch);
        if (e != cudaSuccess) return e;
        g_static_addr[dev] = p;
    }
    *out = g_static_addr[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace fpg

extern "C" fp_status fp_sort_entries_static(const uint64_t *d_in, uint64_t *d_out, uint64_t n, int key_bits,
                                            void *stream) {
    using namespace fpg;
    if ((!d_in || !d_out) && n) return FP_BAD_INPUT;
    if (key_bits < 0 || key_bits > 32) return FP_BAD_INPUT;
    if (n > STATIC_SORT_MAX) return FP_BAD_INPUT;
    if (radix_tmp_bytes(STATIC_SORT_MAX) > STATIC_TMP_BYTES) return FP_DEVICE_ERROR;
    if (n == 0) return FP_OK;
    void *scratch = nullptr;
    if (static_scratch(&scratch) != cudaSuccess) return FP_DEVICE_ERROR;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    u64 *alt = reinterpret_cast<u64 *>(scratch);
    void *tmp = static_cast<unsigned char *>(scratch) + STATIC_ALT_BYTES;
    // nothing in the scratch needs clearing: every histogram, offset and scan entry a pass reads is
    // written earlier in the same pass
    sort_into(reinterpret_cast<const u64 *>(d_in), reinterpret_cast<u64 *>(d_out), alt, n, key_bits, tmp, s);
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_DEVICE_ERROR;
}
