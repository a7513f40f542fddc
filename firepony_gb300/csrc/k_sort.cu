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
// Stable LSD passes over the key bits [32, 32 + key_bits) of packed 64-bit entries, with digits of at most
// RS_MAX_BITS bits: a key width of b bits takes ceil(b / 10) passes of near-equal digit widths (29 bits: 10, 10,
// 9). Each pass is three kernels:
//   k_rs_count   digit counts per chunk of the input (a chunk is a run of consecutive tiles),
//   k_rs_colscan the chunk counts turned into each chunk's first output position per digit (in place),
//   k_rs_scatter one CTA per chunk walks its tiles in order; per tile it ranks every key among the equal digits
//                before it in tile order, reorders the tile by digit in shared memory and writes each digit's
//                run with consecutive threads on consecutive addresses.
// A chunk's tiles are processed in order by one CTA that carries each digit's next output position from tile
// to tile, so the scan runs over one row of digit counts per chunk (about two per SM) instead of one per tile.
constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ROUNDS = 16;                      // keys per thread and tile
constexpr int RS_WARP_KEYS = 32 * RS_ROUNDS;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;    // 4096 keys
constexpr int RS_MAX_BITS = 10;
constexpr int RS_MAXD = 1 << RS_MAX_BITS;
constexpr int RS_COUNT_SPLIT = 3;                  // counting CTAs per chunk
constexpr int RS_CTAS_PER_SM = 2;                  // scatter CTAs resident per SM (shared memory bound)

// shared memory of k_rs_scatter (88 KB)
struct RsScatterSmem {
    u64 buf[RS_TILE];                  // the tile ordered by digit
    u32 peers[RS_WARPS][RS_MAXD];      // per warp: lanes of the current round holding the digit (zero between rounds)
    u16 cnt[RS_WARPS][RS_MAXD];        // per warp: keys of the digit so far in this tile, then the warp's first slot
    u32 next[RS_MAXD];                 // output position of the chunk's next key of the digit
    u32 off[RS_MAXD];                  // output position of tile slot p (digit d) = off[d] + p
};

__device__ __forceinline__ u32 digit_of(u64 v, int shift, u32 mask) { return u32(v >> (32 + shift)) & mask; }

// Digit counts of one chunk: RS_COUNT_SPLIT CTAs per chunk each count a third of its keys into warp-private
// shared counters and add them to the chunk's row of `hist` (zeroed by the caller).
__global__ void __launch_bounds__(RS_THREADS) k_rs_count(const u64 *in, u64 n, int shift, int bits, u32 tpc,
                                                         u32 *hist) {
    __shared__ u32 h[RS_WARPS][RS_MAXD];
    const int D = 1 << bits;
    const u32 mask = u32(D - 1);
    const int warp = threadIdx.x >> 5;
    for (int j = threadIdx.x; j < RS_WARPS * RS_MAXD; j += RS_THREADS) (&h[0][0])[j] = 0;
    __syncthreads();
    const u32 c = blockIdx.x / RS_COUNT_SPLIT, part = blockIdx.x % RS_COUNT_SPLIT;
    const u64 k0 = u64(c) * tpc * RS_TILE;
    const u64 k1 = k0 + u64(tpc) * RS_TILE < n ? k0 + u64(tpc) * RS_TILE : n;
    const u64 len = k1 - k0;
    u64 a = k0 + len * part / RS_COUNT_SPLIT;
    const u64 b = k0 + len * (part + 1) / RS_COUNT_SPLIT;
    // pairs of entries as 16-byte loads from the first 16-byte boundary; one entry before it and one after the
    // last pair are counted by thread 0
    if ((reinterpret_cast<uintptr_t>(in + a) & 15) && a < b) {
        if (threadIdx.x == 0) atomicAdd(&h[warp][digit_of(in[a], shift, mask)], 1u);
        a++;
    }
    const u64 np = (b - a) / 2;
    const ulonglong2 *in2 = reinterpret_cast<const ulonglong2 *>(in + a);
    constexpr int U = 4;
    u64 i = threadIdx.x;
    for (; i + u64(U - 1) * RS_THREADS < np; i += u64(U) * RS_THREADS) {
        ulonglong2 x[U];
#pragma unroll
        for (int j = 0; j < U; j++) x[j] = in2[i + u64(j) * RS_THREADS];
#pragma unroll
        for (int j = 0; j < U; j++) {
            atomicAdd(&h[warp][digit_of(x[j].x, shift, mask)], 1u);
            atomicAdd(&h[warp][digit_of(x[j].y, shift, mask)], 1u);
        }
    }
    for (; i < np; i += RS_THREADS) {
        const ulonglong2 x = in2[i];
        atomicAdd(&h[warp][digit_of(x.x, shift, mask)], 1u);
        atomicAdd(&h[warp][digit_of(x.y, shift, mask)], 1u);
    }
    if (a + 2 * np < b && threadIdx.x == 0) atomicAdd(&h[warp][digit_of(in[b - 1], shift, mask)], 1u);
    __syncthreads();
    for (int d = threadIdx.x; d < D; d += RS_THREADS) {
        u32 s = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) s += h[w][d];
        if (s) atomicAdd(&hist[u64(c) * D + d], s);
    }
}

// Column scan of the chunk counts, in place: hist[c][d] becomes the number of keys with digit d in chunks before
// c; totals[d] = keys with digit d. A CTA takes 32 digits (a lane each) and its 32 warps split the chunk rows.
__global__ void __launch_bounds__(1024) k_rs_colscan(u32 *hist, u32 G, int D, u32 *totals) {
    __shared__ u32 part[32][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int d = blockIdx.x * 32 + lane;
    const u32 rpw = (G + 31) / 32;
    const u32 r0 = u32(w) * rpw < G ? u32(w) * rpw : G;
    const u32 r1 = r0 + rpw < G ? r0 + rpw : G;
    u32 s = 0;
    if (d < D)
        for (u32 r = r0; r < r1; r++) s += hist[u64(r) * D + d];
    part[w][lane] = s;
    __syncthreads();
    u32 p = 0;
    for (int k = 0; k < w; k++) p += part[k][lane];
    if (d < D) {
        for (u32 r = r0; r < r1; r++) {
            const u32 x = hist[u64(r) * D + d];
            hist[u64(r) * D + d] = p;
            p += x;
        }
        if (w == 31) totals[d] = p;
    }
}

// Loads tile t of the input; in a partial tile the keys past n are left unset (they are never ranked).
__device__ __forceinline__ void rs_load_tile(const u64 *in, u64 n, u64 t, int warp, int lane, u64 (&v)[RS_ROUNDS]) {
    const u64 wbase = t * RS_TILE + u64(warp) * RS_WARP_KEYS + lane;
    if (t * RS_TILE + RS_TILE <= n) {
#pragma unroll
        for (int r = 0; r < RS_ROUNDS; r++) v[r] = in[wbase + u64(r) * 32];
    } else {
#pragma unroll
        for (int r = 0; r < RS_ROUNDS; r++) v[r] = wbase + u64(r) * 32 < n ? in[wbase + u64(r) * 32] : 0;
    }
}

__global__ void __launch_bounds__(RS_THREADS, RS_CTAS_PER_SM)
    k_rs_scatter(const u64 *in, u64 n, int shift, int bits, const u32 *colpre, const u32 *totals, u32 tpc,
                 u64 *out) {
    extern __shared__ __align__(16) unsigned char rs_smem[];
    RsScatterSmem &S = *reinterpret_cast<RsScatterSmem *>(rs_smem);
    const int D = 1 << bits;
    const u32 mask = u32(D - 1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u32 lt = (1u << lane) - 1, lanebit = 1u << lane;
    for (int j = threadIdx.x; j < RS_WARPS * RS_MAXD; j += RS_THREADS) (&S.peers[0][0])[j] = 0;
    {
        // the chunk's first output position per digit: keys of smaller digits + keys of the digit in earlier
        // chunks (thread t takes digits 4t..4t+3)
        u32 t4[4], sum = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int d = 4 * threadIdx.x + k;
            t4[k] = d < D ? totals[d] : 0u;
            sum += t4[k];
        }
        u32 total;
        u32 p = block_exclusive_scan(sum, &total);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int d = 4 * threadIdx.x + k;
            S.next[d] = d < D ? p + colpre[u64(blockIdx.x) * D + d] : 0u;
            p += t4[k];
        }
    }
    const u64 ntiles = (n + RS_TILE - 1) / RS_TILE;
    const u64 t_begin = u64(blockIdx.x) * tpc;
    const u64 t_end = t_begin + tpc < ntiles ? t_begin + tpc : ntiles;
    u64 nxt[RS_ROUNDS];
    rs_load_tile(in, n, t_begin, warp, lane, nxt);
    u32 *peers = S.peers[warp];
    u16 *cnt = S.cnt[warp];
    for (u64 t = t_begin; t < t_end; t++) {
        u64 v[RS_ROUNDS];
#pragma unroll
        for (int r = 0; r < RS_ROUNDS; r++) v[r] = nxt[r];
        if (t + 1 < t_end) rs_load_tile(in, n, t + 1, warp, lane, nxt);  // in flight while this tile is ranked
        const u64 tile0 = t * RS_TILE;
        const u32 tile_n = u32(n - tile0 < u64(RS_TILE) ? n - tile0 : u64(RS_TILE));
        const u32 wkeys = tile_n > u32(warp) * RS_WARP_KEYS ? tile_n - u32(warp) * RS_WARP_KEYS : 0u;
        // clear the counters (the previous tile's output loop no longer reads them)
        for (int j = threadIdx.x; j < RS_WARPS * RS_MAXD / 2; j += RS_THREADS)
            reinterpret_cast<u32 *>(&S.cnt[0][0])[j] = 0;
        __syncthreads();
        // rank: per round, the lanes with equal digits find each other through one shared-memory OR per lane;
        // the lowest of them advances the warp's count for the digit and clears the mask
        u32 rank[RS_ROUNDS / 2];
#pragma unroll
        for (int r = 0; r < RS_ROUNDS; r++) {
            const bool valid = u32(r) * 32 + u32(lane) < wkeys;
            const u32 d = digit_of(v[r], shift, mask);
            if (valid) atomicOr(&peers[d], lanebit);
            __syncwarp();
            u32 pm = 0, before = 0;
            if (valid) {
                pm = peers[d];
                before = cnt[d];
            }
            __syncwarp();
            if (valid && (pm & lt) == 0) {
                cnt[d] = u16(before + u32(__popc(pm)));
                peers[d] = 0;
            }
            __syncwarp();
            const u32 rk = before + u32(__popc(pm & lt));
            if (r & 1) rank[r >> 1] |= rk << 16;
            else rank[r >> 1] = rk;
        }
        __syncthreads();
        {
            // per digit (thread t: digits 4t..4t+3, one 8-byte word of counts per warp): the warps' counts become
            // their first slots within the digit, the tile's digit counts are scanned into the digits' first
            // slots in the tile. Two 16-bit counts per word add without carries (a tile holds 4096 keys).
            const int d0 = 4 * threadIdx.x;
            uint2 c[RS_WARPS];
#pragma unroll
            for (int w = 0; w < RS_WARPS; w++) c[w] = *reinterpret_cast<const uint2 *>(&S.cnt[w][d0]);
            uint2 acc = make_uint2(0, 0);
#pragma unroll
            for (int w = 0; w < RS_WARPS; w++) {
                const uint2 x = c[w];
                c[w] = acc;
                acc.x += x.x;
                acc.y += x.y;
            }
            const u32 tc0 = acc.x & 0xFFFFu, tc1 = acc.x >> 16, tc2 = acc.y & 0xFFFFu, tc3 = acc.y >> 16;
            u32 total;
            const u32 s0 = block_exclusive_scan(tc0 + tc1 + tc2 + tc3, &total);
            const u32 s1 = s0 + tc0, s2 = s1 + tc1, s3 = s2 + tc2;
            const uint2 add = make_uint2(s0 | (s1 << 16), s2 | (s3 << 16));
#pragma unroll
            for (int w = 0; w < RS_WARPS; w++)
                *reinterpret_cast<uint2 *>(&S.cnt[w][d0]) = make_uint2(c[w].x + add.x, c[w].y + add.y);
            const uint4 nx = *reinterpret_cast<const uint4 *>(&S.next[d0]);
            *reinterpret_cast<uint4 *>(&S.off[d0]) = make_uint4(nx.x - s0, nx.y - s1, nx.z - s2, nx.w - s3);
            *reinterpret_cast<uint4 *>(&S.next[d0]) = make_uint4(nx.x + tc0, nx.y + tc1, nx.z + tc2, nx.w + tc3);
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < RS_ROUNDS; r++) {
            if (u32(r) * 32 + u32(lane) < wkeys) {
                const u32 d = digit_of(v[r], shift, mask);
                S.buf[u32(cnt[d]) + ((rank[r >> 1] >> ((r & 1) * 16)) & 0xFFFFu)] = v[r];
            }
        }
        __syncthreads();
        if (tile_n == u32(RS_TILE)) {
            // a whole tile: every load issued before the dependent lookups and stores
            u64 kk[RS_ROUNDS];
            u32 oo[RS_ROUNDS];
#pragma unroll
            for (int j = 0; j < RS_ROUNDS; j++) kk[j] = S.buf[threadIdx.x + j * RS_THREADS];
#pragma unroll
            for (int j = 0; j < RS_ROUNDS; j++) oo[j] = S.off[digit_of(kk[j], shift, mask)];
#pragma unroll
            for (int j = 0; j < RS_ROUNDS; j++) out[u32(oo[j] + threadIdx.x + j * RS_THREADS)] = kk[j];
        } else {
            for (u32 p = threadIdx.x; p < tile_n; p += RS_THREADS) {
                const u64 key = S.buf[p];
                out[u32(S.off[digit_of(key, shift, mask)] + p)] = key;
            }
        }
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


// Sort geometry for n entries on the current device: tiles of RS_TILE keys, chunks of `tpc` consecutive tiles,
// one scatter CTA per chunk (at most RS_CTAS_PER_SM per SM, so every chunk's CTA is resident at once).
struct RsPlan {
    u64 ntiles;
    u32 tpc, chunks;
};

int device_sm_count() {
    static int cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!cached[dev]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        cached[dev] = v;
    }
    return cached[dev];
}

RsPlan rs_plan(u64 n) {
    RsPlan p;
    p.ntiles = (n + RS_TILE - 1) / RS_TILE;
    const u64 max_chunks = u64(device_sm_count()) * RS_CTAS_PER_SM;
    const u64 g0 = p.ntiles < max_chunks ? p.ntiles : max_chunks;
    p.tpc = u32((p.ntiles + g0 - 1) / (g0 ? g0 : 1));
    p.chunks = p.tpc ? u32((p.ntiles + p.tpc - 1) / p.tpc) : 0u;
    return p;
}

// Digit widths of the passes for a key width: ceil(bits / RS_MAX_BITS) passes, widths differing by at most one.
int rs_passes(int key_bits, int *width) {
    if (key_bits <= 0) return 0;
    const int passes = (key_bits + RS_MAX_BITS - 1) / RS_MAX_BITS;
    for (int p = 0; p < passes; p++) width[p] = key_bits / passes + (p < key_bits % passes ? 1 : 0);
    return passes;
}

void rs_pass(const u64 *src, u64 *dst, u64 n, int shift, int bits, const RsPlan &plan, void *tmp, cudaStream_t s) {
    static bool attr_set[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr_set[dev]) {
        cudaFuncSetAttribute(k_rs_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(RsScatterSmem)));
        attr_set[dev] = true;
    }
    const int D = 1 << bits;
    u32 *hist = reinterpret_cast<u32 *>(tmp);
    u32 *totals = hist + u64(plan.chunks) * RS_MAXD;
    cudaMemsetAsync(hist, 0, u64(plan.chunks) * D * sizeof(u32), s);
    k_rs_count<<<plan.chunks * RS_COUNT_SPLIT, RS_THREADS, 0, s>>>(src, n, shift, bits, plan.tpc, hist);
    k_rs_colscan<<<(D + 31) / 32, 1024, 0, s>>>(hist, plan.chunks, D, totals);
    k_rs_scatter<<<plan.chunks, RS_THREADS, sizeof(RsScatterSmem), s>>>(src, n, shift, bits, hist, totals, plan.tpc,
                                                                        dst);
    g_kernel_launches += 3;
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
    // one row of digit counts per chunk, then the digit totals
    const RsPlan plan = rs_plan(n);
    return size_t(u64(plan.chunks) * RS_MAXD + RS_MAXD) * sizeof(u32) + 256;
}

size_t fold_tmp_bytes(u64 n) { return size_t(3 * (n + 1)) * sizeof(u32) + scan_tmp_bytes(n) + 256; }

void launch_radix_sort(u64 *keys, u64 *alt, u64 n, int key_bits, void *tmp, size_t tmp_bytes, u64 **result,
                       cudaStream_t s) {
    (void)tmp_bytes;
    u64 *src = keys, *dst = alt;
    int width[4];
    const int passes = n > 1 ? rs_passes(key_bits, width) : 0;
    const RsPlan plan = rs_plan(n);
    for (int p = 0, shift = 0; p < passes; shift += width[p], p++) {
        rs_pass(src, dst, n, shift, width[p], plan, tmp, s);
        u64 *t = src;
        src = dst;
        dst = t;
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
    int width[4];
    const int passes = rs_passes(key_bits, width);
    if (n <= 1 || passes == 0) {
        if (n) cudaMemcpyAsync(out, in, n * sizeof(u64), cudaMemcpyDeviceToDevice, s);
        return;
    }
    const RsPlan plan = rs_plan(n);
    const u64 *src = in;
    for (int p = 0, shift = 0; p < passes; shift += width[p], p++) {
        // pass p writes `out` when the number of passes left (passes - p) is odd
        u64 *dst = ((passes - p) % 2 == 1) ? out : alt;
        rs_pass(src, dst, n, shift, width[p], plan, tmp, s);
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
