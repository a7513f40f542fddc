// Precision trace (FP_FLAG_PRECISION_TRACE): for every BAQ read, the FP32 certified pass's pre-floor MAP
// quality t = -4.343 ln(1 - p_max) + 0.499 (device/baq.cu:619-681, computed there as -4.343 ln(other terms /
// total) + 0.499) against the plain FP64 path's, base by base. Per read: the largest |t32 - t64| over the
// bases whose FP64 value lies below 101 (above that every capped quality is 99, the reference's saturation),
// the widest certified half-interval, and every base whose FP64 value falls outside the FP32 interval
// [lo, hi] (a broken certificate; the expected count is zero). Per-read maxima go into log-binned histograms.
#include "kernels.h"

namespace fpg {

namespace {

constexpr int PREC_THREADS = 256;

__device__ __forceinline__ int prec_bin(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 1.0f) return PREC_BINS - 1;
    const float k = floorf((log10f(v) + 10.0f) * 4.0f);
    if (k < 0.0f) return 1;
    const int b = 1 + int(k);
    return b > PREC_BINS - 2 ? PREC_BINS - 2 : b;
}

// one thread per read of the list
__global__ void __launch_bounds__(PREC_THREADS) k_precision(DevBatch b, BatchWork w, const u32 *list,
                                                            const u32 *count, PrecisionAcc *acc) {
    const u32 n = *count;
    for (u32 li = blockIdx.x * blockDim.x + threadIdx.x; li < n; li += gridDim.x * blockDim.x) {
        const u32 r = list[li];
        const u16 *win = w.win + size_t(r) * 8;
        const int qx = win[0], qy = win[1];
        const u32 qual0 = b.qual_start[r] + u32(qx);
        float max_err = 0.0f, max_width = 0.0f;
        u32 bases = 0, viol = 0;
        bool missing = false;
        for (int i = 0; i <= qy - qx; i++) {
            const size_t qi = qual0 + u32(i);
            const float t32 = w.trace32[3 * qi], lo = w.trace32[3 * qi + 1], hi = w.trace32[3 * qi + 2];
            const double t64 = w.trace64[qi];
            if (t32 != t32) {  // the FP32 pass left this read to the FP64 replay without values
                missing = true;
                break;
            }
            if (!(t64 < 101.0)) continue;
            bases++;
            const float err = float(fabs(double(t32) - t64));
            max_err = fmaxf(max_err, err);
            const float half = fmaxf(t32 - lo, hi - t32);
            if (half < 3.0e38f) max_width = fmaxf(max_width, half);
            if (t64 < double(lo) || t64 > double(hi)) viol++;
        }
        if (missing) {
            atomicAdd(&acc->reads_without_fp32, 1ull);
            continue;
        }
        atomicAdd(&acc->reads, 1ull);
        atomicAdd(&acc->bases, (unsigned long long)bases);
        if (viol) atomicAdd(&acc->violations, (unsigned long long)viol);
        atomicAdd(&acc->err_hist[prec_bin(max_err)], 1ull);
        atomicAdd(&acc->width_hist[prec_bin(max_width)], 1ull);
        atomicMax(&acc->max_err_bits, __float_as_uint(max_err));
        atomicMax(&acc->max_width_bits, __float_as_uint(max_width));
    }
}

}  // namespace

void launch_precision(const DevBatch &b, const BatchWork &w, const u32 *list, const u32 *count, u32 max_reads,
                      PrecisionAcc *acc, cudaStream_t s) {
    if (!max_reads) return;
    u32 blocks = (max_reads + PREC_THREADS - 1) / PREC_THREADS;
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_precision<<<blocks, PREC_THREADS, 0, s>>>(b, w, list, count, acc);
    g_kernel_launches++;
}

}  // namespace fpg
