// K5 post-processing (device/pipeline.cu:206-216): compaction of the dense observation tables into the
// reduced tables, expected errors (device/expected_error.h:37-76), the read-group table
// (device/read_group_table.cu:47-94) and the Bayesian empirical quality (device/empirical_quality.cu:35-198).
// Compiled with -fmad=false: every double is produced by the same IEEE operations in the same order as the
// reference's host code. Values that come from libm (the prior and log10(1 - 10^p) tables, the per-row
// log10 binomial coefficient from lgammaf, and the read-group table's estimated quality, whose exact bits
// steer int() truncation) are computed on the host with the platform libm and passed in.
#include "kernels.h"

namespace fpg {

__constant__ double cp_prior[41];
__constant__ double cp_log10p[61];
__constant__ double cp_l1mp[61];
__constant__ double cp_qual2err[256];

namespace {

__global__ void k_mark_nonzero(const unsigned long long *obs, u32 n, u32 *flags) {
    const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = obs[i] != 0 ? 1u : 0u;
}

__global__ void k_gather_rows(const u32 *flags, const u32 *pos, u32 n, u32 *rows) {
    const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flags[i]) rows[pos[i]] = i;
}

// reference key and quality of a dense index
__device__ __host__ inline void dense_to_key(const KeySpace &ks, u32 d, u32 &key, u32 &q) {
    if (d < ks.cycle_base) {
        const u32 x = d - ks.qual_base, ev = slot_ev(x % EV_SLOTS), rq = x / EV_SLOTS, rg = rq / Q_SPAN;
        q = rq % Q_SPAN;
        key = (rg << 10) | (q << 2) | ev;
    } else if (d < ks.context_base) {
        const u32 x = d - ks.cycle_base, ev = slot_ev(x % EV_SLOTS), y = x / EV_SLOTS, cyc = y % CYCLE_SPAN;
        const u32 rq = y / CYCLE_SPAN;
        const u32 rg = rq / Q_SPAN;
        q = rq % Q_SPAN;
        key = (rg << 20) | (q << 12) | (cyc << 2) | ev;
    } else {
        const u32 x = d - ks.context_base, ev = slot_ev(x % EV_SLOTS), y = x / EV_SLOTS, cr = y % CONTEXT_SPAN;
        const u32 rq = y / CONTEXT_SPAN;
        const u32 rg = rq / Q_SPAN;
        q = rq % Q_SPAN;
        key = (rg << 21) | (q << 13) | (context_value(cr) << 2) | ev;
    }
}

// per compacted row: reference key, observations, mismatches (float widened), expected errors and
// estimated quality (need_rounding tables: the estimate only enters through round(), so CUDA's log10 is
// used here; its last-ulp difference from libm cannot move round(bin - est) off an integer step)
__global__ void k_rows(KeySpace ks, const u32 *rows, u32 n, const unsigned long long *obs, const float *mism,
                       u32 *key_out, u64 *obs_out, double *mism_out, double *exp_out, double *est_out) {
    const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const u32 d = rows[i];
    u32 key, q;
    dense_to_key(ks, d, key, q);
    const u64 o = obs[d];
    const double e = double(o) * cp_qual2err[q];
    key_out[i] = key;
    obs_out[i] = o;
    mism_out[i] = double(mism[d]);
    exp_out[i] = e;
    est_out[i] = double(-10.0 * log10(e / double(o)));
}

// RecalTable0: quality rows with Q masked, folded in ascending Q per (read group, event) in FP64
__global__ void k_rg_fold(KeySpace ks, const unsigned long long *obs, const float *mism, u64 *rg_obs,
                          double *rg_mism, double *rg_exp) {
    const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ks.n_rg * 3) return;
    const u32 rg = i / 3, ev = i % 3;
    u64 o = 0;
    double m = 0.0, e = 0.0;
    bool first = true;
    for (u32 q = 0; q < Q_SPAN; q++) {
        const u32 d = ks.qual_base + (rg * Q_SPAN + q) * EV_SLOTS + ev_slot(ev);
        const u64 oq = obs[d];
        if (!oq) continue;
        const double mq = double(mism[d]);
        const double eq = double(oq) * cp_qual2err[q];
        if (first) {
            o = oq; m = mq; e = eq; first = false;
        } else {
            o += oq; m = m + mq; e = e + eq;
        }
    }
    rg_obs[i] = o;
    rg_mism[i] = m;
    rg_exp[i] = e;
}

__global__ void k_empirical(u32 n, const u64 *obs, const double *mism, const double *est, const double *coef,
                            int need_rounding, double *emp) {
    const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // calcEmpiricalQuality (:165-174)
    const u64 k0 = u64(mism[i] + 0.5) + 1;
    const u64 n0 = obs[i] + 1 + 1;
    u64 nObs = n0, nErr = k0;
    // log10QempLikelihood cap (:103-108)
    const u32 MAXOBS = 2147483647u - 1;
    if (nObs > MAXOBS) {
        const double fraction = double(MAXOBS) / double(nObs);
        nErr = u64(round(double(nErr) * fraction));
        nObs = MAXOBS;
    }
    const double C = coef[i];
    const double Qrep = est[i];
    double best = 0.0;
    int best_bin = 0;
    for (int bin = 0; bin <= 60; bin++) {
        const double Qemp = bin / 1.0;
        double delta = Qemp - Qrep;
        if (need_rounding) delta = round(delta);
        int diff = abs(int(delta));
        diff = diff < 40 ? diff : 40;
        const double lik = C + cp_log10p[bin] * double(nErr) + cp_l1mp[bin] * double(nObs - nErr);
        const double post = cp_prior[diff] + lik;
        if (bin == 0 || post > best) {
            best = post;
            best_bin = bin;
        }
    }
    const double q = best_bin / 1.0;
    emp[i] = q < 93.0 ? q : 93.0;
}

}  // namespace

void post_set_constants(const EmpConst &c, const double *qual2err) {
    cudaMemcpyToSymbol(cp_prior, c.prior, sizeof(c.prior));
    cudaMemcpyToSymbol(cp_log10p, c.log10p, sizeof(c.log10p));
    cudaMemcpyToSymbol(cp_l1mp, c.log10_one_minus_p, sizeof(c.log10_one_minus_p));
    cudaMemcpyToSymbol(cp_qual2err, qual2err, 256 * sizeof(double));
}

void launch_mark_nonzero(const Tables &t, u32 *flags, cudaStream_t s) {
    const u32 n = t.ks.total;
    k_mark_nonzero<<<(n + 255) / 256, 256, 0, s>>>(t.obs, n, flags);
    g_kernel_launches++;
}

void launch_gather_rows(const Tables &t, const u32 *flags, const u32 *pos, u32 *rows, cudaStream_t s) {
    const u32 n = t.ks.total;
    k_gather_rows<<<(n + 255) / 256, 256, 0, s>>>(flags, pos, n, rows);
    g_kernel_launches++;
}

void launch_rows(const Tables &t, const u32 *rows, u32 n, u32 *key, u64 *obs, double *mism, double *exp_,
                 double *est, cudaStream_t s) {
    if (!n) return;
    k_rows<<<(n + 255) / 256, 256, 0, s>>>(t.ks, rows, n, t.obs, t.mism, key, obs, mism, exp_, est);
    g_kernel_launches++;
}

void launch_rg_fold(const Tables &t, u64 *rg_obs, double *rg_mism, double *rg_exp, cudaStream_t s) {
    const u32 n = t.ks.n_rg * 3;
    k_rg_fold<<<(n + 127) / 128, 128, 0, s>>>(t.ks, t.obs, t.mism, rg_obs, rg_mism, rg_exp);
    g_kernel_launches++;
}

void launch_empirical(u32 n, const u64 *obs, const double *mism, const double *est, const double *coef,
                      int need_rounding, double *emp, cudaStream_t s) {
    if (!n) return;
    k_empirical<<<(n + 127) / 128, 128, 0, s>>>(n, obs, mism, est, coef, need_rounding, emp);
    g_kernel_launches++;
}

}  // namespace fpg
