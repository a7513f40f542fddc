// Host-side launch interface of the engine's kernels (one function per kernel or kernel group).
#pragma once

#include "common.cuh"

namespace fpg {

// Per-batch device work arrays (owned by the engine, sized per batch).
struct BatchWork {
    // events (expanded CIGAR): one entry per CIGAR op length unit
    u32 *cigar_offsets;      // num_cigar_ops + 1 (exclusive scan of op lengths)
    u32 *ev_rc;              // read coordinate | reference coordinate << 16
    u8 *ev_type;
    u64 num_events;
    // per read
    u8 *status;
    u16 *win;                // 8 x u16: clipped, no-ins, reference, high-quality windows
    i16 *hmm;                // 2 x i16 HMM reference window
    u16 *bw;
    u16 *nerr;
    // per base (quality index space)
    u8 *bflags;
    u8 *tag;                 // BQ tag after recode (0xFF where none)
    u8 *baq_q;               // HMM MAP quality
    u32 *baq_state;          // HMM MAP state
    u8 *baq_amb;             // FP32 HMM: 1 capped quality undecided, 2 state undecided, 4 more than one
                             // other state within the bound (7 alone: no usable row), 8 state undecided but
                             // every candidate's MAP quality MIN_BASE_QUAL, 16 undecided whether the capped
                             // quality at the expected match equals the base's quality
    u16 *baq_alt;            // FP32 HMM, state undecided with one rival: the rival state
    float *frac;             // 3 x float per base (snp, ins, del fractional errors as stored in the table)
    // work lists
    u32 *baq_list;           // reads that need BAQ, by band class
    u32 *counters;           // [0..2] list sizes per band class, [4]/[10] escalated reads of class 0/1,
                             // [5] filtered, [6] BAQ reads, [7] longest BAQ query, [8..9],[11] work counters,
                             // [12..14] widest band per class, [16..21] u64 band cells per class,
                             // [22]/[23] escalations with an undecided MAP state / with undecided qualities only,
                             // [24] work counter of the class-1 replay
    u32 *esc_list;
    // FP32 mode: 1 certifies every capped quality exactly (FP_FLAG_EXACT_BAQ_TAGS), 0 only whether it equals
    // the base's quality (the one property of a BQ tag the covariate tables depend on)
    u32 exact_tags;
    // precision trace (FP_FLAG_PRECISION_TRACE; null otherwise): per base the FP32 kernels' pre-floor MAP
    // quality t and its certified interval [lo, hi] (t = NaN where the FP32 pass has no value), and the
    // plain FP64 path's t
    float *trace32;          // 3 x float per base
    double *trace64;         // 1 x double per base
    // covariate entries
    u32 *entry_count;        // per read + 1
    u32 *entry_offset;       // per read + 1 (exclusive scan)
    u64 *entries;
    u64 *entries_alt;
    u64 entry_capacity;
    // scratch
    void *scan_tmp;
    size_t scan_tmp_bytes;
    u32 *err;
};

// cycle-covariate I/D observation counts of a batch as range updates: per (read group, sign of the cycle)
// a difference array over |cycle| (0..CYC_DIFF_LEN-1); a run of consecutive bases adds +1 at one end and -1
// past the other
constexpr u32 CYC_DIFF_LEN = 520;

struct Tables {
    KeySpace ks;
    unsigned long long *obs;  // per dense key: observations (merged from stage)
    u32 *stage;               // per dense key: observations since the last merge
    float *mism;              // per dense key
    int *cyc_diff;            // n_rg x 2 x CYC_DIFF_LEN, zero between batches
};
void launch_merge_stage(const Tables &t, cudaStream_t s);
void launch_cycle_pairs(const Tables &t, cudaStream_t s);

// HMM constants computed on the host with the platform libm (exactly the reference's host values)
struct HmmConst {
    double qual2prob[256];
    double gap_open;
};

// k_prep.cu
void launch_validate(const DevBatch &b, u32 n_rg, u32 *err, cudaStream_t s);
void launch_op_lengths(const DevBatch &b, u32 *out, cudaStream_t s);
// batch coalescing: adds the staged totals to the start offsets of n appended reads
void launch_rebase_starts(u32 *cigar_start, u32 *read_start, u32 *qual_start, u32 n, u32 d_cigar, u32 d_sym,
                          u32 d_qual, cudaStream_t s);
void launch_prep(const DevBatch &b, const DevRef &ref, const BatchWork &w, cudaStream_t s);
// BAQ lists of band classes 0 and 1 ordered by query length into sorted (2 x R entries); hist: 1024 words
void launch_sort_baq_lists(const BatchWork &w, u32 R, u32 max_class_reads, u32 *hist, u32 *sorted, cudaStream_t s);
void launch_cap(const DevBatch &b, const BatchWork &w, const u32 *list, const u32 *count, int exact,
                cudaStream_t s, u32 max_reads);

// k_baq64.cu
void baq64_set_constants(const HmmConst &c);
void launch_baq64(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                  u32 max_reads, double *scratch, u64 scratch_doubles, u32 max_qlen, u32 max_bw, cudaStream_t s,
                  u32 min_bw = 0,  // reads of the list with a band narrower than min_bw are skipped
                  bool trace_only = false);  // write only w.trace64 (precision trace)
u64 baq64_scratch_doubles(u32 threads, u32 max_qlen, u32 max_bw);
u32 baq64_threads();

// k_baq_seg.cu (band class 0, FP32 certified: thread per read, packed FP32 pairs, checkpointed forward rows)
void baq_seg_set_constants(const HmmConst &c);
u64 baq_seg_scratch_bytes(u32 max_q);
void launch_baq_seg(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                    u32 max_reads, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q, cudaStream_t s);
// k_baq_tpr.cu (thread per read, band in registers; FP32 certified or exact FP64)
void baq_tpr_set_constants(const HmmConst &c);
// k_baq_exact.cu (exact FP64 replay, a group of lanes per read)
void baq_exact_set_constants(const HmmConst &c);
u64 baq_exact_block_scratch_bytes(int band_class, u32 max_q);  // scratch of one block of the class's kernels
// FP32 certified BAQ for bands wider than 15 (bw <= 31; wider ones are skipped), the band across a warp's lanes
void baq_wide_set_constants(const HmmConst &c);
u64 baq_wide_scratch_bytes(u32 reads, u32 max_q);
void launch_baq_wide(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                     u32 max_reads, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q, cudaStream_t s);
// the same for the class-2 reads of bw 32..63: 32 lanes x 4 slots
void launch_baq_wide64(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                       u32 max_reads, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q, cudaStream_t s);
// the same for band class 1 (bw <= 15): 16 lanes x 2 slots, two reads per warp
void launch_baq_wide16(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                       u32 max_reads, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q, cudaStream_t s);
void launch_baq_exact(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                      u32 max_reads, int band_class, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q,
                      bool all_rows, cudaStream_t s);
void launch_baq_tpr(const DevBatch &b, const DevRef &ref, const BatchWork &w, const u32 *list, const u32 *count,
                    u32 max_reads, int band_class, bool exact, u32 *ctr, void *scratch, u64 scratch_bytes, u32 max_q,
                    u32 reads_per_warp, cudaStream_t s);

// k_precision.cu: FP32 vs FP64 MAP quality per BAQ read (precision trace), accumulated over batches
constexpr int PREC_BINS = 42;  // [0] exactly 0, [1 + k] for 10^(-10 + k/4) <= v < 10^(-10 + (k + 1)/4), [41] v >= 1
struct PrecisionAcc {
    unsigned long long reads, reads_without_fp32, bases, violations;
    unsigned long long err_hist[PREC_BINS], width_hist[PREC_BINS];
    unsigned int max_err_bits, max_width_bits;  // non-negative floats, ordered as integers
};
void launch_precision(const DevBatch &b, const BatchWork &w, const u32 *list, const u32 *count, u32 max_reads,
                      PrecisionAcc *acc, cudaStream_t s);

// k_covariates.cu
void launch_cov_count(const DevBatch &b, const BatchWork &w, const Tables &t, cudaStream_t s);
// second count pass over a replay list (reads left deferred by the first pass)
void launch_cov_count_list(const DevBatch &b, const BatchWork &w, const Tables &t, const u32 *list,
                           const u32 *count, u32 max_items, cudaStream_t s);
void launch_cov_emit(const DevBatch &b, const BatchWork &w, const Tables &t, cudaStream_t s);

// k_sort.cu
size_t scan_tmp_bytes(u64 n);
void launch_exclusive_scan(const u32 *in, u32 *out, u64 n, void *tmp, cudaStream_t s);  // out has n+1 entries
void launch_radix_sort(u64 *keys, u64 *alt, u64 n, int key_bits, void *tmp, size_t tmp_bytes, u64 **result,
                       cudaStream_t s);
size_t radix_tmp_bytes(u64 n);
size_t fold_tmp_bytes(u64 n);
void launch_fold(const u64 *sorted, u64 n, float *mism, void *tmp, cudaStream_t s);

// k_post.cu
struct PostTables {
    // compacted observation rows of the three tables, in ascending dense key (== ascending reference key)
    u32 *dense;                  // dense key per row
    u32 num_rows;
};
void launch_mark_nonzero(const Tables &t, u32 *flags, cudaStream_t s);
void launch_gather_rows(const Tables &t, const u32 *flags, const u32 *pos, u32 *rows_dense, cudaStream_t s);
// empirical quality per row (device/empirical_quality.cu:35-198) with host libm constants
struct EmpConst {
    double prior[41];            // log10(gaussian(difference)), difference 0..40
    double log10p[61];           // bin / -10.0
    double log10_one_minus_p[61];
};
void post_set_constants(const EmpConst &c, const double *qual2err);
void launch_rows(const Tables &t, const u32 *rows, u32 n, u32 *key, u64 *obs, double *mism, double *exp_,
                 double *est, cudaStream_t s);
void launch_rg_fold(const Tables &t, u64 *rg_obs, double *rg_mism, double *rg_exp, cudaStream_t s);
void launch_empirical(u32 n, const u64 *obs, const double *mism, const double *est, const double *binom_coef,
                      int need_rounding, double *emp_out, cudaStream_t s);

extern unsigned long long g_kernel_launches;

}  // namespace fpg
