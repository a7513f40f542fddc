/*
 * BQSR oracle — TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement of broadinstitute/firepony's per-batch BQSR path (host/TBB backend semantics) used to
 * check the GPU engine. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may load it.
 * The engine never calls it.
 *
 * Parity status: UNPINNED against the reference itself. The reference ships no tests, fixtures or golden
 * vectors, and its hot path cannot be compiled here (the lift submodule is empty; device/device_types.h and
 * device/primitives/cuda.h are missing). Each stage is pinned instead by hand-derived known-answer tests in
 * tests/test_oracle_kat.py, worked from the cited reference lines.
 */
#ifndef BQSR_ORACLE_H
#define BQSR_ORACLE_H

#include "../include/firepony_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fpo_ctx fpo_ctx;

fpo_ctx *fpo_create(uint32_t num_read_groups);
void fpo_destroy(fpo_ctx *ctx);
int fpo_set_contig(fpo_ctx *ctx, uint32_t contig_id, const uint32_t *packed4, uint64_t num_bases);
int fpo_set_known_sites(fpo_ctx *ctx, uint32_t contig_id, const uint32_t *start, const uint32_t *stop,
                        uint32_t n);
/* num_threads <= 0: use all OpenMP threads. Results do not depend on the thread count. */
int fpo_process_batch(fpo_ctx *ctx, const fp_batch_view *batch, int num_threads);
int fpo_finalize(fpo_ctx *ctx);
int fpo_get_table(fpo_ctx *ctx, int32_t table_id, fp_table_view *out);
/* total_reads, filtered_reads, baq_reads, num_batches */
void fpo_get_stats(const fpo_ctx *ctx, uint64_t out[4]);
/* Same layout as fp_engine_debug_last_batch. */
int fpo_debug_last_batch(fpo_ctx *ctx, uint8_t *read_status, uint16_t *windows, int16_t *hmm,
                         uint8_t *base_flags, uint8_t *baq_tag, double *frac_errors);

/* Per-stage CPU time, in the categories the reference prints at exit (firepony.cu:195-223): thread-seconds
 * summed over the OpenMP threads (the stages of one read run back to back on one thread). */
enum {
    FPO_STAGE_READ_FILTER = 0, FPO_STAGE_CIGAR_EXPANSION, FPO_STAGE_BP_FILTER, FPO_STAGE_SNP_FILTER,
    FPO_STAGE_BAQ_SETUP, FPO_STAGE_BAQ_HMM, FPO_STAGE_BAQ_POST, FPO_STAGE_FRACTIONAL_ERROR,
    FPO_STAGE_COVARIATES_GATHER, FPO_STAGE_COVARIATES_SORT_PACK, FPO_STAGE_POSTPROCESS, FPO_NUM_STAGES
};
void fpo_get_stage_seconds(const fpo_ctx *ctx, double out[FPO_NUM_STAGES]);

/* Known-answer hooks for single functions. */
/* BAQ HMM of one query against one reference window (device/baq.cu:214-697). ref/query are 4-bit symbols
 * one per byte. Outputs one quality and one state per query base. */
void fpo_kat_hmm(const uint8_t *ref, int ref_len, int bases_bm_ref_len, const uint8_t *query,
                 const uint8_t *qual, int query_len, int band_width, uint8_t *out_qual, uint32_t *out_state);
/* Bayesian empirical quality (device/empirical_quality.cu:165-198). */
double fpo_kat_empirical_quality(uint64_t observations, double mismatches, double estimated_quality,
                                 int need_rounding);
/* (int) conversion used for the MAP quality (device/baq.cu:673). */
int fpo_kat_baq_quality_from_max(double max);

#ifdef __cplusplus
}
#endif

#endif
