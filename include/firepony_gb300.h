/*
 * firepony_gb300 — C ABI of the GB300 (sm_103a) BQSR engine.
 *
 * This header is the drop-in boundary between Firepony's host code (driver, io_thread, loaders) and the
 * GPU hot path. It replaces the per-device pipeline seam `firepony_pipeline` (device/pipeline.h:43-66)
 * and the batch entry `firepony_process_batch` / `firepony_postprocess` (device/pipeline.cu:56-147,
 * :206-228). Plain pointers and sizes only: no C++ or torch types cross this boundary.
 *
 * Input layouts are exactly the reference's host layouts so a caller can pass its buffers unchanged:
 *   - reads:      4-bit IUPAC symbols (=ACMGRSVTWYHKDBN -> 0..15), 8 per uint32 word, symbol j of the
 *                 batch at bits 4*(j%8) of word j/8 (packed_vector<4>, little-endian packing,
 *                 device/primitives/packed_vector.h:43); read_start[r] is a symbol index, each read padded
 *                 to a multiple of 8 symbols (loader/alignments.cu:357-385).
 *   - cigars:     one uint32 per op, bits 0..23 = length, bits 24..27 = op (cigar_op bitfield, types.h:57-86;
 *                 op codes M=0 I=1 D=2 N=3 S=4 H=5 P=6 '='=7 X=8).
 *   - qualities:  one uint8 Phred value per base (no +33 offset), qual_start[r] indexes it.
 *   - contigs:    4-bit symbols packed the same way as reads (sequence_storage, sequence_database.h:37-51);
 *                 only A,C,G,T,N (1,2,4,8,15) occur after FASTA loading (loader/reference.cu:278-316).
 *   - known sites: per contig, 0-based feature start and inclusive stop, sorted by start
 *                 (loader/variants.cu:118-123). The engine builds the prefix-max index itself
 *                 (loader/variants.cu:126-134).
 *
 * Error behaviour: every call returns an fp_status; nothing exits the process. fp_last_error() returns
 * a message for the last failing call on a handle. A handle is single-threaded (one caller thread at a
 * time), like the reference's per-device pipeline thread (device/pipeline_interface.cu:179-225).
 */
#ifndef FIREPONY_GB300_H
#define FIREPONY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FP_OK = 0,
    FP_BAD_INPUT = 1,      /* malformed arguments or batch (sizes, ranges, unsupported read length) */
    FP_OOM = 2,            /* device or pinned host allocation failed */
    FP_DEVICE_ERROR = 3,   /* CUDA error, or a kernel reported an internal error status */
    FP_TIMEOUT = 4,        /* a bounded device wait ran out */
    FP_NOT_READY = 5,      /* call out of order (e.g. submit after finalize) */
} fp_status;

/* BAQ arithmetic. FP_BAQ_FP64 is the plain path: the HMM of device/baq.cu:214-697 replayed in IEEE double
 * with the reference's operation order. FP_BAQ_FP32 runs the HMM in FP32 with per-row scaling and a
 * certified error bound, and recomputes in FP64 every read whose result the bound cannot decide.
 * Both produce identical tables. */
typedef enum {
    FP_BAQ_FP32 = 0,
    FP_BAQ_FP64 = 1,
} fp_baq_mode;

typedef struct {
    int32_t device;              /* CUDA device ordinal */
    int32_t baq_mode;            /* fp_baq_mode */
    uint32_t num_read_groups;    /* read groups known from the header (<= 256, the 8-bit key field) */
    uint32_t max_batch_reads;    /* capacity hints; 0 = defaults. Larger batches return FP_BAD_INPUT */
    uint64_t max_batch_bases;
    uint64_t max_batch_cigar_ops;
    uint32_t replay_reads_per_warp;  /* FP32 mode: reads per warp of the FP64 replay kernels, 1..32
                                        (0 = default). Fewer reads per warp spread a small replay set over
                                        more of the GPU's FP64 units */
    uint32_t flags;              /* FP_FLAG_* bits (0 for normal operation) */
    uint32_t coalesce_reads;     /* 0: every fp_engine_submit_batch is processed as its own device batch.
                                    N > 0: host batches smaller than N reads are validated on the host, copied
                                    into a device staging batch (offsets rebased) and processed together once
                                    N reads are staged; finalize and fp_engine_submit_batch_device process the
                                    staged reads first. Stream order is kept, so the tables are the same.
                                    No reference counterpart (the reference runs each io_thread batch alone). */
    uint32_t reserved;
} fp_options;

/* Test hook: in FP32 mode, run every BAQ read of band width <= 15 through the exact FP64 replay as well
 * (the replay's results replace the FP32 ones), so the replay kernels see the whole workload. */
#define FP_FLAG_REPLAY_ALL 1u
/* Measurement: in FP32 mode, also run every BAQ read through the plain FP64 HMM (results unchanged) and
 * compare the two pre-floor MAP qualities per base; see fp_engine_get_precision_stats. Costs one plain
 * FP64 BAQ pass per batch. No reference counterpart (the reference has only the FP64 HMM). */
#define FP_FLAG_PRECISION_TRACE 2u
/* Check: in FP32 mode, certify every base's capped BAQ quality exactly (BQ tags identical to the FP64
 * path's), not only whether it equals the base's quality. The reference consumes the BQ tags only through
 * that test (fractional_errors.cu:93, tag == NO_BAQ_UNCERTAINTY), so the tables are the same either way;
 * this flag makes the engine's BQ tags (fp_engine_debug_last_batch) match the FP64 path's as well, at the
 * cost of more FP64 replays. */
#define FP_FLAG_EXACT_BAQ_TAGS 4u

/* One alignment batch, mirroring alignment_batch_storage<host> (alignment_data.h:125-173). The engine
 * borrows these host buffers only for the duration of fp_engine_submit_batch. */
typedef struct {
    uint32_t num_reads;
    uint32_t num_cigar_ops;      /* length of cigars[] */
    uint64_t num_read_symbols;   /* length of reads[] in symbols (a multiple of 8) */
    uint64_t num_qualities;      /* length of qualities[] */

    const uint16_t *chromosome;          /* contig id per read */
    const uint32_t *alignment_start;     /* 0-based */
    const uint32_t *alignment_stop;      /* inclusive */
    const uint32_t *mate_alignment_start;
    const int32_t  *inferred_insert_size;
    const uint32_t *cigars;
    const uint32_t *cigar_start;
    const uint32_t *cigar_len;
    const uint32_t *reads;
    const uint32_t *read_start;
    const uint32_t *read_len;
    const uint8_t  *qualities;
    const uint32_t *qual_start;
    const uint32_t *qual_len;
    const uint16_t *flags;               /* AlignmentFlags bits (alignment_data.h:46-72) */
    const uint8_t  *mapq;
    const uint32_t *read_group;          /* uint32(-1) = no read group */
} fp_batch_view;

/* One finalized covariate table (keys in the reference's 32-bit packed format, ascending). */
typedef struct {
    uint32_t num_rows;
    const uint32_t *keys;
    const uint64_t *observations;
    const double *mismatches;            /* float sums widened to double (RecalTable0: double sums) */
    const double *expected_errors;
    const double *estimated_quality;
    const double *empirical_quality;
} fp_table_view;

typedef enum {
    FP_TABLE_READ_GROUP = 0,     /* RecalTable0 */
    FP_TABLE_QUALITY = 1,        /* RecalTable1 */
    FP_TABLE_CYCLE = 2,          /* RecalTable2, cycle rows */
    FP_TABLE_CONTEXT = 3,        /* RecalTable2, context rows */
} fp_table_id;

typedef struct {
    uint64_t total_reads;
    uint64_t filtered_reads;
    uint64_t baq_reads;
    uint64_t num_batches;
    uint64_t baq_fp64_escalated_reads;   /* FP32 mode: reads recomputed in FP64 */
    uint64_t gpu_kernel_launches;        /* kernels launched by this engine since creation */
    double   gpu_ms_per_stage[8];        /* device time per stage (see fp_stage) */
    uint64_t baq_reads_by_band[3];       /* BAQ reads by band class: bw <= 7, bw <= 15, wider */
    uint64_t baq_escalated_by_band[2];   /* FP32 mode: FP64 replays of band class 0 (bw <= 7) and of the
                                            wider classes (bw 8..15 and 16..31) */
    uint64_t baq_escalated_by_cause[2];  /* FP32 mode: replays with an undecided MAP state, with undecided
                                            qualities only */
    uint64_t baq_band_cells[3];          /* HMM band cells (row x in-band reference positions) per class */
    uint64_t baq_main_launches;          /* launches of the dominant BAQ kernel (band class 0, FP32 or FP64) */
    double   baq_main_ms;                /* their device time */
    double   baq_path_ms[4];             /* FP32 mode, device time from the BAQ stage start to the end of: the
                                            class-0 FP32 kernel + capping, the class-0 replay, the class-1
                                            FP32 kernel + capping, the class-1 replay */
    uint64_t baq_escalated_undecided_rows; /* FP32 mode: of the replays with an undecided MAP state, those
                                            holding rows the FP32 pass could not bound at all (the band-class-0
                                            underflow guard, a row without a usable sum, a quality above 93) */
} fp_stats;

/* FP32 vs FP64 per BAQ read (FP_FLAG_PRECISION_TRACE), accumulated since creation or reset. t is the MAP
 * quality before flooring, -4.343 ln(1 - p_max) + 0.499 (device/baq.cu:673); bases whose FP64 t is 101 or more
 * (capped to 99 either way) are left out. Histograms are over reads of the per-read maximum: bin 0 holds
 * exactly 0, bin 1 + k holds 10^(-10 + k/4) <= v < 10^(-10 + (k+1)/4) (k = 0..39, values below 1e-10 in
 * bin 1), bin 41 holds v >= 1. */
typedef struct {
    uint64_t reads;               /* BAQ reads compared */
    uint64_t reads_without_fp32;  /* reads the FP32 pass handed to the FP64 replay without values (underflow
                                     guard, qualities above 93) */
    uint64_t bases;               /* bases compared */
    uint64_t bound_violations;    /* bases whose FP64 t lies outside the FP32 certified interval (expected 0) */
    double max_abs_error;         /* largest |t32 - t64| */
    double max_half_width;        /* widest finite certified half-interval */
    uint64_t err_hist[42];        /* per read: max |t32 - t64| */
    uint64_t width_hist[42];      /* per read: max certified half-interval */
} fp_precision_stats;

typedef enum {
    FP_STAGE_PREP = 0, FP_STAGE_BAQ = 1, FP_STAGE_COVARIATES = 2, FP_STAGE_SORT_REDUCE = 3,
    FP_STAGE_POSTPROCESS = 4, FP_STAGE_H2D = 5, FP_STAGE_D2H = 6, FP_STAGE_OTHER = 7,
} fp_stage;

typedef struct fp_engine fp_engine;

/* Creates an engine on options->device. Replaces firepony_pipeline::create + setup
 * (device/pipeline_interface.cu:246-265, :105-125). */
fp_status fp_engine_create(const fp_options *options, fp_engine **out);
void fp_engine_destroy(fp_engine *engine);
const char *fp_last_error(const fp_engine *engine);

/* Makes a contig resident on the device (sequence_database_storage::update_resident_set,
 * segmented_database.h:224-244). packed4 holds num_bases 4-bit symbols. */
fp_status fp_engine_set_contig(fp_engine *engine, uint32_t contig_id, const uint32_t *packed4, uint64_t num_bases);

/* Makes a contig's known sites resident (variant_database_storage, variant_database.h:42-67). */
fp_status fp_engine_set_known_sites(fp_engine *engine, uint32_t contig_id, const uint32_t *feature_start,
                                    const uint32_t *feature_stop, uint32_t num_sites);

/* Runs the per-batch hot path on one batch and folds it into the resident covariate tables.
 * Replaces batch->download + firepony_process_batch (device/pipeline_interface.cu:206-220,
 * device/pipeline.cu:56-147). Returns once the host buffers may be reused. With coalesce_reads set, a small
 * batch is checked and staged here (FP_BAD_INPUT for a malformed batch, nothing staged), and the staged
 * reads are processed by the submit that brings them to coalesce_reads (a device error then concerns all of
 * them). */
fp_status fp_engine_submit_batch(fp_engine *engine, const fp_batch_view *batch);

/* Queues the host-to-device copy of a batch on the engine's copy stream and returns at once (no reference
 * counterpart: the reference downloads a batch synchronously, device/pipeline_interface.cu:206-220). A
 * following fp_engine_submit_batch with the same view (same pointers and counts) uses the copy instead of
 * copying again, so the copy of batch n+1 overlaps the processing of batch n:
 *     prefetch(b0); for each i: prefetch(b[i+1]); submit(b[i]);
 * The host buffers must stay unchanged until that submit returns; page-locked buffers (fp_host_alloc) make
 * the copy asynchronous. Two batches can be prefetched ahead of their submits. */
fp_status fp_engine_prefetch_batch(fp_engine *engine, const fp_batch_view *batch);

/* Same as fp_engine_submit_batch for a batch whose arrays are already in device memory (device pointers,
 * same layout). For data kept resident on the GPU (serving, benchmarking the kernels alone). */
fp_status fp_engine_submit_batch_device(fp_engine *engine, const fp_batch_view *device_batch);

/* The CUDA stream (cudaStream_t) every kernel of this engine runs on, for event timing by the caller. */
void *fp_engine_cuda_stream(fp_engine *engine);

/* Sorts/reduces the resident tables, builds the read-group table and computes empirical qualities.
 * Replaces firepony_postprocess's compute part (device/pipeline.cu:206-216). The table views stay valid
 * until the engine is destroyed or reset. */
fp_status fp_engine_finalize(fp_engine *engine);
fp_status fp_engine_get_table(fp_engine *engine, int32_t table_id, fp_table_view *out);

/* Writes the GATKReport v1.1 recalibration report (device/pipeline.cu:150-204, output_read_group_table
 * device/read_group_table.cu:122-143, output_covariates device/covariates.cu:285-311).
 * rg_names[i] is the name of read group i (PU, else ID: loader/alignments.cu:179-187).
 * software_version is printed in the Arguments table (Firepony extension, device/pipeline.cu:176-177). */
fp_status fp_engine_write_report(fp_engine *engine, const char *path, const char *const *rg_names,
                                 uint32_t num_rg_names, int disable_rounding, int version_major,
                                 int version_minor, int version_rev);

/* Clears the tables and statistics; contigs and known sites stay resident. */
fp_status fp_engine_reset(fp_engine *engine);

fp_status fp_engine_get_stats(const fp_engine *engine, fp_stats *out);

/* The precision trace's accumulated comparison (all zero unless FP_FLAG_PRECISION_TRACE is set). Waits for
 * the engine's stream. */
fp_status fp_engine_get_precision_stats(fp_engine *engine, fp_precision_stats *out);

/* Test/debug: copies the per-read and per-base intermediates of the most recent batch to the host.
 * Each pointer may be NULL. Per-read arrays have num_reads entries, per-base arrays num_qualities.
 *   read_status:  0 filtered, 1 active, 2 removed (BAQ window off the contig end)
 *   windows:      per read 8 x uint16: clipped (x,y), clipped no-insertions (x,y),
 *                 reference clipped (x,y), high-quality (x,y)
 *   hmm:          per read 4 x int16: hmm window (x,y), bandwidth, num_errors
 *   base_flags:   bit0 snp, bit1 insertion, bit2 deletion, bit3 active location
 *   baq_tag:      BQ tag per base (0xFF where none), as in baq.qualities after recode (device/baq.cu:1058)
 *   frac_errors:  3 doubles per base (snp, insertion, deletion) */
fp_status fp_engine_debug_last_batch(fp_engine *engine, uint8_t *read_status, uint16_t *windows,
                                     int16_t *hmm, uint8_t *base_flags, uint8_t *baq_tag,
                                     double *frac_errors);

/* Stable LSD radix sort of n packed 64-bit covariate entries (key in bits 32..63, payload below) by key
 * bits [32, 32 + key_bits), device pointers in and out (d_in is not modified; the ranges must not
 * overlap). Key bits at and above key_bits do not take part: entries that differ only there keep their
 * input order. The engine's K4 sort, exposed for callers that build their own entry streams, in the role of
 * covariate_table::sort (device/covariate_table.cu:43-57). Runs on `stream` (a cudaStream_t, NULL for the
 * default stream) and returns once the work is queued; scratch is allocated and freed on that stream.
 * n may be at most FP_SORT_MAX_ENTRIES (digit counts and offsets are 32-bit); larger n returns
 * FP_BAD_INPUT. */
#define FP_SORT_MAX_ENTRIES 0xFFFFFFFEull
fp_status fp_sort_entries(const uint64_t *d_in, uint64_t *d_out, uint64_t n, int key_bits, void *stream);

/* fp_sort_entries without any device allocation, for callers that must not allocate while they run (a
 * serving loop admitting jobs against a fixed HBM budget, or a host framework whose own pool owns all device
 * memory). No counterpart in the reference. Scratch is a fixed array inside the library (about 9.25 MiB per
 * GPU, held until the process exits); n may be at most FP_STATIC_SORT_MAX, larger n returns FP_BAD_INPUT.
 * The first call on a device looks up that device's scratch address: make it before any stream capture.
 * All calls share the scratch, so calls whose work overlaps on the GPU race; serialise them. */
#define FP_STATIC_SORT_MAX (1u << 20)
fp_status fp_sort_entries_static(const uint64_t *d_in, uint64_t *d_out, uint64_t n, int key_bits, void *stream);

/* Writes a GATKReport from four table views (indexed by fp_table_id); the same writer as
 * fp_engine_write_report, usable on any tables in this layout. */
fp_status fp_report_write(const char *path, const fp_table_view *tables, const char *const *rg_names,
                          uint32_t num_rg_names, int disable_rounding, int version_major, int version_minor,
                          int version_rev);

/* Measures the device's FP32 SIMT multiply-add throughput in TFLOP/s (2 flops per multiply-add): one resident
 * grid of independent fmaf chains (packed = 0) or of packed two-lane __ffma2_rn chains (packed = 1), best of
 * three timed launches. The roofline denominator of the FP32 BAQ HMM. No reference counterpart. */
fp_status fp_measure_fp32_peak(int device, int packed, double *tflops);

/* Page-locked host memory for batch buffers (so the H2D copies run at full link speed). Replaces nothing in
 * the reference: its io_thread buffers are pageable (io_thread.cu:44-54). */
fp_status fp_host_alloc(size_t bytes, void **out);
void fp_host_free(void *ptr);

#ifdef __cplusplus
}
#endif

#endif /* FIREPONY_GB300_H */
