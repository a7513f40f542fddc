/* BAM input for the engine: BGZF inflate and record decoding into fp_batch_view arrays.
 *
 * Replaces the reference's htslib loader path (loader/alignments.cu:136-437, io_thread.cu:97-147) for
 * feeding batches: BGZF blocks are inflated in parallel, records are located by their length prefixes and
 * converted in parallel straight into the engine's SoA layout (4-bit reads packed 8 per word with each read
 * padded to 8 bases, cigar words len | op << 24, raw qualities). Field meanings follow the reference loader:
 * alignment_stop = end position - 1 (htslib bam_endpos semantics), CIGAR op B becomes X, SAM flag bits are
 * kept, a read's read group is its RG:Z tag mapped through the header's @RG lines (PU if present, else ID)
 * to an index in order of first occurrence, -1 when absent or unknown; the contig id is the BAM target
 * index mapped through a caller-supplied table (identity by default), 0xFFFF for unplaced reads.
 */
#ifndef FIREPONY_GB300_BAM_H
#define FIREPONY_GB300_BAM_H

#include <stdint.h>

#include "firepony_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fpb_reader fpb_reader;

/* Opens a BAM file and reads its header. threads: worker threads for inflate and decoding (0: all cores). */
int fpb_open(const char *path, int threads, fpb_reader **out);
void fpb_close(fpb_reader *reader);
const char *fpb_last_error(const fpb_reader *reader);

uint32_t fpb_num_targets(const fpb_reader *reader);
const char *fpb_target_name(const fpb_reader *reader, uint32_t index);
uint32_t fpb_target_length(const fpb_reader *reader, uint32_t index);
/* tid -> engine contig id for the following batches (n entries; targets past n map to 0xFFFF). */
int fpb_set_target_map(fpb_reader *reader, const uint16_t *contig_of_target, uint32_t n);

/* Decodes up to max_reads records into *batch. Returns the number of reads (0 at the end of the file) or a
 * negative value on error. The arrays belong to the reader, which rotates FPB_BUFFER_SETS buffer sets: batch n
 * stays valid until the call that decodes batch n + FPB_BUFFER_SETS starts. A decoder thread may therefore
 * run ahead of the batch being submitted (n) while batch n+1's copy is queued, as long as it starts batch
 * n+3 only after batch n's submit has returned. */
#define FPB_BUFFER_SETS 3

int64_t fpb_next_batch(fpb_reader *reader, uint32_t max_reads, fp_batch_view *batch);

/* Same batches as fpb_next_batch, decoded on the current CUDA device: the compressed BGZF blocks are copied
 * to the device, inflated there (a thread per block, then a warp per block for the back-references and the
 * CRC-32 check), the records located and converted by kernels into device arrays. *batch holds DEVICE
 * pointers for fp_engine_submit_batch_device; the same FPB_BUFFER_SETS rotation applies (batch n stays valid
 * until the call that decodes batch n + FPB_BUFFER_SETS starts, and by then batch n's submit must have
 * returned). Returns once the arrays are complete. A reader uses one of fpb_next_batch and
 * fpb_next_batch_device for all its batches. Replaces the same loader path as fpb_next_batch
 * (loader/alignments.cu:257-437, io_thread.cu:97-147). */
int64_t fpb_next_batch_device(fpb_reader *reader, uint32_t max_reads, fp_batch_view *batch);

/* Counters of a reader since fpb_open (no reference counterpart: the reference's loader keeps no statistics). */
typedef struct fpb_stats {
    uint64_t batches;            /* non-empty batches returned */
    uint64_t records;            /* records returned */
    uint64_t compressed_bytes;   /* BGZF bytes read from the file */
    uint64_t blocks;             /* BGZF blocks inflated (GPU decoding) */
    uint64_t extra_rounds;       /* GPU decoding: rounds that gathered more blocks after a stream held too few records */
    uint64_t serial_walks;       /* GPU decoding: batches whose record starts were found by the one-thread walk */
    double seconds_read;         /* in file reads */
    double seconds_decode;       /* in fpb_next_batch / fpb_next_batch_device outside file reads (GPU decoding:
                                    the host's block parsing and its waits for the device, copies included) */
} fpb_stats;

int fpb_get_stats(const fpb_reader *reader, fpb_stats *out);

/* Read groups seen so far, in id order (the names the report uses). */
uint32_t fpb_num_read_groups(const fpb_reader *reader);
const char *fpb_read_group_name(const fpb_reader *reader, uint32_t id);

/* Writes a BAM file (BGZF, compression level 1..9) from batches in the engine layout: targets (names and
 * lengths), read group IDs (rg index i of a read is written as RG:Z:read_group_ids[i], with a matching @RG
 * header line) and read names "r<number>". For tests and synthetic inputs. */
int fpb_write_bam(const char *path, uint32_t num_targets, const char *const *target_names,
                  const uint32_t *target_lengths, uint32_t num_read_groups, const char *const *read_group_ids,
                  const fp_batch_view *batches, uint32_t num_batches, int level, int threads);

#ifdef __cplusplus
}
#endif

#endif
