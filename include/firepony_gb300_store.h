/* firepony-gb300 reference store: the contigs and known sites an engine reads, kept as one contiguous image.
 *
 * The image can be
 *   - published as a POSIX shared-memory segment, so later processes map it instead of parsing FASTA and VCF
 *     files again (the preloader);
 *   - uploaded once to a GPU and attached to any number of engines on that GPU, so concurrent jobs share one
 *     device copy of the reference (resident serving).
 *
 * Reference interfaces replaced:
 *   firepony-loader.cu:33-93        loads the FASTA and VCF files and serialises both databases into shared
 *                                   memory segments named after the files;
 *   mmap.cu:57-89                   compute_shmem_path ("/firepony_" + absolute path with '/' -> '_');
 *   mmap.cu:98-190                  shared_memory_file::open (read-only mapping) / create (read-write);
 *   loader/reference.cu:133-143,
 *   loader/variants.cu:48-58        the loaders' try-mmap paths (unserialise from the segment);
 *   segmented_database.h:224-244    per-contig device residency of the databases.
 *
 * Differences from the reference: the image is the device layout itself (4-bit packed contig words with
 * the unused symbols of the last word zeroed, then per contig the known sites' start, stop and prefix-max
 * stop arrays), so attaching a store is one host-to-device copy and no parsing. A segment is published
 * under a fresh name object: an existing one is unlinked first, so processes that still map the previous
 * segment keep a valid mapping. A segment becomes visible to fp_refstore_open only once it is complete.
 *
 * Every call returns fp_status; fp_refstore_last_error gives the message of the store's last failure.
 * A store is not thread-safe for modification; its device copy is read-only and may be read by several
 * engines (each driven by its own thread) at once.
 */
#ifndef FIREPONY_GB300_STORE_H
#define FIREPONY_GB300_STORE_H

#include <stddef.h>
#include <stdint.h>

#include "firepony_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fp_refstore fp_refstore;

typedef struct fp_refstore_info {
    uint32_t num_contigs;
    uint32_t attached_engines; /* engines reading the device copy */
    uint64_t total_bases;
    uint64_t total_sites;
    uint64_t image_bytes;      /* size of the image (the published segment's size) */
    int32_t mapped;            /* 1: a read-only mapping of a published segment */
    int32_t device;            /* GPU holding the device copy, -1 when there is none */
} fp_refstore_info;

/* An empty store in host memory for num_contigs contigs (each empty, with no known sites until set). */
fp_status fp_refstore_create(uint32_t num_contigs, fp_refstore **out);

/* Contig `contig_id` as 4-bit IUPAC symbols packed eight per word (the same input as fp_engine_set_contig).
 * The store keeps a copy. FP_BAD_INPUT for a mapped or uploaded store, or an id out of range. */
fp_status fp_refstore_set_contig(fp_refstore *store, uint32_t contig_id, const uint32_t *packed4,
                                 uint64_t num_bases);

/* Known sites of a contig, sorted by start (the same input as fp_engine_set_known_sites). The store keeps a
 * copy together with the prefix maximum of the stops (loader/variants.cu:125-133). */
fp_status fp_refstore_set_known_sites(fp_refstore *store, uint32_t contig_id, const uint32_t *feature_start,
                                      const uint32_t *feature_stop, uint32_t num_sites);

/* The segment name the reference derives from a file path (mmap.cu:57-89): "/firepony_" followed by the
 * absolute path with every '/' replaced by '_'. The file must exist. FP_BAD_INPUT if it does not or if the
 * name does not fit in `cap` bytes (including the terminating zero). */
fp_status fp_refstore_shm_name(const char *path, char *name, size_t cap);

/* Writes the store's image into a new shared-memory segment `name` (a POSIX shm name: one leading '/',
 * no other '/'). An existing segment of that name is unlinked first. */
fp_status fp_refstore_publish(const fp_refstore *store, const char *name);

/* Maps the published segment `name` read-only. The store's contigs and sites point into the mapping.
 * FP_BAD_INPUT if no complete segment of a known format has that name; fp_refstore_last_error(NULL) then
 * says why. */
fp_status fp_refstore_open(const char *name, fp_refstore **out);

/* Removes the segment name (mappings in use stay valid until they are closed). */
fp_status fp_refstore_unlink(const char *name);

fp_status fp_refstore_get_info(const fp_refstore *store, fp_refstore_info *out);

/* Host pointers into the store (its copy, or the mapping) valid until the store is destroyed. */
fp_status fp_refstore_get_contig(const fp_refstore *store, uint32_t contig_id, const uint32_t **packed4,
                                 uint64_t *num_bases);
fp_status fp_refstore_get_known_sites(const fp_refstore *store, uint32_t contig_id, const uint32_t **feature_start,
                                      const uint32_t **feature_stop, uint32_t *num_sites);

/* Copies the image to GPU `device` (one allocation, one copy). A store holds one device copy: uploading to
 * the device that already holds it does nothing, and another device is FP_BAD_INPUT while engines are
 * attached (otherwise the old copy is freed first). */
fp_status fp_refstore_upload(fp_refstore *store, int device);

/* The engine reads its contigs and known sites from the store's device copy instead of its own (which it
 * frees). The store is uploaded to the engine's device first if it has no device copy; a copy on another
 * device is FP_BAD_INPUT. While attached, fp_engine_set_contig / fp_engine_set_known_sites return
 * FP_BAD_INPUT. A NULL store detaches the engine, which then has no contigs until they are set again.
 * Destroying the engine detaches it. */
fp_status fp_engine_attach_refstore(fp_engine *engine, fp_refstore *store);

/* Frees the store (its device copy, its mapping). FP_BAD_INPUT, freeing nothing, while engines are attached. */
fp_status fp_refstore_destroy(fp_refstore *store);

/* The message of the store's last failure; with NULL, that of the calling thread's last failed
 * fp_refstore_open or fp_refstore_create. */
const char *fp_refstore_last_error(const fp_refstore *store);

#ifdef __cplusplus
}
#endif

#endif
