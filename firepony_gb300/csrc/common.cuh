// Shared device-side definitions of the GB300 BQSR engine: batch/reference descriptors, constants, the
// dense covariate-key layout, and error reporting. All kernels of the engine include this header.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fpg {

typedef uint8_t u8;
typedef uint16_t u16;
typedef uint32_t u32;
typedef uint64_t u64;
typedef int16_t i16;
typedef int32_t i32;

// cigar_op codes (types.h:61-72) and cigar_event codes (device/cigar.h:41-47)
enum { OP_M = 0, OP_I = 1, OP_D = 2, OP_N = 3, OP_S = 4, OP_H = 5, OP_P = 6, OP_EQ = 7, OP_X = 8 };
enum { EV_M = 0, EV_I = 1, EV_D = 2, EV_S = 3 };
// AlignmentFlags (alignment_data.h:46-72)
enum {
    F_PAIRED = 1, F_UNMAP = 4, F_MATE_UNMAP = 8, F_REVERSE = 16, F_MATE_REVERSE = 32, F_READ2 = 128,
    F_SECONDARY = 256, F_QC_FAIL = 512, F_DUPLICATE = 1024,
};
enum { IUPAC_A = 1, IUPAC_C = 2, IUPAC_G = 4, IUPAC_T = 8, IUPAC_N = 15 };

constexpr u16 U16_NONE = 0xFFFF;
constexpr u32 U32_NONE = 0xFFFFFFFFu;
constexpr u32 MAX_READ_LEN = 511;          // cycle covariate field is 10 bits (cycle_illumina.h:38)
constexpr int MIN_BAND_WIDTH = 7;
constexpr int MIN_BASE_QUAL = 4;
constexpr u8 NO_BAQ_UNCERTAINTY = 64;      // device/baq.h:38

// read status values (fp_engine_debug_last_batch)
// RS_DEFERRED: active, its BAQ result waits for the exact replay (counted by the second covariate pass)
enum { RS_FILTERED = 0, RS_ACTIVE = 1, RS_REMOVED = 2, RS_DEFERRED = 3 };

// per-base flag bits
enum { BF_SNP = 1, BF_INS = 2, BF_DEL = 4, BF_ACTIVE = 8 };

// device error bits
enum {
    ERR_BAD_READ_RANGE = 1, ERR_READ_TOO_LONG = 2, ERR_BAD_READ_GROUP = 4, ERR_CAPACITY = 8, ERR_INTERNAL = 16,
    ERR_TIMEOUT = 32,
};

struct DevBatch {
    u32 R, num_cigar_ops;
    u64 num_syms, num_quals;
    const u16 *chromosome;
    const u32 *astart, *astop, *mstart;
    const i32 *isize;
    const u32 *cigars, *cigar_start, *cigar_len;
    const u32 *reads, *read_start, *read_len;
    const u8 *quals;
    const u32 *qual_start, *qual_len;
    const u16 *flags;
    const u8 *mapq;
    const u32 *rg;
};

struct DevContig {
    const u32 *words;
    u64 size;
};

struct DevSites {
    const u32 *start, *stop, *maxend;
    u32 n;
    u32 pad;
};

struct DevRef {
    const DevContig *contigs;
    u32 num_contigs;
    const DevSites *sites;
    u32 num_site_contigs;
};

__device__ __forceinline__ u8 sym4(const u32 *w, u64 i) { return u8((w[i >> 3] >> ((i & 7) * 4)) & 0xF); }

// Contig symbol; positions past the end read as 0 (the packed storage's padding).
__device__ __forceinline__ u8 contig_at(const DevContig &c, u64 i) { return i < c.size ? sym4(c.words, i) : u8(0); }

__device__ __forceinline__ u32 op_len(u32 c) { return c & 0xFFFFFFu; }
__device__ __forceinline__ u32 op_code(u32 c) { return (c >> 24) & 0xFu; }

// ---- dense covariate-key layout ----
// The engine accumulates the three observation tables in dense arrays whose index is a monotone function
// of the reference's 32-bit key, so ascending dense index == ascending key (the reduced tables' order,
// device/covariate_table.cu:43-107):
//   quality: ((rg*256 + q) * 4 + slot)
//   cycle:   ((rg*256 + q) * 1024 + cycle_field) * 4 + slot
//   context: ((rg*256 + q) * 80 + context_rank) * 4 + slot
// with event slots M -> 0, I -> 2, D -> 3 (slot 1 unused) so that the I and D counters of one prefix form
// an aligned 8-byte pair. context_rank enumerates the 80 context values that can occur in a valid key,
// (c<<4)|2 for 2-mers and (c<<4)|3 for 3-mers, in ascending order.
constexpr u32 Q_SPAN = 256;
constexpr u32 CYCLE_SPAN = 1024;
constexpr u32 CONTEXT_SPAN = 80;
constexpr u32 EV_SLOTS = 4;
constexpr u32 QUAL_KEYS_PER_RG = Q_SPAN * EV_SLOTS;
constexpr u32 CYCLE_KEYS_PER_RG = Q_SPAN * CYCLE_SPAN * EV_SLOTS;
constexpr u32 CONTEXT_KEYS_PER_RG = Q_SPAN * CONTEXT_SPAN * EV_SLOTS;
__host__ __device__ inline u32 ev_slot(u32 ev) { return ev == 0 ? 0u : ev + 1u; }
__host__ __device__ inline u32 slot_ev(u32 slot) { return slot == 0 ? 0u : slot - 1u; }
constexpr u32 CYCLE_INVALID = (1u << 10) - 1;
constexpr u32 CONTEXT_INVALID = (1u << 11) - 1;

struct KeySpace {
    u32 n_rg;
    u32 qual_base, cycle_base, context_base, total;
};

__host__ __device__ inline KeySpace make_keyspace(u32 n_rg) {
    KeySpace k;
    k.n_rg = n_rg;
    k.qual_base = 0;
    k.cycle_base = n_rg * QUAL_KEYS_PER_RG;
    k.context_base = k.cycle_base + n_rg * CYCLE_KEYS_PER_RG;
    k.total = k.context_base + n_rg * CONTEXT_KEYS_PER_RG;
    return k;
}

// rank of a valid context value among the 80 valid values (ascending)
__host__ __device__ inline u32 context_rank(u32 v) {
    const u32 c = v >> 4, len = v & 15;
    // values ascending: c<16 pairs (c<<4|2, c<<4|3), then c>=16 only 3-mers
    if (c < 16) return c * 2 + (len == 3 ? 1 : 0);
    return 32 + (c - 16);
}
__host__ __device__ inline u32 context_value(u32 rank) {
    if (rank < 32) return ((rank / 2) << 4) | ((rank & 1) ? 3 : 2);
    return ((rank - 32 + 16) << 4) | 3;
}

// error reporting: a sticky bit mask in device memory
__device__ __forceinline__ void raise_error(u32 *err, u32 bit) { atomicOr(err, bit); }

}  // namespace fpg
