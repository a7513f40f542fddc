/*
 * BQSR oracle — TEST INFRASTRUCTURE ONLY (see bqsr_oracle.h).
 *
 * A restatement, stage by stage, of broadinstitute/firepony's per-batch BQSR path as its host (TBB)
 * backend runs it. Every function cites the reference lines it follows (paths relative to the Firepony
 * tree). Where the reference is undefined (uninitialised or out-of-range reads) the oracle fixes one
 * behaviour and the header of the function says which; the GPU engine implements the same choice.
 *
 * Canonical summation order. The reference accumulates float mismatches per batch by append + stable
 * radix sort + reduce_by_key (device/covariates.cu:172-201, device/covariate_table.cu:43-107). Its
 * association order is not defined (the lift library that implements it is absent), so the oracle
 * defines it as the left fold of a stable sort: per key, a sequential float sum in stream order
 * (batch, read, cigar event, M/I/D slot), starting from the running total.
 *
 * Build: -O2 -ffp-contract=off, no fast-math (the reference's host flags, gcc.cmake:5-7, carry no
 * fast-math). libm (glibc) supplies pow/log/log10/lgammaf/round exactly as the reference's host build.
 */
#include "bqsr_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

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
// DNA_IUPAC symbols (device/from_nvbio/alphabet.h:114-136)
enum { IUPAC_A = 1, IUPAC_C = 2, IUPAC_G = 4, IUPAC_T = 8, IUPAC_N = 15 };

const u16 U16_NONE = 0xFFFF;
const u32 U32_NONE = 0xFFFFFFFFu;

struct us2 { u16 x, y; };
struct ss2 { i16 x, y; };

// lift's min/max take both arguments as the explicit template type (used as min<uint16>(...))
template <typename T> inline T tmin(T a, T b) { return a < b ? a : b; }
template <typename T> inline T tmax(T a, T b) { return a > b ? a : b; }

// abs() local to device/baq.cu:84-87: returns uint32
inline u32 baq_abs(i32 v) { return v < 0 ? u32(-v) : u32(v); }

inline u8 sym4(const u32 *words, u64 i) { return u8((words[i >> 3] >> ((i & 7) * 4)) & 0xF); }

struct Contig {
    std::vector<u32> words;
    u64 size = 0;
    // Symbols past the end of the contig read as 0: the reference reads whatever the packed storage holds
    // there (device/cigar.cu:663-667 and device/baq.cu:322-323 do not bound the access).
    u8 at(u64 i) const { return i < size ? sym4(words.data(), i) : u8(0); }
};

struct KnownSites {
    std::vector<u32> feature_start, feature_stop, max_end_point_left;
};

// ---- covariate key chains (device/covariates/bit_packers/*.h, packer_*.h) ----
// RecalTable1: EventTracker(2) @0 | QualityScore(8) @2 | ReadGroup(8) @10     (18 bits)
// Cycle:       EventTracker(2) @0 | Cycle(10) @2 | QualityScore(8) @12 | RG(8) @20   (28 bits)
// Context:     EventTracker(2) @0 | Context(11) @2 | QualityScore(8) @13 | RG(8) @21 (29 bits)
const u32 CYCLE_INVALID = (1u << 10) - 1;
const u32 CONTEXT_INVALID = (1u << 11) - 1;

struct TableRow {
    u32 key;
    u64 observations;
    float mismatches;
};

struct EmpiricalRow {
    u32 key;
    u64 observations;
    double mismatches, expected_errors, estimated_quality, empirical_quality;
};

struct Entry {
    u32 key;
    float mism;
};

// One running covariate observation table: sorted by key, one row per key (device/covariate_table.h:57-130).
struct ObsTable {
    std::vector<TableRow> rows;

    // Appends entries (in stream order), stable-sorts by key and reduces with a left fold
    // (device/covariates.cu:172-201, device/covariate_table.cu:43-107). fold_sorted takes entries already in
    // that stable order.
    void fold(std::vector<Entry> &entries) {
        std::stable_sort(entries.begin(), entries.end(), [](const Entry &a, const Entry &b) { return a.key < b.key; });
        fold_sorted(entries);
    }
    void fold_sorted(const std::vector<Entry> &entries, int num_threads = 1) {
        if (entries.empty()) return;
        // the key range is cut at entry keys into parts that never split a key; each part merges the running
        // rows and the new entries of its keys on its own thread, and the parts are concatenated in order
        const int P = std::max(1, std::min<int>(num_threads, int(entries.size() / 4096) + 1));
        std::vector<size_t> ecut(P + 1), rcut(P + 1);
        ecut[0] = 0; rcut[0] = 0; ecut[P] = entries.size(); rcut[P] = rows.size();
        for (int p = 1; p < P; p++) {
            const u32 k = entries[entries.size() * p / P].key;
            ecut[p] = size_t(std::lower_bound(entries.begin(), entries.end(), k,
                                              [](const Entry &e, u32 x) { return e.key < x; }) - entries.begin());
            rcut[p] = size_t(std::lower_bound(rows.begin(), rows.end(), k,
                                              [](const TableRow &r, u32 x) { return r.key < x; }) - rows.begin());
        }
        // (the part and output buffers are kept from batch to batch so their pages are reused)
        if (part_buf.size() < size_t(P)) part_buf.resize(size_t(P));
#pragma omp parallel for num_threads(P) schedule(static, 1) if (P > 1)
        for (int p = 0; p < P; p++) {
            part_buf[p].clear();
            merge_range(rows, rcut[p], rcut[p + 1], entries, ecut[p], ecut[p + 1], part_buf[p]);
        }
        spare.clear();
        size_t n = 0;
        for (int p = 0; p < P; p++) n += part_buf[p].size();
        spare.reserve(n);
        for (int p = 0; p < P; p++) spare.insert(spare.end(), part_buf[p].begin(), part_buf[p].end());
        rows.swap(spare);
    }
    std::vector<TableRow> spare;
    std::vector<std::vector<TableRow>> part_buf;

    static void merge_range(const std::vector<TableRow> &rows, size_t i, size_t i_end, const std::vector<Entry> &entries,
                            size_t j, size_t j_end, std::vector<TableRow> &out) {
        out.reserve((i_end - i) + (j_end - j));
        while (i < i_end || j < j_end) {
            u32 key;
            if (j >= j_end || (i < i_end && rows[i].key <= entries[j].key)) key = rows[i].key;
            else key = entries[j].key;
            TableRow acc = {key, 0, 0.0f};
            bool first = true;
            // the running row precedes the new entries of the same key (stable order)
            if (i < i_end && rows[i].key == key) {
                acc = rows[i];
                first = false;
                i++;
            }
            while (j < j_end && entries[j].key == key) {
                if (first) {
                    acc.observations = 1;
                    acc.mismatches = entries[j].mism;
                    first = false;
                } else {
                    acc.observations += 1;
                    acc.mismatches = acc.mismatches + entries[j].mism;
                }
                j++;
            }
            out.push_back(acc);
        }
    }
};

// ---- empirical quality (device/empirical_quality.cu:35-198, device/expected_error.h:37-76) ----
const int MAX_RECALIBRATED_Q_SCORE = 93;
const int MAX_REASONABLE_Q_SCORE = 60;
const int MAX_GATK_USABLE_Q_SCORE = 40;
const u32 MAX_NUMBER_OF_OBSERVATIONS = 2147483647u - 1;

double gaussian(double value) {  // device/empirical_quality.cu:43-53
    const double GF_a = 0.0, GF_b = 0.9, GF_c = 0.0, GF_d = 0.5;
    return GF_a + GF_b * pow(double(M_E), -(pow(value - GF_c, 2.0) / (2 * GF_d * GF_d)));
}

double log10QempPrior(double Qempirical, double Qreported, bool need_rounding) {  // :55-65
    double delta = Qempirical - Qreported;
    if (need_rounding) delta = round(delta);
    int difference = std::min(std::abs(int(delta)), MAX_GATK_USABLE_Q_SCORE);
    return log10(gaussian(double(difference)));
}

double lnToLog10(double ln) { return ln * log10(M_E); }                      // :67-70
double log10Gamma(double x) { return lnToLog10(lgammaf(float(x))); }         // :72-75 (float lgammaf)
double log10Factorial(u64 x) { return log10Gamma(double(x + 1)); }          // :77-80

double log10BinomialCoefficient(u64 n, u64 k) {  // :82-85
    return log10Factorial(n) - log10Factorial(k) - log10Factorial(n - k);
}

double log10BinomialProbability(u64 n, u64 k, double log10p) {  // :87-91
    double log10OneMinusP = log10(1 - pow(10.0, log10p));
    return log10BinomialCoefficient(n, k) + log10p * double(k) + log10OneMinusP * double(n - k);
}

double log10QempLikelihood(double Qempirical, u64 nObservations, u64 nErrors) {  // :98-112
    if (nObservations == 0) return 0.0;
    if (nObservations > MAX_NUMBER_OF_OBSERVATIONS) {
        double fraction = double(MAX_NUMBER_OF_OBSERVATIONS) / double(nObservations);
        nErrors = u64(round(double(nErrors) * fraction));
        nObservations = MAX_NUMBER_OF_OBSERVATIONS;
    }
    return log10BinomialProbability(nObservations, nErrors, Qempirical / -10.0);
}

double bayesianEstimateOfEmpiricalQuality(u64 nObservations, u64 nErrors, double QReported, bool need_rounding) {
    // :137-163; the normalised posterior is computed by the reference but never read, so it is skipped
    const int numBins = MAX_REASONABLE_Q_SCORE + 1;
    double log10Posteriors[numBins];
    for (int bin = 0; bin < numBins; bin++) {
        const double QEmpOfBin = bin / 1.0;
        log10Posteriors[bin] = log10QempPrior(QEmpOfBin, QReported, need_rounding) +
                               log10QempLikelihood(QEmpOfBin, nObservations, nErrors);
    }
    int MLEbin = 0;
    for (int i = 1; i < numBins; i++)
        if (log10Posteriors[i] > log10Posteriors[MLEbin]) MLEbin = i;
    return MLEbin / 1.0;
}

double calcEmpiricalQuality(u64 observations_in, double mismatches_in, double estimated_quality,
                            bool need_rounding) {  // :165-174
    const u64 mismatches = u64(mismatches_in + 0.5) + 1;
    const u64 observations = observations_in + 1 + 1;
    double empiricalQual = bayesianEstimateOfEmpiricalQuality(observations, mismatches, estimated_quality, need_rounding);
    return std::min(empiricalQual, double(MAX_RECALIBRATED_Q_SCORE));
}

void compute_empirical(EmpiricalRow &r, bool need_rounding) {  // :186-190
    r.estimated_quality = double(-10.0 * log10(r.expected_errors / double(r.observations)));
    r.empirical_quality = calcEmpiricalQuality(r.observations, r.mismatches, r.estimated_quality, need_rounding);
}

double qualToErrorProb(u8 qual) { return pow(10.0, qual / -10.0); }  // device/expected_error.h:48-51

// (int) of the MAP quality expression (device/baq.cu:673). The expression is +inf whenever 1.0 - max
// rounds to 0 and NaN when a row has no mass. C leaves that conversion undefined; the reference's CUDA
// build (cvt.rzi.s32.f64), its host build on Arm (fcvtzs) and GATK's Java cast all saturate to INT_MAX
// and map NaN to 0, and this is the behaviour fixed here. (An x86 host build would produce INT_MIN.)
int saturating_int(double t) {
    if (t != t) return 0;
    if (t >= 2147483647.0) return 2147483647;
    if (t <= -2147483648.0) return -2147483647 - 1;
    return int(t);
}

// ---- BAQ HMM (device/baq.cu:214-697) ----
const double EM = 0.33333333333;
const double EI = 0.25;
const int MIN_BAND_WIDTH = 7;
const int MIN_BASE_QUAL = 4;
const double GAP_EXTENSION_PROBABILITY = 0.1;

struct HmmScratch {
    std::vector<double> fwd, bwd, scale;
};

inline int set_u(int b, int i, int k) {  // device/baq.cu:336-341
    int x = i - b;
    x = x > 0 ? x : 0;
    return (k + 1 - x) * 3;
}

inline double calcEpsilon(u8 ref, u8 read, u8 qualB, const double *qual2prob) {  // :361-372
    if (ref == IUPAC_N || read == IUPAC_N) return 1.0;
    double qual = qual2prob[qualB < MIN_BASE_QUAL ? MIN_BASE_QUAL : qualB];
    double e = (ref == read ? 1 - qual : qual * EM);
    return e;
}

// Runs forward / backward / MAP for one read. ref[0..referenceLength) and query/qual[0..queryLen).
// bm_reference_length is the referenceLength used for bM/bI (computed before the left-clamp decrement,
// device/baq.cu:291-315). Writes quality and state per query base.
void hmm_glocal(const u8 *ref, int referenceLength, int bm_reference_length, const u8 *query, const u8 *qual,
                int queryLen, int bandWidth, const double *qual2prob, double gap_open, u8 *outQual, u32 *outState,
                HmmScratch &s) {
    const int bandWidth2 = bandWidth * 2 + 1;
    const int row = bandWidth2 * 3 + 6;
    const double GOP = gap_open;
    s.fwd.assign(size_t(queryLen + 1) * row, 0.0);
    s.bwd.assign(size_t(queryLen + 1) * row, 0.0);
    s.scale.assign(size_t(queryLen + 2), 0.0);
    double *F = s.fwd.data(), *B = s.bwd.data(), *S = s.scale.data();

    // setup (:247-334)
    const double sM = 1.0 / (2 * queryLen + 2);
    const double sI = sM;
    const double bM = (1 - GOP) / bm_reference_length;
    const double bI = GOP / bm_reference_length;
    double m[9];
    m[0 * 3 + 0] = (1 - GOP - GOP) * (1 - sM);
    m[0 * 3 + 1] = GOP * (1 - sM);
    m[0 * 3 + 2] = m[0 * 3 + 1];
    m[1 * 3 + 0] = (1 - GAP_EXTENSION_PROBABILITY) * (1 - sI);
    m[1 * 3 + 1] = GAP_EXTENSION_PROBABILITY * (1 - sI);
    m[1 * 3 + 2] = 0.0;
    m[2 * 3 + 0] = 1 - GAP_EXTENSION_PROBABILITY;
    m[2 * 3 + 1] = 0.0;
    m[2 * 3 + 2] = GAP_EXTENSION_PROBABILITY;

    auto off = [&](int i, int j) { return i * row + j; };
    int i, k;

    // forward (:374-526)
    F[off(0, set_u(bandWidth, 0, 0))] = 1.0;
    S[0] = 1.0;
    {
        double *fi = &F[off(1, 0)];
        double sum;
        int beg = 1;
        int end = referenceLength < bandWidth + 1 ? referenceLength : bandWidth + 1;
        sum = 0.0;
        for (k = beg; k <= end; ++k) {
            double e = calcEpsilon(ref[k - 1], query[0], qual[0], qual2prob);
            int u = set_u(bandWidth, 1, k);
            fi[u + 0] = e * bM;
            fi[u + 1] = EI * bI;
            sum += fi[u] + fi[u + 1];
        }
        S[1] = sum;
        int _beg = set_u(bandWidth, 1, beg);
        int _end = set_u(bandWidth, 1, end) + 2;
        for (k = _beg; k <= _end; ++k) fi[k] /= sum;
    }
    for (i = 2; i <= queryLen; ++i) {
        double *fi = &F[off(i, 0)];
        double *fi1 = &F[off(i - 1, 0)];
        double sum;
        int beg = 1, end = referenceLength, x;
        u8 qyi = query[i - 1];
        x = i - bandWidth;
        beg = beg > x ? beg : x;
        x = i + bandWidth;
        end = end < x ? end : x;
        sum = 0.0;
        for (k = beg; k <= end; ++k) {
            double e = calcEpsilon(ref[k - 1], qyi, qual[i - 1], qual2prob);
            int u = set_u(bandWidth, i, k);
            int v11 = set_u(bandWidth, i - 1, k - 1);
            int v10 = set_u(bandWidth, i - 1, k);
            int v01 = set_u(bandWidth, i, k - 1);
            fi[u + 0] = e * (m[0] * fi1[v11 + 0] + m[3] * fi1[v11 + 1] + m[6] * fi1[v11 + 2]);
            fi[u + 1] = EI * (m[1] * fi1[v10 + 0] + m[4] * fi1[v10 + 1]);
            fi[u + 2] = m[2] * fi[v01 + 0] + m[8] * fi[v01 + 2];
            sum += fi[u] + fi[u + 1] + fi[u + 2];
        }
        S[i] = sum;
        int _beg = set_u(bandWidth, i, beg);
        int _end = set_u(bandWidth, i, end) + 2;
        for (k = _beg, sum = 1. / sum; k <= _end; ++k) fi[k] *= sum;
    }
    {
        double sum = 0.0;
        for (k = 1; k <= referenceLength; ++k) {
            int u = set_u(bandWidth, queryLen, k);
            if (u < 3 || u >= bandWidth2 * 3 + 3) continue;
            sum += F[off(queryLen, u + 0)] * sM + F[off(queryLen, u + 1)] * sI;
        }
        S[queryLen + 1] = sum;
    }

    // backward (:528-617). b[0] (:597-616) is never read by MAP and is not computed.
    for (k = 1; k <= referenceLength; ++k) {
        int u = set_u(bandWidth, queryLen, k);
        double *bi = &B[off(queryLen, 0)];
        if (u < 3 || u >= bandWidth2 * 3 + 3) continue;
        bi[u + 0] = sM / S[queryLen] / S[queryLen + 1];
        bi[u + 1] = sI / S[queryLen] / S[queryLen + 1];
    }
    for (i = queryLen - 1; i >= 1; --i) {
        int beg = 1, end = referenceLength, x;
        double *bi = &B[off(i, 0)];
        double *bi1 = &B[off(i + 1, 0)];
        double y = (i > 1) ? 1. : 0.;
        u8 qyi1 = query[i];
        x = i - bandWidth;
        beg = beg > x ? beg : x;
        x = i + bandWidth;
        end = end < x ? end : x;
        for (k = end; k >= beg; --k) {
            int u = set_u(bandWidth, i, k);
            int v11 = set_u(bandWidth, i + 1, k + 1);
            int v10 = set_u(bandWidth, i + 1, k);
            int v01 = set_u(bandWidth, i, k + 1);
            double e;
            if (k >= referenceLength) e = 0;
            else e = calcEpsilon(ref[k], qyi1, qual[i], qual2prob) * bi1[v11];
            bi[u + 0] = e * m[0] + EI * m[1] * bi1[v10 + 1] + m[2] * bi[v01 + 2];
            bi[u + 1] = e * m[3] + EI * m[4] * bi1[v10 + 1];
            bi[u + 2] = (e * m[6] + m[8] * bi[v01 + 2]) * y;
        }
        int _beg = set_u(bandWidth, i, beg);
        int _end = set_u(bandWidth, i, end) + 2;
        y = 1.0 / S[i];
        for (k = _beg; k <= _end; ++k) bi[k] *= y;
    }

    // MAP (:619-681)
    for (i = 1; i <= queryLen; ++i) {
        double sum = 0.0, max = 0.0;
        const double *fi = &F[off(i, 0)];
        const double *bi = &B[off(i, 0)];
        int beg = 1, end = referenceLength, x, max_k = -1;
        x = i - bandWidth;
        beg = beg > x ? beg : x;
        x = i + bandWidth;
        end = end < x ? end : x;
        for (k = beg; k <= end; ++k) {
            const int u = set_u(bandWidth, i, k);
            double z;
            z = fi[u + 0] * bi[u + 0];
            sum += z;
            if (z > max) {
                max = z;
                max_k = (k - 1) << 2 | 0;
            }
            z = fi[u + 1] * bi[u + 1];
            sum += z;
            if (z > max) {
                max = z;
                max_k = (k - 1) << 2 | 1;
            }
        }
        max /= sum;
        outState[i - 1] = u32(max_k);
        int kq = saturating_int(double(-4.343) * log(double(1.0) - double(max)) + double(.499));
        outQual[i - 1] = u8(kq > 100 ? 99 : (kq < MIN_BASE_QUAL ? MIN_BASE_QUAL : kq));
    }
}

}  // namespace

// ------------------------------------------------------------------------------------------------
struct fpo_ctx {
    u32 num_read_groups;
    std::vector<Contig> contigs;
    std::vector<KnownSites> sites;
    ObsTable quality, cycle, context;
    std::vector<EmpiricalRow> emp[4];
    std::vector<u32> out_keys[4];
    std::vector<u64> out_obs[4];
    std::vector<double> out_mism[4], out_exp[4], out_est[4], out_emp[4];
    u64 total_reads = 0, filtered_reads = 0, baq_reads = 0, num_batches = 0;
    // thread-seconds per stage (FPO_STAGE_*), summed over the OpenMP threads
    double stage_sec[FPO_NUM_STAGES] = {};
    std::vector<std::vector<Entry>> run_q, run_c, run_x;  // per-chunk entry streams of a batch
    double qual2prob[256];
    double gap_open;

    // intermediates of the last batch (for per-stage parity tests)
    std::vector<u8> dbg_status, dbg_flags, dbg_baq;
    std::vector<u16> dbg_windows;
    std::vector<i16> dbg_hmm;
    std::vector<double> dbg_frac;
    u64 dbg_num_quals = 0;
};

namespace {

const Contig *contig_of(const fpo_ctx *c, u32 id) {
    if (id < c->contigs.size() && c->contigs[id].size > 0) return &c->contigs[id];
    return nullptr;
}
u64 contig_size(const fpo_ctx *c, u32 id) {
    const Contig *g = contig_of(c, id);
    return g ? g->size : 0;
}

// lower_bound / upper_bound (device/primitives/algorithms.h:39-100)
size_t ref_lower_bound(u32 x, const u32 *begin, size_t n) {
    if (n == 0) return 0;
    if (x < begin[0]) return 0;
    if (begin[n - 1] < x) return n;
    size_t base = 0, count = n;
    while (count > 0) {
        size_t count2 = count / 2;
        size_t mid = base + count2;
        if (begin[mid] < x) {
            base = mid + 1;
            count -= count2 + 1;
        } else {
            count = count2;
        }
    }
    return base;
}
size_t ref_upper_bound(u32 x, const u32 *begin, size_t n) {
    size_t base = 0, count = n;
    while (count > 0) {
        size_t step = count / 2;
        size_t it = base + step;
        if (!(x < begin[it])) {
            base = it + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    return base;
}

struct BatchState {
    const fp_batch_view *b;
    u32 R;
    std::vector<u8> status;            // 0 filtered, 1 active, 2 removed by the BAQ window check
    std::vector<u32> cigar_offsets;    // device/cigar.cu:823-834
    std::vector<u8> ev_type;
    std::vector<u16> ev_readc, ev_refc;
    std::vector<u32> ev_read_index;
    std::vector<us2> alignment_window_lo, clipped, no_ins, refwin, hq;
    std::vector<u32> alignment_window_x, alignment_window_y;
    std::vector<u16> num_errors;
    std::vector<ss2> hmm_window;
    std::vector<u16> bandwidth;
    // per read symbol (read_start index space)
    std::vector<u8> active_loc, is_snp, is_ins, is_del;
    // per quality (qual_start index space)
    std::vector<u8> baq;
    std::vector<u32> baq_state;
    std::vector<double> frac[3];

    u8 read_sym(u64 i) const { return sym4(b->reads, i); }
};

u32 op_len(u32 c) { return c & 0xFFFFFFu; }
u32 op_code(u32 c) { return (c >> 24) & 0xFu; }

// filter_mapq, filter_if_any_set, filter_if_cigar_malformed (device/read_filters.cu:42-75, :156-258)
bool passes_invalid_filters(const BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    if (b->mapq[r] == 0 || b->mapq[r] == 255) return false;
    if (b->flags[r] & (F_DUPLICATE | F_QC_FAIL | F_UNMAP | F_SECONDARY)) return false;
    enum { LEADING_HARD, LEADING_SOFT, NO_CLIPS, TRAILING_SOFT, TRAILING_HARD } st = LEADING_HARD;
    for (u32 i = b->cigar_start[r]; i < b->cigar_start[r] + b->cigar_len[r]; i++) {
        u32 op = op_code(b->cigars[i]);
        if (op == OP_N) return false;
        if (op == OP_H) {
            switch (st) {
            case LEADING_HARD: break;
            case LEADING_SOFT: return false;
            case NO_CLIPS:
            case TRAILING_SOFT: st = TRAILING_HARD; break;
            case TRAILING_HARD: break;
            }
        } else if (op == OP_S) {
            switch (st) {
            case LEADING_HARD: st = LEADING_SOFT; break;
            case LEADING_SOFT: break;
            case NO_CLIPS: st = TRAILING_SOFT; break;
            case TRAILING_SOFT: break;
            case TRAILING_HARD: return false;
            }
        } else {
            switch (st) {
            case LEADING_HARD:
            case LEADING_SOFT: st = NO_CLIPS; break;
            case NO_CLIPS: break;
            case TRAILING_SOFT:
            case TRAILING_HARD: return false;
            }
        }
    }
    return true;
}

// compute_read_offset_list + compute_alignment_window (device/snp_filter.cu:42-147). The offset list is
// only used for the last base with a reference offset, so the window is derived directly.
void alignment_window(BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    // offsets of each read base in CIGAR order; the read's CIGAR is validated to cover read_len bases
    std::vector<u16> offs;
    u16 offset = 0;
    for (u32 c = 0; c < b->cigar_len[r]; c++) {
        u32 v = b->cigars[b->cigar_start[r] + c], op = op_code(v), len = op_len(v);
        switch (op) {
        case OP_M: case OP_EQ: case OP_X:
            for (u32 i = 0; i < len; i++) offs.push_back(offset++);
            break;
        case OP_I: case OP_N:
            for (u32 i = 0; i < len; i++) offs.push_back(offset);
            break;
        case OP_D: case OP_H: case OP_P:
            offset = u16(offset + len);
            break;
        case OP_S:
            for (u32 i = 0; i < len; i++) offs.push_back(U16_NONE);
            break;
        }
    }
    int c;
    for (c = int(b->read_len[r]) - 1; c >= 0; c--)
        if (c < int(offs.size()) && offs[c] != U16_NONE) break;
    if (c < 0) {
        s.alignment_window_x[r] = U32_NONE;
        s.alignment_window_y[r] = U32_NONE;
    } else {
        s.alignment_window_x[r] = b->alignment_start[r];
        s.alignment_window_y[r] = b->alignment_start[r] + offs[c];
    }
}

// Bases covered by the CIGAR (ops that produce read coordinates in cigar_coordinates_expand).
u64 cigar_read_length(const fp_batch_view *b, u32 r) {
    u64 n = 0;
    for (u32 c = 0; c < b->cigar_len[r]; c++) {
        u32 v = b->cigars[b->cigar_start[r] + c], op = op_code(v);
        if (op == OP_M || op == OP_EQ || op == OP_X || op == OP_I || op == OP_N || op == OP_S) n += op_len(v);
    }
    return n;
}

// filter_if_read_malformed (device/read_filters.cu:77-154). The reference compares the uint16 contig id
// with uint32(-1), which never matches, so those two checks are inert here too. A read on a contig that
// is not resident fails the contig-end check (the reference indexes out of range). Reads whose CIGAR does
// not cover exactly read_len bases, or that hold an op code above X (8), are also rejected: the reference
// then writes past the read's offset list or skips events (device/snp_filter.cu:54-96,
// device/cigar.cu:55-95) and its result is undefined.
bool passes_malformed_filter(const fpo_ctx *ctx, const BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    if (!(b->flags[r] & F_UNMAP)) {
        if (b->alignment_start[r] == U32_NONE) return false;
        if (s.alignment_window_y[r] <= s.alignment_window_x[r]) return false;
        if (s.alignment_window_x[r] >= contig_size(ctx, b->chromosome[r])) return false;
        if (b->cigar_len[r] == 0) return false;
    }
    if (b->read_group[r] == U32_NONE) return false;
    if (b->qual_len[r] != b->read_len[r]) return false;
    if (b->read_len[r] == 0) return false;
    if (cigar_read_length(b, r) != b->read_len[r]) return false;
    for (u32 c = 0; c < b->cigar_len[r]; c++)
        if (op_code(b->cigars[b->cigar_start[r] + c]) > OP_X) return false;
    return true;
}

// cigar_coordinates_expand (device/cigar.cu:536-614) together with cigar_op_expand (:55-95)
void expand_read(BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    u32 base = s.cigar_offsets[b->cigar_start[r]];
    u16 read_offset = 0, reference_offset = 0;
    u32 e = base;
    for (u32 c = 0; c < b->cigar_len[r]; c++) {
        u32 v = b->cigars[b->cigar_start[r] + c], op = op_code(v), len = op_len(v);
        for (u32 i = 0; i < len; i++, e++) {
            s.ev_read_index[e] = r;
            switch (op) {
            case OP_M: case OP_EQ: case OP_X:
                s.ev_type[e] = EV_M; s.ev_readc[e] = read_offset++; s.ev_refc[e] = reference_offset++;
                break;
            case OP_S:
                s.ev_type[e] = EV_S; s.ev_readc[e] = read_offset++; s.ev_refc[e] = U16_NONE;
                break;
            case OP_N: case OP_I:
                s.ev_type[e] = EV_I; s.ev_readc[e] = read_offset++; s.ev_refc[e] = U16_NONE;
                break;
            case OP_D: case OP_H: case OP_P:
                s.ev_type[e] = EV_D; s.ev_readc[e] = U16_NONE; s.ev_refc[e] = reference_offset++;
                break;
            default:  // op codes 9..15 produce no events data (type stays M in the reference's zeroed temp)
                s.ev_type[e] = EV_M; s.ev_readc[e] = U16_NONE; s.ev_refc[e] = U16_NONE;
                break;
            }
        }
    }
}

// remove_adapters (device/cigar.cu:111-344)
struct AdapterClip {
    BatchState &s;
    u32 r, cs, ce;
    AdapterClip(BatchState &s_, u32 r_) : s(s_), r(r_) {
        cs = s.cigar_offsets[s.b->cigar_start[r]];
        ce = s.cigar_offsets[s.b->cigar_start[r] + s.b->cigar_len[r]];
    }

    bool hasWellDefinedFragmentSize() {
        const fp_batch_view *b = s.b;
        const u32 flags = b->flags[r];
        const i32 isize = b->inferred_insert_size[r];
        if (isize == 0) return false;
        if (!(flags & F_PAIRED)) return false;
        if ((flags & F_UNMAP) || (flags & F_MATE_UNMAP)) return false;
        const bool rev = flags & F_REVERSE;
        const bool mate_rev = flags & F_MATE_REVERSE;
        if (rev == mate_rev) return false;
        if (flags & F_REVERSE) return b->alignment_stop[r] > b->mate_alignment_start[r];
        return b->alignment_start[r] <= b->mate_alignment_start[r] + u32(isize);
    }

    u32 getAdaptorBoundary() {
        const fp_batch_view *b = s.b;
        if (!hasWellDefinedFragmentSize()) return U32_NONE;
        if (b->flags[r] & F_REVERSE) return u32(b->mate_alignment_start[r] - 1);
        const int insertSize = b->inferred_insert_size[r] < 0 ? -b->inferred_insert_size[r] : b->inferred_insert_size[r];
        return u32(b->alignment_start[r] + insertSize + 1);
    }

    int getReadCoordinateForReferenceCoordinate(u32 ref_coord, bool right_tail) {
        const u32 start = s.b->alignment_start[r];
        for (u32 ev = cs; ev < ce; ev++) {
            if (start + u32(s.ev_refc[ev]) == ref_coord) {
                u16 read_coord = s.ev_readc[ev];
                if (read_coord == U16_NONE) {
                    if (right_tail) {
                        while (ev < ce) {
                            read_coord = s.ev_readc[ev];
                            if (read_coord != U16_NONE) break;
                            ev++;
                        }
                    } else {
                        while (ev >= cs && ev > 0) {
                            ev--;
                            read_coord = s.ev_readc[ev];
                            if (read_coord != U16_NONE) break;
                        }
                    }
                    if (read_coord == U16_NONE) return -1;
                }
                return read_coord;
            }
        }
        return -1;
    }

    us2 hardClip(int refStart, int refStop) {
        int start, stop;
        if (refStart < 0) {
            start = 0;
            stop = getReadCoordinateForReferenceCoordinate(u32(refStop), false);
        } else {
            start = getReadCoordinateForReferenceCoordinate(u32(refStart), true);
            stop = s.clipped[r].y - s.clipped[r].x - 1;
        }
        return us2{u16(start), u16(stop)};
    }

    us2 current_reference_window() {
        const us2 w = s.clipped[r];
        us2 rw = {0, 0};
        for (u32 i = cs; i < ce; i++) {
            if (s.ev_readc[i] == w.x) {
                while (i < ce && s.ev_refc[i] == U16_NONE) i++;
                if (i == ce) return us2{U16_NONE, U16_NONE};
                rw.x = s.ev_refc[i];
                break;
            }
        }
        for (u32 i = ce - 1; i >= cs && i != U32_NONE; i--) {
            if (s.ev_readc[i] == w.y) {
                while (s.ev_refc[i] == U16_NONE && i > cs) i--;
                if (i == cs) return us2{U16_NONE, U16_NONE};
                rw.y = s.ev_refc[i];
                break;
            }
        }
        return rw;
    }

    void run() {
        u32 boundary = getAdaptorBoundary();
        if (boundary == U32_NONE) return;
        const us2 rw = current_reference_window();
        const u32 start = s.b->alignment_start[r];
        if (boundary < start + u32(rw.x) || boundary > start + u32(rw.y)) return;
        if (s.b->flags[r] & F_REVERSE) {
            us2 adapter = hardClip(-1, int(boundary));
            s.clipped[r].x = tmax<u16>(s.clipped[r].x, u16(adapter.y + 1));
        } else {
            us2 adapter = hardClip(int(boundary), -1);
            s.clipped[r].y = tmin<u16>(s.clipped[r].y, u16(adapter.x - 1));
        }
    }
};

// remove_soft_clips (device/cigar.cu:346-408)
void remove_soft_clips(BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    us2 w = s.clipped[r];
    u32 ci = b->cigar_start[r];
    u32 read_offset = 0;
    const u32 cend = b->cigar_start[r] + b->cigar_len[r];
    while (ci < cend && read_offset < b->read_len[r]) {
        u32 v = b->cigars[ci], op = op_code(v), len = op_len(v);
        if (op == OP_H || op == OP_S) {
            if (read_offset + len > w.x) w.x = tmin<u16>(u16(read_offset + len), w.y);
            read_offset += len;
            ci++;
        } else {
            break;
        }
    }
    if (b->cigar_len[r] > 0) {
        ci = cend - 1;
        read_offset = b->read_len[r] - 1;
        while (ci >= b->cigar_start[r] && ci != U32_NONE && read_offset > w.x) {
            u32 v = b->cigars[ci], op = op_code(v), len = op_len(v);
            if (op == OP_H || op == OP_S) {
                if (read_offset - len < w.y) w.y = tmax<u16>(u16(read_offset - len), w.x);
                read_offset -= len;
                ci--;
            } else {
                break;
            }
        }
    }
    s.clipped[r] = w;
}

// compute_no_insertions_window (device/cigar.cu:410-471). When no event qualifies the reference keeps a
// stale value; here the window starts as (0xFFFF, 0xFFFF).
void no_insertions_window(BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    const u32 cs = s.cigar_offsets[b->cigar_start[r]];
    const u32 ce = s.cigar_offsets[b->cigar_start[r] + b->cigar_len[r]];
    const us2 w = s.clipped[r];
    us2 out = {U16_NONE, U16_NONE};
    u32 ev = cs;
    while (ev < ce) {
        const u16 ro = s.ev_readc[ev];
        if (ro == U16_NONE || ro < w.x) { ev++; continue; }
        if (s.ev_type[ev] == EV_I) { ev++; continue; }
        out.x = ro;
        break;
    }
    ev = ce - 1;
    while (ev >= cs && ev < ce) {
        const u16 ro = s.ev_readc[ev];
        if (ro == U16_NONE || ro > w.y) { ev--; continue; }
        if (s.ev_type[ev] == EV_I) { ev--; continue; }
        out.y = ro;
        break;
    }
    s.no_ins[r] = out;
}

// compute_reference_window (device/cigar.cu:473-534); same stale-value convention as above.
void reference_window(BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    const u32 cs = s.cigar_offsets[b->cigar_start[r]];
    const u32 ce = s.cigar_offsets[b->cigar_start[r] + b->cigar_len[r]];
    const us2 w = s.no_ins[r];
    us2 out = {U16_NONE, U16_NONE};
    for (u32 i = cs; i < ce; i++) {
        if (s.ev_readc[i] == w.x) {
            while (i < ce && s.ev_refc[i] == U16_NONE) i++;
            if (i == ce) { s.refwin[r] = us2{U16_NONE, U16_NONE}; return; }
            out.x = s.ev_refc[i];
            break;
        }
    }
    for (u32 i = ce - 1; i >= cs && i != U32_NONE; i--) {
        if (s.ev_readc[i] == w.y) {
            while (s.ev_refc[i] == U16_NONE && i > cs) i--;
            if (i == cs) { s.refwin[r] = us2{U16_NONE, U16_NONE}; return; }
            out.y = s.ev_refc[i];
            break;
        }
    }
    s.refwin[r] = out;
}

// compute_error_vectors (device/cigar.cu:616-737). The switch tests cigar_op values against the
// cigar_event labels I (=1) and D (=2), so '=' and X ops never count as mismatches.
void error_vectors(const fpo_ctx *ctx, BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    const bool negative_strand = b->flags[r] & F_REVERSE;
    const Contig *g = contig_of(ctx, b->chromosome[r]);
    const u32 astart = b->alignment_start[r];
    const us2 w = s.clipped[r];
    const us2 rw = s.refwin[r];
    const u32 rs = b->read_start[r];
    u16 current_bp_idx = 0;
    u16 num_errors = 0;
    for (u32 event = b->cigar_start[r]; event < b->cigar_start[r] + b->cigar_len[r]; event++) {
        const u32 cs = s.cigar_offsets[event];
        const u32 ce = s.cigar_offsets[event + 1];
        const u32 op = op_code(b->cigars[event]);
        if (op == OP_M) {
            for (u32 i = cs; i < ce; i++) {
                current_bp_idx = s.ev_readc[i];
                const u8 read_bp = s.read_sym(u64(rs) + current_bp_idx);
                const u32 reference_bp_idx = s.ev_refc[i];
                const u8 reference_bp = g->at(u64(astart) + reference_bp_idx);
                if (reference_bp != read_bp) {
                    s.is_snp[rs + current_bp_idx] = 1;
                    if (current_bp_idx >= w.x && current_bp_idx <= w.y) num_errors++;
                }
            }
        } else if (op == 1) {
            current_bp_idx = s.ev_readc[cs];
            if (current_bp_idx >= w.x && current_bp_idx <= w.y) {
                int off;
                if (!negative_strand) off = current_bp_idx - 1;
                else off = current_bp_idx + int(op_len(b->cigars[event]));
                if (off >= 0 && off <= w.y) {
                    s.is_ins[rs + off] = 1;
                    num_errors++;
                }
            }
        } else if (op == 2) {
            const u16 current_ref_idx = s.ev_refc[cs];
            if (current_ref_idx >= rw.x && current_ref_idx <= rw.y) {
                if (!negative_strand) {
                    s.is_del[rs + current_bp_idx] = 1;
                    num_errors++;
                } else {
                    const u16 off = u16(current_bp_idx + 1);
                    if (off < b->read_len[r]) {
                        s.is_del[rs + off] = 1;
                        num_errors++;
                    }
                }
            }
        }
    }
    s.num_errors[r] = num_errors;
}

// filter_non_regular_bases + filter_low_quality_bases (device/read_filters.cu:375-424)
void filter_bases(BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    const u32 rs = b->read_start[r];
    for (u32 i = rs; i < rs + b->read_len[r]; i++) {
        u8 bp = s.read_sym(i);
        if (bp != IUPAC_A && bp != IUPAC_C && bp != IUPAC_G && bp != IUPAC_T) s.active_loc[i] = 0;
    }
    for (u32 i = 0; i < b->read_len[r]; i++)
        if (b->qualities[b->qual_start[r] + i] < 6) s.active_loc[rs + i] = 0;
}

// compute_vcf_ranges + filter_bps (device/snp_filter.cu:162-395)
void filter_known_sites(const fpo_ctx *ctx, BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    const u32 ch = b->chromosome[r];
    if (ch >= ctx->sites.size()) return;
    const KnownSites &db = ctx->sites[ch];
    const us2 rw = s.refwin[r];
    const u32 astart = b->alignment_start[r];
    const u32 wx = astart + u32(rw.x), wy = astart + u32(rw.y);
    u32 vx = u32(ref_lower_bound(wx, db.max_end_point_left.data(), db.max_end_point_left.size()));
    if (vx >= db.feature_start.size()) return;
    u32 vy = u32(ref_upper_bound(wy, db.feature_start.data(), db.feature_start.size()));
    if (vy <= vx) return;
    if (vy >= db.feature_start.size()) vy = u32(db.feature_start.size() - 1);

    const us2 w = s.clipped[r];
    const u32 cigar_start = s.cigar_offsets[b->cigar_start[r]];
    const u32 cigar_end = s.cigar_offsets[b->cigar_start[r] + b->cigar_len[r]];
    const u32 rs = b->read_start[r];
    for (u32 feature = vx; feature <= vy; feature++) {
        const int feature_start = int(db.feature_start[feature] - astart);
        const int feature_end = int(db.feature_stop[feature] - astart);
        u32 ev;
        u16 ref_coord = U16_NONE;
        for (ev = cigar_start; ev < cigar_end; ev++) {
            ref_coord = s.ev_refc[ev];
            if (ref_coord != U16_NONE && int(ref_coord) >= feature_start) break;
        }
        if (ev == cigar_end) continue;
        int feature_bp_left = int(ref_coord) - feature_start;
        u32 ev_feature_start = ev;
        if (feature_bp_left > 0) {
            while (feature_bp_left && ev_feature_start > cigar_start) {
                u8 event = s.ev_type[ev_feature_start];
                if (event == EV_S) break;
                if (event == EV_M || event == EV_D) feature_bp_left--;
                ev_feature_start--;
            }
            while (ev_feature_start > cigar_start && s.ev_type[ev_feature_start - 1] == EV_I) ev_feature_start--;
            while (ev_feature_start < cigar_end && s.ev_readc[ev_feature_start] == U16_NONE) ev_feature_start++;
        } else {
            if (s.ev_refc[ev_feature_start] <= rw.y) {
                while (ev_feature_start > cigar_start && s.ev_type[ev_feature_start] == EV_D) ev_feature_start--;
            }
        }
        int feature_bp_right = feature_end - int(ref_coord);
        while (feature_bp_right > 0 && ev < cigar_end - 1) {
            ev++;
            u8 event = s.ev_type[ev];
            if (event == EV_S) break;
            if (event == EV_M || event == EV_D) feature_bp_right--;
        }
        while (ev > cigar_start && s.ev_readc[ev] == U16_NONE) ev--;
        if (ev < ev_feature_start) continue;
        u32 read_start = s.ev_readc[ev_feature_start];
        u32 read_end = s.ev_readc[ev];
        if ((read_start < w.x && read_end < w.x) || (read_start > w.y && read_end > w.y)) continue;
        read_start = std::max<u32>(read_start, w.x);
        read_start = std::min<u32>(read_start, w.y);
        read_end = std::max<u32>(read_end, w.x);
        read_end = std::min<u32>(read_end, w.y);
        for (u32 dead_bp = read_start; dead_bp <= read_end; dead_bp++) s.active_loc[rs + dead_bp] = 0;
    }
}

// compute_hmm_windows (device/baq.cu:89-187). Returns false when the read needs BAQ but its HMM window
// runs past the contig end; the caller then removes the read.
bool hmm_window(const fpo_ctx *ctx, BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    const bool read_needs_baq = s.num_errors[r] != 0;
    const us2 w = s.clipped[r], ni = s.no_ins[r], rw = s.refwin[r];
    const int offset = MIN_BAND_WIDTH / 2;
    const bool left_clip = (w.x != 0);
    const bool right_clip = (w.y != u16(b->read_len[r] - 1));
    const i16 left_insertion = i16(left_clip ? 0 : int(ni.x) - int(w.x));
    const i16 right_insertion = i16(right_clip ? 0 : int(w.y) - int(ni.y));
    ss2 hw;
    hw.x = i16(int(rw.x) - left_insertion - offset);
    hw.y = i16(int(rw.y) + right_insertion + offset);
    const u64 csize = contig_size(ctx, b->chromosome[r]);
    int left_window_shift = 0;
    if (hw.x < 0 && b->alignment_start[r] < baq_abs(hw.x)) left_window_shift = -1;
    if (read_needs_baq && u32(b->alignment_start[r] + u32(int(hw.y)) + u32(left_window_shift)) >= u32(csize)) {
        s.hmm_window[r] = ss2{-1, -1};
        return false;
    }
    s.hmm_window[r] = hw;
    int referenceLen = hw.y - hw.x + 1;
    int queryLen = w.y - w.x + 1;
    u16 bandWidth = u16(std::max(referenceLen, queryLen));
    if (u32(MIN_BAND_WIDTH) < baq_abs(referenceLen - queryLen)) bandWidth = u16(baq_abs(referenceLen - queryLen) + 3);
    if (bandWidth > MIN_BAND_WIDTH) bandWidth = MIN_BAND_WIDTH;
    if (bandWidth < baq_abs(referenceLen - queryLen)) bandWidth = u16(baq_abs(referenceLen - queryLen));
    s.bandwidth[r] = bandWidth;
    return true;
}

// hmm_glocal setup (device/baq.cu:247-334) + the HMM for one read
void baq_read(const fpo_ctx *ctx, BatchState &s, u32 r, HmmScratch &scratch) {
    const fp_batch_view *b = s.b;
    const ss2 hw = s.hmm_window[r];
    const us2 w = s.clipped[r];
    int referenceLength = hw.y - hw.x + 1;
    const int bm_reference_length = referenceLength;
    const int queryStart = w.x;
    const int queryLen = w.y - w.x + 1;
    u32 hmm_reference_offset;
    if (hw.x < 0 && b->alignment_start[r] < baq_abs(hw.x)) {
        hmm_reference_offset = 0;
        referenceLength--;
    } else {
        hmm_reference_offset = b->alignment_start[r] + u32(int(hw.x));
    }
    const Contig *g = contig_of(ctx, b->chromosome[r]);
    std::vector<u8> ref(std::max(referenceLength, 0) + 1), query(queryLen), qual(queryLen);
    for (int k = 0; k < referenceLength; k++) ref[k] = g->at(u64(hmm_reference_offset) + k);
    for (int i = 0; i < queryLen; i++) {
        query[i] = s.read_sym(u64(b->read_start[r]) + queryStart + i);
        qual[i] = b->qualities[b->qual_start[r] + queryStart + i];
    }
    hmm_glocal(ref.data(), referenceLength, bm_reference_length, query.data(), qual.data(), queryLen, s.bandwidth[r],
               ctx->qual2prob, ctx->gap_open, &s.baq[b->qual_start[r] + queryStart],
               &s.baq_state[b->qual_start[r] + queryStart], scratch);
}

// cap_baq_qualities (device/baq.cu:870-1056)
bool cap_baq(BatchState &s, u32 r, u32 cs, u32 ce, u32 baq_start, bool update) {
    const fp_batch_view *b = s.b;
    const us2 w = s.clipped[r], rw = s.refwin[r];
    const ss2 hw = s.hmm_window[r];
    const u32 qs = b->qual_start[r];
    u32 readI = 0, refI = 0, numD = 0;
    i16 reference_shift, read_shift;
    if (hw.x < 0 && b->alignment_start[r] < baq_abs(hw.x)) {
        reference_shift = i16(baq_abs(hw.x));
        read_shift = i16(b->alignment_start[r]);
    } else {
        reference_shift = 0;
        read_shift = 0;
    }
    const i16 refOffset = i16(int(hw.x) - int(rw.x) + int(reference_shift));
    for (u32 i = baq_start; i < ce - cs; i++) {
        const u16 read_bp_idx = s.ev_readc[cs + i];
        const u32 qual_idx = qs + read_bp_idx;
        if (read_bp_idx != U16_NONE) {
            if (read_bp_idx < w.x) continue;
            if (read_bp_idx > w.y) break;
        }
        switch (s.ev_type[cs + i]) {
        case EV_S:
            refI++;
            break;
        case EV_I:
            if (update) s.baq[qual_idx] = b->qualities[qual_idx];
            readI++;
            break;
        case EV_D:
            refI++;
            numD++;
            break;
        case EV_M:
            if (update) {
                const u32 expectedPos = refI - u32(int(refOffset)) + (i - numD - baq_start - readI) + u32(int(read_shift));
                const u8 oq = b->qualities[qs + read_bp_idx];
                const u8 bq = s.baq[qs + read_bp_idx];
                const u32 state = s.baq_state[qs + read_bp_idx];
                const bool isIndel = (state & 3) != 0;
                const u32 pos = state >> 2;
                s.baq[qual_idx] = (isIndel || pos != expectedPos) ? u8(MIN_BASE_QUAL) : std::min(bq, oq);
            }
            readI++;
            refI++;
            break;
        }
    }
    if (!update) {
        const u32 read_len = u32(w.y - w.x + 1);
        if (readI != read_len) return false;
    }
    return true;
}

void cap_and_recode(BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    const u32 cs = s.cigar_offsets[b->cigar_start[r]];
    const u32 ce = s.cigar_offsets[b->cigar_start[r] + b->cigar_len[r]];
    const us2 w = s.clipped[r];
    u32 baq_start = 0;
    for (u32 i = 0; i < ce - cs; i++) {
        const u16 rb = s.ev_readc[cs + i];
        if (rb != U16_NONE && rb >= w.x) {
            baq_start = i;
            break;
        }
    }
    if (cap_baq(s, r, cs, ce, baq_start, false)) {
        cap_baq(s, r, cs, ce, baq_start, true);
    } else {
        const u32 base_off = b->qual_start[r] + w.x;
        const u32 len = u32(w.y - w.x + 1);
        memcpy(&s.baq[base_off], &b->qualities[base_off], len);
    }
    // recode_baq_qualities (device/baq.cu:1058-1081)
    for (u32 i = b->qual_start[r]; i < b->qual_start[r] + b->qual_len[r]; i++) {
        const u8 baq_i = s.baq[i];
        if (baq_i == 0xFF) continue;
        const u8 bq = u8(b->qualities[i] + 64);
        s.baq[i] = u8(bq - baq_i);
    }
}

// compute_fractional_errors (device/fractional_errors.cu:39-117) for one error vector
void fractional_errors(BatchState &s, u32 r, const std::vector<u8> &errvec, std::vector<double> &out) {
    const fp_batch_view *b = s.b;
    const us2 w = s.clipped[r];
    const u8 *baqArray = &s.baq[b->qual_start[r] + w.x];
    const u8 *errorArray = &errvec[b->read_start[r] + w.x];
    double *fe = &out[b->qual_start[r] + w.x];
    const int n = w.y - w.x + 1;
    auto block = [&](int iii, int blockStartIndex) {
        int totalErrors = 0;
        for (int j = std::max(0, blockStartIndex - 1); j <= iii; j++) totalErrors += errorArray[j];
        for (int j = std::max(0, blockStartIndex - 1); j <= iii; j++)
            fe[j] = double(totalErrors) / double(iii - std::max(0, blockStartIndex - 1) + 1);
    };
    bool inBlock = false;
    int blockStartIndex = -1;
    int iii;
    for (iii = 0; iii < n; iii++) {
        if (baqArray[iii] == 64) {
            if (!inBlock) {
                fe[iii] = double(errorArray[iii]);
            } else {
                block(iii, blockStartIndex);
                inBlock = false;
                blockStartIndex = -1;
            }
        } else {
            inBlock = true;
            if (blockStartIndex == -1) blockStartIndex = iii;
        }
    }
    if (inBlock) block(iii - 1, blockStartIndex);
}

// compute_high_quality_windows (device/covariates.cu:215-246)
void high_quality_window(BatchState &s, u32 r) {
    const fp_batch_view *b = s.b;
    const u8 *q = &b->qualities[b->qual_start[r]];
    us2 w = s.clipped[r];
    while (q[w.x] <= 2 && w.x < w.y) w.x++;
    while (q[w.y] <= 2 && w.y > w.x) w.y--;
    s.hq[r] = w;
}

// covariate_Context::encode (device/covariates/bit_packers/context.h:106-174); returns {mismatch, indel}
void context_covariate(const BatchState &s, u32 r, u16 bp_offset, u32 &ctx_mismatch, u32 &ctx_indel) {
    const fp_batch_view *b = s.b;
    const us2 window = s.hq[r];
    const bool negative_strand = b->flags[r] & F_REVERSE;
    u32 context = 0;
    ctx_mismatch = CONTEXT_INVALID;
    ctx_indel = CONTEXT_INVALID;
    const int direction = negative_strand ? 1 : -1;
    const int context_bases = negative_strand ? std::min<int>(int(window.y) - int(bp_offset) + 1, 3)
                                              : std::min<int>(int(bp_offset) - int(window.x) + 1, 3);
    const int start_offset = bp_offset;
    const int stop_offset = bp_offset + context_bases * direction;
    if (context_bases >= 2) {
        int num_bases = 0;
        for (int i = start_offset; i != stop_offset; i += direction) {
            const u8 bp = s.read_sym(u64(b->read_start[r]) + u32(i));
            if (bp != IUPAC_A && bp != IUPAC_C && bp != IUPAC_T && bp != IUPAC_G) break;
            context <<= 2;
            context |= u32(31 - __builtin_clz(u32(bp)));  // iupac16_to_dna (device/from_nvbio/dna.h:58-67)
            num_bases++;
        }
        if (negative_strand) context = ~context & ((1u << (num_bases * 2)) - 1);
        if (num_bases >= 2) ctx_mismatch = ((context >> (num_bases - 2) * 2) << 4) | 2;
        if (num_bases >= 3) ctx_indel = ((context >> (num_bases - 3) * 2) << 4) | 3;
    }
}

// covariate_Cycle_Illumina::encode (device/covariates/bit_packers/cycle_illumina.h:46-95)
void cycle_covariate(const BatchState &s, u32 r, u16 bp_offset, u32 &sub_key, u32 &indel_key) {
    const fp_batch_view *b = s.b;
    const u32 flags = b->flags[r];
    const bool paired = flags & F_PAIRED;
    const bool second_of_pair = flags & F_READ2;
    const bool negative_strand = flags & F_REVERSE;
    const us2 window = s.clipped[r];
    const int readLength = window.y - window.x + 1;
    const int readOrderFactor = (paired && second_of_pair) ? -1 : 1;
    const int i = int(bp_offset) - int(window.x);
    int cycle, increment;
    if (negative_strand) {
        cycle = readLength * readOrderFactor;
        increment = -1 * readOrderFactor;
    } else {
        cycle = readOrderFactor;
        increment = readOrderFactor;
    }
    cycle += i * increment;
    const int MAX_CYCLE_FOR_INDELS = readLength - 4 - 1;
    u32 result = u32(cycle < 0 ? -cycle : cycle);
    result = result << 1;
    if (cycle < 0) result++;
    sub_key = result;
    indel_key = (i < 4 || i > MAX_CYCLE_FOR_INDELS) ? CYCLE_INVALID : sub_key;
}

// covariate_gatherer for one event (device/covariates.cu:50-103) into the three tables' entry streams
void gather_event(const BatchState &s, u32 e, std::vector<Entry> *outq, std::vector<Entry> *outc,
                  std::vector<Entry> *outx) {
    const fp_batch_view *b = s.b;
    const u32 r = s.ev_read_index[e];
    if (r == U32_NONE) return;
    const u16 off = s.ev_readc[e];
    if (off == U16_NONE) return;
    if (off < s.clipped[r].x || off > s.clipped[r].y) return;
    if (s.active_loc[b->read_start[r] + off] == 0) return;
    if (s.ev_type[e] == EV_S) return;
    const u32 rg = b->read_group[r];
    const u32 q = b->qualities[b->qual_start[r] + off];
    const u32 qi = b->qual_start[r] + off;
    const float mm[3] = {float(s.frac[0][qi]), float(s.frac[1][qi]), float(s.frac[2][qi])};
    const u32 qs[3] = {q, 45, 45};
    // RecalTable1 (packer_quality_score.h:41-44): no sparse covariate, every key is valid
    for (u32 ev = 0; ev < 3; ev++) outq->push_back(Entry{(rg << 10) | (qs[ev] << 2) | ev, mm[ev]});
    // cycle (packer_cycle_illumina.h:41-45)
    u32 sub_key, indel_key;
    cycle_covariate(s, r, off, sub_key, indel_key);
    const u32 cyc[3] = {sub_key, indel_key, indel_key};
    for (u32 ev = 0; ev < 3; ev++) {
        if (cyc[ev] == CYCLE_INVALID) continue;  // is_key_valid (device/covariates.cu:105-122)
        outc->push_back(Entry{(rg << 20) | (qs[ev] << 12) | (cyc[ev] << 2) | ev, mm[ev]});
    }
    // context (packer_context.h:54-58)
    u32 cm, ci;
    context_covariate(s, r, off, cm, ci);
    const u32 ctxv[3] = {cm, ci, ci};
    for (u32 ev = 0; ev < 3; ev++) {
        if (ctxv[ev] == CONTEXT_INVALID) continue;
        outx->push_back(Entry{(rg << 21) | (qs[ev] << 13) | (ctxv[ev] << 2) | ev, mm[ev]});
    }
}

// Thread-seconds per stage: lap(k) charges the time since the previous lap (or start) to stage k.
struct StageClock {
    double sec[FPO_NUM_STAGES] = {};
    double last = 0.0;
    void start() { last = omp_get_wtime(); }
    void lap(int k) {
        const double now = omp_get_wtime();
        sec[k] += now - last;
        last = now;
    }
};

int resolve_threads(int n) {
#ifdef _OPENMP
    return n > 0 ? n : omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

}  // namespace

extern "C" {

fpo_ctx *fpo_create(uint32_t num_read_groups) {
    fpo_ctx *c = new fpo_ctx();
    c->num_read_groups = num_read_groups;
    // qual2prob (device/baq.cu:355-359) and GAP_OPEN_PROBABILITY (:80)
    for (int q = 0; q < 256; q++) c->qual2prob[q] = pow(10.0, -q / 10.0);
    c->gap_open = pow(10.0, (-40.0) / 10.);
    return c;
}

void fpo_destroy(fpo_ctx *c) { delete c; }

int fpo_set_contig(fpo_ctx *c, uint32_t id, const uint32_t *packed4, uint64_t n) {
    if (id >= c->contigs.size()) c->contigs.resize(id + 1);
    Contig &g = c->contigs[id];
    g.size = n;
    g.words.assign(packed4, packed4 + (n + 7) / 8);
    // clear symbols past the end inside the last word (they read as 0)
    if (n % 8) g.words.back() &= (1u << ((n % 8) * 4)) - 1;
    return 0;
}

int fpo_set_known_sites(fpo_ctx *c, uint32_t id, const uint32_t *start, const uint32_t *stop, uint32_t n) {
    if (id >= c->sites.size()) c->sites.resize(id + 1);
    KnownSites &k = c->sites[id];
    k.feature_start.assign(start, start + n);
    k.feature_stop.assign(stop, stop + n);
    k.max_end_point_left.resize(n);
    u32 m = 0;
    for (u32 i = 0; i < n; i++) {  // inclusive max-scan (loader/variants.cu:126-134)
        m = (i == 0) ? stop[0] : std::max(m, stop[i]);
        k.max_end_point_left[i] = m;
    }
    return 0;
}

int fpo_process_batch(fpo_ctx *ctx, const fp_batch_view *b, int num_threads) {
    const int nt = resolve_threads(num_threads);
    BatchState s;
    s.b = b;
    s.R = b->num_reads;
    const u32 R = s.R;
    for (u32 r = 0; r < R; r++)
        if (b->read_len[r] > 511) return 1;  // cycle keys have 10 bits (cycle_illumina.h:38)

    s.status.assign(R, 0);
    // start_batch (device/firepony_context.cu:43-60): all bases active
    s.active_loc.assign(b->num_read_symbols, 1);
    s.is_snp.assign(b->num_read_symbols, 0);
    s.is_ins.assign(b->num_read_symbols, 0);
    s.is_del.assign(b->num_read_symbols, 0);
    s.alignment_window_x.assign(R, 0);
    s.alignment_window_y.assign(R, 0);
    s.clipped.assign(R, us2{0, 0});
    s.no_ins.assign(R, us2{U16_NONE, U16_NONE});
    s.refwin.assign(R, us2{U16_NONE, U16_NONE});
    s.hq.assign(R, us2{0, 0});
    s.num_errors.assign(R, 0);
    s.hmm_window.assign(R, ss2{0, 0});
    s.bandwidth.assign(R, 0);
    s.baq.assign(b->num_qualities, 0xFF);
    s.baq_state.assign(b->num_qualities, U32_NONE);
    for (int t = 0; t < 3; t++) s.frac[t].assign(b->num_qualities, 0.0);

    u64 filtered = 0;
    // per-thread stage clocks, merged into ctx->stage_sec at the end of each parallel region
    std::vector<StageClock> clocks(static_cast<size_t>(nt));
    // filter_invalid_reads (device/read_filters.cu:262-336)
#pragma omp parallel num_threads(nt)
    {
        StageClock &ck = clocks[size_t(omp_get_thread_num())];
        ck.start();
#pragma omp for schedule(static) reduction(+ : filtered)
        for (u32 r = 0; r < R; r++) {
            if (passes_invalid_filters(s, r)) {
                s.status[r] = 1;
            } else {
                filtered++;
            }
        }
        // build_read_offset_list / build_alignment_windows / filter_malformed_reads (device/pipeline.cu:72-80)
#pragma omp for schedule(dynamic, 256) reduction(+ : filtered)
        for (u32 r = 0; r < R; r++) {
            if (!s.status[r]) continue;
            alignment_window(s, r);
            if (!passes_malformed_filter(ctx, s, r)) {
                s.status[r] = 0;
                filtered++;
            }
        }
        ck.lap(FPO_STAGE_READ_FILTER);
    }

    // expand_cigars (device/cigar.cu:815-935)
    s.cigar_offsets.assign(size_t(b->num_cigar_ops) + 1, 0);
    for (u32 i = 0; i < b->num_cigar_ops; i++) s.cigar_offsets[i + 1] = s.cigar_offsets[i] + op_len(b->cigars[i]);
    const u32 E = s.cigar_offsets[b->num_cigar_ops];
    s.ev_type.assign(E, EV_M);
    s.ev_readc.assign(E, U16_NONE);
    s.ev_refc.assign(E, U16_NONE);
    s.ev_read_index.assign(E, U32_NONE);

    u64 baq_count = 0;
#pragma omp parallel num_threads(nt)
    {
        HmmScratch scratch;
        StageClock &ck = clocks[size_t(omp_get_thread_num())];
        ck.start();
#pragma omp for schedule(dynamic, 64)
        for (u32 r = 0; r < R; r++) {
            if (!s.status[r]) continue;
            expand_read(s, r);
        }
        ck.lap(FPO_STAGE_CIGAR_EXPANSION);
#pragma omp for schedule(dynamic, 64)
        for (u32 r = 0; r < R; r++) {
            if (!s.status[r]) continue;
            s.clipped[r] = us2{0, u16(b->read_len[r] - 1)};  // read_window_init (:97-109)
            AdapterClip(s, r).run();
            remove_soft_clips(s, r);
            no_insertions_window(s, r);
            reference_window(s, r);
            error_vectors(ctx, s, r);
            ck.lap(FPO_STAGE_CIGAR_EXPANSION);
            filter_bases(s, r);
            ck.lap(FPO_STAGE_BP_FILTER);
            filter_known_sites(ctx, s, r);
            ck.lap(FPO_STAGE_SNP_FILTER);
            // baq_reads (device/baq.cu:1083-1336): windows for all active reads; reads needing BAQ whose
            // window leaves the contig lose their events. (Whether the batch filters them out of the
            // active list depends on other reads, but with their events cleared they contribute nothing.)
            if (!hmm_window(ctx, s, r)) {
                s.status[r] = 2;
                const u32 cs = s.cigar_offsets[b->cigar_start[r]];
                const u32 ce = s.cigar_offsets[b->cigar_start[r] + b->cigar_len[r]];
                for (u32 i = cs; i < ce; i++) {
                    s.ev_read_index[i] = U32_NONE;
                    s.ev_readc[i] = U16_NONE;
                }
            }
            ck.lap(FPO_STAGE_BAQ_SETUP);
        }
        ck.lap(FPO_STAGE_CIGAR_EXPANSION);  // (waiting at the loop's barrier)
#pragma omp for schedule(dynamic, 16) reduction(+ : baq_count)
        for (u32 r = 0; r < R; r++) {
            if (s.status[r] != 1) continue;
            const us2 w = s.clipped[r];
            if (s.num_errors[r] != 0) {
                baq_read(ctx, s, r, scratch);
                ck.lap(FPO_STAGE_BAQ_HMM);
                cap_and_recode(s, r);
                baq_count++;
            } else {
                // read_flat_baq (:842-868)
                memset(&s.baq[b->qual_start[r] + w.x], 64, u32(w.y - w.x + 1));
            }
            ck.lap(FPO_STAGE_BAQ_POST);
            // build_fractional_error_arrays (device/fractional_errors.cu:119-141)
            fractional_errors(s, r, s.is_snp, s.frac[0]);
            fractional_errors(s, r, s.is_ins, s.frac[1]);
            fractional_errors(s, r, s.is_del, s.frac[2]);
            ck.lap(FPO_STAGE_FRACTIONAL_ERROR);
            high_quality_window(s, r);
            ck.lap(FPO_STAGE_COVARIATES_GATHER);
        }
        ck.lap(FPO_STAGE_BAQ_HMM);  // (waiting at the loop's barrier)
    }

    // gather_covariates (device/covariates.cu:248-262): events in stream order into the three tables.
    // Reads are split into contiguous chunks; each chunk's entries keep stream order and chunks are
    // concatenated in order, so the result is independent of the thread count.
    // per-chunk entry streams, kept in the context so their memory is reused from batch to batch
    std::vector<std::vector<Entry>> &cq = ctx->run_q, &cc = ctx->run_c, &cx = ctx->run_x;
    for (auto *v : {&cq, &cc, &cx}) {
        v->resize(size_t(nt));
        for (auto &run : *v) run.clear();
    }
    std::vector<u32> chunk_start(nt + 1);
    for (int t = 0; t <= nt; t++) chunk_start[t] = u32(u64(R) * t / nt);
#pragma omp parallel num_threads(nt)
    {
        StageClock &ck = clocks[size_t(omp_get_thread_num())];
        ck.start();
#pragma omp for schedule(static, 1)
        for (int t = 0; t < nt; t++) {
            // the streams are filled through vectors on this thread's stack (the shared array of vector
            // headers would put every append of neighbouring chunks on one cache line)
            std::vector<Entry> lq, lc, lx;
            lq.swap(cq[t]);
            lc.swap(cc[t]);
            lx.swap(cx[t]);
            for (u32 r = chunk_start[t]; r < chunk_start[t + 1]; r++) {
                if (s.status[r] != 1) continue;
                const u32 cs = s.cigar_offsets[b->cigar_start[r]];
                const u32 ce = s.cigar_offsets[b->cigar_start[r] + b->cigar_len[r]];
                for (u32 e = cs; e < ce; e++) gather_event(s, e, &lq, &lc, &lx);
            }
            lq.swap(cq[t]);
            lc.swap(cc[t]);
            lx.swap(cx[t]);
        }
        ck.lap(FPO_STAGE_COVARIATES_GATHER);
    }
    // The three tables' entry streams are stable-sorted in parallel: each chunk's run is sorted on its own
    // thread, then runs are merged pairwise in chunk order (std::merge keeps equal keys of the earlier run
    // first), which is the order a stable sort of the concatenation gives. The tables then fold side by side.
    {
        const double t0 = omp_get_wtime();
        std::vector<std::vector<Entry>> *parts[3] = {&cq, &cc, &cx};
        auto by_key = [](const Entry &a, const Entry &b) { return a.key < b.key; };
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1) collapse(2)
        for (int tab = 0; tab < 3; tab++)
            for (int t = 0; t < nt; t++) std::stable_sort((*parts[tab])[t].begin(), (*parts[tab])[t].end(), by_key);
        for (int width = 1; width < nt; width *= 2) {
            const int pairs = (nt + 2 * width - 1) / (2 * width);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1) collapse(2)
            for (int tab = 0; tab < 3; tab++) {
                for (int pi = 0; pi < pairs; pi++) {
                    const int a = pi * 2 * width, b2 = a + width;
                    if (b2 >= nt) continue;
                    std::vector<Entry> &ra = (*parts[tab])[a], &rb = (*parts[tab])[b2];
                    std::vector<Entry> m(ra.size() + rb.size());
                    std::merge(ra.begin(), ra.end(), rb.begin(), rb.end(), m.begin(), by_key);
                    ra.swap(m);
                    rb.clear();
                }
            }
        }
        ObsTable *tabs[3] = {&ctx->quality, &ctx->cycle, &ctx->context};
        for (int tab = 0; tab < 3; tab++) tabs[tab]->fold_sorted((*parts[tab])[0], nt);
        ctx->stage_sec[FPO_STAGE_COVARIATES_SORT_PACK] += omp_get_wtime() - t0;
    }
    for (const StageClock &ck : clocks)
        for (int k = 0; k < FPO_NUM_STAGES; k++) ctx->stage_sec[k] += ck.sec[k];

    ctx->total_reads += R;
    ctx->filtered_reads += filtered;
    ctx->baq_reads += baq_count;
    ctx->num_batches++;

    // keep intermediates for per-stage parity tests
    ctx->dbg_status = s.status;
    ctx->dbg_windows.assign(size_t(R) * 8, 0);
    ctx->dbg_hmm.assign(size_t(R) * 4, 0);
    for (u32 r = 0; r < R; r++) {
        u16 *w = &ctx->dbg_windows[size_t(r) * 8];
        w[0] = s.clipped[r].x; w[1] = s.clipped[r].y;
        w[2] = s.no_ins[r].x; w[3] = s.no_ins[r].y;
        w[4] = s.refwin[r].x; w[5] = s.refwin[r].y;
        w[6] = s.hq[r].x; w[7] = s.hq[r].y;
        i16 *h = &ctx->dbg_hmm[size_t(r) * 4];
        h[0] = s.hmm_window[r].x; h[1] = s.hmm_window[r].y;
        h[2] = i16(s.bandwidth[r]); h[3] = i16(s.num_errors[r]);
    }
    ctx->dbg_num_quals = b->num_qualities;
    ctx->dbg_flags.assign(b->num_qualities, 0);
    for (u32 r = 0; r < R; r++) {
        for (u32 i = 0; i < b->read_len[r] && i < b->qual_len[r]; i++) {
            const u64 rsym = u64(b->read_start[r]) + i;
            ctx->dbg_flags[b->qual_start[r] + i] = u8(s.is_snp[rsym] | (s.is_ins[rsym] << 1) | (s.is_del[rsym] << 2) |
                                                      (s.active_loc[rsym] << 3));
        }
    }
    ctx->dbg_baq = s.baq;
    ctx->dbg_frac.assign(b->num_qualities * 3, 0.0);
    for (u64 i = 0; i < b->num_qualities; i++)
        for (int t = 0; t < 3; t++) ctx->dbg_frac[i * 3 + t] = s.frac[t][i];
    return 0;
}

int fpo_debug_last_batch(fpo_ctx *c, uint8_t *read_status, uint16_t *windows, int16_t *hmm, uint8_t *base_flags,
                         uint8_t *baq_tag, double *frac_errors) {
    if (read_status) memcpy(read_status, c->dbg_status.data(), c->dbg_status.size());
    if (windows) memcpy(windows, c->dbg_windows.data(), c->dbg_windows.size() * 2);
    if (hmm) memcpy(hmm, c->dbg_hmm.data(), c->dbg_hmm.size() * 2);
    if (base_flags) memcpy(base_flags, c->dbg_flags.data(), c->dbg_flags.size());
    if (baq_tag) memcpy(baq_tag, c->dbg_baq.data(), c->dbg_baq.size());
    if (frac_errors) memcpy(frac_errors, c->dbg_frac.data(), c->dbg_frac.size() * 8);
    return 0;
}

// firepony_postprocess compute part (device/pipeline.cu:206-216): postprocess_covariates is a no-op on a
// single device's already reduced tables; build_read_group_table (device/read_group_table.cu:47-94);
// compute_empirical_quality_scores (device/covariates.cu:314-340).
int fpo_finalize(fpo_ctx *c) {
    const double t_start = omp_get_wtime();
    ObsTable *obs[4] = {nullptr, &c->quality, &c->cycle, &c->context};
    const int qshift[4] = {2, 2, 12, 13};
    for (int t = 1; t < 4; t++) {
        auto &emp = c->emp[t];
        emp.clear();
        for (const TableRow &row : obs[t]->rows) {
            EmpiricalRow e;
            e.key = row.key;
            e.observations = row.observations;
            e.mismatches = double(row.mismatches);
            const u8 q = u8((row.key >> qshift[t]) & 0xFF);
            e.expected_errors = double(row.observations) * qualToErrorProb(q);
            e.estimated_quality = 0.0;
            e.empirical_quality = 0.0;
            emp.push_back(e);
        }
    }
    // RecalTable0: quality-table rows with the quality bits masked, stable-sorted, FP64 left fold
    {
        std::vector<EmpiricalRow> rows = c->emp[1];
        for (auto &r : rows) r.key &= ~(0xFFu << 2);
        std::stable_sort(rows.begin(), rows.end(), [](const EmpiricalRow &a, const EmpiricalRow &b) { return a.key < b.key; });
        std::vector<EmpiricalRow> out;
        for (const auto &r : rows) {
            if (!out.empty() && out.back().key == r.key) {
                EmpiricalRow &a = out.back();
                a.observations += r.observations;
                a.mismatches = a.mismatches + r.mismatches;
                a.expected_errors = a.expected_errors + r.expected_errors;
            } else {
                EmpiricalRow n = r;
                n.estimated_quality = 0.0;
                n.empirical_quality = 0.0;
                out.push_back(n);
            }
        }
        for (auto &r : out) compute_empirical(r, false);
        c->emp[0] = out;
    }
    for (int t = 1; t < 4; t++)
        for (auto &r : c->emp[t]) compute_empirical(r, true);
    for (int t = 0; t < 4; t++) {
        // table id order in fp_table_id: 0 RG, 1 quality, 2 cycle, 3 context
        auto &emp = c->emp[t];
        c->out_keys[t].clear(); c->out_obs[t].clear(); c->out_mism[t].clear();
        c->out_exp[t].clear(); c->out_est[t].clear(); c->out_emp[t].clear();
        for (auto &r : emp) {
            c->out_keys[t].push_back(r.key);
            c->out_obs[t].push_back(r.observations);
            c->out_mism[t].push_back(r.mismatches);
            c->out_exp[t].push_back(r.expected_errors);
            c->out_est[t].push_back(r.estimated_quality);
            c->out_emp[t].push_back(r.empirical_quality);
        }
    }
    c->stage_sec[FPO_STAGE_POSTPROCESS] += omp_get_wtime() - t_start;
    return 0;
}

void fpo_get_stage_seconds(const fpo_ctx *c, double out[FPO_NUM_STAGES]) {
    for (int k = 0; k < FPO_NUM_STAGES; k++) out[k] = c->stage_sec[k];
}

int fpo_get_table(fpo_ctx *c, int32_t t, fp_table_view *out) {
    if (t < 0 || t > 3) return 1;
    out->num_rows = u32(c->out_keys[t].size());
    out->keys = c->out_keys[t].data();
    out->observations = c->out_obs[t].data();
    out->mismatches = c->out_mism[t].data();
    out->expected_errors = c->out_exp[t].data();
    out->estimated_quality = c->out_est[t].data();
    out->empirical_quality = c->out_emp[t].data();
    return 0;
}

void fpo_get_stats(const fpo_ctx *c, uint64_t out[4]) {
    out[0] = c->total_reads;
    out[1] = c->filtered_reads;
    out[2] = c->baq_reads;
    out[3] = c->num_batches;
}

void fpo_kat_hmm(const uint8_t *ref, int ref_len, int bm_ref_len, const uint8_t *query, const uint8_t *qual,
                 int query_len, int band_width, uint8_t *out_qual, uint32_t *out_state) {
    double q2p[256];
    for (int q = 0; q < 256; q++) q2p[q] = pow(10.0, -q / 10.0);
    HmmScratch s;
    hmm_glocal(ref, ref_len, bm_ref_len, query, qual, query_len, band_width, q2p, pow(10.0, (-40.0) / 10.), out_qual,
               out_state, s);
}

double fpo_kat_empirical_quality(uint64_t observations, double mismatches, double estimated_quality, int need_rounding) {
    return calcEmpiricalQuality(observations, mismatches, estimated_quality, need_rounding != 0);
}

int fpo_kat_baq_quality_from_max(double max) {
    int kq = saturating_int(double(-4.343) * log(double(1.0) - double(max)) + double(.499));
    return kq > 100 ? 99 : (kq < MIN_BASE_QUAL ? MIN_BASE_QUAL : kq);
}

}  // extern "C"
