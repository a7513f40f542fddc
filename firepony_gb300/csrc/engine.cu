// fp_engine: the C ABI of include/firepony_gb300.h. Owns the device-resident reference, known sites and
// covariate tables, runs the per-batch kernel sequence on one CUDA stream and finalizes the tables.
//
// Per batch (replacing batch->download + firepony_process_batch, device/pipeline_interface.cu:206-220 and
// device/pipeline.cu:56-147):
//   H2D inputs -> validate + CIGAR-length scan -> [sync: errors, event count]
//   -> K1 prep (filters, CIGAR expansion, windows, error vectors, base/known-site masks, BAQ work lists)
//   -> [sync: work-list sizes] -> K2 BAQ (FP32 with FP64 escalation, or plain FP64) + cap/recode
//   -> K3 count (observations, entry counts) -> scan -> [sync: entry count]
//   -> K3 emit -> K4 stable radix sort + ordered fold into the resident mismatch table.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "firepony_gb300.h"
#include "firepony_gb300_store.h"
#include "kernels.h"
#include "refstore_internal.h"

using namespace fpg;

extern "C" fp_status fp_report_write(const char *path, const fp_table_view *tables, const char *const *rg_names,
                                     uint32_t num_rg_names, int disable_rounding, int vmaj, int vmin, int vrev);

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = bytes + bytes / 4 + 256;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
};

struct HostTable {
    std::vector<uint32_t> keys;
    std::vector<uint64_t> obs;
    std::vector<double> mism, exp, est, emp;
};

double log10_factorial(uint64_t x) { return double(lgammaf(float(double(x + 1)))) * log10(M_E); }

// log10BinomialCoefficient of the (capped) row counts (device/empirical_quality.cu:77-112, :165-174)
double binomial_coef(uint64_t observations, double mismatches) {
    uint64_t k = uint64_t(mismatches + 0.5) + 1;
    uint64_t n = observations + 1 + 1;
    const uint32_t MAXOBS = 2147483647u - 1;
    if (n > MAXOBS) {
        const double fraction = double(MAXOBS) / double(n);
        k = uint64_t(round(double(k) * fraction));
        n = MAXOBS;
    }
    return log10_factorial(n) - log10_factorial(k) - log10_factorial(n - k);
}

double gaussian(double value) {  // device/empirical_quality.cu:43-53
    const double a = 0.0, b = 0.9, c = 0.0, d = 0.5;
    return a + b * pow(double(M_E), -(pow(value - c, 2.0) / (2 * d * d)));
}

}  // namespace

struct fp_engine {
    int device = 0;
    int baq_mode = FP_BAQ_FP32;
    u32 replay_rpw = 0;  // FP64 replay: 0 = warp-cooperative kernel, 1..32 = thread-per-read, reads per warp
    u32 flags = 0;       // FP_FLAG_*
    uint32_t n_rg = 1;
    cudaStream_t st = nullptr;
    cudaStream_t st2 = nullptr;          // band-class-1 BAQ, concurrent with class 0
    cudaStream_t st3 = nullptr;          // first covariate count pass, concurrent with the FP64 replays
    // sort + ordered fold of a batch's entries: in batch order on its own stream, beside the next batch's
    // copies and preparation. fold_end marks the last queued fold; its timing is read once it has finished.
    cudaStream_t st_fold = nullptr;
    cudaEvent_t fold_start = nullptr, fold_end = nullptr;
    bool fold_pending = false;
    cudaEvent_t fork = nullptr, join = nullptr, cov1_done = nullptr;
    std::string err;
    bool finalized = false;

    // resident reference and known sites
    std::vector<DevContig> h_contigs;
    std::vector<DevBuf> contig_bufs;
    DevBuf d_contigs;
    std::vector<DevSites> h_sites;
    std::vector<DevBuf> site_bufs;
    DevBuf d_sites;
    DevRef ref{};
    fp_refstore *store = nullptr;  // when set, `ref` is the store's device copy and the buffers above are empty

    // tables
    Tables tables{};
    DevBuf tab_obs, tab_mism, tab_stage, tab_cyc;
    u64 staged_bases = 0;  // bases counted into the u32 stage since the last merge

    // batch buffers
    // two device input buffers: a batch prefetched on the copy stream fills one while the other is in use
    DevBuf in_bufs[2];
    int in_state[2] = {0, 0};  // 0 free, 1 holds a prefetched batch, 2 in use by a submit
    const void *in_src[2][17] = {};
    uint64_t in_counts[2][4] = {};
    cudaEvent_t in_ev[2] = {nullptr, nullptr};
    cudaStream_t st_copy = nullptr;
    std::mutex in_mu;
    // coalescing of small host batches (fp_options.coalesce_reads): a device staging batch of 17 arrays
    u32 co_target = 0;
    DevBuf co_buf;
    size_t co_off[17] = {};
    u64 co_cap[4] = {};  // capacity: reads, cigar ops, read words, qualities
    u64 co_n[4] = {};    // staged
    DevBatch batch{};
    DevBuf oplen, cigoff, ev_rc, ev_type, per_read, per_base, lists, counters, entry_cnt, entry_off;
    DevBuf entries, entries_alt, sort_tmp, scan_tmp, s32, s32b, s64, s32w;  // s32w: wide-band exact FP64 scratch
    DevBuf trace32, trace64, prec_acc;  // precision trace (FP_FLAG_PRECISION_TRACE)
    u64 s64_doubles = 0;
    BatchWork work{};
    uint32_t last_R = 0;
    uint64_t last_Q = 0;

    // finalized tables
    HostTable out[4];

    // statistics
    fp_stats stats{};
    unsigned long long launch_base = 0;
    cudaEvent_t ev[16]{};  // [0..8] stage boundaries, [10..11] the band-class-0 BAQ launch, [12..15] BAQ paths
    HmmConst hmm{};
    double qual2err[256];

    fp_status fail(fp_status s, const std::string &m) {
        err = m;
        return s;
    }
    fp_status cuda_fail(cudaError_t e, const char *where) {
        err = std::string(where) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? FP_OOM : FP_DEVICE_ERROR;
    }
};

#define CK(call, where)                                          \
    do {                                                         \
        cudaError_t _e = (call);                                 \
        if (_e != cudaSuccess) return eng->cuda_fail(_e, where); \
    } while (0)

namespace {

size_t al(size_t x) { return (x + 255) & ~size_t(255); }

fp_status alloc_tables(fp_engine *eng) {
    eng->tables.ks = make_keyspace(eng->n_rg);
    const size_t n = eng->tables.ks.total;
    CK(eng->tab_obs.ensure(n * sizeof(unsigned long long)), "table allocation");
    CK(eng->tab_mism.ensure(n * sizeof(float)), "table allocation");
    CK(eng->tab_stage.ensure(n * sizeof(u32)), "table allocation");
    CK(cudaMemsetAsync(eng->tab_stage.p, 0, n * sizeof(u32), eng->st), "table clear");
    eng->tables.stage = eng->tab_stage.as<u32>();
    const size_t nd = size_t(eng->n_rg) * 2 * CYC_DIFF_LEN;
    CK(eng->tab_cyc.ensure(nd * sizeof(int)), "table allocation");
    CK(cudaMemsetAsync(eng->tab_cyc.p, 0, nd * sizeof(int), eng->st), "table clear");
    eng->tables.cyc_diff = eng->tab_cyc.as<int>();
    eng->staged_bases = 0;
    CK(cudaMemsetAsync(eng->tab_obs.p, 0, n * sizeof(unsigned long long), eng->st), "table clear");
    CK(cudaMemsetAsync(eng->tab_mism.p, 0, n * sizeof(float), eng->st), "table clear");
    eng->tables.obs = eng->tab_obs.as<unsigned long long>();
    eng->tables.mism = eng->tab_mism.as<float>();
    return FP_OK;
}

// Waits for the last queued sort + fold and adds its device time to the statistics.
cudaError_t fold_harvest(fp_engine *eng) {
    if (!eng->fold_pending) return cudaSuccess;
    const cudaError_t e = cudaEventSynchronize(eng->fold_end);
    if (e != cudaSuccess) return e;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, eng->fold_start, eng->fold_end) == cudaSuccess)
        eng->stats.gpu_ms_per_stage[FP_STAGE_SORT_REDUCE] += ms;
    eng->fold_pending = false;
    return cudaSuccess;
}

fp_status upload_refs(fp_engine *eng) {
    CK(eng->d_contigs.ensure(std::max<size_t>(1, eng->h_contigs.size()) * sizeof(DevContig)), "contig table");
    if (!eng->h_contigs.empty())
        CK(cudaMemcpy(eng->d_contigs.p, eng->h_contigs.data(), eng->h_contigs.size() * sizeof(DevContig),
                      cudaMemcpyHostToDevice), "contig table");
    CK(eng->d_sites.ensure(std::max<size_t>(1, eng->h_sites.size()) * sizeof(DevSites)), "site table");
    if (!eng->h_sites.empty())
        CK(cudaMemcpy(eng->d_sites.p, eng->h_sites.data(), eng->h_sites.size() * sizeof(DevSites),
                      cudaMemcpyHostToDevice), "site table");
    eng->ref.contigs = eng->d_contigs.as<DevContig>();
    eng->ref.num_contigs = uint32_t(eng->h_contigs.size());
    eng->ref.sites = eng->d_sites.as<DevSites>();
    eng->ref.num_site_contigs = uint32_t(eng->h_sites.size());
    return FP_OK;
}

// C entry points return a status for host allocation failures and other C++ exceptions instead of letting
// them cross the C ABI (which would terminate the caller's process)
template <typename F> fp_status guarded(fp_engine *eng, F &&body) {
    try {
        return body();
    } catch (const std::bad_alloc &) {
        if (eng) eng->err.assign("host alloc failed");
        return FP_OOM;
    } catch (...) {
        if (eng) eng->err.assign("host exception");
        return FP_DEVICE_ERROR;
    }
}

}  // namespace

extern "C" {

static fp_status create_impl(const fp_options *o, fp_engine **out) {
    if (!o || !out) return FP_BAD_INPUT;
    *out = nullptr;
    if (o->num_read_groups == 0 || o->num_read_groups > 256) return FP_BAD_INPUT;
    if (o->replay_reads_per_warp > 32) return FP_BAD_INPUT;
    fp_engine *eng = new fp_engine();
    eng->device = o->device;
    eng->baq_mode = o->baq_mode;
    if (o->replay_reads_per_warp) eng->replay_rpw = o->replay_reads_per_warp;
    eng->flags = o->flags;
    eng->n_rg = o->num_read_groups;
    eng->co_target = o->coalesce_reads;
    cudaError_t e = cudaSetDevice(eng->device);
    if (e != cudaSuccess) {
        delete eng;
        return FP_DEVICE_ERROR;
    }
    e = cudaStreamCreateWithFlags(&eng->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        // band class 1 runs beside class 0 on a higher-priority stream: its blocks are placed first as SM
        // resources free up
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        e = cudaStreamCreateWithPriority(&eng->st2, cudaStreamNonBlocking, greatest);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&eng->st_copy, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&eng->st3, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&eng->st_fold, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&eng->fold_start);
    if (e == cudaSuccess) e = cudaEventCreate(&eng->fold_end);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&eng->cov1_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&eng->in_ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&eng->in_ev[1], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&eng->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&eng->join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        fp_engine_destroy(eng);
        return FP_DEVICE_ERROR;
    }
    for (auto &x : eng->ev) cudaEventCreate(&x);
    // host libm constants (device/baq.cu:80, :355-359; device/expected_error.h:48-51)
    for (int q = 0; q < 256; q++) {
        eng->hmm.qual2prob[q] = pow(10.0, -q / 10.0);
        eng->qual2err[q] = pow(10.0, q / -10.0);
    }
    eng->hmm.gap_open = pow(10.0, (-40.0) / 10.);
    baq64_set_constants(eng->hmm);
    baq_tpr_set_constants(eng->hmm);
    baq_seg_set_constants(eng->hmm);
    baq_exact_set_constants(eng->hmm);
    baq_wide_set_constants(eng->hmm);
    EmpConst ec;
    for (int d = 0; d <= 40; d++) ec.prior[d] = log10(gaussian(double(d)));
    for (int bin = 0; bin <= 60; bin++) {
        const double Qemp = bin / 1.0;
        ec.log10p[bin] = Qemp / -10.0;
        ec.log10_one_minus_p[bin] = log10(1 - pow(10.0, ec.log10p[bin]));
    }
    post_set_constants(ec, eng->qual2err);
    eng->launch_base = g_kernel_launches;
    fp_status s = alloc_tables(eng);
    if (s == FP_OK) s = upload_refs(eng);
    if (s == FP_OK) {
        e = cudaStreamSynchronize(eng->st);
        if (e != cudaSuccess) s = FP_DEVICE_ERROR;
    }
    if (s != FP_OK) {
        fp_engine_destroy(eng);
        return s;
    }
    *out = eng;
    return FP_OK;
}

void fp_engine_destroy(fp_engine *eng) {
    if (!eng) return;
    cudaSetDevice(eng->device);
    if (eng->st) cudaStreamSynchronize(eng->st);
    if (eng->st2) cudaStreamSynchronize(eng->st2);
    if (eng->st_copy) cudaStreamSynchronize(eng->st_copy);
    if (eng->st3) cudaStreamSynchronize(eng->st3);
    if (eng->st_fold) cudaStreamSynchronize(eng->st_fold);
    if (eng->store) refstore_release(eng->store);
    for (auto &b : eng->contig_bufs) b.release();
    for (auto &b : eng->site_bufs) b.release();
    DevBuf *bufs[] = {&eng->d_contigs, &eng->d_sites, &eng->tab_obs, &eng->tab_mism, &eng->tab_stage, &eng->tab_cyc, &eng->in_bufs[0], &eng->in_bufs[1], &eng->oplen,
                      &eng->cigoff, &eng->ev_rc, &eng->ev_type, &eng->per_read, &eng->per_base, &eng->lists,
                      &eng->counters, &eng->entry_cnt, &eng->entry_off, &eng->entries, &eng->entries_alt,
                      &eng->sort_tmp, &eng->scan_tmp, &eng->s32, &eng->s32b, &eng->s64, &eng->co_buf, &eng->s32w};
    for (DevBuf *b : bufs) b->release();
    for (auto &x : eng->ev)
        if (x) cudaEventDestroy(x);
    if (eng->fork) cudaEventDestroy(eng->fork);
    if (eng->join) cudaEventDestroy(eng->join);
    if (eng->st2) cudaStreamDestroy(eng->st2);
    if (eng->st_copy) cudaStreamDestroy(eng->st_copy);
    if (eng->st3) cudaStreamDestroy(eng->st3);
    if (eng->cov1_done) cudaEventDestroy(eng->cov1_done);
    if (eng->st_fold) cudaStreamDestroy(eng->st_fold);
    if (eng->fold_start) cudaEventDestroy(eng->fold_start);
    if (eng->fold_end) cudaEventDestroy(eng->fold_end);
    for (auto &x : eng->in_ev)
        if (x) cudaEventDestroy(x);
    if (eng->st) cudaStreamDestroy(eng->st);
    delete eng;
}

const char *fp_last_error(const fp_engine *eng) { return eng ? eng->err.c_str() : "null engine"; }

fp_status fp_engine_set_contig(fp_engine *eng, uint32_t id, const uint32_t *packed4, uint64_t n) {
    if (!eng || (!packed4 && n)) return FP_BAD_INPUT;
    if (eng->store) return eng->fail(FP_BAD_INPUT, "the engine reads an attached reference store");
    CK(cudaSetDevice(eng->device), "set device");
    if (id >= eng->h_contigs.size()) {
        eng->h_contigs.resize(id + 1, DevContig{nullptr, 0});
        eng->contig_bufs.resize(id + 1);
    }
    const size_t words = (n + 7) / 8;
    DevBuf &b = eng->contig_bufs[id];
    b.release();
    CK(b.ensure((words + 1) * sizeof(uint32_t)), "contig upload");
    CK(cudaMemset(b.p, 0, (words + 1) * sizeof(uint32_t)), "contig upload");
    if (words) {
        CK(cudaMemcpy(b.p, packed4, words * sizeof(uint32_t), cudaMemcpyHostToDevice), "contig upload");
        if (n % 8) {
            // symbols past the end of the contig read as 0
            uint32_t last = packed4[words - 1] & ((1u << ((n % 8) * 4)) - 1);
            CK(cudaMemcpy(b.as<uint32_t>() + words - 1, &last, 4, cudaMemcpyHostToDevice), "contig upload");
        }
    }
    eng->h_contigs[id] = DevContig{b.as<uint32_t>(), n};
    return upload_refs(eng);
}

static fp_status set_known_sites_impl(fp_engine *eng, uint32_t id, const uint32_t *start, const uint32_t *stop,
                                       uint32_t n) {
    if (!eng || ((!start || !stop) && n)) return FP_BAD_INPUT;
    if (eng->store) return eng->fail(FP_BAD_INPUT, "the engine reads an attached reference store");
    CK(cudaSetDevice(eng->device), "set device");
    if (id >= eng->h_sites.size()) {
        eng->h_sites.resize(id + 1, DevSites{nullptr, nullptr, nullptr, 0, 0});
        eng->site_bufs.resize(id + 1);
    }
    // prefix max of the stops (loader/variants.cu:126-134); sites must be sorted by start
    std::vector<uint32_t> maxend(n);
    for (uint32_t i = 0; i < n; i++) {
        if (i && start[i] < start[i - 1]) return eng->fail(FP_BAD_INPUT, "known sites must be sorted by start");
        maxend[i] = i ? std::max(maxend[i - 1], stop[i]) : stop[0];
    }
    DevBuf &b = eng->site_bufs[id];
    b.release();
    CK(b.ensure(std::max<size_t>(1, size_t(n)) * 3 * sizeof(uint32_t)), "known-site upload");
    uint32_t *p = b.as<uint32_t>();
    if (n) {
        CK(cudaMemcpy(p, start, n * 4, cudaMemcpyHostToDevice), "known-site upload");
        CK(cudaMemcpy(p + n, stop, n * 4, cudaMemcpyHostToDevice), "known-site upload");
        CK(cudaMemcpy(p + 2 * size_t(n), maxend.data(), n * 4, cudaMemcpyHostToDevice), "known-site upload");
    }
    eng->h_sites[id] = DevSites{p, p + n, p + 2 * size_t(n), n, 0};
    return upload_refs(eng);
}

static fp_status co_flush(fp_engine *eng);

// Engines of one GPU share a reference store's device copy (segmented_database.h:224-244 keeps one resident
// set per engine). The engine's own contigs and sites are freed; work already queued is finished first, and
// host batches staged for coalescing are submitted under the reference they were staged with.
static fp_status attach_refstore_impl(fp_engine *eng, fp_refstore *store) {
    if (!eng) return FP_BAD_INPUT;
    if (store == eng->store) return FP_OK;
    CK(cudaSetDevice(eng->device), "set device");
    const fp_status fs = co_flush(eng);
    if (fs != FP_OK) return fs;
    cudaStream_t sts[] = {eng->st, eng->st2, eng->st3, eng->st_copy, eng->st_fold};
    for (cudaStream_t x : sts)
        if (x) CK(cudaStreamSynchronize(x), "attach reference store");
    const DevRef *r = nullptr;
    if (store) {
        std::string m;
        int status = FP_OK;
        r = refstore_acquire(store, eng->device, m, status);
        if (!r) return eng->fail(fp_status(status), m);
    }
    if (eng->store) refstore_release(eng->store);
    for (auto &b : eng->contig_bufs) b.release();
    for (auto &b : eng->site_bufs) b.release();
    eng->contig_bufs.clear();
    eng->site_bufs.clear();
    eng->h_contigs.clear();
    eng->h_sites.clear();
    eng->store = store;
    if (store) {
        eng->ref = *r;
        return FP_OK;
    }
    return upload_refs(eng);
}

// ---- batch inputs: the 17 host arrays of a view, their byte sizes and offsets in a device input buffer ----
struct ViewArrays {
    const void *src[17];
    size_t size[17];
    size_t off[17];
    size_t total;
};
static ViewArrays view_arrays(const fp_batch_view *v) {
    ViewArrays a;
    const uint64_t R = v->num_reads, Q = v->num_qualities, C = v->num_cigar_ops, W = (v->num_read_symbols + 7) / 8;
    const void *src[] = {v->chromosome, v->alignment_start, v->alignment_stop, v->mate_alignment_start,
                         v->inferred_insert_size, v->cigars, v->cigar_start, v->cigar_len, v->reads,
                         v->read_start, v->read_len, v->qualities, v->qual_start, v->qual_len, v->flags, v->mapq,
                         v->read_group};
    const size_t size[] = {R * 2, R * 4, R * 4, R * 4, R * 4, C * 4, R * 4, R * 4, W * 4,
                           R * 4, R * 4, Q, R * 4, R * 4, R * 2, R * 1, R * 4};
    a.total = 0;
    for (int i = 0; i < 17; i++) {
        a.src[i] = src[i];
        a.size[i] = size[i];
        a.off[i] = a.total;
        a.total += al(size[i] ? size[i] : 1);
    }
    return a;
}
static bool same_view(const fp_engine *eng, int k, const fp_batch_view *v, const ViewArrays &a) {
    const uint64_t counts[4] = {v->num_reads, v->num_cigar_ops, v->num_read_symbols, v->num_qualities};
    for (int i = 0; i < 4; i++)
        if (eng->in_counts[k][i] != counts[i]) return false;
    for (int i = 0; i < 17; i++)
        if (eng->in_src[k][i] != a.src[i]) return false;
    return true;
}
// queues the H2D copies of a view into input buffer k on stream s
static fp_status stage_inputs(fp_engine *eng, int k, const fp_batch_view *v, const ViewArrays &a, cudaStream_t s) {
    CK(eng->in_bufs[k].ensure(a.total), "batch input allocation");
    char *base = eng->in_bufs[k].as<char>();
    for (int i = 0; i < 17; i++)
        if (a.size[i]) CK(cudaMemcpyAsync(base + a.off[i], a.src[i], a.size[i], cudaMemcpyHostToDevice, s), "H2D");
    const uint64_t counts[4] = {v->num_reads, v->num_cigar_ops, v->num_read_symbols, v->num_qualities};
    for (int i = 0; i < 4; i++) eng->in_counts[k][i] = counts[i];
    for (int i = 0; i < 17; i++) eng->in_src[k][i] = a.src[i];
    return FP_OK;
}

static fp_status prefetch_batch_impl(fp_engine *eng, const fp_batch_view *v) {
    if (!eng || !v) return FP_BAD_INPUT;
    if (v->num_reads == 0) return FP_OK;
    if (eng->co_target) return FP_OK;  // coalescing copies each batch into the staging batch at its submit
    const ViewArrays a = view_arrays(v);
    for (int i = 0; i < 17; i++)
        if (!a.src[i] && a.size[i]) return eng->fail(FP_BAD_INPUT, "null batch array");
    CK(cudaSetDevice(eng->device), "set device");
    std::lock_guard<std::mutex> lock(eng->in_mu);
    int k = eng->in_state[0] == 0 ? 0 : (eng->in_state[1] == 0 ? 1 : -1);
    if (k < 0) return eng->fail(FP_BAD_INPUT, "both input buffers hold batches not yet submitted");
    const fp_status s = stage_inputs(eng, k, v, a, eng->st_copy);
    if (s != FP_OK) return s;
    CK(cudaEventRecord(eng->in_ev[k], eng->st_copy), "prefetch event");
    eng->in_state[k] = 1;
    return FP_OK;
}

static fp_status submit(fp_engine *eng, const fp_batch_view *v, bool on_device);

static fp_status co_submit(fp_engine *eng, const fp_batch_view *v);
static fp_status co_flush(fp_engine *eng);

static fp_status submit_batch_impl(fp_engine *eng, const fp_batch_view *v) {
    if (eng && v && eng->co_target) return co_submit(eng, v);
    return submit(eng, v, false);
}

static fp_status submit_batch_device_impl(fp_engine *eng, const fp_batch_view *v) {
    if (eng && eng->co_target) {
        const fp_status s = co_flush(eng);  // staged reads come first in stream order
        if (s != FP_OK) return s;
    }
    return submit(eng, v, true);
}

void *fp_engine_cuda_stream(fp_engine *eng) { return eng ? reinterpret_cast<void *>(eng->st) : nullptr; }

static fp_status submit(fp_engine *eng, const fp_batch_view *v, bool on_device) {
    if (!eng || !v) return FP_BAD_INPUT;
    if (eng->finalized) return eng->fail(FP_NOT_READY, "submit after finalize; call fp_engine_reset first");
    CK(cudaSetDevice(eng->device), "set device");
    cudaStream_t st = eng->st;
    const uint32_t R = v->num_reads;
    const uint64_t Q = v->num_qualities;
    const uint32_t C = v->num_cigar_ops;
    const uint64_t W = (v->num_read_symbols + 7) / 8;
    if (R == 0) {
        eng->stats.num_batches++;
        return FP_OK;
    }
    (void)W;
    ViewArrays va = view_arrays(v);
    for (int i = 0; i < 17; i++)
        if (!va.src[i] && va.size[i]) return eng->fail(FP_BAD_INPUT, "null batch array");

    cudaEventRecord(eng->ev[0], st);
    // ---- inputs: a prefetched copy of this view, or copies queued here into a free input buffer ----
    size_t offs[17];
    char *base = nullptr;
    // marks the input buffer free again however this call returns
    struct Release {
        fp_engine *e;
        int k = -1;
        ~Release() {
            if (k >= 0) {
                cudaStreamSynchronize(e->st);  // (already idle unless the batch failed part-way)
                std::lock_guard<std::mutex> lock(e->in_mu);
                e->in_state[k] = 0;
            }
        }
    } release{eng};
    if (on_device) {
        // arrays are device pointers already: address them relative to a null base
        for (int i = 0; i < 17; i++) offs[i] = size_t(reinterpret_cast<uintptr_t>(va.src[i]));
    } else {
        int k = -1;
        bool prefetched = false;
        {
            std::lock_guard<std::mutex> lock(eng->in_mu);
            for (int j = 0; j < 2 && k < 0; j++)
                if (eng->in_state[j] == 1 && same_view(eng, j, v, va)) { k = j; prefetched = true; }
            for (int j = 0; j < 2 && k < 0; j++)
                if (eng->in_state[j] == 0) k = j;
            if (k < 0) {
                // both buffers hold other prefetched views: drop the first one
                CK(cudaEventSynchronize(eng->in_ev[0]), "prefetch");
                k = 0;
            }
            eng->in_state[k] = 2;
        }
        release.k = k;
        if (prefetched) {
            CK(cudaStreamWaitEvent(st, eng->in_ev[k], 0), "prefetch wait");
        } else {
            const fp_status s0 = stage_inputs(eng, k, v, va, st);
            if (s0 != FP_OK) return s0;
        }
        base = eng->in_bufs[k].as<char>();
        for (int i = 0; i < 17; i++) offs[i] = va.off[i];
    }
    DevBatch &b = eng->batch;
    b.R = R;
    b.num_cigar_ops = C;
    b.num_syms = v->num_read_symbols;
    b.num_quals = Q;
    b.chromosome = reinterpret_cast<const u16 *>(base + offs[0]);
    b.astart = reinterpret_cast<const u32 *>(base + offs[1]);
    b.astop = reinterpret_cast<const u32 *>(base + offs[2]);
    b.mstart = reinterpret_cast<const u32 *>(base + offs[3]);
    b.isize = reinterpret_cast<const i32 *>(base + offs[4]);
    b.cigars = reinterpret_cast<const u32 *>(base + offs[5]);
    b.cigar_start = reinterpret_cast<const u32 *>(base + offs[6]);
    b.cigar_len = reinterpret_cast<const u32 *>(base + offs[7]);
    b.reads = reinterpret_cast<const u32 *>(base + offs[8]);
    b.read_start = reinterpret_cast<const u32 *>(base + offs[9]);
    b.read_len = reinterpret_cast<const u32 *>(base + offs[10]);
    b.quals = reinterpret_cast<const u8 *>(base + offs[11]);
    b.qual_start = reinterpret_cast<const u32 *>(base + offs[12]);
    b.qual_len = reinterpret_cast<const u32 *>(base + offs[13]);
    b.flags = reinterpret_cast<const u16 *>(base + offs[14]);
    b.mapq = reinterpret_cast<const u8 *>(base + offs[15]);
    b.rg = reinterpret_cast<const u32 *>(base + offs[16]);
    cudaEventRecord(eng->ev[1], st);

    // ---- validation + CIGAR-length scan ----
    BatchWork &w = eng->work;
    CK(eng->counters.ensure(64 * sizeof(u32)), "counters");
    w.counters = eng->counters.as<u32>();
    w.err = w.counters + 32;
    CK(cudaMemsetAsync(w.counters, 0, 64 * sizeof(u32), st), "counters");
    CK(eng->oplen.ensure(al((C + 1) * 4ull)), "op lengths");
    CK(eng->cigoff.ensure(al((C + 1) * 4ull)), "cigar offsets");
    const size_t scan_need = std::max(scan_tmp_bytes(C + 1), scan_tmp_bytes(R + 1));
    CK(eng->scan_tmp.ensure(scan_need), "scan scratch");
    launch_validate(b, eng->n_rg, w.err, st);
    launch_op_lengths(b, eng->oplen.as<u32>(), st);
    w.cigar_offsets = eng->cigoff.as<u32>();
    launch_exclusive_scan(eng->oplen.as<u32>(), w.cigar_offsets, C, eng->scan_tmp.p, st);
    u32 hdr[2] = {0, 0};
    CK(cudaMemcpyAsync(&hdr[0], w.err, 4, cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaMemcpyAsync(&hdr[1], w.cigar_offsets + C, 4, cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaStreamSynchronize(st), "validation");
    if (hdr[0]) {
        std::string m = "batch rejected:";
        if (hdr[0] & ERR_BAD_READ_RANGE) m += " read/cigar/quality range outside the batch arrays;";
        if (hdr[0] & ERR_READ_TOO_LONG) m += " read longer than 511 bases (10-bit cycle covariate);";
        if (hdr[0] & ERR_BAD_READ_GROUP) m += " read group id >= num_read_groups;";
        return eng->fail(FP_BAD_INPUT, m);
    }
    const u64 E = hdr[1];

    // ---- work arrays ----
    CK(eng->ev_rc.ensure(al(E * 4 + 4)), "events");
    CK(eng->ev_type.ensure(al(E + 4)), "events");
    w.ev_rc = eng->ev_rc.as<u32>();
    w.ev_type = eng->ev_type.as<u8>();
    w.num_events = E;
    const size_t pr_bytes = al(R) + al(R * 16ull) + al(R * 4ull) + al(R * 2ull) + al(R * 2ull);
    CK(eng->per_read.ensure(pr_bytes), "per-read arrays");
    {
        char *p = eng->per_read.as<char>();
        w.status = reinterpret_cast<u8 *>(p); p += al(R);
        w.win = reinterpret_cast<u16 *>(p); p += al(R * 16ull);
        w.hmm = reinterpret_cast<i16 *>(p); p += al(R * 4ull);
        w.bw = reinterpret_cast<u16 *>(p); p += al(R * 2ull);
        w.nerr = reinterpret_cast<u16 *>(p);
    }
    const size_t pb_bytes = al(Q) * 4 + al(Q * 4) + al(Q * 12) + al(Q * 2);
    CK(eng->per_base.ensure(pb_bytes), "per-base arrays");
    {
        char *p = eng->per_base.as<char>();
        w.bflags = reinterpret_cast<u8 *>(p); p += al(Q);
        w.tag = reinterpret_cast<u8 *>(p); p += al(Q);
        w.baq_q = reinterpret_cast<u8 *>(p); p += al(Q);
        w.baq_amb = reinterpret_cast<u8 *>(p); p += al(Q);
        w.baq_state = reinterpret_cast<u32 *>(p); p += al(Q * 4);
        w.baq_alt = reinterpret_cast<u16 *>(p); p += al(Q * 2);
        w.frac = reinterpret_cast<float *>(p);
    }
    CK(eng->lists.ensure(al(R * 4ull) * 9 + 4096), "work lists");
    w.baq_list = eng->lists.as<u32>();
    w.esc_list = w.baq_list + 3ull * R;
    // regions of R entries: BAQ lists of band classes 0-2, escalation lists of classes 0-2, classes 0 and 1
    // ordered by query length, then the length histogram
    u32 *sorted_lists = w.baq_list + 6ull * R;
    u32 *len_hist = w.baq_list + 8ull * R;
    CK(eng->entry_cnt.ensure(al((R + 1) * 4ull)), "entry counts");
    CK(eng->entry_off.ensure(al((R + 1) * 4ull)), "entry offsets");
    w.entry_count = eng->entry_cnt.as<u32>();
    w.entry_offset = eng->entry_off.as<u32>();
    CK(cudaMemsetAsync(w.tag, 0xFF, Q, st), "tag init");
    // precision trace: the FP32 kernels record t and its interval per base; the plain FP64 path is run on
    // the same reads after the BAQ stage (FP32 mode only)
    const bool trace = (eng->flags & FP_FLAG_PRECISION_TRACE) && eng->baq_mode == FP_BAQ_FP32;
    w.trace32 = nullptr;
    w.trace64 = nullptr;
    w.exact_tags = (eng->flags & FP_FLAG_EXACT_BAQ_TAGS) ? 1u : 0u;
    if (trace) {
        CK(eng->trace32.ensure(al(Q * 12 + 12)), "precision trace");
        CK(eng->trace64.ensure(al(Q * 8 + 8)), "precision trace");
        if (!eng->prec_acc.p) {
            CK(eng->prec_acc.ensure(sizeof(PrecisionAcc)), "precision trace");
            CK(cudaMemsetAsync(eng->prec_acc.p, 0, sizeof(PrecisionAcc), st), "precision trace");
        }
        w.trace32 = eng->trace32.as<float>();
        w.trace64 = eng->trace64.as<double>();
        CK(cudaMemsetAsync(w.trace32, 0xFF, Q * 12, st), "precision trace");  // NaN: no FP32 value
        CK(cudaMemsetAsync(w.trace64, 0, Q * 8, st), "precision trace");
    }
    cudaEventRecord(eng->ev[2], st);

    // ---- K1 ----
    launch_prep(b, eng->ref, w, st);
    CK(cudaGetLastError(), "prep launch");
    cudaEventRecord(eng->ev[3], st);
    u32 cnt[16];
    CK(cudaMemcpyAsync(cnt, w.counters, sizeof(cnt), cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaStreamSynchronize(st), "prep");
    const u32 bw_max[3] = {cnt[12], cnt[13], cnt[14]};
    const u32 n_cls[3] = {cnt[0], cnt[1], cnt[2]};

    // ---- K2 BAQ ----
    const uint32_t max_q = cnt[7] ? cnt[7] : 1;  // longest BAQ query window of the batch
    auto run_fp64 = [&](const u32 *list, const u32 *count, u32 nmax, u32 max_bw, u32 min_bw = 0,
                        bool cap = true) -> fp_status {
        if (!nmax) return FP_OK;
        const u32 threads = std::min<u32>(baq64_threads(), ((nmax + 127) / 128) * 128);
        u64 need = baq64_scratch_doubles(threads, max_q, max_bw);
        const u64 budget = (u64(6) << 30) / 8;  // at most 6 GiB of FP64 scratch
        if (need > budget) need = std::max<u64>(budget, baq64_scratch_doubles(128, max_q, max_bw));
        CK(eng->s64.ensure(need * 8), "FP64 BAQ scratch");
        eng->s64_doubles = eng->s64.cap / 8;
        launch_baq64(b, eng->ref, w, list, count, nmax, eng->s64.as<double>(), eng->s64_doubles, max_q, max_bw, st,
                     min_bw);
        if (cap) launch_cap(b, w, list, count, 1, st, nmax);
        return FP_OK;
    };
    fp_status s;
    bool timed_main = false, timed_paths = false, cov1_overlapped = false;
    // K3 first count pass (every active read except the deferred ones). Observation counts go to u32 stage
    // counters; a key gains at most one count per base of the batch, so the stage is merged into the u64 table
    // before the bases counted since the last merge could reach 2^32
    auto count_first_pass = [&](cudaStream_t cs) {
        if (eng->staged_bases + Q > 0xFFFFFFFFull) {
            launch_merge_stage(eng->tables, cs);
            eng->staged_bases = 0;
        }
        eng->staged_bases += Q;
        launch_cov_count(b, w, eng->tables, cs);
    };
    if (eng->baq_mode == FP_BAQ_FP64) {
        for (int c = 0; c < 3; c++) {
            if (c == 0 && n_cls[0]) { cudaEventRecord(eng->ev[10], st); }
            if ((s = run_fp64(w.baq_list + size_t(c) * R, w.counters + c, n_cls[c], bw_max[c])) != FP_OK) return s;
            if (c == 0 && n_cls[0]) { cudaEventRecord(eng->ev[11], st); timed_main = true; }
        }
    } else {
        // FP32 with certified bounds (band classes 0 and 1), exact FP64 replay of the undecided reads, and exact
        // FP64 for bands wider than 15. Band class 1 (few reads, latency-bound kernels)
        // runs on a second stream with its own scratch and work counters, alongside the class-0 kernels.
        const u64 budget = u64(3) << 30, budget1 = u64(1) << 30;
        CK(eng->s32.ensure(budget), "BAQ scratch");
        const bool replay_all = (eng->flags & FP_FLAG_REPLAY_ALL) != 0;
        launch_sort_baq_lists(w, R, std::max(n_cls[0], n_cls[1]), len_hist, sorted_lists, st);
        auto run_fp32 = [&](int c, cudaStream_t cs, void *scr, u64 scr_bytes, u32 *ctr) {
            const u32 *list = sorted_lists + size_t(c) * R;
            if (c == 0) cudaEventRecord(eng->ev[10], cs);
            if (c == 0)
                launch_baq_seg(b, eng->ref, w, list, w.counters + c, n_cls[c], ctr, scr, scr_bytes, max_q, cs);
            else
                launch_baq_wide16(b, eng->ref, w, list, w.counters + c, n_cls[c], ctr, scr, scr_bytes, max_q, cs);
            if (c == 0) { cudaEventRecord(eng->ev[11], cs); timed_main = true; }
            launch_cap(b, w, list, w.counters + c, 0, cs, n_cls[c]);
        };
        auto run_replay = [&](int c, cudaStream_t cs, void *scr, u64 scr_bytes, u32 *ctr) {
            const u32 *list = w.baq_list + size_t(c) * R;
            const u32 *esc = replay_all ? list : w.esc_list + size_t(c) * R;
            u32 *esc_count = replay_all ? w.counters + c : w.counters + (c == 0 ? 4 : (c == 1 ? 10 : 27));
            if (eng->replay_rpw && c < 2)
                launch_baq_tpr(b, eng->ref, w, esc, esc_count, n_cls[c], c, true, ctr, scr, scr_bytes, max_q,
                               eng->replay_rpw, cs);
            else
                launch_baq_exact(b, eng->ref, w, esc, esc_count, n_cls[c], c, ctr, scr, scr_bytes, max_q, replay_all,
                                 cs);
            launch_cap(b, w, esc, esc_count, 1, cs, n_cls[c]);
        };
        // the class-1 FP32 kernel (few reads, latency-bound) is queued first on the high-priority stream; the
        // class-0 FP32 kernel then fills what is left of the GPU
        const bool split = n_cls[1] > 0;
        if (split) {
            CK(eng->s32b.ensure(budget1), "BAQ scratch");
            CK(cudaEventRecord(eng->fork, st), "fork");
            CK(cudaStreamWaitEvent(eng->st2, eng->fork, 0), "fork");
            run_fp32(1, eng->st2, eng->s32b.p, budget1, w.counters + 9);
            cudaEventRecord(eng->ev[12], eng->st2);
        }
        if (n_cls[0]) {
            run_fp32(0, st, eng->s32.p, budget, w.counters + 8);
            cudaEventRecord(eng->ev[14], st);
        }
        // bands wider than 15: FP32 with certified bounds, the band across a warp's lanes, for bw <= 63 (its
        // undecided reads join the replays); exact FP64 for wider ones (each kernel skips the others' reads; the
        // FP64 results are final, so the capping step finds them decided)
        if (n_cls[2]) {
            const u32 *list2 = w.baq_list + 2ull * R;
            // (the class-2 replay reuses the buffer)
            CK(eng->s32w.ensure(std::max(baq_wide_scratch_bytes(n_cls[2], max_q), baq_exact_block_scratch_bytes(2, max_q))),
               "BAQ scratch");
            launch_baq_wide(b, eng->ref, w, list2, w.counters + 2, n_cls[2], w.counters + 26, eng->s32w.p,
                            eng->s32w.cap, max_q, st);
            // bw 32..63: the same with 32 lanes x 4 slots; wider: the thread-per-read FP64 kernel
            if (bw_max[2] > 31)
                launch_baq_wide64(b, eng->ref, w, list2, w.counters + 2, n_cls[2], w.counters + 29, eng->s32w.p,
                                  eng->s32w.cap, max_q, st);
            if (bw_max[2] > 63 && (s = run_fp64(list2, w.counters + 2, n_cls[2], bw_max[2], 64, false)) != FP_OK)
                return s;
            launch_cap(b, w, list2, w.counters + 2, 0, st, n_cls[2]);
        }
        // every certified read now has its final BQ tags; the reads left for the replay are marked deferred.
        // The first covariate count pass runs on its own stream beside the replays (with the test hook every
        // read is replayed, so the pass waits for the whole BAQ stage instead)
        if (!replay_all) {
            cudaEventRecord(eng->ev[9], st);
            CK(cudaStreamWaitEvent(eng->st3, eng->ev[9], 0), "fork");
            if (split) CK(cudaStreamWaitEvent(eng->st3, eng->ev[12], 0), "fork");
            count_first_pass(eng->st3);
            CK(cudaEventRecord(eng->cov1_done, eng->st3), "join");
            cov1_overlapped = true;
        }
        if (split) {
            // FP64 replays slow to a crawl beside the FP32 kernel (they share its pipes): the class-1 replay
            // waits for it and then runs beside the class-0 replay
            CK(cudaStreamWaitEvent(eng->st2, eng->ev[14], 0), "fork");
            run_replay(1, eng->st2, eng->s32b.p, budget1, w.counters + 24);
            cudaEventRecord(eng->ev[13], eng->st2);
            CK(cudaEventRecord(eng->join, eng->st2), "join");
        }
        if (n_cls[0]) {
            run_replay(0, st, eng->s32.p, budget, w.counters + 11);
            cudaEventRecord(eng->ev[15], st);
        }
        if (n_cls[2]) run_replay(2, st, eng->s32w.p, eng->s32w.cap, w.counters + 28);
        timed_paths = split && n_cls[0];
        if (split) CK(cudaStreamWaitEvent(st, eng->join, 0), "join");
    }
    CK(cudaGetLastError(), "BAQ launch");
    if (trace) {
        // every BAQ read once more through the plain FP64 kernel, writing only its pre-floor qualities, then
        // the per-read comparison with the FP32 pass (after the replays: the first count pass may still run
        // beside it, it reads none of the trace)
        const u32 bwm = std::max(bw_max[0], std::max(bw_max[1], bw_max[2]));
        const u32 nmax = std::max(n_cls[0], std::max(n_cls[1], n_cls[2]));
        if (nmax) {
            const u32 threads = std::min<u32>(baq64_threads(), ((nmax + 127) / 128) * 128);
            u64 need = baq64_scratch_doubles(threads, max_q, bwm);
            const u64 budget = (u64(6) << 30) / 8;
            if (need > budget) need = std::max<u64>(budget, baq64_scratch_doubles(128, max_q, bwm));
            CK(eng->s64.ensure(need * 8), "FP64 BAQ scratch");
            eng->s64_doubles = eng->s64.cap / 8;
            for (int c = 0; c < 3; c++)
                launch_baq64(b, eng->ref, w, w.baq_list + size_t(c) * R, w.counters + c, n_cls[c], eng->s64.as<double>(),
                             eng->s64_doubles, max_q, bwm, st, 0, true);
            for (int c = 0; c < 3; c++)
                launch_precision(b, w, w.baq_list + size_t(c) * R, w.counters + c, n_cls[c],
                                 eng->prec_acc.as<PrecisionAcc>(), st);
        }
    }
    cudaEventRecord(eng->ev[4], st);

    // ---- K3 count (second pass: the replayed reads) + scan ----
    if (cov1_overlapped) CK(cudaStreamWaitEvent(st, eng->cov1_done, 0), "join");
    else count_first_pass(st);
    if (eng->baq_mode != FP_BAQ_FP64) {
        for (int c = 0; c < 3; c++)
            launch_cov_count_list(b, w, eng->tables, w.esc_list + size_t(c) * R,
                                  w.counters + (c == 0 ? 4 : (c == 1 ? 10 : 27)), n_cls[c], st);
    }
    launch_cycle_pairs(eng->tables, st);
    launch_exclusive_scan(w.entry_count, w.entry_offset, R, eng->scan_tmp.p, st);
    u32 tail[2];
    CK(cudaMemcpyAsync(&tail[0], w.entry_offset + R, 4, cudaMemcpyDeviceToHost, st), "D2H");
    u32 esc1 = 0, esc2 = 0;
    CK(cudaMemcpyAsync(&tail[1], w.counters + 4, 4, cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaMemcpyAsync(&esc1, w.counters + 10, 4, cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaMemcpyAsync(&esc2, w.counters + 27, 4, cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaStreamSynchronize(st), "covariates");
    const u64 N = tail[0];
    const size_t sort_bytes = std::max(radix_tmp_bytes(N), fold_tmp_bytes(N));
    // the previous batch's sort + fold may still read the entry buffers and their scratch: growing them waits
    // for it; otherwise the emit below waits for it on the device
    if (eng->entries.cap < al(N * 8 + 8) || eng->entries_alt.cap < al(N * 8 + 8) || eng->sort_tmp.cap < sort_bytes)
        CK(fold_harvest(eng), "sort + fold");
    CK(eng->entries.ensure(al(N * 8 + 8)), "entries");
    CK(eng->entries_alt.ensure(al(N * 8 + 8)), "entries");
    w.entries = eng->entries.as<u64>();
    w.entries_alt = eng->entries_alt.as<u64>();
    CK(eng->sort_tmp.ensure(sort_bytes), "sort scratch");
    if (eng->fold_pending) CK(cudaStreamWaitEvent(st, eng->fold_end, 0), "fold wait");
    launch_cov_emit(b, w, eng->tables, st);
    CK(cudaGetLastError(), "covariate launch");
    cudaEventRecord(eng->ev[5], st);

    // ---- K4 sort + ordered fold, on the fold stream: batches fold in submission order there, and the next
    // batch's copies and preparation run beside it ----
    CK(fold_harvest(eng), "sort + fold");  // the previous fold's events are read before they are recorded again
    CK(cudaStreamWaitEvent(eng->st_fold, eng->ev[5], 0), "fold fork");
    cudaEventRecord(eng->fold_start, eng->st_fold);
    int key_bits = 1;
    while (key_bits < 32 && (1ull << key_bits) < eng->tables.ks.total) key_bits++;
    u64 *sorted = w.entries;
    launch_radix_sort(w.entries, w.entries_alt, N, key_bits, eng->sort_tmp.p, eng->sort_tmp.cap, &sorted,
                      eng->st_fold);
    launch_fold(sorted, N, eng->tables.mism, eng->sort_tmp.p, eng->st_fold);
    CK(cudaGetLastError(), "sort launch");
    CK(cudaEventRecord(eng->fold_end, eng->st_fold), "fold join");
    eng->fold_pending = true;
    cudaEventRecord(eng->ev[6], st);
    u32 dev_err = 0;
    unsigned long long cells[3] = {0, 0, 0};
    u32 cause[4] = {0, 0, 0, 0};  // counters 22..25: state, quality, (class-1 replay work counter), unbounded rows
    CK(cudaMemcpyAsync(cells, w.counters + 16, sizeof(cells), cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaMemcpyAsync(cause, w.counters + 22, sizeof(cause), cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaMemcpyAsync(cnt, w.counters, sizeof(cnt), cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaMemcpyAsync(&dev_err, w.err, 4, cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaStreamSynchronize(st), "batch");
    if (dev_err & (ERR_INTERNAL | ERR_TIMEOUT | ERR_CAPACITY))
        return eng->fail(FP_DEVICE_ERROR, "kernel reported an internal error status");
    float ms;
    // (the sort + fold stage is timed on its own stream, fold_harvest)
    const int stage_of[5] = {FP_STAGE_H2D, FP_STAGE_OTHER, FP_STAGE_PREP, FP_STAGE_BAQ, FP_STAGE_COVARIATES};
    for (int i = 0; i < 5; i++) {
        if (cudaEventElapsedTime(&ms, eng->ev[i], eng->ev[i + 1]) == cudaSuccess)
            eng->stats.gpu_ms_per_stage[stage_of[i]] += ms;
    }
    eng->stats.total_reads += R;
    eng->stats.filtered_reads += cnt[5];
    eng->stats.baq_reads += cnt[6];
    eng->stats.baq_fp64_escalated_reads += u64(tail[1]) + esc1 + esc2;
    for (int c = 0; c < 3; c++) {
        eng->stats.baq_reads_by_band[c] += n_cls[c];
        eng->stats.baq_band_cells[c] += cells[c];
    }
    eng->stats.baq_escalated_by_cause[0] += cause[0];
    eng->stats.baq_escalated_by_cause[1] += cause[1];
    eng->stats.baq_escalated_undecided_rows += cause[3];
    eng->stats.baq_escalated_by_band[0] += tail[1];
    eng->stats.baq_escalated_by_band[1] += u64(esc1) + esc2;
    if (timed_paths) {
        const int ids[4] = {14, 15, 12, 13};
        for (int k = 0; k < 4; k++)
            if (cudaEventElapsedTime(&ms, eng->ev[3], eng->ev[ids[k]]) == cudaSuccess) eng->stats.baq_path_ms[k] += ms;
    }
    if (timed_main && cudaEventElapsedTime(&ms, eng->ev[10], eng->ev[11]) == cudaSuccess) {
        eng->stats.baq_main_ms += ms;
        eng->stats.baq_main_launches++;
    }
    eng->stats.num_batches++;
    eng->last_R = R;
    eng->last_Q = Q;
    return FP_OK;
}

// ---- coalescing of small host batches ----
// Array i of a batch view counts reads (dim 0), cigar ops (1), read words (2) or qualities (3).
static const int kCoDim[17] = {0, 0, 0, 0, 0, 1, 0, 0, 2, 0, 0, 3, 0, 0, 0, 0, 0};
static const int kCoElem[17] = {2, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 1, 4, 4, 2, 1, 4};

// The checks of k_validate, on the host, so that a malformed batch is refused at its own submit.
static fp_status validate_host(fp_engine *eng, const fp_batch_view *v, const ViewArrays &va) {
    for (int i = 0; i < 17; i++)
        if (!va.src[i] && va.size[i]) return eng->fail(FP_BAD_INPUT, "null batch array");
    u32 e = 0;
    for (uint32_t r = 0; r < v->num_reads; r++) {
        if (uint64_t(v->cigar_start[r]) + v->cigar_len[r] > v->num_cigar_ops) e |= ERR_BAD_READ_RANGE;
        if (uint64_t(v->read_start[r]) + v->read_len[r] > v->num_read_symbols) e |= ERR_BAD_READ_RANGE;
        if (uint64_t(v->qual_start[r]) + v->qual_len[r] > v->num_qualities) e |= ERR_BAD_READ_RANGE;
        if (v->read_len[r] > MAX_READ_LEN) e |= ERR_READ_TOO_LONG;
        if (v->read_group[r] != U32_NONE && v->read_group[r] >= eng->n_rg) e |= ERR_BAD_READ_GROUP;
    }
    if (!e) return FP_OK;
    std::string m = "batch rejected:";
    if (e & ERR_BAD_READ_RANGE) m += " read/cigar/quality range outside the batch arrays;";
    if (e & ERR_READ_TOO_LONG) m += " read longer than 511 bases (10-bit cycle covariate);";
    if (e & ERR_BAD_READ_GROUP) m += " read group id >= num_read_groups;";
    return eng->fail(FP_BAD_INPUT, m);
}

// Processes the staged reads as one device batch (nothing to do when none are staged).
static fp_status co_flush(fp_engine *eng) {
    if (eng->co_n[0] == 0) return FP_OK;
    char *base = eng->co_buf.as<char>();
    const void *p[17];
    for (int i = 0; i < 17; i++) p[i] = base + eng->co_off[i];
    fp_batch_view v;
    v.num_reads = uint32_t(eng->co_n[0]);
    v.num_cigar_ops = uint32_t(eng->co_n[1]);
    v.num_read_symbols = eng->co_n[2] * 8;
    v.num_qualities = eng->co_n[3];
    v.chromosome = (const uint16_t *)p[0];
    v.alignment_start = (const uint32_t *)p[1];
    v.alignment_stop = (const uint32_t *)p[2];
    v.mate_alignment_start = (const uint32_t *)p[3];
    v.inferred_insert_size = (const int32_t *)p[4];
    v.cigars = (const uint32_t *)p[5];
    v.cigar_start = (const uint32_t *)p[6];
    v.cigar_len = (const uint32_t *)p[7];
    v.reads = (const uint32_t *)p[8];
    v.read_start = (const uint32_t *)p[9];
    v.read_len = (const uint32_t *)p[10];
    v.qualities = (const uint8_t *)p[11];
    v.qual_start = (const uint32_t *)p[12];
    v.qual_len = (const uint32_t *)p[13];
    v.flags = (const uint16_t *)p[14];
    v.mapq = (const uint8_t *)p[15];
    v.read_group = (const uint32_t *)p[16];
    const uint64_t batches = eng->stats.num_batches;
    const fp_status s = submit(eng, &v, true);
    for (auto &x : eng->co_n) x = 0;
    eng->stats.num_batches = batches;  // input batches are counted as they are staged
    return s;
}

static fp_status co_submit(fp_engine *eng, const fp_batch_view *v) {
    if (eng->finalized) return eng->fail(FP_NOT_READY, "submit after finalize; call fp_engine_reset first");
    if (v->num_reads == 0) {
        eng->stats.num_batches++;
        return FP_OK;
    }
    CK(cudaSetDevice(eng->device), "set device");
    const ViewArrays va = view_arrays(v);
    fp_status s = validate_host(eng, v, va);
    if (s != FP_OK) return s;
    const uint64_t need[4] = {v->num_reads, v->num_cigar_ops, (v->num_read_symbols + 7) / 8, v->num_qualities};
    if (need[0] >= eng->co_target) {  // large enough alone: the staged reads first, then this batch
        s = co_flush(eng);
        if (s != FP_OK) return s;
        return submit(eng, v, false);
    }
    // the staged batch must stay within the 32-bit counts and offsets of a batch view
    const uint64_t lim[4] = {0xFFFFFFFFull, 0xFFFFFFFFull, 0xFFFFFFFFull / 8, 0xFFFFFFFFull};
    bool fits = true, room = true;
    for (int d = 0; d < 4; d++) {
        if (eng->co_n[d] + need[d] > lim[d]) fits = false;
        if (eng->co_n[d] + need[d] > eng->co_cap[d]) room = false;
    }
    if (!fits || !room) {
        s = co_flush(eng);
        if (s != FP_OK) return s;
    }
    if (!room) {
        // (empty now) capacity for about two targets' worth of reads at this batch's density
        uint64_t cap[4];
        cap[0] = std::max<uint64_t>(2ull * eng->co_target, need[0]);
        for (int d = 1; d < 4; d++)
            cap[d] = std::max<uint64_t>(eng->co_cap[d],
                                        std::max<uint64_t>(need[d], (2ull * eng->co_target * need[d] + need[0] - 1) / need[0]));
        size_t total = 0, off[17];
        for (int i = 0; i < 17; i++) {
            off[i] = total;
            total += al(std::max<uint64_t>(1, cap[kCoDim[i]]) * kCoElem[i]);
        }
        eng->co_buf.release();
        CK(eng->co_buf.ensure(total), "coalescing buffer");
        for (int i = 0; i < 17; i++) eng->co_off[i] = off[i];
        for (int d = 0; d < 4; d++) eng->co_cap[d] = cap[d];
    }
    cudaStream_t st = eng->st;
    char *base = eng->co_buf.as<char>();
    for (int i = 0; i < 17; i++) {
        if (!va.size[i]) continue;
        CK(cudaMemcpyAsync(base + eng->co_off[i] + eng->co_n[kCoDim[i]] * kCoElem[i], va.src[i], va.size[i],
                           cudaMemcpyHostToDevice, st), "coalescing copy");
    }
    u32 *starts[3];
    const int idx[3] = {6, 9, 12};  // cigar_start, read_start, qual_start
    for (int k = 0; k < 3; k++)
        starts[k] = reinterpret_cast<u32 *>(base + eng->co_off[idx[k]]) + eng->co_n[0];
    launch_rebase_starts(starts[0], starts[1], starts[2], v->num_reads, u32(eng->co_n[1]), u32(eng->co_n[2] * 8),
                         u32(eng->co_n[3]), st);
    CK(cudaGetLastError(), "coalescing rebase");
    CK(cudaStreamSynchronize(st), "coalescing copy");  // the host buffers may be reused from here on
    for (int d = 0; d < 4; d++) eng->co_n[d] += need[d];
    eng->stats.num_batches++;
    if (eng->co_n[0] >= eng->co_target) return co_flush(eng);
    return FP_OK;
}

}  // extern "C"

extern "C" {

static fp_status finalize_impl(fp_engine *eng) {
    if (!eng) return FP_BAD_INPUT;
    CK(cudaSetDevice(eng->device), "set device");
    if (eng->co_target && !eng->finalized) {
        const fp_status s0 = co_flush(eng);
        if (s0 != FP_OK) return s0;
    }
    cudaStream_t st = eng->st;
    CK(fold_harvest(eng), "sort + fold");
    cudaEventRecord(eng->ev[7], st);
    const KeySpace ks = eng->tables.ks;
    const u32 T = ks.total;
    launch_merge_stage(eng->tables, st);
    eng->staged_bases = 0;
    DevBuf flags, pos, rows, rkey, robs, rmism, rexp, rest, rcoef, remp, rg, tmp;
    auto cleanup = [&]() {
        DevBuf *bs[] = {&flags, &pos, &rows, &rkey, &robs, &rmism, &rexp, &rest, &rcoef, &remp, &rg, &tmp};
        for (DevBuf *x : bs) x->release();
    };
    auto bail = [&](cudaError_t e, const char *w) {
        cleanup();
        return eng->cuda_fail(e, w);
    };
#define CKF(call, where)                          \
    do {                                          \
        cudaError_t _e = (call);                  \
        if (_e != cudaSuccess) return bail(_e, where); \
    } while (0)
    CKF(flags.ensure(al(T * 4ull + 4)), "finalize");
    CKF(pos.ensure(al(T * 4ull + 8)), "finalize");
    CKF(tmp.ensure(scan_tmp_bytes(T)), "finalize");
    launch_mark_nonzero(eng->tables, flags.as<u32>(), st);
    launch_exclusive_scan(flags.as<u32>(), pos.as<u32>(), T, tmp.p, st);
    u32 nrows = 0;
    CKF(cudaMemcpyAsync(&nrows, pos.as<u32>() + T, 4, cudaMemcpyDeviceToHost, st), "finalize");
    CKF(cudaStreamSynchronize(st), "finalize");
    const size_t n = std::max<u32>(nrows, 1);
    CKF(rows.ensure(n * 4), "finalize");
    CKF(rkey.ensure(n * 4), "finalize");
    CKF(robs.ensure(n * 8), "finalize");
    CKF(rmism.ensure(n * 8), "finalize");
    CKF(rexp.ensure(n * 8), "finalize");
    CKF(rest.ensure(n * 8), "finalize");
    CKF(rcoef.ensure((n + 768) * 8), "finalize");
    CKF(remp.ensure((n + 768) * 8), "finalize");
    CKF(rg.ensure(768 * 8 * 3 + 768 * 8 * 3), "finalize");
    launch_gather_rows(eng->tables, flags.as<u32>(), pos.as<u32>(), rows.as<u32>(), st);
    launch_rows(eng->tables, rows.as<u32>(), nrows, rkey.as<u32>(), robs.as<u64>(), rmism.as<double>(),
                rexp.as<double>(), rest.as<double>(), st);
    u64 *rg_obs = rg.as<u64>();
    double *rg_mism = reinterpret_cast<double *>(rg_obs + 768);
    double *rg_exp = rg_mism + 768;
    launch_rg_fold(eng->tables, rg_obs, rg_mism, rg_exp, st);

    std::vector<u32> key(nrows), dense(nrows);
    std::vector<u64> obs(nrows);
    std::vector<double> mism(nrows), ex(nrows), est(nrows);
    const u32 ng = ks.n_rg * 3;
    std::vector<u64> g_obs(ng);
    std::vector<double> g_mism(ng), g_exp(ng);
    if (nrows) {
        CKF(cudaMemcpyAsync(key.data(), rkey.p, nrows * 4ull, cudaMemcpyDeviceToHost, st), "finalize");
        CKF(cudaMemcpyAsync(dense.data(), rows.p, nrows * 4ull, cudaMemcpyDeviceToHost, st), "finalize");
        CKF(cudaMemcpyAsync(obs.data(), robs.p, nrows * 8ull, cudaMemcpyDeviceToHost, st), "finalize");
        CKF(cudaMemcpyAsync(mism.data(), rmism.p, nrows * 8ull, cudaMemcpyDeviceToHost, st), "finalize");
        CKF(cudaMemcpyAsync(ex.data(), rexp.p, nrows * 8ull, cudaMemcpyDeviceToHost, st), "finalize");
        CKF(cudaMemcpyAsync(est.data(), rest.p, nrows * 8ull, cudaMemcpyDeviceToHost, st), "finalize");
    }
    CKF(cudaMemcpyAsync(g_obs.data(), rg_obs, ng * 8ull, cudaMemcpyDeviceToHost, st), "finalize");
    CKF(cudaMemcpyAsync(g_mism.data(), rg_mism, ng * 8ull, cudaMemcpyDeviceToHost, st), "finalize");
    CKF(cudaMemcpyAsync(g_exp.data(), rg_exp, ng * 8ull, cudaMemcpyDeviceToHost, st), "finalize");
    CKF(cudaStreamSynchronize(st), "finalize");

    // read-group rows (keys rg<<10 | ev) and the host libm values of the empirical-quality model
    std::vector<u32> gkey;
    std::vector<u64> gobs;
    std::vector<double> gmism, gexp, gest;
    for (u32 i = 0; i < ng; i++) {
        if (!g_obs[i]) continue;
        gkey.push_back(((i / 3) << 10) | (i % 3));
        gobs.push_back(g_obs[i]);
        gmism.push_back(g_mism[i]);
        gexp.push_back(g_exp[i]);
        gest.push_back(double(-10.0 * log10(g_exp[i] / double(g_obs[i]))));
    }
    const u32 ngr = u32(gkey.size());
    std::vector<double> coef(size_t(nrows) + ngr);
    for (u32 i = 0; i < nrows; i++) coef[i] = binomial_coef(obs[i], mism[i]);
    for (u32 i = 0; i < ngr; i++) coef[size_t(nrows) + i] = binomial_coef(gobs[i], gmism[i]);

    // empirical qualities: table rows (rounded prior) and read-group rows (truncated prior)
    double *d_coef = rcoef.as<double>();
    double *d_emp = remp.as<double>();
    if (nrows + ngr)
        CKF(cudaMemcpyAsync(d_coef, coef.data(), (size_t(nrows) + ngr) * 8, cudaMemcpyHostToDevice, st), "finalize");
    launch_empirical(nrows, robs.as<u64>(), rmism.as<double>(), rest.as<double>(), d_coef, 1, d_emp, st);
    DevBuf gb;
    if (ngr) {
        CKF(gb.ensure(ngr * 24ull), "finalize");
        u64 *gdo = gb.as<u64>();
        double *gdm = reinterpret_cast<double *>(gdo + ngr);
        double *gde = gdm + ngr;
        CKF(cudaMemcpyAsync(gdo, gobs.data(), ngr * 8ull, cudaMemcpyHostToDevice, st), "finalize");
        CKF(cudaMemcpyAsync(gdm, gmism.data(), ngr * 8ull, cudaMemcpyHostToDevice, st), "finalize");
        CKF(cudaMemcpyAsync(gde, gest.data(), ngr * 8ull, cudaMemcpyHostToDevice, st), "finalize");
        launch_empirical(ngr, gdo, gdm, gde, d_coef + nrows, 0, d_emp + nrows, st);
    }
    std::vector<double> emp(size_t(nrows) + ngr);
    if (nrows + ngr)
        CKF(cudaMemcpyAsync(emp.data(), d_emp, (size_t(nrows) + ngr) * 8, cudaMemcpyDeviceToHost, st), "finalize");
    CK(cudaGetLastError(), "postprocess launch");
    cudaEventRecord(eng->ev[8], st);
    CKF(cudaStreamSynchronize(st), "finalize");
    gb.release();
    cleanup();
#undef CKF

    for (auto &t : eng->out) t = HostTable();
    HostTable &tg = eng->out[FP_TABLE_READ_GROUP];
    tg.keys = gkey;
    tg.obs = gobs;
    tg.mism = gmism;
    tg.exp = gexp;
    tg.est = gest;
    tg.emp.assign(emp.begin() + nrows, emp.end());
    // rows ascend in dense index: quality rows, then cycle rows, then context rows (the dense ranges are
    // ordered), so the table of a row follows from its dense index
    for (u32 i = 0; i < nrows; i++) {
        const u32 d = dense[i];
        const int t = d < ks.cycle_base ? FP_TABLE_QUALITY : (d < ks.context_base ? FP_TABLE_CYCLE : FP_TABLE_CONTEXT);
        HostTable &h = eng->out[t];
        h.keys.push_back(key[i]);
        h.obs.push_back(obs[i]);
        h.mism.push_back(mism[i]);
        h.exp.push_back(ex[i]);
        h.est.push_back(est[i]);
        h.emp.push_back(emp[i]);
    }
    float ms;
    if (cudaEventElapsedTime(&ms, eng->ev[7], eng->ev[8]) == cudaSuccess)
        eng->stats.gpu_ms_per_stage[FP_STAGE_POSTPROCESS] += ms;
    eng->finalized = true;
    return FP_OK;
}

fp_status fp_engine_get_table(fp_engine *eng, int32_t id, fp_table_view *out) {
    if (!eng || !out || id < 0 || id > 3) return FP_BAD_INPUT;
    if (!eng->finalized) return eng->fail(FP_NOT_READY, "tables are available after fp_engine_finalize");
    const HostTable &h = eng->out[id];
    out->num_rows = uint32_t(h.keys.size());
    out->keys = h.keys.data();
    out->observations = h.obs.data();
    out->mismatches = h.mism.data();
    out->expected_errors = h.exp.data();
    out->estimated_quality = h.est.data();
    out->empirical_quality = h.emp.data();
    return FP_OK;
}

static fp_status write_report_impl(fp_engine *eng, const char *path, const char *const *rg_names,
                                   uint32_t num_rg_names, int disable_rounding, int vmaj, int vmin, int vrev) {
    if (!eng) return FP_BAD_INPUT;
    if (!eng->finalized) return eng->fail(FP_NOT_READY, "write_report needs fp_engine_finalize first");
    fp_table_view t[4];
    for (int i = 0; i < 4; i++) fp_engine_get_table(eng, i, &t[i]);
    const fp_status s = fp_report_write(path, t, rg_names, num_rg_names, disable_rounding, vmaj, vmin, vrev);
    if (s != FP_OK) eng->err = "cannot open report output";
    return s;
}

fp_status fp_engine_reset(fp_engine *eng) {
    if (!eng) return FP_BAD_INPUT;
    CK(cudaSetDevice(eng->device), "set device");
    CK(fold_harvest(eng), "sort + fold");
    const size_t n = eng->tables.ks.total;
    CK(cudaMemsetAsync(eng->tab_obs.p, 0, n * sizeof(unsigned long long), eng->st), "reset");
    CK(cudaMemsetAsync(eng->tab_mism.p, 0, n * sizeof(float), eng->st), "reset");
    CK(cudaMemsetAsync(eng->tab_stage.p, 0, n * sizeof(u32), eng->st), "reset");
    CK(cudaMemsetAsync(eng->tab_cyc.p, 0, size_t(eng->n_rg) * 2 * CYC_DIFF_LEN * sizeof(int), eng->st), "reset");
    eng->staged_bases = 0;
    for (auto &x : eng->co_n) x = 0;  // staged reads of the previous job are dropped
    if (eng->prec_acc.p) CK(cudaMemsetAsync(eng->prec_acc.p, 0, sizeof(PrecisionAcc), eng->st), "reset");
    CK(cudaStreamSynchronize(eng->st), "reset");
    for (auto &t : eng->out) t = HostTable();
    eng->finalized = false;
    eng->stats = fp_stats{};
    eng->launch_base = g_kernel_launches;
    return FP_OK;
}

fp_status fp_engine_get_stats(const fp_engine *eng, fp_stats *out) {
    if (!eng || !out) return FP_BAD_INPUT;
    *out = eng->stats;
    out->gpu_kernel_launches = g_kernel_launches - eng->launch_base;
    return FP_OK;
}

fp_status fp_engine_get_precision_stats(fp_engine *eng, fp_precision_stats *out) {
    if (!eng || !out) return FP_BAD_INPUT;
    *out = fp_precision_stats{};
    if (!eng->prec_acc.p) return FP_OK;
    CK(cudaSetDevice(eng->device), "set device");
    PrecisionAcc a{};
    CK(cudaMemcpyAsync(&a, eng->prec_acc.p, sizeof(a), cudaMemcpyDeviceToHost, eng->st), "D2H");
    CK(cudaStreamSynchronize(eng->st), "precision stats");
    static_assert(PREC_BINS == sizeof(out->err_hist) / sizeof(out->err_hist[0]), "histogram bins");
    out->reads = a.reads;
    out->reads_without_fp32 = a.reads_without_fp32;
    out->bases = a.bases;
    out->bound_violations = a.violations;
    float f;
    memcpy(&f, &a.max_err_bits, 4);
    out->max_abs_error = f;
    memcpy(&f, &a.max_width_bits, 4);
    out->max_half_width = f;
    for (int i = 0; i < PREC_BINS; i++) {
        out->err_hist[i] = a.err_hist[i];
        out->width_hist[i] = a.width_hist[i];
    }
    return FP_OK;
}

static fp_status debug_last_batch_impl(fp_engine *eng, uint8_t *read_status, uint16_t *windows, int16_t *hmm,
                                       uint8_t *base_flags, uint8_t *baq_tag, double *frac_errors) {
    if (!eng) return FP_BAD_INPUT;
    CK(cudaSetDevice(eng->device), "set device");
    CK(cudaStreamSynchronize(eng->st), "debug");
    const uint32_t R = eng->last_R;
    const uint64_t Q = eng->last_Q;
    const BatchWork &w = eng->work;
    if (read_status) CK(cudaMemcpy(read_status, w.status, R, cudaMemcpyDeviceToHost), "debug");
    if (windows) CK(cudaMemcpy(windows, w.win, R * 16ull, cudaMemcpyDeviceToHost), "debug");
    if (hmm) {
        std::vector<int16_t> hw(size_t(R) * 2);
        std::vector<uint16_t> bw(R), ne(R);
        CK(cudaMemcpy(hw.data(), w.hmm, R * 4ull, cudaMemcpyDeviceToHost), "debug");
        CK(cudaMemcpy(bw.data(), w.bw, R * 2ull, cudaMemcpyDeviceToHost), "debug");
        CK(cudaMemcpy(ne.data(), w.nerr, R * 2ull, cudaMemcpyDeviceToHost), "debug");
        for (uint32_t r = 0; r < R; r++) {
            hmm[r * 4 + 0] = hw[r * 2];
            hmm[r * 4 + 1] = hw[r * 2 + 1];
            hmm[r * 4 + 2] = int16_t(bw[r]);
            hmm[r * 4 + 3] = int16_t(ne[r]);
        }
    }
    if (base_flags) CK(cudaMemcpy(base_flags, w.bflags, Q, cudaMemcpyDeviceToHost), "debug");
    if (baq_tag) CK(cudaMemcpy(baq_tag, w.tag, Q, cudaMemcpyDeviceToHost), "debug");
    if (frac_errors) {
        std::vector<float> f(Q * 3);
        CK(cudaMemcpy(f.data(), w.frac, Q * 12, cudaMemcpyDeviceToHost), "debug");
        for (uint64_t i = 0; i < Q * 3; i++) frac_errors[i] = f[i];
    }
    return FP_OK;
}

fp_status fp_host_alloc(size_t bytes, void **out) {
    if (!out) return FP_BAD_INPUT;
    return cudaMallocHost(out, bytes ? bytes : 1) == cudaSuccess ? FP_OK : FP_OOM;
}

void fp_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"

// ---- C entry points that allocate host memory, guarded (see `guarded`) ----
extern "C" {

fp_status fp_engine_set_known_sites(fp_engine *eng, uint32_t id, const uint32_t *start, const uint32_t *stop,
                                    uint32_t n) {
    return guarded(eng, [&] { return set_known_sites_impl(eng, id, start, stop, n); });
}

fp_status fp_engine_attach_refstore(fp_engine *eng, fp_refstore *store) {
    return guarded(eng, [&] { return attach_refstore_impl(eng, store); });
}

fp_status fp_engine_prefetch_batch(fp_engine *eng, const fp_batch_view *v) {
    return guarded(eng, [&] { return prefetch_batch_impl(eng, v); });
}

fp_status fp_engine_submit_batch(fp_engine *eng, const fp_batch_view *v) {
    return guarded(eng, [&] { return submit_batch_impl(eng, v); });
}

fp_status fp_engine_submit_batch_device(fp_engine *eng, const fp_batch_view *v) {
    return guarded(eng, [&] { return submit_batch_device_impl(eng, v); });
}

fp_status fp_engine_finalize(fp_engine *eng) {
    return guarded(eng, [&] { return finalize_impl(eng); });
}

fp_status fp_engine_write_report(fp_engine *eng, const char *path, const char *const *rg_names, uint32_t num_rg_names,
                                 int disable_rounding, int vmaj, int vmin, int vrev) {
    return guarded(eng, [&] {
        return write_report_impl(eng, path, rg_names, num_rg_names, disable_rounding, vmaj, vmin, vrev);
    });
}

fp_status fp_engine_debug_last_batch(fp_engine *eng, uint8_t *read_status, uint16_t *windows, int16_t *hmm,
                                     uint8_t *base_flags, uint8_t *baq_tag, double *frac_errors) {
    return guarded(eng, [&] {
        return debug_last_batch_impl(eng, read_status, windows, hmm, base_flags, baq_tag, frac_errors);
    });
}

fp_status fp_engine_create(const fp_options *o, fp_engine **out) {
    return guarded(nullptr, [&] { return create_impl(o, out); });
}

}  // extern "C"
