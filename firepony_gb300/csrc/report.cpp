// GATKReport v1.1 writer for the recalibration tables. The layout is the reference's output format and must
// stay byte-identical: the fixed header and Arguments table (device/pipeline.cu:150-204), the dummy
// Quantized table, RecalTable0 (device/read_group_table.cu:96-143), RecalTable1
// (device/covariates/packer_quality_score.h:57-117) and RecalTable2 with context rows then cycle rows
// (device/covariates.cu:285-311, packer_context.h, packer_cycle_illumina.h). Tables are written in two
// passes: the first measures column widths, the second prints (table_formatter.cu:34-231); floats are
// rounded with round(v*10^n)/10^n before printf (device/util.cu:107-116).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "firepony_gb300.h"

namespace {

enum Fmt { STRING, CHAR, UINT64, FLOAT2, FLOAT4 };
enum Align { LEFT, RIGHT };

struct Column {
    std::string name;
    Fmt fmt;
    Align align, header_align;
    size_t width;
};

double round_n(double v, int n) {
    v = v * pow(10.0, n);
    v = round(v);
    return v / pow(10.0, n);
}

class Table {
  public:
    Table(FILE *f, std::string name, std::string description, bool raw)
        : f_(f), name_(std::move(name)), desc_(std::move(description)), raw_(raw) {}

    void column(const std::string &name, Fmt fmt, int align = -1, int header_align = -1) {
        Align a = align >= 0 ? Align(align) : ((fmt == STRING || fmt == CHAR) ? LEFT : RIGHT);
        Align h = header_align >= 0 ? Align(header_align) : a;
        cols_.push_back(Column{name, fmt, a, h, name.size()});
    }
    void start_row() {
        col_ = 0;
        rows_++;
    }
    void end_row() {
        if (!measuring_) fputc('\n', f_);
    }
    void str(const std::string &v) { cell(v); }
    void chr(char c) { cell(std::string(1, c)); }
    void u64v(uint64_t v) {
        char b[64];
        snprintf(b, sizeof(b), "%lu", (unsigned long)v);
        cell(b);
    }
    void dbl(double v) {
        char b[256];
        const Fmt fmt = cols_[col_].fmt;
        if (raw_) {
            snprintf(b, sizeof(b), "%.64f", v);
        } else if (fmt == FLOAT2) {
            snprintf(b, sizeof(b), "%.2f", round_n(v, 2));
        } else {
            snprintf(b, sizeof(b), "%.4f", round_n(v, 4));
        }
        cell(b);
    }
    void int_str(int v) {
        char b[32];
        snprintf(b, sizeof(b), "%d", v);
        cell(b);
    }
    void end_table() {
        if (measuring_) {
            measuring_ = false;
            fprintf(f_, "#:GATKTable:%d:%d:", int(cols_.size()), int(rows_));
            for (const Column &c : cols_) {
                switch (c.fmt) {
                case STRING: case CHAR: fputs("%s:", f_); break;
                case UINT64: fputs("%d:", f_); break;
                case FLOAT2: fputs(raw_ ? "%.64f:" : "%.2f:", f_); break;
                case FLOAT4: fputs(raw_ ? "%.64f:" : "%.4f:", f_); break;
                }
            }
            fputs(";\n", f_);
            fprintf(f_, "#:GATKTable:%s:%s\n", name_.c_str(), desc_.c_str());
            for (size_t i = 0; i < cols_.size(); i++) {
                pad(cols_[i].name, cols_[i].width, cols_[i].header_align);
                fputs(i + 1 == cols_.size() ? "\n" : "  ", f_);
            }
        } else {
            fputc('\n', f_);
        }
    }

  private:
    void pad(const std::string &v, size_t width, Align a) {
        if (a == RIGHT) fprintf(f_, "%*s", int(width), v.c_str());
        else fprintf(f_, "%-*s", int(width), v.c_str());
    }
    void cell(const std::string &v) {
        Column &c = cols_[col_];
        if (measuring_) {
            if (v.size() > c.width) c.width = v.size();
        } else {
            pad(v, c.width, c.align);
            if (col_ + 1 < cols_.size()) fputs("  ", f_);
        }
        col_++;
    }

    FILE *f_;
    std::string name_, desc_;
    bool raw_;
    std::vector<Column> cols_;
    size_t col_ = 0;
    size_t rows_ = 0;
    bool measuring_ = true;
};

const char EV_CHAR[4] = {'M', 'I', 'D', 'S'};
const char DNA_CHAR[5] = {'A', 'C', 'G', 'T', 'N'};

const std::string &rg_name(const char *const *names, uint32_t n, uint32_t id, std::string &tmp) {
    if (id < n && names[id]) tmp = names[id];
    else tmp = std::to_string(id);
    return tmp;
}

}  // namespace

static fp_status report_write(FILE *f, const fp_table_view *tables, const char *const *rg_names,
                              uint32_t num_rg_names, int disable_rounding, int vmaj, int vmin, int vrev);

// The writer's strings and vectors may fail to allocate: that is reported as FP_OOM (with the file closed),
// never as an exception through the C ABI.
extern "C" fp_status fp_report_write(const char *path, const fp_table_view *tables, const char *const *rg_names,
                                     uint32_t num_rg_names, int disable_rounding, int vmaj, int vmin, int vrev) {
    FILE *f = (path && *path) ? fopen(path, "w") : stdout;
    if (!f) return FP_BAD_INPUT;
    fp_status st;
    try {
        st = report_write(f, tables, rg_names, num_rg_names, disable_rounding, vmaj, vmin, vrev);
    } catch (...) {
        if (f != stdout) fclose(f);
        return FP_OOM;
    }
    return st;
}

static fp_status report_write(FILE *f, const fp_table_view *tables, const char *const *rg_names,
                              uint32_t num_rg_names, int disable_rounding, int vmaj, int vmin, int vrev) {
    const bool raw = disable_rounding != 0;
    // header and Arguments table (device/pipeline.cu:150-178)
    fputs("#:GATKReport.v1.1:5\n", f);
    fputs("#:GATKTable:2:18:%s:%s:;\n", f);
    fputs("#:GATKTable:Arguments:Recalibration argument collection values used in this run\n", f);
    static const char *args[][2] = {
        {"Argument", "Value"},
        {"binary_tag_name", "null"},
        {"covariate", "ReadGroupCovariate,QualityScoreCovariate,ContextCovariate,CycleCovariate"},
        {"default_platform", "null"},
        {"deletions_default_quality", "45"},
        {"force_platform", "null"},
        {"indels_context_size", "3"},
        {"insertions_default_quality", "45"},
        {"low_quality_tail", "2"},
        {"maximum_cycle_value", "500"},
        {"mismatches_context_size", "2"},
        {"mismatches_default_quality", "-1"},
        {"no_standard_covs", "false"},
        {"quantizing_levels", "16"},
        {"recalibration_report", "null"},
        {"run_without_dbsnp", "false"},
        {"solid_nocall_strategy", "THROW_EXCEPTION"},
        {"solid_recal_mode", "SET_Q_ZERO"},
    };
    for (auto &a : args) fprintf(f, "%-28s%-72s\n", a[0], a[1]);
    fprintf(f, "%-28sFirepony_%d.%d.%d%55s\n", "software", vmaj, vmin, vrev, "");
    fputc('\n', f);

    // dummy quantization table (device/pipeline.cu:180-203)
    {
        Table t(f, "Quantized", "Quality quantization map", raw);
        t.column("QualityScore", STRING, RIGHT);
        t.column("Count", STRING, RIGHT);
        t.column("QuantizedScore", STRING, RIGHT);
        for (int pass = 0; pass < 2; pass++) {
            for (int i = 0; i < 94; i++) {
                char b[32];
                snprintf(b, sizeof(b), "%d", i);
                t.start_row();
                t.str(b);
                t.str("0");
                t.str(b);
                t.end_row();
            }
            t.end_table();
        }
    }
    std::string tmp;
    // RecalTable0 (device/read_group_table.cu:96-143)
    {
        const fp_table_view &v = tables[FP_TABLE_READ_GROUP];
        Table t(f, "RecalTable0", "", raw);
        t.column("ReadGroup", STRING);
        t.column("EventType", CHAR);
        t.column("EmpiricalQuality", FLOAT4);
        t.column("EstimatedQReported", FLOAT4);
        t.column("Observations", UINT64);
        t.column("Errors", FLOAT2, RIGHT, LEFT);
        for (int pass = 0; pass < 2; pass++) {
            for (uint32_t i = 0; i < v.num_rows; i++) {
                const uint32_t k = v.keys[i];
                t.start_row();
                t.str(rg_name(rg_names, num_rg_names, (k >> 10) & 0xFF, tmp));
                t.chr(EV_CHAR[k & 3]);
                t.dbl(v.empirical_quality[i]);
                t.dbl(v.estimated_quality[i]);
                t.u64v(v.observations[i]);
                t.dbl(v.mismatches[i]);
                t.end_row();
            }
            t.end_table();
        }
    }
    // RecalTable1 (packer_quality_score.h:57-117)
    {
        const fp_table_view &v = tables[FP_TABLE_QUALITY];
        Table t(f, "RecalTable1", "", raw);
        t.column("ReadGroup", STRING);
        t.column("QualityScore", STRING);
        t.column("EventType", CHAR);
        t.column("EmpiricalQuality", FLOAT4);
        t.column("Observations", UINT64);
        t.column("Errors", FLOAT2, RIGHT, LEFT);
        for (int pass = 0; pass < 2; pass++) {
            for (uint32_t i = 0; i < v.num_rows; i++) {
                if (v.observations[i] == 0) continue;
                const uint32_t k = v.keys[i];
                char qb[16];
                snprintf(qb, sizeof(qb), "%d", int((k >> 2) & 0xFF));
                t.start_row();
                t.str(rg_name(rg_names, num_rg_names, (k >> 10) & 0xFF, tmp));
                t.str(qb);
                t.chr(EV_CHAR[k & 3]);
                t.dbl(v.empirical_quality[i]);
                t.u64v(v.observations[i]);
                t.dbl(v.mismatches[i]);
                t.end_row();
            }
            t.end_table();
        }
    }
    // RecalTable2: context rows then cycle rows (device/covariates.cu:285-311)
    {
        const fp_table_view &cx = tables[FP_TABLE_CONTEXT];
        const fp_table_view &cy = tables[FP_TABLE_CYCLE];
        Table t(f, "RecalTable2", "", raw);
        t.column("ReadGroup", STRING);
        t.column("QualityScore", STRING);
        t.column("CovariateValue", STRING);
        t.column("CovariateName", STRING);
        t.column("EventType", CHAR);
        t.column("EmpiricalQuality", FLOAT4);
        t.column("Observations", UINT64);
        t.column("Errors", FLOAT2, RIGHT, LEFT);
        for (int pass = 0; pass < 2; pass++) {
            for (uint32_t i = 0; i < cx.num_rows; i++) {
                if (cx.observations[i] == 0) continue;
                const uint32_t k = cx.keys[i];
                const uint32_t raw_ctx = (k >> 2) & 0x7FF;
                const int size = int(raw_ctx & 15);
                const uint32_t ctx = raw_ctx >> 4;
                std::string seq;
                for (int j = 0; j < size; j++) seq.push_back(DNA_CHAR[(ctx >> (j * 2)) & 3]);
                t.start_row();
                t.str(rg_name(rg_names, num_rg_names, (k >> 21) & 0xFF, tmp));
                t.int_str(int((k >> 13) & 0xFF));
                t.str(seq);
                t.str("Context");
                t.chr(EV_CHAR[k & 3]);
                t.dbl(cx.empirical_quality[i]);
                t.u64v(cx.observations[i]);
                t.dbl(cx.mismatches[i]);
                t.end_row();
            }
            for (uint32_t i = 0; i < cy.num_rows; i++) {
                if (cy.observations[i] == 0) continue;
                const uint32_t k = cy.keys[i];
                const uint32_t raw_group = (k >> 2) & 0x3FF;
                int group = int(raw_group >> 1);
                if (raw_group & 1) group = -group;
                t.start_row();
                t.str(rg_name(rg_names, num_rg_names, (k >> 20) & 0xFF, tmp));
                t.int_str(int((k >> 12) & 0xFF));
                t.int_str(group);
                t.str("Cycle");
                t.chr(EV_CHAR[k & 3]);
                t.dbl(cy.empirical_quality[i]);
                t.u64v(cy.observations[i]);
                t.dbl(cy.mismatches[i]);
                t.end_row();
            }
            t.end_table();
        }
    }
    if (f != stdout) fclose(f);
    return FP_OK;
}
