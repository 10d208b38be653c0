// superdca-gb300: SuperDCA's command line on the GB300 engine.
//
// The flow follows SuperDCA's main (SuperDCA/src/SuperDCA.cpp:232-408) and
// run_plmDCA (SuperDCA/include/plmDCA.hpp:436-697):
//   read the FASTA alignment -> (filter list | MAF/gap filter) -> sample list
//   -> 4-state (triallelic) envelope -> loci list -> weights (GPU, or 1.0
//   with --no-reweighting) -> per-locus solves (GPU) -> symmetrised coupling
//   lines "%.8f r n" in <id>.SuperDCA_couplings.1-based.all.
// Option spellings and defaults are those of SuperDCA/src/SuperDCA_options.cpp:
// 155-190 and SuperDCA/src/plmDCA_options.cpp:131-150; the alignment options
// that apegrunt defines (absent from the reference tree) use the spellings of
// the reference README.  GPU options are prefixed --gpu-.
//
// The alignment rules (symbols, allele ranking, MAF and gap frequency, the
// three-allele envelope) are the ones of superdca_gb300/alignment.py, which
// the tests hold this program to.
#include <algorithm>
#include <atomic>
#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <vector>

#include "superdca_gb300.h"

namespace {

const char *USAGE =
    "superdca-gb300 [options] alignmentfile\n"
    "\n"
    "General:\n"
    "  -h [ --help ]                      Print this help message.\n"
    "  -v [ --verbose ]                   Be verbose.\n"
    "  --alignmentfile arg                The input alignment filename (FASTA).\n"
    "  --filterlistfile arg               The loci filter list input filename.\n"
    "  --output-filtered-alignment        Write filtered alignment to file.\n"
    "  --output-filterlist-alignment      Output alignment after filterlist selection.\n"
    "  --samplelistfile arg               The sample filter list input filename.\n"
    "  --output-samplelist-alignment      Output alignment after samplelist selection.\n"
    "  --locilistfile arg                 Analysable loci list filename.\n"
    "  -t [ --threads ] arg (=-1)         Host threads for output formatting (-1 = all).\n"
    "Alignment:\n"
    "  --maf-threshold arg (=0.01)        Minimum minor allele frequency of a kept locus.\n"
    "  --gap-threshold arg (=0.15)        Maximum gap frequency of a kept locus.\n"
    "  --no-filter-alignment              Keep every locus that fits the 4-state envelope.\n"
    "  --begin-locus arg (=0)             First analysed locus when no loci list is given.\n"
    "  --end-locus arg (=-1)              Last analysed locus (-1 = the last one).\n"
    "  --input-indexing-base arg (=1)     Index base of list files.\n"
    "  --output-indexing-base arg (=1)    Index base of written loci indices.\n"
    "  --no-reweighting                   Do not reweight samples.\n"
    "  --reweighting-threshold arg (=0.9) Fraction of identical positions required for two\n"
    "                                     sequences to be considered identical.\n"
    "  --output-weights                   Write sample weights to file.\n"
    "plmDCA:\n"
    "  --gradient-threshold arg (=0.001)  L-BFGS gradient threshold stopping criterion.\n"
    "  --lambda-h arg (=-1)               h regularization factor (< 0: automatic).\n"
    "  --lambda-J arg (=-1)               J regularization factor (< 0: automatic).\n"
    "  --no-dca                           Don't run DCA.\n"
    "  --no-coupling-output               Don't write coupling scores to file.\n"
    "GPU:\n"
    "  --gpu-device arg (=0)              CUDA device.\n"
    "  --gpu-devices arg                  Comma-separated CUDA devices (e.g. 0,1,2,3): one engine\n"
    "                                     per device, each solving a contiguous share of the loci.\n"
    "  --gpu-form arg (=dual)             Engine form: dual (span of the sequences), tc (tensor-core\n"
    "                                     contractions) or plain.\n"
    "  --gpu-batch arg                    Loci solved together per lane (default: autotuned;\n"
    "                                     512 dual, 64 otherwise without the autotuner).\n"
    "  --gpu-lanes arg                    Solver lanes, each with its own stream and host thread\n"
    "                                     (default: autotuned; 4 dual, 1 otherwise without it).\n"
    "  --gpu-no-autotune                  Do not measure batch and lanes on the first loci.\n"
    "  --gpu-tune-cache arg               File that keeps the autotuner's choice per shape.\n"
    "  --gpu-warm-start arg               Learned start: a parameter blob (.npy of float32, or raw\n"
    "                                     float32), per-sequence for the dual form, per-pair otherwise.\n"
    "  --gpu-history arg (=fp32)          L-BFGS history storage: fp32 or bf16.\n"
    "  --gpu-chunk arg (=4096)            Loci per solve call (bounds host memory).\n"
    "  --gpu-top-k arg (=0)               Write only the K strongest pairs, strongest first.\n"
    "  --gpu-binary-output                Also write <id>.SuperDCA_couplings.<base>-based.bin:\n"
    "                                     records of float score, int32 r, int32 n (little endian).\n";

struct Options {
    std::vector<std::string> alignment_files;
    std::string filterlist, samplelist, locilist;
    bool verbose = false, out_filtered = false, out_filterlist = false, out_samplelist = false;
    int threads = -1;
    double maf = 0.01, gap = 0.15;
    bool no_filter = false;
    long begin_locus = 0, end_locus = -1;
    int in_base = 1, out_base = 1;
    bool no_reweighting = false, output_weights = false;
    double reweighting_threshold = 0.9;
    bool norm_of_mean = false;
    double gradient_threshold = 1e-3, lambda_h = -1.0, lambda_J = -1.0;
    bool no_dca = false, no_coupling_output = false;
    int device = 0, batch = 0, lanes = 0, form = SDCA_FORM_DUAL;
    std::vector<int> devices;       // --gpu-devices; empty: {device}
    bool history_bf16 = false, binary_output = false;
    long chunk = 4096, top_k = 0;
    bool no_autotune = false;
    std::string tune_cache, warm_start;
};

[[noreturn]] void fail(const std::string &msg)
{
    std::cerr << "superdca-gb300 error: " << msg << "\n";
    std::exit(EXIT_FAILURE);
}

// A learned-start parameter blob: a NumPy .npy file of little-endian float32
// (format versions 1-3, C order), or raw float32 values.
std::vector<float> read_blob(const std::string &path)
{
    std::FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) fail("cannot open \"" + path + "\"");
    std::vector<unsigned char> bytes;
    unsigned char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) bytes.insert(bytes.end(), buf, buf + got);
    std::fclose(f);
    size_t off = 0;
    if (bytes.size() >= 10 && std::memcmp(bytes.data(), "\x93NUMPY", 6) == 0) {
        const int major = bytes[6];
        size_t hlen = 0, hoff = 0;
        if (major == 1) {
            hlen = (size_t)bytes[8] | ((size_t)bytes[9] << 8);
            hoff = 10;
        } else if ((major == 2 || major == 3) && bytes.size() >= 12) {
            hlen = (size_t)bytes[8] | ((size_t)bytes[9] << 8) | ((size_t)bytes[10] << 16) | ((size_t)bytes[11] << 24);
            hoff = 12;
        } else {
            fail("\"" + path + "\": unknown .npy format version");
        }
        if (hoff + hlen > bytes.size()) fail("\"" + path + "\": truncated .npy header");
        const std::string header(bytes.begin() + (long)hoff, bytes.begin() + (long)(hoff + hlen));
        if (header.find("'<f4'") == std::string::npos || header.find("'fortran_order': False") == std::string::npos)
            fail("\"" + path + "\": expected a C-ordered little-endian float32 array");
        off = hoff + hlen;
    }
    if ((bytes.size() - off) % 4 != 0) fail("\"" + path + "\": size is not a whole number of float32 values");
    std::vector<float> v((bytes.size() - off) / 4);
    std::memcpy(v.data(), bytes.data() + off, v.size() * 4);
    return v;
}

template <typename T> T parse_number(const std::string &opt, const std::string &v)
{
    T out{};
    const char *b = v.data(), *e = v.data() + v.size();
    std::from_chars_result r;
    if constexpr (std::is_floating_point_v<T>) {
        char *end = nullptr;
        out = (T)std::strtod(v.c_str(), &end);
        if (v.empty() || end != v.c_str() + v.size()) fail("invalid value '" + v + "' for " + opt);
        return out;
    } else {
        r = std::from_chars(b, e, out);
        if (r.ec != std::errc() || r.ptr != e) fail("invalid value '" + v + "' for " + opt);
        return out;
    }
}

// Boost.Program_options style: --name value, --name=value, -x value, positionals.
Options parse_options(int argc, char **argv)
{
    Options o;
    struct Flag { const char *name; bool *dst; };
    const Flag flags[] = {
        {"verbose", &o.verbose}, {"output-filtered-alignment", &o.out_filtered},
        {"output-filterlist-alignment", &o.out_filterlist},
        {"output-samplelist-alignment", &o.out_samplelist}, {"no-filter-alignment", &o.no_filter},
        {"no-reweighting", &o.no_reweighting}, {"output-weights", &o.output_weights},
        {"norm-of-mean-scoring", &o.norm_of_mean}, {"no-dca", &o.no_dca},
        {"no-coupling-output", &o.no_coupling_output}, {"gpu-binary-output", &o.binary_output},
        {"gpu-no-autotune", &o.no_autotune},
    };
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a == "-h" || a == "--help") {
            std::cout << USAGE;
            std::exit(EXIT_SUCCESS);
        }
        if (a == "-v") a = "--verbose";
        if (a == "-t") a = "--threads";
        if (a.size() < 2 || a[0] != '-' || a == "-") {
            o.alignment_files.push_back(a);
            continue;
        }
        if (a.rfind("--", 0) != 0) fail("unrecognised option '" + a + "'");
        std::string name = a.substr(2), value;
        bool has_value = false;
        const size_t eq = name.find('=');
        if (eq != std::string::npos) {
            value = name.substr(eq + 1);
            name = name.substr(0, eq);
            has_value = true;
        }
        bool matched = false;
        for (const Flag &f : flags)
            if (name == f.name) {
                if (has_value) fail("option '--" + name + "' takes no value");
                *f.dst = true;
                matched = true;
            }
        if (matched) continue;
        if (!has_value) {
            if (i + 1 >= argc) fail("option '--" + name + "' requires an argument");
            value = argv[++i];
        }
        const std::string opt = "--" + name;
        if (name == "alignmentfile") o.alignment_files.push_back(value);
        else if (name == "filterlistfile") o.filterlist = value;
        else if (name == "samplelistfile") o.samplelist = value;
        else if (name == "locilistfile") o.locilist = value;
        else if (name == "threads") o.threads = parse_number<int>(opt, value);
        else if (name == "maf-threshold") o.maf = parse_number<double>(opt, value);
        else if (name == "gap-threshold") o.gap = parse_number<double>(opt, value);
        else if (name == "begin-locus") o.begin_locus = parse_number<long>(opt, value);
        else if (name == "end-locus") o.end_locus = parse_number<long>(opt, value);
        else if (name == "input-indexing-base") o.in_base = parse_number<int>(opt, value);
        else if (name == "output-indexing-base") o.out_base = parse_number<int>(opt, value);
        else if (name == "reweighting-threshold") o.reweighting_threshold = parse_number<double>(opt, value);
        else if (name == "gradient-threshold") o.gradient_threshold = parse_number<double>(opt, value);
        else if (name == "lambda-h") o.lambda_h = parse_number<double>(opt, value);
        else if (name == "lambda-J") o.lambda_J = parse_number<double>(opt, value);
        else if (name == "gpu-device") o.device = parse_number<int>(opt, value);
        else if (name == "gpu-devices") {
            o.devices.clear();
            size_t p = 0;
            while (p <= value.size()) {
                const size_t q = std::min(value.find(',', p), value.size());
                const int d = parse_number<int>(opt, value.substr(p, q - p));
                if (d < 0) fail("--gpu-devices entries must be >= 0");
                o.devices.push_back(d);
                p = q + 1;
            }
        }
        else if (name == "gpu-batch") o.batch = parse_number<int>(opt, value);
        else if (name == "gpu-lanes") o.lanes = parse_number<int>(opt, value);
        else if (name == "gpu-tune-cache") o.tune_cache = value;
        else if (name == "gpu-warm-start") o.warm_start = value;
        else if (name == "gpu-chunk") o.chunk = parse_number<long>(opt, value);
        else if (name == "gpu-top-k") o.top_k = parse_number<long>(opt, value);
        else if (name == "gpu-form") {
            if (value == "tc") o.form = SDCA_FORM_TC;
            else if (value == "plain") o.form = SDCA_FORM_GATHER;
            else if (value == "dual") o.form = SDCA_FORM_DUAL;
            else fail("--gpu-form must be dual, tc or plain");
        } else if (name == "gpu-history") {
            if (value == "fp32") o.history_bf16 = false;
            else if (value == "bf16") o.history_bf16 = true;
            else fail("--gpu-history must be fp32 or bf16");
        } else fail("unrecognised option '" + opt + "'");
    }
    if (o.alignment_files.empty()) fail("no input alignment (see --help)");
    if (o.alignment_files.size() > 2) fail("at most two alignment files");
    if (o.gradient_threshold <= 0) fail("--gradient-threshold must be positive");
    if (o.chunk < 1) fail("--gpu-chunk must be positive");
    if (o.top_k < 0) fail("--gpu-top-k must be >= 0");
    return o;
}

// ---------------------------------------------------------------- alignment

struct Alignment {
    std::string id;                 // output file stem
    std::vector<std::string> names; // sequence headers
    int64_t N = 0, L = 0;
    std::vector<uint8_t> nuc;       // N x L codes A0 C1 G2 T3 gap4
    std::vector<int64_t> translation;  // column -> original column index
};

std::string stem(const std::string &path)
{
    std::string base = path.substr(path.find_last_of('/') == std::string::npos ? 0 : path.find_last_of('/') + 1);
    const size_t dot = base.find_last_of('.');
    return (dot == std::string::npos || dot == 0) ? base : base.substr(0, dot);
}

uint8_t nucleotide_code(unsigned char c)
{
    switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 4;   // '-', 'N' and every other symbol count as gap
    }
}

Alignment read_fasta(const std::string &path)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) fail("cannot open alignment file \"" + path + "\"");
    Alignment a;
    a.id = stem(path);
    std::vector<std::string> seqs;
    std::string line;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line.empty()) continue;
        if (line[0] == '>') {
            a.names.push_back(line.substr(1));
            seqs.emplace_back();
        } else if (line[0] == ';') {
            continue;
        } else {
            if (seqs.empty()) fail("\"" + path + "\" is not FASTA: sequence data before the first header");
            for (char c : line)
                if (!std::isspace((unsigned char)c)) seqs.back().push_back(c);
        }
    }
    if (seqs.empty()) fail("no sequences in \"" + path + "\"");
    a.N = (int64_t)seqs.size();
    a.L = (int64_t)seqs[0].size();
    for (size_t i = 0; i < seqs.size(); ++i)
        if ((int64_t)seqs[i].size() != a.L)
            fail("sequence " + std::to_string(i + 1) + " of \"" + path + "\" has length " +
                 std::to_string(seqs[i].size()) + ", expected " + std::to_string(a.L));
    a.nuc.resize((size_t)(a.N * a.L));
    for (int64_t i = 0; i < a.N; ++i)
        for (int64_t n = 0; n < a.L; ++n) a.nuc[i * a.L + n] = nucleotide_code((unsigned char)seqs[i][n]);
    a.translation.resize(a.L);
    for (int64_t n = 0; n < a.L; ++n) a.translation[n] = n;
    return a;
}

Alignment select_columns(const Alignment &a, const std::vector<int64_t> &cols)
{
    Alignment b;
    b.id = a.id;
    b.names = a.names;
    b.N = a.N;
    b.L = (int64_t)cols.size();
    b.nuc.resize((size_t)(b.N * b.L));
    for (int64_t i = 0; i < a.N; ++i)
        for (int64_t k = 0; k < b.L; ++k) b.nuc[i * b.L + k] = a.nuc[i * a.L + cols[k]];
    b.translation.resize(b.L);
    for (int64_t k = 0; k < b.L; ++k) b.translation[k] = a.translation[cols[k]];
    return b;
}

Alignment select_rows(const Alignment &a, const std::vector<int64_t> &rows, const std::string &id)
{
    Alignment b;
    b.id = id;
    b.N = (int64_t)rows.size();
    b.L = a.L;
    b.translation = a.translation;
    b.nuc.resize((size_t)(b.N * b.L));
    for (int64_t k = 0; k < b.N; ++k) {
        b.names.push_back(a.names[rows[k]]);
        std::memcpy(&b.nuc[k * b.L], &a.nuc[rows[k] * a.L], (size_t)a.L);
    }
    return b;
}

// Per-column allele counts and the rank of each nucleotide (by count, ties
// A<C<G<T); gaps are not alleles.
struct ColumnStats {
    int64_t count[5];
    int rank[4];
    int alleles;
};

std::vector<ColumnStats> column_stats(const Alignment &a)
{
    std::vector<ColumnStats> cs((size_t)a.L);
    for (auto &c : cs) std::memset(&c, 0, sizeof c);
    for (int64_t i = 0; i < a.N; ++i) {
        const uint8_t *row = &a.nuc[i * a.L];
        for (int64_t n = 0; n < a.L; ++n) ++cs[n].count[row[n]];
    }
    for (auto &c : cs) {
        int order[4] = {0, 1, 2, 3};
        std::stable_sort(order, order + 4, [&](int x, int y) { return c.count[x] > c.count[y]; });
        for (int k = 0; k < 4; ++k) c.rank[order[k]] = k;
        c.alleles = 0;
        for (int k = 0; k < 4; ++k) c.alleles += c.count[k] > 0;
    }
    return cs;
}

// MAF / gap filter: more than one allele, MAF >= maf, gap frequency <= gap.
std::vector<int64_t> filter_columns(const Alignment &a, double maf, double gap)
{
    const auto cs = column_stats(a);
    std::vector<int64_t> keep;
    for (int64_t n = 0; n < a.L; ++n) {
        const ColumnStats &c = cs[n];
        int64_t sorted[4] = {c.count[0], c.count[1], c.count[2], c.count[3]};
        std::sort(sorted, sorted + 4, [](int64_t x, int64_t y) { return x > y; });
        const int64_t nongap = a.N - c.count[4];
        const double f_minor = nongap > 0 ? (double)sorted[1] / (double)nongap : 0.0;
        const double f_gap = (double)c.count[4] / (double)a.N;
        if (c.alleles > 1 && f_minor >= maf && f_gap <= gap) keep.push_back(n);
    }
    return keep;
}

// The 4-state envelope: a locus with four alleles is dropped; the others are
// coded by allele rank (0, 1, 2) with gap = 3.
std::vector<uint8_t> four_state(const Alignment &a, std::vector<int64_t> &kept)
{
    const auto cs = column_stats(a);
    kept.clear();
    for (int64_t n = 0; n < a.L; ++n)
        if (cs[n].alleles <= 3) kept.push_back(n);
    const int64_t Lk = (int64_t)kept.size();
    std::vector<uint8_t> lut((size_t)Lk * 5);
    for (int64_t k = 0; k < Lk; ++k) {
        for (int v = 0; v < 4; ++v) lut[k * 5 + v] = (uint8_t)std::min(cs[kept[k]].rank[v], 3);
        lut[k * 5 + 4] = 3;
    }
    std::vector<uint8_t> st((size_t)(a.N * Lk));
    for (int64_t i = 0; i < a.N; ++i)
        for (int64_t k = 0; k < Lk; ++k) st[i * Lk + k] = lut[k * 5 + a.nuc[i * a.L + kept[k]]];
    return st;
}

// List files: integers separated by whitespace or commas, '#' starts a comment.
std::vector<int64_t> read_index_list(const std::string &path, int base)
{
    std::ifstream in(path);
    if (!in) fail("cannot open list file \"" + path + "\"");
    std::vector<int64_t> out;
    std::string line;
    while (std::getline(in, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        for (char &c : line)
            if (c == ',') c = ' ';
        std::istringstream ls(line);
        std::string tok;
        while (ls >> tok) {
            const int64_t v = parse_number<int64_t>("list file \"" + path + "\"", tok) - base;
            if (v < 0) fail("index " + tok + " in \"" + path + "\" is below the index base");
            out.push_back(v);
        }
    }
    return out;
}

// SuperDCA's get_unique_ofstream (SuperDCA/include/SuperDCA_commons.h:66-81):
// name, name.1, name.2, ... whichever does not exist yet.
std::string unique_name(const std::string &name)
{
    for (int index = 0;; ++index) {
        const std::string p = index == 0 ? name : name + "." + std::to_string(index);
        struct stat sb;
        if (stat(p.c_str(), &sb) != 0) return p;
    }
}

void write_fasta(const Alignment &a, const Options &o, const char *what)
{
    static const char sym[5] = {'A', 'C', 'G', 'T', '-'};
    const std::string path = unique_name(a.id + ".fasta");
    if (o.verbose) std::cout << "superdca-gb300: write " << what << " alignment to file " << path << "\n";
    std::ofstream out(path, std::ios::binary);
    std::string row((size_t)a.L, ' ');
    for (int64_t i = 0; i < a.N; ++i) {
        for (int64_t n = 0; n < a.L; ++n) row[n] = sym[a.nuc[i * a.L + n]];
        out << '>' << a.names[i] << '\n' << row << '\n';
    }
    if (!out) fail("failed to write \"" + path + "\"");
}

void write_loci(const Alignment &a, const Options &o)
{
    const std::string path = unique_name(a.id + ".loci");
    if (o.verbose) std::cout << "superdca-gb300: write original loci indices to file " << path << "\n";
    std::ofstream out(path, std::ios::binary);
    for (int64_t n = 0; n < a.L; ++n) out << a.translation[n] + o.out_base << '\n';
    if (!out) fail("failed to write \"" + path + "\"");
}

// ---------------------------------------------------------------- engine

struct Handle {
    sdca_handle *h = nullptr;
    ~Handle() { if (h) sdca_destroy(h); }
};

void check(int rc, sdca_handle *h, const char *what)
{
    if (rc != SDCA_OK) fail(std::string(what) + ": " + sdca_last_error(h));
}

// Coupling lines of mean-of-norms scoring (plmDCA.hpp:667-693): for r over
// the loci list and n over the entries before r,
// (double)(float)(S[r][n] + S[n][r]) * 0.5 with std::fixed precision 8.
void write_couplings(const std::string &path, const std::vector<float> &S, const std::vector<uint32_t> &loci,
                     const std::vector<int64_t> &translation, int base, int threads)
{
    std::FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) fail("cannot open \"" + path + "\" for writing");
    const size_t n = loci.size();
    const int T = std::max(1, threads);
    const size_t window = 64;  // rows formatted per thread per round
    std::vector<std::string> buf((size_t)T);
    for (size_t k0 = 0; k0 < n; k0 += window * T) {
        std::vector<std::thread> pool;
        for (int t = 0; t < T; ++t) {
            pool.emplace_back([&, t] {
                std::string &out = buf[t];
                out.clear();
                char tmp[64];
                const size_t lo = k0 + (size_t)t * window, hi = std::min(n, lo + window);
                for (size_t k = lo; k < hi; ++k) {
                    const int64_t r_index = translation[loci[k]] + base;
                    char rbuf[24];
                    const auto rr = std::to_chars(rbuf, rbuf + sizeof rbuf, r_index);
                    for (size_t j = 0; j < k; ++j) {
                        const float sum = S[k * n + j] + S[j * n + k];
                        const double v = (double)sum * 0.5;
                        char *p = std::to_chars(tmp, tmp + sizeof tmp, v, std::chars_format::fixed, 8).ptr;
                        *p++ = ' ';
                        out.append(tmp, p);
                        out.append(rbuf, rr.ptr);
                        out.push_back(' ');
                        p = std::to_chars(tmp, tmp + sizeof tmp, translation[loci[j]] + base).ptr;
                        *p++ = '\n';
                        out.append(tmp, p);
                    }
                }
            });
        }
        for (auto &th : pool) th.join();
        for (int t = 0; t < T; ++t)
            if (!buf[t].empty() && std::fwrite(buf[t].data(), 1, buf[t].size(), f) != buf[t].size())
                fail("failed to write \"" + path + "\"");
    }
    if (std::fclose(f) != 0) fail("failed to write \"" + path + "\"");
}

// ---- norm-of-mean scoring (plmDCA.hpp:335-363, 617-666)

// J_r[n][s][a] in SuperDCA's parameter layout (16-locus blocks, STATES order)
inline int64_t ref_index(int64_t L, int64_t n, int s, int a)
{
    const int64_t b = n / 16, p = n % 16;
    const int64_t e = b < L / 16 ? 16 : L % 16;
    return b * 256 + (s * e + p) * 4 + a;
}

// The reference keeps each block as a float matrix, transposed for n < r
// (plmDCA.hpp:338-361): rows are then the state of r for n < r and the
// state of n for n > r.
void stored_block(const double *x, int64_t L, int64_t r, int64_t n, float M[4][4])
{
    for (int s = 0; s < 4; ++s)
        for (int a = 0; a < 4; ++a) {
            const float v = (float)x[ref_index(L, n, s, a)];
            if (n < r) M[a][s] = v;
            else M[s][a] = v;
        }
}

// ising_gauge as SuperDCA evaluates it (plmDCA_utility.hpp:57-83): the row
// means are spread along columns and the column means along rows.
void ising_gauge(const float M[4][4], float G[4][4])
{
    float rm[4], cm[4], gm = 0.f;
    for (int i = 0; i < 4; ++i) rm[i] = (M[i][0] + M[i][1] + M[i][2] + M[i][3]) / 4.f;
    for (int j = 0; j < 4; ++j) cm[j] = (M[0][j] + M[1][j] + M[2][j] + M[3][j]) / 4.f;
    for (int i = 0; i < 4; ++i) gm += rm[i];
    gm /= 4.f;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) G[i][j] = ((M[i][j] - rm[j]) - cm[i]) + gm;
}

// Frobenius norm without the GAP row and column (Matrix_math.hpp:166-213)
float frobenius(const float G[4][4], int gap)
{
    float sum = 0.f;
    for (int i = 0; i < 4; ++i) {
        if (i == gap) continue;
        for (int j = 0; j < 4; ++j)
            if (j != gap) sum += G[i][j] * G[i][j];
    }
    return std::sqrt(sum);
}

// Lines of norm-of-mean scoring (plmDCA.hpp:617-666): for r over the loci
// list and n before it, "|mean of the gauged blocks| r n |J_rn| |J_nr| mean
// of the two norms".  Blocks: B[k][j] = block (loci[k], loci[j]), 16 floats.
// (The reference's storage indexes row i from i (d - 1), so block (i, d - 1)
// shares its memory with (i + 1, 0), plmDCA.hpp:129-137; every block here
// has its own storage.)
void write_norm_of_mean(const std::string &path, const std::vector<float> &B, const std::vector<uint32_t> &loci,
                        const std::vector<int64_t> &translation, int base, int gap)
{
    std::FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) fail("cannot open \"" + path + "\" for writing");
    const size_t n = loci.size();
    std::string out;
    char tmp[64];
    auto put = [&](double v) {
        char *p = std::to_chars(tmp, tmp + sizeof tmp, v, std::chars_format::fixed, 8).ptr;
        out.append(tmp, p);
    };
    for (size_t k = 0; k < n; ++k) {
        out.clear();
        for (size_t j = 0; j < k; ++j) {
            const float(*Mrn)[4] = reinterpret_cast<const float(*)[4]>(&B[(k * n + j) * 16]);
            const float(*Mnr)[4] = reinterpret_cast<const float(*)[4]>(&B[(j * n + k) * 16]);
            float Ga[4][4], Gb[4][4], Gm[4][4];
            ising_gauge(Mrn, Ga);
            ising_gauge(Mnr, Gb);
            for (int a = 0; a < 4; ++a)
                for (int c = 0; c < 4; ++c) Gm[a][c] = (Ga[a][c] + Gb[a][c]) * 0.5f;
            const float jn = frobenius(Gm, gap), jij = frobenius(Ga, gap), jji = frobenius(Gb, gap);
            put(jn);
            out += ' ' + std::to_string(translation[loci[k]] + base) + ' ' +
                   std::to_string(translation[loci[j]] + base) + ' ';
            put(jij);
            out += ' ';
            put(jji);
            out += ' ';
            put((double)(jij + jji) * 0.5);
            out += '\n';
        }
        if (!out.empty() && std::fwrite(out.data(), 1, out.size(), f) != out.size())
            fail("failed to write \"" + path + "\"");
    }
    if (std::fclose(f) != 0) fail("failed to write \"" + path + "\"");
}

// The strongest pairs of mean-of-norms scoring, strongest first (ties by
// list order), in the text format; optionally every pair as binary records.
void write_top_and_binary(const std::string &stem, const std::vector<float> &S, const std::vector<uint32_t> &loci,
                          const std::vector<int64_t> &translation, int base, long top_k, bool binary, bool verbose)
{
    const size_t n = loci.size();
    struct Rec { float v; int32_t r, m; };
    std::vector<Rec> recs;
    recs.reserve(n * (n - 1) / 2);
    for (size_t k = 0; k < n; ++k)
        for (size_t j = 0; j < k; ++j) {
            const float sum = S[k * n + j] + S[j * n + k];
            recs.push_back({(float)((double)sum * 0.5), (int32_t)(translation[loci[k]] + base),
                            (int32_t)(translation[loci[j]] + base)});
        }
    if (binary) {
        const std::string path = unique_name(stem + ".bin");
        if (verbose) std::cout << "superdca-gb300: writing binary coupling records to \"" << path << "\"\n";
        std::FILE *f = std::fopen(path.c_str(), "wb");
        if (!f) fail("cannot open \"" + path + "\" for writing");
        for (const Rec &q : recs) {
            unsigned char buf[12];
            uint32_t u;
            std::memcpy(&u, &q.v, 4);
            const uint32_t w[3] = {u, (uint32_t)q.r, (uint32_t)q.m};
            for (int t = 0; t < 3; ++t)
                for (int byte = 0; byte < 4; ++byte) buf[4 * t + byte] = (unsigned char)(w[t] >> (8 * byte));
            if (std::fwrite(buf, 1, 12, f) != 12) fail("failed to write \"" + path + "\"");
        }
        if (std::fclose(f) != 0) fail("failed to write \"" + path + "\"");
    }
    if (top_k > 0) {
        const size_t kk = std::min<size_t>((size_t)top_k, recs.size());
        std::vector<size_t> idx(recs.size());
        for (size_t t = 0; t < idx.size(); ++t) idx[t] = t;
        std::partial_sort(idx.begin(), idx.begin() + kk, idx.end(), [&](size_t a, size_t b) {
            return recs[a].v > recs[b].v || (recs[a].v == recs[b].v && a < b);
        });
        const std::string path = unique_name(stem + ".top" + std::to_string(kk));
        if (verbose) std::cout << "superdca-gb300: writing the " << kk << " strongest pairs to \"" << path << "\"\n";
        std::FILE *f = std::fopen(path.c_str(), "wb");
        if (!f) fail("cannot open \"" + path + "\" for writing");
        for (size_t t = 0; t < kk; ++t) {
            const Rec &q = recs[idx[t]];
            std::fprintf(f, "%.8f %d %d\n", (double)q.v, q.r, q.m);
        }
        if (std::fclose(f) != 0) fail("failed to write \"" + path + "\"");
    }
}

} // namespace

int main(int argc, char **argv)
{
    const Options o = parse_options(argc, argv);
    const int threads = o.threads > 0 ? o.threads : (int)std::max(1u, std::thread::hardware_concurrency());
    // Two alignment files: the scan mode (SuperDCA.cpp:271-301, plmDCA.hpp:470-493).
    // The loci of the first are the targets, every locus of the second a
    // feature; the sequences (rows) are the same.
    const bool scan = o.alignment_files.size() == 2;

    if (o.verbose) std::cout << "superdca-gb300: read alignment \"" << o.alignment_files[0] << "\"\n";
    Alignment a = read_fasta(o.alignment_files[0]);
    if (o.verbose) std::cout << "superdca-gb300: " << a.N << " sequences, " << a.L << " loci\n";
    Alignment a2;
    if (scan) {
        if (o.verbose) std::cout << "superdca-gb300: read alignment \"" << o.alignment_files[1] << "\"\n";
        a2 = read_fasta(o.alignment_files[1]);
        if (a2.N != a.N) fail("the two alignments must hold the same sequences (" + std::to_string(a.N) + " and " +
                              std::to_string(a2.N) + " rows)");
    }

    if (!o.filterlist.empty()) {
        std::vector<int64_t> cols = read_index_list(o.filterlist, o.in_base);
        for (int64_t c : cols)
            if (c >= a.L) fail("filter list index " + std::to_string(c + o.in_base) + " is beyond the alignment");
        std::sort(cols.begin(), cols.end());
        cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
        a = select_columns(a, cols);
        if (o.out_filterlist) write_fasta(a, o, "filterlist-selected");
    } else {
        for (Alignment *al : {&a, &a2}) {
            if (al == &a2 && !scan) continue;
            if (!o.no_filter) *al = select_columns(*al, filter_columns(*al, o.maf, o.gap));
            if (o.out_filtered) {
                write_fasta(*al, o, "filtered");
                write_loci(*al, o);
            }
        }
    }
    if (!o.samplelist.empty()) {
        // (SuperDCA selects the samples of the first alignment only; the rows
        // of the two must stay matched, so here both are selected)
        std::vector<int64_t> rows = read_index_list(o.samplelist, o.in_base);
        for (int64_t r : rows)
            if (r >= a.N) fail("sample list index " + std::to_string(r + o.in_base) + " is beyond the alignment");
        a = select_rows(a, rows, stem(o.samplelist));
        if (scan) a2 = select_rows(a2, rows, a2.id);
        if (o.out_samplelist) write_fasta(a, o, "samplelist-selected");
    }

    std::vector<int64_t> kept;
    const std::vector<uint8_t> states1 = four_state(a, kept);
    std::vector<int64_t> translation(kept.size());
    for (size_t k = 0; k < kept.size(); ++k) translation[k] = a.translation[kept[k]];
    const int64_t N = a.N, L1 = (int64_t)kept.size();
    // features: the alignment itself, or the second one in the scan mode
    std::vector<uint8_t> states2;
    std::vector<int64_t> translation2;
    if (scan) {
        std::vector<int64_t> kept2;
        states2 = four_state(a2, kept2);
        translation2.resize(kept2.size());
        for (size_t k = 0; k < kept2.size(); ++k) translation2[k] = a2.translation[kept2[k]];
    }
    const std::vector<uint8_t> &states = scan ? states2 : states1;
    const int64_t L = scan ? (int64_t)translation2.size() : L1;
    if (o.verbose) {
        std::cout << "superdca-gb300: 4-state alignment has " << N << " sequences and " << L1 << " loci\n";
        if (scan) std::cout << "superdca-gb300: scan against " << L << " loci of the second alignment\n";
    }

    std::vector<uint32_t> loci;
    if (!o.locilist.empty()) {
        for (int64_t v : read_index_list(o.locilist, o.in_base)) {
            if (v >= L1) fail("loci list index " + std::to_string(v + o.in_base) + " is beyond the alignment");
            loci.push_back((uint32_t)v);
        }
    } else {
        const int64_t end = o.end_locus < 0 ? L1 : std::min<int64_t>(L1, o.end_locus + 1);
        for (int64_t n = o.begin_locus; n < end; ++n) loci.push_back((uint32_t)n);
    }
    if (L1 == 0 || L == 0) {
        std::cerr << "superdca-gb300: there are no loci to analyze (need at least 2)\n";
        return EXIT_FAILURE;
    }
    if (scan && loci.empty()) {
        std::cerr << "superdca-gb300: there are no target loci to analyze\n";
        return EXIT_FAILURE;
    }
    if (!scan && loci.size() < 2) {
        std::cerr << "superdca-gb300: there are not enough loci for plmDCA analysis (found " << loci.size()
                  << " loci that qualify, but need at least 2)\n";
        return EXIT_FAILURE;
    }

    const bool need_gpu = !o.no_reweighting || !o.no_dca;
    const std::vector<int> devices = o.devices.empty() ? std::vector<int>{o.device} : o.devices;
    Handle H;
    sdca_config cfg;
    sdca_config_default(&cfg);
    if (need_gpu) {
        cfg.n_seqs = N;
        cfg.n_loci = L;
        cfg.lambda_h = o.lambda_h;
        cfg.lambda_J = o.lambda_J;
        cfg.gradient_threshold = o.gradient_threshold;
        cfg.form = o.form;
        if (cfg.form == SDCA_FORM_DUAL && N > 16383) {
            // the dual form keeps N x N agreement counts; larger alignments use the tensor cores
            if (o.verbose) std::cout << "superdca-gb300: " << N << " sequences: using the tensor-core form\n";
            cfg.form = SDCA_FORM_TC;
        }
        const bool dual = cfg.form == SDCA_FORM_DUAL;
        cfg.batch = o.batch > 0 ? o.batch : (dual ? 512 : 64);
        cfg.lanes = o.lanes > 0 ? o.lanes : (dual ? 4 : 1);
        cfg.flags = o.history_bf16 ? SDCA_FLAG_HISTORY_BF16 : 0;
        cfg.device = devices[0];
        check(sdca_create(&cfg, &H.h), nullptr, "engine set-up failed");
    }

    std::vector<double> weights((size_t)N, 1.0);
    if (!o.no_reweighting) {
        if (o.verbose) std::cout << "superdca-gb300: calculate sequence weights\n";
        check(sdca_compute_weights(H.h, states.data(), nullptr, o.reweighting_threshold, weights.data()), H.h,
              "reweighting failed");
    }
    if (o.output_weights) {
        // std::scientific, precision 8 (plmDCA.hpp:547-556)
        const std::string path = unique_name(a.id + ".weights");
        std::FILE *f = std::fopen(path.c_str(), "wb");
        if (!f) fail("cannot open \"" + path + "\" for writing");
        for (double w : weights) std::fprintf(f, "%.8e\n", w);
        if (std::fclose(f) != 0) fail("failed to write \"" + path + "\"");
    }
    if (o.no_dca) {
        if (o.verbose) std::cout << "superdca-gb300: exit on users request without performing DCA\n";
        return EXIT_SUCCESS;
    }

    std::vector<float> blob;
    if (!o.warm_start.empty()) blob = read_blob(o.warm_start);
    // alignment, weights, targets and learned start of one engine
    auto prepare = [&](sdca_handle *h) {
        check(sdca_set_alignment(h, states.data(), weights.data()), h, "alignment upload failed");
        if (scan) check(sdca_set_targets(h, states1.data(), L1), h, "target upload failed");
        if (!blob.empty()) check(sdca_set_warm_start(h, blob.data(), blob.size()), h, "learned start rejected");
    };
    prepare(H.h);
    if (o.verbose) {
        double lh, lJ, beff;
        sdca_get_lambdas(H.h, &lh, &lJ, &beff);
        std::cout << "superdca-gb300: B_eff = " << beff << ", lambda_h = " << lh << ", lambda_J = " << lJ << "\n";
    }

    // One engine per further device of --gpu-devices, with the configuration
    // of the first (after autotuning) and its own copy of the alignment.
    std::vector<std::unique_ptr<Handle>> extra;
    std::vector<sdca_handle *> hs;
    auto open_devices = [&] {
        hs.assign(1, H.h);
        for (size_t d = 1; d < devices.size(); ++d) {
            sdca_config c = cfg;
            c.device = devices[d];
            extra.push_back(std::make_unique<Handle>());
            check(sdca_create(&c, &extra.back()->h), nullptr,
                  ("engine set-up failed on device " + std::to_string(devices[d])).c_str());
            prepare(extra.back()->h);
            hs.push_back(extra.back()->h);
        }
        if (o.verbose && hs.size() > 1) {
            std::cout << "superdca-gb300: " << hs.size() << " engines, on devices";
            for (int d : devices) std::cout << ' ' << d;
            std::cout << "\n";
        }
    };

    // Solve loci[lo, hi) over the engines: engine d takes the d-th of
    // hs.size() contiguous ranges and solves it in calls of at most `chunk`
    // loci on its own host thread.  take(k0, m, rows, xs, stats) receives
    // each solved call; the ranges are disjoint, so it may write row k0 + k
    // of shared output without a lock.
    const int64_t D = 16 * L + 4;
    auto solve_sharded = [&](size_t lo, size_t hi, size_t chunk, bool want_x, const auto &take) {
        const size_t nd = hs.size();
        std::vector<std::string> err(nd);
        std::vector<std::thread> pool;
        for (size_t d = 0; d < nd; ++d)
            pool.emplace_back([&, d] {
                const size_t b0 = lo + (hi - lo) * d / nd, b1 = lo + (hi - lo) * (d + 1) / nd;
                std::vector<float> rows;
                std::vector<double> xs;
                std::vector<sdca_locus_stat> stats;
                for (size_t k0 = b0; k0 < b1; k0 += chunk) {
                    const size_t m = std::min(b1 - k0, chunk);
                    rows.resize(m * (size_t)L);
                    stats.resize(m);
                    if (want_x) xs.resize(m * (size_t)D);
                    if (sdca_solve_ex(hs[d], loci.data() + k0, m, nullptr, want_x ? xs.data() : nullptr, rows.data(),
                                      stats.data()) != SDCA_OK) {
                        err[d] = sdca_last_error(hs[d]);
                        return;
                    }
                    take(k0, m, rows.data(), xs.data(), stats.data());
                }
            });
        for (auto &t : pool) t.join();
        for (size_t d = 0; d < nd; ++d)
            if (!err[d].empty()) fail("solve failed on device " + std::to_string(devices[d]) + ": " + err[d]);
    };
    std::atomic<size_t> not_converged{0};

    if (scan) {
        // lines "S[r][n] r n" for r over the target list and every feature
        // locus n (plmDCA.hpp:638-645, 673-680); the norm-of-mean mode prints
        // the same norm of the untransposed block
        open_devices();
        std::FILE *f = nullptr;
        std::string path;
        if (!o.no_coupling_output) {
            path = unique_name(a.id + "_scan.SuperDCA_couplings." + std::to_string(o.out_base) + "-based.all");
            if (o.verbose) std::cout << "superdca-gb300: writing coupling values to file \"" << path << "\"\n";
            f = std::fopen(path.c_str(), "wb");
            if (!f) fail("cannot open \"" + path + "\" for writing");
        }
        std::vector<float> rows;
        std::string out;
        char tmp[64];
        // each chunk of the target list is shared out over the engines, then
        // written in list order
        for (size_t c0 = 0; c0 < loci.size(); c0 += (size_t)o.chunk) {
            const size_t m = std::min(loci.size() - c0, (size_t)o.chunk);
            rows.resize(m * (size_t)L);
            solve_sharded(c0, c0 + m, m, false,
                          [&](size_t k0, size_t mm, const float *r, const double *, const sdca_locus_stat *st) {
                              std::memcpy(rows.data() + (k0 - c0) * (size_t)L, r, mm * (size_t)L * sizeof(float));
                              for (size_t k = 0; k < mm; ++k) not_converged += st[k].status != 0;
                          });
            for (size_t k = 0; k < m && f; ++k) {
                out.clear();
                const std::string rs = std::to_string(translation[loci[c0 + k]] + o.out_base);
                for (int64_t nn = 0; nn < L; ++nn) {
                    char *p = std::to_chars(tmp, tmp + sizeof tmp, (double)rows[k * (size_t)L + nn],
                                            std::chars_format::fixed, 8).ptr;
                    out.append(tmp, p);
                    out += ' ' + rs + ' ' + std::to_string(translation2[nn] + o.out_base) + '\n';
                }
                if (std::fwrite(out.data(), 1, out.size(), f) != out.size()) fail("failed to write \"" + path + "\"");
            }
        }
        if (f && std::fclose(f) != 0) fail("failed to write \"" + path + "\"");
        if (not_converged)
            std::cerr << "superdca-gb300: " << not_converged << " loci stopped before the gradient threshold\n";
        return EXIT_SUCCESS;
    }

    // Solve the loci list; keep the scores of the listed columns (and, for
    // norm-of-mean scoring, their 4 x 4 blocks).
    const size_t n = loci.size();
    std::vector<float> S(n * n), blocks;
    if (o.norm_of_mean) blocks.assign(n * n * 16, 0.f);
    size_t start = 0;
    // Without --gpu-batch / --gpu-lanes the first loci (at most a quarter of
    // the list, and at most 4 GB of score rows) are solved with candidate
    // configurations in turn on the first device, and the rest with the
    // fastest.  Norm-of-mean scoring needs every solution, which the probes
    // do not return; in the scan mode the loci index the second alignment,
    // which the probes do not hold.
    if (!o.no_autotune && o.batch <= 0 && o.lanes <= 0 && !o.norm_of_mean) {
        const size_t prefix = std::min(n / 4, (size_t)((1ull << 30) / (uint64_t)L));
        std::vector<float> rows(prefix * (size_t)L);
        std::vector<sdca_locus_stat> stats(std::max<size_t>(prefix, 1));
        sdca_config best;
        size_t done = 0;
        sdca_tune_entry ents[SDCA_TUNE_MAX_ENTRIES];
        int32_t nent = 0;
        check(sdca_autotune(&cfg, states.data(), weights.data(), loci.data(), prefix, 1.0,
                            o.tune_cache.empty() ? nullptr : o.tune_cache.c_str(), rows.data(), stats.data(), &done,
                            &best, ents, &nent),
              nullptr, "autotuning failed");
        for (size_t k = 0; k < done; ++k) {
            for (size_t j = 0; j < n; ++j) S[k * n + j] = rows[k * (size_t)L + loci[j]];
            not_converged += stats[k].status != 0;
        }
        if (o.verbose) {
            for (int e = 0; e < nent; ++e)
                if (ents[e].status == SDCA_OK)
                    std::cout << "superdca-gb300: autotune batch " << ents[e].batch << " x " << ents[e].lanes
                              << " lanes: " << ents[e].iterations_per_s << " iterations/s (" << ents[e].n_loci
                              << " loci)\n";
            std::cout << "superdca-gb300: using batch " << best.batch << " x " << best.lanes << " lanes\n";
        }
        if (best.batch != cfg.batch || best.lanes != cfg.lanes) {
            sdca_destroy(H.h);
            H.h = nullptr;
            cfg = best;
            check(sdca_create(&cfg, &H.h), nullptr, "engine set-up failed");
            prepare(H.h);
        }
        start = done;
    }
    open_devices();
    // solutions are D doubles per locus: keep a call's worth under ~1 GB
    const size_t chunk = o.norm_of_mean ? std::max<size_t>(1, std::min<size_t>((size_t)o.chunk, (1ull << 27) / D))
                                        : (size_t)o.chunk;
    std::mutex progress;
    size_t solved = start;
    solve_sharded(start, n, chunk, o.norm_of_mean,
                  [&](size_t k0, size_t m, const float *rows, const double *xs, const sdca_locus_stat *stats) {
                      for (size_t k = 0; k < m; ++k) {
                          for (size_t j = 0; j < n; ++j) S[(k0 + k) * n + j] = rows[k * (size_t)L + loci[j]];
                          not_converged += stats[k].status != 0;
                          if (o.norm_of_mean)
                              for (size_t j = 0; j < n; ++j) {
                                  if (loci[j] == loci[k0 + k]) continue;
                                  stored_block(xs + k * D, L, loci[k0 + k], loci[j],
                                               reinterpret_cast<float(*)[4]>(&blocks[((k0 + k) * n + j) * 16]));
                              }
                      }
                      if (o.verbose) {
                          std::lock_guard<std::mutex> g(progress);
                          solved += m;
                          std::cout << "superdca-gb300: solved " << solved << " of " << n << " loci\n" << std::flush;
                      }
                  });
    if (not_converged)
        std::cerr << "superdca-gb300: " << not_converged << " loci stopped before the gradient threshold\n";

    if (!o.no_coupling_output) {
        const std::string path =
            unique_name(a.id + ".SuperDCA_couplings." + std::to_string(o.out_base) + "-based.all");
        if (o.verbose) std::cout << "superdca-gb300: writing coupling values to file \"" << path << "\"\n";
        if (o.norm_of_mean) write_norm_of_mean(path, blocks, loci, translation, o.out_base, 3);
        else write_couplings(path, S, loci, translation, o.out_base, threads);
        if (o.top_k > 0 || o.binary_output)
            write_top_and_binary(a.id + ".SuperDCA_couplings." + std::to_string(o.out_base) + "-based", S, loci,
                                 translation, o.out_base, o.top_k, o.binary_output, o.verbose);
    }
    return EXIT_SUCCESS;
}
