// autotune.cpp -- choice of slots per lane and solver lanes by measurement.
//
// SuperDCA hands loci to TBB with grain 1 and lets the scheduler balance
// them (SuperDCA/include/plmDCA.hpp:581-586).  Here the equivalent choice is
// how many loci each solver lane holds at once (sdca_config.batch) and how
// many lanes share the GPU (sdca_config.lanes).  The best pair depends on
// the alignment's shape (N sets the cost of a slot's vectors and of K rho, L
// the cost of the exact max-norm checks and solutions), on the form and on
// the device, so it is measured rather than modelled: the first loci of the
// caller's own list are solved with each candidate in turn (their results are
// kept), and the candidate that ran the most L-BFGS iterations per device
// second wins.  Iterations per second, rather than loci per second, makes
// probes on different loci comparable: loci differ in how many iterations
// they need, not in what an iteration costs.  Every probe holds twice its
// candidate's slots, so each fills its slots, refills them once and drains.
// The choice can be kept in a small text file, one line per shape:
//   N L form device-name free-memory-class(GiB/16) batch lanes
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/superdca_gb300.h"

namespace {

struct Candidate {
    int batch, lanes;
};

std::vector<Candidate> candidates(int form)
{
    if (form == SDCA_FORM_DUAL)
        // largest first: on a small list the ones its probe budget cannot fill are skipped
        return {{2048, 4}, {2048, 3}, {1536, 4}, {1536, 3}, {1280, 3}, {1024, 3}, {1024, 4}, {1536, 2}, {768, 3},
                {1024, 2}, {512, 4}, {512, 2}, {256, 4}, {256, 2}, {512, 1}};
    return {{64, 1}, {32, 2}, {64, 2}, {128, 1}, {32, 1}};
}

std::string cache_key(const sdca_config &c)
{
    cudaDeviceProp prop;
    std::string name = "unknown";
    if (cudaGetDeviceProperties(&prop, c.device) == cudaSuccess) name = prop.name;
    for (char &ch : name)
        if (ch == ' ') ch = '_';
    size_t fr = 0, tot = 0;
    int dev0 = 0;
    cudaGetDevice(&dev0);
    cudaSetDevice(c.device);
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) fr = 0;
    cudaSetDevice(dev0);
    cudaGetLastError();
    std::ostringstream o;
    o << c.n_seqs << ' ' << c.n_loci << ' ' << c.form << ' ' << name << ' ' << (fr >> 34);
    return o.str();
}

bool cache_lookup(const char *path, const std::string &key, int *batch, int *lanes)
{
    if (!path) return false;
    std::ifstream f(path);
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        if (line.compare(0, key.size(), key) != 0 || line.size() <= key.size() || line[key.size()] != ' ') continue;
        std::istringstream rest(line.substr(key.size()));
        int b = 0, l = 0;
        if (rest >> b >> l && b > 0 && l > 0) {
            *batch = b;
            *lanes = l;
            found = true;   // the last line for a key wins
        }
    }
    return found;
}

void cache_store(const char *path, const std::string &key, int batch, int lanes)
{
    if (!path) return;
    std::ofstream f(path, std::ios::app);
    if (f) f << key << ' ' << batch << ' ' << lanes << '\n';
}

} // namespace

extern "C" int sdca_autotune(const sdca_config *base, const uint8_t *states, const double *weights,
                             const uint32_t *loci, size_t n_loci, double max_fraction, const char *cache_path,
                             float *scores, sdca_locus_stat *stats, size_t *n_done, sdca_config *best,
                             sdca_tune_entry *entries, int32_t *n_entries)
{
    if (!base || !states || !weights || !best || !n_done || !n_entries) return SDCA_E_ARG;
    if (n_loci > 0 && !loci) return SDCA_E_ARG;
    if (!(max_fraction >= 0.0 && max_fraction <= 1.0)) return SDCA_E_ARG;
    *n_done = 0;
    *n_entries = 0;
    *best = *base;
    const std::string key = cache_key(*base);
    int cb = 0, cl = 0;
    if (cache_lookup(cache_path, key, &cb, &cl)) {
        best->batch = cb;
        best->lanes = cl;
        return SDCA_OK;
    }
    const size_t budget = (size_t)(max_fraction * (double)n_loci);
    const size_t L = (size_t)base->n_loci;
    double best_rate = -1.0;
    size_t pos = 0;
    for (const Candidate &c : candidates(base->form)) {
        if (*n_entries >= SDCA_TUNE_MAX_ENTRIES) break;
        sdca_tune_entry e;
        std::memset(&e, 0, sizeof(e));
        e.batch = c.batch;
        e.lanes = c.lanes;
        const size_t probe = 2 * (size_t)c.batch * (size_t)c.lanes;
        if (pos + probe > budget) {
            e.status = SDCA_E_ARG;   // not enough loci left in the budget for a fair probe
            if (entries) entries[*n_entries] = e;
            ++*n_entries;
            continue;
        }
        sdca_config cfg = *base;
        cfg.batch = c.batch;
        cfg.lanes = c.lanes;
        sdca_handle *h = nullptr;
        int rc = sdca_create(&cfg, &h);
        if (rc == SDCA_OK) rc = sdca_set_alignment(h, states, weights);
        if (rc == SDCA_OK)
            rc = sdca_solve(h, loci + pos, probe, scores ? scores + pos * L : nullptr, stats ? stats + pos : nullptr);
        sdca_profile prof;
        if (rc == SDCA_OK) rc = sdca_get_profile(h, &prof);
        if (h) sdca_destroy(h);
        e.status = rc;
        if (rc == SDCA_OK) {
            e.n_loci = (int32_t)probe;
            e.device_ms = prof.solve_ms;
            e.iterations_per_s = prof.solve_ms > 0.0 ? (double)prof.iterations / (prof.solve_ms * 1e-3) : 0.0;
            pos += probe;
            if (e.iterations_per_s > best_rate) {
                best_rate = e.iterations_per_s;
                best->batch = c.batch;
                best->lanes = c.lanes;
            }
        } else if (rc != SDCA_E_NOMEM) {
            // anything but a candidate too large for the device is the caller's problem
            if (entries) entries[*n_entries] = e;
            ++*n_entries;
            *n_done = pos;
            return rc;
        }
        if (entries) entries[*n_entries] = e;
        ++*n_entries;
    }
    *n_done = pos;
    if (best_rate > 0.0) cache_store(cache_path, key, best->batch, best->lanes);
    return SDCA_OK;
}
