// engine.cu -- host driver and C ABI of the GB300 plmDCA solve engine.
//
// What it replaces in SuperDCA:
//   run_plmDCA / plmDCA_solver::operator()   SuperDCA/include/plmDCA.hpp:277-396, 436-587
//   plmDCA_optimizer_parameters (lambdas)    SuperDCA/include/plmDCA_optimizer_parameters.hpp:257-295
//   LbfgsSolver + MoreThuente (absent)       driven as in plmDCA.hpp:218-221, 298-304
//   tbb::parallel_reduce over loci           plmDCA.hpp:581-586
//
// A batch of `batch` slots holds one target locus each.  Per L-BFGS iteration
// the engine runs, for all active slots together:
//   A. line-search rounds: one k_trial launch per round for every slot still
//      searching (O(N q) per slot, no contraction), the More-Thuente state
//      machine on the host between rounds;
//   B. accept (x += stp d, push s), backward contraction (gradient, push y),
//      convergence tests, history dots, compact-form coefficients, direction,
//      forward contraction u = X . d for the next search.
// Slots whose locus converged are scored and refilled from the queue, so loci
// retire and enter independently.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"
#include "lbfgs_host.h"
#include "linesearch.h"

using namespace sdca;

namespace {

std::mutex g_err_mu;
std::string g_create_err;

enum Phase {
    PH_EMPTY = 0,
    PH_INIT,        // needs the evaluation at its start point
    PH_LS,          // line search: needs a trial at ls.stp
    PH_FINAL_EVAL,  // search ended without a trial at its step: evaluate there
    PH_READY_INIT,  // start point evaluated, waiting for the gradient pass
    PH_READY_STEP,  // step accepted, waiting for the gradient pass
    PH_FINALIZE,    // converged: logits refreshed, needs the final evaluation
    PH_REFRESH,     // logits recomputed from the stored parameters: needs the evaluation there
    PH_READY_REFRESH,  // re-evaluated, waiting for the gradient pass (history kept)
    PH_CONVERT,     // dual form: stopped, waiting for its parameters to be formed
    PH_WARM,        // dual form: its learned start is formed this round (then PH_INIT)
};

struct SlotHost {
    int phase = PH_EMPTY;
    int64_t k = -1;          // index in the caller's loci list
    int32_t locus = -1;
    int iter = 0;            // pairs since the last restart (bounded by m)
    int iterations = 0;
    int64_t nfeval = 0;
    int64_t contractions = 0;
    int status = 0;
    double gamma = 1.0;      // H0 scaling s.y / y.y
    std::deque<int> hist;    // ring positions, oldest first
    double SY[MAXHIST + 1][MAXHIST + 1];
    double YY[MAXHIST + 1][MAXHIST + 1];
    double f = 0, gmax = 0, g2 = 0, x2J = 0, x2H = 0;
    double gd = 0, ddJ = 0, ddH = 0, xdJ = 0, xdH = 0;
    double stp = 0;
    int trials = 0;
    bool use_u = false;
    bool push = false;
    int ring_new = -1;
    int gcur = 0;
    double rs[Q] = {0, 0, 0, 0};
    double f_final = 0;
    int restarts = 0, skipped = 0, weak = 0, max_trials = 0, refreshes = 0;
    bool force_restart = false;
    bool stalled = false;    // steepest descent itself was not downhill: stop
    int last_refresh = 0;    // iteration of the last logit refresh
    int since_refresh = 0;   // accepted steps since the logits were last recomputed
    double xmax = 0.0;       // bound on max|x| (sets the fp16 scale of a refresh)
    double dmax = 0.0;       // max|d| of the current direction
    double f_fresh = 0.0;    // pseudo-likelihood part of f at recomputed logits
    // dual form: from the device's summary of the slot (its solver state
    // lives on the device): h part of x, max |a| of the gradient and of x
    double eta_x[Q] = {0, 0, 0, 0};
    double amax_g = 0.0, amax_x = 0.0;
    MoreThuente ls;
};

struct ProfRec {
    int cls;
    int kernels;
    int64_t units;
    cudaEvent_t a, b;
};

} // namespace

// Per-class timing of one replay of the dual form's iteration core: the
// events recorded by its event nodes and, per class, the list (counts index)
// whose length gives the units.
struct GraphRec {
    int cls, kernels, cidx;
    cudaEvent_t a, b;
};

// The round's list lengths, in the order they follow the lists in device
// memory: searching slots, gradient pass, K rho pass (gradient pass and
// learned starts), learned starts
enum { DC_T = 0, DC_G = 1, DC_GW = 2, DC_W = 3, DC_N = 4 };

struct DualGraph {
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev_round = nullptr;     // recorded after the summary copy (the host waits on it)
    std::vector<cudaEvent_t> ev;        // timing events of the event nodes
    std::vector<GraphRec> recs;
    bool pending = false;               // replayed, its timings not collected yet
    int64_t counts[DC_N] = {};          // the list lengths of that replay
};

struct sdca_handle {
    sdca_config cfg{};
    std::string err;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    Problem P;
    bool has_alignment = false;
    std::vector<double> w_host;

    // device memory
    std::vector<void *> allocs;
    uint8_t *X = nullptr, *XT = nullptr, *rstate = nullptr;
    double *w = nullptr;
    float *wf = nullptr;           // the weights in FP32 (kernels that need no more)
    float *wa = nullptr, *d = nullptr, *gpool = nullptr, *u = nullptr, *R = nullptr;
    float *partial = nullptr, *rows = nullptr;
    void *Spool = nullptr, *Ypool = nullptr;
    double *lbase = nullptr, *acc = nullptr, *dots = nullptr, *partial64 = nullptr;
    SlotDev *sd = nullptr;
    int32_t *list = nullptr;
    int *flag = nullptr;
    // pinned host mirrors
    SlotDev *sd_h = nullptr;       // host-side slot parameters (edited freely)
    uint8_t *stage = nullptr;      // pinned staging arena for host->device copies: a
    size_t stage_cap = 0, stage_off = 0;  // region is reused only after a stream sync
    int32_t *list_h = nullptr;
    double *acc_h = nullptr, *dots_h = nullptr;
    float *rows_h = nullptr;
    int *flag_h = nullptr;
    int hist_bf16 = 0;

    // tensor-core form
    int form = SDCA_FORM_GATHER;
    TcPlan *tc = nullptr;
    __half *Dhi = nullptr, *Dlo = nullptr, *Rhi = nullptr, *Rlo = nullptr;
    int *tc_err = nullptr;
    float r_scale = 1.0f;
    // logit refresh policy: when max|g| first falls
    // below refresh_factor x threshold, and again every refresh_every
    // iterations while it stays there
    double refresh_factor = 8.0;
    int refresh_every = 30;
    int tc_refresh_every = 5;   // tensor-core form: recompute logits every this many accepted steps

    // dual form (kernels_dual.cu)
    float2 *dv = nullptr, *KR = nullptr;   // coefficient vectors and K rho, double-float (df.cuh)
    double *amax = nullptr, *J64 = nullptr, *amax_h = nullptr;
    int32_t *rq = nullptr, *Kmat = nullptr;
    long long *csum = nullptr;
    float *Rchk = nullptr, *P0 = nullptr;   // P0: probabilities at the current point, base of the step trials
    float *ud = nullptr;                    // u_a - u_y per sequence (single precision, step trials)
    double qscale = 1.0;
    DualCtl *ctl = nullptr;        // per-slot solver state, owned by the device while a slot iterates
    DualSum *sum = nullptr, *sum_h = nullptr;   // per-slot summary the host reads after each round
    double *dacc = nullptr;        // direction sums for the next line search
    int32_t *dlist = nullptr;      // the round's slot lists: [evaluations | searching | gradient pass + starts |
                                   // starts], then their lengths (DualCounts)
    cudaEvent_t ev_round = nullptr;   // end of a round's control kernel
    // the iteration core of a round as two alternating CUDA graphs (DualGraph)
    DualGraph dgraph[2];
    int dgraph_next = 0;
    bool dgraph_off = false;       // SDCA_DUAL_GRAPH=0, or a capture failed: launch the kernels one by one
    std::vector<int64_t> rows_pending;   // list positions whose score rows are on their way to rows_h
    KdPlan *kd = nullptr;          // exact K rho on the tensor cores (N <= 4000), else CUDA cores
    __half *Kd = nullptr, *Rd = nullptr;

    // two-alignment scan mode: target columns from a second alignment
    uint8_t *TT = nullptr;        // [LT][Nx] target states, locus-major
    int64_t LT = 0;
    bool scan = false;

    // learned warm start (warmstart.cu, mlp.cu)
    float *ws_params = nullptr;
    uint16_t *ws_wb = nullptr;     // BF16 image of the network's weights (tensor-core forward)
    int *ws_err = nullptr;         // set when a wait of the tensor-core forward gives up
    bool ws_on = false;
    int ws_k = 0;
    float ws_eps = 0.f;
    bool ws_hfit = false;          // fit h to the predicted J (blob flag) or start from h = 0
    int32_t *knn = nullptr, *knn_d = nullptr;   // neighbours and their Hamming distances
    int knn_k = 0;                 // k of the nearest-neighbour table held (0: none)
    // the dual form's learned start (blob version 2): shrinkage and buffers
    // for up to dws_cap slots per network pass
    bool ws_dual = false;
    float ws_alpha = 0.f;
    float *dws_feats = nullptr, *dws_out = nullptr;
    int dws_cap = 0;
    float *ws_R = nullptr, *ws_feats = nullptr, *ws_out = nullptr;
    int32_t *ws_idx = nullptr;     // [0, WS_G): slots, [WS_G, 2 WS_G): loci
    double *ws_xmax = nullptr;

    std::vector<SlotHost> slots;

    // solver lanes: sub[i] is a further lane with its own slots, stream and
    // host thread; its alignment buffers (X, XT, w, K and its digits) are
    // this handle's (shared_alignment set in the lane, which frees none)
    std::vector<sdca_handle *> sub;
    bool shared_alignment = false;
    cudaEvent_t ev_lanes = nullptr;   // start of a multi-lane solve

    // profiling
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<ProfRec> recs;
    sdca_profile prof{};
};

namespace {

int fail(sdca_handle *h, int code, const std::string &msg)
{
    if (h) h->err = msg;
    else {
        std::lock_guard<std::mutex> lk(g_err_mu);
        g_create_err = msg;
    }
    return code;
}

#define CK(call)                                                                         \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return fail(h, SDCA_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define CKL()                                                                            \
    do {                                                                                 \
        cudaError_t e_ = cudaGetLastError();                                             \
        if (e_ != cudaSuccess)                                                           \
            return fail(h, SDCA_E_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
    } while (0)

int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

// the dual form keeps its logits in double-float: the same 8 bytes per value

cudaEvent_t take_event(sdca_handle *h)
{
    if (h->ev_used == h->ev_pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        h->ev_pool.push_back(e);
    }
    return h->ev_pool[h->ev_used++];
}

// Times the kernels launched in its scope: `kernels` launches working on
// `units` target loci each.
struct Timed {
    sdca_handle *h;
    ProfRec rec;
    Timed(sdca_handle *hh, int cls, int kernels, int64_t units) : h(hh)
    {
        rec.cls = cls;
        rec.kernels = kernels;
        rec.units = units;
        h->prof.gpu_launches += kernels;
        rec.a = take_event(h);
        rec.b = take_event(h);
        if (rec.a) cudaEventRecord(rec.a, h->stream);
    }
    ~Timed()
    {
        if (rec.b) cudaEventRecord(rec.b, h->stream);
        if (rec.a && rec.b) h->recs.push_back(rec);
    }
};

void prof_reset(sdca_handle *h)
{
    h->ev_used = 0;
    h->recs.clear();
    std::memset(&h->prof, 0, sizeof(h->prof));
}

void prof_collect(sdca_handle *h)
{
    for (auto &r : h->recs) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            h->prof.kernel_ms[r.cls] += ms;
            h->prof.kernel_launches[r.cls] += r.kernels;
            h->prof.kernel_units[r.cls] += r.units;
        }
    }
    h->recs.clear();
}

template <typename T> int dalloc(sdca_handle *h, T **p, size_t count)
{
    void *q = nullptr;
    const size_t bytes = std::max<size_t>(count * sizeof(T), 256);
    if (cudaMalloc(&q, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, SDCA_E_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed");
    }
    if (cudaMemsetAsync(q, 0, bytes, h->stream) != cudaSuccess)
        return fail(h, SDCA_E_CUDA, "cudaMemsetAsync failed");
    h->allocs.push_back(q);
    *p = static_cast<T *>(q);
    return SDCA_OK;
}

template <typename T> int halloc(sdca_handle *h, T **p, size_t count)
{
    void *q = nullptr;
    if (cudaMallocHost(&q, std::max<size_t>(count * sizeof(T), 64)) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, SDCA_E_NOMEM, "pinned host allocation failed");
    }
    std::memset(q, 0, std::max<size_t>(count * sizeof(T), 64));
    *p = static_cast<T *>(q);
    return SDCA_OK;
}

void free_all(sdca_handle *h)
{
    for (void *p : h->allocs) cudaFree(p);
    h->allocs.clear();
    if (h->sd_h) cudaFreeHost(h->sd_h);
    if (h->list_h) cudaFreeHost(h->list_h);
    if (h->acc_h) cudaFreeHost(h->acc_h);
    if (h->dots_h) cudaFreeHost(h->dots_h);
    if (h->rows_h) cudaFreeHost(h->rows_h);
    if (h->flag_h) cudaFreeHost(h->flag_h);
    if (h->stage) cudaFreeHost(h->stage);
    if (h->sum_h) cudaFreeHost(h->sum_h);
    h->stage = nullptr;
    h->sum_h = nullptr;
    h->sd_h = nullptr; h->list_h = nullptr; h->acc_h = nullptr; h->dots_h = nullptr;
    h->rows_h = nullptr; h->flag_h = nullptr;
    h->X = h->XT = h->rstate = nullptr;
    h->has_alignment = false;
}

// X [N][Lx] -> XT [L][Nx]; flags codes >= Q
__global__ void k_transpose(const uint8_t *__restrict__ X, int64_t Lx, int N, int L,
                            uint8_t *__restrict__ XT, int64_t Nx, int *__restrict__ bad)
{
    __shared__ uint8_t tile[64][65];
    const int n0 = blockIdx.x * 64, i0 = blockIdx.y * 64;
    for (int k = threadIdx.x; k < 64 * 64; k += blockDim.x) {
        const int ii = k / 64, nn = k % 64;
        const int i = i0 + ii, n = n0 + nn;
        uint8_t v = 0;
        if (i < N && n < L) {
            v = X[(int64_t)i * Lx + n];
            if (v >= Q) atomicOr(bad, 1);
        }
        tile[ii][nn] = v;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 64 * 64; k += blockDim.x) {
        const int nn = k / 64, ii = k % 64;
        const int i = i0 + ii, n = n0 + nn;
        if (n < L && i < (int)Nx) XT[(int64_t)n * Nx + i] = (i < N) ? tile[ii][nn] : 0;
    }
}

// reference layout (double, 16-locus STATES blocks) <-> engine layout (float)
int64_t ref_index(int64_t L, int64_t n, int s, int a)
{
    const int64_t b = n / 16, p = n % 16, nfull = L / 16;
    const int64_t e = b < nfull ? 16 : L % 16;
    return b * 16 * QQ + ((int64_t)s * e + p) * Q + a;
}

void ref_to_engine(const Problem &P, int64_t r, const double *x, float *out)
{
    std::memset(out, 0, sizeof(float) * P.Dp);
    for (int64_t n = 0; n < P.L; ++n) {
        if (n == r) continue;  // J_rr never enters the objective
        for (int s = 0; s < Q; ++s)
            for (int a = 0; a < Q; ++a) out[n * QQ + s * Q + a] = (float)x[ref_index(P.L, n, s, a)];
    }
    for (int a = 0; a < Q; ++a) out[QQ * P.L + a] = (float)x[QQ * P.L + a];
}

void engine_to_ref(const Problem &P, const float *v, double *out)
{
    for (int64_t n = 0; n < P.L; ++n)
        for (int s = 0; s < Q; ++s)
            for (int a = 0; a < Q; ++a) out[ref_index(P.L, n, s, a)] = v[n * QQ + s * Q + a];
    for (int a = 0; a < Q; ++a) out[QQ * P.L + a] = v[QQ * P.L + a];
}

// Synchronise the stream; every staged host region is free afterwards.
int stream_sync(sdca_handle *h)
{
    CK(cudaStreamSynchronize(h->stream));
    h->stage_off = 0;
    return SDCA_OK;
}

// Copy `bytes` from src to device dst through a staging region that no copy
// still queued on the stream reads.
int staged_h2d(sdca_handle *h, void *dst, const void *src, size_t bytes)
{
    const size_t need = (bytes + 255) & ~(size_t)255;
    if (need > h->stage_cap) return fail(h, SDCA_E_ARG, "staging arena too small");
    if (h->stage_off + need > h->stage_cap) {
        int rc = stream_sync(h);
        if (rc) return rc;
    }
    uint8_t *p = h->stage + h->stage_off;
    h->stage_off += need;
    std::memcpy(p, src, bytes);
    CK(cudaMemcpyAsync(dst, p, bytes, cudaMemcpyHostToDevice, h->stream));
    return SDCA_OK;
}

int upload_list(sdca_handle *h, const std::vector<int32_t> &lst)
{
    if (lst.empty()) return SDCA_OK;
    return staged_h2d(h, h->list, lst.data(), sizeof(int32_t) * lst.size());
}

// copy the host slot parameters of `lst` into the device mirror
int upload_slots(sdca_handle *h, const std::vector<int32_t> &lst)
{
    for (int b : lst) {
        SlotHost &S = h->slots[b];
        SlotDev &D = h->sd_h[b];
        D.locus = h->scan ? -1 : S.locus;   // scan mode: no feature locus is excluded
        D.gcur = S.gcur;
        D.ring_new = S.ring_new;
        D.nhist = (int)S.hist.size();
        for (int j = 0; j < D.nhist; ++j) D.ring[j] = S.hist[j];
        D.flags = (S.use_u ? SLOT_F_USE_U : 0) | (S.push ? SLOT_F_PUSH : 0);
        D.stp = S.stp;
        for (int a = 0; a < Q; ++a) D.rs[a] = S.rs[a];
    }
    // the mirror is small; copy it whole
    int rc = staged_h2d(h, h->sd, h->sd_h, sizeof(SlotDev) * h->P.Bmax);
    if (rc) return rc;
    return upload_list(h, lst);
}

int zero_acc(sdca_handle *h)
{
    CK(cudaMemsetAsync(h->acc, 0, sizeof(double) * NACC * h->P.Bmax, h->stream));
    return SDCA_OK;
}

int fetch_acc(sdca_handle *h)
{
    CK(cudaMemcpyAsync(h->acc_h, h->acc, sizeof(double) * NACC * h->P.Bmax, cudaMemcpyDeviceToHost,
                       h->stream));
    if (h->tc_err) CK(cudaMemcpyAsync(h->flag_h + 1, h->tc_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    int rc = stream_sync(h);
    if (rc) return rc;
    if (h->tc_err && h->flag_h[1])
        return fail(h, SDCA_E_CUDA, "tensor-core pipeline wait timed out (kernel abandoned its tile)");
    return SDCA_OK;
}

// power of two that brings max|v| into (2^13, 2^14] for the fp16 hi/lo split
double pow2_scale(double vmax)
{
    if (!(vmax > 0.0) || !std::isfinite(vmax)) return 1.0;
    const int e = (int)std::floor(std::log2(16384.0 / vmax));
    return std::ldexp(1.0, std::max(-120, std::min(120, e)));
}

double acc_get(sdca_handle *h, int b, int k) { return h->acc_h[(int64_t)b * NACC + k]; }

// forward contraction u = X . v_J (+ v_h): into `u` (float) or `lbase` (double).
// The tensor-core form serves the per-iteration direction (and, with
// tc_lbase, the periodic recomputation of a slot's logits at its accepted
// point); logits that a locus starts from or reports use the gather with
// FP64 accumulation.
int run_forward(sdca_handle *h, const std::vector<int32_t> &lst, const float *vecs, bool to_lbase,
                bool tc_lbase = false)
{
    if (lst.empty()) return SDCA_OK;
    const bool use_tc = h->form == SDCA_FORM_TC && (!to_lbase || tc_lbase);
    int rc = use_tc ? upload_slots(h, lst) : upload_list(h, lst);
    if (rc) return rc;
    if (use_tc && to_lbase) {
        const int splits = tc_fwd_splits(h->P, (int)lst.size());
        Timed t(h, SDCA_K_FORWARD, 3, (int64_t)lst.size());
        CK(tc_launch_fwd(h->tc, h->P, h->sd, h->list, (int)lst.size(), vecs, h->Dhi, h->Dlo, h->partial,
                         splits, h->tc_err, h->stream));
        launch_reduce_partial(h->P, h->list, (int)lst.size(), h->partial, vecs, 1, nullptr, h->lbase,
                              h->stream, splits);
    } else if (use_tc) {
        const int splits = tc_fwd_splits(h->P, (int)lst.size());
        Timed t(h, SDCA_K_FORWARD, 3, (int64_t)lst.size());
        CK(tc_launch_fwd(h->tc, h->P, h->sd, h->list, (int)lst.size(), vecs, h->Dhi, h->Dlo, h->partial,
                         splits, h->tc_err, h->stream));
        launch_reduce_partial(h->P, h->list, (int)lst.size(), h->partial, vecs, 1, h->u, nullptr,
                              h->stream, splits, h->R, h->acc);
    } else if (to_lbase) {
        Timed t(h, SDCA_K_FORWARD, 2, (int64_t)lst.size());
        launch_fwd_exact(h->P, h->X, h->list, (int)lst.size(), vecs, h->partial64, h->lbase, h->stream);
    } else {
        Timed t(h, SDCA_K_FORWARD, 2, (int64_t)lst.size());
        launch_fwd_gather(h->P, h->X, h->list, (int)lst.size(), vecs, h->partial, h->stream);
        launch_reduce_partial(h->P, h->list, (int)lst.size(), h->partial, vecs, 1, h->u, nullptr, h->stream, 0,
                              h->R, h->acc);
    }
    CKL();
    for (int b : lst) h->slots[b].contractions++;
    return SDCA_OK;
}

// begin a locus in slot b: zero or given start point, logits at the start point
int dual_ctl_begin(sdca_handle *h, int b);

int slot_begin(sdca_handle *h, int b, int64_t k, int32_t locus, const float *x0_engine)
{
    SlotHost &S = h->slots[b];
    S = SlotHost();
    S.phase = PH_INIT;
    S.k = k;
    S.locus = locus;
    S.gcur = 0;
    const Problem &P = h->P;
    float *wab = h->wa + (int64_t)b * P.Dp;
    if (x0_engine) {
        CK(cudaMemcpyAsync(wab, x0_engine, sizeof(float) * P.Dp, cudaMemcpyHostToDevice, h->stream));
        for (int64_t e = 0; e < P.Dp; ++e) S.xmax = std::max(S.xmax, (double)std::fabs(x0_engine[e]));
    }
    else
        CK(cudaMemsetAsync(wab, 0, sizeof(float) * P.Dp, h->stream));
    if (h->d) CK(cudaMemsetAsync(h->d + (int64_t)b * P.Dp, 0, sizeof(float) * P.Dp, h->stream));
    CK(cudaMemcpyAsync(h->rstate + (int64_t)b * P.Nx, (h->scan ? h->TT : h->XT) + (int64_t)locus * P.Nx, P.Nx,
                       cudaMemcpyDeviceToDevice, h->stream));
    if (!x0_engine)
        CK(cudaMemsetAsync(h->lbase + (int64_t)b * P.Nx * 4, 0, sizeof(double) * P.Nx * 4, h->stream));
    if (h->form == SDCA_FORM_DUAL) {
        const size_t NV = DV_S + 2 * (size_t)P.ring;
        CK(cudaMemsetAsync(h->dv + (size_t)b * NV * 2 * P.Nx * 4, 0, sizeof(double) * NV * 2 * P.Nx * 4, h->stream));
        const int rc = dual_ctl_begin(h, b);
        if (rc) return rc;
    }
    S.stp = 0.0;
    S.use_u = false;
    S.push = false;
    S.ring_new = -1;
    return SDCA_OK;
}

// ---- learned warm start

constexpr int WS_G = 32;              // loci whose start points are prepared together
constexpr int64_t WS_ROWS = 65536;    // network rows per inference pass

int ws_buffers(sdca_handle *h)
{
    if (h->ws_feats) return SDCA_OK;
    const Problem &P = h->P;
    int rc;
    if ((rc = dalloc(h, &h->ws_R, (size_t)WS_G * P.Nx * 8))) return rc;   // [g][Nx][8], or R2 [g][Nx][4]
    if ((rc = dalloc(h, &h->ws_out, (size_t)WS_G * P.L * MLP_OUT))) return rc;
    if ((rc = dalloc(h, &h->ws_idx, 2 * WS_G))) return rc;
    if ((rc = dalloc(h, &h->ws_xmax, WS_G))) return rc;
    return dalloc(h, &h->ws_feats, (size_t)WS_G * P.L * MLP_IN);
}

// each sequence's k nearest neighbours in Hamming distance (kept until the
// alignment changes)
int ws_knn(sdca_handle *h, int k)
{
    if (h->knn_k == k) return SDCA_OK;
    const Problem &P = h->P;
    if (P.N > 32768) return fail(h, SDCA_E_UNSUPPORTED, "the warm start supports at most 32768 sequences");
    int rc;
    if (!h->knn && (rc = dalloc(h, &h->knn, (size_t)P.N * WS_MAX_K))) return rc;
    if (!h->knn_d && (rc = dalloc(h, &h->knn_d, (size_t)P.N * WS_MAX_K))) return rc;
    const int64_t W = (P.L + 31) / 32;
    uint64_t *packed = nullptr;
    int32_t *dist = nullptr;
    if (cudaMalloc(&packed, sizeof(uint64_t) * P.N * W) != cudaSuccess ||
        cudaMalloc(&dist, sizeof(int32_t) * P.N * P.N) != cudaSuccess) {
        cudaGetLastError();
        if (packed) cudaFree(packed);
        return fail(h, SDCA_E_NOMEM, "device allocation for the neighbour table failed");
    }
    launch_distances(h->X, P.Lx, (int)P.N, (int)P.L, packed, dist, h->stream);
    launch_knn(dist, (int)P.N, k, h->knn, h->stream, h->knn_d);
    const cudaError_t e1 = cudaGetLastError();
    const cudaError_t e2 = cudaStreamSynchronize(h->stream);
    cudaFree(packed);
    cudaFree(dist);
    if (e1 != cudaSuccess || e2 != cudaSuccess)
        return fail(h, SDCA_E_CUDA, std::string("neighbour table: ") + cudaGetErrorString(e1 ? e1 : e2));
    h->knn_k = k;
    return SDCA_OK;
}

// pair statistics of up to WS_G loci into ws_feats ([g][n][MLP_IN])
int ws_features(sdca_handle *h, const std::vector<int32_t> &loci, int k, float eps)
{
    const Problem &P = h->P;
    const int G = (int)loci.size();
    int rc = ws_buffers(h);
    if (rc) return rc;
    if ((rc = ws_knn(h, k))) return rc;
    CK(cudaMemcpyAsync(h->ws_idx + WS_G, loci.data(), sizeof(int32_t) * G, cudaMemcpyHostToDevice, h->stream));
    Timed t(h, SDCA_K_OTHER, 2, G);
    launch_ws_residual(h->XT, P.Nx, (int)P.N, h->ws_idx + WS_G, G, h->w, h->knn, k, eps, h->ws_R, h->stream);
    launch_ws_pairs(h->XT, P.Nx, (int)P.N, (int)P.L, G, h->ws_R, P.b_eff, h->ws_feats, h->stream);
    CKL();
    return SDCA_OK;
}

// the same statistics for slots that are about to start, by two tensor-core
// backward contractions X^T R through the slots' own R rows and gradient
// buffers (both free until the slot's first evaluation)
int ws_features_tc(sdca_handle *h, const std::vector<int32_t> &grp, int k, float eps)
{
    const Problem &P = h->P;
    const int G = (int)grp.size();
    int rc = ws_buffers(h);
    if (rc) return rc;
    if ((rc = ws_knn(h, k))) return rc;
    // ws_idx: slots then loci, as ws_begin expects them
    std::vector<int32_t> loci(G);
    for (int g = 0; g < G; ++g) loci[g] = h->slots[grp[g]].locus;
    CK(cudaMemcpyAsync(h->ws_idx, grp.data(), sizeof(int32_t) * G, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->ws_idx + WS_G, loci.data(), sizeof(int32_t) * G, cudaMemcpyHostToDevice, h->stream));
    {
        Timed t(h, SDCA_K_OTHER, 1, G);
        launch_ws_residual_split(h->XT, P.Nx, (int)P.N, h->ws_idx + WS_G, h->ws_idx, G, h->w, h->knn, k, eps, h->R,
                                 h->ws_R, h->stream);
    }
    CKL();
    for (int pass = 0; pass < 2; ++pass) {
        for (int b : grp) h->slots[b].gcur = pass;   // pass 0 fills buffer 2b+1, pass 1 buffer 2b
        if ((rc = upload_slots(h, grp))) return rc;
        if (pass == 1) {
            Timed t(h, SDCA_K_OTHER, 1, G);
            launch_ws_copy_r(P.Nx, h->ws_idx, G, h->ws_R, h->R, h->stream);
        }
        Timed t(h, SDCA_K_OTHER, 2, G);
        CK(tc_launch_bwd(h->tc, P, h->sd, h->list, G, h->R, h->r_scale, h->Rhi, h->Rlo, h->gpool, h->tc_err,
                         h->stream));
    }
    for (int b : grp) h->slots[b].gcur = 0;
    {
        Timed t(h, SDCA_K_OTHER, 1, G);
        launch_ws_assemble((int)P.L, P.Dp, h->ws_idx, G, h->gpool, P.b_eff, h->ws_feats, h->stream);
    }
    CKL();
    return SDCA_OK;
}

// start points of slots `bs` from the network: J blocks with h = 0, or h
// fitted with J fixed when the blob asks for it
int ws_begin(sdca_handle *h, const std::vector<int32_t> &bs)
{
    const Problem &P = h->P;
    for (size_t g0 = 0; g0 < bs.size(); g0 += WS_G) {
        const int G = (int)std::min<size_t>(WS_G, bs.size() - g0);
        std::vector<int32_t> grp(bs.begin() + g0, bs.begin() + g0 + G), loci(G);
        for (int g = 0; g < G; ++g) loci[g] = h->slots[grp[g]].locus;
        int rc = h->form == SDCA_FORM_TC ? ws_features_tc(h, grp, h->ws_k, h->ws_eps)
                                         : ws_features(h, loci, h->ws_k, h->ws_eps);
        if (rc) return rc;
        CK(cudaMemcpyAsync(h->ws_idx, grp.data(), sizeof(int32_t) * G, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemsetAsync(h->ws_xmax, 0, sizeof(double) * WS_G, h->stream));
        {
            const int64_t M = (int64_t)G * P.L, rows = std::min<int64_t>(WS_ROWS, WS_G * P.L);
            Timed t(h, SDCA_K_OTHER, (int)((M + rows - 1) / rows + 1), G);
            for (int64_t r0 = 0; r0 < M; r0 += rows)
                mlp_infer(h->ws_params, h->ws_wb, h->ws_feats + r0 * MLP_IN, std::min(rows, M - r0),
                          h->ws_out + r0 * MLP_OUT, h->ws_err, h->stream);
            launch_ws_scatter((int)P.L, P.Dp, h->ws_idx, h->ws_idx + WS_G, G, h->ws_out, h->ws_params,
                              P.b_eff / (2.0 * P.lambda_J), h->wa, h->ws_xmax, h->stream);
        }
        CKL();
        std::vector<double> xm(G);
        auto fetch_xmax = [&]() -> int {
            CK(cudaMemcpyAsync(xm.data(), h->ws_xmax, sizeof(double) * G, cudaMemcpyDeviceToHost, h->stream));
            CK(cudaMemcpyAsync(h->flag_h + 2, h->ws_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
            const int r_ = stream_sync(h);
            if (r_) return r_;
            if (h->flag_h[2]) return fail(h, SDCA_E_CUDA, "warm start: a tensor-core pipeline wait gave up");
            for (int g = 0; g < G; ++g) {
                const int b = grp[g];
                h->slots[b].xmax = xm[g];
                h->sd_h[b].tc_scale = pow2_scale(xm[g]);
                h->sd_h[b].tc_inv_scale = 1.0 / h->sd_h[b].tc_scale;
            }
            return SDCA_OK;
        };
        if ((rc = fetch_xmax())) return rc;
        // logits at the start point: the tensor-core form uses its own forward
        // (as for its periodic logit refresh), the plain form the FP64-accumulated gather
        if ((rc = run_forward(h, grp, h->wa, true, h->form == SDCA_FORM_TC))) return rc;
        if (h->ws_hfit) {
            {
                Timed t(h, SDCA_K_OTHER, 1, G);
                launch_ws_hfit(P, h->ws_idx, h->rstate, h->w, G, h->wa, h->lbase, h->ws_xmax, h->stream);
            }
            CKL();
            if ((rc = fetch_xmax())) return rc;
        }
    }
    return SDCA_OK;
}

// the per-solve queue
struct Queue {
    const uint32_t *loci = nullptr;
    size_t n = 0;
    std::atomic<size_t> *next = nullptr;   // shared by the lanes of one solve
    std::atomic<bool> *abort = nullptr;    // a lane failed: take no further loci
    const double *x_init = nullptr;
    double *x_out = nullptr;
    const int64_t *x_rows = nullptr;       // row of x_out per list position (-1: none); null: row k
    float *rho_out = nullptr;              // dual form: converged residual rows (n x N x 4) or null
    float *scores = nullptr;
    sdca_locus_stat *stats = nullptr;
    std::vector<float> xbuf;
};

// next position of the loci list, or -1 when it is exhausted
int64_t take(Queue &Qu)
{
    if (Qu.abort && Qu.abort->load()) return -1;
    const size_t k = Qu.next->fetch_add(1);
    return k < Qu.n ? (int64_t)k : -1;
}

int refill(sdca_handle *h, Queue &Qu)
{
    std::vector<int32_t> warm, learned;
    for (int b = 0; b < h->P.Bmax; ++b) {
        if (h->slots[b].phase != PH_EMPTY) continue;
        const int64_t k = take(Qu);
        if (k < 0) break;
        const float *x0 = nullptr;
        if (Qu.x_init && h->form == SDCA_FORM_DUAL)
            return fail(h, SDCA_E_UNSUPPORTED,
                        "the dual form takes no arbitrary start point (x_init): it starts from zero or learned");
        if (Qu.x_init) {
            const double *xr = Qu.x_init + k * (QQ * h->P.L + Q);
            ref_to_engine(h->P, h->scan ? -1 : (int64_t)Qu.loci[k], xr, Qu.xbuf.data());
            x0 = Qu.xbuf.data();
        }
        int rc = slot_begin(h, b, k, (int32_t)Qu.loci[k], x0);
        if (rc) return rc;
        if (h->form == SDCA_FORM_DUAL && h->ws_dual) h->slots[b].phase = PH_WARM;
        if (x0) {
            // the copy reads the staging buffer: finish it before the next slot reuses it
            { const int r_ = stream_sync(h); if (r_) return r_; }
            warm.push_back(b);
        } else if (h->ws_on && h->form != SDCA_FORM_DUAL && !h->scan) {
            learned.push_back(b);
        }
    }
    if (!warm.empty()) {
        const int rc = run_forward(h, warm, h->wa, true);
        if (rc) return rc;
    }
    if (!learned.empty()) return ws_begin(h, learned);
    return SDCA_OK;
}

// record the results of a finished slot and free it
int retire(sdca_handle *h, Queue &Qu, const std::vector<int32_t> &done)
{
    if (done.empty()) return SDCA_OK;
    const Problem &P = h->P;
    int rc = upload_slots(h, done);
    if (rc) return rc;
    if (Qu.scores) {
        {
            Timed t(h, SDCA_K_SCORE, 1, (int64_t)done.size());
            launch_score(P, h->sd, h->list, (int)done.size(), h->wa, h->cfg.gap_state, h->rows,
                         h->stream);
        }
        CKL();
        CK(cudaMemcpyAsync(h->rows_h, h->rows, sizeof(float) * P.L * done.size(),
                           cudaMemcpyDeviceToHost, h->stream));
        h->prof.d2h_bytes += (int64_t)sizeof(float) * P.L * done.size();
    }
    std::vector<float> xe;
    if (Qu.x_out) xe.resize(P.Dp);
    for (size_t j = 0; j < done.size(); ++j) {
        const int b = done[j];
        SlotHost &S = h->slots[b];
        const int64_t row = Qu.x_rows ? Qu.x_rows[S.k] : S.k;
        if (Qu.x_out && row >= 0) {
            CK(cudaMemcpyAsync(xe.data(), h->wa + (int64_t)b * P.Dp, sizeof(float) * P.Dp,
                               cudaMemcpyDeviceToHost, h->stream));
            { const int r_ = stream_sync(h); if (r_) return r_; }
            engine_to_ref(P, xe.data(), Qu.x_out + row * (QQ * P.L + Q));
            h->prof.d2h_bytes += (int64_t)sizeof(float) * P.Dp;
        }
    }
    { const int r_ = stream_sync(h); if (r_) return r_; }
    for (size_t j = 0; j < done.size(); ++j) {
        const int b = done[j];
        SlotHost &S = h->slots[b];
        if (Qu.scores) std::memcpy(Qu.scores + S.k * P.L, h->rows_h + j * P.L, sizeof(float) * P.L);
        if (Qu.stats) {
            sdca_locus_stat &st = Qu.stats[S.k];
            st.f = S.f_final;
            st.gnorm = S.gmax;
            st.iterations = S.iterations;
            st.nfeval = (int32_t)S.nfeval;
            st.contractions = (int32_t)S.contractions;
            st.status = S.status;
            st.restarts = S.restarts;
            st.skipped_pairs = S.skipped;
            st.weak_searches = S.weak;
            st.max_trials = S.max_trials;
        }
        h->prof.iterations += S.iterations;
        h->prof.contractions += S.contractions;
        S.phase = PH_EMPTY;
    }
    return SDCA_OK;
}

double l2_along(const Problem &P, const SlotHost &S, double stp)
{
    const double j2 = S.x2J + 2.0 * stp * S.xdJ + stp * stp * S.ddJ;
    const double h2 = S.x2H + 2.0 * stp * S.xdH + stp * stp * S.ddH;
    return P.lambda_J * j2 + P.lambda_h * h2;
}

double dl2_along(const Problem &P, const SlotHost &S, double stp)
{
    return 2.0 * P.lambda_J * (S.xdJ + stp * S.ddJ) + 2.0 * P.lambda_h * (S.xdH + stp * S.ddH);
}

// phase A: line-search rounds until no slot needs a trial
int phase_trials(sdca_handle *h, Queue &Qu)
{
    const Problem &P = h->P;
    for (;;) {
        std::vector<int32_t> lst;
        for (int b = 0; b < P.Bmax; ++b) {
            const int ph = h->slots[b].phase;
            if (ph == PH_INIT || ph == PH_LS || ph == PH_FINAL_EVAL || ph == PH_FINALIZE || ph == PH_REFRESH)
                lst.push_back(b);
        }
        if (lst.empty()) return SDCA_OK;
        int rc = upload_slots(h, lst);
        if (rc) return rc;
        rc = zero_acc(h);
        if (rc) return rc;
        {
            Timed t(h, SDCA_K_LINESEARCH, 1, (int64_t)lst.size());
            launch_trial(P, h->sd, h->list, (int)lst.size(), h->lbase, h->u, h->rstate, h->w, h->R, h->acc,
                         h->stream);
        }
        CKL();
        rc = fetch_acc(h);
        if (rc) return rc;
        std::vector<int32_t> done;
        for (int b : lst) {
            SlotHost &S = h->slots[b];
            const double fdata = acc_get(h, b, ACC_F);
            for (int a = 0; a < Q; ++a) S.rs[a] = acc_get(h, b, ACC_RS0 + a);
            if (S.phase == PH_INIT) {
                S.f = fdata;  // the L2 part is added once |x|^2 is known
                S.phase = PH_READY_INIT;
            } else if (S.phase == PH_REFRESH) {
                S.f = fdata;
                S.phase = PH_READY_REFRESH;
            } else if (S.phase == PH_FINALIZE) {
                S.f_final = fdata + P.lambda_J * S.x2J + P.lambda_h * S.x2H;
                done.push_back(b);
            } else if (S.phase == PH_FINAL_EVAL) {
                S.f = fdata + l2_along(P, S, S.stp);
                S.phase = PH_READY_STEP;
            } else {  // PH_LS
                const double f = fdata + l2_along(P, S, S.stp);
                const double dg = acc_get(h, b, ACC_DG) + dl2_along(P, S, S.stp);
                S.trials++;
                if (!std::isfinite(f) || !std::isfinite(dg)) {
                    S.f = f;
                    S.phase = PH_READY_STEP;
                    continue;
                }
                const double stp_eval = S.stp;
                if (S.ls.feed(f, dg) == MoreThuente::DONE) {
                    S.stp = stp_eval;  // the accepted point is the last trial
                    S.f = f;
                    S.phase = PH_READY_STEP;
                    if (S.ls.info != 1) S.weak++;
                    S.max_trials = std::max(S.max_trials, S.trials);
                } else {
                    S.stp = S.ls.stp;
                }
            }
        }
        if (!done.empty()) {
            rc = retire(h, Qu, done);
            if (rc) return rc;
            rc = refill(h, Qu);
            if (rc) return rc;
        }
    }
}

// phase B: accept, gradient, tests, new direction, forward contraction
int phase_step(sdca_handle *h)
{
    const Problem &P = h->P;
    const int m = P.m;
    std::vector<int32_t> all, steps;
    for (int b = 0; b < P.Bmax; ++b) {
        SlotHost &S = h->slots[b];
        if (S.phase == PH_READY_STEP) {
            steps.push_back(b);
            all.push_back(b);
            S.push = true;
            // a ring position outside the live history (there are m + 1)
            int pos = 0;
            while (std::find(S.hist.begin(), S.hist.end(), pos) != S.hist.end()) ++pos;
            S.ring_new = pos;
        } else if (S.phase == PH_READY_INIT || S.phase == PH_READY_REFRESH) {
            all.push_back(b);
            S.push = false;
            S.ring_new = -1;
        }
    }
    if (all.empty()) return SDCA_OK;
    int rc = upload_slots(h, all);
    if (rc) return rc;
    // The running logits lbase += stp u carry the rounding of every forward
    // contraction, and the sequences share that rounding; every
    // refresh_every accepted steps a slot's logits are recomputed at its
    // accepted point instead (tensor-core form: one extra forward).
    std::vector<int32_t> fresh, drift;
    for (int b : steps) {
        SlotHost &S = h->slots[b];
        S.xmax += S.stp * S.dmax;
        if (h->form == SDCA_FORM_TC && ++S.since_refresh >= h->tc_refresh_every) {
            S.since_refresh = 0;
            fresh.push_back(b);
        } else {
            drift.push_back(b);
        }
    }
    if (!steps.empty()) {
        rc = upload_slots(h, steps);
        if (rc) return rc;
        {
            Timed t(h, SDCA_K_ACCEPT, 1, (int64_t)steps.size());
            launch_accept(P, h->sd, h->list, (int)steps.size(), h->wa, h->d, h->Spool, h->hist_bf16,
                          h->stream);
        }
        CKL();
        if (!drift.empty()) {
            rc = upload_list(h, drift);
            if (rc) return rc;
            Timed t(h, SDCA_K_ACCEPT, 1, (int64_t)drift.size());
            launch_lbase_update(P, h->sd, h->list, (int)drift.size(), h->lbase, h->u, h->stream);
        }
        CKL();
        if (!fresh.empty()) {
            for (int b : fresh) {
                h->sd_h[b].tc_scale = pow2_scale(h->slots[b].xmax);
                h->sd_h[b].tc_inv_scale = 1.0 / h->sd_h[b].tc_scale;
            }
            rc = run_forward(h, fresh, h->wa, true, true);
            if (rc) return rc;
            // node beliefs and objective at the recomputed logits
            for (int b : fresh) {
                h->slots[b].stp = 0.0;
                h->slots[b].use_u = false;
            }
            rc = upload_slots(h, fresh);
            if (rc) return rc;
            rc = zero_acc(h);
            if (rc) return rc;
            {
                Timed t(h, SDCA_K_LINESEARCH, 1, (int64_t)fresh.size());
                launch_trial(P, h->sd, h->list, (int)fresh.size(), h->lbase, h->u, h->rstate, h->w, h->R,
                             h->acc, h->stream);
            }
            CKL();
            rc = fetch_acc(h);
            if (rc) return rc;
            for (int b : fresh) {
                SlotHost &S = h->slots[b];
                S.f_fresh = acc_get(h, b, ACC_F);
                for (int a = 0; a < Q; ++a) S.rs[a] = acc_get(h, b, ACC_RS0 + a);
            }
            rc = upload_slots(h, all);
            if (rc) return rc;
        }
        rc = upload_list(h, all);
        if (rc) return rc;
    }
    std::vector<char> was_fresh(P.Bmax, 0);
    for (int b : fresh) was_fresh[b] = 1;
    rc = zero_acc(h);
    if (rc) return rc;
    if (h->form == SDCA_FORM_TC) {
        Timed t(h, SDCA_K_BACKWARD, 4, (int64_t)all.size());
        CK(tc_launch_bwd(h->tc, P, h->sd, h->list, (int)all.size(), h->R, h->r_scale, h->Rhi, h->Rlo,
                         h->gpool, h->tc_err, h->stream));
        launch_grad_finalize(P, h->sd, h->list, (int)all.size(), h->wa, h->gpool, h->Ypool, h->Spool,
                             h->hist_bf16, h->acc, h->stream);
        launch_hpart(P, h->sd, h->list, (int)all.size(), h->wa, h->gpool, h->Ypool, h->Spool,
                     h->hist_bf16, h->acc, h->stream);
    } else {
        Timed t(h, SDCA_K_BACKWARD, 2, (int64_t)all.size());
        launch_bwd_gather(P, h->XT, h->sd, h->list, (int)all.size(), h->R, h->wa, h->gpool, h->Ypool,
                          h->Spool, h->hist_bf16, h->acc, h->stream);
        launch_hpart(P, h->sd, h->list, (int)all.size(), h->wa, h->gpool, h->Ypool, h->Spool,
                     h->hist_bf16, h->acc, h->stream);
    }
    CKL();
    rc = fetch_acc(h);
    if (rc) return rc;

    std::vector<int32_t> cont, fin;
    for (int b : all) {
        SlotHost &S = h->slots[b];
        S.contractions++;
        S.gcur = 1 - S.gcur;
        S.g2 = acc_get(h, b, ACC_G2);
        S.x2J = acc_get(h, b, ACC_X2J);
        S.x2H = acc_get(h, b, ACC_X2H);
        {
            const double gm = acc_get(h, b, ACC_GMAX);
            S.gmax = gm;
        }
        bool stop = false;
        if (S.phase == PH_READY_INIT) {
            S.f += P.lambda_J * S.x2J + P.lambda_h * S.x2H;
            S.nfeval = 1;
        } else if (S.phase == PH_READY_REFRESH) {
            // same point, logits recomputed exactly: a fresh gradient, no new pair
            S.f += P.lambda_J * S.x2J + P.lambda_h * S.x2H;
            if (S.gmax < h->cfg.gradient_threshold) {
                S.status = 0;
                stop = true;
            }
        } else {
            S.iterations++;
            S.nfeval += 2 + S.trials;
            const double sy = acc_get(h, b, ACC_SY), yy = acc_get(h, b, ACC_YY), ss = acc_get(h, b, ACC_SS);
            // keep a pair only if it carries curvature above the rounding of
            // the FP32 gradients: cos(s, y) > 1e-3
            if (sy > 1e-3 * std::sqrt(ss * yy) && yy > 0.0 && std::isfinite(sy) && std::isfinite(yy)) {
                if ((int)S.hist.size() == m) S.hist.pop_front();
                S.hist.push_back(S.ring_new);
                S.gamma = sy / yy;
                S.iter++;
            } else {
                S.ring_new = -1;  // pair not usable: keep the history as it is
                S.skipped++;
            }
            if (was_fresh[b]) S.f = S.f_fresh + P.lambda_J * S.x2J + P.lambda_h * S.x2H;
            if (S.iterations > h->cfg.max_iterations) {
                S.status = 1;
                stop = true;
            } else if (S.gmax < h->cfg.gradient_threshold) {
                S.status = 0;
                stop = true;
            } else if (S.stalled) {
                S.status = 2;  // no downhill step left at working precision
                stop = true;
            }
        }
        if (!std::isfinite(S.f) || !std::isfinite(S.g2) || !std::isfinite(S.gmax)) {
            S.status = -1;
            stop = true;
        }
        if (!stop) {
            const double releps = 1e-4 * std::max(1.0, std::sqrt(S.x2J + S.x2H));
            if (std::sqrt(S.g2) < releps) {
                S.status = 2;
                stop = true;
            }
        }
        if (stop) fin.push_back(b);
        else cont.push_back(b);
    }

    // Slots approaching the threshold get their logits recomputed from the
    // stored parameters: the running logits lbase += stp u carry the rounding
    // of every forward contraction, and near the threshold that drift is
    // larger than the gradient left to remove.
    {
        std::vector<int32_t> keep, refresh;
        for (int b : cont) {
            SlotHost &S = h->slots[b];
            const bool near = S.gmax < h->refresh_factor * h->cfg.gradient_threshold;
            if (h->form != SDCA_FORM_TC && S.phase == PH_READY_STEP && near &&
                S.iterations - S.last_refresh >= h->refresh_every) {
                refresh.push_back(b);
                S.last_refresh = S.iterations;
            } else {
                keep.push_back(b);
            }
        }
        if (!refresh.empty()) {
            rc = run_forward(h, refresh, h->wa, true);
            if (rc) return rc;
            for (int b : refresh) {
                SlotHost &S = h->slots[b];
                S.phase = PH_REFRESH;
                S.stp = 0.0;
                S.use_u = false;
                S.refreshes++;
            }
            cont.swap(keep);
        }
    }

    // converged slots: refresh their logits from the stored parameters
    if (!fin.empty()) {
        rc = run_forward(h, fin, h->wa, true);
        if (rc) return rc;
        for (int b : fin) {
            SlotHost &S = h->slots[b];
            S.phase = PH_FINALIZE;
            S.stp = 0.0;
            S.use_u = false;
        }
    }
    if (cont.empty()) return SDCA_OK;

    // history dots for slots with history
    std::vector<int32_t> withh;
    for (int b : cont)
        if (!h->slots[b].hist.empty()) withh.push_back(b);
    if (!withh.empty()) {
        rc = upload_slots(h, withh);
        if (rc) return rc;
        CK(cudaMemsetAsync(h->dots, 0, sizeof(double) * 4 * MAXHIST * P.Bmax, h->stream));
        {
            Timed t(h, SDCA_K_HISTORY, 1, (int64_t)withh.size());
            launch_hist_dots(P, h->sd, h->list, (int)withh.size(), h->gpool, h->Spool, h->Ypool,
                             h->hist_bf16, h->dots, h->stream);
        }
        CKL();
        CK(cudaMemcpyAsync(h->dots_h, h->dots, sizeof(double) * 4 * MAXHIST * P.Bmax,
                           cudaMemcpyDeviceToHost, h->stream));
        { const int r_ = stream_sync(h); if (r_) return r_; }
    }
    for (int b : cont) {
        SlotHost &S = h->slots[b];
        SlotDev &D = h->sd_h[b];
        const int k = (int)S.hist.size();
        D.coef_g = -1.0;
        if (k > 0) {
            const double *dt = h->dots_h + (int64_t)b * 4 * MAXHIST;
            // the newest pair supplies a new column of S^T Y and a row of Y^T Y
            if (S.ring_new >= 0) {
                const int pn = S.ring_new;
                for (int j = 0; j < k; ++j) {
                    const int pj = S.hist[j];
                    S.SY[pj][pn] = dt[2 * MAXHIST + j];
                    S.YY[pj][pn] = dt[3 * MAXHIST + j];
                    S.YY[pn][pj] = dt[3 * MAXHIST + j];
                }
            }
            double Rm[MAXHIST * MAXHIST], YYm[MAXHIST * MAXHIST], sg[MAXHIST], yg[MAXHIST];
            for (int a = 0; a < k; ++a) {
                sg[a] = dt[a];
                yg[a] = dt[MAXHIST + a];
                for (int c = 0; c < k; ++c) {
                    Rm[a * k + c] = (a <= c) ? S.SY[S.hist[a]][S.hist[c]] : 0.0;
                    YYm[a * k + c] = S.YY[S.hist[a]][S.hist[c]];
                }
            }
            double cg, cS[MAXHIST], cY[MAXHIST];
            if (lbfgs_compact_coeffs(k, Rm, YYm, sg, yg, S.gamma, &cg, cS, cY)) {
                D.coef_g = cg;
                for (int a = 0; a < k; ++a) {
                    D.coefS[a] = cS[a];
                    D.coefY[a] = cY[a];
                }
            } else {
                S.hist.clear();
                S.iter = 0;
            }
        }
    }
    // direction (the coefficient fields of the mirror are already set)
    auto run_direction = [&](const std::vector<int32_t> &lst) -> int {
        for (int b : lst) {
            SlotHost &S = h->slots[b];
            SlotDev &D = h->sd_h[b];
            D.nhist = (int)S.hist.size();
            for (int j = 0; j < D.nhist; ++j) D.ring[j] = S.hist[j];
        }
        int r2 = staged_h2d(h, h->sd, h->sd_h, sizeof(SlotDev) * P.Bmax);
        if (r2) return r2;
        r2 = upload_list(h, lst);
        if (r2) return r2;
        r2 = zero_acc(h);
        if (r2) return r2;
        {
            Timed t(h, SDCA_K_DIRECTION, 1, (int64_t)lst.size());
            launch_direction(P, h->sd, h->list, (int)lst.size(), h->gpool, h->Spool, h->Ypool,
                             h->hist_bf16, h->wa, h->d, h->acc, h->stream);
        }
        CKL();
        return fetch_acc(h);
    };
    for (int b : cont) h->sd_h[b].gcur = h->slots[b].gcur;
    rc = run_direction(cont);
    if (rc) return rc;
    std::vector<int32_t> restart;
    for (int b : cont) {
        SlotHost &S = h->slots[b];
        S.gd = acc_get(h, b, ACC_GD);
        S.ddJ = acc_get(h, b, ACC_DDJ);
        S.ddH = acc_get(h, b, ACC_DDH);
        S.xdJ = acc_get(h, b, ACC_XDJ);
        S.xdH = acc_get(h, b, ACC_XDH);
        S.dmax = acc_get(h, b, ACC_DMAX);
        h->sd_h[b].tc_scale = pow2_scale(S.dmax);
        h->sd_h[b].tc_inv_scale = 1.0 / h->sd_h[b].tc_scale;
        const double releps = 1e-4 * std::max(1.0, std::sqrt(S.x2J + S.x2H));
        if (!S.hist.empty() && (S.force_restart || !(S.gd <= -1e-4 * releps))) restart.push_back(b);
        S.force_restart = false;
    }
    std::vector<char> restarted(P.Bmax, 0);
    if (!restart.empty()) {
        // not a usable descent direction: restart from steepest descent
        for (int b : restart) {
            h->slots[b].hist.clear();
            h->slots[b].iter = 0;
            h->slots[b].restarts++;
            h->sd_h[b].coef_g = -1.0;
            restarted[b] = 1;
        }
        rc = run_direction(restart);
        if (rc) return rc;
        for (int b : restart) {
            SlotHost &S = h->slots[b];
            S.gd = acc_get(h, b, ACC_GD);
            S.ddJ = acc_get(h, b, ACC_DDJ);
            S.ddH = acc_get(h, b, ACC_DDH);
            S.xdJ = acc_get(h, b, ACC_XDJ);
            S.xdH = acc_get(h, b, ACC_XDH);
            S.dmax = acc_get(h, b, ACC_DMAX);
            h->sd_h[b].tc_scale = pow2_scale(S.dmax);
            h->sd_h[b].tc_inv_scale = 1.0 / h->sd_h[b].tc_scale;
        }
    }
    rc = zero_acc(h);
    if (rc) return rc;
    rc = run_forward(h, cont, h->d, false);
    if (rc) return rc;
    rc = fetch_acc(h);
    if (rc) return rc;
    for (int b : cont) {
        SlotHost &S = h->slots[b];
        const double alpha_init = restarted[b] ? 1.0 : 1.0 / std::sqrt(S.g2);
        S.trials = 0;
        S.use_u = true;
        S.push = false;
        // slope of the search line at 0 from the numbers the trials use
        const double dg0 = acc_get(h, b, ACC_DG0) + dl2_along(P, S, 0.0);
        if (S.ls.start(S.f, dg0, alpha_init) == MoreThuente::NEED_EVAL) {
            S.stp = S.ls.stp;
            S.phase = PH_LS;
        } else {
            // not downhill along this line: stay, and restart from steepest
            // descent at the next iteration
            S.stp = 0.0;
            S.phase = PH_FINAL_EVAL;
            if (S.hist.empty()) S.stalled = true;
            else S.force_restart = true;
            S.weak++;
        }
    }
    return SDCA_OK;
}

// ---- dual form: device-driven rounds.  The L-BFGS iteration of every slot
// runs on the device (k_dual_linesearch: restart test, More-Thuente search
// and its trials; K rho; k_dual_grad: the accept and the gradient; k_dual_control:
// history, tests and the next direction's coefficients; k_dual_direction).
// The host, once per round, reads a summary of every slot (one stream
// event, taken before the direction kernel so that the host's work overlaps
// it), batches the exact max-norm checks, forms the solutions of stopped
// slots, retires finished loci and admits new ones.

double dot4h(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3]; }

// A new locus in slot b: the device state of its solver.
int dual_ctl_begin(sdca_handle *h, int b)
{
    DualCtl c;
    std::memset(&c, 0, sizeof(c));
    c.phase = DC_EVAL0;
    c.ring_new = -1;
    c.last_check = -1000;
    return staged_h2d(h, h->ctl + b, &c, sizeof(c));
}

// Stopped slots of the dual form: x in the engine layout (J = Phi^T a_x,
// J_rr = 0, h = eta_x), then the final evaluation.  J is formed exactly:
// the logits K a_x are O(1) while sum_j |K_ij a_j| is hundreds, so a
// rounding of a in the last bits of single precision would move the gradient
// at the reported x by far more than the threshold.  A tensor-core pass
// costs about the same for 1 and for 21 slots (its CTAs take two 128-column
// N tiles, 64 slot-planes: 21 slots' three planes), so stopped slots wait
// until 21 of them are ready or no slot is still iterating (`force`: now),
// and a pass takes whole groups of 21 while it can.
int dual_convert(sdca_handle *h, bool force)
{
    const Problem &P = h->P;
    constexpr int GROUP = 21;
    std::vector<int32_t> fin;
    int active = 0;
    for (int b = 0; b < P.Bmax; ++b) {
        const int ph = h->slots[b].phase;
        if (ph == PH_CONVERT) fin.push_back(b);
        else if (ph != PH_EMPTY && ph != PH_FINALIZE) ++active;
    }
    if (fin.empty() || (!force && active > 0 && (int)fin.size() < std::min(GROUP, P.Bmax))) return SDCA_OK;
    // the three digit planes of up to Bmax / 3 slots go through one tensor-core
    // pass (the one-hot operand is streamed once for all of them)
    const int per_pass = P.Bmax / 3;
    if (per_pass >= 1 && (int)fin.size() > per_pass) fin.resize(per_pass);
    if (!force && active > 0 && (int)fin.size() > GROUP) fin.resize(fin.size() / GROUP * GROUP);
    for (int b : fin) {
        const SlotHost &S = h->slots[b];
        h->sd_h[b].tc_scale = S.amax_x > 0.0 ? std::ldexp(1.0, 32) / S.amax_x : 1.0;
        for (int a = 0; a < Q; ++a) h->sd_h[b].eta[a] = S.eta_x[a];
    }
    int rc = upload_slots(h, fin);
    if (rc) return rc;
    if (per_pass >= 1) {
        Timed t(h, SDCA_K_BACKWARD, 4, 3 * (int64_t)fin.size());
        const int nf = (int)fin.size();
        launch_dual_digits3(P, h->sd, h->list, nf, h->dv, h->Rchk, h->stream);
        CK(tc_launch_bwd(h->tc, P, h->sd, h->list, nf, h->Rchk, 1.0f, h->Rhi, h->Rlo, h->gpool, h->tc_err,
                         h->stream, true, nullptr, 0, 3));   // digits |D| <= 2^10: exact in fp16
        launch_dual_planes_to_wa(P, h->sd, h->list, nf, h->gpool, h->wa, h->stream);
    } else {
        Timed t(h, SDCA_K_BACKWARD, 3 * 4 + 1, 3 * (int64_t)fin.size());
        for (int d = 0; d < 3; ++d) {
            launch_dual_digits(P, h->sd, h->list, (int)fin.size(), d, h->dv, h->Rchk, h->stream);
            CK(tc_launch_bwd(h->tc, P, h->sd, h->list, (int)fin.size(), h->Rchk, 1.0f, h->Rhi, h->Rlo, h->gpool,
                             h->tc_err, h->stream, true));   // digits |D| <= 2^10: exact in fp16
            launch_dual_digit_acc(P, h->sd, h->list, (int)fin.size(), d, h->gpool, h->J64, h->stream);
        }
        launch_dual_to_wa(P, h->sd, h->list, (int)fin.size(), h->J64, h->wa, h->stream);
    }
    CKL();
    for (int b : fin) {
        SlotHost &S = h->slots[b];
        S.phase = PH_FINALIZE;
        S.stp = 0.0;
        S.use_u = false;
    }
    return SDCA_OK;
}

// Score rows of retired slots travel to the host without a wait: copied into
// the caller's array after the next round's event (or at the end).
int dual_flush_rows(sdca_handle *h, Queue &Qu)
{
    const Problem &P = h->P;
    for (size_t j = 0; j < h->rows_pending.size(); ++j)
        std::memcpy(Qu.scores + h->rows_pending[j] * P.L, h->rows_h + j * P.L, sizeof(float) * P.L);
    h->rows_pending.clear();
    return SDCA_OK;
}

int dual_retire(sdca_handle *h, Queue &Qu, const std::vector<int32_t> &done)
{
    if (done.empty()) return SDCA_OK;
    const Problem &P = h->P;
    int rc = upload_slots(h, done);
    if (rc) return rc;
    if (Qu.scores) {
        {
            Timed t(h, SDCA_K_SCORE, 1, (int64_t)done.size());
            launch_score(P, h->sd, h->list, (int)done.size(), h->wa, h->cfg.gap_state, h->rows, h->stream);
        }
        CKL();
        CK(cudaMemcpyAsync(h->rows_h, h->rows, sizeof(float) * P.L * done.size(), cudaMemcpyDeviceToHost,
                           h->stream));
        h->prof.d2h_bytes += (int64_t)sizeof(float) * P.L * done.size();
        for (int b : done) h->rows_pending.push_back(h->slots[b].k);
    }
    std::vector<float> xe;
    for (int b : done) {
        SlotHost &S = h->slots[b];
        const int64_t row = Qu.x_rows ? Qu.x_rows[S.k] : S.k;
        if (Qu.x_out && row >= 0) {
            if (xe.empty()) xe.resize(P.Dp);
            CK(cudaMemcpyAsync(xe.data(), h->wa + (int64_t)b * P.Dp, sizeof(float) * P.Dp, cudaMemcpyDeviceToHost,
                               h->stream));
            { const int r_ = stream_sync(h); if (r_) return r_; }
            engine_to_ref(P, xe.data(), Qu.x_out + row * (QQ * P.L + Q));
            h->prof.d2h_bytes += (int64_t)sizeof(float) * P.Dp;
        }
        if (Qu.rho_out) {
            // the final evaluation's residual rows w_i (p_i - onehot(y_i))
            CK(cudaMemcpyAsync(Qu.rho_out + S.k * P.N * 4, h->R + (int64_t)b * P.Nx * 4, sizeof(float) * P.N * 4,
                               cudaMemcpyDeviceToHost, h->stream));
            { const int r_ = stream_sync(h); if (r_) return r_; }
        }
        if (Qu.stats) {
            sdca_locus_stat &st = Qu.stats[S.k];
            st.f = S.f_final;
            st.gnorm = S.gmax;
            st.iterations = S.iterations;
            st.nfeval = (int32_t)S.nfeval;
            st.contractions = S.iterations + 1;
            st.status = S.status;
            st.restarts = S.restarts;
            st.skipped_pairs = S.skipped;
            st.weak_searches = S.weak;
            st.max_trials = S.max_trials;
        }
        h->prof.iterations += S.iterations;
        h->prof.contractions += S.iterations + 1;
        S.phase = PH_EMPTY;
    }
    return SDCA_OK;
}

void dual_take_summary(SlotHost &S, const DualSum &D)
{
    S.status = D.status;
    S.iterations = D.iterations;
    S.nfeval = D.nfeval;
    S.restarts = D.restarts;
    S.skipped = D.skipped;
    S.weak = D.weak;
    S.max_trials = D.max_trials;
    S.f = D.f;
    S.gmax = D.gmax;
    S.amax_g = D.amax_g;
    S.amax_x = D.amax_x;
    S.x2J = D.x2J;
    for (int a = 0; a < Q; ++a) S.eta_x[a] = D.eta_x[a];
}

// The dual form's learned start, first half: per-sequence statistics of the
// slots' target columns, the network, and its residual prediction into the
// slots' R rows (the round's K rho pass and k_dual_ws_init finish it).
int dual_ws_rows(sdca_handle *h, int nW, const int32_t *l_W)
{
    const Problem &P = h->P;
    int rc;
    if (h->knn_k != DWS_K && (rc = ws_knn(h, DWS_K))) return rc;
    Timed t(h, SDCA_K_OTHER, 3 * ((nW + h->dws_cap - 1) / h->dws_cap), nW);   // statistics, network, rows
    for (int c0 = 0; c0 < nW; c0 += h->dws_cap) {
        const int n = std::min(h->dws_cap, nW - c0);
        launch_dual_ws_feats(h->rstate, l_W + c0, n, (int)P.N, P.Nx, (int)P.L, h->w, h->knn, h->knn_d, h->dws_feats,
                             h->stream);
        mlp_infer(h->ws_params, h->ws_wb, h->dws_feats, (int64_t)n * P.Nx, h->dws_out, h->ws_err, h->stream);
        launch_dual_ws_r(l_W + c0, n, (int)P.N, P.Nx, h->dws_out, h->ws_params, h->ws_alpha, h->wf, h->R, h->stream);
    }
    CKL();
    return SDCA_OK;
}

// The iteration core of a round (dual_round has written the lists and their
// lengths): the line search of the searching slots, the K rho pass over
// the gradient pass and the learned starts, the starts themselves, the
// accept and gradient, history-dot and control kernels, the summary
// copy and the event `ev`, then the directions.  dev: every grid covers
// Bmax slots and the kernels read the list lengths from device memory -- the
// form captured in a CUDA graph and replayed every round, its classes timed
// by event nodes into `g`; otherwise the grids are the host's list lengths
// and the classes are timed as usual.
int dual_core(sdca_handle *h, const int64_t (&n)[DC_N], bool dev, cudaEvent_t ev, DualGraph *g)
{
    const Problem &P = h->P;
    const int B = (int)P.Bmax;
    const double gtol = h->cfg.gradient_threshold;
    const int32_t *l_T = h->dlist + B, *l_G = h->dlist + 2 * B, *l_W = h->dlist + 3 * B;
    const int *cnt = h->dlist + 4 * (size_t)B;
    auto len = [&](int i) { return dev ? B : (int)n[i]; };
    auto dcnt = [&](int i) -> const int * { return dev ? cnt + i : nullptr; };
    // one profile class: Timed, or an event pair recorded by the graph
    auto region = [&](int cls, int kernels, int cidx, auto &&fn) -> int {
        if (!dev) {
            if (n[cidx] <= 0) return SDCA_OK;
            Timed t(h, cls, kernels, n[cidx]);
            return fn();
        }
        const size_t k = 2 * g->recs.size();
        if (k + 1 >= g->ev.size()) return fn();   // (no event pair left: untimed)
        GraphRec r{cls, kernels, cidx, g->ev[k], g->ev[k + 1]};
        // (external: event nodes that record the event at every replay)
        CK(cudaEventRecordWithFlags(r.a, h->stream, cudaEventRecordExternal));
        const int rc = fn();
        CK(cudaEventRecordWithFlags(r.b, h->stream, cudaEventRecordExternal));
        g->recs.push_back(r);
        return rc;
    };
    int rc;
    // Profile classes of this form: "forward" is K rho (a coefficient vector's
    // logit image, as X d is in the other forms), "backward" the one-hot
    // contractions X^T a (max-norm checks, final J), "accept" the iterate
    // update and gradient assembly, "other" the control kernel and the
    // learned starts.
    if ((rc = region(SDCA_K_LINESEARCH, 1, DC_T, [&] {
             launch_dual_linesearch(P, h->ctl, l_T, len(DC_T), h->dacc, h->dv, h->ud, h->rstate,
                                    h->wf, h->P0, h->R, h->acc, h->stream, dcnt(DC_T));
             return SDCA_OK;
         })))
        return rc;
    CKL();
    if (dev || n[DC_GW] > 0) {
        CK(cudaMemsetAsync(h->csum, 0, sizeof(long long) * 16 * P.Bmax, h->stream));
        CK(cudaMemsetAsync(h->amax, 0, sizeof(double) * 2 * P.Bmax, h->stream));
        CK(cudaMemsetAsync(h->dots, 0, sizeof(double) * 4 * MAXHIST * P.Bmax, h->stream));
    }
    if ((rc = region(SDCA_K_ACCEPT, 1, DC_GW, [&] {
             launch_dual_quant(P, h->sd, l_G, len(DC_GW), h->R, h->rstate, h->qscale, h->rq, h->csum, h->stream,
                               dcnt(DC_GW));
             return SDCA_OK;
         })))
        return rc;
    if ((rc = region(SDCA_K_FORWARD, h->kd ? 2 : 1, DC_GW, [&] {
             if (h->kd)
                 CK(tc_launch_kdig(h->kd, P, l_G, len(DC_GW), h->rq, h->rstate, h->csum, 1.0 / h->qscale, h->Rd,
                                   h->KR, h->tc_err, h->stream, dcnt(DC_GW)));
             else
                 launch_dual_kprod(P, l_G, len(DC_GW), h->rstate, h->Kmat, h->qscale, h->rq, h->csum, h->KR,
                                   h->stream, dcnt(DC_GW));
             return SDCA_OK;
         })))
        return rc;
    if (!dev || h->ws_dual) {
        // the learned start: a_x = -rho^ / (2 lambda_J), K a_x exactly from the pass above
        if ((rc = region(SDCA_K_OTHER, 1, DC_W, [&] {
                 launch_dual_ws_init(P, l_W, len(DC_W), -0.5 / P.lambda_J, h->qscale, h->rq, h->KR, h->dv,
                                     h->stream, dcnt(DC_W));
                 return SDCA_OK;
             })))
            return rc;
    }
    if ((rc = region(SDCA_K_ACCEPT, 1, DC_G, [&] {
             launch_dual_grad(P, h->ctl, l_G, len(DC_G), h->qscale, h->rq, h->KR, h->dv, h->acc, h->amax, h->stream,
                              dcnt(DC_G));
             return SDCA_OK;
         })))
        return rc;
    if ((rc = region(SDCA_K_HISTORY, 1, DC_G, [&] {
             launch_dual_dots(P, h->ctl, l_G, len(DC_G), 1, h->dv, h->dots, h->stream, dcnt(DC_G));
             return SDCA_OK;
         })))
        return rc;
    if ((rc = region(SDCA_K_OTHER, 1, DC_G, [&] {
             launch_dual_control(P, h->ctl, h->sum, l_G, len(DC_G), h->cfg.max_iterations, gtol, h->acc, h->amax,
                                 h->dots, h->stream, dcnt(DC_G));
             return SDCA_OK;
         })))
        return rc;
    CKL();
    CK(cudaMemcpyAsync(h->sum_h, h->sum, sizeof(DualSum) * P.Bmax, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(h->acc_h, h->acc, sizeof(double) * NACC * P.Bmax, cudaMemcpyDeviceToHost, h->stream));
    if (h->tc_err) CK(cudaMemcpyAsync(h->flag_h + 1, h->tc_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (h->ws_err && (dev ? h->ws_dual : n[DC_W] > 0))
        CK(cudaMemcpyAsync(h->flag_h + 2, h->ws_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (dev) CK(cudaEventRecordWithFlags(ev, h->stream, cudaEventRecordExternal));
    else CK(cudaEventRecord(ev, h->stream));
    if (dev || n[DC_G] > 0) CK(cudaMemsetAsync(h->dacc, 0, sizeof(double) * NDACC * P.Bmax, h->stream));
    if ((rc = region(SDCA_K_DIRECTION, 1, DC_G, [&] {
             launch_dual_direction(P, h->ctl, l_G, len(DC_G), h->dv, h->P0, h->wf, h->rstate, h->ud, h->dacc,
                                   h->stream, dcnt(DC_G));
             return SDCA_OK;
         })))
        return rc;
    CKL();
    return SDCA_OK;
}

// Capture the iteration core into g's CUDA graph (on the lane's stream, in
// this thread's capture mode) and instantiate it.
int dual_graph_build(sdca_handle *h, DualGraph &g)
{
    if (!g.ev_round) CK(cudaEventCreateWithFlags(&g.ev_round, cudaEventDisableTiming));
    while (g.ev.size() < 24) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        g.ev.push_back(e);
    }
    g.recs.clear();
    const int64_t any[DC_N] = {1, 1, 1, 1};
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = dual_core(h, any, true, g.ev_round, &g);
    const cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (rc || e != cudaSuccess || !graph) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        g.recs.clear();
        return rc ? rc : SDCA_E_CUDA;
    }
    const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        g.exec = nullptr;
        cudaGetLastError();
        return SDCA_E_CUDA;
    }
    return SDCA_OK;
}

// A completed replay's class timings into the profile (units: the list
// lengths of that replay).
void dual_graph_collect(sdca_handle *h, DualGraph &g)
{
    if (!g.pending) return;
    for (const GraphRec &r : g.recs) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            h->prof.kernel_ms[r.cls] += ms;
            h->prof.kernel_launches[r.cls] += r.kernels;
            h->prof.kernel_units[r.cls] += g.counts[r.cidx];
        }
        h->prof.gpu_launches += r.kernels;
    }
    g.pending = false;
}

// Drop the lane's graphs (the alignment, the targets or the learned start
// changed, or the handle ends); they are captured again at the next round.
void dual_graph_reset(sdca_handle *h)
{
    for (DualGraph &g : h->dgraph) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        g.recs.clear();
        g.pending = false;
    }
    h->dgraph_next = 0;
}

void dual_graph_free(sdca_handle *h)
{
    dual_graph_reset(h);
    for (DualGraph &g : h->dgraph) {
        for (cudaEvent_t e : g.ev) cudaEventDestroy(e);
        g.ev.clear();
        if (g.ev_round) cudaEventDestroy(g.ev_round);
        g.ev_round = nullptr;
    }
}

// One round: start/final evaluations, line searches, accepts, the gradient
// pass and the control kernel for every slot, then the directions.
int dual_round(sdca_handle *h, Queue &Qu)
{
    const Problem &P = h->P;
    const double gtol = h->cfg.gradient_threshold;
    std::vector<int32_t> ef, T, G, W;
    for (int b = 0; b < P.Bmax; ++b) {
        const int ph = h->slots[b].phase;
        if (ph == PH_INIT || ph == PH_FINALIZE) ef.push_back(b);
        if (ph == PH_LS) T.push_back(b);   // iterating on the device
        if (ph == PH_WARM) W.push_back(b); // learned start formed this round
    }
    G = T;
    for (int b : ef)
        if (h->slots[b].phase == PH_INIT) G.push_back(b);
    if (ef.empty() && G.empty() && W.empty()) return dual_convert(h, true);
    // the lists [ef | T | G, W | W] and their lengths in one upload
    const int32_t *l_ef = h->dlist, *l_W = h->dlist + 3 * P.Bmax;
    const int64_t counts[DC_N] = {(int64_t)T.size(), (int64_t)G.size(), (int64_t)(G.size() + W.size()),
                                  (int64_t)W.size()};
    {
        std::vector<int32_t> all(4 * (size_t)P.Bmax + DC_N, 0);
        std::copy(ef.begin(), ef.end(), all.begin());
        std::copy(T.begin(), T.end(), all.begin() + P.Bmax);
        std::copy(G.begin(), G.end(), all.begin() + 2 * P.Bmax);
        std::copy(W.begin(), W.end(), all.begin() + 2 * P.Bmax + G.size());
        std::copy(W.begin(), W.end(), all.begin() + 3 * P.Bmax);
        for (int i = 0; i < DC_N; ++i) all[4 * (size_t)P.Bmax + i] = (int32_t)counts[i];
        for (int b : W) h->sd_h[b].locus = h->scan ? -1 : h->slots[b].locus;
        for (int b : ef) {
            h->sd_h[b].locus = h->scan ? -1 : h->slots[b].locus;
            h->sd_h[b].gcur = 0;
            h->sd_h[b].stp = 0.0;
            h->sd_h[b].flags = 0;
            // the evaluation's logits are k_x + eta: eta is zero at a start
            // (zero or learned) and eta_x at the end (set by dual_convert)
            if (h->slots[b].phase == PH_INIT)
                for (int a = 0; a < Q; ++a) h->sd_h[b].eta[a] = 0.0;
        }
        int rc = staged_h2d(h, h->sd, h->sd_h, sizeof(SlotDev) * P.Bmax);
        if (rc) return rc;
        if ((rc = staged_h2d(h, h->dlist, all.data(), sizeof(int32_t) * all.size()))) return rc;
    }
    int rc;
    if (!W.empty() && (rc = dual_ws_rows(h, (int)W.size(), l_W))) return rc;
    if ((rc = zero_acc(h))) return rc;
    if (!ef.empty()) {
        Timed t(h, SDCA_K_LINESEARCH, 1, (int64_t)ef.size());
        launch_dual_eval(P, h->sd, l_ef, (int)ef.size(), h->dv, h->rstate, h->w, h->R, h->acc, h->stream);
    }
    CKL();
    // the iteration core: a replay of this lane's CUDA graph, or the kernels one by one
    cudaEvent_t ev_sum = h->ev_round;
    DualGraph *other = nullptr;
    if (!h->dgraph_off) {
        DualGraph &g = h->dgraph[h->dgraph_next];
        if (!g.exec && dual_graph_build(h, g) != SDCA_OK) {
            h->dgraph_off = true;   // fall back to the direct launches for the rest of the handle's life
            cudaGetLastError();
        }
        if (!h->dgraph_off) {
            CK(cudaGraphLaunch(g.exec, h->stream));
            std::copy(counts, counts + DC_N, g.counts);
            g.pending = true;
            ev_sum = g.ev_round;
            other = &h->dgraph[1 - h->dgraph_next];
            h->dgraph_next = 1 - h->dgraph_next;
        }
    }
    if (h->dgraph_off && (rc = dual_core(h, counts, false, h->ev_round, nullptr))) return rc;
    CK(cudaEventSynchronize(ev_sum));
    // the previous round's replay has completed: its timings can be read
    if (other) dual_graph_collect(h, *other);
    // every staged host-to-device copy was queued before the event
    h->stage_off = 0;
    if (h->tc_err && h->flag_h[1])
        return fail(h, SDCA_E_CUDA, "tensor-core pipeline wait timed out (kernel abandoned its tile)");
    if (!W.empty() && h->flag_h[2])
        return fail(h, SDCA_E_CUDA, "warm start: a tensor-core pipeline wait gave up");
    if (Qu.scores) dual_flush_rows(h, Qu);

    std::vector<int32_t> done, chk;
    for (int b : W) h->slots[b].phase = PH_INIT;   // start evaluation next round
    for (int b : ef) {
        SlotHost &S = h->slots[b];
        if (S.phase != PH_FINALIZE) continue;
        S.f_final = acc_get(h, b, ACC_F) + P.lambda_J * S.x2J + P.lambda_h * dot4h(S.eta_x, S.eta_x);
        done.push_back(b);
    }
    for (int b : G) {
        SlotHost &S = h->slots[b];
        const DualSum &D = h->sum_h[b];
        dual_take_summary(S, D);
        if (D.phase == DC_STOP) {
            S.phase = PH_CONVERT;
            continue;
        }
        S.phase = PH_LS;
        if (D.want_check) chk.push_back(b);
    }
    // A check pass costs one tensor-core contraction whether it serves 1 or
    // 32 slots, while a slot's extra iteration costs a small fraction of
    // that: slots wanting a check keep iterating until 8 want one, one has
    // waited 3 iterations, a relative-norm stop is pending, or at most 8
    // slots are left.  The check's verdict reaches the host with the next
    // round's summary; meanwhile the slot's kernels see it on the device.
    if (!chk.empty()) {
        int active = 0;
        bool urgent = false;
        for (int b = 0; b < P.Bmax; ++b)
            if (h->slots[b].phase == PH_LS) ++active;
        for (int b : chk) urgent = urgent || h->sum_h[b].chk_wait >= 3 || h->sum_h[b].releps_stop;
        if (!(urgent || (int)chk.size() >= 8 || active <= 8)) chk.clear();
    }
    if (!chk.empty()) {
        double sc = 0.0;
        for (int b : chk) sc = std::max(sc, h->slots[b].amax_g);
        if ((rc = upload_slots(h, chk))) return rc;
        if ((rc = zero_acc(h))) return rc;
        {
            // X^T a_g on the tensor cores with a max-only epilogue: no gradient is written
            Timed t(h, SDCA_K_BACKWARD, 4, (int64_t)chk.size());
            launch_dual_to_r(P, h->ctl, h->list, (int)chk.size(), 0, h->dv, h->Rchk, h->stream);
            CK(tc_launch_bwd(h->tc, P, h->sd, h->list, (int)chk.size(), h->Rchk, (float)pow2_scale(sc), h->Rhi,
                             h->Rlo, h->gpool, h->tc_err, h->stream, false, h->acc + ACC_GMAX, NACC));
            launch_dual_check_apply(h->ctl, h->sum, h->list, (int)chk.size(), gtol, h->acc, h->stream);
        }
        CKL();
    }
    if ((rc = dual_retire(h, Qu, done))) return rc;
    bool any_active = false;
    for (int b = 0; b < P.Bmax; ++b) any_active = any_active || h->slots[b].phase == PH_LS;
    if ((rc = dual_convert(h, !any_active))) return rc;
    if (!done.empty()) return refill(h, Qu);
    return SDCA_OK;
}

// One lane's solve over the shared queue.  Device time runs from t0_common
// (the multi-lane solve's start) or from this lane's own start event.
int solve_lane(sdca_handle *h, Queue &Qu, cudaEvent_t t0_common)
{
    CK(cudaSetDevice(h->cfg.device));
    prof_reset(h);
    h->prof.h2d_bytes = 0;
    cudaEvent_t t0 = t0_common ? t0_common : take_event(h), t1 = take_event(h);
    if (!t0 || !t1) return fail(h, SDCA_E_CUDA, "cudaEventCreate failed");
    if (!t0_common) CK(cudaEventRecord(t0, h->stream));
    for (auto &S : h->slots) S.phase = PH_EMPTY;
    int rc = refill(h, Qu);
    if (rc) return rc;
    for (;;) {
        bool any = false;
        for (auto &S : h->slots)
            if (S.phase != PH_EMPTY) any = true;
        if (!any) break;
        if (h->form == SDCA_FORM_DUAL) {
            rc = dual_round(h, Qu);
            if (rc) return rc;
            continue;
        }
        rc = phase_trials(h, Qu);
        if (rc) return rc;
        rc = phase_step(h);
        if (rc) return rc;
    }
    CK(cudaEventRecord(t1, h->stream));
    { const int r_ = stream_sync(h); if (r_) return r_; }
    if (Qu.scores) dual_flush_rows(h, Qu);
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, t0, t1));
    h->prof.solve_ms = ms;
    for (DualGraph &g : h->dgraph) dual_graph_collect(h, g);
    prof_collect(h);
    return SDCA_OK;
}

int check_ready(sdca_handle *h)
{
    if (!h) return SDCA_E_ARG;
    if (!h->has_alignment) return fail(h, SDCA_E_STATE, "no alignment set (call sdca_set_alignment)");
    return SDCA_OK;
}

} // namespace

// the network on the device: the parameter blob, its BF16 weight image and
// the error word of the tensor-core forward
static int ws_network(sdca_handle *h, const float *params)
{
    int rc;
    if (!h->ws_params && (rc = dalloc(h, &h->ws_params, MLP_BLOB_SIZE))) return rc;
    if (!h->ws_wb && (rc = dalloc(h, &h->ws_wb, MLP_WB_ELEMS))) return rc;
    if (!h->ws_err && (rc = dalloc(h, &h->ws_err, 1))) return rc;
    CK(cudaMemcpyAsync(h->ws_params, params, sizeof(float) * MLP_BLOB_SIZE, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(h->ws_err, 0, sizeof(int), h->stream));
    mlp_pack(h->ws_params, h->ws_wb, h->stream);
    CKL();
    return stream_sync(h);
}

// the solve of a loci list over the handle's lanes (sdca_solve_sel, and the
// training data of the dual form's start with rho_out)
static int solve_queue(sdca_handle *h, const uint32_t *loci, size_t n_loci, const double *x_init,
                       const int64_t *x_rows, double *x_out, float *scores, sdca_locus_stat *stats, float *rho_out)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (n_loci > 0 && !loci) return fail(h, SDCA_E_ARG, "null loci list");
    const int64_t nt = h->scan ? h->LT : h->P.L;   // scan mode: loci are target columns
    for (size_t k = 0; k < n_loci; ++k)
        if ((int64_t)loci[k] >= nt) return fail(h, SDCA_E_ARG, "locus index out of range");
    if (x_rows && !x_out) return fail(h, SDCA_E_ARG, "x_rows given without x_out");
    if (x_rows)
        for (size_t k = 0; k < n_loci; ++k)
            if (x_rows[k] < -1) return fail(h, SDCA_E_ARG, "x_rows entries must be -1 or a row index");
    std::atomic<size_t> next{0};
    std::atomic<bool> abort{false};
    auto queue_for = [&](sdca_handle *l, Queue &Qu) {
        Qu.loci = loci;
        Qu.n = n_loci;
        Qu.next = &next;
        Qu.abort = &abort;
        Qu.x_init = x_init;
        Qu.x_out = x_out;
        Qu.x_rows = x_rows;
        Qu.rho_out = rho_out;
        Qu.scores = scores;
        Qu.stats = stats;
        if (x_init) Qu.xbuf.resize(l->P.Dp);
    };
    if (h->sub.empty()) {
        Queue Qu;
        queue_for(h, Qu);
        return solve_lane(h, Qu, nullptr);
    }
    // lanes: this thread runs lane 0, one thread per further lane; all take
    // loci from the same queue and write disjoint rows of the outputs
    CK(cudaSetDevice(h->cfg.device));
    CK(cudaEventRecord(h->ev_lanes, h->stream));
    const size_t nl = 1 + h->sub.size();
    std::vector<int> rcs(nl, SDCA_OK);
    auto run = [&](size_t i) {
        sdca_handle *l = i == 0 ? h : h->sub[i - 1];
        Queue Qu;
        queue_for(l, Qu);
        rcs[i] = solve_lane(l, Qu, h->ev_lanes);
        if (rcs[i]) abort.store(true);
    };
    std::vector<std::thread> th;
    for (size_t i = 1; i < nl; ++i) {
        try {
            th.emplace_back(run, i);
        } catch (...) {
            // no thread: the lanes that run take this lane's loci
        }
    }
    run(0);
    for (auto &t : th) t.join();
    for (size_t i = 0; i < nl; ++i)
        if (rcs[i]) return i == 0 ? rcs[i] : fail(h, rcs[i], "lane " + std::to_string(i) + ": " + h->sub[i - 1]->err);
    for (const sdca_handle *l : h->sub) {
        const sdca_profile &q = l->prof;
        sdca_profile &p = h->prof;
        p.solve_ms = std::max(p.solve_ms, q.solve_ms);
        for (int c = 0; c < 8; ++c) {
            p.kernel_ms[c] += q.kernel_ms[c];
            p.kernel_launches[c] += q.kernel_launches[c];
            p.kernel_units[c] += q.kernel_units[c];
        }
        p.gpu_launches += q.gpu_launches;
        p.iterations += q.iterations;
        p.contractions += q.contractions;
        p.h2d_bytes += q.h2d_bytes;
        p.d2h_bytes += q.d2h_bytes;
    }
    return SDCA_OK;
}


extern "C" {

int sdca_abi_version(void) { return SDCA_ABI_VERSION; }

int sdca_config_default(sdca_config *cfg)
{
    if (!cfg) return SDCA_E_ARG;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->q = 4;
    cfg->gap_state = 3;
    cfg->lambda_h = -1.0;
    cfg->lambda_J = -1.0;
    cfg->gradient_threshold = 1e-3;
    cfg->max_iterations = 2000;
    cfg->history = 10;
    cfg->batch = 64;
    cfg->form = SDCA_FORM_GATHER;
    cfg->flags = 0;
    cfg->device = 0;
    cfg->stream = nullptr;
    return SDCA_OK;
}

static int create_lane(const sdca_config *cfg, const sdca_handle *owner, sdca_handle **out);

int sdca_create(const sdca_config *cfg, sdca_handle **out)
{
    if (!cfg || !out) return fail(nullptr, SDCA_E_ARG, "sdca_create: null argument");
    *out = nullptr;
    if (cfg->lanes < 0 || cfg->lanes > 16) return fail(nullptr, SDCA_E_ARG, "lanes must be in 0..16");
    sdca_handle *h = nullptr;
    int rc = create_lane(cfg, nullptr, &h);
    if (rc) return rc;
    for (int i = 1; i < cfg->lanes; ++i) {
        sdca_config c = *cfg;
        c.lanes = 1;
        c.stream = nullptr;
        sdca_handle *s = nullptr;
        if ((rc = create_lane(&c, h, &s)) == SDCA_OK) {
            h->sub.push_back(s);
            continue;
        }
        sdca_destroy(h);
        return rc;
    }
    if (!h->sub.empty() && cudaEventCreate(&h->ev_lanes) != cudaSuccess) {
        sdca_destroy(h);
        return fail(nullptr, SDCA_E_CUDA, "cudaEventCreate failed");
    }
    *out = h;
    return SDCA_OK;
}

// one lane; with an owner, the lane uses the owner's alignment buffers
static int create_lane(const sdca_config *cfg, const sdca_handle *owner, sdca_handle **out)
{
    sdca_handle *h = nullptr;
    if (cfg->q != Q) return fail(nullptr, SDCA_E_UNSUPPORTED, "only q = 4 (the triallelic envelope) is supported");
    if (cfg->n_seqs < 1 || cfg->n_loci < 2)
        return fail(nullptr, SDCA_E_ARG, "need at least 1 sequence and 2 loci");
    if (cfg->n_seqs > (1LL << 30) || cfg->n_loci > (1LL << 26))
        return fail(nullptr, SDCA_E_ARG, "alignment too large");
    if (cfg->history < 1 || cfg->history > MAXHIST)
        return fail(nullptr, SDCA_E_ARG, "history must be in 1..10");
    if (cfg->batch < 1 || cfg->batch > 4096) return fail(nullptr, SDCA_E_ARG, "batch must be in 1..4096");
    if (cfg->gap_state < -1 || cfg->gap_state >= Q) return fail(nullptr, SDCA_E_ARG, "gap_state out of range");
    if (cfg->form != SDCA_FORM_GATHER && cfg->form != SDCA_FORM_TC && cfg->form != SDCA_FORM_DUAL)
        return fail(nullptr, SDCA_E_UNSUPPORTED, "unknown contraction form");
    if (cfg->form == SDCA_FORM_DUAL && cfg->n_seqs > 16383)
        return fail(nullptr, SDCA_E_UNSUPPORTED, "the dual form supports at most 16383 sequences");
    if (!(cfg->gradient_threshold >= 0.0) || cfg->max_iterations < 0)
        return fail(nullptr, SDCA_E_ARG, "invalid stopping criteria");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(nullptr, SDCA_E_CUDA, "no CUDA device available");
    }
    if (cfg->device < 0 || cfg->device >= ndev) return fail(nullptr, SDCA_E_ARG, "device ordinal out of range");
    if (cudaSetDevice(cfg->device) != cudaSuccess) return fail(nullptr, SDCA_E_CUDA, "cudaSetDevice failed");
    h = new (std::nothrow) sdca_handle();
    if (!h) return fail(nullptr, SDCA_E_NOMEM, "host allocation failed");
    h->cfg = *cfg;
    if (cfg->stream) {
        h->stream = static_cast<cudaStream_t>(cfg->stream);
    } else {
        if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete h;
            return fail(nullptr, SDCA_E_CUDA, "cudaStreamCreate failed");
        }
        h->own_stream = true;
    }
    h->hist_bf16 = (cfg->flags & SDCA_FLAG_HISTORY_BF16) ? 1 : 0;
    Problem &P = h->P;
    P.N = cfg->n_seqs;
    P.L = cfg->n_loci;
    P.Lx = round_up(P.L, 64);
    P.Nx = round_up(P.N, 64);
    P.Dp = round_up(QQ * P.L + Q, 64);
    P.m = cfg->history;
    P.ring = P.m + 1;
    P.Bmax = cfg->batch;
    {
        // locus chunks of the forward gather: enough CTAs to fill the GPU
        const int64_t seq_tiles = (P.N + 255) / 256, slot_groups = (P.Bmax + 7) / 8;
        int64_t want = (2 * 152 + seq_tiles * slot_groups - 1) / (seq_tiles * slot_groups);
        want = std::max<int64_t>(1, want);
        P.LC = round_up((P.L + want - 1) / want, 32);
        P.LC = std::max<int64_t>(P.LC, 512);
        P.Cg = (P.L + P.LC - 1) / P.LC;
        P.C = std::max<int64_t>(P.Cg, cfg->form != SDCA_FORM_GATHER ? 24 : 1);
    }
    h->form = cfg->form;
    if (const char *e = std::getenv("SDCA_REFRESH_EVERY")) h->refresh_every = std::max(1, std::atoi(e));
    if (const char *e = std::getenv("SDCA_REFRESH_FACTOR")) h->refresh_factor = std::atof(e);
    if (const char *e = std::getenv("SDCA_TC_REFRESH_EVERY")) h->tc_refresh_every = std::max(1, std::atoi(e));
    h->slots.resize(P.Bmax);
    int rc = SDCA_OK;
    const size_t B = P.Bmax;
    const size_t hsz = h->hist_bf16 ? 2 : 4;
    const bool dual = h->form == SDCA_FORM_DUAL;
    const bool tcres = h->form != SDCA_FORM_GATHER;   // the dual form uses the tensor-core backward too
    // the dual form keeps its history as N x 4 coefficient pairs, not as D-vectors
    const size_t hist_bytes = dual ? 256 : B * P.ring * P.Dp * hsz;
    const size_t NV = DV_S + 2 * (size_t)P.ring;
    const bool shared = owner != nullptr;
    if (shared) {
        h->shared_alignment = true;
        h->X = owner->X;
        h->XT = owner->XT;
        h->w = owner->w;
        h->wf = owner->wf;
        h->Kmat = owner->Kmat;
        h->Kd = owner->Kd;
    }
    // The dual form keeps its iteration in N x 4 vectors: of the D-vectors it
    // needs x (the formed solution, wa) per slot, gradient buffers for its
    // one-hot contractions (the digit planes of up to B / 3 slots, or two per
    // slot below 3 slots, which also serve sdca_eval) and the FP64 solution
    // image only below 3 slots; no primal direction and no forward operand.
    const bool dual_small = dual && B < 3;
    const size_t n_d = dual ? 0 : B, n_gpool = dual && !dual_small ? std::max<size_t>(B, 2) : 2 * B;
    if ((!shared && ((rc = dalloc(h, &h->X, (size_t)P.N * P.Lx)) || (rc = dalloc(h, &h->XT, (size_t)P.L * P.Nx)) ||
                     (rc = dalloc(h, &h->w, (size_t)P.Nx)) || (rc = dalloc(h, &h->wf, (size_t)P.Nx)))) ||
        (rc = dalloc(h, &h->rstate, B * P.Nx)) ||
        (rc = dalloc(h, &h->wa, B * P.Dp)) || (n_d && (rc = dalloc(h, &h->d, n_d * P.Dp))) ||
        (rc = dalloc(h, &h->gpool, n_gpool * P.Dp)) || (rc = dalloc(h, &h->u, B * P.Nx * 4)) ||
        (rc = dalloc(h, &h->R, B * P.Nx * 4)) || (rc = dalloc(h, &h->lbase, B * P.Nx * 4)) ||
        (rc = dalloc(h, &h->partial, (size_t)P.C * B * P.Nx * 4)) ||
        (rc = dalloc(h, &h->partial64, (size_t)P.Cg * B * P.Nx * 4)) ||
        (rc = dalloc(h, &h->rows, B * P.L)) || (rc = dalloc(h, &h->acc, B * NACC)) ||
        (rc = dalloc(h, &h->dots, B * 4 * MAXHIST)) || (rc = dalloc(h, &h->sd, B)) ||
        (rc = dalloc(h, &h->list, B)) || (rc = dalloc(h, &h->flag, 4)) ||
        (rc = dalloc(h, reinterpret_cast<uint8_t **>(&h->Spool), hist_bytes)) ||
        (rc = dalloc(h, reinterpret_cast<uint8_t **>(&h->Ypool), hist_bytes)) ||
        (rc = halloc(h, &h->sd_h, B)) || (rc = halloc(h, &h->list_h, B)) ||
        (rc = halloc(h, &h->acc_h, B * NACC)) || (rc = halloc(h, &h->dots_h, B * 4 * MAXHIST)) ||
        (rc = halloc(h, &h->rows_h, B * P.L)) || (rc = halloc(h, &h->flag_h, 4)) ||
        (rc = halloc(h, &h->stage, (h->stage_cap = 64 * (((sizeof(SlotDev) + 4) * B + 1024 + 255) & ~(size_t)255)))) ||
        (dual && ((rc = halloc(h, &h->amax_h, 2 * B)) || (rc = halloc(h, &h->sum_h, B)) ||
                  (rc = dalloc(h, &h->ctl, B)) || (rc = dalloc(h, &h->sum, B)) ||
                  (rc = dalloc(h, &h->dacc, B * NDACC)) || (rc = dalloc(h, &h->dlist, 4 * B + DC_N)) ||
                  (rc = dalloc(h, &h->dv, B * NV * 2 * P.Nx * 4)) ||
                  (rc = dalloc(h, &h->KR, B * P.Nx * 4)) || (rc = dalloc(h, &h->amax, 2 * B)) ||
                  (rc = dalloc(h, &h->rq, B * P.Nx * 4)) || (rc = dalloc(h, &h->csum, 16 * B)) ||
                  (rc = dalloc(h, &h->Rchk, B * P.Nx * 4)) || (dual_small && (rc = dalloc(h, &h->J64, B * P.Dp))) ||
                  (rc = dalloc(h, &h->P0, B * P.Nx * 4)) || (rc = dalloc(h, &h->ud, B * P.Nx * 4)) ||
                  (!shared && (rc = dalloc(h, &h->Kmat, (size_t)P.Nx * P.Nx))) ||
                  (P.N <= 4000 && P.L < (1 << 18) &&
                   ((!shared && (rc = dalloc(h, &h->Kd, (size_t)3 * kd_nk_rows(P) * P.Nx))) ||
                    (rc = dalloc(h, &h->Rd, (size_t)4 * kd_nr_rows(P) * P.Nx)))))) ||
        (tcres &&
         ((!dual && (rc = dalloc(h, &h->Dhi, 4 * B * (size_t)round_up(4 * P.L, 64)))) ||
          (!dual && (rc = dalloc(h, &h->Dlo, 4 * B * (size_t)round_up(4 * P.L, 64)))) ||
          (rc = dalloc(h, &h->Rhi, 4 * B * (size_t)P.Nx)) || (rc = dalloc(h, &h->Rlo, 4 * B * (size_t)P.Nx)) ||
          (rc = dalloc(h, &h->tc_err, 4))))) {
        std::string msg = h->err;
        free_all(h);
        if (h->own_stream) cudaStreamDestroy(h->stream);
        delete h;
        return fail(nullptr, rc, msg);
    }
    if (cudaStreamSynchronize(h->stream) != cudaSuccess ||
        (dual && cudaEventCreateWithFlags(&h->ev_round, cudaEventDisableTiming) != cudaSuccess)) {
        free_all(h);
        if (h->own_stream) cudaStreamDestroy(h->stream);
        delete h;
        return fail(nullptr, SDCA_E_CUDA, "initialisation failed");
    }
    {
        // the dual form replays its iteration core as a CUDA graph unless SDCA_DUAL_GRAPH=0
        const char *e = std::getenv("SDCA_DUAL_GRAPH");
        h->dgraph_off = !dual || (e && e[0] == '0');
    }
    if (tcres) {
        int major = 0, minor = 0;
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, cfg->device);
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, cfg->device);
        std::string why;
        if (major != 10 || minor != 3) why = "the tensor-core and dual forms need an sm_103 (GB300) device";
        else if (tc_configure() != cudaSuccess) why = "could not reserve the tensor-core kernel's shared memory";
        else if (!(h->tc = tc_plan_create(P, h->X, h->XT, h->Dhi, h->Dlo, h->Rhi, h->Rlo, round_up(4 * P.L, 64))))
            why = "TMA tensor-map encoding failed";
        else if (h->Kd && !(h->kd = tc_kdig_plan_create(P, h->Kd, h->Rd)))
            why = "TMA tensor-map encoding failed";
        if (!why.empty()) {
            cudaGetLastError();
            free_all(h);
            if (h->own_stream) cudaStreamDestroy(h->stream);
            delete h;
            return fail(nullptr, SDCA_E_UNSUPPORTED, why);
        }
    }
    *out = h;
    return SDCA_OK;
}

int sdca_set_alignment(sdca_handle *h, const uint8_t *states, const double *weights)
{
    if (!h) return SDCA_E_ARG;
    h->knn_k = 0;
    h->scan = false;
    dual_graph_reset(h);
    for (sdca_handle *s : h->sub) {
        dual_graph_reset(s);
        s->has_alignment = false;
        s->knn_k = 0;
        s->scan = false;
    }
    if (!states || !weights) return fail(h, SDCA_E_ARG, "states and weights are required");
    Problem &P = h->P;
    for (int64_t i = 0; i < P.N; ++i)
        if (!(weights[i] >= 0.0) || !std::isfinite(weights[i]))
            return fail(h, SDCA_E_ARG, "weights must be finite and non-negative");
    CK(cudaSetDevice(h->cfg.device));
    h->w_host.assign(weights, weights + P.N);
    CK(cudaMemcpy2DAsync(h->X, P.Lx, states, P.L, P.L, P.N, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->w, weights, sizeof(double) * P.N, cudaMemcpyHostToDevice, h->stream));
    std::vector<float> wf(weights, weights + P.N);   // the copy completes before the sync below
    CK(cudaMemcpyAsync(h->wf, wf.data(), sizeof(float) * P.N, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(h->flag, 0, sizeof(int), h->stream));
    {
        dim3 grid((unsigned)((P.L + 63) / 64), (unsigned)((P.Nx + 63) / 64));
        k_transpose<<<grid, 256, 0, h->stream>>>(h->X, P.Lx, (int)P.N, (int)P.L, h->XT, P.Nx, h->flag);
    }
    CKL();
    CK(cudaMemcpyAsync(h->flag_h, h->flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    { const int r_ = stream_sync(h); if (r_) return r_; }
    if (h->flag_h[0]) {
        h->has_alignment = false;
        return fail(h, SDCA_E_ARG, "state codes must be in 0..q-1");
    }
    // B_eff and lambdas: SuperDCA/include/plmDCA_optimizer_parameters.hpp:257-284
    double beff = 0.0;
    for (int64_t i = 0; i < P.N; ++i) beff += weights[i];
    const double autol = (beff > 500.0) ? 0.1 : 1.0 - ((1.0 - 0.1) * beff / 500.0);
    P.b_eff = beff;
    {
        double wmax = 0.0;
        for (int64_t i = 0; i < P.N; ++i) wmax = std::max(wmax, weights[i]);
        h->r_scale = (float)pow2_scale(wmax);
    }
    P.lambda_J = (h->cfg.lambda_J < 0.0) ? autol * beff / 2.0 : h->cfg.lambda_J * beff;
    P.lambda_h = (h->cfg.lambda_h < 0.0) ? autol * beff : h->cfg.lambda_h * beff;
    if (h->form == SDCA_FORM_DUAL) {
        // K_ij = loci where sequences i and j agree; rho is rounded to QB
        // fractional bits of w_max so that |sum_j K_ij rho_q| < 2^62
        const int64_t W = (P.L + 31) / 32;
        uint64_t *packed = nullptr;
        int32_t *dist = nullptr;
        if (cudaMalloc(&packed, sizeof(uint64_t) * P.N * W) != cudaSuccess ||
            cudaMalloc(&dist, sizeof(int32_t) * P.N * P.N) != cudaSuccess) {
            cudaGetLastError();
            if (packed) cudaFree(packed);
            h->has_alignment = false;
            return fail(h, SDCA_E_NOMEM, "device allocation for the agreement matrix failed");
        }
        launch_distances(h->X, P.Lx, (int)P.N, (int)P.L, packed, dist, h->stream);
        launch_dual_kmat(dist, (int)P.N, P.Nx, (int)P.L, h->Kmat, h->stream);
        if (h->kd) tc_kdig_fill_k(h->kd, P, h->Kmat, h->Kd, h->stream);
        const cudaError_t e1 = cudaGetLastError();
        const cudaError_t e2 = cudaStreamSynchronize(h->stream);
        cudaFree(packed);
        cudaFree(dist);
        if (e1 != cudaSuccess || e2 != cudaSuccess) {
            h->has_alignment = false;
            return fail(h, SDCA_E_CUDA, std::string("agreement matrix: ") + cudaGetErrorString(e1 ? e1 : e2));
        }
        double wmax = 0.0;
        for (int64_t i = 0; i < P.N; ++i) wmax = std::max(wmax, weights[i]);
        // the tensor-core product's four base-128 digit planes hold |rho_q| <= 2^27
        const int qb = std::min(h->kd ? 27 : 30, 62 - (int)std::ceil(std::log2((double)P.N * (double)P.L + 1.0)));
        h->qscale = wmax > 0.0 ? std::ldexp(1.0, qb) / wmax : 1.0;
    }
    h->has_alignment = true;
    h->prof.h2d_bytes = (int64_t)P.N * P.L + (int64_t)sizeof(double) * P.N;
    // the other lanes read the same buffers: they take the scalars
    for (sdca_handle *s : h->sub) {
        s->w_host = h->w_host;
        s->P.b_eff = P.b_eff;
        s->P.lambda_J = P.lambda_J;
        s->P.lambda_h = P.lambda_h;
        s->r_scale = h->r_scale;
        s->qscale = h->qscale;
        s->has_alignment = true;
    }
    return SDCA_OK;
}

int sdca_get_lambdas(const sdca_handle *h, double *lambda_h, double *lambda_J, double *b_eff)
{
    if (!h || !h->has_alignment) return SDCA_E_STATE;
    if (lambda_h) *lambda_h = h->P.lambda_h;
    if (lambda_J) *lambda_J = h->P.lambda_J;
    if (b_eff) *b_eff = h->P.b_eff;
    return SDCA_OK;
}

int sdca_solve_sel(sdca_handle *h, const uint32_t *loci, size_t n_loci, const double *x_init,
                   const int64_t *x_rows, double *x_out, float *scores, sdca_locus_stat *stats)
{
    return solve_queue(h, loci, n_loci, x_init, x_rows, x_out, scores, stats, nullptr);
}

int sdca_ws_dual_data(sdca_handle *h, const uint32_t *loci, size_t n_loci, float *feats, float *rho,
                      sdca_locus_stat *stats)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (h->form != SDCA_FORM_DUAL) return fail(h, SDCA_E_UNSUPPORTED, "training data of the dual form's start");
    if (n_loci > 0 && (!loci || !feats || !rho)) return fail(h, SDCA_E_ARG, "null loci, feats or rho");
    const Problem &P = h->P;
    const int64_t nt = h->scan ? h->LT : P.L;
    for (size_t k = 0; k < n_loci; ++k)
        if ((int64_t)loci[k] >= nt) return fail(h, SDCA_E_ARG, "locus index out of range");
    CK(cudaSetDevice(h->cfg.device));
    if ((rc = ws_knn(h, DWS_K))) return rc;
    // statistics: the target columns of the listed loci, in chunks
    const int cap = 32;
    float *fe = nullptr;
    int32_t *idx = nullptr;
    if (cudaMalloc(&fe, sizeof(float) * cap * P.Nx * MLP_IN) != cudaSuccess ||
        cudaMalloc(&idx, sizeof(int32_t) * cap) != cudaSuccess) {
        cudaGetLastError();
        if (fe) cudaFree(fe);
        return fail(h, SDCA_E_NOMEM, "device allocation for the statistics failed");
    }
    std::vector<float> buf((size_t)cap * P.Nx * MLP_IN);
    int err = SDCA_OK;
    for (size_t c0 = 0; c0 < n_loci && err == SDCA_OK; c0 += cap) {
        const int n = (int)std::min<size_t>(cap, n_loci - c0);
        std::vector<int32_t> li(loci + c0, loci + c0 + n);
        if (cudaMemcpyAsync(idx, li.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) {
            err = fail(h, SDCA_E_CUDA, "statistics upload failed");
            break;
        }
        launch_dual_ws_feats(h->scan ? h->TT : h->XT, idx, n, (int)P.N, P.Nx, (int)P.L, h->w, h->knn, h->knn_d, fe,
                             h->stream);
        if (cudaMemcpyAsync(buf.data(), fe, sizeof(float) * n * P.Nx * MLP_IN, cudaMemcpyDeviceToHost, h->stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(h->stream) != cudaSuccess) {
            err = fail(h, SDCA_E_CUDA, "statistics kernel failed");
            break;
        }
        for (int g = 0; g < n; ++g)
            std::memcpy(feats + ((c0 + g) * (size_t)P.N) * MLP_IN, buf.data() + (size_t)g * P.Nx * MLP_IN,
                        sizeof(float) * P.N * MLP_IN);
    }
    cudaFree(fe);
    cudaFree(idx);
    if (err) return err;
    return solve_queue(h, loci, n_loci, nullptr, nullptr, nullptr, nullptr, stats, rho);
}

int sdca_solve_ex(sdca_handle *h, const uint32_t *loci, size_t n_loci, const double *x_init,
                  double *x_out, float *scores, sdca_locus_stat *stats)
{
    return sdca_solve_sel(h, loci, n_loci, x_init, nullptr, x_out, scores, stats);
}

int sdca_solve(sdca_handle *h, const uint32_t *loci, size_t n_loci, float *scores,
               sdca_locus_stat *stats)
{
    return sdca_solve_ex(h, loci, n_loci, nullptr, nullptr, scores, stats);
}

int sdca_eval(sdca_handle *h, uint32_t r, const double *x, double *f, double *g)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (!x || !f) return fail(h, SDCA_E_ARG, "null argument");
    const Problem &P = h->P;
    if ((int64_t)r >= (h->scan ? h->LT : P.L)) return fail(h, SDCA_E_ARG, "locus index out of range");
    CK(cudaSetDevice(h->cfg.device));
    prof_reset(h);
    std::vector<float> xe(P.Dp);
    ref_to_engine(P, h->scan ? -1 : (int64_t)r, x, xe.data());
    const int b = 0;
    rc = slot_begin(h, b, 0, (int32_t)r, xe.data());
    if (rc) return rc;
    std::vector<int32_t> one{b};
    rc = run_forward(h, one, h->wa, true);
    if (rc) return rc;
    SlotHost &S = h->slots[b];
    rc = upload_slots(h, one);
    if (rc) return rc;
    rc = zero_acc(h);
    if (rc) return rc;
    launch_trial(P, h->sd, h->list, 1, h->lbase, h->u, h->rstate, h->w, h->R, h->acc, h->stream);
    CKL();
    rc = fetch_acc(h);
    if (rc) return rc;
    const double fdata = acc_get(h, b, ACC_F);
    for (int a = 0; a < Q; ++a) S.rs[a] = acc_get(h, b, ACC_RS0 + a);
    S.push = false;
    S.ring_new = -1;
    rc = upload_slots(h, one);
    if (rc) return rc;
    rc = zero_acc(h);
    if (rc) return rc;
    launch_bwd_gather(P, h->XT, h->sd, h->list, 1, h->R, h->wa, h->gpool, h->Ypool, h->Spool,
                      h->hist_bf16, h->acc, h->stream);
    launch_hpart(P, h->sd, h->list, 1, h->wa, h->gpool, h->Ypool, h->Spool, h->hist_bf16, h->acc,
                 h->stream);
    CKL();
    rc = fetch_acc(h);
    if (rc) return rc;
    *f = fdata + P.lambda_J * acc_get(h, b, ACC_X2J) + P.lambda_h * acc_get(h, b, ACC_X2H);
    if (g) {
        std::vector<float> ge(P.Dp);
        CK(cudaMemcpyAsync(ge.data(), h->gpool + (int64_t)(2 * b + 1 - S.gcur) * P.Dp,
                           sizeof(float) * P.Dp, cudaMemcpyDeviceToHost, h->stream));
        { const int r_ = stream_sync(h); if (r_) return r_; }
        engine_to_ref(P, ge.data(), g);
    }
    S.phase = PH_EMPTY;
    return SDCA_OK;
}

int sdca_compute_weights(sdca_handle *h, const uint8_t *states, const double *mult,
                         double threshold, double *weights_out)
{
    if (!h) return SDCA_E_ARG;
    if (!states || !weights_out) return fail(h, SDCA_E_ARG, "states and weights_out are required");
    const Problem &P = h->P;
    if (mult)
        for (int64_t i = 0; i < P.N; ++i)
            if (!(mult[i] >= 0.0) || !std::isfinite(mult[i]))
                return fail(h, SDCA_E_ARG, "multiplicities must be finite and non-negative");
    CK(cudaSetDevice(h->cfg.device));
    // the states go through the alignment buffer: a following
    // sdca_set_alignment overwrites it anyway
    h->has_alignment = false;
    h->knn_k = 0;
    for (sdca_handle *s : h->sub) {
        s->has_alignment = false;
        s->knn_k = 0;
    }
    const int64_t W = (P.L + 31) / 32;
    uint64_t *packed = nullptr;
    double *d = nullptr;
    unsigned long long *nonid = nullptr;
    auto release = [&]() {
        if (packed) cudaFree(packed);
        if (d) cudaFree(d);
    };
    if (cudaMalloc(&packed, sizeof(uint64_t) * P.N * W) != cudaSuccess ||
        cudaMalloc(&d, sizeof(double) * (2 * P.N + 1)) != cudaSuccess) {
        cudaGetLastError();
        release();
        return fail(h, SDCA_E_NOMEM, "device allocation for reweighting failed");
    }
    double *nbr = d, *dmult = d + P.N;
    nonid = reinterpret_cast<unsigned long long *>(d + 2 * P.N);
    int rc = SDCA_OK;
    do {
        if (cudaMemcpy2DAsync(h->X, P.Lx, states, P.L, P.L, P.N, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
            cudaMemsetAsync(d, 0, sizeof(double) * (2 * P.N + 1), h->stream) != cudaSuccess ||
            (mult && cudaMemcpyAsync(dmult, mult, sizeof(double) * P.N, cudaMemcpyHostToDevice, h->stream) !=
                         cudaSuccess)) {
            rc = fail(h, SDCA_E_CUDA, "reweighting upload failed");
            break;
        }
        launch_weights(h->X, P.Lx, (int)P.N, (int)P.L, packed, threshold, mult ? dmult : nullptr, nbr, nonid,
                       h->stream);
        if (cudaGetLastError() != cudaSuccess) {
            rc = fail(h, SDCA_E_CUDA, "reweighting kernel launch failed");
            break;
        }
        std::vector<double> hn(P.N);
        if (cudaMemcpyAsync(hn.data(), nbr, sizeof(double) * P.N, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
            cudaStreamSynchronize(h->stream) != cudaSuccess) {
            rc = fail(h, SDCA_E_CUDA, "reweighting failed");
            break;
        }
        // w_i = mult_i / (mult_i + sum of neighbour multiplicities)
        for (int64_t i = 0; i < P.N; ++i) {
            const double mi = mult ? mult[i] : 1.0;
            weights_out[i] = mi / (mi + hn[i]);
        }
    } while (0);
    release();
    return rc;
}

int sdca_set_targets(sdca_handle *h, const uint8_t *targets, int64_t n_target_loci)
{
    if (!h) return SDCA_E_ARG;
    if (!h->has_alignment) return fail(h, SDCA_E_STATE, "sdca_set_alignment must come first");
    dual_graph_reset(h);
    for (sdca_handle *s : h->sub) dual_graph_reset(s);
    if (h->TT) {
        cudaFree(h->TT);
        h->TT = nullptr;
    }
    h->scan = false;
    h->LT = 0;
    if (!targets) {
        for (sdca_handle *s : h->sub) sdca_set_targets(s, nullptr, 0);
        return SDCA_OK;
    }
    const Problem &P = h->P;
    if (n_target_loci < 1 || n_target_loci > (1LL << 26)) return fail(h, SDCA_E_ARG, "invalid number of target loci");
    for (int64_t e = 0; e < P.N * n_target_loci; ++e)
        if (targets[e] >= Q) return fail(h, SDCA_E_ARG, "state codes must be in 0..q-1");
    CK(cudaSetDevice(h->cfg.device));
    const int64_t LTx = round_up(n_target_loci, 64);
    uint8_t *tmp = nullptr;
    if (cudaMalloc(&tmp, (size_t)P.N * LTx) != cudaSuccess ||
        cudaMalloc(&h->TT, (size_t)n_target_loci * P.Nx) != cudaSuccess) {
        cudaGetLastError();
        if (tmp) cudaFree(tmp);
        h->TT = nullptr;
        return fail(h, SDCA_E_NOMEM, "device allocation for the target columns failed");
    }
    int rc = SDCA_OK;
    do {
        if (cudaMemsetAsync(h->TT, 0, (size_t)n_target_loci * P.Nx, h->stream) != cudaSuccess ||
            cudaMemcpy2DAsync(tmp, LTx, targets, n_target_loci, n_target_loci, P.N, cudaMemcpyHostToDevice,
                              h->stream) != cudaSuccess ||
            cudaMemsetAsync(h->flag, 0, sizeof(int), h->stream) != cudaSuccess) {
            rc = fail(h, SDCA_E_CUDA, "target upload failed");
            break;
        }
        dim3 grid((unsigned)((n_target_loci + 63) / 64), (unsigned)((P.Nx + 63) / 64));
        k_transpose<<<grid, 256, 0, h->stream>>>(tmp, LTx, (int)P.N, (int)n_target_loci, h->TT, P.Nx, h->flag);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(h->stream) != cudaSuccess)
            rc = fail(h, SDCA_E_CUDA, "target transpose failed");
    } while (0);
    cudaFree(tmp);
    if (rc) {
        cudaFree(h->TT);
        h->TT = nullptr;
        return rc;
    }
    h->LT = n_target_loci;
    h->scan = true;
    for (sdca_handle *s : h->sub)
        if ((rc = sdca_set_targets(s, targets, n_target_loci))) return fail(h, rc, s->err);
    return SDCA_OK;
}

int sdca_set_warm_start(sdca_handle *h, const float *params, size_t n_params)
{
    if (!h) return SDCA_E_ARG;
    dual_graph_reset(h);   // the dual form's graph holds the learned start's kernels or not
    for (sdca_handle *s : h->sub) dual_graph_reset(s);
    if (!params) {
        h->ws_on = false;
        h->ws_dual = false;
        for (sdca_handle *s : h->sub) s->ws_on = s->ws_dual = false;
        return SDCA_OK;
    }
    if (n_params != (size_t)MLP_BLOB_SIZE)
        return fail(h, SDCA_E_ARG, "warm-start parameters: expected " + std::to_string(MLP_BLOB_SIZE) + " floats");
    for (size_t i = 0; i < n_params; ++i)
        if (!std::isfinite(params[i])) return fail(h, SDCA_E_ARG, "warm-start parameters must be finite");
    int rc;
    if (h->form == SDCA_FORM_DUAL) {
        // per-sequence blob (version 2): the start a0 = -alpha rho^ / (2 lambda_J)
        if (params[MLP_VERSION] != (float)MLP_BLOB_VERSION_DUAL)
            return fail(h, SDCA_E_ARG, "the dual form takes a per-sequence warm-start blob (version 2)");
        if (params[MLP_KNN] != (float)DWS_K) return fail(h, SDCA_E_ARG, "warm-start parameters: neighbours must be 16");
        const float alpha = params[MLP_ALPHA];
        if (!(alpha > 0.f && alpha <= 1.f))
            return fail(h, SDCA_E_ARG, "warm-start parameters: shrinkage must be in (0, 1]");
        CK(cudaSetDevice(h->cfg.device));
        if ((rc = ws_network(h, params))) return rc;
        if (!h->dws_feats) {
            const int cap = 32;
            const size_t rows = (size_t)cap * h->P.Nx;
            if ((rc = dalloc(h, &h->dws_feats, rows * MLP_IN)) || (rc = dalloc(h, &h->dws_out, rows * MLP_OUT)))
                return rc;
            h->dws_cap = cap;
        }
        h->ws_alpha = alpha;
        h->ws_dual = true;
        for (sdca_handle *s : h->sub)
            if ((rc = sdca_set_warm_start(s, params, n_params))) return fail(h, rc, s->err);
        return SDCA_OK;
    }
    if (params[MLP_VERSION] != (float)MLP_BLOB_VERSION)
        return fail(h, SDCA_E_ARG, "warm-start parameters: this form takes a per-pair blob (version 1)");
    const float kf = params[MLP_KNN], eps = params[MLP_EPS];
    if (!(kf >= 1.f && kf <= (float)WS_MAX_K && kf == std::floor(kf)) || !(eps >= 0.f))
        return fail(h, SDCA_E_ARG, "warm-start parameters: neighbours must be 1..16 and eps >= 0");
    CK(cudaSetDevice(h->cfg.device));
    if ((rc = ws_network(h, params))) return rc;
    h->ws_k = (int)kf;
    h->ws_eps = eps;
    h->ws_hfit = params[MLP_HFIT] != 0.f;
    h->ws_on = true;
    for (sdca_handle *s : h->sub)
        if ((rc = sdca_set_warm_start(s, params, n_params))) return fail(h, rc, s->err);
    return SDCA_OK;
}

int sdca_ws_features(sdca_handle *h, int k, float eps, const uint32_t *loci, size_t n_loci, const uint32_t *sel,
                     size_t n_sel, float *out)
{
    if (!h) return SDCA_E_ARG;
    if (!h->has_alignment) return fail(h, SDCA_E_STATE, "sdca_set_alignment must come first");
    if (!loci || !out) return fail(h, SDCA_E_ARG, "loci and out are required");
    if (k < 1 || k > WS_MAX_K || !(eps >= 0.f)) return fail(h, SDCA_E_ARG, "k must be 1..16 and eps >= 0");
    const Problem &P = h->P;
    for (size_t i = 0; i < n_loci; ++i)
        if (loci[i] >= (uint32_t)P.L) return fail(h, SDCA_E_ARG, "locus index out of range");
    if (sel)
        for (size_t i = 0; i < n_loci * n_sel; ++i)
            if (sel[i] >= (uint32_t)P.L) return fail(h, SDCA_E_ARG, "pair index out of range");
    CK(cudaSetDevice(h->cfg.device));
    std::vector<float> buf;
    for (size_t g0 = 0; g0 < n_loci; g0 += WS_G) {
        const int G = (int)std::min<size_t>(WS_G, n_loci - g0);
        std::vector<int32_t> grp(G);
        for (int g = 0; g < G; ++g) grp[g] = (int32_t)loci[g0 + g];
        int rc = ws_features(h, grp, k, eps);
        if (rc) return rc;
        const size_t per = (size_t)P.L * MLP_IN;
        if (!sel) {
            CK(cudaMemcpyAsync(out + g0 * per, h->ws_feats, sizeof(float) * per * G, cudaMemcpyDeviceToHost,
                               h->stream));
            if ((rc = stream_sync(h))) return rc;
            continue;
        }
        buf.resize(per * G);
        CK(cudaMemcpyAsync(buf.data(), h->ws_feats, sizeof(float) * per * G, cudaMemcpyDeviceToHost, h->stream));
        if ((rc = stream_sync(h))) return rc;
        for (int g = 0; g < G; ++g)
            for (size_t j = 0; j < n_sel; ++j)
                std::memcpy(out + ((g0 + g) * n_sel + j) * MLP_IN,
                            buf.data() + ((size_t)g * P.L + sel[(g0 + g) * n_sel + j]) * MLP_IN,
                            sizeof(float) * MLP_IN);
    }
    return SDCA_OK;
}

int sdca_get_profile(const sdca_handle *h, sdca_profile *out)
{
    if (!h || !out) return SDCA_E_ARG;
    *out = h->prof;
    return SDCA_OK;
}

const char *sdca_last_error(const sdca_handle *h)
{
    if (!h) {
        std::lock_guard<std::mutex> lk(g_err_mu);
        return g_create_err.c_str();
    }
    return h->err.c_str();
}

int sdca_destroy(sdca_handle *h)
{
    if (!h) return SDCA_OK;
    for (sdca_handle *s : h->sub) sdca_destroy(s);   // before the buffers they share
    h->sub.clear();
    cudaSetDevice(h->cfg.device);
    if (h->ev_lanes) cudaEventDestroy(h->ev_lanes);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->ev_round) cudaEventDestroy(h->ev_round);
    dual_graph_free(h);
    for (auto e : h->ev_pool) cudaEventDestroy(e);
    if (h->tc) tc_plan_destroy(h->tc);
    if (h->kd) tc_kdig_plan_destroy(h->kd);
    if (h->TT) cudaFree(h->TT);
    free_all(h);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return SDCA_OK;
}

// Test hook (not part of the public header): the compact-form coefficients.
int sdca_internal_lbfgs_coeffs(int k, const double *R, const double *YY, const double *sg,
                               const double *yg, double gamma, double *coef_g, double *coefS,
                               double *coefY)
{
    return lbfgs_compact_coeffs(k, R, YY, sg, yg, gamma, coef_g, coefS, coefY) ? 0 : -1;
}

} // extern "C"
