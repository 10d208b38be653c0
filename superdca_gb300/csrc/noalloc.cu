// noalloc.cu -- one objective evaluation that allocates no memory.
//
// sdca_eval needs a handle, and a handle allocates device memory for the
// alignment and the solver state.  Some callers cannot let a library
// allocate: host programs that own all device memory through their own
// allocator (a framework's caching allocator, or an embedded runtime with a
// fixed memory budget) and forbid libraries from calling cudaMalloc or
// cudaFree behind their back.  sdca_eval_noalloc serves them: the caller
// passes device pointers for every input and output, and the intermediate
// values (per-sequence node beliefs, per-block partial sums and an error
// word) live in one file-scope __device__ array of fixed size, SCRATCH_BYTES
// below, which every GPU that loads this library holds until the process
// exits.
//
// The array is shared by every call: two calls whose kernels overlap on the
// GPU (different streams, or different host threads) race on it.  Each call
// writes every scratch element it reads before reading it, and the error
// word is returned to zero by the last kernel of every call, so nothing needs
// clearing between calls.
//
// The array's device address is looked up with cudaGetSymbolAddress once per
// CUDA context (the first call made while that context is current), and
// cached under the context's unique id; a context created anew (for example
// after cudaDeviceReset) has a new id, so its first call looks the address up
// again.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/superdca_gb300.h"

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_MAX_BLOCKS = (int)((SDCA_NOALLOC_MAX_LOCI + NA_THREADS - 1) / NA_THREADS);  // partial-sum slots
constexpr int64_t NA_MAX_SEQS = SDCA_NOALLOC_MAX_SEQS;
// node beliefs (N x 4 doubles) + per-block partials (5 doubles per block,
// two passes) + one error word (8 bytes)
constexpr size_t NA_ERR_OFFSET = (size_t)NA_MAX_SEQS * 4 + (size_t)2 * NA_MAX_BLOCKS * 8;   // in doubles
constexpr size_t SCRATCH_BYTES = (NA_ERR_OFFSET + 1) * sizeof(double);

__device__ __align__(256) unsigned char g_na_scratch[SCRATCH_BYTES];

// scratch address per CUDA context, keyed by the context's unique id
std::mutex g_na_mu;
std::vector<std::pair<unsigned long long, double *>> g_na_ptr;

// The current context's unique id (cuCtxGetCurrent + cuCtxGetId, reached
// through the runtime's driver entry points, so no link to libcuda).
bool current_context_id(unsigned long long *id)
{
    using get_current_fn = int (*)(void **);
    using get_id_fn = int (*)(void *, unsigned long long *);
    static get_current_fn get_current = nullptr;
    static get_id_fn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<get_current_fn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<get_id_fn>(p);
        cudaGetLastError();
    });
    if (!get_current || !get_id) return false;
    void *ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return false;
    return get_id(ctx, id) == 0;
}

// Position of J_r[n][s][a] in SuperDCA's parameter layout: 16-locus blocks,
// STATES order inside a block (SuperDCA/include/Matrix_kernel_access_order.hpp:
// 28-34, Coupling_matrix_view.hpp:156-168).
__device__ __forceinline__ int64_t na_index(int64_t L, int64_t n, int s, int a)
{
    const int64_t b = n / 16, p = n % 16, nfull = L / 16;
    const int64_t e = b < nfull ? 16 : L % 16;
    return b * 256 + ((int64_t)s * e + p) * 4 + a;
}

__device__ __forceinline__ double na_warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block sum of K values; thread 0 gets the totals
template <int K>
__device__ __forceinline__ void na_block_sum(double (&v)[K])
{
    __shared__ double red[NA_THREADS / 32][K];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < K; ++k) v[k] = na_warp_sum(v[k]);
    if (lane == 0)
        for (int k = 0; k < K; ++k) red[w][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < K; ++k) {
            double t = 0.0;
            for (int j = 0; j < NA_THREADS / 32; ++j) t += red[j][k];
            v[k] = t;
        }
}

// pass 1, one thread per sequence: logits, objective term, node beliefs
// (SuperDCA/include/plmDCA_objective.hpp:86-151)
__global__ void k_na_beliefs(const uint8_t *__restrict__ states, int64_t N, int64_t L, int64_t r,
                             const double *__restrict__ w, const double *__restrict__ x,
                             double *__restrict__ scratch)
{
    double *nb = scratch;                         // N x 4
    double *part = scratch + NA_MAX_SEQS * 4;     // blocks x 8
    const int64_t i = (int64_t)blockIdx.x * NA_THREADS + threadIdx.x;
    double v[5] = {0, 0, 0, 0, 0};
    if (i < N) {
        const double *h = x + 16 * L;
        double l[4] = {h[0], h[1], h[2], h[3]};
        const uint8_t *si = states + i * L;
        int bad = 0;
        for (int64_t n = 0; n < L; ++n) {
            bad |= si[n] >> 2;   // a code >= 4 (the & 3 below only keeps the loads in bounds)
            if (n == r) continue;
            const int s = si[n] & 3;
            for (int a = 0; a < 4; ++a) l[a] += x[na_index(L, n, s, a)];
        }
        if (bad) atomicOr(reinterpret_cast<unsigned long long *>(scratch + NA_ERR_OFFSET), 1ull);
        const double mx = fmax(fmax(l[0], l[1]), fmax(l[2], l[3]));
        double e[4], z = 0.0;
        for (int a = 0; a < 4; ++a) {
            e[a] = exp(l[a] - mx);
            z += e[a];
        }
        const int sr = si[r] & 3;
        const double wi = w[i];
        v[0] = wi * ((mx + log(z)) - l[sr]);
        for (int a = 0; a < 4; ++a) {
            const double b = wi * (e[a] / z) - (a == sr ? wi : 0.0);
            nb[i * 4 + a] = b;
            v[1 + a] = b;
        }
    }
    na_block_sum<5>(v);
    if (threadIdx.x == 0)
        for (int k = 0; k < 5; ++k) part[blockIdx.x * 8 + k] = v[k];
}

// pass 2, one thread per locus: gradient of J_r and the L2 part of the
// objective (plmDCA_objective.hpp:153-190, 192-244)
__global__ void k_na_gradient(const uint8_t *__restrict__ states, int64_t N, int64_t L, int64_t r,
                              double lambda_J, const double *__restrict__ x, double *__restrict__ g,
                              double *__restrict__ scratch)
{
    const double *nb = scratch;
    double *part = scratch + NA_MAX_SEQS * 4 + (size_t)NA_MAX_BLOCKS * 8;
    const int64_t n = (int64_t)blockIdx.x * NA_THREADS + threadIdx.x;
    double v[1] = {0.0};
    if (n < L) {
        double c[16];
        for (int k = 0; k < 16; ++k) c[k] = 0.0;
        if (n != r)
            for (int64_t i = 0; i < N; ++i) {
                const int s = states[i * L + n] & 3;
                for (int a = 0; a < 4; ++a) c[s * 4 + a] += nb[i * 4 + a];
            }
        for (int s = 0; s < 4; ++s)
            for (int a = 0; a < 4; ++a) {
                const int64_t o = na_index(L, n, s, a);
                if (n == r) {
                    g[o] = 0.0;
                } else {
                    g[o] = c[s * 4 + a] + 2.0 * lambda_J * x[o];
                    v[0] += lambda_J * x[o] * x[o];
                }
            }
    }
    na_block_sum<1>(v);
    if (threadIdx.x == 0) part[blockIdx.x * 8] = v[0];
}

// pass 3, one block: totals, h gradient and the h part of the objective.
// A state code >= 4 seen by pass 1 makes f and the h gradient NaN; the
// error word is returned to zero for the next call.
__global__ void k_na_total(int64_t L, int nb1, int nb2, double lambda_h, const double *__restrict__ x,
                           double *__restrict__ f, double *__restrict__ g, double *__restrict__ scratch)
{
    const double *p1 = scratch + NA_MAX_SEQS * 4;
    const double *p2 = p1 + (size_t)NA_MAX_BLOCKS * 8;
    double v[6] = {0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < nb1; b += NA_THREADS)
        for (int k = 0; k < 5; ++k) v[k] += p1[b * 8 + k];
    for (int b = threadIdx.x; b < nb2; b += NA_THREADS) v[5] += p2[b * 8];
    na_block_sum<6>(v);
    if (threadIdx.x == 0) {
        unsigned long long *err = reinterpret_cast<unsigned long long *>(scratch + NA_ERR_OFFSET);
        const bool bad = *err != 0ull;
        *err = 0ull;
        const double *h = x + 16 * L;
        double fv = v[0] + v[5];
        for (int a = 0; a < 4; ++a) {
            fv += lambda_h * h[a] * h[a];
            g[16 * L + a] = bad ? nan("") : v[1 + a] + 2.0 * lambda_h * h[a];
        }
        *f = bad ? nan("") : fv;
    }
}

} // namespace

extern "C" int sdca_eval_noalloc(const uint8_t *states, int64_t n_seqs, int64_t n_loci,
                                 const double *weights, double lambda_h, double lambda_J, uint32_t r,
                                 const double *x, double *f, double *g, void *stream)
{
    // every rejection happens before any work is queued
    if (!states || !weights || !x || !f || !g) return SDCA_E_ARG;
    if (n_seqs < 1 || n_loci < 2 || (int64_t)r >= n_loci) return SDCA_E_ARG;
    if (n_seqs > NA_MAX_SEQS || n_loci > SDCA_NOALLOC_MAX_LOCI) return SDCA_E_ARG;
    // an error left pending by the caller's earlier work is theirs: report
    // it without consuming it, and queue nothing
    if (cudaPeekAtLastError() != cudaSuccess) return SDCA_E_CUDA;
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_na_mu);
        unsigned long long id = 0;
        bool have_id = current_context_id(&id);
        if (have_id)
            for (const auto &e : g_na_ptr)
                if (e.first == id) scratch = e.second;
        if (!scratch) {
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);   // makes the context current
            if (e != cudaSuccess) {
                cudaGetLastError();
                return SDCA_E_CUDA;
            }
            scratch = static_cast<double *>(p);
            if (!have_id) have_id = current_context_id(&id);
            if (have_id && g_na_ptr.size() < 256) g_na_ptr.emplace_back(id, scratch);
        }
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nb1 = (int)((n_seqs + NA_THREADS - 1) / NA_THREADS);
    const int nb2 = (int)((n_loci + NA_THREADS - 1) / NA_THREADS);
    k_na_beliefs<<<nb1, NA_THREADS, 0, st>>>(states, n_seqs, n_loci, r, weights, x, scratch);
    k_na_gradient<<<nb2, NA_THREADS, 0, st>>>(states, n_seqs, n_loci, r, lambda_J, x, g, scratch);
    k_na_total<<<1, NA_THREADS, 0, st>>>(n_loci, nb1, nb2, lambda_h, x, f, g, scratch);
    return cudaGetLastError() == cudaSuccess ? SDCA_OK : SDCA_E_CUDA;
}
