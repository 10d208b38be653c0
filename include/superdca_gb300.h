/* superdca_gb300.h -- C ABI of the GB300 plmDCA per-locus solve engine.
 *
 * One handle owns one GPU stream and all device memory of one alignment.  The
 * caller owns every host buffer.  Every function returns 0 on success and a
 * negative SDCA_E* code otherwise; sdca_last_error() gives the message.  A
 * handle is not thread-safe; separate handles are independent.
 *
 * The entry points replace SuperDCA's only solve boundary, the template call
 *   run_plmDCA<double, triallelic_state_t>(alignments, loci_list)
 * (SuperDCA/include/plmDCA.hpp:436-437, called from SuperDCA/src/SuperDCA.cpp:408),
 * together with the option getters it reads (SuperDCA/include/plmDCA_options.h).
 * File output, FASTA parsing and filtering stay with the caller.
 *
 * Parameter vectors crossing this ABI (x, g) use SuperDCA's own layout,
 * D = q*q*L + q doubles: J_r in 16-locus blocks, STATES order inside a block
 * (SuperDCA/include/Matrix_kernel_access_order.hpp:28-34,
 *  SuperDCA/include/Coupling_matrix_view.hpp:156-168), then h_r
 * (SuperDCA/include/plmDCA_optimizer_parameters.hpp:219-247).
 */
#ifndef SUPERDCA_GB300_H
#define SUPERDCA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDCA_ABI_VERSION 2

/* status codes */
#define SDCA_OK 0
#define SDCA_E_ARG (-1)       /* invalid argument */
#define SDCA_E_CUDA (-2)      /* CUDA runtime error */
#define SDCA_E_STATE (-3)     /* call out of order (e.g. no alignment yet) */
#define SDCA_E_NOMEM (-4)     /* device allocation failed */
#define SDCA_E_NUMERIC (-5)   /* non-finite objective or gradient */
#define SDCA_E_UNSUPPORTED (-6)

/* contraction forms (sdca_config.form) */
#define SDCA_FORM_GATHER 0    /* plain form: FP32 gather/scatter on CUDA cores */
#define SDCA_FORM_TC 1        /* tcgen05 one-hot GEMMs, fp16 hi+lo, FP32 accumulate */
#define SDCA_FORM_DUAL 2      /* the same L-BFGS iteration kept in the span of the sequences:
                                 N x 4 coefficients, one exact integer product with the
                                 N x N agreement matrix per iteration; starts from zero
                                 or from the per-sequence learned start (version-2 blob) */

/* sdca_config.flags */
#define SDCA_FLAG_HISTORY_BF16 0x1 /* keep L-BFGS (s, y) history in BF16 */

typedef struct sdca_handle sdca_handle;

typedef struct {
    int64_t n_seqs;            /* N: sequences */
    int64_t n_loci;            /* L: loci (columns) */
    int32_t q;                 /* states per locus: 4 (SuperDCA triallelic envelope) */
    int32_t gap_state;         /* state left out of the coupling norm (3) */
    double lambda_h;           /* --lambda-h option value; < 0 selects the automatic rule */
    double lambda_J;           /* --lambda-J option value; < 0 selects the automatic rule */
    double gradient_threshold; /* --gradient-threshold (1e-3): stop on max-norm of g */
    int32_t max_iterations;    /* L-BFGS iteration limit (2000) */
    int32_t history;           /* L-BFGS history length m (10) */
    int32_t batch;             /* loci solved concurrently (slots) */
    int32_t form;              /* SDCA_FORM_* */
    int32_t flags;             /* SDCA_FLAG_* */
    int32_t device;            /* CUDA device ordinal */
    void *stream;              /* cudaStream_t to run on, or NULL for a private stream */
    int32_t lanes;             /* solver lanes (1..16; 0 means 1): each lane holds `batch`
                                  slots with its own stream and host thread, all lanes share
                                  the resident alignment and draw loci from one queue, so one
                                  lane's host decisions overlap the others' kernels */
    int32_t reserved0;         /* 0 */
} sdca_config;

typedef struct {
    double f;                  /* objective at the returned point (FP64 reduction) */
    double gnorm;              /* max-norm of the gradient there */
    int32_t iterations;        /* L-BFGS iterations */
    int32_t nfeval;            /* objective evaluations as SuperDCA counts them */
    int32_t contractions;      /* forward + backward contraction passes run */
    int32_t status;            /* 0 gradient tolerance, 1 iteration limit,
                                  2 relative-epsilon stop, -1 non-finite */
    int32_t restarts;          /* steepest-descent restarts (non-descent direction) */
    int32_t skipped_pairs;     /* history pairs not stored (s.y <= 0) */
    int32_t weak_searches;     /* line searches that ended without the Wolfe conditions */
    int32_t max_trials;        /* most trial steps any line search took */
} sdca_locus_stat;

typedef struct {
    double solve_ms;           /* device time of the last sdca_solve* call (CUDA events) */
    double kernel_ms[8];       /* device time per kernel class (see SDCA_K_*) */
    int64_t kernel_launches[8];/* kernels launched per class */
    int64_t kernel_units[8];   /* slot-passes per class: one unit = one target locus
                                  through one launch of that class */
    int64_t gpu_launches;      /* all kernels launched by the last call */
    int64_t iterations;        /* summed over loci of the last solve */
    int64_t contractions;
    int64_t h2d_bytes;
    int64_t d2h_bytes;
} sdca_profile;

/* kernel classes in sdca_profile */
#define SDCA_K_FORWARD 0       /* u = X . d (logit direction) */
#define SDCA_K_BACKWARD 1      /* g = X^T R + 2 lambda x (gradient) */
#define SDCA_K_LINESEARCH 2    /* per-trial softmax, objective and g.d */
#define SDCA_K_HISTORY 3       /* L-BFGS history dot products */
#define SDCA_K_DIRECTION 4     /* L-BFGS direction */
#define SDCA_K_ACCEPT 5        /* iterate update and history push */
#define SDCA_K_SCORE 6         /* Ising gauge + Frobenius scoring */
#define SDCA_K_OTHER 7

/* Defaults: q=4, gap 3, lambdas automatic, threshold 1e-3, 2000 iterations,
 * m=10, batch 64, gather form.  Replaces the option defaults of
 * SuperDCA/src/plmDCA_options.cpp:30-61 and plmDCA.hpp:218-221. */
int sdca_config_default(sdca_config *cfg);

/* Create a handle on cfg->device. */
int sdca_create(const sdca_config *cfg, sdca_handle **out);

/* Upload the encoded alignment (N x L row-major state codes 0..q-1) and the
 * sequence weights (N doubles; SuperDCA computes them in calculate_weights,
 * SuperDCA/include/plmDCA_optimizer_parameters.hpp:39-98, or uses 1.0 with
 * --no-reweighting, plmDCA.hpp:541-544).  Sets B_eff and the lambdas
 * (plmDCA_optimizer_parameters.hpp:257-284). */
int sdca_set_alignment(sdca_handle *h, const uint8_t *states, const double *weights);

/* Sequence reweighting on the GPU: weights of SuperDCA's calculate_weights
 * (plmDCA_optimizer_parameters.hpp:39-98) with identity = (L - d_ij)/L, d_ij
 * the number of loci whose codes differ.  mult: per-sequence multiplicities
 * or NULL. */
int sdca_compute_weights(sdca_handle *h, const uint8_t *states, const double *mult,
                         double threshold, double *weights_out);

/* Two-alignment scan mode (SuperDCA with two alignment files:
 * plmDCA_objective.hpp:67, plmDCA.hpp:338-346, 370-377, 484-490): the
 * targets are the columns of a second alignment of the same sequences
 * (N x n_target_loci row-major codes), the features are every locus of the
 * alignment set by sdca_set_alignment, none excluded, and scores are taken
 * from the blocks as stored (untransposed).  Afterwards the loci of
 * sdca_solve* and sdca_eval index target columns.  NULL targets return to
 * the single-alignment mode; sdca_set_alignment does too. */
int sdca_set_targets(sdca_handle *h, const uint8_t *targets, int64_t n_target_loci);

/* B_eff and the absolute regularisation strengths in force. */
int sdca_get_lambdas(const sdca_handle *h, double *lambda_h, double *lambda_J,
                     double *b_eff);

/* Solve the listed target loci (the per-locus loop of plmDCA_solver,
 * SuperDCA/include/plmDCA.hpp:277-396, over tbb::parallel_reduce,
 * plmDCA.hpp:581-586).  scores: n_loci x L floats, row k holds S[loci[k]][n]
 * = ||gauge(J_rn)||_F without GAP for n != r and NaN at n == r
 * (plmDCA.hpp:366-394); may be NULL.  stats: n_loci records; may be NULL. */
int sdca_solve(sdca_handle *h, const uint32_t *loci, size_t n_loci, float *scores,
               sdca_locus_stat *stats);

/* As sdca_solve, with optional start points x_init (n_loci x D, reference
 * layout; NULL = zero start as in plmDCA.hpp:298) and optional solutions
 * x_out (n_loci x D). */
int sdca_solve_ex(sdca_handle *h, const uint32_t *loci, size_t n_loci, const double *x_init,
                  double *x_out, float *scores, sdca_locus_stat *stats);

/* As sdca_solve_ex, with solutions for chosen loci only: x_rows[k] is the
 * row of x_out (n_rows x D, reference layout) that receives the solution of
 * loci[k], or -1 for none; rows may repeat only for repeated loci.  x_rows
 * NULL means row k for every k (sdca_solve_ex).  Lets a caller check or keep
 * a few solutions of a long loci list (SuperDCA keeps each locus's solution
 * only for its scoring, plmDCA.hpp:298-394) without n_loci x D doubles of
 * host memory. */
int sdca_solve_sel(sdca_handle *h, const uint32_t *loci, size_t n_loci, const double *x_init,
                   const int64_t *x_rows, double *x_out, float *scores, sdca_locus_stat *stats);

/* One objective evaluation for target locus r at x (reference layout):
 * plmDCA_objective_fval_and_gradient (SuperDCA/include/plmDCA_objective.hpp:
 * 38-249) as reached through value_and_gradient
 * (SuperDCA/include/LBFGS_interface_CppNumericalSolvers.hpp:111-117).
 * g may be NULL. */
int sdca_eval(sdca_handle *h, uint32_t r, const double *x, double *f, double *g);

/* ---- Autotuner.  SuperDCA balances its loci with TBB, grain 1
 * (SuperDCA/include/plmDCA.hpp:581-586); the engine's counterpart is the
 * choice of sdca_config.batch (slots per lane) and sdca_config.lanes.
 * sdca_autotune solves the first loci of `loci` with candidate (batch,
 * lanes) pairs in turn -- each probe holds twice its candidate's slots --
 * and picks the pair that ran the most L-BFGS iterations per device second.
 * The probe loci are solved for real: their score rows (n_loci x L, may be
 * NULL) and statistics (may be NULL) are written, and *n_done tells how many
 * leading entries of `loci` are done (at most max_fraction of n_loci;
 * candidates whose probe does not fit in that budget are skipped).  *best
 * is *base with the chosen batch and lanes.  cache_path (may be NULL): a
 * text file that keeps one choice per (N, L, form, device, free-memory
 * class); a cached choice is returned at once with *n_done = 0.  entries
 * (may be NULL; SDCA_TUNE_MAX_ENTRIES of them) and *n_entries report every
 * candidate: status SDCA_OK (measured), SDCA_E_NOMEM (did not fit on the
 * device) or SDCA_E_ARG (no room left in the probe budget). */
#define SDCA_TUNE_MAX_ENTRIES 16

typedef struct {
    int32_t batch;             /* slots per lane */
    int32_t lanes;             /* solver lanes */
    int32_t n_loci;            /* loci its probe solved (0: not measured) */
    int32_t status;            /* SDCA_OK, or why it was not measured */
    double device_ms;          /* device time of the probe (CUDA events) */
    double iterations_per_s;   /* L-BFGS iterations of the probe per device second */
} sdca_tune_entry;

int sdca_autotune(const sdca_config *base, const uint8_t *states, const double *weights,
                  const uint32_t *loci, size_t n_loci, double max_fraction, const char *cache_path,
                  float *scores, sdca_locus_stat *stats, size_t *n_done, sdca_config *best,
                  sdca_tune_entry *entries, int32_t *n_entries);

/* Device timings and counters of the last sdca_solve* call. */
int sdca_get_profile(const sdca_handle *h, sdca_profile *out);

/* Message of the last failed call on h (or of the last failed sdca_create
 * when h is NULL). */
const char *sdca_last_error(const sdca_handle *h);

int sdca_destroy(sdca_handle *h);

int sdca_abi_version(void);

/* ---- Learned warm start.  No counterpart in the reference: SuperDCA starts
 * every locus from zero (SuperDCA/include/plmDCA.hpp:298).  A per-pair MLP
 * (40 -> 128 -> 128 -> 16, ReLU) maps the statistics of each pair (r, n) to
 * an initial block J_rn (and optionally h fitted with J fixed).  The optimum is
 * unchanged (the objective is strictly convex); only the start moves.
 * The parameter blob holds sdca_mlp_blob_size() floats:
 *   [0] version (1), [1] neighbours k (1..16), [2] smoothing eps,
 *   [3] 1: fit h by Newton's method with J fixed, 0: start from h = 0,
 *   [4, 44) input mean, [44, 84) input scale, W1 (128 x 40), b1 (128),
 *   W2 (128 x 128), b2 (128), W3 (16 x 128), b3 (16), output scale (16).
 * Pair statistics per (r, n), in this order: joint[s][a] (16), residual-
 * weighted joint[s][a] (16), f_n[s] (4), f_r[a] (4), with s the state at n
 * and a the state at r, all divided by B_eff; the residuals come from each
 * sequence's k nearest neighbours in Hamming distance.  The start block is
 * output[s][a] * scale[s*4+a] * B_eff / (2 lambda_J). */

/* Enable the warm start with this blob for later sdca_solve* calls whose
 * x_init is NULL; params = NULL disables it.  The tensor-core and plain
 * forms take the per-pair blob above (version 1).  The dual form takes a
 * per-sequence blob (version 2, the same network and layout; [1] = 16
 * neighbours, [2] = shrinkage alpha in (0, 1], [3] = 0): from statistics of
 * each sequence at the target column -- onehot(s_i(r)), the column's weighted
 * state frequencies, the state frequencies among its 1, 3, 8 and 16 nearest
 * neighbours in Hamming distance and those neighbours' distances over L
 * (inputs 0..27; 28..39 are 0) -- the network predicts the sequence's
 * converged residual p_i - onehot(s_i(r)) (outputs 0..3 times the output
 * scale), centred over the states and scaled into [-1, 1] where larger.
 * The start is x0 = (Phi^T a0, 0) with a0 = -alpha w_i (predicted residual)
 * / (2 lambda_J), the form an optimum has in the span of the sequences, and
 * K a0 is formed exactly, so the iteration stays exact.  The network runs on
 * the tensor cores with BF16 weights (an image of the blob's FP32 weights). */
int sdca_set_warm_start(sdca_handle *h, const float *params, size_t n_params);

/* Training data for the dual form's per-sequence start: for each listed
 * locus, the statistics above for every sequence (feats: n_loci x N x 40
 * floats) and, from a solve of the loci (stats as sdca_solve), the
 * converged residual rows w_i (p_i - onehot(s_i(r))) (rho: n_loci x N x 4
 * floats).  Dual form only. */
int sdca_ws_dual_data(sdca_handle *h, const uint32_t *loci, size_t n_loci, float *feats, float *rho,
                      sdca_locus_stat *stats);

/* Pair statistics of target loci (for training): out holds n_loci x n_sel x
 * 40 floats for pairs (loci[k], sel[k*n_sel + j]), or n_loci x L x 40 when
 * sel is NULL. */
int sdca_ws_features(sdca_handle *h, int k, float eps, const uint32_t *loci, size_t n_loci,
                     const uint32_t *sel, size_t n_sel, float *out);

/* The network on the GPU (current device), host buffers: X is M x 40 raw
 * pair statistics, T is M x 16 targets in output units (before the output
 * scale).  Loss = mean over rows of the squared error summed over the 16
 * outputs.  sdca_mlp_grad: loss and its gradient (blob layout, zero outside
 * W1..b3).  sdca_mlp_train: Adam over shuffled minibatches, params updated in
 * place, mean minibatch loss per epoch into losses (may be NULL). */
int sdca_mlp_blob_size(void);
int sdca_mlp_grad(const float *params, const float *X, const float *T, int64_t M, double *loss, float *grad);
int sdca_mlp_predict(const float *params, const float *X, int64_t M, float *out);
int sdca_mlp_train(float *params, const float *X, const float *T, int64_t M, int epochs, int batch, float lr,
                   uint64_t seed, double *losses);
const char *sdca_mlp_last_error(void);

/* Largest alignment sdca_eval_noalloc accepts: its scratch is a fixed array. */
#define SDCA_NOALLOC_MAX_SEQS 65536
#define SDCA_NOALLOC_MAX_LOCI 262144

/* One objective + gradient evaluation that allocates nothing (no counterpart
 * in SuperDCA; same value as sdca_eval).  For host programs that own all
 * device memory through their own allocator (a framework's caching
 * allocator, an embedded runtime with a fixed memory budget) and do not let
 * a library call cudaMalloc or cudaFree.  Every pointer is a DEVICE pointer
 * the caller allocated: states (n_seqs x n_loci codes 0..3), weights
 * (n_seqs), x and g (16 n_loci + 4 doubles, SuperDCA's parameter layout) and
 * f (one double).  lambda_h and lambda_J are absolute strengths (as
 * sdca_get_lambdas reports them).  Work is queued on `stream` (a cudaStream_t
 * or NULL) of the current device and is complete when that stream is.
 * Intermediate values live in one fixed __device__ array of the library
 * (about 2.1 MB, held by every GPU that loads the library until exit), so
 * n_seqs <= SDCA_NOALLOC_MAX_SEQS and n_loci <= SDCA_NOALLOC_MAX_LOCI, else
 * SDCA_E_ARG before any work is queued.  All calls share that array: calls
 * whose work overlaps on the GPU race.  The first call made with a CUDA
 * context current looks up the array's address in that context.  The states
 * are not read on the host, so a code >= 4 cannot be refused here as
 * sdca_set_alignment refuses it: it makes *f and the h part of g NaN.  An
 * error already pending in the CUDA runtime when the call starts is left in
 * place for the caller and reported as SDCA_E_CUDA, with nothing queued. */
int sdca_eval_noalloc(const uint8_t *states, int64_t n_seqs, int64_t n_loci,
                      const double *weights, double lambda_h, double lambda_J, uint32_t r,
                      const double *x, double *f, double *g, void *stream);

#ifdef __cplusplus
}
#endif
#endif
