// engine.h -- internal structures of the GB300 plmDCA solve engine.
//
// Device data layout ("engine layout"), q = 4:
//   X   [N][Lx]  uint8 state codes, sequence-major (Lx = L rounded up to 64)
//   XT  [L][Nx]  uint8 state codes, locus-major    (Nx = N rounded up to 64)
//   per slot b, a parameter vector of Dp floats (Dp = 16 L + 4 rounded up to
//   64): J_r[n][s][a] at 16 n + 4 s + a, h_r[a] at 16 L + a, zero padding.
//   The J_rr block (n == r) is held at zero and never enters the objective,
//   as in SuperDCA/include/plmDCA_objective.hpp:107-120,174-188,224-242.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/superdca_gb300.h"

namespace sdca {

constexpr int Q = 4;
constexpr int QQ = Q * Q;
constexpr int MAXHIST = 10;      // upper bound on the L-BFGS history length m

// Learned warm start: per-pair MLP MLP_IN -> MLP_H -> MLP_H -> MLP_OUT (ReLU).
// Parameter blob (floats): version, neighbours k, smoothing eps, h-fit flag,
// input mean and scale, W1 b1 W2 b2 W3 b3 (trained), output scale.
constexpr int MLP_IN = 40, MLP_H = 128, MLP_OUT = 16;
constexpr int MLP_BLOB_VERSION = 1;
constexpr int MLP_VERSION = 0, MLP_KNN = 1, MLP_EPS = 2, MLP_HFIT = 3;
constexpr int MLP_IN_MEAN = 4;
constexpr int MLP_IN_SCALE = MLP_IN_MEAN + MLP_IN;
constexpr int MLP_W1 = MLP_IN_SCALE + MLP_IN;
constexpr int MLP_B1 = MLP_W1 + MLP_H * MLP_IN;
constexpr int MLP_W2 = MLP_B1 + MLP_H;
constexpr int MLP_B2 = MLP_W2 + MLP_H * MLP_H;
constexpr int MLP_W3 = MLP_B2 + MLP_H;
constexpr int MLP_B3 = MLP_W3 + MLP_OUT * MLP_H;
constexpr int MLP_TRAIN_END = MLP_B3 + MLP_OUT;
constexpr int MLP_OUT_SCALE = MLP_TRAIN_END;
constexpr int MLP_BLOB_SIZE = MLP_OUT_SCALE + MLP_OUT;
constexpr int MLP_WB_ELEMS = MLP_H * 64 + MLP_H * MLP_H + MLP_OUT * MLP_H;   // BF16 weight image
constexpr int WS_MAX_K = 16;      // nearest neighbours per sequence, at most
// Dual form's learned start (blob version 2, same network): per-sequence
// statistics of a target column, DWS_K nearest neighbours
constexpr int MLP_BLOB_VERSION_DUAL = 2;
constexpr int DWS_K = 16;
constexpr int MLP_ALPHA = 2;      // version 2: the shrinkage of the predicted residuals (blob[2])

// per-slot accumulators (doubles), zeroed by the host before each use
enum Acc {
    ACC_F = 0,      // sum_i w_i (lse_i - l_i[s_i(r)])             (trial)
    ACC_DG,         // sum_i R_i . u_i                              (trial)
    ACC_RS0,        // sum_i R_i[a], a = 0..3                       (trial)
    ACC_RS1, ACC_RS2, ACC_RS3,
    ACC_G2,         // ||g||^2                                      (gradient)
    ACC_X2J,        // ||x_J||^2                                    (gradient)
    ACC_X2H,        // ||x_h||^2                                    (gradient)
    ACC_SY,         // s_k . y_k                                    (gradient)
    ACC_YY,         // y_k . y_k                                    (gradient)
    ACC_GD,         // g . d                                        (direction)
    ACC_DDJ,        // d_J . d_J                                    (direction)
    ACC_DDH,        // d_h . d_h                                    (direction)
    ACC_XDJ,        // x_J . d_J                                    (direction)
    ACC_XDH,        // x_h . d_h                                    (direction)
    ACC_GMAX,       // max |g| (bits of a non-negative double, atomicMax) (gradient)
    ACC_DMAX,       // max |d| (bits of a non-negative double, atomicMax) (direction)
    ACC_DG0,        // sum_i R_i . u_i at the current point: slope of the search line at 0 (forward)
    ACC_SS,         // s_k . s_k                                    (gradient)
    NACC = 20
};

// Per-slot parameters the kernels read; mirrored from the host before launches.
struct SlotDev {
    int32_t locus;          // target locus r
    int32_t gcur;           // g buffer holding the accepted gradient (0/1)
    int32_t ring_new;       // history position written by the last accept, -1 none
    int32_t nhist;          // history pairs in use
    int32_t ring[MAXHIST + 1];  // history positions, oldest first (dual-form dots: all live positions)
    int32_t flags;          // SLOT_F_*
    int32_t pad_;
    double stp;             // trial (or accepted) step along d
    double coef_g;          // direction = coef_g g + sum coefS_j s_j + coefY_j y_j
    double coefS[MAXHIST];
    double coefY[MAXHIST];
    double rs[Q];           // R sums at the accepted point (h gradient)
    double tc_scale;        // power of two applied to d before the fp16 hi/lo split
    double tc_inv_scale;
    double eta[Q];          // dual form: h part of the direction (trial logits) or of x (final layout)
};

// dual form: per slot, vectors (a, k = K a) of N x 4 doubles each:
// x, d, two gradients, then the s ring and the y ring (P.ring positions each)
constexpr int DV_X = 0, DV_D = 1, DV_G = 2, DV_S = 4;
constexpr int DOT_Y = 2 * MAXHIST;  // dual-form dots by ring position: s at [p], y at [DOT_Y + p]

// Dual form: the solver state of one slot, owned by the device while the
// slot iterates.  The host writes it once when a locus enters the slot and
// reads the DualSum summary after each round; the line-search kernel, the
// accept and gradient kernels and the control kernel advance it.
enum DualPhase {
    DC_EVAL0 = 0,   // start point evaluated by k_trial_dual: the next gradient pass is the first
    DC_STEP = 1,    // a direction is ready: line search, accept, gradient pass
    DC_STOP = 2,    // stopped (status set): the host forms the solution
};

struct DualCtl {
    int32_t phase;          // DualPhase
    int32_t gcur;           // gradient buffer holding the accepted gradient (0/1)
    int32_t ring_new;       // ring position of the pair the next accept forms, -1 none
    int32_t push;           // the next accept pushes s (and the gradient pass y)
    int32_t nhist;          // live history pairs, oldest first in hist[]
    int32_t hist[MAXHIST];
    int32_t iter;           // pairs since the last restart
    int32_t iterations, nfeval, restarts, skipped, weak, max_trials, trials;
    int32_t status;         // 0 gradient tolerance, 1 iteration limit, 2 relative-epsilon stop, -1 non-finite
    int32_t force_restart, stalled;
    int32_t last_check, chk_wait, want_check, releps_stop;
    double f;               // objective at the accepted point
    double g2, g2J;         // ||g||^2 (all, J part)
    double x2J;             // ||x_J||^2
    double gmax;            // max|g| (exact at a check, else the estimate chk_ratio ||g||)
    double chk_ratio;       // max|g| / ||g|| at the last check (0: none yet)
    double amax_g, amax_x;  // max |a| of the gradient and of x (FP32 scales of a check and of the solution)
    double gamma, sy_new, yy_new;
    double stp;             // accepted step of the last search
    double coef_g, coefS[MAXHIST], coefY[MAXHIST];
    double eta_x[Q], eta_d[Q], eta_g[2][Q], eta_s[MAXHIST + 1][Q], eta_y[MAXHIST + 1][Q];
    double SY[MAXHIST + 1][MAXHIST + 1], YY[MAXHIST + 1][MAXHIST + 1];
    double sg_prev[MAXHIST + 1], yg_prev[MAXHIST + 1];
    // the direction's coefficients as double-float for the direction kernel:
    // [0, m) coefS, [MAXHIST, MAXHIST + m) coefY, [2 MAXHIST] coef_g,
    // [2 MAXHIST + 1, + Q) eta_d
    float2 cdf[2 * MAXHIST + 1 + Q];
    float2 stp_df;          // stp as double-float (the accept kernel's step)
};

// What the host reads of each slot after a round (a copy of DualCtl fields).
struct DualSum {
    int32_t phase, status, want_check, chk_wait, releps_stop, iterations, nfeval, restarts, skipped, weak,
        max_trials, pad_;
    double f, gmax, amax_g, amax_x, x2J;
    double eta_x[Q];
};

// per-slot line-search and direction sums (doubles) of the dual form
enum DualAcc {
    DA_GD = 0,      // g.d, J part (direction kernel)
    DA_DDJ,         // d_J . d_J
    DA_XDJ,         // x_J . d_J
    DA_DG0,         // slope of the search line at 0, data part
    NDACC = 4
};

enum SlotFlags {
    SLOT_F_USE_U = 1,       // trial logits use lbase + stp u (else lbase)
    SLOT_F_PUSH = 2,        // accept pushes an (s, y) pair into the history
};

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

// launch configuration for the kernels of one call
struct SlotList {
    const int32_t *list;    // device array of slot indices
    int n;
};

struct Problem {
    int64_t N = 0, L = 0, Lx = 0, Nx = 0, Dp = 0, LC = 0;
    int64_t Cg = 0;  // locus chunks of the gather forward
    int64_t C = 0;   // partial-sum slices allocated (>= Cg and >= tensor-core K splits)
    int m = 10;
    int ring = 11;   // history positions per slot: m + 1 (one spare for the pending pair)
    int Bmax = 0;
    double lambda_h = 0, lambda_J = 0, b_eff = 0;
};

// kernel launchers (kernels_*.cu)
void launch_fwd_gather(const Problem &P, const uint8_t *X, const int32_t *list, int n,
                       const float *vecs, float *partial, cudaStream_t st);
void launch_reduce_partial(const Problem &P, const int32_t *list, int n, const float *partial,
                           const float *vecs, int add_h, float *out_f, double *out_d,
                           cudaStream_t st, int C = 0, const float *R = nullptr, double *acc = nullptr);
void launch_fwd_exact(const Problem &P, const uint8_t *X, const int32_t *list, int n, const float *vecs,
                      double *partial64, double *lbase, cudaStream_t st);
void launch_grad_finalize(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                          const float *wa, float *gpool, void *Ypool, const void *Spool, int hist_bf16,
                          double *acc, cudaStream_t st);
void launch_bwd_gather(const Problem &P, const uint8_t *XT, const SlotDev *sd,
                       const int32_t *list, int n, const float *R, const float *wa,
                       float *gpool, void *Ypool, const void *Spool, int hist_bf16,
                       double *acc, cudaStream_t st);
void launch_hpart(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                  const float *wa, float *gpool, void *Ypool, const void *Spool, int hist_bf16,
                  double *acc, cudaStream_t st);
void launch_trial(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                  const double *lbase, const float *u, const uint8_t *rstate, const double *w,
                  float *R, double *acc, cudaStream_t st);
void launch_accept(const Problem &P, const SlotDev *sd, const int32_t *list, int n, float *wa,
                   const float *d, void *Spool, int hist_bf16, cudaStream_t st);
void launch_lbase_update(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                         double *lbase, const float *u, cudaStream_t st);
void launch_hist_dots(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                      const float *gpool, const void *Spool, const void *Ypool, int hist_bf16,
                      double *dots, cudaStream_t st);
void launch_direction(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                      const float *gpool, const void *Spool, const void *Ypool, int hist_bf16,
                      const float *wa, float *d, double *acc, cudaStream_t st);
void launch_score(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                  const float *wa, int gap, float *rows, cudaStream_t st);

// dual form (kernels_dual.cu)
void launch_dual_kmat(const int32_t *dist, int N, int64_t Nx, int L, int32_t *K, cudaStream_t st);
void launch_dual_quant(const Problem &P, const SlotDev *sd, const int32_t *list, int n, const float *R,
                       const uint8_t *rstate, double qscale, int32_t *rq, long long *csum, cudaStream_t st, const int *cnt = nullptr);
void launch_dual_kprod(const Problem &P, const int32_t *list, int n, const uint8_t *rstate, const int32_t *K,
                       double qscale, const int32_t *rq, const long long *csum, float2 *KR, cudaStream_t st, const int *cnt = nullptr);
// the accept (x += stp d, s push, logits += stp u) of the slots that searched
// this round, then the gradient at the new point (y push, sums)
void launch_dual_grad(const Problem &P, const DualCtl *ctl, const int32_t *list, int n, double qscale,
                      const int32_t *rq, const float2 *KR, float2 *dv, double *acc, double *amax, cudaStream_t st,
                      const int *cnt = nullptr);
void launch_dual_dots(const Problem &P, const DualCtl *ctl, const int32_t *list, int n, int newg, const float2 *dv,
                      double *dots, cudaStream_t st, const int *cnt = nullptr);
void launch_dual_direction(const Problem &P, const DualCtl *ctl, const int32_t *list, int n, float2 *dv,
                           float *P0, const float *w, const uint8_t *rstate, float *ud, double *dacc,
                           cudaStream_t st, const int *cnt = nullptr);
// start and final evaluations of the dual form (logits k_x + eta, FP64 log-sum-exp)
void launch_dual_eval(const Problem &P, const SlotDev *sd, const int32_t *list, int n, const float2 *dv,
                      const uint8_t *rstate, const double *w, float *R, double *acc, cudaStream_t st);
void launch_dual_to_r(const Problem &P, const DualCtl *ctl, const int32_t *list, int n, int which,
                      const float2 *dv, float *R, cudaStream_t st);
// the per-iteration decisions of the dual form on the device
void launch_dual_linesearch(const Problem &P, DualCtl *ctl, const int32_t *list, int n, const double *dacc,
                            float2 *dv, float *ud, const uint8_t *rstate,
                            const float *w, const float *P0, float *R, double *acc, cudaStream_t st, const int *cnt = nullptr);
void launch_dual_control(const Problem &P, DualCtl *ctl, DualSum *sum, const int32_t *list, int n,
                         int max_iterations, double gtol, const double *acc, const double *amax, const double *dots,
                         cudaStream_t st, const int *cnt = nullptr);
void launch_dual_check_apply(DualCtl *ctl, DualSum *sum, const int32_t *list, int n, double gtol, const double *acc,
                             cudaStream_t st);
void launch_dual_digits(const Problem &P, const SlotDev *sd, const int32_t *list, int n, int d, const float2 *dv,
                        float *R, cudaStream_t st);
void launch_dual_digit_acc(const Problem &P, const SlotDev *sd, const int32_t *list, int n, int d,
                           const float *gpool, double *J64, cudaStream_t st);
// all three digit planes of x's a part in one pass: R rows d n + s, and their
// combination from gpool buffers d n + s
void launch_dual_digits3(const Problem &P, const SlotDev *sd, const int32_t *list, int n, const float2 *dv, float *R,
                         cudaStream_t st);
void launch_dual_planes_to_wa(const Problem &P, const SlotDev *sd, const int32_t *list, int n, const float *gpool,
                              float *wa, cudaStream_t st);
void launch_dual_to_wa(const Problem &P, const SlotDev *sd, const int32_t *list, int n, const double *J64,
                       float *wa, cudaStream_t st);

// warm start (mlp.cu, warmstart.cu)
// the BF16 image of the blob's weights that the tensor-core forward reads
// (MLP_WB_ELEMS BF16 values), and inference: raw features (M x MLP_IN) ->
// outputs (M x MLP_OUT) in the blob's output units; *err is set when a wait
// of the kernel gives up
void mlp_pack(const float *p_dev, void *wb, cudaStream_t st);
void mlp_infer(const float *p_dev, const void *wb, const float *X, int64_t M, float *out, int *err,
               cudaStream_t st);
void launch_distances(const uint8_t *X, int64_t ld, int N, int L, uint64_t *packed, int32_t *dist,
                      cudaStream_t st);
void launch_knn(const int32_t *dist, int N, int k, int32_t *knn, cudaStream_t st, int32_t *knn_d = nullptr);
// dual form's learned start: per-sequence statistics of the target columns
// cols + idx[g] * Nx (g < n) into feats [g][Nx][MLP_IN]; the network's
// residual prediction into the R rows of slots[g]; and the start point from
// the exact K rho of those rows
void launch_dual_ws_feats(const uint8_t *cols, const int32_t *idx, int n, int N, int64_t Nx, int L, const double *w,
                          const int32_t *knn, const int32_t *knn_d, float *feats, cudaStream_t st);
void launch_dual_ws_r(const int32_t *slots, int n, int N, int64_t Nx, const float *out, const float *p_dev, float alpha,
                      const float *w, float *R, cudaStream_t st);
void launch_dual_ws_init(const Problem &P, const int32_t *list, int n, double c, double qscale, const int32_t *rq,
                         const float2 *KR, float2 *dv, cudaStream_t st, const int *cnt = nullptr);
void launch_ws_residual(const uint8_t *XT, int64_t Nx, int N, const int32_t *loci, int G, const double *w,
                        const int32_t *knn, int k, float eps, float *Rws, cudaStream_t st);
void launch_ws_residual_split(const uint8_t *XT, int64_t Nx, int N, const int32_t *loci, const int32_t *slots, int G,
                              const double *w, const int32_t *knn, int k, float eps, float *R, float *R2,
                              cudaStream_t st);
void launch_ws_copy_r(int64_t Nx, const int32_t *slots, int G, const float *R2, float *R, cudaStream_t st);
void launch_ws_assemble(int L, int64_t Dp, const int32_t *slots, int G, const float *gpool, double b_eff,
                        float *feats, cudaStream_t st);
void launch_ws_pairs(const uint8_t *XT, int64_t Nx, int N, int L, int G, const float *Rws, double b_eff,
                     float *feats, cudaStream_t st);
void launch_ws_scatter(int L, int64_t Dp, const int32_t *slots, const int32_t *loci, int G, const float *out,
                       const float *p_dev, double out_mult, float *wa, double *xmax, cudaStream_t st);
void launch_ws_hfit(const Problem &P, const int32_t *slots, const uint8_t *rstate, const double *w, int G,
                    float *wa, double *lbase, double *xmax, cudaStream_t st);
void launch_weights(const uint8_t *X, int64_t ld, int N, int L, uint64_t *packed, double threshold,
                    const double *mult, double *nbr, unsigned long long *nonidentical, cudaStream_t st);

// tensor-core form (kernels_tc.cu)
struct TcPlan;
TcPlan *tc_plan_create(const Problem &P, const uint8_t *X, const uint8_t *XT, __half *Dhi, __half *Dlo,
                       __half *Rhi, __half *Rlo, int64_t Kp);
void tc_plan_destroy(TcPlan *p);
int tc_fwd_splits(const Problem &P, int nlist);
cudaError_t tc_configure();
cudaError_t tc_launch_fwd(const TcPlan *pl, const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                          const float *vecs, __half *Dhi, __half *Dlo, float *partial, int splits, int *err,
                          cudaStream_t st);
// exact_fp16: R holds values exact in fp16 (the dual form's digit planes), so
// the lo half of the split is zero and its MMA is skipped
// gmax_acc: max-only backward (no gradient written): each slot's max |g|
// over the blocks n != locus into gmax_acc[slot * gmax_stride].
// planes > 1: R holds planes x n rows by position (plane d of list position
// s at row d n + s) and row P's product goes to gpool buffer P; needs
// planes x n <= Bmax.
cudaError_t tc_launch_bwd(const TcPlan *pl, const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                          const float *R, float r_scale, __half *Rhi, __half *Rlo, float *gpool, int *err,
                          cudaStream_t st, bool exact_fp16 = false, double *gmax_acc = nullptr,
                          int gmax_stride = 0, int planes = 1);
// dual form: exact K rho on the tensor cores (N <= 4000, L < 2^18)
struct KdPlan;
int kd_nk_rows(const Problem &P);
int kd_nr_rows(const Problem &P);
KdPlan *tc_kdig_plan_create(const Problem &P, __half *Kd, __half *Rd);
void tc_kdig_plan_destroy(KdPlan *p);
void tc_kdig_fill_k(const KdPlan *pl, const Problem &P, const int32_t *K, __half *Kd, cudaStream_t st);
cudaError_t tc_launch_kdig(const KdPlan *pl, const Problem &P, const int32_t *list, int n, const int32_t *rq,
                           const uint8_t *rstate, const long long *csum, double inv_qscale, __half *Rd, float2 *KR,
                           int *err, cudaStream_t st, const int *cnt = nullptr);

} // namespace sdca
