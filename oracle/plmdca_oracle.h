/* plmdca_oracle.h -- FP64 CPU oracle for the plmDCA per-locus solve.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of SuperDCA's
 * per-locus pseudo-likelihood solve, used as the checker for the CUDA engine
 * (tests/, __graft_entry__.smoke()) and as the timed CPU baseline
 * (bench.py cpu_baseline / --impl reference).  The product path never links,
 * loads or calls anything in this directory.
 *
 * Parity status of each part:
 *   - objective/gradient, lambda rule, scoring (Ising gauge + Frobenius norm
 *     without GAP): pinned against SuperDCA's own headers compiled with shims
 *     (oracle/ref_golden.cpp -> oracle/_ref, fixtures in tests/golden/).
 *   - sequence weights: the reweighting arithmetic is pinned the same way; the
 *     Hamming distance it consumes comes from apegrunt (absent), so the
 *     distance definition itself is unpinned (see orc_weights).
 *   - L-BFGS + More-Thuente: restated from the published CppNumericalSolvers
 *     algorithm (no pinned commit available); trajectory parity unpinned, the
 *     converged objective is pinned by strict convexity.
 *
 * Parameter layout ("reference layout", D = q*q*L + q doubles):
 *   J_r occupies the first q*q*L entries in blocks of 16 loci.  For locus n in
 *   block b = n/16 with local position p = n%16 and block extent e (16, or
 *   L%16 for a partial last block), J_r[n][s][a] lives at
 *       b*16*q*q + (s*e + p)*q + a
 *   (SuperDCA/include/Matrix_kernel_access_order.hpp:28-34,
 *    SuperDCA/include/Coupling_matrix_view.hpp:156-168).
 *   h_r[a] follows at q*q*L + a
 *   (SuperDCA/include/plmDCA_optimizer_parameters.hpp:219-247).
 */
#ifndef PLMDCA_ORACLE_H
#define PLMDCA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_BLOCK 16

typedef struct {
    const uint8_t *states;   /* N x L, row-major (sequence-major), codes 0..q-1 */
    const double *weights;   /* N sequence weights */
    int64_t N;               /* sequences */
    int64_t L;               /* loci */
    int q;                   /* states per locus (4 in SuperDCA) */
    double lambda_h;         /* absolute strengths (already times B_eff) */
    double lambda_J;
    const uint8_t *targets;  /* two-alignment scan mode (plmDCA_objective.hpp:67): N x LT target
                                columns; locus r is targets[:, r] and no feature locus is
                                excluded.  NULL: the target is states[:, r]. */
    int64_t LT;
} orc_problem;

typedef struct {
    int64_t iterations;      /* L-BFGS iterations taken */
    int64_t nfeval;          /* objective evaluations, counted like SuperDCA */
    double f;                /* objective at the returned point */
    double gnorm_inf;        /* max-norm of the gradient at the returned point */
    int status;              /* 0 gradient tolerance, 1 iteration limit,
                                2 relative-epsilon stop, -1 non-finite */
} orc_stat;

int64_t orc_dim(int64_t L, int q);
int64_t orc_index(int64_t L, int q, int64_t n, int s, int a);

/* B_eff and the regularisation strengths
 * (SuperDCA/include/plmDCA_optimizer_parameters.hpp:257-284).  A negative
 * option value selects the automatic rule. */
void orc_lambdas(const double *w, int64_t N, double lambda_h_opt,
                 double lambda_J_opt, double *lambda_h, double *lambda_J,
                 double *b_eff);

/* Objective value and gradient for target locus r
 * (SuperDCA/include/plmDCA_objective.hpp:38-249).  g may be NULL. */
double orc_objective(const orc_problem *p, int64_t r, const double *x,
                     double *g);

/* Sequence reweighting (SuperDCA/include/plmDCA_optimizer_parameters.hpp:39-98)
 * over a Hamming distance that counts loci whose state codes differ.
 * mult may be NULL (all multiplicities 1).  Returns the number of
 * non-identical pairs. */
int64_t orc_weights(const uint8_t *states, int64_t N, int64_t L,
                    const double *mult, double threshold, double *w);

/* Minimise the objective for locus r from x (in/out), L-BFGS with history m
 * and a More-Thuente line search, stopping when the gradient max-norm drops
 * below gtol or after max_iter iterations. */
int orc_minimize(const orc_problem *p, int64_t r, double *x, int max_iter,
                 double gtol, int m, orc_stat *st);

/* Coupling scores of one solved locus: row[n] = || gauge(J_rn) ||_F with the
 * GAP row and column left out, for n != r; row[r] = NaN
 * (SuperDCA/include/plmDCA.hpp:366-394, plmDCA_utility.hpp:57-83,
 *  Matrix_math.hpp:134-178). */
void orc_score_row(const double *x, int64_t L, int q, int64_t r, int gap,
                   float *row);

/* Solve a list of loci on `threads` host threads with dynamic grain-1
 * scheduling (the tbb::parallel_reduce loop of SuperDCA/include/plmDCA.hpp:
 * 581-586).  scores: nloci x L floats (may be NULL), stats: nloci (may be
 * NULL), x_out: nloci x D doubles (may be NULL).  x_init: optional nloci x D
 * start points (NULL = zero start). */
int orc_solve(const orc_problem *p, const int64_t *loci, int64_t nloci,
              int threads, int max_iter, double gtol, int m, int gap,
              const double *x_init, float *scores, orc_stat *stats,
              double *x_out);

/* Evaluate the objective (with gradient) for `count` loci on `threads`
 * threads, for timing the evaluation rate. f_out: count values. */
int orc_eval_many(const orc_problem *p, const int64_t *loci, int64_t count,
                  int threads, const double *x, double *f_out);

#ifdef __cplusplus
}
#endif
#endif
