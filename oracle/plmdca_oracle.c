/* plmdca_oracle.c -- FP64 CPU oracle for the plmDCA per-locus solve.
 *
 * TEST INFRASTRUCTURE ONLY (see plmdca_oracle.h): the checker and the timed
 * CPU baseline, never the product path.
 */
#include "plmdca_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

int64_t orc_dim(int64_t L, int q) { return (int64_t)q * q * L + q; }

int64_t orc_index(int64_t L, int q, int64_t n, int s, int a)
{
    /* SuperDCA/include/Matrix_kernel_access_order.hpp:28-34 (STATES order)
     * inside 16-locus blocks, SuperDCA/include/Coupling_matrix_view.hpp:156-168 */
    const int64_t b = n / ORC_BLOCK, p = n % ORC_BLOCK;
    const int64_t nfull = L / ORC_BLOCK;
    const int64_t e = (b < nfull) ? ORC_BLOCK : (L % ORC_BLOCK);
    return b * ORC_BLOCK * q * q + ((int64_t)s * e + p) * q + a;
}

/* Horizontal sum of a 4-lane vector in the order SuperDCA's AVX `sum` uses:
 * (v0+v2)+(v1+v3) (SuperDCA/include/Vector_operations.hpp:39-48). */
static inline double hsum(const double *v, int q)
{
    if (q == 4) return (v[0] + v[2]) + (v[1] + v[3]);
    double s = 0.0;
    for (int a = 0; a < q; ++a) s += v[a];
    return s;
}

void orc_lambdas(const double *w, int64_t N, double lambda_h_opt,
                 double lambda_J_opt, double *lambda_h, double *lambda_J,
                 double *b_eff)
{
    /* SuperDCA/include/plmDCA_optimizer_parameters.hpp:257-284 */
    double beff = 0.0;
    for (int64_t i = 0; i < N; ++i) beff += w[i];
    const double autol = (beff > 500.0) ? 0.1 : 1.0 - ((1.0 - 0.1) * beff / 500.0);
    *lambda_J = (lambda_J_opt < 0.0) ? autol * beff / 2.0 : lambda_J_opt * beff;
    *lambda_h = (lambda_h_opt < 0.0) ? autol * beff : lambda_h_opt * beff;
    if (b_eff) *b_eff = beff;
}

double orc_objective(const orc_problem *p, int64_t r, const double *x,
                     double *g)
{
    /* SuperDCA/include/plmDCA_objective.hpp:38-249 */
    const int q = p->q;
    const int64_t N = p->N, L = p->L, qq = (int64_t)q * q;
    const int64_t nblocks = (L + ORC_BLOCK - 1) / ORC_BLOCK;
    const int scan = p->targets != NULL;   /* scan: r_block is past the last block, nothing excluded */
    const int64_t r_block = scan ? -1 : r / ORC_BLOCK, r_local = scan ? -1 : r % ORC_BLOCK;
    const double *h = x + qq * L;
    double *lp = (double *)malloc(sizeof(double) * N * q);
    double *nb = (double *)malloc(sizeof(double) * N * q);
    double acc[8], e[8];
    double fval = 0.0;

    if (g) memset(g, 0, sizeof(double) * orc_dim(L, q));

    /* logPot_i = h_r + sum over blocks of the block's 16-locus partial sum
     * (plmDCA_objective.hpp:86-121; Coupling_matrix_view.hpp:59-86) */
    for (int64_t i = 0; i < N; ++i)
        for (int a = 0; a < q; ++a) lp[i * q + a] = h[a];
    for (int64_t b = 0; b < nblocks; ++b) {
        const int64_t ext = (b == nblocks - 1 && L % ORC_BLOCK) ? L % ORC_BLOCK : ORC_BLOCK;
        const double *Jb = x + b * ORC_BLOCK * qq;
        for (int64_t i = 0; i < N; ++i) {
            const uint8_t *si = p->states + i * L + b * ORC_BLOCK;
            for (int a = 0; a < q; ++a) acc[a] = 0.0;
            for (int64_t pp = 0; pp < ext; ++pp) {
                if (b == r_block && pp == r_local) continue;
                const double *Jv = Jb + ((int64_t)si[pp] * ext + pp) * q;
                for (int a = 0; a < q; ++a) acc[a] += Jv[a];
            }
            for (int a = 0; a < q; ++a) lp[i * q + a] += acc[a];
        }
    }

    /* pseudo-likelihood terms and node beliefs (plmDCA_objective.hpp:126-151) */
    for (int64_t i = 0; i < N; ++i) {
        const double *l = lp + i * q;
        const int sr = scan ? p->targets[i * p->LT + r] : p->states[i * L + r];
        const double w = p->weights[i];
        for (int a = 0; a < q; ++a) e[a] = exp(l[a]);
        const double z = log(hsum(e, q));
        fval += w * (z - l[sr]);
        double *nbi = nb + i * q;
        for (int a = 0; a < q; ++a) nbi[a] = w * exp(l[a] - z);
        nbi[sr] -= w;
        if (g)
            for (int a = 0; a < q; ++a) g[qq * L + a] += nbi[a];
    }

    /* gradient scatter (plmDCA_objective.hpp:153-190) */
    if (g) {
        for (int64_t b = 0; b < nblocks; ++b) {
            const int64_t ext = (b == nblocks - 1 && L % ORC_BLOCK) ? L % ORC_BLOCK : ORC_BLOCK;
            double *Gb = g + b * ORC_BLOCK * qq;
            for (int64_t i = 0; i < N; ++i) {
                const uint8_t *si = p->states + i * L + b * ORC_BLOCK;
                const double *nbi = nb + i * q;
                for (int64_t pp = 0; pp < ext; ++pp) {
                    if (b == r_block && pp == r_local) continue;
                    double *Gv = Gb + ((int64_t)si[pp] * ext + pp) * q;
                    for (int a = 0; a < q; ++a) Gv[a] += nbi[a];
                }
            }
        }
    }

    /* L2 regularisation (plmDCA_objective.hpp:192-244) */
    for (int a = 0; a < q; ++a) e[a] = p->lambda_h * (h[a] * h[a]);
    fval += hsum(e, q);
    if (g)
        for (int a = 0; a < q; ++a) g[qq * L + a] += (p->lambda_h * 2.0) * h[a];
    for (int64_t b = 0; b < nblocks; ++b) {
        const int64_t ext = (b == nblocks - 1 && L % ORC_BLOCK) ? L % ORC_BLOCK : ORC_BLOCK;
        const double *Jb = x + b * ORC_BLOCK * qq;
        for (int s = 0; s < q; ++s) {
            for (int64_t pp = 0; pp < ext; ++pp) {
                if (b == r_block && pp == r_local) continue;
                const int64_t off = b * ORC_BLOCK * qq + ((int64_t)s * ext + pp) * q;
                const double *Jv = Jb + ((int64_t)s * ext + pp) * q;
                if (g)
                    for (int a = 0; a < q; ++a) g[off + a] += (p->lambda_J * 2.0) * Jv[a];
                for (int a = 0; a < q; ++a) e[a] = p->lambda_J * (Jv[a] * Jv[a]);
                fval += hsum(e, q);
            }
        }
    }
    free(lp);
    free(nb);
    return fval;
}

int64_t orc_weights(const uint8_t *states, int64_t N, int64_t L,
                    const double *mult, double threshold, double *w)
{
    /* SuperDCA/include/plmDCA_optimizer_parameters.hpp:39-98.  The distance
     * d_ij is the number of loci at which the two state codes differ. */
    double *iw = (double *)malloc(sizeof(double) * N);
    int64_t nonidentical = 0;
    for (int64_t i = 0; i < N; ++i) iw[i] = mult ? mult[i] : 1.0;
    for (int64_t i = 0; i < N; ++i) {
        const uint8_t *si = states + i * L;
        const double mi = mult ? mult[i] : 1.0;
        for (int64_t j = 0; j < i; ++j) {
            const uint8_t *sj = states + j * L;
            int64_t d = 0;
            for (int64_t n = 0; n < L; ++n) d += (si[n] != sj[n]);
            const double identity = (double)(L - d) / (double)L;
            if (identity >= threshold) {
                iw[i] += mult ? mult[j] : 1.0;
                iw[j] += mi;
            } else {
                ++nonidentical;
            }
        }
    }
    for (int64_t i = 0; i < N; ++i) w[i] = (mult ? mult[i] : 1.0) / iw[i];
    free(iw);
    return nonidentical;
}

/* ---------------------------------------------------------------------- */
/* L-BFGS with More-Thuente line search.
 *
 * Restates the published CppNumericalSolvers LbfgsSolver / MoreThuente pair
 * as SuperDCA drives it (history 10, stop on the gradient max-norm or on the
 * iteration limit; SuperDCA/include/plmDCA.hpp:218-221, 298-304 and the
 * value_and_gradient patch in SuperDCA/externals/CppNumericalSolvers.*.patch).
 * The line search follows More & Thuente, ACM TOMS 20(3) 1994 (MINPACK
 * cvsrch/cstep). */

typedef struct {
    const orc_problem *p;
    int64_t r, D;
    int64_t nfeval;
} orc_fn;

static double fn_eval(orc_fn *fn, const double *x, double *g)
{
    fn->nfeval++;
    return orc_objective(fn->p, fn->r, x, g);
}

static double dot(const double *a, const double *b, int64_t n)
{
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

static double nrm2(const double *a, int64_t n) { return sqrt(dot(a, a, n)); }

static double nrminf(const double *a, int64_t n)
{
    double m = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double v = fabs(a[i]);
        if (v > m) m = v;
    }
    return m;
}

static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }

/* Safeguarded cubic/quadratic step (More-Thuente cstep). */
static int cstep(double *stx, double *fx, double *dx, double *sty, double *fy,
                 double *dy, double *stp, double fp, double dp, int *brackt,
                 double stpmin, double stpmax, int *info)
{
    *info = 0;
    int bound = 0;
    if ((*brackt && ((*stp <= dmin(*stx, *sty)) || (*stp >= dmax(*stx, *sty)))) ||
        (*dx * (*stp - *stx) >= 0.0) || (stpmax < stpmin))
        return -1;
    const double sgnd = dp * (*dx / fabs(*dx));
    double stpf = 0, stpc = 0, stpq = 0;
    if (fp > *fx) {
        *info = 1;
        bound = 1;
        const double theta = 3.0 * (*fx - fp) / (*stp - *stx) + *dx + dp;
        const double s = dmax(fabs(theta), dmax(fabs(*dx), fabs(dp)));
        double gamma = s * sqrt((theta / s) * (theta / s) - (*dx / s) * (dp / s));
        if (*stp < *stx) gamma = -gamma;
        const double pp = (gamma - *dx) + theta;
        const double qq = ((gamma - *dx) + gamma) + dp;
        const double rr = pp / qq;
        stpc = *stx + rr * (*stp - *stx);
        stpq = *stx + ((*dx / ((*fx - fp) / (*stp - *stx) + *dx)) / 2.0) * (*stp - *stx);
        if (fabs(stpc - *stx) < fabs(stpq - *stx))
            stpf = stpc;
        else
            stpf = stpc + (stpq - stpc) / 2.0;
        *brackt = 1;
    } else if (sgnd < 0.0) {
        *info = 2;
        bound = 0;
        const double theta = 3.0 * (*fx - fp) / (*stp - *stx) + *dx + dp;
        const double s = dmax(fabs(theta), dmax(fabs(*dx), fabs(dp)));
        double gamma = s * sqrt((theta / s) * (theta / s) - (*dx / s) * (dp / s));
        if (*stp > *stx) gamma = -gamma;
        const double pp = (gamma - dp) + theta;
        const double qq = ((gamma - dp) + gamma) + *dx;
        const double rr = pp / qq;
        stpc = *stp + rr * (*stx - *stp);
        stpq = *stp + (dp / (dp - *dx)) * (*stx - *stp);
        if (fabs(stpc - *stp) > fabs(stpq - *stp))
            stpf = stpc;
        else
            stpf = stpq;
        *brackt = 1;
    } else if (fabs(dp) < fabs(*dx)) {
        *info = 3;
        bound = 1;
        const double theta = 3.0 * (*fx - fp) / (*stp - *stx) + *dx + dp;
        const double s = dmax(fabs(theta), dmax(fabs(*dx), fabs(dp)));
        double gamma = s * sqrt(dmax(0.0, (theta / s) * (theta / s) - (*dx / s) * (dp / s)));
        if (*stp > *stx) gamma = -gamma;
        const double pp = (gamma - dp) + theta;
        const double qq = (gamma + (*dx - dp)) + gamma;
        const double rr = pp / qq;
        if (rr < 0.0 && gamma != 0.0)
            stpc = *stp + rr * (*stx - *stp);
        else if (*stp > *stx)
            stpc = stpmax;
        else
            stpc = stpmin;
        stpq = *stp + (dp / (dp - *dx)) * (*stx - *stp);
        if (*brackt) {
            stpf = (fabs(*stp - stpc) < fabs(*stp - stpq)) ? stpc : stpq;
        } else {
            stpf = (fabs(*stp - stpc) > fabs(*stp - stpq)) ? stpc : stpq;
        }
    } else {
        *info = 4;
        bound = 0;
        if (*brackt) {
            const double theta = 3.0 * (fp - *fy) / (*sty - *stp) + *dy + dp;
            const double s = dmax(fabs(theta), dmax(fabs(*dy), fabs(dp)));
            double gamma = s * sqrt((theta / s) * (theta / s) - (*dy / s) * (dp / s));
            if (*stp > *sty) gamma = -gamma;
            const double pp = (gamma - dp) + theta;
            const double qq = ((gamma - dp) + gamma) + *dy;
            const double rr = pp / qq;
            stpc = *stp + rr * (*sty - *stp);
            stpf = stpc;
        } else if (*stp > *stx) {
            stpf = stpmax;
        } else {
            stpf = stpmin;
        }
    }
    if (fp > *fx) {
        *sty = *stp;
        *fy = fp;
        *dy = dp;
    } else {
        if (sgnd < 0.0) {
            *sty = *stx;
            *fy = *fx;
            *dy = *dx;
        }
        *stx = *stp;
        *fx = fp;
        *dx = dp;
    }
    stpf = dmin(stpmax, stpf);
    stpf = dmax(stpmin, stpf);
    *stp = stpf;
    if (*brackt && bound) {
        if (*sty > *stx)
            *stp = dmin(*stx + 0.66 * (*sty - *stx), *stp);
        else
            *stp = dmax(*stx + 0.66 * (*sty - *stx), *stp);
    }
    return 0;
}

/* Line search along s from x (f, g at x given).  On return x, f, g hold the
 * last evaluated point and *stp its step.  Returns the number of trial
 * evaluations. */
static int cvsrch(orc_fn *fn, double *x, double *f, double *g, double *stp,
                  const double *s, double *wa)
{
    const int64_t D = fn->D;
    const double xtol = 1e-15, ftol = 1e-4, gtol = 1e-2;
    const double stpmin = 1e-15, stpmax = 1e15, xtrapf = 4.0;
    const int maxfev = 20;
    int info = 0, infoc = 1, nfev = 0;
    const double dginit = dot(g, s, D);
    if (dginit >= 0.0) return 0; /* not a descent direction: no trial */
    int brackt = 0, stage1 = 1;
    const double finit = *f, dgtest = ftol * dginit;
    double width = stpmax - stpmin, width1 = 2.0 * width;
    memcpy(wa, x, sizeof(double) * D);
    double stx = 0.0, fx = finit, dgx = dginit;
    double sty = 0.0, fy = finit, dgy = dginit;
    double stmin, stmax;
    for (;;) {
        if (brackt) {
            stmin = dmin(stx, sty);
            stmax = dmax(stx, sty);
        } else {
            stmin = stx;
            stmax = *stp + xtrapf * (*stp - stx);
        }
        *stp = dmax(*stp, stpmin);
        *stp = dmin(*stp, stpmax);
        if ((brackt && ((*stp <= stmin) || (*stp >= stmax))) || (nfev >= maxfev - 1) ||
            (infoc == 0) || (brackt && ((stmax - stmin) <= (xtol * stmax))))
            *stp = stx;
        for (int64_t i = 0; i < D; ++i) x[i] = wa[i] + *stp * s[i];
        *f = fn_eval(fn, x, g);
        nfev++;
        const double dg = dot(g, s, D);
        const double ftest1 = finit + *stp * dgtest;
        if ((brackt && ((*stp <= stmin) || (*stp >= stmax))) || (infoc == 0)) info = 6;
        if ((*stp == stpmax) && (*f <= ftest1) && (dg <= dgtest)) info = 5;
        if ((*stp == stpmin) && ((*f > ftest1) || (dg >= dgtest))) info = 4;
        if (nfev >= maxfev) info = 3;
        if (brackt && (stmax - stmin <= xtol * stmax)) info = 2;
        if ((*f <= ftest1) && (fabs(dg) <= gtol * (-dginit))) info = 1;
        if (info != 0) return nfev;
        if (stage1 && (*f <= ftest1) && (dg >= dmin(ftol, gtol) * dginit)) stage1 = 0;
        if (stage1 && (*f <= fx) && (*f > ftest1)) {
            const double fm = *f - *stp * dgtest;
            double fxm = fx - stx * dgtest;
            double fym = fy - sty * dgtest;
            const double dgm = dg - dgtest;
            double dgxm = dgx - dgtest;
            double dgym = dgy - dgtest;
            cstep(&stx, &fxm, &dgxm, &sty, &fym, &dgym, stp, fm, dgm, &brackt, stmin, stmax, &infoc);
            fx = fxm + stx * dgtest;
            fy = fym + sty * dgtest;
            dgx = dgxm + dgtest;
            dgy = dgym + dgtest;
        } else {
            cstep(&stx, &fx, &dgx, &sty, &fy, &dgy, stp, *f, dg, &brackt, stmin, stmax, &infoc);
        }
        if (brackt) {
            if (fabs(sty - stx) >= 0.66 * width1) *stp = stx + 0.5 * (sty - stx);
            width1 = width;
            width = fabs(sty - stx);
        }
    }
}

int orc_minimize(const orc_problem *p, int64_t r, double *x, int max_iter,
                 double gtol, int m, orc_stat *st)
{
    const int64_t D = orc_dim(p->L, p->q);
    orc_fn fn = {p, r, D, 0};
    double *S = (double *)calloc((size_t)D * m, sizeof(double));
    double *Y = (double *)calloc((size_t)D * m, sizeof(double));
    double *alpha = (double *)calloc(m, sizeof(double));
    double *grad = (double *)malloc(sizeof(double) * D);
    double *gold = (double *)malloc(sizeof(double) * D);
    double *qv = (double *)malloc(sizeof(double) * D);
    double *sdir = (double *)malloc(sizeof(double) * D);
    double *xt = (double *)malloc(sizeof(double) * D);
    double *wa = (double *)malloc(sizeof(double) * D);
    double *xold = (double *)malloc(sizeof(double) * D);
    int status = 1;
    int64_t iterations = 0;
    int iter = 0;
    double H0k = 1.0;

    double f = fn_eval(&fn, x, grad);
    memcpy(xold, x, sizeof(double) * D);
    double gnorm = nrminf(grad, D);
    for (;;) {
        const double releps = 1e-4 * dmax(1.0, nrm2(x, D));
        if (nrm2(grad, D) < releps) {
            status = 2;
            break;
        }
        /* two-loop recursion over the k most recent pairs (column 0 oldest) */
        memcpy(qv, grad, sizeof(double) * D);
        const int k = iter < m ? iter : m;
        for (int i = k - 1; i >= 0; --i) {
            const double rho = 1.0 / dot(S + (int64_t)i * D, Y + (int64_t)i * D, D);
            alpha[i] = rho * dot(S + (int64_t)i * D, qv, D);
            const double *yi = Y + (int64_t)i * D;
            for (int64_t j = 0; j < D; ++j) qv[j] -= alpha[i] * yi[j];
        }
        for (int64_t j = 0; j < D; ++j) qv[j] *= H0k;
        for (int i = 0; i < k; ++i) {
            const double rho = 1.0 / dot(S + (int64_t)i * D, Y + (int64_t)i * D, D);
            const double beta = rho * dot(Y + (int64_t)i * D, qv, D);
            const double *si = S + (int64_t)i * D;
            for (int64_t j = 0; j < D; ++j) qv[j] += si[j] * (alpha[i] - beta);
        }
        const double descent = -dot(grad, qv, D);
        double alpha_init = 1.0 / nrm2(grad, D);
        if (descent > -1e-4 * releps) {
            /* not a usable descent direction: restart from steepest descent */
            memcpy(qv, grad, sizeof(double) * D);
            iter = 0;
            alpha_init = 1.0;
        }
        /* line search along -q from x: the search evaluates f at x first
         * (SuperDCA counts that evaluation), which equals the value held */
        fn.nfeval++;
        for (int64_t j = 0; j < D; ++j) sdir[j] = -qv[j];
        memcpy(xt, x, sizeof(double) * D);
        memcpy(gold, grad, sizeof(double) * D);
        double ft = f, stp = alpha_init;
        const int trials = cvsrch(&fn, xt, &ft, grad, &stp, sdir, wa);
        /* x <- x - rate * q, then the gradient there; when the search made
         * no trial the new point has to be evaluated here */
        for (int64_t j = 0; j < D; ++j) x[j] = x[j] - stp * qv[j];
        if (trials == 0) {
            f = fn_eval(&fn, x, grad);
        } else {
            fn.nfeval++; /* SuperDCA re-evaluates the accepted point */
            f = ft;
        }
        double ys = 0.0, yy = 0.0;
        {
            const int col = iter < m ? iter : m - 1;
            if (iter >= m) {
                memmove(S, S + D, sizeof(double) * D * (m - 1));
                memmove(Y, Y + D, sizeof(double) * D * (m - 1));
            }
            double *sc = S + (int64_t)col * D, *yc = Y + (int64_t)col * D;
            for (int64_t j = 0; j < D; ++j) {
                sc[j] = x[j] - xold[j];
                yc[j] = grad[j] - gold[j];
            }
            ys = dot(yc, sc, D);
            yy = dot(yc, yc, D);
        }
        H0k = ys / yy;
        memcpy(xold, x, sizeof(double) * D);
        iter++;
        iterations++;
        gnorm = nrminf(grad, D);
        if (!isfinite(f) || !isfinite(gnorm)) {
            status = -1;
            break;
        }
        if (iterations > max_iter) {
            status = 1;
            break;
        }
        if (gtol > 0 && gnorm < gtol) {
            status = 0;
            break;
        }
    }
    if (st) {
        st->iterations = iterations;
        st->nfeval = fn.nfeval;
        st->f = f;
        st->gnorm_inf = gnorm;
        st->status = status;
    }
    free(S); free(Y); free(alpha); free(grad); free(gold); free(qv);
    free(sdir); free(xt); free(wa); free(xold);
    return status;
}

void orc_score_row(const double *x, int64_t L, int q, int64_t r, int gap,
                   float *row)
{
    /* SuperDCA/include/plmDCA.hpp:378-393 with ising_gauge
     * (plmDCA_utility.hpp:57-83) and frobenius_norm without GAP
     * (Matrix_math.hpp:166-213).  M = J_rn (rows: state of n, columns: state
     * of r), transposed when n < r.  The gauge is
     *   G[i][j] = ((M[i][j] - rowmean(M)[j]) - colmean(M)[i]) + mean(rowmean)
     * which is what the reference's mean/repmat composition evaluates (the row
     * mean is spread along columns and the column mean along rows). */
    double J[8][8], G[8][8], rm[8], cm[8];
    for (int64_t n = 0; n < L; ++n) {
        if (n == r) {
            row[n] = NAN;
            continue;
        }
        double gm = 0.0;
        for (int s = 0; s < q; ++s)
            for (int a = 0; a < q; ++a) {
                const double v = x[orc_index(L, q, n, s, a)];
                if (n < r) J[a][s] = v; else J[s][a] = v;
            }
        for (int i = 0; i < q; ++i) {
            double t = 0.0;
            for (int j = 0; j < q; ++j) t = t + J[i][j];
            rm[i] = t / q;
        }
        for (int j = 0; j < q; ++j) {
            double t = 0.0;
            for (int i = 0; i < q; ++i) t = t + J[i][j];
            cm[j] = t / q;
        }
        {
            double t = 0.0;
            for (int i = 0; i < q; ++i) t += rm[i];
            gm = t / q;
        }
        for (int i = 0; i < q; ++i)
            for (int j = 0; j < q; ++j) G[i][j] = ((J[i][j] - rm[j]) - cm[i]) + gm;
        double sum = 0.0;
        for (int i = 0; i < q; ++i) {
            if (i == gap) continue;
            for (int j = 0; j < q; ++j) {
                if (j == gap) continue;
                sum += G[i][j] * G[i][j];
            }
        }
        row[n] = (float)sqrt(sum);
    }
}

/* ---------------------------------------------------------------------- */
/* host-thread loop over loci (dynamic scheduling, grain 1) */

typedef struct {
    const orc_problem *p;
    const int64_t *loci;
    int64_t nloci;
    int max_iter, m, gap;
    double gtol;
    const double *x_init;
    float *scores;
    orc_stat *stats;
    double *x_out;
    const double *x_eval;
    double *f_out;
    int64_t next;
    pthread_mutex_t lock;
} orc_pool;

static int64_t pool_take(orc_pool *pl)
{
    pthread_mutex_lock(&pl->lock);
    const int64_t k = pl->next < pl->nloci ? pl->next++ : -1;
    pthread_mutex_unlock(&pl->lock);
    return k;
}

static void *solve_worker(void *arg)
{
    orc_pool *pl = (orc_pool *)arg;
    const int64_t D = orc_dim(pl->p->L, pl->p->q);
    double *x = (double *)malloc(sizeof(double) * D);
    for (int64_t k; (k = pool_take(pl)) >= 0;) {
        const int64_t r = pl->loci[k];
        if (pl->x_init)
            memcpy(x, pl->x_init + k * D, sizeof(double) * D);
        else
            memset(x, 0, sizeof(double) * D);
        orc_stat st;
        orc_minimize(pl->p, r, x, pl->max_iter, pl->gtol, pl->m, &st);
        if (pl->stats) pl->stats[k] = st;
        /* scan mode scores every block as stored, untransposed (plmDCA.hpp:370-377) */
        if (pl->scores)
            orc_score_row(x, pl->p->L, pl->p->q, pl->p->targets ? -1 : r, pl->gap, pl->scores + k * pl->p->L);
        if (pl->x_out) memcpy(pl->x_out + k * D, x, sizeof(double) * D);
    }
    free(x);
    return NULL;
}

static void *eval_worker(void *arg)
{
    orc_pool *pl = (orc_pool *)arg;
    const int64_t D = orc_dim(pl->p->L, pl->p->q);
    double *g = (double *)malloc(sizeof(double) * D);
    for (int64_t k; (k = pool_take(pl)) >= 0;) {
        const double f = orc_objective(pl->p, pl->loci[k], pl->x_eval, g);
        if (pl->f_out) pl->f_out[k] = f;
    }
    free(g);
    return NULL;
}

static int run_pool(orc_pool *pl, int threads, void *(*fnp)(void *))
{
    if (threads < 1) threads = 1;
    pthread_t *t = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    pthread_mutex_init(&pl->lock, NULL);
    int started = 0;
    for (int i = 0; i < threads; ++i)
        if (pthread_create(&t[i], NULL, fnp, pl) == 0) started++;
        else break;
    if (started == 0) fnp(pl);
    for (int i = 0; i < started; ++i) pthread_join(t[i], NULL);
    pthread_mutex_destroy(&pl->lock);
    free(t);
    return 0;
}

int orc_solve(const orc_problem *p, const int64_t *loci, int64_t nloci,
              int threads, int max_iter, double gtol, int m, int gap,
              const double *x_init, float *scores, orc_stat *stats,
              double *x_out)
{
    orc_pool pl;
    memset(&pl, 0, sizeof(pl));
    pl.p = p; pl.loci = loci; pl.nloci = nloci; pl.max_iter = max_iter;
    pl.m = m; pl.gap = gap; pl.gtol = gtol; pl.x_init = x_init;
    pl.scores = scores; pl.stats = stats; pl.x_out = x_out;
    return run_pool(&pl, threads, solve_worker);
}

int orc_eval_many(const orc_problem *p, const int64_t *loci, int64_t count,
                  int threads, const double *x, double *f_out)
{
    orc_pool pl;
    memset(&pl, 0, sizeof(pl));
    pl.p = p; pl.loci = loci; pl.nloci = count; pl.x_eval = x; pl.f_out = f_out;
    return run_pool(&pl, threads, eval_worker);
}
