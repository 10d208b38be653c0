// linesearch.h -- resumable More-Thuente line search (host, FP64).
//
// SuperDCA minimises each locus with CppNumericalSolvers' LbfgsSolver, whose
// line search is More & Thuente's (ACM TOMS 20(3), 1994; MINPACK cvsrch /
// cstep) with ftol 1e-4, gtol 1e-2, xtol 1e-15, step bounds [1e-15, 1e15],
// extrapolation factor 4 and at most 20 evaluations.  The CppNumericalSolvers
// source is an absent submodule of SuperDCA (SuperDCA/externals/
// CppNumericalSolvers.*.patch patches it to call value_and_gradient once per
// trial), so this restates the published method.
//
// The search is written as a state machine so that every slot of a batch can
// hold its own search: start() gives the first trial step, each feed() takes
// f and g.s at the last trial and either asks for another step or finishes.
// The accepted point is always the last trial evaluated.  The same code runs
// on the host (tensor-core and plain forms) and on the device (the dual
// form's line-search kernel, one search per thread block).
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define SDCA_HD __host__ __device__
#else
#define SDCA_HD
#endif

namespace sdca {

// std::min / std::max semantics (the first operand wins ties and NaN
// comparisons), usable in device code
SDCA_HD inline double mt_min(double a, double b) { return (b < a) ? b : a; }
SDCA_HD inline double mt_max(double a, double b) { return (a < b) ? b : a; }

class MoreThuente {
public:
    enum Result { NEED_EVAL = 0, DONE = 1, NO_DESCENT = 2 };

    double stp = 0;  // the step to evaluate next (NEED_EVAL) or the final step
    int nfev = 0;    // trials evaluated
    int info = 0;

    SDCA_HD Result start(double f0, double dg0, double stp0)
    {
        stp = stp0;
        nfev = 0;
        info = 0;
        infoc = 1;
        if (!(dg0 < 0.0)) return NO_DESCENT;
        brackt = false;
        stage1 = true;
        finit = f0;
        dginit = dg0;
        dgtest = kFtol * dginit;
        width = kStpmax - kStpmin;
        width1 = 2.0 * width;
        stx = 0.0; fx = finit; dgx = dginit;
        sty = 0.0; fy = finit; dgy = dginit;
        prepare();
        return NEED_EVAL;
    }

    SDCA_HD Result feed(double f, double dg)
    {
        nfev++;
        const double ftest1 = finit + stp * dgtest;
        if ((brackt && ((stp <= stmin) || (stp >= stmax))) || (infoc == 0)) info = 6;
        if ((stp == kStpmax) && (f <= ftest1) && (dg <= dgtest)) info = 5;
        if ((stp == kStpmin) && ((f > ftest1) || (dg >= dgtest))) info = 4;
        if (nfev >= kMaxfev) info = 3;
        if (brackt && (stmax - stmin <= kXtol * stmax)) info = 2;
        if ((f <= ftest1) && (fabs(dg) <= kGtol * (-dginit))) info = 1;
        if (info != 0) return DONE;
        if (stage1 && (f <= ftest1) && (dg >= mt_min(kFtol, kGtol) * dginit)) stage1 = false;
        if (stage1 && (f <= fx) && (f > ftest1)) {
            // modified function psi(stp) = f(stp) - f(0) - stp * dgtest
            const double fm = f - stp * dgtest;
            double fxm = fx - stx * dgtest, fym = fy - sty * dgtest;
            const double dgm = dg - dgtest;
            double dgxm = dgx - dgtest, dgym = dgy - dgtest;
            step(stx, fxm, dgxm, sty, fym, dgym, stp, fm, dgm);
            fx = fxm + stx * dgtest;
            fy = fym + sty * dgtest;
            dgx = dgxm + dgtest;
            dgy = dgym + dgtest;
        } else {
            step(stx, fx, dgx, sty, fy, dgy, stp, f, dg);
        }
        if (brackt) {
            if (fabs(sty - stx) >= 0.66 * width1) stp = stx + 0.5 * (sty - stx);
            width1 = width;
            width = fabs(sty - stx);
        }
        prepare();
        return NEED_EVAL;
    }

private:
    static constexpr double kXtol = 1e-15, kFtol = 1e-4, kGtol = 1e-2;
    static constexpr double kStpmin = 1e-15, kStpmax = 1e15, kXtrapf = 4.0;
    static constexpr int kMaxfev = 20;

    bool brackt = false, stage1 = true;
    int infoc = 1;
    double finit = 0, dginit = 0, dgtest = 0, width = 0, width1 = 0;
    double stx = 0, fx = 0, dgx = 0, sty = 0, fy = 0, dgy = 0, stmin = 0, stmax = 0;

    // interval of uncertainty and safeguards for the next trial
    SDCA_HD void prepare()
    {
        if (brackt) {
            stmin = mt_min(stx, sty);
            stmax = mt_max(stx, sty);
        } else {
            stmin = stx;
            stmax = stp + kXtrapf * (stp - stx);
        }
        stp = mt_max(stp, kStpmin);
        stp = mt_min(stp, kStpmax);
        if ((brackt && ((stp <= stmin) || (stp >= stmax))) || (nfev >= kMaxfev - 1) ||
            (infoc == 0) || (brackt && ((stmax - stmin) <= (kXtol * stmax))))
            stp = stx;
    }

    // safeguarded step: minimiser of a cubic or quadratic interpolant
    SDCA_HD void step(double &sx, double &fxv, double &dx, double &sy, double &fyv, double &dy,
                      double &st, double fp, double dp)
    {
        infoc = 0;
        if ((brackt && ((st <= mt_min(sx, sy)) || (st >= mt_max(sx, sy)))) ||
            (dx * (st - sx) >= 0.0) || (stmax < stmin))
            return;
        bool bound = false;
        const double sgnd = dp * (dx / fabs(dx));
        double stpf, stpc, stpq;
        if (fp > fxv) {
            infoc = 1;
            bound = true;
            const double theta = 3.0 * (fxv - fp) / (st - sx) + dx + dp;
            const double s = mt_max(fabs(theta), mt_max(fabs(dx), fabs(dp)));
            double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
            if (st < sx) gamma = -gamma;
            const double p = (gamma - dx) + theta, q = ((gamma - dx) + gamma) + dp;
            stpc = sx + (p / q) * (st - sx);
            stpq = sx + ((dx / ((fxv - fp) / (st - sx) + dx)) / 2.0) * (st - sx);
            stpf = (fabs(stpc - sx) < fabs(stpq - sx)) ? stpc : stpc + (stpq - stpc) / 2.0;
            brackt = true;
        } else if (sgnd < 0.0) {
            infoc = 2;
            const double theta = 3.0 * (fxv - fp) / (st - sx) + dx + dp;
            const double s = mt_max(fabs(theta), mt_max(fabs(dx), fabs(dp)));
            double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
            if (st > sx) gamma = -gamma;
            const double p = (gamma - dp) + theta, q = ((gamma - dp) + gamma) + dx;
            stpc = st + (p / q) * (sx - st);
            stpq = st + (dp / (dp - dx)) * (sx - st);
            stpf = (fabs(stpc - st) > fabs(stpq - st)) ? stpc : stpq;
            brackt = true;
        } else if (fabs(dp) < fabs(dx)) {
            infoc = 3;
            bound = true;
            const double theta = 3.0 * (fxv - fp) / (st - sx) + dx + dp;
            const double s = mt_max(fabs(theta), mt_max(fabs(dx), fabs(dp)));
            double gamma = s * sqrt(mt_max(0.0, (theta / s) * (theta / s) - (dx / s) * (dp / s)));
            if (st > sx) gamma = -gamma;
            const double p = (gamma - dp) + theta, q = (gamma + (dx - dp)) + gamma;
            const double r = p / q;
            if (r < 0.0 && gamma != 0.0) stpc = st + r * (sx - st);
            else if (st > sx) stpc = stmax;
            else stpc = stmin;
            stpq = st + (dp / (dp - dx)) * (sx - st);
            if (brackt) stpf = (fabs(st - stpc) < fabs(st - stpq)) ? stpc : stpq;
            else stpf = (fabs(st - stpc) > fabs(st - stpq)) ? stpc : stpq;
        } else {
            infoc = 4;
            if (brackt) {
                const double theta = 3.0 * (fp - fyv) / (sy - st) + dy + dp;
                const double s = mt_max(fabs(theta), mt_max(fabs(dy), fabs(dp)));
                double gamma = s * sqrt((theta / s) * (theta / s) - (dy / s) * (dp / s));
                if (st > sy) gamma = -gamma;
                const double p = (gamma - dp) + theta, q = ((gamma - dp) + gamma) + dy;
                stpc = st + (p / q) * (sy - st);
                stpf = stpc;
            } else {
                stpf = (st > sx) ? stmax : stmin;
            }
        }
        if (fp > fxv) {
            sy = st; fyv = fp; dy = dp;
        } else {
            if (sgnd < 0.0) { sy = sx; fyv = fxv; dy = dx; }
            sx = st; fxv = fp; dx = dp;
        }
        stpf = mt_min(stmax, stpf);
        stpf = mt_max(stmin, stpf);
        st = stpf;
        if (brackt && bound) {
            if (sy > sx) st = mt_min(sx + 0.66 * (sy - sx), st);
            else st = mt_max(sx + 0.66 * (sy - sx), st);
        }
    }
};

} // namespace sdca
