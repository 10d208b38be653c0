// lbfgs_host.h -- L-BFGS direction coefficients in compact form (host, FP64).
//
// SuperDCA's optimiser (CppNumericalSolvers LbfgsSolver, history m = 10,
// H0 = s.y / y.y of the newest pair) applies the inverse-Hessian estimate by
// the two-loop recursion.  The engine applies the same operator through its
// compact representation (Byrd, Nocedal & Schnabel, Math. Prog. 63, 1994):
//
//   H g = gamma g + [S  gamma Y] [[R^-T (D + gamma Y^T Y) R^-1, -R^-T],
//                                 [-R^-1,                       0  ]] [S^T g; gamma Y^T g]
//
// with R = upper triangle of S^T Y (diagonal D).  Mathematically identical to
// the two-loop recursion; it needs only the dot products S^T g, Y^T g and the
// small Gram matrices, so the device reads the history twice per iteration
// (dots, then the direction) instead of 4m times.  The same code runs on the
// host (tensor-core and plain forms) and on the device (the dual form's
// control kernel).
#pragma once

#ifdef __CUDACC__
#define SDCA_HD_L __host__ __device__
#else
#define SDCA_HD_L
#endif

namespace sdca {

// k pairs, oldest first.  R: k x k row-major, R[a*k+b] = s_a . y_b for a <= b.
// YY: k x k, YY[a*k+b] = y_a . y_b.  sg[a] = s_a . g, yg[a] = y_a . g.
// Output d = coef_g g + sum_a coefS[a] s_a + coefY[a] y_a  (= -H g).
// Returns false if R is singular.
SDCA_HD_L inline bool lbfgs_compact_coeffs(int k, const double *R, const double *YY, const double *sg,
                                 const double *yg, double gamma, double *coef_g, double *coefS,
                                 double *coefY)
{
    double t[32], w[32], p[32];
    if (k > 32) return false;
    *coef_g = -gamma;
    // t = R^-1 sg (back substitution)
    for (int a = k - 1; a >= 0; --a) {
        double v = sg[a];
        for (int b = a + 1; b < k; ++b) v -= R[a * k + b] * t[b];
        const double diag = R[a * k + a];
        if (!(diag != 0.0)) return false;
        t[a] = v / diag;
    }
    // w = (D + gamma YY) t - gamma yg
    for (int a = 0; a < k; ++a) {
        double v = R[a * k + a] * t[a];
        for (int b = 0; b < k; ++b) v += gamma * YY[a * k + b] * t[b];
        w[a] = v - gamma * yg[a];
    }
    // p = R^-T w (forward substitution)
    for (int a = 0; a < k; ++a) {
        double v = w[a];
        for (int b = 0; b < a; ++b) v -= R[b * k + a] * p[b];
        p[a] = v / R[a * k + a];
    }
    for (int a = 0; a < k; ++a) {
        coefS[a] = -p[a];
        coefY[a] = gamma * t[a];
    }
    return true;
}

} // namespace sdca
