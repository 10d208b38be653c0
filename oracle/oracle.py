"""ctypes front end of the FP64 CPU oracle (oracle/liborc_plmdca.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py, as the checker or the timed
CPU baseline.  The product path (superdca_gb300) never imports this module.

The reference-layout parameter vector (D = q*q*L + q doubles) is described in
oracle/plmdca_oracle.h.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc_plmdca.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_plmdca.so")

_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


class OrcProblem(C.Structure):
    _fields_ = [("states", C.c_void_p), ("weights", C.c_void_p), ("N", C.c_int64),
                ("L", C.c_int64), ("q", C.c_int), ("lambda_h", C.c_double),
                ("lambda_J", C.c_double), ("targets", C.c_void_p), ("LT", C.c_int64)]


class OrcStat(C.Structure):
    _fields_ = [("iterations", C.c_int64), ("nfeval", C.c_int64), ("f", C.c_double),
                ("gnorm_inf", C.c_double), ("status", C.c_int)]


def build(quiet: bool = True) -> None:
    """Compile the C oracle with its Makefile (gcc; portable C11)."""
    out = subprocess.run(["make", "-C", HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_dim.restype = C.c_int64
        L.orc_dim.argtypes = [C.c_int64, C.c_int]
        L.orc_objective.restype = C.c_double
        L.orc_objective.argtypes = [C.POINTER(OrcProblem), C.c_int64, _f64p, C.c_void_p]
        L.orc_lambdas.argtypes = [_f64p, C.c_int64, C.c_double, C.c_double,
                                  C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]
        L.orc_weights.restype = C.c_int64
        L.orc_weights.argtypes = [_u8p, C.c_int64, C.c_int64, C.c_void_p, C.c_double, _f64p]
        L.orc_minimize.restype = C.c_int
        L.orc_minimize.argtypes = [C.POINTER(OrcProblem), C.c_int64, _f64p, C.c_int,
                                   C.c_double, C.c_int, C.POINTER(OrcStat)]
        L.orc_score_row.argtypes = [_f64p, C.c_int64, C.c_int, C.c_int64, C.c_int, _f32p]
        L.orc_solve.restype = C.c_int
        L.orc_solve.argtypes = [C.POINTER(OrcProblem), _i64p, C.c_int64, C.c_int, C.c_int,
                                C.c_double, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p]
        L.orc_eval_many.restype = C.c_int
        L.orc_eval_many.argtypes = [C.POINTER(OrcProblem), _i64p, C.c_int64, C.c_int, _f64p,
                                    C.c_void_p]
        _lib = L
    return _lib


def dim(L: int, q: int = 4) -> int:
    return q * q * L + q


def ref_index(L: int, q: int = 4):
    """Index array I[n, s, a] -> position of J_r[n][s][a] in the reference layout."""
    n = np.arange(L)[:, None, None]
    s = np.arange(q)[None, :, None]
    a = np.arange(q)[None, None, :]
    b, p = n // 16, n % 16
    nfull = L // 16
    e = np.where(b < nfull, 16, L % 16)
    return b * 16 * q * q + (s * e + p) * q + a


def lambdas(weights, lambda_h_opt=-1.0, lambda_J_opt=-1.0):
    w = np.ascontiguousarray(weights, dtype=np.float64)
    lh, lJ, be = C.c_double(), C.c_double(), C.c_double()
    lib().orc_lambdas(w, len(w), lambda_h_opt, lambda_J_opt, C.byref(lh), C.byref(lJ), C.byref(be))
    return lh.value, lJ.value, be.value


def weights(states, threshold=0.9, mult=None):
    st = np.ascontiguousarray(states, dtype=np.uint8)
    N, L = st.shape
    w = np.zeros(N, dtype=np.float64)
    m = None if mult is None else np.ascontiguousarray(mult, dtype=np.float64)
    lib().orc_weights(st, N, L, None if m is None else m.ctypes.data, threshold, w)
    return w


class Problem:
    """An alignment (N x L codes 0..q-1), weights and absolute lambdas."""

    def __init__(self, states, weights, lambda_h, lambda_J, q=4, targets=None):
        """targets: N x LT target columns for the two-alignment scan mode
        (plmDCA_objective.hpp:67): locus r is targets[:, r] and every column
        of states is a feature."""
        self.states = np.ascontiguousarray(states, dtype=np.uint8)
        self.weights = np.ascontiguousarray(weights, dtype=np.float64)
        self.N, self.L = self.states.shape
        self.q = q
        self.lambda_h, self.lambda_J = float(lambda_h), float(lambda_J)
        self.targets = None if targets is None else np.ascontiguousarray(targets, dtype=np.uint8)
        LT = 0 if self.targets is None else self.targets.shape[1]
        self._c = OrcProblem(self.states.ctypes.data, self.weights.ctypes.data, self.N,
                             self.L, q, self.lambda_h, self.lambda_J,
                             None if self.targets is None else self.targets.ctypes.data, LT)

    @property
    def D(self):
        return dim(self.L, self.q)

    def objective(self, r, x, grad=True):
        x = np.ascontiguousarray(x, dtype=np.float64)
        g = np.zeros(self.D, dtype=np.float64) if grad else None
        f = lib().orc_objective(C.byref(self._c), int(r), x,
                                None if g is None else g.ctypes.data)
        return (f, g) if grad else f

    def minimize(self, r, x0=None, max_iter=2000, gtol=1e-3, m=10):
        x = np.zeros(self.D) if x0 is None else np.array(x0, dtype=np.float64)
        st = OrcStat()
        lib().orc_minimize(C.byref(self._c), int(r), x, max_iter, gtol, m, C.byref(st))
        return x, dict(iterations=st.iterations, nfeval=st.nfeval, f=st.f,
                       gnorm_inf=st.gnorm_inf, status=st.status)

    def solve(self, loci, threads=1, max_iter=2000, gtol=1e-3, m=10, gap=3, x_init=None,
              want_x=False):
        loci = np.ascontiguousarray(loci, dtype=np.int64)
        n = len(loci)
        scores = np.zeros((n, self.L), dtype=np.float32)
        stats = (OrcStat * max(n, 1))()
        xo = np.zeros((n, self.D)) if want_x else None
        xi = None if x_init is None else np.ascontiguousarray(x_init, dtype=np.float64)
        lib().orc_solve(C.byref(self._c), loci, n, threads, max_iter, gtol, m, gap,
                        None if xi is None else xi.ctypes.data, scores.ctypes.data,
                        C.cast(stats, C.c_void_p), None if xo is None else xo.ctypes.data)
        st = [dict(iterations=s.iterations, nfeval=s.nfeval, f=s.f, gnorm_inf=s.gnorm_inf,
                   status=s.status) for s in stats[:n]]
        return (scores, st, xo) if want_x else (scores, st)

    def eval_many(self, loci, x, threads=1):
        loci = np.ascontiguousarray(loci, dtype=np.int64)
        f = np.zeros(len(loci))
        lib().orc_eval_many(C.byref(self._c), loci, len(loci), threads,
                            np.ascontiguousarray(x, dtype=np.float64), f.ctypes.data)
        return f


def score_row(x, L, r, q=4, gap=3):
    row = np.zeros(L, dtype=np.float32)
    lib().orc_score_row(np.ascontiguousarray(x, dtype=np.float64), L, q, int(r), gap, row)
    return row


def symmetrize(scores_rows, loci):
    """Coupling lines (S[r][n]+S[n][r])/2 for n before r in the loci list, as
    SuperDCA/include/plmDCA.hpp:684-691 writes them (float sum, times 0.5)."""
    pos = {int(r): k for k, r in enumerate(loci)}
    out = []
    for k, r in enumerate(loci):
        for n in loci[:k]:
            a = np.float32(scores_rows[k, n])
            b = np.float32(scores_rows[pos[int(n)], r])
            out.append((float(np.float32(a + b)) * 0.5, int(r), int(n)))
    return out


# --------------------------------------------------------------------------
# SuperDCA's own headers (oracle/_ref), available only where the reference
# sources were present at build time.

_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_LIB_PATH)
        R.ref_problem_new.restype = C.c_void_p
        R.ref_problem_new.argtypes = [_u8p, C.c_int64, C.c_int64, C.c_void_p, C.c_double,
                                      C.c_double, C.c_double]
        R.ref_problem_free.argtypes = [C.c_void_p]
        R.ref_dim.restype = C.c_int64
        R.ref_dim.argtypes = [C.c_void_p]
        R.ref_lambdas.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        R.ref_weights.argtypes = [C.c_void_p, _f64p]
        R.ref_objective.restype = C.c_double
        R.ref_objective.argtypes = [C.c_void_p, C.c_int64, _f64p, C.c_void_p]
        R.ref_score_row.argtypes = [C.c_void_p, C.c_int64, _f64p, C.c_int64, _f32p]
        _ref = R
    return _ref


class RefProblem:
    """SuperDCA's parameter class, objective and scoring on one alignment."""

    def __init__(self, states, weights=None, threshold=0.9, lambda_h_opt=-1.0,
                 lambda_J_opt=-1.0):
        self.states = np.ascontiguousarray(states, dtype=np.uint8)
        self.N, self.L = self.states.shape
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        self._w = w
        self.h = ref_lib().ref_problem_new(self.states, self.N, self.L,
                                           None if w is None else w.ctypes.data, threshold,
                                           lambda_h_opt, lambda_J_opt)
        self.D = ref_lib().ref_dim(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            ref_lib().ref_problem_free(self.h)
            self.h = None

    def lambdas(self):
        lh, lJ = C.c_double(), C.c_double()
        ref_lib().ref_lambdas(self.h, C.byref(lh), C.byref(lJ))
        return lh.value, lJ.value

    def weights(self):
        w = np.zeros(self.N)
        ref_lib().ref_weights(self.h, w)
        return w

    def objective(self, r, x):
        g = np.zeros(self.D)
        f = ref_lib().ref_objective(self.h, int(r), np.ascontiguousarray(x, dtype=np.float64),
                                    g.ctypes.data)
        return f, g

    def score_row(self, r, x, gap=3):
        row = np.zeros(self.L, dtype=np.float32)
        ref_lib().ref_score_row(self.h, int(r), np.ascontiguousarray(x, dtype=np.float64), gap,
                                row)
        return row
