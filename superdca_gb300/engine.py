"""Host-side mirror of SuperDCA's solve boundary over the engine's C ABI.

SuperDCA runs its per-locus solve as
    run_plmDCA<double, triallelic_state_t>(alignments, loci_list)
(SuperDCA/include/plmDCA.hpp:436-437), configured through plmDCA_options
(--lambda-h, --lambda-J, --gradient-threshold; SuperDCA/src/plmDCA_options.cpp)
and writing its results to files.  `Engine` takes the same inputs (encoded
alignment, weights, loci list, option values) and returns the per-locus score
rows and statistics; `run_plmDCA` adds the symmetrised coupling lines that
SuperDCA writes (plmDCA.hpp:667-693).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import EngineError


def _ptr(a):
    return None if a is None else a.ctypes.data


@dataclass
class SolveResult:
    scores: np.ndarray       # n_loci x L float32, NaN on the diagonal
    f: np.ndarray            # objective per locus
    gnorm: np.ndarray        # gradient max-norm per locus
    iterations: np.ndarray
    nfeval: np.ndarray       # evaluations counted as SuperDCA counts them
    contractions: np.ndarray
    status: np.ndarray
    x: np.ndarray | None = None  # solutions, reference layout
    restarts: np.ndarray | None = None
    skipped_pairs: np.ndarray | None = None
    weak_searches: np.ndarray | None = None
    max_trials: np.ndarray | None = None


class Engine:
    """One alignment resident on one GPU; solves batches of target loci.

    batch: loci solved together per solver lane (slots).  lanes: solver
    lanes, each with its own slots, CUDA stream and host thread; they share
    the resident alignment and take loci from one queue, so one lane's host
    decisions overlap the other lanes' kernels.  form: FORM_GATHER (plain),
    FORM_TC (tensor-core contractions) or FORM_DUAL (the span of the
    sequences; zero start, or the per-sequence learned start of a version-2
    blob)."""

    def __init__(self, n_seqs: int, n_loci: int, *, lambda_h: float = -1.0,
                 lambda_J: float = -1.0, gradient_threshold: float = 1e-3,
                 max_iterations: int = 2000, history: int = 10, batch: int = 64,
                 form: int = _lib.FORM_GATHER, history_bf16: bool = False, gap_state: int = 3,
                 device: int = 0, stream: int | None = None, lanes: int = 1):
        self.lib = _lib.load()
        cfg = _lib.Config()
        self.lib.sdca_config_default(C.byref(cfg))
        cfg.n_seqs, cfg.n_loci = int(n_seqs), int(n_loci)
        cfg.lambda_h, cfg.lambda_J = float(lambda_h), float(lambda_J)
        cfg.gradient_threshold = float(gradient_threshold)
        cfg.max_iterations, cfg.history, cfg.batch = int(max_iterations), int(history), int(batch)
        cfg.form = int(form)
        cfg.flags = _lib.FLAG_HISTORY_BF16 if history_bf16 else 0
        cfg.gap_state, cfg.device = int(gap_state), int(device)
        cfg.stream = stream
        cfg.lanes = int(lanes)
        self.cfg = cfg
        h = C.c_void_p()
        rc = self.lib.sdca_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise EngineError(rc, self.lib.sdca_last_error(None).decode())
        self.h = h
        self.N, self.L = int(n_seqs), int(n_loci)
        self.D = 16 * self.L + 4

    def _check(self, rc):
        if rc != 0:
            raise EngineError(rc, self.lib.sdca_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.sdca_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_alignment(self, states: np.ndarray, weights: np.ndarray):
        self._states = np.ascontiguousarray(states, dtype=np.uint8)
        self._weights = np.ascontiguousarray(weights, dtype=np.float64)
        assert self._states.shape == (self.N, self.L) and self._weights.shape == (self.N,)
        self._check(self.lib.sdca_set_alignment(self.h, _ptr(self._states), _ptr(self._weights)))

    def compute_weights(self, states: np.ndarray, threshold: float = 0.9, mult=None) -> np.ndarray:
        """SuperDCA's sequence weights computed on the GPU (calculate_weights,
        SuperDCA/include/plmDCA_optimizer_parameters.hpp:39-98).  Leaves the
        handle without an alignment: call set_alignment afterwards."""
        st = np.ascontiguousarray(states, dtype=np.uint8)
        assert st.shape == (self.N, self.L)
        m = None if mult is None else np.ascontiguousarray(mult, dtype=np.float64)
        w = np.zeros(self.N, dtype=np.float64)
        self._check(self.lib.sdca_compute_weights(self.h, _ptr(st), _ptr(m), float(threshold), _ptr(w)))
        return w

    def lambdas(self):
        lh, lJ, be = C.c_double(), C.c_double(), C.c_double()
        self._check(self.lib.sdca_get_lambdas(self.h, C.byref(lh), C.byref(lJ), C.byref(be)))
        return lh.value, lJ.value, be.value

    def solve(self, loci, x_init=None, want_x=False, want_scores=True, x_positions=None) -> SolveResult:
        """Solve the listed target loci.  want_x: the solution of every locus
        (n x D doubles); x_positions: solutions of the loci at these list
        positions only (result.x row j belongs to loci[x_positions[j]])."""
        loci = np.ascontiguousarray(loci, dtype=np.uint32)
        n = len(loci)
        scores = np.zeros((n, self.L), dtype=np.float32) if want_scores else None
        stats = (_lib.LocusStat * max(n, 1))()
        xi = None if x_init is None else np.ascontiguousarray(x_init, dtype=np.float64)
        if x_positions is not None:
            pos = np.asarray(x_positions, dtype=np.int64)
            rows = np.full(n, -1, dtype=np.int64)
            rows[pos] = np.arange(len(pos))
            xo = np.zeros((len(pos), self.D), dtype=np.float64)
            self._check(self.lib.sdca_solve_sel(self.h, _ptr(loci), n, _ptr(xi), _ptr(rows), _ptr(xo),
                                                _ptr(scores), C.cast(stats, C.c_void_p)))
        else:
            xo = np.zeros((n, self.D), dtype=np.float64) if want_x else None
            self._check(self.lib.sdca_solve_ex(self.h, _ptr(loci), n, _ptr(xi), _ptr(xo), _ptr(scores),
                                               C.cast(stats, C.c_void_p)))
        st = stats[:n]
        return SolveResult(
            scores=scores,
            f=np.array([s.f for s in st]), gnorm=np.array([s.gnorm for s in st]),
            iterations=np.array([s.iterations for s in st]),
            nfeval=np.array([s.nfeval for s in st]),
            contractions=np.array([s.contractions for s in st]),
            status=np.array([s.status for s in st]), x=xo,
            restarts=np.array([s.restarts for s in st]),
            skipped_pairs=np.array([s.skipped_pairs for s in st]),
            weak_searches=np.array([s.weak_searches for s in st]),
            max_trials=np.array([s.max_trials for s in st]))

    def set_targets(self, targets):
        """Two-alignment scan mode: solve the columns of `targets` (N x LT codes,
        the same sequences) against every locus of the alignment; loci of
        later solves index target columns.  None returns to the usual mode."""
        if targets is None:
            self._targets = None
            self._check(self.lib.sdca_set_targets(self.h, None, 0))
            return
        self._targets = np.ascontiguousarray(targets, dtype=np.uint8)
        assert self._targets.shape[0] == self.N
        self._check(self.lib.sdca_set_targets(self.h, _ptr(self._targets), self._targets.shape[1]))

    def set_warm_start(self, blob):
        """Start later solves (without x_init) from the learned warm start
        given by a parameter blob (superdca_gb300.warmstart); None disables."""
        if blob is None:
            self._ws_blob = None
            self._check(self.lib.sdca_set_warm_start(self.h, None, 0))
            return
        self._ws_blob = np.ascontiguousarray(blob, dtype=np.float32)
        self._check(self.lib.sdca_set_warm_start(self.h, _ptr(self._ws_blob), self._ws_blob.size))

    def ws_features(self, loci, k: int, eps: float, sel=None) -> np.ndarray:
        """Pair statistics of the warm start for target loci: n x L x 40, or
        n x P x 40 for the pairs sel (n x P locus indices)."""
        loci = np.ascontiguousarray(loci, dtype=np.uint32)
        n = len(loci)
        if sel is None:
            out = np.zeros((n, self.L, 40), dtype=np.float32)
            self._check(self.lib.sdca_ws_features(self.h, int(k), float(eps), _ptr(loci), n, None, 0, _ptr(out)))
            return out
        sel = np.ascontiguousarray(sel, dtype=np.uint32)
        assert sel.shape[0] == n
        out = np.zeros((n, sel.shape[1], 40), dtype=np.float32)
        self._check(self.lib.sdca_ws_features(self.h, int(k), float(eps), _ptr(loci), n, _ptr(sel), sel.shape[1],
                                              _ptr(out)))
        return out

    def ws_dual_data(self, loci):
        """Training data of the dual form's per-sequence start: statistics
        (n x N x 40) and converged residual rows w_i (p_i - onehot) (n x N x 4)
        of the listed loci, with their solve statistics (sdca_ws_dual_data)."""
        loci = np.ascontiguousarray(loci, dtype=np.uint32)
        n = len(loci)
        feats = np.zeros((n, self.N, 40), dtype=np.float32)
        rho = np.zeros((n, self.N, 4), dtype=np.float32)
        stats = (_lib.LocusStat * max(n, 1))()
        self._check(self.lib.sdca_ws_dual_data(self.h, _ptr(loci), n, _ptr(feats), _ptr(rho),
                                               C.cast(stats, C.c_void_p)))
        st = stats[:n]
        return feats, rho, dict(f=np.array([s.f for s in st]), iterations=np.array([s.iterations for s in st]),
                                status=np.array([s.status for s in st]))

    def eval(self, r: int, x: np.ndarray, grad: bool = True):
        x = np.ascontiguousarray(x, dtype=np.float64)
        f = C.c_double()
        g = np.zeros(self.D) if grad else None
        self._check(self.lib.sdca_eval(self.h, int(r), _ptr(x), C.byref(f), _ptr(g)))
        return (f.value, g) if grad else f.value

    def profile(self) -> dict:
        p = _lib.Profile()
        self._check(self.lib.sdca_get_profile(self.h, C.byref(p)))
        return dict(solve_ms=p.solve_ms,
                    kernel_ms={k: p.kernel_ms[i] for i, k in enumerate(_lib.KERNEL_CLASSES)},
                    kernel_launches={k: p.kernel_launches[i] for i, k in enumerate(_lib.KERNEL_CLASSES)},
                    kernel_units={k: p.kernel_units[i] for i, k in enumerate(_lib.KERNEL_CLASSES)},
                    gpu_launches=p.gpu_launches, iterations=p.iterations, contractions=p.contractions,
                    h2d_bytes=p.h2d_bytes, d2h_bytes=p.d2h_bytes)


@dataclass
class TuneResult:
    batch: int               # chosen slots per lane
    lanes: int               # chosen solver lanes
    n_done: int              # leading loci of the list solved by the probes
    scores: np.ndarray | None  # their score rows (n_done x L)
    stats: list              # their per-locus statistics (dicts)
    entries: list            # per candidate: batch, lanes, n_loci, status, device_ms, iterations_per_s
    cached: bool             # the choice came from the cache file (no probe ran)


def autotune(states: np.ndarray, weights: np.ndarray, loci, *, form: int = _lib.FORM_DUAL,
             max_fraction: float = 0.25, cache_path: str | None = None, device: int = 0,
             lambda_h: float = -1.0, lambda_J: float = -1.0, gradient_threshold: float = 1e-3,
             want_scores: bool = True) -> TuneResult:
    """Choose batch and lanes for this alignment shape by solving the first
    loci of `loci` with candidate configurations (sdca_autotune).  The probe
    loci are solved for real: result.scores / result.stats hold their rows
    and statistics; continue with loci[result.n_done:] on an Engine built
    with result.batch and result.lanes."""
    lib = _lib.load()
    st = np.ascontiguousarray(states, dtype=np.uint8)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    loci = np.ascontiguousarray(loci, dtype=np.uint32)
    N, L = st.shape
    cfg = _lib.Config()
    lib.sdca_config_default(C.byref(cfg))
    cfg.n_seqs, cfg.n_loci = N, L
    cfg.lambda_h, cfg.lambda_J, cfg.gradient_threshold = float(lambda_h), float(lambda_J), float(gradient_threshold)
    cfg.form, cfg.device = int(form), int(device)
    n = len(loci)
    budget = int(max_fraction * n)
    scores = np.zeros((budget, L), dtype=np.float32) if want_scores and budget > 0 else None
    sc_full = None
    if scores is not None:
        # the library writes rows by list position; the probes stay within the budget
        sc_full = scores
    stats = (_lib.LocusStat * max(budget, 1))()
    best = _lib.Config()
    done = C.c_size_t()
    ents = (_lib.TuneEntry * _lib.TUNE_MAX_ENTRIES)()
    nent = C.c_int32()
    rc = lib.sdca_autotune(C.byref(cfg), _ptr(st), _ptr(w), _ptr(loci), min(n, budget if budget > 0 else 0),
                           1.0 if budget > 0 else 0.0,
                           None if cache_path is None else cache_path.encode(), _ptr(sc_full),
                           C.cast(stats, C.c_void_p), C.byref(done), C.byref(best), C.cast(ents, C.c_void_p),
                           C.byref(nent))
    if rc != 0:
        raise EngineError(rc, lib.sdca_last_error(None).decode())
    nd = int(done.value)
    st_list = [dict(f=s.f, gnorm=s.gnorm, iterations=s.iterations, nfeval=s.nfeval, status=s.status)
               for s in stats[:nd]]
    entries = [dict(batch=e.batch, lanes=e.lanes, n_loci=e.n_loci, status=e.status, device_ms=e.device_ms,
                    iterations_per_s=e.iterations_per_s) for e in ents[:nent.value]]
    return TuneResult(batch=best.batch, lanes=best.lanes, n_done=nd,
                      scores=None if scores is None else scores[:nd], stats=st_list, entries=entries,
                      cached=nent.value == 0)


def coupling_lines(scores: np.ndarray, loci, translation=None, base: int = 1):
    """The lines SuperDCA writes for mean-of-norms scoring
    (SuperDCA/include/plmDCA.hpp:667-693): for each r in the loci list and each
    n before it, ((float)(S[r][n] + S[n][r])) * 0.5 with 1-based original
    column indices."""
    loci = [int(v) for v in loci]
    pos = {r: k for k, r in enumerate(loci)}
    tr = (lambda v: v) if translation is None else (lambda v: int(translation[v]))
    out = []
    for k, r in enumerate(loci):
        for n in loci[:k]:
            a = np.float32(scores[k, n])
            b = np.float32(scores[pos[n], r])
            out.append((float(np.float32(a + b)) * 0.5, tr(r) + base, tr(n) + base))
    return out


def format_coupling_lines(lines) -> str:
    """Text as SuperDCA streams it: std::fixed, precision 8, space separated."""
    return "".join(f"{v:.8f} {r} {n}\n" for v, r, n in lines)
