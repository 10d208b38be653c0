"""The learned warm starts: training data, training and parameter blobs.

SuperDCA starts every per-locus solve from zero (SuperDCA/include/plmDCA.hpp:
298).  Here a per-pair MLP (csrc/mlp.cu), trained on the GPU on this engine's
own converged solves, gives an initial coupling block J_rn for every pair
from the pair's statistics (csrc/warmstart.cu); the engine starts h from 0
(or fits it with J fixed) and runs the same L-BFGS.  The optimum of each
locus is unique, so
the warm start changes the iterations, not the result.

Training targets are converged blocks in natural units:
    t[s][a] = J*_rn[s][a] * 2 lambda_J / B_eff / out_scale[s*4+a].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import EngineError

N_IN, N_H, N_OUT = 40, 128, 16
VERSION = 1
IN_MEAN, IN_SCALE = 4, 4 + N_IN
W1 = IN_SCALE + N_IN
B1 = W1 + N_H * N_IN
W2 = B1 + N_H
B2 = W2 + N_H * N_H
W3 = B2 + N_H
B3 = W3 + N_OUT * N_H
TRAIN_END = B3 + N_OUT
OUT_SCALE = TRAIN_END
SIZE = OUT_SCALE + N_OUT


def ref_layout_index(L: int) -> np.ndarray:
    """I[n, s, a]: position of J_r[n][s][a] in SuperDCA's parameter vector
    (16-locus blocks, STATES order: Coupling_matrix_view.hpp:59-111,
    Matrix_kernel_access_order.hpp:28-34)."""
    n = np.arange(L)[:, None, None]
    s = np.arange(4)[None, :, None]
    a = np.arange(4)[None, None, :]
    b, p = n // 16, n % 16
    e = np.where(b < L // 16, 16, L % 16)
    return b * 256 + (s * e + p) * 4 + a


def new_blob(X: np.ndarray, J_nat: np.ndarray, k: int = 3, eps: float = 0.5, seed: int = 0,
             fit_h: bool = False) -> np.ndarray:
    """A fresh parameter blob: normalisation from the training inputs X (M x
    40) and natural-unit targets J_nat (M x 16), He-initialised weights.
    fit_h: fit h to the predicted J instead of starting from h = 0 (on the
    tree workloads h = 0 needed fewer iterations)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(SIZE, dtype=np.float32)
    p[0], p[1], p[2], p[3] = VERSION, k, eps, 1.0 if fit_h else 0.0
    mu = X.mean(0)
    sd = X.std(0)
    p[IN_MEAN:IN_MEAN + N_IN] = mu
    p[IN_SCALE:IN_SCALE + N_IN] = 1.0 / np.maximum(sd, 1e-6)
    p[W1:B1] = rng.normal(0, np.sqrt(2.0 / N_IN), N_H * N_IN)
    p[W2:B2] = rng.normal(0, np.sqrt(2.0 / N_H), N_H * N_H)
    p[W3:B3] = rng.normal(0, np.sqrt(1.0 / N_H), N_OUT * N_H)
    p[OUT_SCALE:] = np.maximum(J_nat.std(0), 1e-12)
    return p


def targets(blob: np.ndarray, J_nat: np.ndarray) -> np.ndarray:
    return (J_nat / blob[OUT_SCALE:][None, :]).astype(np.float32)


def collect(engine, loci, pairs: int, rng, k: int = 3, eps: float = 0.5):
    """Training pairs from converged solves of `loci` on `engine` (alignment
    set): inputs M x 40, natural-unit targets M x 16, solve statistics."""
    loci = np.asarray(loci)
    L = engine.L
    res = engine.solve(loci, want_x=True, want_scores=False)
    sel = np.empty((len(loci), pairs), dtype=np.int64)
    for i, r in enumerate(loci):
        cand = rng.choice(L - 1, size=min(pairs, L - 1), replace=pairs > L - 1)
        sel[i] = cand + (cand >= r)          # skip n = r
    X = engine.ws_features(loci, k, eps, sel).reshape(-1, N_IN)
    lh, lJ, beff = engine.lambdas()
    I = ref_layout_index(L)
    J = np.stack([res.x[i][I[sel[i]]].reshape(pairs, 16) for i in range(len(loci))])
    return X, (J * (2.0 * lJ / beff)).reshape(-1, N_OUT).astype(np.float32), res


def train(blob: np.ndarray, X: np.ndarray, T: np.ndarray, epochs: int = 20, batch: int = 4096,
          lr: float = 1e-3, seed: int = 0):
    """Adam on the GPU (csrc/mlp.cu); returns (new blob, loss per epoch)."""
    lib = _lib.load()
    p = np.ascontiguousarray(blob, dtype=np.float32).copy()
    X = np.ascontiguousarray(X, dtype=np.float32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    losses = np.zeros(epochs, dtype=np.float64)
    rc = lib.sdca_mlp_train(p.ctypes.data, X.ctypes.data, T.ctypes.data, len(X), epochs, batch, lr, seed,
                            losses.ctypes.data)
    if rc != 0:
        raise EngineError(rc, lib.sdca_mlp_last_error().decode())
    return p, losses


def grad(blob: np.ndarray, X: np.ndarray, T: np.ndarray):
    """Loss and gradient (blob layout) on the GPU."""
    lib = _lib.load()
    p = np.ascontiguousarray(blob, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    g = np.zeros(SIZE, dtype=np.float32)
    loss = C.c_double()
    rc = lib.sdca_mlp_grad(p.ctypes.data, X.ctypes.data, T.ctypes.data, len(X), C.byref(loss), g.ctypes.data)
    if rc != 0:
        raise EngineError(rc, lib.sdca_mlp_last_error().decode())
    return loss.value, g


def predict(blob: np.ndarray, X: np.ndarray) -> np.ndarray:
    lib = _lib.load()
    p = np.ascontiguousarray(blob, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    out = np.zeros((len(X), N_OUT), dtype=np.float32)
    rc = lib.sdca_mlp_predict(p.ctypes.data, X.ctypes.data, len(X), out.ctypes.data)
    if rc != 0:
        raise EngineError(rc, lib.sdca_mlp_last_error().decode())
    return out


def load(path: str) -> np.ndarray:
    blob = np.load(path).astype(np.float32)
    if blob.shape != (SIZE,) or int(blob[0]) not in (VERSION, VERSION_DUAL):
        raise ValueError(f"{path} is not a warm-start parameter blob")
    return blob


# ---- the dual form's per-sequence start (blob version 2)
#
# Inputs per (locus, sequence): the 28 statistics of sdca_ws_dual_data
# (padded to 40); targets: the converged residual p_i - onehot(s_i(r)) (4
# outputs; the other 12 are trained to 0).  The start is a0 = -alpha w_i
# (predicted residual) / (2 lambda_J).

VERSION_DUAL = 2
DUAL_K = 16


def new_blob_dual(X: np.ndarray, T4: np.ndarray, alpha: float, seed: int = 0) -> np.ndarray:
    """A fresh version-2 blob: normalisation from the inputs X (M x 40),
    output scale from the residual targets T4 (M x 4)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(SIZE, dtype=np.float32)
    p[0], p[1], p[2], p[3] = VERSION_DUAL, DUAL_K, alpha, 0.0
    p[IN_MEAN:IN_MEAN + N_IN] = X.mean(0)
    p[IN_SCALE:IN_SCALE + N_IN] = 1.0 / np.maximum(X.std(0), 1e-6)
    p[W1:B1] = rng.normal(0, np.sqrt(2.0 / N_IN), N_H * N_IN)
    p[W2:B2] = rng.normal(0, np.sqrt(2.0 / N_H), N_H * N_H)
    p[W3:B3] = rng.normal(0, np.sqrt(1.0 / N_H), N_OUT * N_H)
    p[OUT_SCALE:] = 1.0
    p[OUT_SCALE:OUT_SCALE + 4] = np.maximum(T4.std(0), 1e-6)
    return p


def dual_rows(engine, loci, weights, rows_per_locus: int = 0, rng=None, chunk: int = 1000):
    """Training rows from converged solves of `loci` on a dual-form engine:
    statistics (M x 40) and residual targets p - onehot (M x 4) of the
    sequences with a positive weight (rows_per_locus > 0: that many of them
    at random per locus), and the loci's solve statistics.  The loci are
    solved in chunks so that host memory stays bounded."""
    w = np.asarray(weights, dtype=np.float32)
    live = np.flatnonzero(w > 0)
    rng = rng or np.random.default_rng(0)
    Xs, Ts, sts = [], [], []
    loci = np.asarray(loci)
    for c0 in range(0, len(loci), chunk):
        feats, rho, st = engine.ws_dual_data(loci[c0:c0 + chunk])
        for j in range(len(feats)):
            rows = live if rows_per_locus <= 0 or rows_per_locus >= len(live) else \
                np.sort(rng.choice(live, rows_per_locus, replace=False))
            Xs.append(feats[j, rows])
            Ts.append(rho[j, rows] / w[rows, None])
        sts.append(st)
    st = {k: np.concatenate([s[k] for s in sts]) for k in sts[0]}
    return np.concatenate(Xs).astype(np.float32), np.concatenate(Ts).astype(np.float32), st


def train_dual(X: np.ndarray, T4: np.ndarray, alpha: float, epochs: int = 15, batch: int = 8192,
               lr: float = 1e-3, seed: int = 0):
    """Train a version-2 blob on the GPU (the project's MLP kernels, csrc/mlp.cu)."""
    blob = new_blob_dual(X, T4, alpha, seed=seed)
    T = np.zeros((len(X), N_OUT), dtype=np.float32)
    T[:, :4] = T4 / blob[OUT_SCALE:OUT_SCALE + 4][None, :]
    return train(blob, X, T, epochs=epochs, batch=batch, lr=lr, seed=seed)


def train_dual_on_workload(name: str, seeds, loci_per_seed: int, *, alpha: float = 0.4, epochs: int = 15,
                           lr: float = 1e-3, sizes: dict | None = None, batch_slots: int = 256,
                           rows_per_locus: int = 0, log=print):
    """Train the dual form's start on converged solves of synthetic
    alignments (workload `name` at the given seeds), unit weights."""
    from . import synthetic
    from .engine import Engine

    rng = np.random.default_rng(4321)
    Xs, Ts = [], []
    for seed in seeds:
        states, _, _ = synthetic.workload(name, seed=seed, **(sizes or {}))
        N, L = states.shape
        w = np.ones(N)
        with Engine(N, L, form=_lib.FORM_DUAL, batch=batch_slots) as E:
            E.set_alignment(states, w)
            loci = rng.choice(L, size=min(loci_per_seed, L), replace=False)
            X, T4, st = dual_rows(E, loci, w, rows_per_locus, rng)
        log(f"seed {seed}: {N} x {L}, {len(loci)} loci solved, median iterations {np.median(st['iterations']):.0f}")
        Xs.append(X)
        Ts.append(T4)
    X = np.concatenate(Xs)
    T4 = np.concatenate(Ts)
    blob, losses = train_dual(X, T4, alpha, epochs=epochs, lr=lr)
    log(f"trained on {len(X)} sequence rows: loss {losses[0]:.4f} -> {losses[-1]:.4f}")
    return blob, losses


def train_on_workload(name: str, seeds, loci_per_seed: int, pairs: int, *, epochs: int = 20, batch: int = 4096,
                      lr: float = 1e-3, k: int = 3, eps: float = 0.5, form: int = _lib.FORM_TC, batch_slots: int = 64,
                      sizes: dict | None = None, log=print):
    """Train a blob on converged solves of synthetic alignments (workload
    `name` of superdca_gb300.synthetic at the given seeds, with `sizes`
    overriding its generator arguments), unit weights."""
    from . import synthetic
    from .engine import Engine

    rng = np.random.default_rng(1234)
    Xs, Js = [], []
    for seed in seeds:
        states, _, _ = synthetic.workload(name, seed=seed, **(sizes or {}))
        N, L = states.shape
        with Engine(N, L, form=form, batch=batch_slots) as E:
            E.set_alignment(states, np.ones(N))
            loci = rng.choice(L, size=min(loci_per_seed, L), replace=False)
            X, J, res = collect(E, loci, pairs, rng, k, eps)
        log(f"seed {seed}: {N} x {L}, {len(loci)} loci solved, median iterations {np.median(res.iterations):.0f}")
        Xs.append(X)
        Js.append(J)
    X = np.concatenate(Xs)
    J = np.concatenate(Js)
    blob = new_blob(X, J, k=k, eps=eps)
    blob, losses = train(blob, X, targets(blob, J), epochs=epochs, batch=batch, lr=lr)
    log(f"trained on {len(X)} pairs: loss {losses[0]:.4f} -> {losses[-1]:.4f}")
    return blob, losses


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description="Train the learned warm start on synthetic workloads.")
    ap.add_argument("--workload", default="tree-3000x94000")
    ap.add_argument("--N", type=int, default=None, help="override the workload's sequence count")
    ap.add_argument("--L", type=int, default=None, help="override the workload's locus count")
    ap.add_argument("--seeds", type=int, nargs="+", default=[1, 2])
    ap.add_argument("--loci", type=int, default=256, help="solved loci per seed")
    ap.add_argument("--pairs", type=int, default=2048, help="training pairs per solved locus")
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--dual", action="store_true", help="the dual form's per-sequence start (version 2)")
    ap.add_argument("--alpha", type=float, default=0.4, help="dual: shrinkage of the predicted residuals")
    ap.add_argument("--rows-per-locus", type=int, default=0, help="dual: sequences sampled per locus (0: all)")
    ap.add_argument("--batch-slots", type=int, default=0,
                    help="slots of the engine that solves the training loci (default: 256 dual, 64 otherwise)")
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    sizes = {k: v for k, v in (("N", a.N), ("L", a.L)) if v is not None}
    if a.dual:
        blob, _ = train_dual_on_workload(a.workload, a.seeds, a.loci, alpha=a.alpha, epochs=a.epochs, lr=a.lr,
                                         sizes=sizes, rows_per_locus=a.rows_per_locus,
                                         batch_slots=a.batch_slots or 256)
    else:
        blob, _ = train_on_workload(a.workload, a.seeds, a.loci, a.pairs, epochs=a.epochs, lr=a.lr, sizes=sizes,
                                    batch_slots=a.batch_slots or 64)
    np.save(a.out, blob)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
