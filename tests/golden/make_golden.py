"""Write the golden fixtures in tests/golden from SuperDCA's own code.

Runs only where the reference sources were available to build oracle/_ref
(`make -C oracle ref`): the objective, gradient, lambda rule, sequence
weights and coupling scores below come from SuperDCA's headers compiled there
(plmDCA_objective.hpp, plmDCA_optimizer_parameters.hpp, plmDCA_utility.hpp,
Matrix_math.hpp).  Converged optima are found by an optimiser independent of
both the reference's and this project's L-BFGS (scipy L-BFGS-B, tight
tolerances) on the reference objective, so they pin the minimiser of the
strictly convex per-locus objective, not an optimiser trajectory.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def random_alignment(rng, N, L, n_dup=3):
    st = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
    # a few biased columns and duplicated / near-duplicated sequences
    for c in range(0, L, 3):
        st[:, c] = np.where(rng.random(N) < 0.8, 0, st[:, c])
    for k in range(n_dup):
        i, j = rng.integers(0, N, size=2)
        st[i] = st[j]
        if k % 2:
            st[i, rng.integers(0, L)] = rng.integers(0, 4)
    return st


def objective_cases():
    rng = np.random.default_rng(20240601)
    out = {}
    cases = [(40, 7, 0.8), (60, 16, 0.9), (80, 37, 0.9), (50, 33, 0.7), (30, 2, 0.9),
             (120, 50, 0.9)]
    for ci, (N, L, thr) in enumerate(cases):
        st = random_alignment(rng, N, L)
        R = O.RefProblem(st, threshold=thr)
        w = R.weights()
        lh, lJ = R.lambdas()
        rs = sorted(set([0, L // 2, L - 1, min(15, L - 1), min(16, L - 1)]))
        xs, fs, gs, rows = [], [], [], []
        for r in rs:
            x = rng.normal(size=R.D) * 0.2
            f, g = R.objective(r, x)
            xs.append(x); fs.append(f); gs.append(g); rows.append(R.score_row(r, x))
        out[f"obj{ci}"] = dict(states=st, threshold=np.float64(thr), weights=w, lambda_h=np.float64(lh),
                               lambda_J=np.float64(lJ), loci=np.array(rs), x=np.array(xs),
                               f=np.array(fs), g=np.array(gs), scores=np.array(rows))
    return out


def converged_cases():
    from scipy.optimize import minimize

    rng = np.random.default_rng(777)
    out = {}
    for ci, (N, L) in enumerate([(60, 20), (100, 37), (40, 5)]):
        st = random_alignment(rng, N, L)
        # planted coupling between columns 1 and 3
        st[:, 3] = np.where(rng.random(N) < 0.85, st[:, 1], st[:, 3])
        R = O.RefProblem(st, threshold=0.9)
        w = R.weights()
        lh, lJ = R.lambdas()
        rs = list(range(L)) if L <= 20 else [0, 1, 3, 17, L - 1]
        xs, fs, rows = [], [], []
        for r in rs:
            res = minimize(lambda x: R.objective(r, x), np.zeros(R.D), jac=True, method="L-BFGS-B",
                           options=dict(maxiter=20000, maxcor=30, gtol=1e-11, ftol=1e-15))
            x = res.x
            f, g = R.objective(r, x)
            assert np.abs(g).max() < 1e-5, (ci, r, np.abs(g).max())
            xs.append(x); fs.append(f); rows.append(R.score_row(r, x))
        out[f"opt{ci}"] = dict(states=st, weights=w, lambda_h=np.float64(lh), lambda_J=np.float64(lJ),
                               loci=np.array(rs), x=np.array(xs), f=np.array(fs),
                               scores=np.array(rows))
    return out


def main():
    if not O.ref_available():
        raise SystemExit("oracle/_ref is not built: run `make -C oracle ref` where the reference is present")
    for name, d in {**objective_cases(), **converged_cases()}.items():
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **d)
        print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
