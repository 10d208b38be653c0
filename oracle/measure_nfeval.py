"""Evaluations per locus of the CPU oracle on a full-size workload.

TEST/BENCH INFRASTRUCTURE.  Solves a seeded sample of target loci of the
3000 x 94,000 tree workload (unit weights, threshold 1e-3) with the FP64
oracle (full L-BFGS + More-Thuente, SuperDCA's evaluation counting) and
writes oracle/nfeval_<workload>.json.  bench.py's CPU legs time single
full-size objective evaluations on the host cores and convert that rate to
loci/s with the evaluations-per-locus measured here, because a complete CPU
solve of one locus at this size takes minutes.

    python oracle/measure_nfeval.py [--loci 8] [--threads 8]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402
from superdca_gb300 import synthetic  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="tree-3000x94000")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--loci", type=int, default=8)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    a = ap.parse_args()
    O.build()
    st, _, _ = synthetic.workload(a.workload, seed=a.seed)
    N, L = st.shape
    w = np.ones(N)
    lh, lJ, _ = O.lambdas(w)
    P = O.Problem(st, w, lh, lJ)
    rng = np.random.default_rng(1234)
    loci = np.sort(rng.choice(L, size=a.loci, replace=False))
    t0 = time.time()
    _, stats = P.solve(loci, threads=a.threads, gtol=1e-3)
    dt = time.time() - t0
    out = dict(workload=a.workload, seed=a.seed, N=int(N), L=int(L), weights="unit",
               gradient_threshold=1e-3, loci=loci.tolist(),
               nfeval=[int(s["nfeval"]) for s in stats],
               iterations=[int(s["iterations"]) for s in stats],
               status=[int(s["status"]) for s in stats], f=[float(s["f"]) for s in stats],
               threads=a.threads, wall_s=round(dt, 1))
    path = os.path.join(HERE, f"nfeval_{a.workload}.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
