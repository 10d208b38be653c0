#!/usr/bin/env python
"""Throughput of the plmDCA per-locus solve: target loci solved per second.

Workload: the seeded 3000-sequence x 94,000-locus coalescent-tree alignment
(synthetic stand-in for a genome alignment of that shape), unit sequence
weights (SuperDCA's --no-reweighting path), automatic lambdas, gradient
threshold 1e-3, learned start (--warm-start none: zero start).  A step
solves one batch of target loci to convergence (L-BFGS + More-Thuente, every
locus independent); steps take disjoint loci.  --form picks the engine
form: dual (default: the iteration kept in the span of the sequences, with
the per-sequence learned start), tc (tensor-core contractions, with the
per-pair learned start) or gather (plain).  A step's working set (alignment
282 MB, agreement digits 54 MB, per-slot solver state) is larger than the
129 MB L2, so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

--impl engine (default) prints one JSON line with:
  value       loci/s over all ranks, inputs resident in HBM, device time from
              CUDA events around each solve (max over ranks)
  e2e         the same metric through the C ABI with host buffers: each step
              uploads the alignment from pinned host memory and reads the
              score rows back
  roofline    for the kernel class with the most device time
  accuracy    the FP64 oracle's objective and max|gradient| at the engine's
              returned parameters, for a seeded sample of the first timed
              step's loci (relative objective error; SuperDCA stops at
              max|g| < 1e-3)
  vs_plain    the plain GPU form (FP32 gather contractions, zero start) timed
              on loci of the same step in the same process, and value / its
              loci/s
  warm_start_effect  the first timed step's loci solved again from zero:
              loci/s and mean iterations with and without the learned start
  cpu_baseline the FP64 C oracle on this host's cores (rank 0, N=1)
  parity_small every locus of the 200 x 500 workload solved by the engine and
              by the FP64 oracle: objective and coupling agreement, and the
              overlap of the 10,000 strongest pairs (rank 0, N=1)
--impl reference times the CPU reference path (the FP64 C oracle restating
SuperDCA's solve) on all host cores, on rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

Q = 4
METRIC = "loci/s at N=3000,L=94k: mixed+batched+warm-start vs plain GPU at <=1e-6 rel obj"
# committed learned-start blobs, trained on the GPU on converged solves of
# 3000 x 94,000 tree alignments: the dual form's per-sequence network on
# seeds 1-4 (1024 loci each), the per-pair network on seeds 1, 2; the bench
# alignment is seed 0 (held out)
WS_DEFAULT = {"dual": "warmstart_dual_tree-3000x94000.npy", "tc": "warmstart_tree-3000x94000.npy",
              "gather": "warmstart_tree-3000x94000.npy"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="tree-3000x94000")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--batch", type=int, default=0, help="slots per solver lane (default: 512 dual, 64 otherwise)")
    ap.add_argument("--lanes", type=int, default=0,
                    help="solver lanes (own stream and host thread each; default: 4 dual, 1 otherwise)")
    ap.add_argument("--loci-per-step", type=int, default=0, help="default: 2 x batch x lanes")
    ap.add_argument("--form", default="dual", choices=["gather", "tc", "dual"])
    ap.add_argument("--history-bf16", action="store_true")
    ap.add_argument("--warm-start", default="auto",
                    help="learned warm-start parameter blob ('none': zero start; 'auto': the committed blob of "
                         "the form: per-sequence for dual, per-pair otherwise)")
    ap.add_argument("--no-zero-start", action="store_true", help="skip the zero-start comparison")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form arm")
    ap.add_argument("--plain-loci", type=int, default=64, help="loci timed in the plain-form arm")
    ap.add_argument("--accuracy-sample", type=int, default=16,
                    help="loci of the first timed step checked against the FP64 oracle (0: none)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the autotuner (default when --batch/--lanes are not given: measure them on a "
                         "probe list of loci outside the timed steps)")
    ap.add_argument("--tune-loci", type=int, default=57856, help="loci the autotuner may solve as probes")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the skewed 616 x 78,700 workload measured after the headline")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the full 200 x 500 comparison with the oracle")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--cache-dir", default="", help="keep the generated alignment here between runs")
    return ap.parse_args()


def dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Clocks:
    """nvidia-smi samples of SM clock, throttle reasons and kernel occupancy
    (utilization.gpu: the share of each sample period in which at least one
    kernel ran) during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device), "-f", self.path], stdout=subprocess.DEVNULL,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        try:
            for line in open(self.path):
                p = [v.strip() for v in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
            os.unlink(self.path)
        except Exception:
            return None
        if not rows:
            return None

        def num(v):
            try:
                return float(v)
            except ValueError:
                return float("nan")

        sm = np.array([num(r[1]) for r in rows])
        mx = np.array([num(r[2]) for r in rows])
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        load = sm[sm > 0.5 * np.nanmax(sm)] if np.isfinite(sm).any() else sm
        util = np.array([num(r[9]) for r in rows if len(r) >= 10])
        util = util[np.isfinite(util)]
        return {"sm_mhz": float(np.nanmedian(load)) if len(load) else None,
                "sm_max_mhz": float(np.nanmax(mx)) if np.isfinite(mx).any() else None,
                "reasons": sorted(reasons), "samples": len(rows),
                "gpu_util_pct": {"median": float(np.median(util)), "min": float(util.min())} if len(util) else None}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def load_workload(args):
    from superdca_gb300 import synthetic

    path = None
    if args.cache_dir:
        os.makedirs(args.cache_dir, exist_ok=True)
        path = os.path.join(args.cache_dir, f"{args.workload}-seed{args.seed}.npy")
        if os.path.exists(path):
            return np.load(path)
    st, cols, _ = synthetic.workload(args.workload, seed=args.seed)
    if path:
        np.save(path, st)
    return st


# DRAM bytes per unit (one target locus through one launch) from one ncu
# capture, scaled to a launch by its units (the traffic grows with the slots):
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum --clock-control none \
#       -k regex:k_dual_direction -s 40 -c 2 python bench.py --steps 1 --warmup 0 --batch 128 --lanes 1 \
#       --loci-per-step 128 --no-cpu --no-e2e --no-plain --no-secondary --no-autotune --no-parity \
#       --accuracy-sample 0 --no-zero-start
#   dram__bytes_read.sum 542.70 MB + dram__bytes_write.sum 29.29 MB per launch of 128 slots (mean of 2)
NCU_TRAFFIC_PER_UNIT = {("tree-3000x94000", "direction"): (542.70e6 + 29.29e6) / 128}


def mean_history(iterations, m):
    """Mean live L-BFGS history length over a solve of `iterations`
    iterations: the direction of iteration i combines min(i, m) pairs."""
    it = max(1, int(iterations))
    return sum(min(i, m) for i in range(it)) / it


def roofline_dual(prof_tot, N, L, m, cls=None):
    """Roofline of the dual form's dominant kernel class.

    m: the mean live history length (mean_history).  Work per unit (one
    target locus through one launch of the class):
      forward (K rho, exact on the tensor cores): 2 N^2 (q - 1) FLOP -- the
        rows of rho sum to zero, so three of the four columns determine the
        product -- counted once (the digit expansion issues 12 fp16
        products of it on the pipe);
      backward (one-hot contraction X^T a on the tensor cores: max-norm
        checks and the final J): 2 N L q^2 FLOP, as in the other forms;
      history dots: 2k + 1 vectors of N x q doubles read (32 N bytes each);
      direction: (4k + 3) vectors read (history, g, a_x), 2 written (d),
        the k part of x read (32 N: the logits are k_x + eta_x), the
        single-precision differences u - u_y (16 N) and the base
        probabilities (16 N) written;
      line search (step trials): base probabilities, u differences, R
        (16 N each), states, w.
    With several solver lanes the classes of different lanes overlap in
    time, and a launch's duration includes the share of the GPU the other
    lanes' kernels take."""
    hbm, tflops, src = measured_peaks()
    ms, units = prof_tot["kernel_ms"], prof_tot["kernel_units"]
    if cls is None:
        cls = max(ms, key=lambda k: ms[k])
    t = ms[cls] / 1e3
    if units[cls] == 0 or t <= 0:
        return None, cls
    if cls == "forward":
        ach = 2.0 * N * N * (Q - 1) * units[cls] / t / 1e12
        return dict(bound="tensor", achieved=round(ach, 3), peak=tflops, unit="TFLOP/s", frac=round(ach / tflops, 5),
                    traffic=None, kernel="k_kdig (K rho)", issued_factor=12, peak_source=src), cls
    if cls == "backward":
        ach = 2.0 * N * L * Q * Q * units[cls] / t / 1e12
        return dict(bound="tensor", achieved=round(ach, 3), peak=tflops, unit="TFLOP/s", frac=round(ach / tflops, 5),
                    traffic=None, kernel="k_gemm (X^T a)", peak_source=src), cls
    per = {"history": (2 * m + 1) * 32 * N, "direction": ((4 * m + 3) + 2 + 1 + 1) * 32 * N,
           "linesearch": 16 * N * 3 + 9 * N}.get(cls)
    if per is None:
        return None, cls
    ach = per * units[cls] / t / 1e9
    return dict(bound="hbm", achieved=round(ach, 1), peak=hbm, unit="GB/s", frac=round(ach / hbm, 4),
                traffic=None, kernel=cls, peak_source=src), cls


def whole_solve_dual(prof_tot, N, L, m, trials, t_dev):
    """The whole timed solve against both roofs: every dual-form class's
    algorithmic HBM bytes and tensor FLOP over the timed device time.
    Per slot-iteration (one history-dot launch unit), in parts of N x q
    double-float values (32 N bytes): history dots 2k + 1; direction
    (4k + 3) + 2 + 1 + 1; accept and gradient 15.5 (x, d, K rho, rho_q, old g
    read; x, s, g, y written); quantiser 1; line search 1.5 + 9/32 per trial
    (P0, u - u_y, R written; states and weights).
    Tensor work: 2 N^2 (q - 1) per K rho unit, 2 N L q^2 per one-hot
    contraction unit (counted once, as in the class rooflines)."""
    hbm, tflops, src = measured_peaks()
    units = prof_tot["kernel_units"]
    its = units["history"]
    parts = (2 * m + 1) + (4 * m + 7) + 15.5 + 1 + trials * (1.5 + 9 / 32)
    nbytes = its * parts * 32 * N
    flop = units["forward"] * 2.0 * N * N * (Q - 1) + units["backward"] * 2.0 * N * L * Q * Q
    gbs = nbytes / t_dev / 1e9
    tf = flop / t_dev / 1e12
    return dict(hbm_bytes_per_slot_iteration=round(parts * 32 * N), slot_iterations=int(its),
                hbm_achieved_gbs=round(gbs, 1), hbm_frac=round(gbs / hbm, 4), tensor_achieved_tflops=round(tf, 2),
                tensor_frac=round(tf / tflops, 4), peak_source=src,
                how="algorithmic bytes and FLOP of every class over the timed device time (the kernels of "
                    "different lanes overlap, so the two fractions share the same seconds)")


def roofline(prof_tot, N, L, Dp, m, hist_bytes):
    """Roofline of the kernel class with the most device time.

    Work per unit (one target locus through one launch of the class):
      forward / backward contraction: 2 N L q^2 FLOP (the one-hot GEMM
        X . J or X^T . R for one locus: bound by the tensor pipe);
      history dots: (2k+2) Dp elements read, direction (2k+2) Dp read and Dp
        written, accept 3 Dp read/written + Dp history: bound by HBM, with k
        the history depth (m when full)."""
    hbm, tflops, src = measured_peaks()
    ms, units, launches = prof_tot["kernel_ms"], prof_tot["kernel_units"], prof_tot["kernel_launches"]
    cls = max(ms, key=lambda k: ms[k])
    t = ms[cls] / 1e3
    if units[cls] == 0 or t <= 0:
        return None, cls
    per_launch_units = units[cls] / max(1, launches[cls] / (2 if cls in ("forward", "backward", "accept") else 1))
    if cls in ("forward", "backward"):
        work = 2.0 * N * L * Q * Q * units[cls]
        ach = work / t / 1e12
        return dict(bound="tensor", achieved=round(ach, 3), peak=tflops, unit="TFLOP/s",
                    frac=round(ach / tflops, 5), traffic=None, kernel=cls,
                    work_per_launch=2.0 * N * L * Q * Q * per_launch_units,
                    peak_source=src), cls
    k = m
    if cls == "history":
        byts = (2 * k * hist_bytes + 2 * 4) * Dp * units[cls]
    elif cls == "direction":
        byts = (2 * k * hist_bytes + 3 * 4) * Dp * units[cls]
    elif cls == "accept":
        byts = (3 * 4 + hist_bytes) * Dp * units[cls]
    else:
        return None, cls
    ach = byts / t / 1e9
    return dict(bound="hbm", achieved=round(ach, 1), peak=hbm, unit="GB/s", frac=round(ach / hbm, 4),
                traffic=None, kernel=cls, peak_source=src), cls


def cpu_eval_rate(st, seconds, threads, seed=5):
    """Full-size FP64 objective+gradient evaluations on `threads` host
    threads (distinct loci, zero start): returns seconds per evaluation per
    thread and the number of evaluations timed."""
    from oracle import oracle as O

    O.build()
    N, L = st.shape
    w = np.ones(N)
    lh, lJ, _ = O.lambdas(w)
    P = O.Problem(st, w, lh, lJ)
    rng = np.random.default_rng(seed)
    x = np.zeros(O.dim(L))
    done, t_all = 0, 0.0
    while t_all < seconds or done == 0:
        loci = rng.choice(L, size=threads, replace=False).astype(np.int64)
        t0 = time.time()
        P.eval_many(loci, x, threads=threads)
        t_all += time.time() - t0
        done += threads
    return t_all * threads / done, done, t_all


def oracle_check(st, w, lh, lJ, loci, X, threads):
    """FP64 oracle objective and max |gradient| at each (locus, parameters)
    pair, evaluated on `threads` host threads (ctypes releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O

    O.build()
    P = O.Problem(st, w, lh, lJ)

    def one(k):
        f, g = P.objective(int(loci[k]), X[k])
        return f, float(np.abs(g).max())

    with ThreadPoolExecutor(max(1, threads)) as ex:
        out = list(ex.map(one, range(len(loci))))
    return np.array([o[0] for o in out]), np.array([o[1] for o in out])


def top_overlap(a, b, k=10000):
    """Overlap of the k strongest pairs of two coupling-line lists (same
    pairs, same order): |top_k(a) & top_k(b)| / k."""
    va = np.array([v for v, _, _ in a])
    vb = np.array([v for v, _, _ in b])
    k = min(k, len(va))
    ta = set(np.argsort(-va, kind="stable")[:k].tolist())
    tb = set(np.argsort(-vb, kind="stable")[:k].tolist())
    return len(ta & tb) / max(k, 1)


def parity_small(local, seed=0, gtol=1e-5):
    """The reference-runnable workload (200 x 500 biallelic loci with planted
    pairs, GPU reweighting) solved in full by the engine's dual form and by the
    FP64 oracle (SuperDCA's solve restated), both to max|g| < gtol: per-locus
    objective agreement, coupling agreement, and the overlap of the 10,000
    strongest pairs of the two coupling files."""
    from oracle import oracle as O
    from superdca_gb300 import Engine, FORM_DUAL, synthetic
    from superdca_gb300.engine import coupling_lines

    O.build()
    st, _, _ = synthetic.workload("independent-200x500", seed=seed)
    N, L = st.shape
    loci = np.arange(L)
    t0 = time.time()
    with Engine(N, L, batch=128, device=local, form=FORM_DUAL, gradient_threshold=gtol) as E:
        w = E.compute_weights(st, 0.9)
        E.set_alignment(st, w)
        r = E.solve(loci)
    t_gpu = time.time() - t0
    lh, lJ, _ = O.lambdas(w)
    t0 = time.time()
    osc, ost = O.Problem(st, w, lh, lJ).solve(loci, threads=os.cpu_count() or 1, gtol=gtol)
    t_cpu = time.time() - t0
    f_o = np.array([x["f"] for x in ost])
    el, ol = coupling_lines(r.scores, loci), coupling_lines(osc, loci)
    dv = np.abs(np.array([v for v, _, _ in el]) - np.array([v for v, _, _ in ol]))
    return {"workload": f"independent-200x500 seed {seed}", "N": int(N), "L": int(L), "gradient_threshold": gtol,
            "max_rel_obj_err": float(np.max(np.abs(r.f - f_o) / np.abs(f_o))),
            "max_abs_coupling_diff": float(dv.max()), "pairs": int(len(el)),
            "top10k_overlap": round(top_overlap(el, ol), 5),
            "status_counts": {str(k): int((r.status == k).sum()) for k in sorted(set(r.status.tolist()))},
            "seconds": {"engine": round(t_gpu, 2), "oracle": round(t_cpu, 2)},
            "how": ("every locus solved by the engine (dual form) and by the FP64 oracle to max|g| < gradient_threshold "
                    "with the same GPU-computed weights; coupling lines as SuperDCA writes them; top-10k: the 10,000 "
                    "strongest pairs of each file")}


def nfeval_reference(workload):
    path = os.path.join(ROOT, "oracle", f"nfeval_{workload}.json")
    with open(path) as fh:
        d = json.load(fh)
    return float(np.median(d["nfeval"])), d


def secondary_skewed(args, local, steps=3, warmup=1, seed=2):
    """The uneven-convergence workload: 616 sequences x 78,700 generated loci
    (MAF from Beta(0.5, 2), 10 % multi-allelic loci, gaps up to 15 %), GPU
    sequence weights, autotuned batch and lanes, and the distribution of
    iterations per locus.  Device time from CUDA events, as the headline."""
    from superdca_gb300 import Engine, FORM_DUAL, autotune, synthetic

    t0 = time.time()
    st, _, _ = synthetic.workload("skewed-616x78700", seed=seed)
    N, L = st.shape
    with Engine(N, L, batch=64, device=local, form=FORM_DUAL) as E0:
        w = E0.compute_weights(st, 0.9)
    order = (np.arange(L) * 7919) % L
    tr = autotune(st, w, order[L - min(36864, L // 2):], form=FORM_DUAL, max_fraction=1.0, device=local,
                  want_scores=False)
    B, lanes = (tr.batch, tr.lanes) if tr.batch > 0 else (512, 4)
    per_step = 2 * B * lanes
    iters, statuses, dev_ms = [], [], 0.0
    with Engine(N, L, batch=B, lanes=lanes, device=local, form=FORM_DUAL) as E:
        E.set_alignment(st, w)
        for s in range(warmup + steps):
            res = E.solve(order[s * per_step:(s + 1) * per_step], want_scores=True)
            if s >= warmup:
                dev_ms += E.profile()["solve_ms"]
                iters += res.iterations.tolist()
                statuses += res.status.tolist()
    it = np.array(iters)
    return {"workload": f"skewed-616x78700 seed {seed}", "N": int(N), "L": int(L), "batch": B, "lanes": lanes,
            "value": round(steps * per_step / (dev_ms / 1e3), 2), "unit": "loci/s", "steps": steps,
            "warmup": warmup, "loci_per_step": per_step, "weights": "GPU reweighting, threshold 0.9",
            "iterations": {"median": float(np.median(it)), "p10": float(np.percentile(it, 10)),
                           "p90": float(np.percentile(it, 90)), "max": int(it.max()), "min": int(it.min())},
            "status_counts": {str(k): statuses.count(k) for k in sorted(set(statuses))},
            "autotune": {"chosen": [tr.batch, tr.lanes], "probe_loci": tr.n_done,
                         "candidates": [{k: (round(v, 1) if isinstance(v, float) else v) for k, v in e.items()}
                                        for e in tr.entries]},
            "seconds": round(time.time() - t0, 1)}


def engine_arm(args):
    world, rank, local = dist()
    import torch

    if world > 1:
        import torch.distributed as tdist

        torch.cuda.set_device(local)
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from superdca_gb300 import Engine, FORM_DUAL, FORM_GATHER, FORM_TC, autotune

    st = load_workload(args)
    N, L = st.shape
    w = np.ones(N)
    form = {"tc": FORM_TC, "gather": FORM_GATHER, "dual": FORM_DUAL}[args.form]
    tune = None
    if not args.no_autotune and not args.batch and not args.lanes and args.tune_loci > 0:
        # batch and lanes measured on probe loci taken from the end of the
        # locus order the steps walk (the timed steps start at its front)
        t_tune = time.time()
        order = (np.arange(L) * 7919) % L
        probe = order[L - min(args.tune_loci, L):]
        tr = autotune(st, w, probe, form=form, max_fraction=1.0, device=local, want_scores=False)
        tune = {"chosen": [tr.batch, tr.lanes], "probe_loci": tr.n_done, "seconds": round(time.time() - t_tune, 2),
                "candidates": [{k: (round(v, 1) if isinstance(v, float) else v) for k, v in e.items()}
                               for e in tr.entries],
                "how": ("sdca_autotune: each candidate (batch, lanes) solves 2 x its slots of the probe loci; the "
                        "most L-BFGS iterations per device second wins; untimed, before the warm-up")}
        if tr.batch > 0 and tr.lanes > 0:
            args.batch, args.lanes = tr.batch, tr.lanes
    B = args.batch or (512 if args.form == "dual" else 64)
    lanes = args.lanes or (4 if args.form == "dual" else 1)
    per_step = args.loci_per_step or 2 * B * lanes   # slots refill once per step
    E = Engine(N, L, batch=B, device=local, form=form, history_bf16=args.history_bf16, lanes=lanes)
    E.set_alignment(st, w)
    ws = None if args.warm_start in ("", "none") else args.warm_start
    if ws == "auto":
        ws = os.path.join(ROOT, "superdca_gb300", WS_DEFAULT[args.form])
    if ws:
        from superdca_gb300 import warmstart
        E.set_warm_start(warmstart.load(ws))

    def loci_for(step):
        base = (step * world + rank) * per_step
        return (np.arange(base, base + per_step) * 7919) % L  # spread over the genome

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(local)

    for s in range(args.warmup):
        E.solve(loci_for(s), want_scores=True)
    keys = ["forward", "backward", "linesearch", "history", "direction", "accept", "score", "other"]
    tot = dict(kernel_ms={k: 0.0 for k in keys}, kernel_units={k: 0 for k in keys},
               kernel_launches={k: 0 for k in keys})
    launches = 0
    dev_ms = 0.0
    nfe, iters, contr, statuses = [], [], [], []
    clocks = Clocks(local)
    walls = []
    barrier()
    clocks.start()
    t0 = time.time()
    first = None
    for s in range(args.steps):
        res = E.solve(loci_for(args.warmup + s), want_scores=True)
        p = E.profile()
        if first is None:
            first = (res, p["solve_ms"])
        walls.append(time.time() - t0 - sum(walls))
        dev_ms += p["solve_ms"]
        launches += p["gpu_launches"]
        for k in keys:
            tot["kernel_ms"][k] += p["kernel_ms"][k]
            tot["kernel_units"][k] += p["kernel_units"][k]
            tot["kernel_launches"][k] += p["kernel_launches"][k]
        nfe += res.nfeval.tolist(); iters += res.iterations.tolist()
        contr += res.contractions.tolist(); statuses += res.status.tolist()
    barrier()
    wall = time.time() - t0
    clk = clocks.stop()
    t_dev = dev_ms / 1e3
    if world > 1:
        tt = torch.tensor([t_dev], dtype=torch.float64, device=f"cuda:{local}")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_dev = float(tt.item())
    total_loci = args.steps * per_step * world
    value = total_loci / t_dev

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        pinned = torch.empty((N, L), dtype=torch.uint8, pin_memory=True)
        pinned.numpy()[:] = st
        hst = pinned.numpy()
        barrier()
        t1 = time.time()
        t_up = t_sol = 0.0
        for s in range(args.steps):
            ta = time.time()
            E.set_alignment(hst, w)
            tb = time.time()
            E.solve(loci_for(args.warmup + s), want_scores=True)
            tc_ = time.time()
            t_up += tb - ta
            t_sol += tc_ - tb
        barrier()
        t_e2e = time.time() - t1
        if world > 1:
            tt = torch.tensor([t_e2e], dtype=torch.float64, device=f"cuda:{local}")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t_e2e = float(tt.item())
        e2e = dict(value=round(args.steps * per_step * world / t_e2e, 4), unit="loci/s",
                   h2d_bytes_per_step=int(N * L + 8 * N), d2h_bytes_per_step=int(per_step * L * 4 + per_step * 32),
                   upload_s_per_step=round(t_up / args.steps, 4), solve_s_per_step=round(t_sol / args.steps, 4))

    # sequence reweighting on the GPU at this size (outside the solve metric)
    rw = None
    if rank == 0:
        torch.cuda.synchronize(local)
        t_rw = time.time()
        w_gpu = E.compute_weights(st, 0.9)
        t_rw = time.time() - t_rw
        E.set_alignment(st, w)
        rw = {"seconds": round(t_rw, 4), "pairs": int(N * (N - 1) // 2),
              "pair_loci_per_s": float(N * (N - 1) / 2 * L / t_rw), "b_eff": round(float(w_gpu.sum()), 3)}

    Dp = ((16 * L + 4 + 63) // 64) * 64
    iso = None
    if args.form == "dual" and lanes > 1:
        # Launches of different lanes overlap, so their event durations
        # include the GPU share the other lanes take.  One untimed step on a
        # single lane (after the timed region) gives the isolated durations:
        # the class that dominates there is the one the roofline reports.
        E1 = Engine(N, L, batch=B, device=local, form=form, history_bf16=args.history_bf16, lanes=1)
        E1.set_alignment(st, w)
        E1.solve(loci_for(0)[:B], want_scores=True)
        E1.solve(loci_for(1)[:B], want_scores=True)
        p1 = E1.profile()
        E1.close()
        iso = {k: p1[k] for k in ("kernel_ms", "kernel_units", "kernel_launches")}
    if args.form == "dual":
        dom_cls = max(iso["kernel_ms"], key=lambda k: iso["kernel_ms"][k]) if iso else None
        m_mean = mean_history(np.median(iters), 10)
        rf, dom = roofline_dual(tot, N, L, m_mean, dom_cls)
        if rf is not None:
            rf["mean_history"] = round(m_mean, 3)
        if rf is not None and iso is not None:
            ri, _ = roofline_dual(iso, N, L, m_mean, dom)
            if ri is not None:
                rf["isolated"] = {"achieved": ri["achieved"], "frac": ri["frac"], "lanes": 1,
                                  "avg_launch_ms": round(iso["kernel_ms"][dom] /
                                                         max(1, iso["kernel_launches"][dom]), 4),
                                  "measured": f"one untimed step of {B} loci on a single lane"}
        if rf is not None:
            trials = float(np.median(nfe)) / max(1.0, float(np.median(iters)))
            rf["whole_solve"] = whole_solve_dual(tot, N, L, m_mean, trials, dev_ms / 1e3)
    else:
        rf, dom = roofline(tot, N, L, Dp, 10, 2 if args.history_bf16 else 4)
    # accuracy: the FP64 oracle's objective and gradient at the parameters
    # the engine returns, for a seeded sample of the first timed step's loci.
    # The step is solved again after the timed region (same engine, same
    # queue of loci, so the slots refill as they did), returning solutions
    # only at the sampled positions.
    accuracy, f_step = None, None
    if rank == 0 and args.accuracy_sample > 0:
        vloci = loci_for(args.warmup)
        pos = np.sort(np.random.default_rng(1234).choice(len(vloci), min(args.accuracy_sample, len(vloci)),
                                                         replace=False))
        rv = E.solve(vloci, x_positions=pos, want_scores=False)
        f_step = rv.f
        lh, lJ, _ = E.lambdas()
        f_orc, g_orc = oracle_check(st, w, lh, lJ, vloci[pos], rv.x, os.cpu_count() or 1)
        rel = np.abs(rv.f[pos] - f_orc) / np.abs(f_orc)
        accuracy = {"n": int(len(pos)), "max_rel_obj_err": float(rel.max()),
                    "median_rel_obj_err": float(np.median(rel)), "max_oracle_gnorm": float(g_orc.max()),
                    "gradient_threshold": 1e-3, "status_counts": {str(k): int((rv.status[pos] == k).sum())
                                                                   for k in sorted(set(rv.status[pos].tolist()))},
                    "loci": [int(v) for v in vloci[pos]],
                    "how": ("|f_engine - f_oracle(x_engine)| / f_oracle(x_engine), the FP64 oracle evaluated at "
                            "the engine's returned parameters; max_oracle_gnorm: the oracle's max|g| there "
                            "(SuperDCA's stop test is max|g| < 1e-3); sampled from the first timed step's loci, "
                            "re-solved after the timed region in the same queue")}
    # what the learned start gains: the first timed step's loci solved again
    # from zero (same engine and queue), against the timed warm-started solve
    ws_effect = None
    if ws and not args.no_zero_start and first is not None:
        E.set_warm_start(None)
        rz = E.solve(loci_for(args.warmup), want_scores=True)
        pz = E.profile()
        rw_, ms_w = first
        ws_effect = {"warm_loci_s": round(per_step / (ms_w / 1e3), 4),
                     "zero_start_loci_s": round(per_step / (pz["solve_ms"] / 1e3), 4),
                     "speedup": round(pz["solve_ms"] / ms_w, 4),
                     "warm_mean_iterations": round(float(rw_.iterations.mean()), 2),
                     "zero_mean_iterations": round(float(rz.iterations.mean()), 2),
                     "max_rel_f_diff": float(np.max(np.abs(rw_.f - rz.f) / np.abs(rz.f))),
                     "zero_status_counts": {str(k): int((rz.status == k).sum()) for k in sorted(set(rz.status.tolist()))},
                     "how": ("the first timed step's loci solved again with the warm start disabled, after the "
                             "timed region; device time of each solve (CUDA events)")}
    E.close()

    # the plain GPU form (FP32 gather contractions, FP32 L-BFGS history,
    # zero start) on the same alignment: the spec ratio's denominator
    vs_plain = None
    if rank == 0 and args.form != "gather" and not args.no_plain and args.plain_loci > 0:
        pB = 64
        Ep = Engine(N, L, batch=pB, device=local, form=FORM_GATHER, lanes=1)
        Ep.set_alignment(st, w)
        ploci = loci_for(args.warmup)[:args.plain_loci]
        Ep.solve(loci_for(args.warmup + args.steps)[:8], want_scores=True)   # warm-up (other loci)
        rp = Ep.solve(ploci, want_scores=True)
        pp = Ep.profile()
        Ep.close()
        plain = len(ploci) / (pp["solve_ms"] / 1e3)
        vs_plain = {"plain_loci_s": round(plain, 4), "ratio": round(value / plain, 2),
                    "plain_form": "gather (FP32 contractions on the CUDA cores, FP32 L-BFGS history, zero start)",
                    "plain_batch": pB, "plain_loci": int(len(ploci)),
                    "plain_median_iterations": float(np.median(rp.iterations)),
                    "plain_status_counts": {str(k): int((rp.status == k).sum()) for k in sorted(set(rp.status.tolist()))},
                    "how": ("device time (CUDA events) of one solve of the first timed step's first "
                            f"{len(ploci)} loci, after a warm-up solve; ratio = value / plain_loci_s")}
        if f_step is not None:
            fd = f_step[:len(ploci)]
            vs_plain["max_rel_f_diff_vs_headline"] = float(np.max(np.abs(rp.f - fd) / np.abs(fd)))

    if rf is not None:
        rf["avg_launch_ms"] = round(tot["kernel_ms"][dom] / max(1, tot["kernel_launches"][dom]), 4)
        rf["lanes"] = lanes   # launches of different lanes overlap in time
        per_unit = NCU_TRAFFIC_PER_UNIT.get((args.workload, dom))
        if per_unit is not None and tot["kernel_launches"][dom] > 0:
            units = tot["kernel_units"][dom] / tot["kernel_launches"][dom]
            rf["traffic"] = round(per_unit * units)   # bytes per launch, scaled from a 128-slot capture
            rf["traffic_source"] = "ncu dram bytes of a 128-slot launch, scaled by the units per launch"
    out = {
        "metric": METRIC,
        "value": round(value, 4), "unit": "loci/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_dev * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"tc": "fp16x2->fp32 (tensor cores), fp64 reductions",
                  "dual": "exact integer K.rho (fp16 digits, fp32 accumulators), double-float (2 x fp32) L-BFGS vectors",
                  "gather": "fp32"}[args.form],
        "data": "synthetic (seeded coalescent-tree alignment)",
        "config": {"workload": f"{args.workload} seed {args.seed}", "N": int(N), "L": int(L),
                   "batch": B, "lanes": lanes, "loci_per_step": per_step, "form": args.form,
                   "history": "bf16" if args.history_bf16 else "fp32",
                   "warm_start": os.path.basename(ws) if ws else None,
                   "weights": "unit (--no-reweighting)", "gradient_threshold": 1e-3,
                   "l2": (f"inputs larger than L2 ({N * L / 1e6:.0f} MB alignment; per-slot solver state "
                          f"{B * lanes} slots)"),
                   "parallelism": f"loci sharded over {world} rank(s)"},
        "clocks": clk, "e2e": e2e, "gpu_launches": int(launches), "roofline": rf,
        "accuracy": accuracy, "vs_plain": vs_plain, "warm_start_effect": ws_effect, "autotune": tune,
        "reweighting": rw,
        "kernel_ms": {k: round(v, 2) for k, v in tot["kernel_ms"].items()},
        "kernel_launches": dict(tot["kernel_launches"]), "kernel_units": dict(tot["kernel_units"]),
        "solver": {"median_nfeval": float(np.median(nfe)), "median_iterations": float(np.median(iters)),
                   "p90_iterations": float(np.percentile(iters, 90)), "max_iterations": int(np.max(iters)),
                   "median_contractions": float(np.median(contr)),
                   "status_counts": {str(k): statuses.count(k) for k in sorted(set(statuses))},
                   "wall_s": round(wall, 2), "wall_s_per_step": [round(v, 3) for v in walls]},
    }
    if rank == 0 and world == 1 and not args.no_secondary and args.form == "dual":
        out["secondary"] = secondary_skewed(args, local)
    if rank == 0 and world == 1 and not args.no_parity:
        out["parity_small"] = parity_small(local)
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        spe, n_eval, t_cpu = cpu_eval_rate(st, args.cpu_seconds, threads)
        try:
            nf, meta = nfeval_reference(args.workload)
            nf_src = (f"median of full FP64 oracle solves of {len(meta['loci'])} loci, "
                      f"oracle/nfeval_{args.workload}.json, as in --impl reference")
        except OSError:
            nf = float(np.median(nfe))
            nf_src = "median of this run's engine solves (no oracle count for this workload)"
        out["cpu_baseline"] = {
            "value": round(threads / (spe * nf), 6), "unit": "loci/s", "cores": threads,
            "kind": "port",
            "sample": (f"{n_eval} full-size FP64 objective+gradient evaluations ({t_cpu:.1f} s) on "
                       f"{threads} threads, {spe:.3f} s each; loci/s = threads / (s per evaluation x "
                       f"{nf:.0f} evaluations per locus, SuperDCA counting, {nf_src})")}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def reference_arm(args):
    world, rank, local = dist()
    if rank != 0:
        return
    st = load_workload(args)
    N, L = st.shape
    threads = os.cpu_count() or 1
    nf, meta = nfeval_reference(args.workload)
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_eval_rate(st, 0.0, threads)
    vals, spes = [], []
    t0 = time.time()
    for _ in range(args.steps):
        spe, n_eval, t = cpu_eval_rate(st, per_step, threads)
        spes.append(spe)
        vals.append(threads / (spe * nf))
    wall = time.time() - t0
    value = float(np.mean(vals))
    sample = (f"each step: >= {per_step:.0f} s of full-size FP64 objective+gradient evaluations on "
              f"{threads} threads ({np.mean(spes):.3f} s each); loci/s = threads / (s per evaluation x "
              f"{nf:.0f} evaluations per locus, median of full oracle solves of {len(meta['loci'])} loci, "
              f"oracle/nfeval_{args.workload}.json)")
    out = {
        "metric": METRIC,
        "value": round(value, 6), "unit": "loci/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(wall * 1e3 / args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded coalescent-tree alignment)", "impl": "reference",
        "config": {"workload": f"{args.workload} seed {args.seed}", "N": int(N), "L": int(L),
                   "weights": "unit (--no-reweighting)", "gradient_threshold": 1e-3},
        "cpu_baseline": {"value": round(value, 6), "unit": "loci/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 6), "unit": "loci/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    else:
        engine_arm(args)


if __name__ == "__main__":
    main()
