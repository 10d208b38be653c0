"""The bench's CPU legs (the oracle timed on host cores) and its contract
helpers, on small inputs: no GPU."""
import json
import os

import numpy as np

import bench


def test_cpu_eval_rate_runs_at_least_one_batch(oracle_mod):
    """A zero-second request (the reference arm's warm-up) still times one
    batch of evaluations instead of dividing by zero."""
    st = np.random.default_rng(0).integers(0, 4, size=(24, 40)).astype(np.uint8)
    spe, done, t = bench.cpu_eval_rate(st, 0.0, 2)
    assert done == 2 and t > 0.0 and np.isfinite(spe) and spe > 0.0


def test_nfeval_reference_file_is_consistent():
    """The evaluations per locus the reference arm divides by come from full
    oracle solves of the headline workload, committed beside the oracle."""
    nf, meta = bench.nfeval_reference("tree-3000x94000")
    assert nf > 100
    assert len(meta["nfeval"]) == len(meta["loci"])
    with open(os.path.join(bench.ROOT, "oracle", "nfeval_tree-3000x94000.json")) as fh:
        assert json.load(fh)["nfeval"] == meta["nfeval"]


def test_roofline_dual_picks_the_requested_class():
    """With overlapping lanes the bench names the class from an isolated step;
    roofline_dual reports that class, not the one with the most summed time."""
    keys = ["forward", "backward", "linesearch", "history", "direction", "accept", "score", "other"]
    tot = {"kernel_ms": {k: 1.0 for k in keys}, "kernel_units": {k: 10 for k in keys},
           "kernel_launches": {k: 1 for k in keys}}
    tot["kernel_ms"]["linesearch"] = 50.0
    rf, cls = bench.roofline_dual(tot, 3000, 94000, 10)
    assert cls == "linesearch"
    rf, cls = bench.roofline_dual(tot, 3000, 94000, 10, "direction")
    assert cls == "direction" and rf["bound"] == "hbm" and rf["kernel"] == "direction"
    # per unit: (4k + 3) vectors read, d written, k_x read, u - u_y with P0
    # written: (4k + 7) parts of 32 N bytes, over 1 ms for 10 units
    per = ((4 * 10 + 3) + 2 + 1 + 1) * 32 * 3000
    assert abs(rf["achieved"] - round(per * 10 / 1e-3 / 1e9, 1)) < 0.2


def test_top_overlap_counts_shared_strongest_pairs():
    a = [(float(v), 1, 2) for v in [5, 4, 3, 2, 1]]
    b = [(float(v), 1, 2) for v in [5, 4, 0, 2, 3]]
    assert bench.top_overlap(a, b, k=2) == 1.0          # {0, 1} in both
    assert bench.top_overlap(a, b, k=3) == 2 / 3        # {0, 1, 2} vs {0, 1, 4}
    assert bench.top_overlap(a, a, k=10) == 1.0         # k above the length: all pairs


def test_whole_solve_roofline_counts_every_class():
    """The whole-solve figure sums the HBM classes' algorithmic bytes per
    slot-iteration ((2k + 1) + (4k + 7) + 15.5 + 1 + trials x (1.5 + 9/32)
    parts of 32 N bytes) and the tensor classes' FLOP, over the device time."""
    keys = ["forward", "backward", "linesearch", "history", "direction", "accept", "score", "other"]
    tot = {"kernel_ms": {k: 1.0 for k in keys}, "kernel_units": {k: 0 for k in keys},
           "kernel_launches": {k: 1 for k in keys}}
    N, L, m, trials = 3000, 94000, 10, 6.0
    tot["kernel_units"]["history"] = 100
    tot["kernel_units"]["forward"] = 100
    tot["kernel_units"]["backward"] = 2
    ws = bench.whole_solve_dual(tot, N, L, m, trials, 2.0)
    parts = (2 * m + 1) + (4 * m + 7) + 15.5 + 1 + trials * (1.5 + 9 / 32)
    assert ws["hbm_bytes_per_slot_iteration"] == round(parts * 32 * N)
    assert abs(ws["hbm_achieved_gbs"] - round(100 * parts * 32 * N / 2.0 / 1e9, 1)) < 0.11
    flop = 100 * 2.0 * N * N * 3 + 2 * 2.0 * N * L * 16
    assert abs(ws["tensor_achieved_tflops"] - round(flop / 2.0 / 1e12, 2)) < 0.011
    hbm, tflops, _ = bench.measured_peaks()
    assert abs(ws["hbm_frac"] - ws["hbm_achieved_gbs"] / hbm) < 1e-3


def test_clocks_summary_reads_throttle_reasons_and_utilisation(tmp_path):
    """The nvidia-smi sampler's summary: median SM clock under load, the
    throttle reasons seen, and the kernel-occupancy column (utilization.gpu)."""

    class Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

        def kill(self):
            pass

    path = tmp_path / "clocks.csv"
    path.write_text("0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active, 100\n"
                    "0, 2070, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active, 93\n"
                    "0, 600, 2070, 120.0, 0x0, Not Active, Not Active, Not Active, Not Active, 0\n")
    c = bench.Clocks(0)
    c.proc, c.path = Done(), str(path)
    out = c.stop()
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0 and out["samples"] == 3
    assert out["reasons"] == ["sw_power_cap"]
    assert out["gpu_util_pct"] == {"median": 93.0, "min": 0.0}
    assert not path.exists()
