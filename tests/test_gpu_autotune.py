"""The autotuner (sdca_autotune): candidate (batch, lanes) pairs solve the
first loci of the caller's list for real; the pair with the most L-BFGS
iterations per device second is chosen and can be kept in a cache file.
The probe loci's results must be those of an ordinary solve (the same
optimum, against the FP64 oracle), and a cached choice must come back
without a probe."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_probes_are_real_solves_and_cache(oracle_mod, tmp_path):
    from superdca_gb300 import FORM_DUAL, Engine, autotune, synthetic
    O = oracle_mod
    states, _, _ = synthetic.workload("tree-3000x10000", seed=5, N=400, L=2600)
    N, L = states.shape
    w = np.ones(N)
    loci = np.random.default_rng(3).permutation(L)[:2400]
    cache = str(tmp_path / "tune.txt")
    tr = autotune(states, w, loci, form=FORM_DUAL, max_fraction=1.0, cache_path=cache)
    measured = [e for e in tr.entries if e["status"] == 0]
    assert measured, tr.entries
    assert (tr.batch, tr.lanes) in [(e["batch"], e["lanes"]) for e in measured]
    assert tr.n_done == sum(e["n_loci"] for e in measured) and tr.n_done <= len(loci)
    for e in measured:
        assert e["n_loci"] == 2 * e["batch"] * e["lanes"] and e["iterations_per_s"] > 0
    assert all(s["status"] == 0 for s in tr.stats)
    # the probes' results equal an ordinary solve's (same optimum), and the oracle's
    sub = loci[:12]
    with Engine(N, L, batch=16, form=FORM_DUAL) as E:
        E.set_alignment(states, w)
        res = E.solve(sub, want_x=True)
        lh, lJ, _ = E.lambdas()
    f_tune = np.array([s["f"] for s in tr.stats[:12]])
    np.testing.assert_allclose(f_tune, res.f, rtol=1e-6)
    P = O.Problem(states, w, lh, lJ)
    f_orc = np.array([P.objective(int(r), res.x[k], grad=False) for k, r in enumerate(sub)])
    np.testing.assert_allclose(f_tune, f_orc, rtol=1e-6)
    np.testing.assert_allclose(tr.scores[:12][~np.isnan(res.scores)], res.scores[~np.isnan(res.scores)],
                               rtol=0, atol=1e-4)
    # the choice is cached per shape: a second call runs no probe
    tr2 = autotune(states, w, loci, form=FORM_DUAL, max_fraction=1.0, cache_path=cache)
    assert tr2.cached and tr2.n_done == 0 and (tr2.batch, tr2.lanes) == (tr.batch, tr.lanes)
