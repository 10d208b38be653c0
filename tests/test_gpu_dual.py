"""The dual form (SDCA_FORM_DUAL): SuperDCA's per-locus L-BFGS kept in the
span of the sequences, with one exact integer product per iteration.

It must reach the reference's optimum (objective rel 1e-6 against the FP64
oracle at the engine's own parameters and against the oracle's solves,
scores within 1e-4), stop by the reference's test (max|g| below the
threshold, checked on the oracle's gradient), and take the iterations of the
other forms (the same iteration in exact arithmetic)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _f_at(P, loci, X):
    """FP64 oracle objective of each locus at its own parameters."""
    return np.array([P.objective(int(r), X[k], grad=False) for k, r in enumerate(loci)])


def _solve(states, w, loci, form, **kw):
    from superdca_gb300.engine import Engine
    n, L = states.shape
    with Engine(n, L, form=form, **kw) as E:
        E.set_alignment(states, w)
        return E.solve(loci, want_x=True), E.lambdas()


@pytest.mark.parametrize("shape,seed", [((200, 500), 7), ((301, 45), 3), ((64, 2), 5), ((1, 20), 1)])
def test_dual_matches_oracle(oracle_mod, shape, seed):
    from superdca_gb300 import _lib, synthetic
    O = oracle_mod
    N, L = shape
    rng = np.random.default_rng(seed)
    if L >= 100:
        states, _, _ = synthetic.workload("independent-200x500", seed=seed, N=N, L=L)
    else:
        states = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
    N, L = states.shape
    w = rng.uniform(0.2, 1.0, N)
    w[rng.random(N) < 0.05] = 0.0
    loci = np.arange(L) if L <= 64 else rng.choice(L, 40, replace=False)
    res, (lh, lJ, _) = _solve(states, w, loci, _lib.FORM_DUAL, batch=16)
    P = O.Problem(states, w, lh, lJ)
    assert np.all(res.status == 0), res.status
    f_at = _f_at(P, loci, res.x)
    np.testing.assert_allclose(res.f, f_at, rtol=1e-6)
    sc, st = P.solve(loci, threads=4)
    np.testing.assert_allclose(res.f, [s["f"] for s in st], rtol=1e-6)
    mask = ~np.isnan(res.scores)
    np.testing.assert_allclose(res.scores[mask], sc[mask], rtol=0, atol=1e-4)
    for k, r in enumerate(loci[:8]):
        g = P.objective(r, res.x[k])[1]
        assert np.abs(g).max() < 1.05e-3, (r, np.abs(g).max())


def test_dual_iterations_match_other_forms():
    from superdca_gb300 import _lib, synthetic
    states, _, _ = synthetic.workload("tree-3000x10000", seed=4, N=600, L=2500)
    N, L = states.shape
    loci = np.random.default_rng(2).choice(L, 48, replace=False)
    w = np.ones(N)
    d, _ = _solve(states, w, loci, _lib.FORM_DUAL, batch=48)
    g, _ = _solve(states, w, loci, _lib.FORM_GATHER, batch=48)
    assert np.all(d.status == 0) and np.all(g.status == 0)
    np.testing.assert_allclose(d.f, g.f, rtol=1e-6)
    print(f"\nmean iterations dual {d.iterations.mean():.1f}, plain {g.iterations.mean():.1f}")
    assert abs(d.iterations.mean() - g.iterations.mean()) <= 0.1 * g.iterations.mean()


def test_dual_tree_subset_against_oracle(oracle_mod):
    from superdca_gb300 import _lib, synthetic
    O = oracle_mod
    states, _, _ = synthetic.workload("tree-3000x10000", seed=0)
    N, L = states.shape
    w = np.ones(N)
    loci = np.random.default_rng(0).choice(L, 16, replace=False)
    res, (lh, lJ, _) = _solve(states, w, loci, _lib.FORM_DUAL, batch=16)
    assert np.all(res.status == 0)
    P = O.Problem(states, w, lh, lJ)
    np.testing.assert_allclose(res.f, _f_at(P, loci, res.x), rtol=1e-6)
    for k in range(4):
        g = P.objective(loci[k], res.x[k])[1]
        assert np.abs(g).max() < 1.05e-3


def test_dual_refuses_start_points_and_per_pair_blobs():
    """The dual form keeps every iterate in the span of the sequences: it
    refuses an arbitrary start point and the per-pair network (version 1);
    its own start comes from the per-sequence network (version 2)."""
    from superdca_gb300 import _lib, synthetic
    from superdca_gb300 import warmstart as W
    from superdca_gb300._lib import EngineError
    from superdca_gb300.engine import Engine
    states = np.random.default_rng(0).integers(0, 4, size=(30, 12)).astype(np.uint8)
    with Engine(30, 12, form=_lib.FORM_DUAL, batch=4) as E:
        E.set_alignment(states, np.ones(30))
        with pytest.raises(EngineError):
            E.solve([0, 1], x_init=np.zeros((2, 16 * 12 + 4)))
        X = np.random.default_rng(1).normal(size=(10, 40)).astype(np.float32)
        with pytest.raises(EngineError):
            E.set_warm_start(W.new_blob(X, np.ones((10, 16), np.float32)))
        r = E.solve([0, 1, 2])
        assert np.all(r.status == 0)


@pytest.mark.parametrize("form", ["dual", "tc"])
def test_skewed_workload_subset(oracle_mod, form):
    """The 616 x 78,700 skewed workload (multi-allelic loci, MAF from a Beta
    distribution, gaps up to 15 %): 12 loci against the FP64 oracle at the
    engine's parameters, and the oracle's gradient there."""
    from superdca_gb300 import _lib, synthetic
    O = oracle_mod
    states, _, _ = synthetic.workload("skewed-616x78700", seed=2)
    N, L = states.shape
    w = O.weights(states, 0.9)
    loci = np.random.default_rng(6).choice(L, 12, replace=False)
    fm = _lib.FORM_DUAL if form == "dual" else _lib.FORM_TC
    res, (lh, lJ, _) = _solve(states, w, loci, fm, batch=12)
    assert np.all(res.status == 0)
    P = O.Problem(states, w, lh, lJ)
    np.testing.assert_allclose(res.f, _f_at(P, loci, res.x), rtol=1e-6)
    for k in range(3):
        g = P.objective(int(loci[k]), res.x[k])[1]
        assert np.abs(g).max() < 1.05e-3


def test_dual_graph_rounds_match_direct_launches():
    """Each round's iteration core replayed as a CUDA graph (the default)
    against the same kernels launched one by one (SDCA_DUAL_GRAPH=0): the same
    optimum per locus and the same statuses, with slots refilled; and the
    graph's class timings are collected."""
    import os
    from superdca_gb300 import _lib, synthetic
    from superdca_gb300.engine import Engine
    states, _, _ = synthetic.workload("tree-3000x10000", seed=5, N=400, L=900)
    n, L = states.shape
    loci = np.random.default_rng(2).choice(L, 40, replace=False)
    out = {}
    for mode in ("1", "0"):
        os.environ["SDCA_DUAL_GRAPH"] = mode
        try:
            with Engine(n, L, form=_lib.FORM_DUAL, batch=12, lanes=2) as E:
                E.set_alignment(states, np.ones(n))
                out[mode] = (E.solve(loci), E.profile())
        finally:
            os.environ.pop("SDCA_DUAL_GRAPH", None)
    (rg, pg), (rd, pd) = out["1"], out["0"]
    assert np.all(rg.status == 0) and np.all(rd.status == 0)
    # the runs differ in the order of atomic sums, so each stops at its own
    # point below the threshold: the converged-objective tolerance
    np.testing.assert_allclose(rg.f, rd.f, rtol=1e-6)
    np.testing.assert_allclose(rg.scores, rd.scores, atol=1e-4, equal_nan=True)
    assert abs(rg.iterations.mean() - rd.iterations.mean()) <= 0.05 * rd.iterations.mean()
    for cls in ("forward", "direction", "history", "linesearch"):
        assert pg["kernel_ms"][cls] > 0 and pg["kernel_units"][cls] > 0
