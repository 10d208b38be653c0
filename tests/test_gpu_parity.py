"""Engine (CUDA, through the C ABI) against the FP64 oracle and SuperDCA's own
code (golden fixtures).

Tolerances: the engine contracts in FP32 and reduces the objective in FP64.
  objective at a given x          rel 1e-6
  gradient at a given x           abs 1e-4 x max(1, max|g|)
  converged objective vs optimum  rel 1e-6
  coupling scores                 abs 1e-4
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_engine(states, weights, **kw):
    from superdca_gb300 import Engine

    N, L = states.shape
    E = Engine(N, L, **kw)
    E.set_alignment(states, weights)
    return E


def fp64_check(O, states, weights, E, loci, res, rel=1e-6):
    """Engine objective == FP64 oracle objective at the engine's parameters."""
    lh, lJ, _ = E.lambdas()
    P = O.Problem(states, weights, lh, lJ)
    for k, r in enumerate(loci):
        f64, g64 = P.objective(int(r), res.x[k])
        assert res.f[k] == pytest.approx(f64, rel=rel), (r, res.f[k], f64)
    return P


def test_eval_matches_reference_golden(engine_lib, golden_obj):
    for name, d in golden_obj.items():
        E = make_engine(d["states"], d["weights"])
        lh, lJ, _ = E.lambdas()
        assert lh == pytest.approx(d["lambda_h"], rel=1e-15)
        assert lJ == pytest.approx(d["lambda_J"], rel=1e-15)
        for r, x, f_ref, g_ref in zip(d["loci"], d["x"], d["f"], d["g"]):
            f, g = E.eval(int(r), x)
            assert f == pytest.approx(f_ref, rel=1e-6), (name, r)
            tol = 1e-4 * max(1.0, np.abs(g_ref).max())
            np.testing.assert_allclose(g, g_ref, rtol=0, atol=tol, err_msg=f"{name} r={r}")
        E.close()


def test_solve_reaches_reference_optimum(engine_lib, golden_opt, oracle_mod):
    for name, d in golden_opt.items():
        E = make_engine(d["states"], d["weights"], gradient_threshold=1e-6, batch=4)
        loci = d["loci"]
        res = E.solve(loci, want_x=True)
        assert set(res.status.tolist()) <= {0, 2}, res.status
        np.testing.assert_allclose(res.f, d["f"], rtol=1e-6, err_msg=name)
        np.testing.assert_allclose(res.scores, d["scores"], atol=1e-4, equal_nan=True, err_msg=name)
        fp64_check(oracle_mod, d["states"], d["weights"], E, loci, res)
        E.close()


@pytest.fixture(scope="module")
def cfg_small(oracle_mod):
    from superdca_gb300 import synthetic

    st, cols, pairs = synthetic.workload("independent-200x500", seed=1)
    w = oracle_mod.weights(st, 0.9)
    return st, w, pairs


def test_solve_default_threshold_small_workload(engine_lib, oracle_mod, cfg_small):
    O = oracle_mod
    st, w, pairs = cfg_small
    loci = np.arange(64)
    E = make_engine(st, w, batch=64)
    res = E.solve(loci, want_x=True)
    assert np.all(res.status == 0), res.status
    assert np.all(res.gnorm < 1e-3)
    P = fp64_check(O, st, w, E, loci, res)
    _, ost = P.solve(loci, threads=8, gtol=1e-3)
    f_orc = np.array([s["f"] for s in ost])
    np.testing.assert_allclose(res.f, f_orc, rtol=1e-6)
    # SuperDCA-counted evaluations are comparable with the oracle's
    n_orc = np.array([s["nfeval"] for s in ost])
    assert abs(np.median(res.nfeval) - np.median(n_orc)) <= 0.5 * np.median(n_orc)
    E.close()


def test_scores_and_topk_small_workload(engine_lib, oracle_mod, cfg_small):
    from superdca_gb300 import coupling_lines

    O = oracle_mod
    st, w, pairs = cfg_small
    N, L = st.shape
    loci = np.arange(L)
    E = make_engine(st, w, batch=128, gradient_threshold=1e-5)
    res = E.solve(loci)
    lh, lJ, _ = O.lambdas(w)
    P = O.Problem(st, w, lh, lJ)
    sub = np.arange(0, L, 5)
    osc, _ = P.solve(sub, threads=8, gtol=1e-5)
    np.testing.assert_allclose(res.scores[sub], osc, atol=1e-4, equal_nan=True)
    # the 10,000 strongest pairs against the oracle's (every locus solved)
    import bench
    oall, _ = P.solve(loci, threads=os.cpu_count() or 1, gtol=1e-5)
    ov = bench.top_overlap(coupling_lines(res.scores, loci), coupling_lines(oall, loci))
    print(f"\n[200 x 500] top-10k pair overlap with the oracle: {ov:.5f}")
    assert ov >= 0.99
    # planted pairs lead the ranking
    lines = coupling_lines(res.scores, loci)
    top = sorted(lines, reverse=True)[:len(pairs)]
    planted = {tuple(sorted((int(a) + 1, int(b) + 1))) for a, b in pairs}
    hit = sum(tuple(sorted((r, n))) in planted for _, r, n in top)
    assert hit >= 0.8 * len(pairs)
    E.close()


def test_batch_refill_is_order_independent(engine_lib, cfg_small):
    st, w, _ = cfg_small
    loci = np.array([5, 0, 7, 3, 499, 250, 17, 16, 15, 31, 32, 100, 1, 2, 498, 64, 65, 66, 67, 68])
    E1 = make_engine(st, w, batch=64)
    a = E1.solve(loci)
    E2 = make_engine(st, w, batch=3)
    b = E2.solve(loci)
    # batch composition changes the order of the FP64 reductions, so the
    # trajectories and stopping points differ at rounding level
    np.testing.assert_allclose(a.f, b.f, rtol=1e-6)
    np.testing.assert_allclose(a.scores, b.scores, atol=1e-4, equal_nan=True)
    E1.close(); E2.close()


def test_warm_start_and_solution_roundtrip(engine_lib, golden_opt, oracle_mod):
    d = golden_opt["opt0"]
    E = make_engine(d["states"], d["weights"], gradient_threshold=1e-4)
    loci = d["loci"][:6]
    res = E.solve(loci, x_init=d["x"][:6], want_x=True)
    assert np.all(res.iterations <= 1), res.iterations
    np.testing.assert_allclose(res.f, d["f"][:6], rtol=1e-7)
    for k, r in enumerate(loci):
        f, g = E.eval(int(r), res.x[k])
        assert f == pytest.approx(res.f[k], rel=1e-6)
    E.close()


@pytest.mark.parametrize("N,L", [(1, 2), (5, 17), (70, 33), (300, 16)])
def test_edge_shapes(engine_lib, oracle_mod, N, L):
    O = oracle_mod
    rng = np.random.default_rng(N * 100 + L)
    st = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
    w = rng.uniform(0.0, 1.0, size=N)
    w[:: 7] = 0.0
    if N == 1:
        w[0] = 1.0
    E = make_engine(st, w, batch=5, gradient_threshold=1e-5)
    loci = np.arange(L)
    res = E.solve(loci, want_x=True)
    assert set(res.status.tolist()) <= {0, 2}, res.status
    P = fp64_check(O, st, w, E, loci, res)
    _, ost = P.solve(loci, threads=4, gtol=1e-6)
    np.testing.assert_allclose(res.f, [s["f"] for s in ost], rtol=1e-6)
    assert np.all(np.isnan(res.scores[np.arange(L), loci]))
    E.close()


def test_invalid_inputs(engine_lib):
    from superdca_gb300 import Engine, EngineError

    E = Engine(4, 5)
    with pytest.raises(EngineError):
        E.solve([0])  # no alignment yet
    st = np.zeros((4, 5), dtype=np.uint8)
    st[2, 3] = 4
    with pytest.raises(EngineError, match="0..q-1"):
        E.set_alignment(st, np.ones(4))
    with pytest.raises(EngineError):
        E.set_alignment(np.zeros((4, 5), dtype=np.uint8), -np.ones(4))
    E.set_alignment(np.zeros((4, 5), dtype=np.uint8), np.ones(4))
    with pytest.raises(EngineError, match="out of range"):
        E.solve([5])
    res = E.solve([])
    assert len(res.f) == 0
    E.close()


def test_tree_workload_subset(engine_lib, oracle_mod):
    """3000 sequences x 10,000 loci, unit weights (--no-reweighting)."""
    from superdca_gb300 import synthetic

    O = oracle_mod
    st, _, _ = synthetic.workload("tree-3000x10000", seed=2)
    w = np.ones(st.shape[0])
    loci = np.array([0, 4999, 9998, 1234])
    E = make_engine(st, w, batch=4)
    res = E.solve(loci, want_x=True)
    assert np.all(res.status == 0), res.status
    P = fp64_check(O, st, w, E, loci, res)
    _, ost = P.solve(loci, threads=4, gtol=1e-3)
    np.testing.assert_allclose(res.f, [s["f"] for s in ost], rtol=1e-6)
    E.close()


def test_gpu_weights_match_reference_rule(engine_lib, oracle_mod, golden_obj):
    """Sequence reweighting on the GPU equals the oracle (itself bit-exact with
    SuperDCA's calculate_weights on the golden fixtures) exactly."""
    from superdca_gb300 import Engine

    O = oracle_mod
    # golden fixtures: weights produced by SuperDCA's own calculate_weights
    for name, d in golden_obj.items():
        st = d["states"]
        E = Engine(*st.shape)
        w = E.compute_weights(st, float(d["threshold"]))
        np.testing.assert_array_equal(w, d["weights"], err_msg=name)
        E.close()
    rng = np.random.default_rng(41)
    for N, L, thr in [(300, 777, 0.9), (129, 64, 0.8), (65, 33, 1.0), (1000, 5000, 0.95)]:
        st = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
        base = st[0].copy()
        for i in range(1, N, 3):  # clusters of near-identical sequences
            st[i] = base
            flip = rng.random(L) < 0.05
            st[i, flip] = rng.integers(0, 4, size=flip.sum())
        mult = rng.integers(1, 4, size=N).astype(np.float64)
        E = Engine(N, L)
        for m in (None, mult):
            w = E.compute_weights(st, thr, mult=m)
            np.testing.assert_array_equal(w, O.weights(st, thr, mult=m), err_msg=f"{N}x{L} thr {thr}")
        E.close()
