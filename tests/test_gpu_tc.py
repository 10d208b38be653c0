"""The tensor-core contraction form (tcgen05 one-hot GEMMs, fp16 hi+lo
operands, FP32 accumulation) against the FP64 oracle, SuperDCA's own optimum
(golden fixtures) and the FP32 gather form.

Same tolerances as the gather form: objective rel 1e-6, scores abs 1e-4."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_engine(states, weights, **kw):
    from superdca_gb300 import Engine, FORM_TC

    N, L = states.shape
    E = Engine(N, L, form=FORM_TC, **kw)
    E.set_alignment(states, weights)
    return E


def fp64_check(O, states, weights, E, loci, res, rel=1e-6):
    """Reported objective == FP64 oracle objective at the returned parameters;
    returns the FP64 values."""
    lh, lJ, _ = E.lambdas()
    P = O.Problem(states, weights, lh, lJ)
    f64s = []
    for k, r in enumerate(loci):
        f64 = P.objective(int(r), res.x[k], grad=False)
        assert res.f[k] == pytest.approx(f64, rel=rel), (r, res.f[k], f64)
        f64s.append(f64)
    P.f64 = np.array(f64s)
    return P


def test_tc_small_shapes(engine_lib, oracle_mod):
    """Shapes below one tile in every dimension and with ragged edges."""
    O = oracle_mod
    for N, L, B in [(40, 5, 4), (70, 33, 5), (130, 17, 33)]:
        rng = np.random.default_rng(N + L)
        st = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
        w = rng.uniform(0.1, 1.0, size=N)
        E = make_engine(st, w, batch=B, gradient_threshold=1e-5)
        loci = np.arange(L)
        res = E.solve(loci, want_x=True)
        assert set(res.status.tolist()) <= {0, 2}, res.status
        P = fp64_check(O, st, w, E, loci, res)
        _, ost = P.solve(loci, threads=4, gtol=1e-6)
        np.testing.assert_allclose(res.f, [s["f"] for s in ost], rtol=1e-6)
        E.close()


def test_tc_reaches_reference_optimum(engine_lib, golden_opt, oracle_mod):
    for name, d in golden_opt.items():
        E = make_engine(d["states"], d["weights"], gradient_threshold=1e-6, batch=4)
        loci = d["loci"]
        res = E.solve(loci, want_x=True)
        assert set(res.status.tolist()) <= {0, 2}, res.status
        np.testing.assert_allclose(res.f, d["f"], rtol=1e-6, err_msg=name)
        np.testing.assert_allclose(res.scores, d["scores"], atol=1e-4, equal_nan=True, err_msg=name)
        fp64_check(oracle_mod, d["states"], d["weights"], E, loci, res)
        E.close()


def test_tc_matches_gather_small_workload(engine_lib, oracle_mod):
    from superdca_gb300 import Engine, synthetic

    O = oracle_mod
    st, _, _ = synthetic.workload("independent-200x500", seed=1)
    w = O.weights(st, 0.9)
    N, L = st.shape
    loci = np.arange(0, L, 4)
    E = make_engine(st, w, batch=64)
    res = E.solve(loci, want_x=True)
    assert np.all(res.status == 0), res.status
    a = fp64_check(O, st, w, E, loci, res, rel=1e-7).f64
    G = Engine(N, L, batch=64)
    G.set_alignment(st, w)
    ref = G.solve(loci, want_x=True)
    b = fp64_check(O, st, w, G, loci, ref, rel=1e-7).f64
    # both forms stop at max|g| < 1e-3 of a strictly convex objective: the
    # FP64 objectives at their two solutions agree far inside the bar
    np.testing.assert_allclose(a, b, rtol=1e-6)
    np.testing.assert_allclose(res.f, ref.f, rtol=1e-6)
    np.testing.assert_allclose(res.scores, ref.scores, atol=1e-4, equal_nan=True)
    E.close(); G.close()


def test_tc_tree_workload_subset(engine_lib, oracle_mod):
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


def test_tc_bf16_history(engine_lib, oracle_mod):
    """L-BFGS (s, y) pairs stored in BF16: the direction is still a descent
    direction built from consistent dot products; the optimum is unchanged."""
    from superdca_gb300 import synthetic

    O = oracle_mod
    st, _, _ = synthetic.workload("independent-200x500", seed=3)
    w = O.weights(st, 0.9)
    loci = np.arange(0, 500, 10)
    E = make_engine(st, w, batch=32, history_bf16=True)
    res = E.solve(loci, want_x=True)
    assert np.all(res.status == 0), res.status
    P = fp64_check(O, st, w, E, loci, res)
    _, ost = P.solve(loci, threads=8, gtol=1e-3)
    np.testing.assert_allclose(res.f, [s["f"] for s in ost], rtol=1e-6)
    E.close()
