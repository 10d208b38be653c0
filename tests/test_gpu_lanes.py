"""Solver lanes (sdca_config.lanes): several slot sets, each with its own
stream and host thread, over one resident alignment and one queue of loci.
A locus's solve does not depend on the lane that takes it, so results match
a single lane's (up to the check batching, which moves a stop by at most a
few iterations: objective rel 1e-6, scores 1e-4), and the profile adds up
the lanes' work."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solve(states, w, loci, form, lanes, batch, targets=None, blob=None, want_x=False):
    from superdca_gb300.engine import Engine
    N, L = states.shape
    with Engine(N, L, form=form, batch=batch, lanes=lanes) as E:
        E.set_alignment(states, w)
        if targets is not None:
            E.set_targets(targets)
        if blob is not None:
            E.set_warm_start(blob)
        r = E.solve(loci, want_x=want_x)
        return r, E.profile()


@pytest.mark.parametrize("form", ["dual", "tc", "gather"])
def test_lanes_match_one_lane(oracle_mod, form):
    from superdca_gb300 import _lib, synthetic
    O = oracle_mod
    states, _, _ = synthetic.workload("independent-200x500", seed=3, N=240, L=300)
    N, L = states.shape
    w = np.random.default_rng(1).uniform(0.3, 1.0, N)
    loci = np.random.default_rng(2).choice(L, 40, replace=False)
    fm = {"dual": _lib.FORM_DUAL, "tc": _lib.FORM_TC, "gather": _lib.FORM_GATHER}[form]
    one, p1 = _solve(states, w, loci, fm, 1, 6)
    many, p3 = _solve(states, w, loci, fm, 3, 6, want_x=True)
    assert np.all(one.status == 0) and np.all(many.status == 0)
    np.testing.assert_allclose(many.f, one.f, rtol=1e-6)
    mask = ~np.isnan(one.scores)
    np.testing.assert_allclose(many.scores[mask], one.scores[mask], rtol=0, atol=1e-4)
    # each row belongs to its own locus: the oracle at the returned parameters
    lh, lJ = O.lambdas(w)[:2]
    P = O.Problem(states, w, lh, lJ)
    for k in (0, 17, 39):
        assert abs(P.objective(int(loci[k]), many.x[k], grad=False) - many.f[k]) <= 1e-6 * abs(many.f[k])
    assert p3["iterations"] == int(many.iterations.sum())
    assert p3["gpu_launches"] > p1["gpu_launches"] // 2


def test_lanes_scan_mode_and_empty_queue():
    from superdca_gb300 import _lib
    from superdca_gb300.engine import Engine
    rng = np.random.default_rng(5)
    feats = rng.integers(0, 4, size=(90, 40)).astype(np.uint8)
    tg = rng.integers(0, 4, size=(90, 7)).astype(np.uint8)
    w = np.ones(90)
    res = []
    for lanes in (1, 4):
        with Engine(90, 40, form=_lib.FORM_DUAL, batch=2, lanes=lanes) as E:
            E.set_alignment(feats, w)
            E.set_targets(tg)
            res.append(E.solve(np.arange(7)))
            # fewer loci than lanes x batch, and none at all
            r1 = E.solve([3])
            assert r1.status[0] == 0
            r0 = E.solve(np.zeros(0, dtype=np.uint32))
            assert len(r0.f) == 0
    np.testing.assert_allclose(res[1].f, res[0].f, rtol=1e-6)


def test_lanes_warm_start_reaches_each_lane():
    from superdca_gb300 import _lib, synthetic
    from superdca_gb300 import warmstart as W
    states, _, _ = synthetic.workload("independent-200x500", seed=4, N=160, L=120)
    N, L = states.shape
    w = np.ones(N)
    loci = np.arange(0, L, 5)
    blob = W.new_blob(np.random.default_rng(0).normal(size=(64, 40)).astype(np.float32),
                      np.full((64, 16), 0.01, np.float32))
    one, _ = _solve(states, w, loci, _lib.FORM_TC, 1, 4, blob=blob)
    many, _ = _solve(states, w, loci, _lib.FORM_TC, 3, 4, blob=blob)
    assert np.all(many.status == 0)
    np.testing.assert_allclose(many.f, one.f, rtol=1e-6)


def test_lanes_argument_checks():
    from superdca_gb300 import _lib
    from superdca_gb300.engine import Engine, EngineError
    with pytest.raises(EngineError):
        Engine(10, 5, lanes=17)
    with Engine(30, 8, form=_lib.FORM_GATHER, batch=2, lanes=2) as E:
        E.set_alignment(np.random.default_rng(0).integers(0, 4, size=(30, 8)).astype(np.uint8), np.ones(30))
        with pytest.raises(EngineError):
            E.solve([0, 8])      # out of range: refused before any lane starts
        assert np.all(E.solve([0, 1, 2, 3, 4]).status == 0)
