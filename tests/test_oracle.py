"""The FP64 oracle against SuperDCA's own code (golden fixtures) and against
known answers.  CPU only."""
import numpy as np
import pytest


def test_objective_gradient_match_reference(oracle_mod, golden_obj):
    O = oracle_mod
    assert len(golden_obj) >= 6
    for name, d in golden_obj.items():
        P = O.Problem(d["states"], d["weights"], d["lambda_h"], d["lambda_J"])
        for r, x, f_ref, g_ref in zip(d["loci"], d["x"], d["f"], d["g"]):
            f, g = P.objective(r, x)
            assert f == pytest.approx(f_ref, rel=1e-14), (name, r)
            # the reference sums the gradient per unique 16-locus pattern; the
            # oracle per sequence: identical up to summation order
            np.testing.assert_allclose(g, g_ref, rtol=0, atol=1e-12 * max(1.0, np.abs(g_ref).max()))


def test_weights_and_lambdas_match_reference(oracle_mod, golden_obj):
    O = oracle_mod
    for name, d in golden_obj.items():
        w = O.weights(d["states"], float(d["threshold"]))
        np.testing.assert_array_equal(w, d["weights"], err_msg=name)
        lh, lJ, _ = O.lambdas(w)
        assert lh == d["lambda_h"] and lJ == d["lambda_J"], name


def test_scores_match_reference_bitwise(oracle_mod, golden_obj):
    O = oracle_mod
    for name, d in golden_obj.items():
        L = d["states"].shape[1]
        for r, x, row_ref in zip(d["loci"], d["x"], d["scores"]):
            row = O.score_row(x, L, r)
            np.testing.assert_array_equal(row, row_ref, err_msg=f"{name} r={r}")


def test_converged_optimum_matches_reference(oracle_mod, golden_opt):
    """The optimum of SuperDCA's objective found by an independent optimiser
    is what the oracle's L-BFGS reaches."""
    O = oracle_mod
    for name, d in golden_opt.items():
        P = O.Problem(d["states"], d["weights"], d["lambda_h"], d["lambda_J"])
        L = d["states"].shape[1]
        for r, f_ref, row_ref in zip(d["loci"], d["f"], d["scores"]):
            x, st = P.minimize(r, gtol=1e-9, max_iter=5000)
            assert st["f"] == pytest.approx(f_ref, rel=1e-10), (name, r, st)
            row = O.score_row(x, L, r)
            np.testing.assert_allclose(row, row_ref, atol=1e-5, equal_nan=True)


def test_gradient_is_derivative_of_objective(oracle_mod):
    O = oracle_mod
    rng = np.random.default_rng(3)
    st = rng.integers(0, 4, size=(8, 5)).astype(np.uint8)
    w = rng.uniform(0.2, 1.0, size=8)
    P = O.Problem(st, w, 0.7, 0.3)
    x = rng.normal(size=P.D) * 0.3
    for r in range(5):
        f, g = P.objective(r, x)
        num = np.zeros_like(g)
        for k in range(P.D):
            e = np.zeros(P.D); e[k] = 1e-6
            num[k] = (P.objective(r, x + e, grad=False) - P.objective(r, x - e, grad=False)) / 2e-6
        # J_rr entries do not enter the objective: zero derivative and zero gradient
        np.testing.assert_allclose(g, num, atol=1e-7)


def test_known_answers(oracle_mod):
    O = oracle_mod
    # all sequences identical: every locus has one state; at x = 0 each
    # sequence contributes w * log(q)
    N, L = 10, 19
    st = np.zeros((N, L), dtype=np.uint8)
    w = np.ones(N)
    P = O.Problem(st, w, 1.0, 1.0)
    f = P.objective(3, np.zeros(P.D), grad=False)
    assert f == pytest.approx(N * np.log(4.0), rel=1e-15)
    # the J_rr slot never receives gradient and stays zero through a solve,
    # including in a partial last block (L = 19: blocks of 16 and 3)
    for r in (2, 17):
        x, s = P.minimize(r, gtol=1e-8)
        idx = O.ref_index(L)[r].ravel()
        assert np.all(x[idx] == 0.0)
    # two perfectly coupled loci score above an independent pair
    rng = np.random.default_rng(5)
    st = rng.integers(0, 2, size=(200, 6)).astype(np.uint8)
    st[:, 4] = st[:, 1]
    w = O.weights(st, 0.9)
    lh, lJ, _ = O.lambdas(w)
    P = O.Problem(st, w, lh, lJ)
    x, _ = P.minimize(1, gtol=1e-7)
    row = O.score_row(x, 6, 1)
    assert np.nanargmax(row) == 4


def test_weights_rule(oracle_mod):
    O = oracle_mod
    st = np.array([[0, 0, 0, 0, 0, 0, 0, 0, 0, 0],
                   [0, 0, 0, 0, 0, 0, 0, 0, 0, 1],   # 90% identical to row 0
                   [1, 1, 1, 1, 1, 1, 1, 1, 1, 1]], dtype=np.uint8)
    w = O.weights(st, 0.9)
    np.testing.assert_allclose(w, [0.5, 0.5, 1.0])
    w = O.weights(st, 0.95)
    np.testing.assert_allclose(w, [1.0, 1.0, 1.0])
    # multiplicities count towards the neighbour weights
    w = O.weights(st, 0.9, mult=np.array([2.0, 1.0, 1.0]))
    np.testing.assert_allclose(w, [2.0 / 3.0, 1.0 / 3.0, 1.0])
    lh, lJ, be = O.lambdas(np.ones(1000))
    assert (lh, lJ, be) == (0.1 * 1000, 0.1 * 1000 / 2, 1000.0)
    lh, lJ, be = O.lambdas(np.ones(100), lambda_h_opt=0.5, lambda_J_opt=0.25)
    assert (lh, lJ) == (50.0, 25.0)


@pytest.mark.skipif("not __import__('oracle.oracle', fromlist=['x']).ref_available()")
def test_oracle_against_live_reference(oracle_mod):
    """Where oracle/_ref was built (reference sources present), compare on
    fresh random cases too."""
    O = oracle_mod
    rng = np.random.default_rng(11)
    for N, L in [(33, 21), (64, 48), (17, 3)]:
        st = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
        R = O.RefProblem(st, threshold=0.85)
        w = O.weights(st, 0.85)
        np.testing.assert_array_equal(w, R.weights())
        lh, lJ, _ = O.lambdas(w)
        assert (lh, lJ) == R.lambdas()
        P = O.Problem(st, w, lh, lJ)
        for r in (0, L - 1, L // 2):
            x = rng.normal(size=P.D) * 0.1
            f1, g1 = R.objective(r, x)
            f2, g2 = P.objective(r, x)
            assert f1 == f2
            np.testing.assert_allclose(g1, g2, atol=1e-12)
            np.testing.assert_array_equal(R.score_row(r, x), O.score_row(x, L, r))


def test_mlp_oracle_gradient_matches_finite_differences():
    """The FP64 restatement of the warm-start network (oracle/mlp_oracle.py),
    which the GPU gradients are checked against, against central differences."""
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(3)
    p = np.zeros(M.SIZE)
    p[0], p[1], p[2] = 1, 3, 0.5
    p[M.IN_MEAN:M.IN_MEAN + M.N_IN] = rng.normal(size=M.N_IN) * 0.1
    p[M.IN_SCALE:M.IN_SCALE + M.N_IN] = rng.uniform(0.5, 2.0, M.N_IN)
    p[M.W1:M.TRAIN_END] = rng.normal(size=M.TRAIN_END - M.W1) * 0.2
    X = rng.normal(size=(20, M.N_IN))
    T = rng.normal(size=(20, M.N_OUT))
    f0, g = M.loss_and_grad(p, X, T)
    idx = np.concatenate([rng.choice(np.arange(M.W1, M.TRAIN_END), 60, replace=False),
                          [M.B1, M.B2 + 5, M.B3 + 15, M.W3]])
    h = 1e-6
    for i in idx:
        q = p.copy(); q[i] += h
        fp = M.loss_and_grad(q, X, T)[0]
        q[i] -= 2 * h
        fm = M.loss_and_grad(q, X, T)[0]
        assert abs((fp - fm) / (2 * h) - g[i]) <= 1e-6 * max(1.0, abs(g[i])), i


def test_oracle_scan_objective_matches_direct_statement():
    """Two-alignment scan mode (plmDCA_objective.hpp:67): the target is a
    column of the second alignment and no feature locus is excluded.  The
    oracle against a direct numpy statement of the objective and gradient."""
    from oracle import oracle as O
    rng = np.random.default_rng(8)
    N, L, LT = 40, 21, 3
    st = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
    tg = rng.integers(0, 4, size=(N, LT)).astype(np.uint8)
    w = rng.uniform(0.2, 1.0, N)
    lh, lJ = 0.7, 0.3
    P = O.Problem(st, w, lh, lJ, targets=tg)
    I = O.ref_index(L)
    oh = np.eye(4)[st]                                  # N L s
    for r in range(LT):
        x = rng.normal(size=16 * L + 4) * 0.3
        J = x[I]                                        # [n][s][a]
        h = x[16 * L:]
        l = h + np.einsum('ins,nsa->ia', oh, J)
        m = l.max(1, keepdims=True)
        lse = (m + np.log(np.exp(l - m).sum(1, keepdims=True)))[:, 0]
        y = tg[:, r]
        f = (w * (lse - l[np.arange(N), y])).sum() + lh * (h ** 2).sum() + lJ * (J ** 2).sum()
        R = w[:, None] * (np.exp(l - lse[:, None]) - np.eye(4)[y])
        gJ = np.einsum('ins,ia->nsa', oh, R) + 2 * lJ * J
        gh = R.sum(0) + 2 * lh * h
        fo, go = P.objective(r, x)
        assert fo == pytest.approx(f, rel=1e-12)
        np.testing.assert_allclose(go[I], gJ, rtol=0, atol=1e-11)
        np.testing.assert_allclose(go[16 * L:], gh, rtol=0, atol=1e-11)
