"""The algebra the dual form rests on, checked on the CPU against the FP64
oracle (plmDCA_objective.hpp:86-151, 192-244 restated in oracle/).

For target locus r, with phi_i sequence i's one-hot features over the loci
n != r and K_ij = #{n != r : s_i(n) = s_j(n)}: a point x = (J, h) with
J = Phi^T a (J_r[n][s][c] = sum_j a_jc [s_j(n) = s], J_rr = 0) and h = eta has
  logits   l_i = (K a)_i + eta,
  f        = sum_i w_i (lse(l_i) - l_i[s_i(r)]) + lambda_J a . K a + lambda_h |eta|^2,
  gradient g_J = Phi^T (rho + 2 lambda_J a),  g_h = sum_i rho_i + 2 lambda_h eta,
with rho_i = w_i (softmax(l_i) - onehot(s_i(r))).  The engine's dual form
evaluates exactly these expressions; here numpy does, in FP64."""
import numpy as np
import pytest


def _phi_t(states, r, a):
    """J = Phi^T a in the engine's [n][s][c] order, J_rr = 0."""
    N, L = states.shape
    J = np.zeros((L, 4, 4))
    for n in range(L):
        if n == r:
            continue
        for s in range(4):
            J[n, s, :] = a[states[:, n] == s].sum(axis=0)
    return J


def _kmat(states, r):
    agree = (states[:, None, :] == states[None, :, :]).sum(axis=2)
    own = (states[:, None, r] == states[None, :, r]).astype(int)
    return agree - own


@pytest.mark.parametrize("seed,N,L,r", [(0, 23, 9, 4), (1, 40, 17, 0), (2, 7, 5, 4)])
def test_dual_point_matches_the_oracle(oracle_mod, seed, N, L, r):
    O = oracle_mod
    rng = np.random.default_rng(seed)
    states = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
    states[rng.random((N, L)) < 0.1] = 3          # gaps are a state like the others
    w = rng.uniform(0.2, 1.0, N)
    lh, lJ = O.lambdas(w)[:2]
    P = O.Problem(states, w, lh, lJ)

    a = rng.normal(scale=0.05, size=(N, 4))
    eta = rng.normal(scale=0.1, size=4)
    J = _phi_t(states, r, a)
    idx = O.ref_index(L)
    x = np.zeros(O.dim(L))
    x[idx.ravel()] = J.ravel()
    x[16 * L:16 * L + 4] = eta
    f_ref, g_ref = P.objective(r, x)

    K = _kmat(states, r)
    logits = K @ a + eta
    m = logits.max(axis=1, keepdims=True)
    lse = (m + np.log(np.exp(logits - m).sum(axis=1, keepdims=True)))[:, 0]
    y = states[:, r].astype(int)
    f_dual = (w * (lse - logits[np.arange(N), y])).sum() + lJ * np.sum(a * (K @ a)) + lh * eta @ eta
    assert f_dual == pytest.approx(f_ref, rel=1e-12)

    p = np.exp(logits - lse[:, None])
    rho = w[:, None] * (p - np.eye(4)[y])
    gJ = _phi_t(states, r, rho + 2.0 * lJ * a)
    gJ[r] = 2.0 * lJ * J[r]                       # the oracle's own block: only the L2 term (J_rr = 0)
    g = np.zeros(O.dim(L))
    g[idx.ravel()] = gJ.ravel()
    g[16 * L:16 * L + 4] = rho.sum(axis=0) + 2.0 * lh * eta
    np.testing.assert_allclose(g, g_ref, rtol=1e-10, atol=1e-12)

    # inner products in the dual: <Phi^T a, Phi^T b> = a . K b
    b = rng.normal(size=(N, 4))
    assert np.sum(J * _phi_t(states, r, b)) == pytest.approx(np.sum(a * (K @ b)), rel=1e-12)


def test_agreement_matrix_from_hamming_distances():
    """K = L - d - [s_i(r) = s_j(r)]: the engine builds it from the reweighting
    kernel's Hamming distances d and a class sum per state of r."""
    rng = np.random.default_rng(3)
    states = rng.integers(0, 4, size=(31, 12)).astype(np.uint8)
    N, L = states.shape
    d = (states[:, None, :] != states[None, :, :]).sum(axis=2)
    for r in (0, 5, 11):
        K = L - d - (states[:, None, r] == states[None, :, r])
        np.testing.assert_array_equal(K, _kmat(states, r))
        # K rho = K_all rho - (class sum of rho over the sequences sharing i's state at r)
        rho = rng.integers(-1000, 1000, size=(N, 4))
        K_all = L - d
        cls = np.stack([rho[states[:, r] == s].sum(axis=0) for s in range(4)])
        np.testing.assert_array_equal(K @ rho, K_all @ rho - cls[states[:, r]])
