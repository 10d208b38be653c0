"""The learned warm start: network kernels, pair statistics, and what the
trained network gains over the zero start of SuperDCA
(SuperDCA/include/plmDCA.hpp:298) on held-out data.

The network's gradients are checked against the FP64 CPU restatement in
oracle/mlp_oracle.py; the pair statistics against numpy; and a solve with the
warm start must reach the same objective (rel 1e-6, the tolerance of the
converged-objective tests) in fewer iterations."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_mlp_gradient_matches_cpu_oracle(engine_lib):
    from oracle import mlp_oracle as MO
    from superdca_gb300 import warmstart as W
    rng = np.random.default_rng(0)
    for M in (1, 300, 5000):
        X = rng.normal(size=(M, 40)).astype(np.float32)
        J = (rng.normal(size=(M, 16)) * 0.01).astype(np.float32)
        blob = W.new_blob(X, J, seed=M)
        blob[W.B1:W.W2] = rng.normal(size=128) * 0.1
        blob[W.B2:W.W3] = rng.normal(size=128) * 0.1
        T = W.targets(blob, J)
        lg, gg = W.grad(blob, X, T)
        lc, gc = MO.loss_and_grad(blob, X, T)
        assert lg == pytest.approx(lc, rel=1e-5)
        # FP32 kernels against FP64: 1e-4 of the largest gradient entry
        assert np.abs(gg - gc).max() <= 1e-4 * np.abs(gc).max()
        assert np.all(gg[:W.W1] == 0) and np.all(gg[W.TRAIN_END:] == 0)
        # the tensor-core forward (BF16 weights and activations, FP32 sums):
        # against its own arithmetic restated on the CPU, and against FP64
        out = W.predict(blob, X)
        emu = MO.forward_bf16(blob, X)
        ref = MO.forward(blob, X)[3]
        scale = max(1.0, np.abs(ref).max())
        assert np.abs(out - emu).max() <= 2e-3 * scale
        assert np.abs(out - ref).max() <= 3e-2 * scale


@pytest.mark.parametrize("M", [1, 127, 128, 129, 40000, 100003])
def test_mlp_tensor_core_forward_ragged_rows(engine_lib, M):
    """Row counts around the 128-row tile and beyond one tile per CTA."""
    from oracle import mlp_oracle as MO
    from superdca_gb300 import warmstart as W
    rng = np.random.default_rng(M)
    X = rng.normal(size=(M, 40)).astype(np.float32)
    blob = W.new_blob(X, rng.normal(size=(M, 16)).astype(np.float32) * 0.1, seed=3)
    blob[W.B1:W.W2] = rng.normal(size=128) * 0.1
    blob[W.B3:W.TRAIN_END] = rng.normal(size=16) * 0.1
    out = W.predict(blob, X)
    emu = MO.forward_bf16(blob, X)
    assert out.shape == (M, 16) and np.all(np.isfinite(out))
    assert np.abs(out - emu).max() <= 2e-3 * max(1.0, np.abs(emu).max())


def test_mlp_training_fits_a_teacher(engine_lib):
    """Adam on the GPU recovers a random teacher network of the same shape."""
    from oracle import mlp_oracle as MO
    from superdca_gb300 import warmstart as W
    rng = np.random.default_rng(1)
    X = rng.normal(size=(20000, 40)).astype(np.float32)
    teacher = W.new_blob(X, np.ones((2, 16), np.float32), seed=7)
    T = MO.forward(teacher, X)[3].astype(np.float32)
    student = W.new_blob(X, np.ones((2, 16), np.float32), seed=8)
    l0 = MO.loss_and_grad(student, X, T)[0]
    trained, losses = W.train(student, X, T, epochs=40, batch=1024, lr=2e-3)
    l1 = MO.loss_and_grad(trained, X, T)[0]
    assert np.all(np.isfinite(losses))
    assert l1 < 0.05 * l0, (l0, l1, losses[-3:])


def test_ws_features_match_numpy(engine_lib):
    """Pair statistics: joint and residual-weighted joint frequencies with the
    k-nearest-neighbour residuals, against numpy (weighted, ragged sizes)."""
    from superdca_gb300 import _lib, synthetic
    from superdca_gb300.engine import Engine
    states, _, _ = synthetic.workload("tree-3000x10000", seed=9, N=301, L=700)
    n, L = states.shape
    w = np.random.default_rng(1).uniform(0.3, 1.0, n)
    onehot = np.eye(4)[states]
    d = (states[:, None, :] != states[None, :, :]).sum(2)
    np.fill_diagonal(d, 10 ** 9)
    for k, eps in ((3, 0.5), (1, 0.0), (8, 2.0)):
        nn = np.argsort(d, axis=1, kind="stable")[:, :k]
        with Engine(n, L, form=_lib.FORM_GATHER, batch=8) as E:
            E.set_alignment(states, w)
            loci = np.array([0, 5, 77, L - 1, 300])
            F = E.ws_features(loci, k, eps)
            sel = np.stack([np.arange(0, L, 7)[:50] for _ in loci])
            Fs = E.ws_features(loci, k, eps, sel)
        beff = w.sum()
        for t, r in enumerate(loci):
            y = onehot[:, r]
            fr = (w[:, None] * y).sum(0) / beff
            ph = (y[nn].sum(1) + eps * fr) / (k + eps)
            joint = np.einsum('ins,ia->nsa', onehot, w[:, None] * y) / beff
            resid = np.einsum('ins,ia->nsa', onehot, w[:, None] * (ph - y)) / beff
            ref = np.concatenate([joint.reshape(L, 16), resid.reshape(L, 16), joint.sum(2), joint.sum(1)], 1)
            np.testing.assert_allclose(F[t], ref, rtol=0, atol=2e-6)
            np.testing.assert_array_equal(Fs[t], F[t][sel[t]])


@pytest.mark.parametrize("form", ["tc", "gather"])
def test_warm_start_same_optimum_fewer_iterations(engine_lib, form):
    """Train on two tree alignments, solve loci of a third (held out) with and
    without the warm start: the same optimum, fewer iterations."""
    from superdca_gb300 import _lib, synthetic
    from superdca_gb300 import warmstart as W
    from superdca_gb300.engine import Engine
    N, L = 1000, 4000
    fm = _lib.FORM_TC if form == "tc" else _lib.FORM_GATHER
    blob, losses = W.train_on_workload("tree-3000x10000", [31, 32], 128, 512, epochs=30, form=fm,
                                       sizes=dict(N=N, L=L), log=lambda *a: None)
    assert losses[-1] < 0.2 * losses[0]
    states, _, _ = synthetic.workload("tree-3000x10000", seed=33, N=N, L=L)
    n, Lf = states.shape
    with Engine(n, Lf, form=fm, batch=32) as E:
        E.set_alignment(states, np.ones(n))
        loci = np.random.default_rng(5).choice(Lf, 64, replace=False)
        zero = E.solve(loci)
        E.set_warm_start(blob)
        warm = E.solve(loci)
        E.set_warm_start(None)
        again = E.solve(loci[:8])
    assert np.all(zero.status == 0) and np.all(warm.status == 0)
    np.testing.assert_allclose(warm.f, zero.f, rtol=1e-6)
    np.testing.assert_allclose(again.f, zero.f[:8], rtol=1e-6)   # disabled again
    gain = 1.0 - warm.iterations.mean() / zero.iterations.mean()
    print(f"\n[{form}] mean iterations zero start {zero.iterations.mean():.1f}, "
          f"warm start {warm.iterations.mean():.1f} ({100 * gain:.1f} % fewer)")
    assert gain > 0.03


def test_set_warm_start_rejects_bad_blobs(engine_lib):
    from superdca_gb300 import _lib
    from superdca_gb300 import warmstart as W
    from superdca_gb300._lib import EngineError
    from superdca_gb300.engine import Engine
    rng = np.random.default_rng(0)
    X = rng.normal(size=(10, 40)).astype(np.float32)
    good = W.new_blob(X, np.ones((10, 16), np.float32))
    with Engine(10, 20, form=_lib.FORM_GATHER, batch=2) as E:
        for bad in (good[:-1], np.where(np.arange(W.SIZE) == 0, 2, good), np.where(np.arange(W.SIZE) == 1, 17, good),
                    np.where(np.arange(W.SIZE) == W.W2, np.nan, good)):
            with pytest.raises(EngineError):
                E.set_warm_start(bad.astype(np.float32))
        E.set_warm_start(good)
        E.set_warm_start(None)


def test_dual_warm_start_same_optimum_fewer_iterations(engine_lib):
    """The dual form's per-sequence start (blob version 2): trained on the
    engine's own converged residuals of two tree alignments, it must reach
    the same objective on a held-out alignment in fewer iterations."""
    from superdca_gb300 import _lib, synthetic
    from superdca_gb300 import warmstart as W
    from superdca_gb300.engine import Engine
    N, L = 1000, 4000
    blob, losses = W.train_dual_on_workload("tree-3000x10000", [31, 32], 128, alpha=0.4, epochs=15,
                                            sizes=dict(N=N, L=L), batch_slots=64, log=lambda *a: None)
    assert np.all(np.isfinite(losses)) and losses[-1] < losses[0]
    states, _, _ = synthetic.workload("tree-3000x10000", seed=33, N=N, L=L)
    n, Lf = states.shape
    with Engine(n, Lf, form=_lib.FORM_DUAL, batch=32) as E:
        E.set_alignment(states, np.ones(n))
        loci = np.random.default_rng(5).choice(Lf, 64, replace=False)
        zero = E.solve(loci)
        E.set_warm_start(blob)
        warm = E.solve(loci)
        E.set_warm_start(None)
        again = E.solve(loci[:8])
    assert np.all(zero.status == 0) and np.all(warm.status == 0)
    np.testing.assert_allclose(warm.f, zero.f, rtol=1e-6)
    np.testing.assert_allclose(again.f, zero.f[:8], rtol=1e-6)
    np.testing.assert_allclose(warm.scores, zero.scores, atol=1e-4, equal_nan=True)
    gain = 1.0 - warm.iterations.mean() / zero.iterations.mean()
    print(f"\n[dual] mean iterations zero start {zero.iterations.mean():.1f}, "
          f"warm start {warm.iterations.mean():.1f} ({100 * gain:.1f} % fewer)")
    assert gain > 0.03
