"""The single-precision step trial of the dual form (k_trial_delta), restated
in numpy float32, against FP64 on badly fitted sequences and large steps.

Per sequence, with base probabilities p0 (the softmax of the logits at the
current point), state y at r and t_a = stp (u_a - u_y):
  dl = log Z,  Z = sum_a p0_a exp(t_a)   (log1p(q), q = sum_a p0_a expm1(t_a), near Z = 1)
  p_a(stp) = p0_a exp(t_a) / Z
The change dl keeps ~1e-7 relative error of itself, and every new probability
keeps its relative precision (products of positive terms), also where a
probability has become tiny: a form p0 + (p - p0) built by differences does
not, and carried over iterations such noise was amplified by later steps."""
import numpy as np

f32 = np.float32


def trial32(p0, du, stp):
    t = (f32(stp) * du).astype(f32)
    e = np.expm1(t).astype(f32)
    x = (p0 * np.exp(t)).astype(f32)
    q = np.sum(p0 * e, axis=1, dtype=f32)
    z = np.sum(x, axis=1, dtype=f32)
    dl = np.log(z).astype(f32)
    small = np.abs(q) < 0.5
    dl[small] = np.log1p(q[small])
    p = (x / z[:, None]).astype(f32)
    return dl, p


def truth64(l0, u, y, stp):
    def lse(l):
        m = l.max(axis=1, keepdims=True)
        return (m + np.log(np.exp(l - m).sum(axis=1, keepdims=True)))[:, 0]
    l1 = l0 + stp * u
    dl = (lse(l1) - l1[np.arange(len(y)), y]) - (lse(l0) - l0[np.arange(len(y)), y])
    p1 = np.exp(l1 - lse(l1)[:, None])
    return dl, p1


def test_trial_change_and_probabilities_keep_their_precision():
    rng = np.random.default_rng(5)
    n = 20000
    y = rng.integers(0, 4, size=n)
    l0 = rng.normal(scale=3.0, size=(n, 4))
    # badly fitted sequences: the observed state far below the others
    bad = rng.random(n) < 0.3
    l0[bad, y[bad]] -= rng.uniform(8.0, 14.0, size=bad.sum())
    u = rng.normal(scale=2.0, size=(n, 4))
    p0_64 = np.exp(l0 - l0.max(axis=1, keepdims=True))
    p0_64 /= p0_64.sum(axis=1, keepdims=True)
    p0 = p0_64.astype(f32)
    du = (u - u[np.arange(n), y][:, None]).astype(f32)
    for stp in (1e-3, 0.1, 1.0, 4.0):
        t = np.abs(stp * du).max(axis=1)
        keep = t < 29.0                      # larger steps take the FP64 path
        dl32, p32 = trial32(p0, du, stp)
        dl64, p64 = truth64(l0, u, y, stp)
        err = np.abs(dl32[keep] - dl64[keep])
        assert np.all(err <= 2e-6 * np.abs(dl64[keep]) + 1e-6 * np.maximum(1.0, t[keep])), stp
        rel = np.abs(p32[keep] - p64[keep]) / np.maximum(p64[keep], 1e-30)
        assert np.all(rel[p64[keep] > 1e-30] < 5e-5), stp   # relative, also for tiny probabilities


def test_differences_lose_tiny_probabilities():
    """The form p0 + (p - p0) (the residual built by differences) cannot
    represent a probability far below the ulp of p0: the product form can."""
    p0 = np.array([[0.5, 0.5 - 1e-9, 1e-9, 0.0]], dtype=np.float64)
    p0[0, 3] = 1.0 - p0[0, :3].sum()
    du = np.array([[0.0, -25.0, 0.0, 0.0]], dtype=f32)
    _, p_prod = trial32(p0.astype(f32), du, 1.0)
    true = p0[0, 1] * np.exp(-25.0) / (p0[0, 0] + p0[0, 1] * np.exp(-25.0) + p0[0, 2] + p0[0, 3])
    assert abs(p_prod[0, 1] - true) / true < 1e-5
    diff_form = f32(p0[0, 1]) + (f32(true) - f32(p0[0, 1]))      # p0 + dp in float32
    assert abs(diff_form - true) / true > 1e-2
