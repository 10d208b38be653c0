"""The digit scheme of the exact K rho product (k_kdig) at its limits, in
numpy integers and float32: K < 2^18 as three base-64 digits, |rho_q| <= 2^27
as four balanced base-128 digits, N <= 4000 sequences.  Every digit-pair
product must stay below 4096 and every sum over the sequences below 2^24
(so the FP32 accumulators are exact), and the combination with weights
2^(6k + 7p) must give K rho exactly."""
import numpy as np


def split_k(K):
    return [K & 63, (K >> 6) & 63, K >> 12]


def split_rho(v):
    v = v.astype(np.int64).copy()
    out = []
    for _ in range(3):
        d = ((v + 64) & 127) - 64          # balanced digit; v - d divisible by 128
        out.append(d)
        v = (v - d) // 128
    out.append(v)
    return out


def test_digit_bounds_at_the_extremes():
    lim = 2 ** 27
    v = np.array([lim, -lim, lim - 1, -(lim - 1), 64 * (1 + 128 + 128 ** 2), -64 * (1 + 128 + 128 ** 2), 0, 1, -1,
                  int(lim * (1 + 2.0 ** -23))], dtype=np.int64)
    ds = split_rho(v)
    for d in ds[:3]:
        assert np.all(np.abs(d) <= 64)
    assert np.all(np.abs(ds[3]) <= 65)
    back = sum(d * 128 ** p for p, d in enumerate(ds))
    np.testing.assert_array_equal(back, v)
    K = np.array([0, 1, 63, 64, 4095, 4096, 2 ** 18 - 1], dtype=np.int64)
    kd = split_k(K)
    assert all(np.all((d >= 0) & (d <= 63)) for d in kd)
    np.testing.assert_array_equal(kd[0] + 64 * kd[1] + 4096 * kd[2], K)
    assert 63 * 65 < 4096


def test_worst_case_sums_are_exact_in_fp32():
    """N = 4000 products of the largest digits, summed in float32 one at a
    time (any order a tensor-core accumulator might take), stay exact."""
    N = 4000
    prods = np.full(N, 63 * 65, dtype=np.float32)
    acc = np.float32(0.0)
    for p in prods:
        acc = np.float32(acc + p)
    assert int(acc) == 63 * 65 * N and 63 * 65 * N < 2 ** 24


def test_combination_reproduces_k_rho():
    rng = np.random.default_rng(7)
    N = 4000
    K = rng.integers(0, 2 ** 18, size=(64, N), dtype=np.int64)
    K[:, :8] = 2 ** 18 - 1
    rho = rng.integers(-2 ** 27, 2 ** 27 + 1, size=(N, 4), dtype=np.int64)
    rho[:8] = 2 ** 27
    exact = K @ rho
    kd, rd = split_k(K), split_rho(rho)
    total = np.zeros_like(exact)
    for k in range(3):
        for p in range(4):
            # each digit-pair product in float32, as the TMEM accumulator holds it
            part32 = kd[k].astype(np.float32) @ rd[p].astype(np.float32)
            part = kd[k] @ rd[p]
            np.testing.assert_array_equal(part32.astype(np.int64), part)
            assert np.abs(part).max() < 2 ** 24
            total += part * (1 << (6 * k + 7 * p))
    np.testing.assert_array_equal(total, exact)


def test_solution_digit_planes_are_exact():
    """The reported J = Phi^T a_x: A = round(a qa) with |A| <= 2^32 split into
    A = D0 2^22 + D1 2^11 + D2 (|D| <= 2^10, exact in fp16); each one-hot
    contraction sum over at most 16383 sequences stays below 2^24, and the
    64-bit combination gives the integer sum of A."""
    rng = np.random.default_rng(11)
    N = 16383
    A = rng.integers(-2 ** 32, 2 ** 32 + 1, size=N, dtype=np.int64)
    A[:4] = [2 ** 32, -2 ** 32, 2 ** 32 - 1, -(2 ** 32 - 1)]
    d0 = (A + (1 << 21)) >> 22
    r0 = A - (d0 << 22)
    d1 = (r0 + (1 << 10)) >> 11
    d2 = r0 - (d1 << 11)
    for d in (d0, d1, d2):
        assert np.abs(d).max() <= 1024
    np.testing.assert_array_equal((d0 << 22) + (d1 << 11) + d2, A)
    state = rng.integers(0, 4, size=N)
    for s in range(4):
        m = state == s
        G = [np.float32(0.0)] * 3
        for k, d in enumerate((d0, d1, d2)):
            G[k] = np.sum(d[m].astype(np.float32), dtype=np.float32)
            assert abs(int(G[k])) < 2 ** 24 and int(G[k]) == int(d[m].sum())
        J = int(G[0]) * (1 << 22) + int(G[1]) * (1 << 11) + int(G[2])
        assert J == int(A[m].sum())
    assert 16383 * 1024 < 2 ** 24


def test_three_columns_give_the_fourth():
    """Rows of rho_q made to sum to zero exactly (the own-state entry set to
    minus the sum of the others, as the quantiser does): the product needs
    three columns, the fourth of K rho - csum is minus their sum."""
    rng = np.random.default_rng(3)
    N, L = 500, 3000
    y = rng.integers(0, 4, size=N)
    p = rng.dirichlet(np.ones(4), size=N)
    R = p - np.eye(4)[y]
    q = np.rint(R * 2 ** 27).astype(np.int64)
    q[np.arange(N), y] = 0
    q[np.arange(N), y] = -q.sum(1)
    assert np.all(q.sum(1) == 0) and np.abs(q).max() <= 2 ** 27 + 2
    K = rng.integers(0, L, size=(N, N), dtype=np.int64)
    csum = np.stack([q[y == a].sum(0) for a in range(4)])
    full = K @ q - csum[y]
    three = K @ q[:, :3] - csum[y][:, :3]
    np.testing.assert_array_equal(full[:, :3], three)
    np.testing.assert_array_equal(full[:, 3], -three.sum(1))
