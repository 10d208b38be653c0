"""sdca_eval_noalloc: the objective + gradient evaluation for host programs
that do not let a library allocate device memory (their own allocator owns
all of it).  The caller hands in device buffers it allocated; the library's
intermediates live in its fixed scratch array.

This file is collected last on purpose: a failure here leaves every other
test already run.  It must pass both alone in a fresh process and after the
other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, d_states, N, L, d_w, lh, lJ, r, d_x, d_f, d_g, stream):
    p = lambda t: C.c_void_p(t.data_ptr())
    return lib.sdca_eval_noalloc(p(d_states), N, L, p(d_w), lh, lJ, r, p(d_x), p(d_f), p(d_g),
                                 None if stream is None else C.c_void_p(stream.cuda_stream))


# (333, 37): one partial-sum block per pass and a partial last 16-locus block;
# (700, 600): several blocks in both passes, so the cross-block sums run
@pytest.mark.parametrize("N,L,loci", [(333, 37, (5, 33)), (700, 600, (0, 599))])
def test_eval_noalloc_matches_eval(engine_lib, oracle_mod, N, L, loci):
    import torch

    from superdca_gb300 import Engine, _lib

    lib = engine_lib
    rng = np.random.default_rng(2024 + L)
    st = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
    w = rng.uniform(0.2, 1.0, size=N)
    E = Engine(N, L)
    E.set_alignment(st, w)
    lh, lJ, _ = E.lambdas()
    P = oracle_mod.Problem(st, w, lh, lJ)
    D = 16 * L + 4

    # the caller's own device buffers
    dev = torch.device("cuda", 0)
    d_states = torch.from_numpy(st).to(dev)
    d_w = torch.from_numpy(w).to(dev)
    d_x = torch.empty(D, dtype=torch.float64, device=dev)
    d_f = torch.empty(1, dtype=torch.float64, device=dev)
    d_g = torch.empty(D, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    # two calls in a row, each against the allocating entry point and the
    # FP64 oracle directly
    for r in loci:
        x = rng.normal(size=D) * 0.2
        d_x.copy_(torch.from_numpy(x))
        d_f.fill_(float("nan"))
        d_g.fill_(float("nan"))
        assert _call(lib, d_states, N, L, d_w, lh, lJ, r, d_x, d_f, d_g, stream) == _lib.SDCA_OK
        stream.synchronize()
        f, g = float(d_f.cpu()[0]), d_g.cpu().numpy()
        f_ref, g_ref = E.eval(r, x)
        assert f == pytest.approx(f_ref, rel=1e-6)
        np.testing.assert_allclose(g, g_ref, rtol=0, atol=1e-4 * max(1.0, np.abs(g_ref).max()))
        f_orc, g_orc = P.objective(r, x)
        assert f == pytest.approx(f_orc, rel=1e-6)
        np.testing.assert_allclose(g, g_orc, rtol=0, atol=1e-4 * max(1.0, np.abs(g_orc).max()))

    # sizes beyond the fixed scratch array are refused before any work
    assert _call(lib, d_states, 65537, L, d_w, lh, lJ, 0, d_x, d_f, d_g, None) == _lib.SDCA_E_ARG
    assert _call(lib, d_states, N, 262145, d_w, lh, lJ, 0, d_x, d_f, d_g, None) == _lib.SDCA_E_ARG
    E.close()


def test_eval_noalloc_state_code_out_of_range(engine_lib):
    """A code >= 4 cannot be refused on the host (the states are device
    memory): the kernels read it masked to 0..3, so every load stays in
    bounds, and report it as a NaN objective.  The next call, with valid
    codes, is unaffected."""
    import torch

    from superdca_gb300 import _lib

    lib = engine_lib
    rng = np.random.default_rng(9)
    N, L = 64, 20
    st = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
    dev = torch.device("cuda", 0)
    d_w = torch.ones(N, dtype=torch.float64, device=dev)
    d_x = torch.zeros(16 * L + 4, dtype=torch.float64, device=dev)
    d_f = torch.empty(1, dtype=torch.float64, device=dev)
    d_g = torch.empty(16 * L + 4, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    bad = st.copy()
    bad[3, 7] = 5
    d_bad = torch.from_numpy(bad).to(dev)
    assert _call(lib, d_bad, N, L, d_w, 0.01, 0.01, 2, d_x, d_f, d_g, stream) == _lib.SDCA_OK
    stream.synchronize()
    assert np.isnan(float(d_f.cpu()[0]))
    d_ok = torch.from_numpy(st).to(dev)
    assert _call(lib, d_ok, N, L, d_w, 0.01, 0.01, 2, d_x, d_f, d_g, stream) == _lib.SDCA_OK
    stream.synchronize()
    # at x = 0 every sequence's softmax is uniform: f = sum_i w_i log 4
    assert float(d_f.cpu()[0]) == pytest.approx(N * np.log(4.0), rel=1e-12)
