"""sdca_eval_noalloc: the objective + gradient evaluation for callers that
cannot allocate device memory themselves through the library -- code running
while a CUDA graph is being captured, or a host program whose own allocator
owns all device memory.  The caller hands in device buffers it allocated;
the library's intermediates live in its fixed scratch array.

This file is collected last on purpose: a failure here leaves every other
test already run.  It must pass both alone in a fresh process and after the
other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_eval_noalloc_matches_eval(engine_lib):
    import torch

    from superdca_gb300 import Engine, _lib

    lib = engine_lib
    rng = np.random.default_rng(2024)
    N, L = 333, 37  # ragged: a partial last 16-locus block
    st = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
    w = rng.uniform(0.2, 1.0, size=N)
    E = Engine(N, L)
    E.set_alignment(st, w)
    lh, lJ, _ = E.lambdas()
    D = 16 * L + 4

    # the caller's own device buffers
    dev = torch.device("cuda", 0)
    d_states = torch.from_numpy(st).to(dev)
    d_w = torch.from_numpy(w).to(dev)
    d_x = torch.empty(D, dtype=torch.float64, device=dev)
    d_f = torch.empty(1, dtype=torch.float64, device=dev)
    d_g = torch.empty(D, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    p = lambda t: C.c_void_p(t.data_ptr())

    # two calls in a row, each against the allocating entry point
    for r in (5, 33):
        x = rng.normal(size=D) * 0.2
        d_x.copy_(torch.from_numpy(x))
        d_f.fill_(float("nan"))
        d_g.fill_(float("nan"))
        rc = lib.sdca_eval_noalloc(p(d_states), N, L, p(d_w), lh, lJ, r, p(d_x), p(d_f), p(d_g),
                                   C.c_void_p(stream.cuda_stream))
        assert rc == _lib.SDCA_OK
        stream.synchronize()
        f_ref, g_ref = E.eval(r, x)
        f, g = float(d_f.cpu()[0]), d_g.cpu().numpy()
        assert f == pytest.approx(f_ref, rel=1e-6)
        np.testing.assert_allclose(g, g_ref, rtol=0, atol=1e-4 * max(1.0, np.abs(g_ref).max()))

    # sizes beyond the fixed scratch array are refused before any work
    rc = lib.sdca_eval_noalloc(p(d_states), 65537, L, p(d_w), lh, lJ, 0, p(d_x), p(d_f), p(d_g), None)
    assert rc == _lib.SDCA_E_ARG
    rc = lib.sdca_eval_noalloc(p(d_states), N, 262145, p(d_w), lh, lJ, 0, p(d_x), p(d_f), p(d_g), None)
    assert rc == _lib.SDCA_E_ARG
    E.close()
