"""Host-side logic and the C ABI surface (no GPU compute)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def test_library_exports_every_declared_symbol(engine_lib):
    header = open(os.path.join(ROOT, "include", "superdca_gb300.h")).read()
    declared = sorted(set(re.findall(r"\b(sdca_\w+)\s*\(", header)))
    assert "sdca_solve" in declared and "sdca_eval" in declared
    from superdca_gb300 import _lib

    assert sorted(_lib.EXPORTS) == declared
    for name in declared:
        assert hasattr(engine_lib, name), name
    assert engine_lib.sdca_abi_version() == 2


def test_config_defaults_follow_superdca_options(engine_lib):
    from superdca_gb300 import _lib

    cfg = _lib.Config()
    assert engine_lib.sdca_config_default(C.byref(cfg)) == 0
    # plmDCA_options.cpp: lambda -1 (automatic), gradient threshold 1e-3;
    # plmDCA.hpp:218-221: 2000 iterations; history 10; q = 4, GAP = 3
    assert (cfg.q, cfg.gap_state, cfg.lambda_h, cfg.lambda_J) == (4, 3, -1.0, -1.0)
    assert (cfg.gradient_threshold, cfg.max_iterations, cfg.history) == (1e-3, 2000, 10)


def test_create_rejects_bad_arguments(engine_lib):
    from superdca_gb300 import _lib

    cfg = _lib.Config()
    engine_lib.sdca_config_default(C.byref(cfg))
    h = C.c_void_p()
    cfg.n_seqs, cfg.n_loci, cfg.q = 10, 10, 5
    assert engine_lib.sdca_create(C.byref(cfg), C.byref(h)) == _lib.SDCA_E_UNSUPPORTED
    assert b"q = 4" in engine_lib.sdca_last_error(None)
    cfg.q, cfg.n_loci = 4, 1
    assert engine_lib.sdca_create(C.byref(cfg), C.byref(h)) == _lib.SDCA_E_ARG
    cfg.n_loci, cfg.history = 10, 11
    assert engine_lib.sdca_create(C.byref(cfg), C.byref(h)) == _lib.SDCA_E_ARG
    assert engine_lib.sdca_create(None, C.byref(h)) == _lib.SDCA_E_ARG
    assert engine_lib.sdca_destroy(None) == 0


def two_loop(S, Y, g, gamma):
    """CppNumericalSolvers' two-loop recursion (columns oldest first)."""
    q = g.copy()
    k = S.shape[1]
    alpha = np.zeros(k)
    for i in range(k - 1, -1, -1):
        rho = 1.0 / (S[:, i] @ Y[:, i])
        alpha[i] = rho * (S[:, i] @ q)
        q = q - alpha[i] * Y[:, i]
    q = gamma * q
    for i in range(k):
        rho = 1.0 / (S[:, i] @ Y[:, i])
        beta = rho * (Y[:, i] @ q)
        q = q + S[:, i] * (alpha[i] - beta)
    return q


@pytest.mark.parametrize("k", [1, 2, 5, 10])
def test_compact_lbfgs_equals_two_loop(engine_lib, k):
    rng = np.random.default_rng(k)
    D = 40
    A = rng.normal(size=(D, D))
    H = A @ A.T + D * np.eye(D)  # SPD curvature so that s.y > 0
    S = rng.normal(size=(D, k))
    Y = H @ S + 0.01 * rng.normal(size=(D, k))
    g = rng.normal(size=D)
    gamma = (S[:, -1] @ Y[:, -1]) / (Y[:, -1] @ Y[:, -1])
    SY = S.T @ Y
    R = np.triu(SY)
    YY = Y.T @ Y
    sg, yg = S.T @ g, Y.T @ g
    cg = C.c_double()
    cS, cY = np.zeros(k), np.zeros(k)
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data
    R_, YY_ = np.ascontiguousarray(R), np.ascontiguousarray(YY)
    rc = engine_lib.sdca_internal_lbfgs_coeffs(k, f(R_), f(YY_), f(sg), f(yg), gamma, C.byref(cg),
                                               cS.ctypes.data, cY.ctypes.data)
    assert rc == 0
    d = cg.value * g + S @ cS + Y @ cY
    np.testing.assert_allclose(d, -two_loop(S, Y, g, gamma), rtol=1e-9, atol=1e-12)


def test_encode_filter_and_triallelic_rules():
    from superdca_gb300.alignment import encode, nucleotide_codes

    seqs = [
        # c0: monomorphic  c1: A/C 1 minor of 5  c2: A/G/T  c3: A/C/G/T  c4: gappy  c5: C/T tie
        "AAAAGC",
        "ACGCAT",
        "AAAG-C",
        "AATT-T",
        "AAGA-C",
    ]
    nuc = nucleotide_codes(seqs)
    assert nuc[3, 4] == 4 and nuc[0, 0] == 0
    st, cols = encode(nuc, maf_threshold=0.2, gap_threshold=0.5)
    # c0 one allele: dropped; c1 MAF 0.2 kept; c2 kept; c3 four alleles:
    # dropped; c4 gap 3/5 > 0.5 dropped; c5 kept
    assert list(cols) == [1, 2, 5]
    # c1: A (4) rank 0, C (1) rank 1
    assert list(st[:, 0]) == [0, 1, 0, 0, 0]
    # c2: A x3 rank0, G x1 / T x1 tie -> G rank 1, T rank 2
    assert list(st[:, 1]) == [0, 1, 0, 2, 1]
    # c5: C x3, T x2 -> C 0, T 1
    assert list(st[:, 2]) == [0, 1, 0, 1, 0]
    # gaps map to state 3
    st2, cols2 = encode(nucleotide_codes(["AC", "A-", "CC", "C-"]), maf_threshold=0.0,
                        gap_threshold=1.0)
    assert list(cols2) == [0] and list(st2[:, 0]) == [0, 0, 1, 1]
    st3, cols3 = encode(nucleotide_codes(["AC", "A-", "CC", "G-"]), filter_alignment=False)
    assert list(cols3) == [0, 1]
    assert list(st3[:, 1]) == [0, 3, 0, 3]


def test_coupling_lines_format():
    from superdca_gb300 import coupling_lines, format_coupling_lines

    S = np.array([[np.nan, 0.25, 0.5], [0.75, np.nan, 0.125], [0.375, 0.0625, np.nan]], dtype=np.float32)
    lines = coupling_lines(S, [0, 1, 2])
    # for r in the list, n before r: (S[r][n] + S[n][r]) / 2, 1-based indices
    assert lines == [((0.75 + 0.25) / 2, 2, 1), ((0.375 + 0.5) / 2, 3, 1),
                     ((0.0625 + 0.125) / 2, 3, 2)]
    txt = format_coupling_lines(lines)
    assert txt.splitlines()[0] == "0.50000000 2 1"
    # original column numbering through a translation table
    lines = coupling_lines(S, [0, 1, 2], translation=[4, 9, 11])
    assert [(r, n) for _, r, n in lines] == [(10, 5), (12, 5), (12, 10)]


def test_synthetic_workloads_are_seeded():
    from superdca_gb300 import synthetic

    a, ca, pa = synthetic.workload("independent-200x500", seed=3)
    b, cb, pb = synthetic.workload("independent-200x500", seed=3)
    c, _, _ = synthetic.workload("independent-200x500", seed=4)
    assert np.array_equal(a, b) and np.array_equal(ca, cb) and np.array_equal(pa, pb)
    assert not np.array_equal(a, c)
    assert a.max() <= 3 and a.shape[0] == 200
    t, ct, _ = synthetic.workload("tree-3000x10000", seed=1, N=64, L=300)
    assert t.shape[0] == 64 and t.max() <= 3


def test_ctypes_structs_match_the_header_layout(tmp_path):
    """The ctypes mirrors of sdca_config, sdca_locus_stat, sdca_profile and
    sdca_tune_entry have the C compiler's sizes and field offsets."""
    import shutil
    import subprocess

    from superdca_gb300 import _lib

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"sdca_config": _lib.Config, "sdca_locus_stat": _lib.LocusStat, "sdca_profile": _lib.Profile,
               "sdca_tune_entry": _lib.TuneEntry}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "superdca_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l}
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
