"""Two-alignment scan mode: the target loci are the columns of a second
alignment of the same sequences (plmDCA_objective.hpp:67, plmDCA.hpp:338-346,
370-377, 484-490), every locus of the first a feature, none excluded, and the
scores taken from the blocks as stored.  Each engine form against the FP64
oracle run in the same mode; the command line end to end."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scan_data(seed=3, N=180, L=70, LT=9):
    rng = np.random.default_rng(seed)
    feats = rng.integers(0, 2, size=(N, L)).astype(np.uint8) * rng.integers(1, 3, size=(1, L)).astype(np.uint8)
    tg = np.empty((N, LT), dtype=np.uint8)
    for k in range(LT):                 # targets copy a feature column with noise
        src = feats[:, rng.integers(0, L)].copy()
        flip = rng.random(N) < 0.15
        src[flip] = rng.integers(0, 4, size=flip.sum())
        tg[:, k] = src
    feats[rng.random((N, L)) < 0.03] = 3
    return feats, tg


@pytest.mark.parametrize("form", ["dual", "tc", "gather"])
def test_scan_mode_matches_oracle(oracle_mod, form):
    from superdca_gb300 import _lib
    from superdca_gb300.engine import Engine
    O = oracle_mod
    feats, tg = _scan_data()
    N, L = feats.shape
    LT = tg.shape[1]
    w = np.random.default_rng(4).uniform(0.3, 1.0, N)
    fm = {"dual": _lib.FORM_DUAL, "tc": _lib.FORM_TC, "gather": _lib.FORM_GATHER}[form]
    with Engine(N, L, form=fm, batch=4) as E:
        E.set_alignment(feats, w)
        E.set_targets(tg)
        lh, lJ, _ = E.lambdas()
        res = E.solve(np.arange(LT), want_x=True)
        f_eval, g_eval = E.eval(2, res.x[2])
        with pytest.raises(_lib.EngineError):
            E.solve([LT])                      # loci index target columns
        E.set_targets(None)
        back = E.solve([0, 1])                 # the single-alignment mode again
    P = O.Problem(feats, w, lh, lJ, targets=tg)
    assert np.all(res.status == 0)
    f_at = np.array([P.objective(k, res.x[k], grad=False) for k in range(LT)])
    np.testing.assert_allclose(res.f, f_at, rtol=1e-6)
    sc, st = P.solve(np.arange(LT), threads=4)
    np.testing.assert_allclose(res.f, [s["f"] for s in st], rtol=1e-6)
    assert not np.isnan(res.scores).any()       # no excluded block
    np.testing.assert_allclose(res.scores, sc, rtol=0, atol=1e-4)
    for k in range(LT):
        g = P.objective(k, res.x[k])[1]
        assert np.abs(g).max() < 1.05e-3
    fo, go = P.objective(2, res.x[2])
    assert f_eval == pytest.approx(fo, rel=1e-6)
    np.testing.assert_allclose(g_eval, go, rtol=0, atol=1e-4 * max(1.0, np.abs(go).max()))
    P1 = O.Problem(feats, w, lh, lJ)
    np.testing.assert_allclose(back.f, [s["f"] for s in P1.solve([0, 1])[1]], rtol=1e-6)


def test_cli_scan_mode(oracle_mod, tmp_path):
    from superdca_gb300 import alignment as A
    from superdca_gb300 import build, synthetic
    O = oracle_mod
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cli = build.build_cli()
    nuc, _ = synthetic.independent(N=160, L=110, n_pairs=5, seed=21)
    nucA, nucB = nuc[:, :30], nuc[:, 30:]
    A.write_fasta(str(tmp_path / "tgt.fasta"), nucA)
    A.write_fasta(str(tmp_path / "feat.fasta"), nucB)
    r = subprocess.run([cli, "--output-weights", "tgt.fasta", "feat.fasta"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    sA, cA = A.encode(nucA)
    sB, cB = A.encode(nucB)
    w = O.weights(sB, 0.9)
    np.testing.assert_allclose(np.loadtxt(tmp_path / "tgt.weights"), w, rtol=1e-8)
    lh, lJ = O.lambdas(w)[:2]
    sc, _ = O.Problem(sB, w, lh, lJ, targets=sA).solve(np.arange(sA.shape[1]), threads=os.cpu_count() or 1)
    lines = (tmp_path / "tgt_scan.SuperDCA_couplings.1-based.all").read_text().splitlines()
    assert len(lines) == sA.shape[1] * sB.shape[1]
    k = 0
    for rr in range(sA.shape[1]):
        for nn in range(sB.shape[1]):
            v, a, b = lines[k].split()
            k += 1
            assert (int(a), int(b)) == (cA[rr] + 1, cB[nn] + 1)
            assert abs(float(v) - sc[rr, nn]) < 1e-4
    # two engines on device 0, each taking part of every 7-target call:
    # the same lines in the same order, values within the oracle tolerance
    # (the stop iterate of a locus depends on its batch neighbours)
    (tmp_path / "tgt2.fasta").write_bytes((tmp_path / "tgt.fasta").read_bytes())
    r = subprocess.run([cli, "--gpu-devices", "0,0", "--gpu-chunk", "7", "tgt2.fasta", "feat.fasta"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    two = (tmp_path / "tgt2_scan.SuperDCA_couplings.1-based.all").read_text().splitlines()
    assert [l.split()[1:] for l in two] == [l.split()[1:] for l in lines]
    np.testing.assert_allclose([float(l.split()[0]) for l in two], [float(l.split()[0]) for l in lines],
                               rtol=0, atol=1e-4)
