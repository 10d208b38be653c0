"""The superdca-gb300 command line: SuperDCA's flow from FASTA to coupling file.

CPU tests hold the C++ parser, filter and 4-state encoding to the rules of
superdca_gb300/alignment.py and check the side outputs (.fasta, .loci,
.weights) and the file-name uniquifier of SuperDCA_commons.h:66-81.  The GPU
test runs the whole program and compares the coupling file with the oracle's
solves of the same encoded alignment."""
import os
import subprocess

import numpy as np
import pytest

from superdca_gb300 import alignment as A
from superdca_gb300 import synthetic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "superdca_gb300", "superdca-gb300")


@pytest.fixture(scope="module")
def cli():
    from superdca_gb300 import build
    if not os.path.exists(os.path.join(ROOT, "superdca_gb300", "libsuperdca_gb300.so")):
        pytest.skip("engine library not built")
    build.build_cli()
    return CLI


def run(cli, args, cwd):
    return subprocess.run([cli, *args], cwd=cwd, capture_output=True, text=True, timeout=600)


def messy_alignment(seed=0, N=60, L=400):
    """Nucleotides with every case the rules distinguish: gaps as '-' and 'N',
    lower case, monomorphic, rare-allele, gappy and four-allele columns."""
    rng = np.random.default_rng(seed)
    nuc = rng.integers(0, 4, size=(N, L)).astype(np.uint8)
    nuc[:, 0:20] = nuc[0, 0:20]                                  # monomorphic
    nuc[:, 20:40] = 0
    nuc[0, 20:40] = 2                                            # MAF 1/60 above 0.01
    nuc[:, 40:60] = rng.integers(0, 2, size=(N, 20))
    blk = nuc[:, 40:60]
    blk[rng.random((N, 20)) < 0.3] = 4                            # gappy
    nuc[:, 60:80] = rng.integers(0, 3, size=(N, 20))              # three alleles
    nuc[rng.random((N, L)) < 0.02] = 4
    return nuc


def write_messy_fasta(path, nuc, seed=0):
    rng = np.random.default_rng(seed + 1)
    with open(path, "w") as f:
        for i, row in enumerate(nuc):
            s = "".join("ACGT-"[v] for v in row)
            s = "".join(c.lower() if rng.random() < 0.1 else c for c in s)
            s = "".join("N" if (c == "-" and rng.random() < 0.5) else c for c in s)
            f.write(f">sample_{i} some description\n")
            for k in range(0, len(s), 70):                       # wrapped lines
                f.write(s[k:k + 70] + "\n")


def test_cli_help_and_option_errors(cli, tmp_path):
    r = run(cli, ["--help"], tmp_path)
    assert r.returncode == 0 and "--gradient-threshold" in r.stdout and "--no-reweighting" in r.stdout
    r = run(cli, ["--no-such-flag", "x.fasta"], tmp_path)
    assert r.returncode == 1 and "unrecognised option" in r.stderr
    r = run(cli, [], tmp_path)
    assert r.returncode == 1 and "no input alignment" in r.stderr
    r = run(cli, ["--gradient-threshold", "abc", "x.fasta"], tmp_path)
    assert r.returncode == 1 and "invalid value" in r.stderr
    r = run(cli, ["missing.fasta"], tmp_path)
    assert r.returncode == 1 and "cannot open" in r.stderr
    for bad in ("0,,1", "0,x", "", "0,"):
        r = run(cli, ["--gpu-devices", bad, "x.fasta"], tmp_path)
        assert r.returncode == 1 and "invalid value" in r.stderr, bad
    r = run(cli, ["--gpu-devices", "0,-1", "x.fasta"], tmp_path)
    assert r.returncode == 1 and "--gpu-devices entries must be >= 0" in r.stderr
    (tmp_path / "bad.fasta").write_text(">a\nACGT\n>b\nACG\n")
    r = run(cli, ["bad.fasta"], tmp_path)
    assert r.returncode == 1 and "has length 3, expected 4" in r.stderr
    r = run(cli, ["a.fasta", "b.fasta", "c.fasta"], tmp_path)
    assert r.returncode == 1 and "at most two alignment files" in r.stderr
    (tmp_path / "b.fasta").write_text(">a\nACGT\n")
    r = run(cli, ["bad.fasta", "b.fasta"], tmp_path)
    assert r.returncode == 1


def test_cli_filter_encode_and_side_outputs(cli, tmp_path):
    nuc = messy_alignment()
    write_messy_fasta(tmp_path / "aln.fasta", nuc)
    names, seqs = A.read_fasta(str(tmp_path / "aln.fasta"))
    parsed = A.nucleotide_codes(seqs)
    assert np.array_equal(parsed, nuc)

    args = ["--no-reweighting", "--no-dca", "--output-filtered-alignment", "--output-weights",
            "aln.fasta"]
    r = run(cli, args, tmp_path)
    assert r.returncode == 0, r.stderr
    # the filtered alignment is written next to the input: aln.fasta exists, so .1
    cols = A.filter_columns(nuc)
    got_loci = np.loadtxt(tmp_path / "aln.loci", dtype=np.int64, ndmin=1)
    assert np.array_equal(got_loci, cols + 1)
    fn, fs = A.read_fasta(str(tmp_path / "aln.fasta.1"))
    assert fn == names
    assert np.array_equal(A.nucleotide_codes(fs), nuc[:, cols])
    w = (tmp_path / "aln.weights").read_text().splitlines()
    assert w == ["1.00000000e+00"] * nuc.shape[0]

    # a second run finds every name taken and appends .1 / .2
    r = run(cli, args, tmp_path)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "aln.loci.1").exists() and (tmp_path / "aln.weights.1").exists()
    assert (tmp_path / "aln.fasta.2").exists()

    # thresholds and --no-filter-alignment
    r = run(cli, ["--no-reweighting", "--no-dca", "--output-filtered-alignment", "--maf-threshold", "0.2",
                  "--gap-threshold=0.05", "--output-indexing-base", "0", "aln.fasta"], tmp_path)
    assert r.returncode == 0, r.stderr
    got = np.loadtxt(tmp_path / "aln.loci.2", dtype=np.int64, ndmin=1)
    assert np.array_equal(got, A.filter_columns(nuc, 0.2, 0.05))


def test_cli_filter_and_sample_lists(cli, tmp_path):
    nuc = messy_alignment(seed=3)
    write_messy_fasta(tmp_path / "aln.fasta", nuc, seed=3)
    sel_cols = [5, 61, 62, 300, 301, 399, 61]          # 1-based, with a duplicate
    (tmp_path / "keep.txt").write_text("# loci\n" + ", ".join(str(c) for c in sel_cols) + "\n")
    (tmp_path / "samples.txt").write_text("1 3 5\n7\n60\n")
    r = run(cli, ["--no-reweighting", "--no-dca", "--filterlistfile", "keep.txt", "--output-filterlist-alignment",
                  "--samplelistfile", "samples.txt", "--output-samplelist-alignment", "aln.fasta"], tmp_path)
    assert r.returncode == 0, r.stderr
    cols = sorted(set(c - 1 for c in sel_cols))
    _, fs = A.read_fasta(str(tmp_path / "aln.fasta.1"))
    assert np.array_equal(A.nucleotide_codes(fs), nuc[:, cols])
    rows = [0, 2, 4, 6, 59]
    _, ss = A.read_fasta(str(tmp_path / "samples.fasta"))
    assert np.array_equal(A.nucleotide_codes(ss), nuc[np.ix_(rows, cols)])
    (tmp_path / "bad.txt").write_text("0\n")
    r = run(cli, ["--no-reweighting", "--no-dca", "--filterlistfile", "bad.txt", "aln.fasta"], tmp_path)
    assert r.returncode == 1 and "below the index base" in r.stderr


@pytest.mark.gpu
def test_gpu_cli_couplings_match_oracle(cli, tmp_path, oracle_mod):
    """Full run: GPU reweighting, GPU solves of every locus, coupling file.
    Lines, their order and indices exactly; values within 1e-4."""
    O = oracle_mod
    nuc, _ = synthetic.independent(N=200, L=500, seed=7)
    A.write_fasta(str(tmp_path / "ind.fasta"), nuc, width=60)
    r = run(cli, ["-v", "--output-weights", "--gpu-batch", "32", "ind.fasta"], tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    states, cols = A.encode(nuc)
    w_ref = O.weights(states, 0.9)
    w_got = np.loadtxt(tmp_path / "ind.weights")
    np.testing.assert_allclose(w_got, w_ref, rtol=1e-8, atol=0)
    lh, lJ = O.lambdas(w_ref)[:2]
    P = O.Problem(states, w_ref, lh, lJ)
    L = states.shape[1]
    loci = np.arange(L)
    scores, st = P.solve(loci, threads=os.cpu_count() or 1)
    from superdca_gb300.engine import coupling_lines
    want = coupling_lines(scores, loci, translation=cols, base=1)
    got = (tmp_path / "ind.SuperDCA_couplings.1-based.all").read_text().splitlines()
    assert len(got) == len(want) == L * (L - 1) // 2
    vals = np.array([float(g.split()[0]) for g in got])
    idx = [tuple(int(t) for t in g.split()[1:]) for g in got]
    assert idx == [(rr, nn) for _, rr, nn in want]
    assert all(len(g.split()[0].split(".")[1]) == 8 for g in got[:100])
    np.testing.assert_allclose(vals, [v for v, _, _ in want], rtol=0, atol=1e-4)


@pytest.mark.gpu
def test_gpu_cli_warm_start_same_couplings(cli, tmp_path):
    """--gpu-warm-start with the committed per-sequence blob: the optimum of
    each locus is unique, so the coupling file matches the zero-start run's
    (same lines and order, values within 1e-4)."""
    import shutil
    nuc, _ = synthetic.independent(N=200, L=300, seed=8)
    A.write_fasta(str(tmp_path / "a.fasta"), nuc, width=60)
    shutil.copy(tmp_path / "a.fasta", tmp_path / "b.fasta")
    blob = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "superdca_gb300",
                        "warmstart_dual_tree-3000x94000.npy")
    r0 = run(cli, ["--gpu-batch", "32", "a.fasta"], tmp_path)
    r1 = run(cli, ["--gpu-batch", "32", "--gpu-warm-start", blob, "b.fasta"], tmp_path)
    assert r0.returncode == 0 and r1.returncode == 0, r0.stderr + r1.stderr
    z = (tmp_path / "a.SuperDCA_couplings.1-based.all").read_text().splitlines()
    w = (tmp_path / "b.SuperDCA_couplings.1-based.all").read_text().splitlines()
    assert len(z) == len(w) > 0   # (the MAF filter may drop columns; the same ones in both runs)
    assert [l.split()[1:] for l in z] == [l.split()[1:] for l in w]
    np.testing.assert_allclose([float(l.split()[0]) for l in w], [float(l.split()[0]) for l in z], rtol=0, atol=1e-4)
    (tmp_path / "bad.bin").write_bytes(b"\x00" * 12)
    r2 = run(cli, ["--gpu-batch", "32", "--gpu-warm-start", "bad.bin", "a.fasta"], tmp_path)
    assert r2.returncode == 1 and "learned start rejected" in r2.stderr


@pytest.mark.gpu
def test_gpu_cli_devices_share_the_loci(cli, tmp_path):
    """--gpu-devices: one engine per listed device, each solving a contiguous
    share of the loci list on its own host thread.  Two engines on device 0
    give the single-engine coupling file: the same lines in the same order,
    values within 1e-4 (a slot's exact stop test waits for a few slots to
    want one, so the iterate a locus stops at, below the gradient threshold
    either way, depends on the loci it shares a batch with).  Small calls
    (--gpu-chunk 13) make each engine solve several."""
    import shutil
    nuc, _ = synthetic.independent(N=180, L=260, seed=9)
    A.write_fasta(str(tmp_path / "one.fasta"), nuc, width=60)
    shutil.copy(tmp_path / "one.fasta", tmp_path / "two.fasta")
    flags = ["--gpu-batch", "24", "--gpu-lanes", "2", "--gpu-chunk", "13"]
    r1 = run(cli, [*flags, "one.fasta"], tmp_path)
    r2 = run(cli, ["-v", *flags, "--gpu-devices", "0,0", "two.fasta"], tmp_path)
    assert r1.returncode == 0 and r2.returncode == 0, r1.stderr + r2.stderr
    assert "2 engines, on devices 0 0" in r2.stdout
    one = (tmp_path / "one.SuperDCA_couplings.1-based.all").read_text().splitlines()
    two = (tmp_path / "two.SuperDCA_couplings.1-based.all").read_text().splitlines()
    assert len(one) == len(two) > 0
    assert [l.split()[1:] for l in one] == [l.split()[1:] for l in two]
    np.testing.assert_allclose([float(l.split()[0]) for l in two], [float(l.split()[0]) for l in one],
                               rtol=0, atol=1e-4)


def _gauge(M):
    """SuperDCA's ising_gauge as it evaluates (row means spread along columns),
    in single precision."""
    M = M.astype(np.float32)
    rm = M.sum(1, dtype=np.float32) / np.float32(4)
    cm = M.sum(0, dtype=np.float32) / np.float32(4)
    gm = rm.sum(dtype=np.float32) / np.float32(4)
    return ((M - rm[None, :]) - cm[:, None]) + gm


def _frob(G, gap=3):
    keep = [i for i in range(4) if i != gap]
    return float(np.sqrt((G[np.ix_(keep, keep)].astype(np.float64) ** 2).sum()))


@pytest.mark.gpu
def test_gpu_cli_norm_of_mean_top_k_and_binary(cli, tmp_path, oracle_mod):
    """--norm-of-mean-scoring (plmDCA.hpp:335-363, 617-666) against blocks
    from the oracle's solutions; --gpu-top-k and --gpu-binary-output against
    the text file of the same run."""
    O = oracle_mod
    nuc, _ = synthetic.independent(N=150, L=90, n_pairs=6, seed=11)
    A.write_fasta(str(tmp_path / "nm.fasta"), nuc)
    r = run(cli, ["--no-reweighting", "--norm-of-mean-scoring", "nm.fasta"], tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    states, cols = A.encode(nuc)
    N, L = states.shape
    w = np.ones(N)
    lh, lJ = O.lambdas(w)[:2]
    _, _, xs = O.Problem(states, w, lh, lJ).solve(np.arange(L), threads=os.cpu_count() or 1, want_x=True)
    I = O.ref_index(L)

    def block(r, n):
        J = xs[r][I[n]]                      # [s][a]
        return (J.T if n < r else J).astype(np.float32)

    got = (tmp_path / "nm.SuperDCA_couplings.1-based.all").read_text().splitlines()
    assert len(got) == L * (L - 1) // 2
    k = 0
    for rr in range(L):
        for nn in range(rr):
            f = got[k].split()
            k += 1
            assert (int(f[1]), int(f[2])) == (cols[rr] + 1, cols[nn] + 1)
            Ga, Gb = _gauge(block(rr, nn)), _gauge(block(nn, rr))
            want = [_frob((Ga + Gb) * np.float32(0.5)), _frob(Ga), _frob(Gb)]
            np.testing.assert_allclose([float(f[0]), float(f[3]), float(f[4])], want, rtol=0, atol=1e-4)
            assert abs(float(f[5]) - 0.5 * (float(f[3]) + float(f[4]))) < 2e-8

    r = run(cli, ["--no-reweighting", "--gpu-top-k", "25", "--gpu-binary-output", "nm.fasta"], tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    text = (tmp_path / "nm.SuperDCA_couplings.1-based.all.1").read_text().splitlines()
    vals = np.array([float(t.split()[0]) for t in text])
    recs = np.fromfile(tmp_path / "nm.SuperDCA_couplings.1-based.bin", dtype=[("v", "<f4"), ("r", "<i4"), ("n", "<i4")])
    assert len(recs) == len(text)
    np.testing.assert_allclose(recs["v"].astype(np.float64), vals, rtol=0, atol=1e-8)
    assert [(int(t.split()[1]), int(t.split()[2])) for t in text] == list(zip(recs["r"].tolist(), recs["n"].tolist()))
    top = (tmp_path / "nm.SuperDCA_couplings.1-based.top25").read_text().splitlines()
    assert len(top) == 25
    np.testing.assert_allclose([float(t.split()[0]) for t in top], np.sort(vals)[::-1][:25], rtol=0, atol=1e-8)
