"""Alignment encoding: nucleotide columns -> filtered 4-state codes.

SuperDCA reads a FASTA genome alignment, keeps loci with more than one allele
(gaps not counted), minor allele frequency at least 1% and gap frequency at
most 15% (README.md, "Basic usage"; --maf-threshold / --gap-threshold /
--no-filter-alignment), then forces every locus into a 4-state envelope of up
to three alleles plus gap ("some loci may be dropped",
SuperDCA/src/SuperDCA.cpp:349-360).  Those steps live in apegrunt, a SuperDCA
submodule that is absent, so the rules below are written from the README and
the call sites and are not pinned against apegrunt itself:

  * nucleotide input codes: A=0 C=1 G=2 T=3, gap (-, N and any other symbol)=4;
  * allele counts ignore gaps; alleles are ranked by count, ties by A<C<G<T;
  * minor allele frequency = count of the second-ranked allele / non-gap count;
  * gap frequency = gaps / sequences;
  * keep a locus iff alleles > 1, MAF >= maf_threshold, gap frequency <=
    gap_threshold, and alleles <= 3 (a fourth allele does not fit the
    envelope, so the locus is dropped);
  * 4-state code = allele rank (0, 1, 2), gap = 3 (the GAP state left out of
    the coupling norm).
"""
from __future__ import annotations

import numpy as np

NUC = "ACGT-"
GAP_CODE = 4
STATE_GAP = 3


def nucleotide_codes(seqs: list[str]) -> np.ndarray:
    """FASTA sequence strings -> uint8 codes A0 C1 G2 T3, everything else 4."""
    lut = np.full(256, GAP_CODE, dtype=np.uint8)
    for c, v in zip("ACGT", range(4)):
        lut[ord(c)] = v
        lut[ord(c.lower())] = v
    L = len(seqs[0])
    out = np.empty((len(seqs), L), dtype=np.uint8)
    for i, s in enumerate(seqs):
        if len(s) != L:
            raise ValueError("sequences of unequal length")
        out[i] = lut[np.frombuffer(s.encode("ascii"), dtype=np.uint8)]
    return out


def _column_counts(nuc: np.ndarray) -> np.ndarray:
    N, L = nuc.shape
    counts = np.zeros((L, 5), dtype=np.int64)
    step = max(1, (1 << 26) // max(N, 1))
    for c0 in range(0, L, step):
        blk = nuc[:, c0:c0 + step]
        for v in range(5):
            counts[c0:c0 + step, v] = (blk == v).sum(axis=0)
    return counts


def filter_columns(nuc: np.ndarray, maf_threshold: float = 0.01, gap_threshold: float = 0.15) -> np.ndarray:
    """The MAF / gap filter: columns with more than one allele, minor allele
    frequency >= maf_threshold and gap frequency <= gap_threshold."""
    nuc = np.ascontiguousarray(nuc, dtype=np.uint8)
    N = nuc.shape[0]
    counts = _column_counts(nuc)
    allele = counts[:, :4]
    nalleles = (allele > 0).sum(axis=1)
    second = -np.sort(-allele, axis=1)[:, 1]
    nongap = N - counts[:, 4]
    maf = np.where(nongap > 0, second / np.maximum(nongap, 1), 0.0)
    gapf = counts[:, 4] / N
    return np.nonzero((nalleles > 1) & (maf >= maf_threshold) & (gapf <= gap_threshold))[0]


def four_state(nuc: np.ndarray):
    """The 4-state envelope: drop columns with four alleles, code the others by
    allele rank (0, 1, 2) with gap = 3.  Returns (states, kept columns)."""
    nuc = np.ascontiguousarray(nuc, dtype=np.uint8)
    N, L = nuc.shape
    counts = _column_counts(nuc)
    allele = counts[:, :4]
    nalleles = (allele > 0).sum(axis=1)
    # rank alleles by count, ties by nucleotide order (stable sort on -count)
    order = np.argsort(-allele, axis=1, kind="stable")
    cols = np.nonzero(nalleles <= 3)[0]
    rank = np.empty((L, 4), dtype=np.uint8)
    np.put_along_axis(rank, order, np.arange(4, dtype=np.uint8)[None, :].repeat(L, 0), axis=1)
    lut = np.full((len(cols), 5), STATE_GAP, dtype=np.uint8)
    lut[:, :4] = np.minimum(rank[cols], 3)
    out = np.empty((N, len(cols)), dtype=np.uint8)
    step = max(1, (1 << 26) // max(N, 1))
    for c0 in range(0, len(cols), step):
        cc = cols[c0:c0 + step]
        sub = nuc[:, cc]
        out[:, c0:c0 + step] = lut[np.arange(c0, c0 + len(cc))[None, :], sub]
    return out, cols


def encode(nuc: np.ndarray, maf_threshold: float = 0.01, gap_threshold: float = 0.15,
           filter_alignment: bool = True):
    """Filter and encode an N x L nucleotide-code matrix.

    Returns (states N x L' uint8 in 0..3, kept original column indices)."""
    nuc = np.ascontiguousarray(nuc, dtype=np.uint8)
    cols = filter_columns(nuc, maf_threshold, gap_threshold) if filter_alignment else np.arange(nuc.shape[1])
    states, kept = four_state(nuc[:, cols])
    return states, cols[kept]


def read_fasta(path: str):
    """(names, sequences) of a FASTA file; sequences may span several lines."""
    names, seqs = [], []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\r\n")
            if not line or line.startswith(";"):
                continue
            if line.startswith(">"):
                names.append(line[1:])
                seqs.append([])
            else:
                if not seqs:
                    raise ValueError("sequence data before the first header")
                seqs[-1].append("".join(line.split()))
    return names, ["".join(s) for s in seqs]


def write_fasta(path: str, nuc: np.ndarray, names=None, width: int = 0):
    """Write nucleotide codes as FASTA (width > 0 wraps the sequence lines)."""
    with open(path, "w") as f:
        for i, row in enumerate(np.asarray(nuc)):
            f.write(f">{names[i] if names else f'seq{i}'}\n")
            s = "".join(NUC[v] for v in row)
            if width:
                for k in range(0, len(s), width):
                    f.write(s[k:k + width] + "\n")
            else:
                f.write(s + "\n")
