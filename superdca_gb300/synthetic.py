"""Seeded synthetic alignments with the shapes of the benchmark workloads.

The real genome alignments behind SuperDCA's published coupling tables are not
available, so these generators stand in for them with the stated shapes and
value distributions (all in the 5-letter nucleotide alphabet, codes A0 C1 G2
T3 gap4):

  independent   N x L biallelic loci, MAF ~ U(0.01, 0.5), per-locus gap rate
                ~ U(0, 0.10), planted pairs where the minor allele at b
                follows the minor allele at a with probability 0.8
                (default 200 x 500, 20 pairs);
  tree          a random coalescent (Kingman-topology) binary tree over N
                leaves; the root is a random biallelic sequence and every
                branch flips each locus with probability 0.05; planted pairs
                copy locus a's allele into locus b with probability 0.8;
                3% gaps (3000 x 10,000 with 200 pairs, or 3000 x 94,000);
  skewed        N x L loci, 10% multiallelic (3-4 alleles), MAF ~ Beta(0.5, 2)
                floored at 0.01, gap rate ~ U(0, 0.15) (616 x 78,700).
"""
from __future__ import annotations

import numpy as np

from .alignment import encode


def _pairs(rng, L, n_pairs):
    n_pairs = min(n_pairs, L // 2)
    idx = rng.permutation(L)[: 2 * n_pairs]
    return idx.reshape(n_pairs, 2)


def independent(N=200, L=500, n_pairs=20, seed=0):
    rng = np.random.default_rng(seed)
    alle = np.stack([rng.permutation(4)[:2] for _ in range(L)])  # major, minor
    maf = rng.uniform(0.01, 0.5, size=L)
    gap = rng.uniform(0.0, 0.10, size=L)
    minor = rng.random((N, L)) < maf[None, :]
    pairs = _pairs(rng, L, n_pairs)
    for a, b in pairs:
        follow = rng.random(N) < 0.8
        minor[:, b] |= minor[:, a] & follow
    nuc = np.where(minor, alle[None, :, 1], alle[None, :, 0]).astype(np.uint8)
    nuc[rng.random((N, L)) < gap[None, :]] = 4
    return nuc, pairs


def _kingman_children(rng, N):
    """Random binary tree by repeated random joins; returns child lists."""
    active = list(range(N))
    children = {}
    nxt = N
    while len(active) > 1:
        i, j = rng.choice(len(active), size=2, replace=False)
        a, b = active[i], active[j]
        children[nxt] = (a, b)
        for k in sorted((i, j), reverse=True):
            active.pop(k)
        active.append(nxt)
        nxt += 1
    return children, active[0]


def tree(N=3000, L=10000, n_pairs=200, flip=0.05, gap=0.03, seed=0, chunk=16384):
    rng = np.random.default_rng(seed)
    children, root = _kingman_children(rng, N)
    order = [root]
    for node in order:
        if node in children:
            order.extend(children[node])
    alle = np.stack([rng.permutation(4)[:2] for _ in range(L)])
    root_bits = rng.integers(0, 2, size=L, dtype=np.uint8)
    leaves = np.empty((N, L), dtype=np.uint8)
    nnodes = 2 * N - 1
    for c0 in range(0, L, chunk):
        C = min(chunk, L - c0)
        bits = np.empty((nnodes, C), dtype=np.uint8)
        bits[root] = root_bits[c0:c0 + C]
        for node in order:
            if node not in children:
                continue
            for ch in children[node]:
                row = bits[node].copy()
                k = rng.binomial(C, flip)
                if k:
                    pos = rng.integers(0, C, size=k)
                    row[pos] ^= 1
                bits[ch] = row
        leaves[:, c0:c0 + C] = bits[:N]
    pairs = _pairs(rng, L, n_pairs)
    for a, b in pairs:
        copy = rng.random(N) < 0.8
        leaves[copy, b] = leaves[copy, a]
    nuc = np.where(leaves == 1, alle[None, :, 1], alle[None, :, 0]).astype(np.uint8)
    nuc[rng.random((N, L), dtype=np.float32) < gap] = 4
    return nuc, pairs


def skewed(N=616, L=78700, n_pairs=100, multi_frac=0.10, seed=0):
    rng = np.random.default_rng(seed)
    nuc = np.empty((N, L), dtype=np.uint8)
    gap = rng.uniform(0.0, 0.15, size=L)
    multi = rng.random(L) < multi_frac
    for c0 in range(0, L, 4096):
        C = min(4096, L - c0)
        u = rng.random((N, C))
        for j in range(C):
            l = c0 + j
            perm = rng.permutation(4)
            if multi[l]:
                k = rng.integers(3, 5)
                p = rng.dirichlet(np.ones(k))
                cdf = np.cumsum(p)
                col = perm[np.searchsorted(cdf, u[:, j], side="right").clip(0, k - 1)]
            else:
                maf = min(0.5, max(0.01, rng.beta(0.5, 2.0)))
                col = np.where(u[:, j] < maf, perm[1], perm[0])
            nuc[:, l] = col
    nuc[rng.random((N, L), dtype=np.float32) < gap[None, :]] = 4
    pairs = _pairs(rng, L, n_pairs)
    for a, b in pairs:
        copy = rng.random(N) < 0.8
        nuc[copy, b] = nuc[copy, a]
    return nuc, pairs


WORKLOADS = {
    # name: (generator, kwargs)
    "independent-200x500": (independent, dict(N=200, L=500, n_pairs=20)),
    "tree-3000x10000": (tree, dict(N=3000, L=10000, n_pairs=200)),
    "tree-3000x94000": (tree, dict(N=3000, L=94000, n_pairs=200)),
    "skewed-616x78700": (skewed, dict(N=616, L=78700, n_pairs=100)),
}


def workload(name: str, seed: int = 0, **over):
    """Generate, filter and encode a named workload.

    Returns (states N x L' uint8 codes 0..3, kept columns, planted pairs)."""
    gen, kw = WORKLOADS[name]
    kw = {**kw, **over}
    nuc, pairs = gen(seed=seed, **kw)
    states, cols = encode(nuc)
    return states, cols, pairs
