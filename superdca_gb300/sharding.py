"""Several GPUs: the loci list split over ranks, score rows gathered on rank 0.

SuperDCA's per-locus solves are independent (the TBB loop over loci,
SuperDCA/include/plmDCA.hpp:581-586); the alignment and the weights are
replicated.  The one exchange is the symmetrisation of the coupling writer
(plmDCA.hpp:667-693), which needs S[r][n] and S[n][r]: every rank solves a
contiguous part of the loci list on its own GPU, with no collective during the
solve, and the score rows are then gathered on rank 0 over torch.distributed
(NCCL between GPUs, gloo on the host).
"""
from __future__ import annotations

import numpy as np


def shard(n_loci: int, rank: int, world: int) -> slice:
    """Contiguous part of a list of n_loci entries owned by rank (sizes differ
    by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    q, r = divmod(int(n_loci), world)
    lo = rank * q + min(rank, r)
    return slice(lo, lo + q + (1 if rank < r else 0))


def solve_sharded(solve_rows, loci, L: int, group=None, rows_per_message: int = 1024):
    """Solve `loci` over all ranks of `group` and gather the score rows.

    solve_rows(local_loci) -> float32 array (len(local_loci) x L), the rows
    of this rank's part (normally `Engine.solve(...).scores`).  Returns the
    full len(loci) x L float32 array on rank 0 and None elsewhere.  Rows travel
    in messages of at most rows_per_message rows, padded to equal size."""
    import torch
    import torch.distributed as dist

    loci = np.asarray(loci)
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    part = shard(len(loci), rank, world)
    local = np.asarray(solve_rows(loci[part]), dtype=np.float32).reshape(-1, L)
    if local.shape[0] != part.stop - part.start:
        raise ValueError("solve_rows returned the wrong number of rows")
    parts = [shard(len(loci), k, world) for k in range(world)]
    longest = max(p.stop - p.start for p in parts)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    out = np.empty((len(loci), L), dtype=np.float32) if rank == 0 else None
    for m0 in range(0, longest, rows_per_message):
        m = min(rows_per_message, longest - m0)
        buf = torch.zeros((m, L), dtype=torch.float32)
        have = max(0, min(m, local.shape[0] - m0))
        if have:
            buf[:have] = torch.from_numpy(local[m0:m0 + have])
        buf = buf.to(dev)
        # only rank 0 keeps rows: point-to-point sends to it (works on gloo
        # and NCCL alike), so no other rank receives anyone's rows
        if rank == 0:
            for k, p in enumerate(parts):
                if k == 0:
                    got = buf
                else:
                    got = torch.empty_like(buf)
                    dist.recv(got, src=dist.get_global_rank(group, k) if group is not None else k, group=group)
                n_k = max(0, min(m, (p.stop - p.start) - m0))
                if n_k:
                    out[p.start + m0:p.start + m0 + n_k] = got[:n_k].cpu().numpy()
        else:
            dist.send(buf, dst=dist.get_global_rank(group, 0) if group is not None else 0, group=group)
    return out
