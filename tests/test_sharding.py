"""Loci sharded over ranks: two gloo ranks on the CPU.

The rows each rank solves here come from the oracle (the solve itself is
tested on the GPU elsewhere); what is under test is the split of the loci
list, the gather of score rows on rank 0 and the coupling lines built from
them, which must equal the single-process result exactly."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from superdca_gb300.sharding import shard, solve_sharded


def test_shard_covers_list_once():
    for n in (0, 1, 2, 7, 64, 1001):
        for world in (1, 2, 3, 8):
            parts = [shard(n, r, world) for r in range(world)]
            idx = np.concatenate([np.arange(n)[p] for p in parts]) if n else np.array([])
            assert np.array_equal(idx, np.arange(n))
            sizes = [p.stop - p.start for p in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def _problem():
    from superdca_gb300 import synthetic
    from superdca_gb300.alignment import encode
    nuc, _ = synthetic.independent(N=80, L=60, n_pairs=4, seed=5)
    states, cols = encode(nuc)
    return states, cols


def _rank_main(rank, world, port, loci, out_path):
    import torch.distributed as dist

    from oracle import oracle as O
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    states, _ = _problem()
    w = np.ones(states.shape[0])
    lh, lJ = O.lambdas(w)[:2]
    P = O.Problem(states, w, lh, lJ)
    L = states.shape[1]
    rows = solve_sharded(lambda part: P.solve(part)[0], loci, L, rows_per_message=3)
    if rank == 0:
        np.save(out_path, rows)
    else:
        assert rows is None
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2])
def test_gloo_sharded_rows_equal_single_process(tmp_path, oracle_mod, world):
    O = oracle_mod
    states, cols = _problem()
    L = states.shape[1]
    loci = np.array([3, 0, 7, 11, 5, 2, 9, L - 1, 1], dtype=np.int64)   # an odd count, unsorted
    out = str(tmp_path / "rows.npy")
    mp.start_processes(_rank_main, args=(world, _free_port(), loci, out), nprocs=world, join=True,
                       start_method="spawn")
    rows = np.load(out)
    w = np.ones(states.shape[0])
    lh, lJ = O.lambdas(w)[:2]
    single = O.Problem(states, w, lh, lJ).solve(loci)[0]
    np.testing.assert_array_equal(rows, single)
    from superdca_gb300.engine import coupling_lines, format_coupling_lines
    assert format_coupling_lines(coupling_lines(rows, loci, cols)) == \
        format_coupling_lines(coupling_lines(single, loci, cols))
