"""CPU: the multi-rank chain split, run as two gloo ranks.

Each rank samples its own block of chain ids with the oracle; the gathered
blocks must equal one single-process run over all chain ids, and the timing
reduction must return the slowest rank's time."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, golden_path, result_path):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import __graft_entry__ as ge
    import oracle

    pkg = ge.load_package()
    import importlib
    sharding = importlib.import_module("achr_gb300.sharding")
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = np.load(golden_path)
    model = pkg.HostModel(int(g["n_rxns"]), int(g["n_mets"]), g["row"], g["col"], g["val"], g["lb"], g["ub"])
    off, cnt = sharding.chain_block(rank, world, 6)
    pts, st = oracle.sample(model, g["warmup"], g["N"], 99, cnt, 12, chain_offset=off, threads=1)
    blocks = [None] * world
    dist.all_gather_object(blocks, (off, cnt, pts, st["accepted"]))
    t = sharding.max_over_ranks(0.5 + rank)  # rank r "took" 0.5 + r seconds
    if rank == 0:
        np.savez(result_path, offsets=[b[0] for b in blocks], counts=[b[1] for b in blocks],
                 pts=np.concatenate([b[2] for b in blocks], axis=1), accepted=sum(b[3] for b in blocks), tmax=t)
    dist.barrier()
    dist.destroy_process_group()


def test_split_is_disjoint_and_covers():
    import importlib

    import __graft_entry__ as ge
    ge.load_package()
    sharding = importlib.import_module("achr_gb300.sharding")
    for total in (0, 1, 7, 100):
        for world in (1, 2, 3, 8):
            spans = [sharding.split_chains(r, world, total) for r in range(world)]
            ids = [i for off, cnt in spans for i in range(off, off + cnt)]
            assert ids == list(range(total))
    assert sharding.chain_block(3, 4, 25) == (75, 25)
    with pytest.raises(ValueError):
        sharding.chain_block(4, 4, 25)


def test_two_gloo_ranks_equal_one_process(tmp_path):
    import torch.multiprocessing as mp

    import __graft_entry__ as ge
    import oracle

    golden_path = os.path.join(os.path.dirname(__file__), "golden", "small_golden.npz")
    result_path = str(tmp_path / "ranks.npz")
    mp.start_processes(_rank_main, args=(2, _free_port(), golden_path, result_path), nprocs=2, join=True,
                       start_method="spawn")
    r = np.load(result_path)
    assert list(r["offsets"]) == [0, 6] and list(r["counts"]) == [6, 6]
    assert float(r["tmax"]) == 1.5
    pkg = ge.load_package()
    g = np.load(golden_path)
    model = pkg.HostModel(int(g["n_rxns"]), int(g["n_mets"]), g["row"], g["col"], g["val"], g["lb"], g["ub"])
    ref, st = oracle.sample(model, g["warmup"], g["N"], 99, 12, 12, threads=1)
    assert np.array_equal(r["pts"], ref) and int(r["accepted"]) == st["accepted"]
