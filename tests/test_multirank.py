"""Multi-rank path on CPU (gloo, world size 2): basins of an ensemble are
sharded over ranks with no data-path exchange; each rank advances its
shard (here with the oracle), and the gathered results equal a single-rank
run bit for bit.  Also the sharding itself and the max-over-ranks timing
reduction the benchmark uses."""
import os
import socket

import numpy as np
import pytest

from hycadv import shard as S

SPECS = [(60, 45, False, 2, 11), (70, 40, True, 3, 12), (33, 27, False, 2, 13), (50, 50, True, 1, 14),
         (41, 30, False, 2, 15)]  # nx, ny, periodic, kdm, seed


def test_shard_lpt_balances_and_covers():
    work = [5, 9, 1, 7, 3, 3, 8, 2]
    parts = S.shard(work, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(work)))
    assert S.imbalance(work, parts) < 1.1
    assert S.shard(work, 1) == [list(range(len(work)))]
    assert S.shard([], 2) == [[], []]
    with pytest.raises(ValueError):
        S.shard(work, 0)


def _advance(i, steps=3):
    """FP64 oracle steps of basin i (T, S): a checksum of the new levels and
    the content of salinity after the last step."""
    from helpers import basin, levels, np_case, oracle_grid

    nx, ny, per, kdm, seed = SPECS[i]
    b = basin(nx, ny, per, seed)
    g = oracle_grid(b, threads=1)
    c = np_case(b, g, kdm=kdm, ntracr=0, seed=seed, courant=0.6, delt1=1800.0)
    for step in range(1, steps + 1):
        m, n = levels(step)
        g.tsadvc(m, n, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], uflx=c["uflx"], vflx=c["vflx"], dp=c["dp"],
                 delt1=1800.0, advtyp=2, nstep=step)
    return np.concatenate([c["temp"].ravel(), c["saln"].ravel()])


def _rank(rank, world, port, out_dir):
    import sys

    import torch
    import torch.distributed as dist

    here = os.path.dirname(os.path.abspath(__file__))
    for p in (here, os.path.join(os.path.dirname(here), "hycom-src_gb300"), os.path.dirname(here)):
        if p not in sys.path:
            sys.path.insert(0, p)
    from hycadv import shard as S2

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    work = [nx * ny * kdm for nx, ny, _, kdm, _ in SPECS]
    mine = S2.shard(work, world)[rank]
    dist.barrier()
    res = {i: _advance(i) for i in mine}
    ms = torch.tensor([10.0 + rank], dtype=torch.float64)  # this rank's timed region
    dist.all_reduce(ms, op=dist.ReduceOp.MAX)              # as bench.py reduces it
    gathered = [None] * world
    dist.all_gather_object(gathered, res)
    if rank == 0:
        allres = {}
        for d in gathered:
            allres.update(d)
        np.savez(os.path.join(out_dir, "sharded.npz"), ms=ms.numpy(),
                 **{f"b{i}": v for i, v in allres.items()})
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_equal_one_rank(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    got = np.load(tmp_path / "sharded.npz")
    assert float(got["ms"][0]) == 11.0  # max over ranks
    for i in range(len(SPECS)):
        want = _advance(i)
        assert np.array_equal(got[f"b{i}"], want), f"basin {i}"
