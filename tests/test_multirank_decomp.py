"""One basin split over ranks (the reference's MPI tiling, mod_xc_mp.h:
4664-4987): each rank advances its block with halos exchanged over
torch.distributed (gloo on CPU) and the oracle in external-halo mode; every
block's interior equals the single-domain run bit for bit, closed and
periodic basins, 2 and 2x2 ranks.  Also the exchange against the basin's own
xctilr, in process."""
import os
import socket

import numpy as np
import pytest

from hycadv.decomp import Decomp

FIELDS = ("temp", "saln", "th3d", "uflx", "vflx", "dp")


def _case(nx, ny, periodic, seed, kdm=3, ntracr=1):
    from helpers import basin, np_case, oracle_grid

    b = basin(nx, ny, periodic, seed)
    g = oracle_grid(b, threads=1)
    c = np_case(b, g, kdm=kdm, ntracr=ntracr, seed=seed, courant=0.7, delt1=1800.0)
    g.xctilr(c["dp"], b.nbdy, b.nbdy)  # the halo tsadvc expects up to date on entry
    return b, g, c


def _steps(g, c, steps, advtyp, ntracr):
    from helpers import levels

    tf = np.zeros(max(ntracr, 1), np.int32)
    for step in steps:
        m, n = levels(step)
        g.tsadvc(m, n, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], uflx=c["uflx"], vflx=c["vflx"], dp=c["dp"],
                 delt1=1800.0, advtyp=advtyp, tracer=c["tracer"], trcflg=tf, nstep=step)


def test_exchange_equals_xctilr():
    """In process: a field split into 2x3 blocks and exchanged has, in every
    block's halo, what the basin's xctilr leaves there (closed and periodic)."""
    from helpers import basin, oracle_grid

    for periodic in (False, True):
        b = basin(40, 33, periodic, 5)
        g = oracle_grid(b, threads=1)
        rng = np.random.default_rng(5)
        a = rng.standard_normal((2, b.ld2, b.ld1))
        d = Decomp(b.nx, b.ny, b.nbdy, 2, 3, periodic)
        tiles = [d.window(a, r) for r in range(d.size)]
        for t in tiles:  # garbage in the halos
            t[..., :d.nbdy, :] = np.nan
            t[..., :, :d.nbdy] = np.nan
        d.exchange_tiles(tiles, b.nbdy)
        ref = a.copy()
        g.xctilr(ref, b.nbdy, b.nbdy)
        for r, t in enumerate(tiles):
            assert np.array_equal(t, d.window(ref, r)), (periodic, r)


def test_xcsum_tiles_equal_single_domain():
    """In process: the reproducible sum over blocks (strips straddling block
    edges, the last block owning the strips past its edge) equals the
    single-domain xcsum bit for bit, closed and periodic, several layouts."""
    from helpers import basin, oracle_grid

    for periodic, nx, ny, px, py in ((False, 40, 33, 3, 2), (True, 41, 30, 2, 3), (False, 27, 19, 4, 1)):
        b = basin(nx, ny, periodic, 9)
        g = oracle_grid(b, threads=1)
        rng = np.random.default_rng(nx)
        a = rng.standard_normal((b.ld2, b.ld1)) * 1.0e3
        g.xctilr(a, b.nbdy, b.nbdy)
        want = g.xcsum(a, g.masks["ip"])
        d = Decomp(b.nx, b.ny, b.nbdy, px, py, periodic)
        tiles = [d.window(a, r) for r in range(d.size)]
        masks = [d.window(g.masks["ip"], r) for r in range(d.size)]
        assert d.xcsum_tiles(tiles, masks) == want, (periodic, px, py)


def _rank(rank, world, port, out_dir, cfg):
    import sys

    import torch
    import torch.distributed as dist

    here = os.path.dirname(os.path.abspath(__file__))
    for p in (here, os.path.join(os.path.dirname(here), "hycom-src_gb300"), os.path.dirname(here)):
        if p not in sys.path:
            sys.path.insert(0, p)
    from hycadv.decomp import Decomp as D
    from oracle import oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    nx, ny, periodic, seed, px, py, advtyp = cfg
    b, g, c = _case(nx, ny, periodic, seed)
    d = D(b.nx, b.ny, b.nbdy, px, py, periodic)
    win = lambda a: d.window(a, rank)
    loc = {k: np.ascontiguousarray(win(c[k])) for k in FIELDS}
    loc["tracer"] = np.ascontiguousarray(win(c["tracer"]))
    gl = O.Grid.from_masks(win(g.masks["ip"]), win(g.masks["iu"]), win(g.masks["iv"]), win(g.scp2),
                           win(g.scp2i), nbdy=b.nbdy, nreg=-1, threads=1)
    nb = b.nbdy
    for a in loc.values():  # nothing of the basin's halos is given: the exchange fills them
        a[..., :nb, :] = np.nan
        a[..., -nb:, :] = np.nan
        a[..., :, :nb] = np.nan
        a[..., :, -nb:] = np.nan
    t0 = loc["temp"].copy()
    ok = True
    for step in range(1, 4):
        # the halos tsadvc would refresh (mod_tsadvc.F90:1829-1840), and dp's
        for k in FIELDS + ("tracer",):
            d.exchange(torch.from_numpy(loc[k]), b.nbdy, dist, rank)
        _steps(gl, loc, [step], advtyp, 1)
        _steps(g, c, [step], advtyp, 1)
        for k in ("temp", "saln", "tracer"):
            ok &= bool(np.array_equal(d.interior(loc[k], rank), d.interior(win(c[k]), rank)))
    ok &= not np.array_equal(d.interior(loc["temp"], rank), d.interior(t0, rank))  # the blocks did advance
    # the conservation sum of the new level over all blocks (one gather of
    # partial sums) equals the single-domain xcsum bit for bit
    from helpers import levels

    nn = levels(3)[1]
    d.exchange(torch.from_numpy(loc["temp"]), b.nbdy, dist, rank)
    ipl = win(g.masks["ip"])
    for k in range(loc["temp"].shape[1]):
        ok &= d.xcsum(loc["temp"][nn - 1, k], ipl, dist, rank) == g.xcsum(c["temp"][nn - 1, k], g.masks["ip"])
    flag = torch.tensor([0 if ok else 1], dtype=torch.int64)
    dist.all_reduce(flag, op=dist.ReduceOp.SUM)
    if rank == 0:
        np.save(os.path.join(out_dir, "bad.npy"), flag.numpy())
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("cfg", [(64, 40, True, 21, 2, 1, 2), (52, 44, False, 22, 2, 2, 4),
                                 (60, 36, True, 23, 2, 2, 1)])
def test_blocks_equal_single_domain(tmp_path, cfg):
    import torch.multiprocessing as mp

    world = cfg[4] * cfg[5]
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path), cfg), nprocs=world, join=True)
    assert int(np.load(tmp_path / "bad.npy")[0]) == 0
