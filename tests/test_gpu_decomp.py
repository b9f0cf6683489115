"""One basin split into blocks on the GPU: contexts in external-halo mode
(HYC_NREG_EXTERNAL), halos exchanged between the blocks in process (the data
movement hycadv.decomp does over NCCL between GPUs), every block's interior
equal to the single-domain run bit for bit.  The blocks run one after the
other on one GPU: no kernel waits for another block."""
import numpy as np
import pytest

import hycadv
from hycadv.decomp import Decomp
from helpers import basin, levels, np_case, oracle_grid

pytestmark = pytest.mark.gpu
FIELDS = ("temp", "saln", "th3d", "uflx", "vflx", "dp", "tracer")


@pytest.mark.parametrize("periodic,px,py,advtyp", [(True, 2, 1, 2), (False, 2, 2, 4), (True, 3, 2, 1)])
def test_blocks_equal_single_domain(cuda, periodic, px, py, advtyp):
    import torch

    b = basin(96, 60, periodic, 31)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=3, ntracr=1, seed=31, courant=0.7, delt1=1800.0)
    g.xctilr(c["dp"], b.nbdy, b.nbdy)
    sc, si = b.metrics()
    d = Decomp(b.nx, b.ny, b.nbdy, px, py, periodic)
    # single domain
    whole = {k: torch.from_numpy(c[k].copy()).to(cuda) for k in FIELDS}
    ctx = hycadv.Context.from_masks(g.masks, sc, si, kdm=3, nreg=g.nreg, nbdy=b.nbdy)
    for k, v in whole.items():
        ctx.bind(k, v)
    # blocks
    nb = b.nbdy
    tiles, ctxs = [], []
    for r in range(d.size):
        t = {}
        for k in FIELDS:
            a = torch.from_numpy(np.ascontiguousarray(d.window(c[k], r))).to(cuda)
            a[..., :nb, :] = float("nan")  # the halos come from the exchange only
            a[..., -nb:, :] = float("nan")
            a[..., :, :nb] = float("nan")
            a[..., :, -nb:] = float("nan")
            t[k] = a
        nx, ny = d.dims(r)
        w = lambda a: np.ascontiguousarray(d.window(a, r))
        cr = hycadv.Context(nx, ny, 3, nb, hycadv.NREG_EXTERNAL, w(g.masks["ip"]), w(g.masks["iu"]),
                            w(g.masks["iv"]), w(sc), w(si))
        for k, v in t.items():
            cr.bind(k, v)
        tiles.append(t)
        ctxs.append(cr)
    tf = np.zeros(1, np.int32)
    for step in range(1, 4):
        m, n = levels(step)
        ctx.tsadvc(m, n, delt1=1800.0, advtyp=advtyp, ntracr=1, trcflg=tf, nstep=step)
        for k in FIELDS:
            d.exchange_tiles([t[k] for t in tiles], nb)
        for cr in ctxs:
            cr.tsadvc(m, n, delt1=1800.0, advtyp=advtyp, ntracr=1, trcflg=tf, nstep=step)
    torch.cuda.synchronize()
    for k in ("temp", "saln", "tracer"):
        ref = whole[k].cpu().numpy()
        for r, t in enumerate(tiles):
            got = d.interior(t[k].cpu().numpy(), r)
            want = d.interior(d.window(ref, r), r)
            assert np.array_equal(got, want), (k, r)
    ctxs[0].bind("oneta", torch.ones((2,) + tuple(tiles[0]["dp"].shape[-2:]), dtype=torch.float64, device=cuda))
    with pytest.raises(hycadv.HycError) as e:  # advem_fct2c refreshes halos in mid-scheme
        ctxs[0].tsadvc(1, 2, delt1=1800.0, advtyp=2, btrmas=True)
    assert e.value.code == -8  # HYC_ERR_UNSUPPORTED
