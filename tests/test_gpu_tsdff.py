"""GPU parity of the lateral diffusion at the end of tsadvc
(mod_tsadvc.F90:2138-2230: tsdff_1x/tsdff_2x and the density update) through
the C ABI against the CPU oracle, bit for bit (-0.0 == +0.0)."""
import numpy as np
import pytest

import hycadv
from helpers import basin, diff_grid, levels, np_case, oneta_field, oracle_grid, same
from test_gpu_parity import bind_all, compare, make_ctx, torchify

pytestmark = pytest.mark.gpu


def setup(cuda, nx, ny, periodic, seed, kdm=3, ntracr=2, mxlmy=False, courant=0.8, delt1=1800.0):
    b = basin(nx, ny, periodic, seed)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=kdm, ntracr=ntracr, seed=seed, courant=courant, delt1=delt1)
    c["delt1"] = delt1
    c["oneta"] = oneta_field(b, seed)
    if mxlmy:
        rng = np.random.default_rng(seed + 2)
        c["q2"] = 0.01 + rng.random((2, kdm + 2, b.ld2, b.ld1)) * 0.1
        c["q2l"] = 0.1 + rng.random((2, kdm + 2, b.ld2, b.ld1))
    d = diff_grid(b, seed)
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, kdm)
    bind_all(ctx, t, extra=("oneta",) + (("q2", "q2l") if mxlmy else ()))
    ctx.set_diffusion_grid(**d)
    return b, g, c, d, t, ctx


def run_both(g, c, d, ctx, steps, advtyp, ntracr, temdf2, mxlmy=False, thbase=34.0):
    """tsadvc then its diffusion block, step after step, on the oracle and the GPU."""
    tf = np.zeros(max(ntracr, 1), np.int32)
    q = dict(q2=c.get("q2"), q2l=c.get("q2l")) if mxlmy else {}
    for step in steps:
        m, n = levels(step)
        g.tsadvc(m, n, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], uflx=c["uflx"], vflx=c["vflx"], dp=c["dp"],
                 delt1=c["delt1"], advtyp=advtyp, tracer=c["tracer"], trcflg=tf, nstep=step, mxlmy=mxlmy, **q)
        g.tsdff(m, n, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], dp=c["dp"], oneta=c["oneta"],
                delt1=c["delt1"], temdf2=temdf2, thbase=thbase, tracer=c["tracer"], **q, **d)
        ctx.tsadvc(m, n, delt1=c["delt1"], advtyp=advtyp, ntracr=ntracr, trcflg=tf, nstep=step, mxlmy=mxlmy)
        ctx.tsdff(m, n, delt1=c["delt1"], temdf2=temdf2, thbase=thbase, ntracr=ntracr, mxlmy=mxlmy)


@pytest.mark.parametrize("periodic", [False, True])
def test_tsadvc_with_diffusion_bitwise(cuda, periodic):
    """Three FCT2 steps with Laplacian diffusion of T, S and two tracers;
    th3d follows from the diffused T and S."""
    b, g, c, d, t, ctx = setup(cuda, 90, 60, periodic, seed=51)
    run_both(g, c, d, ctx, range(1, 4), 2, 2, temdf2=0.3)
    compare(c, t, keys=("temp", "saln", "th3d", "tracer"))


def test_diffusion_mxlmy_and_chunked_fields(cuda):
    """q2/q2l diffused with T, S and 15 tracers: 19 fields, two launches."""
    b, g, c, d, t, ctx = setup(cuda, 64, 40, False, seed=52, kdm=2, ntracr=15, mxlmy=True)
    run_both(g, c, d, ctx, range(1, 3), 1, 15, temdf2=0.2, mxlmy=True)
    compare(c, t, keys=("temp", "saln", "th3d", "tracer", "q2", "q2l"))


@pytest.mark.parametrize("nx,ny", [(37, 29), (100, 17), (33, 65)])
def test_diffusion_ragged_tiles(cuda, nx, ny):
    """Basins whose sizes are not multiples of the 32x32 tile."""
    b, g, c, d, t, ctx = setup(cuda, nx, ny, nx == 100, seed=53, kdm=2, ntracr=1)
    run_both(g, c, d, ctx, range(1, 3), 0, 1, temdf2=0.25)
    compare(c, t, keys=("temp", "saln", "th3d", "tracer"))


def test_diffusion_options(cuda):
    """temdf2 <= 0 is a no-op; temdfc != 1 and exactly isopycnal layers are
    refused; the diffusion grid must be set."""
    b, g, c, d, t, ctx = setup(cuda, 40, 30, False, seed=54, kdm=2, ntracr=0)
    before = {k: t[k].clone() for k in ("temp", "saln", "th3d")}
    ctx.tsdff(1, 2, delt1=1800.0, temdf2=0.0)
    for k, v in before.items():
        assert same(t[k].cpu().numpy(), v.cpu().numpy())
    with pytest.raises(hycadv.HycError) as e:
        ctx.tsdff(1, 2, delt1=1800.0, temdf2=0.1, temdfc=0.5)
    assert e.value.code == -8  # HYC_ERR_UNSUPPORTED
    with pytest.raises(hycadv.HycError) as e:
        ctx.tsdff(1, 2, delt1=1800.0, temdf2=0.1, nhybrd=1)
    assert e.value.code == -8  # HYC_ERR_UNSUPPORTED
    sc, si = b.metrics()
    bare = hycadv.Context.from_masks(g.masks, sc, si, kdm=2, nreg=g.nreg, nbdy=b.nbdy)
    bind_all(bare, t, extra=("oneta",))
    with pytest.raises(hycadv.HycError) as e:
        bare.tsdff(1, 2, delt1=1800.0, temdf2=0.1)
    assert e.value.code == -6  # HYC_ERR_FIELD
    bare.close()
