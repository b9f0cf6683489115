"""GPU parity of the continuity equation (cnuity.F90) through the C ABI
against the CPU oracle, bit for bit (-0.0 == +0.0), halos included."""
import numpy as np
import pytest

import hycadv
from helpers import basin, cnuity_case, oracle_grid, same
from test_gpu_parity import make_ctx

pytestmark = pytest.mark.gpu

OUT = ("dp", "dpo", "p", "uflx", "vflx", "uflxav", "vflxav", "dpav", "onetacnt")


def setup(cuda, nx, ny, periodic, seed, kdm=3, btrmas=False, thkdf=0, umax=0.5):
    import torch

    b = basin(nx, ny, periodic, seed)
    g = oracle_grid(b)
    c = cnuity_case(b, g, kdm=kdm, seed=seed, umax=umax, btrmas=btrmas, thkdf=thkdf != 0)
    t = {k: (None if v is None else torch.from_numpy(v.copy()).to(cuda)) for k, v in c.items()}
    ctx = make_ctx(b, g, kdm)
    for k, v in t.items():
        if v is not None and k in hycadv.FIELDS:
            ctx.bind(k, v)
    ctx.set_cnuity_grid(c["scuy"], c["scvx"], c["depthu"], c["depthv"], c.get("thkdfu"), c.get("thkdfv"))
    return b, g, c, t, ctx


def compare(c, t):
    for k in OUT:
        if c.get(k) is None:
            continue
        got = t[k].cpu().numpy()
        assert same(got, c[k]), f"{k}: max |diff| = {np.nanmax(np.abs(got - c[k]))}"


@pytest.mark.parametrize("periodic,btrmas,thkdf", [(False, False, 0), (True, False, 4), (False, True, 2),
                                                    (True, True, 4), (False, False, 4)])
def test_cnuity_bitwise(cuda, periodic, btrmas, thkdf):
    """Two leapfrog steps (the biharmonic diffusion alternates its direction)."""
    b, g, c, t, ctx = setup(cuda, 70, 50, periodic, 91, btrmas=btrmas, thkdf=thkdf)
    for step in (1, 2):
        m, n = ((step + 1) % 2) + 1, (step % 2) + 1
        want = g.cnuity(m, n, c, delt1=1800.0, nstep=step, btrmas=btrmas, thkdf4=thkdf == 4, thkdf2=thkdf == 2)
        got = ctx.cnuity(m, n, delt1=1800.0, nstep=step, btrmas=btrmas, thkdf=thkdf, want_dpkmin=True)
        assert same(got, want)
        compare(c, t)


@pytest.mark.parametrize("nx,ny", [(37, 29), (100, 17)])
def test_cnuity_ragged(cuda, nx, ny):
    b, g, c, t, ctx = setup(cuda, nx, ny, nx == 100, 92, kdm=2, thkdf=4)
    want = g.cnuity(1, 2, c, delt1=1800.0, nstep=3, thkdf4=True)
    got = ctx.cnuity(1, 2, delt1=1800.0, nstep=3, thkdf=4, want_dpkmin=True)
    assert same(got, want)
    compare(c, t)


def test_cnuity_fatal_negative_thickness(cuda):
    """A Courant number far above one: the oracle stops (dpfatal), the
    library returns HYC_ERR_NEGDP on a checked step and goes on otherwise."""
    from oracle import oracle as O

    b, g, c, t, ctx = setup(cuda, 40, 30, False, 93, kdm=2, umax=400.0)
    with pytest.raises(O.OracleError):
        g.cnuity(1, 2, c, delt1=1800.0, nstep=3)
    with pytest.raises(hycadv.HycError) as e:
        ctx.cnuity(1, 2, delt1=1800.0, nstep=3)
    assert e.value.code == -10  # HYC_ERR_NEGDP
    b, g, c, t, ctx = setup(cuda, 40, 30, False, 93, kdm=2, umax=400.0)
    want = g.cnuity(1, 2, c, delt1=1800.0, nstep=1)
    got = ctx.cnuity(1, 2, delt1=1800.0, nstep=1, want_dpkmin=True)
    assert same(got, want)
    compare(c, t)
