"""A basin with no sea point (the empty input of this path): every routine
runs, changes nothing at the interior, and agrees with the oracle."""
import numpy as np
import pytest

import hycadv
from helpers import basin, cnuity_case, diff_grid, np_case, oneta_field, oracle_grid, same
from test_gpu_parity import bind_all, make_ctx, torchify

pytestmark = pytest.mark.gpu


def land_basin():
    b = basin(40, 30, False, 95)
    b.depth[:] = 0.0
    return b, oracle_grid(b)


def test_all_land_tsadvc_tsdff(cuda):
    b, g = land_basin()
    assert not g.masks["ip"].any()
    c = np_case(b, g, kdm=2, ntracr=1, seed=95, courant=0.5, delt1=1800.0)
    c["delt1"] = 1800.0
    c["oneta"] = oneta_field(b, 95)
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, 2)
    bind_all(ctx, t, extra=("oneta",))
    ctx.set_diffusion_grid(**diff_grid(b, 95))
    inner = np.zeros((b.ld2, b.ld1), bool)
    inner[b.J, b.I] = True
    before = {k: c[k].copy() for k in ("temp", "saln", "tracer")}
    tf = np.zeros(1, np.int32)
    for adv in (0, 1, 2, 4):
        ctx.tsadvc(1, 2, delt1=1800.0, advtyp=adv, ntracr=1, trcflg=tf)
    ctx.tsdff(1, 2, delt1=1800.0, temdf2=0.3, ntracr=1)
    for k, v in before.items():
        assert same(t[k].cpu().numpy()[..., inner], v[..., inner]), k


def test_all_land_cnuity(cuda):
    import torch

    b, g = land_basin()
    c = cnuity_case(b, g, kdm=2, seed=96, thkdf=True)
    tt = {k: (None if v is None else torch.from_numpy(v.copy()).to(cuda)) for k, v in c.items()}
    ctx = make_ctx(b, g, 2)
    for k, v in tt.items():
        if v is not None and k in hycadv.FIELDS:
            ctx.bind(k, v)
    ctx.set_cnuity_grid(c["scuy"], c["scvx"], c["depthu"], c["depthv"], c["thkdfu"], c["thkdfv"])
    want = g.cnuity(1, 2, c, delt1=1800.0, nstep=3, thkdf4=True)
    got = ctx.cnuity(1, 2, delt1=1800.0, nstep=3, thkdf=4, want_dpkmin=True)
    assert same(got, want) and np.all(got == 999.0)  # no sea point: the minima keep their start value
    for k in ("dp", "dpo", "p", "uflx", "vflx"):
        assert same(tt[k].cpu().numpy(), c[k]), k
