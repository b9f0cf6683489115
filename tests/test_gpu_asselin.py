"""GPU parity of the Robert-Asselin filter (mod_asselin.F90: asselin_save,
asselin_filter) through the C ABI against the CPU oracle, bit for bit."""
import numpy as np
import pytest

import hycadv
from helpers import basin, oracle_grid, same
from test_gpu_parity import make_ctx
from test_oracle_asselin import advance, assel_case

pytestmark = pytest.mark.gpu


def bind_assel(ctx, t):
    for k, v in t.items():
        if v is not None and k in hycadv.FIELDS:
            ctx.bind(k, v)


def to_dev(a, dev):
    import torch

    return {k: (None if v is None else torch.from_numpy(np.ascontiguousarray(v).copy()).to(dev)) for k, v in a.items()}


def compare(a, t, keys):
    for k in keys:
        if a.get(k) is None:
            continue
        got = t[k].cpu().numpy()
        assert same(got, a[k]), f"{k}: max |diff| = {np.nanmax(np.abs(got - a[k]))}"


ALL = ("temp", "saln", "th3d", "tracer", "q2", "q2l", "dp", "oneta", "onetao", "otemp", "osaln", "oth3d", "otracer",
       "oq2", "oq2l")


@pytest.mark.parametrize("periodic,mxlmy,ntracr", [(False, False, 2), (True, True, 3), (False, True, 0)])
def test_asselin_save_and_filter_bitwise(cuda, periodic, mxlmy, ntracr):
    """Three steps of save -> (new level n) -> filter, with the leapfrog
    levels swapping, on the oracle and the GPU from the same inputs."""
    b = basin(70, 50, periodic, 71)
    g = oracle_grid(b)
    kdm = 3
    a = assel_case(b, g, kdm=kdm, ntracr=ntracr, mxlmy=mxlmy, seed=71)
    t = to_dev(a, cuda)
    ctx = make_ctx(b, g, kdm)
    bind_assel(ctx, t)
    rng = np.random.default_rng(71)
    for step in range(1, 4):
        m, n = ((step + 1) % 2) + 1, (step % 2) + 1
        g.asselin_save(m, n, a, oneta0=0.1)
        ctx.asselin_save(m, n, oneta0=0.1, ntracr=ntracr, mxlmy=mxlmy)
        compare(a, t, ALL)
        advance(a, n, rng)
        for k in ("temp", "saln", "tracer", "q2", "q2l", "dp", "pbavg"):
            if a.get(k) is not None:
                t[k].copy_(__import__("torch").from_numpy(a[k]))
        g.asselin_filter(m, n, a, ra2fac=0.125, oneta0=0.1, thbase=34.0)
        ctx.asselin_filter(m, n, ra2fac=0.125, oneta0=0.1, thbase=34.0, ntracr=ntracr, mxlmy=mxlmy)
        compare(a, t, ALL)


def test_asselin_options(cuda):
    b = basin(40, 30, False, 72)
    g = oracle_grid(b)
    a = assel_case(b, g, kdm=2, ntracr=0, seed=72)
    t = to_dev(a, cuda)
    ctx = make_ctx(b, g, 2)
    bind_assel(ctx, t)
    with pytest.raises(hycadv.HycError) as e:
        ctx.asselin_filter(1, 2, ra2fac=0.125, oneta0=0.1, advflg=1)
    assert e.value.code == -8  # HYC_ERR_UNSUPPORTED
    with pytest.raises(hycadv.HycError) as e:
        ctx.asselin_filter(1, 2, ra2fac=0.125, oneta0=0.1, nhybrd=1)
    assert e.value.code == -8
    bare = make_ctx(b, g, 2)
    bare.bind("temp", t["temp"])
    with pytest.raises(hycadv.HycError) as e:
        bare.asselin_save(1, 2, oneta0=0.1)
    assert e.value.code == -6  # HYC_ERR_FIELD
