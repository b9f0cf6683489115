"""Parity with the oracle on the 4500x3298 basin of the benchmark
(periodic in x, closed in y, ~30 % land, Courant 0.8, delt1 240 s), T and S:
hyc_tsadvc (FP64 plain form) equals the oracle's tsadvc bit for bit over
two leapfrog steps -- FCT2 on all 41 layers, FCT4 and MPDATA on the first
8 layers.

The oracle runs on the host cores (about 3.5 s per 41-layer FCT2 step on
16 cores).  The advection part of tsadvc treats every layer on its own
(mod_tsadvc.F90:1905-2048), so the oracle is called on runs of 8 layers at
a time to bound the host memory; the GPU advances all layers in one call.
"""
import numpy as np
import pytest

from helpers import levels, same

pytestmark = pytest.mark.gpu

CHUNK = 8


@pytest.fixture(scope="module")
def c1(cuda):
    import bench
    from oracle import oracle

    wl = dict(bench.WORKLOADS["c1"])
    b, masks, nreg, case = bench.make_workload(wl, cuda)
    sc, si = b.metrics()
    g = oracle.Grid(b.depth, sc, si, nbdy=b.nbdy)
    for k in ("ip", "iu", "iv"):  # the library's bigrid and the oracle's give the same masks
        assert np.array_equal(np.asarray(masks[k]), g.masks[k]), k
    yield wl, b, masks, nreg, case, g
    import torch

    del case
    torch.cuda.empty_cache()  # the next modules' ensembles allocate outside torch


def _gpu_tsadvc(case, masks, nreg, b, kdm, advtyp, delt1, steps):
    import torch

    import hycadv

    sc, si = b.metrics()
    ctx = hycadv.Context.from_masks(masks, sc, si, kdm=kdm, nreg=nreg, nbdy=b.nbdy)
    ctx.set_stream(torch.cuda.current_stream())
    f = {k: getattr(case, k)[..., :kdm, :, :].clone() for k in ("temp", "saln", "th3d", "dp")}
    f["uflx"] = case.uflx[:kdm].clone()
    f["vflx"] = case.vflx[:kdm].clone()
    for k, t in f.items():
        ctx.bind(k, t)
    for step in range(1, steps + 1):
        m, n = levels(step)
        ctx.tsadvc(m, n, delt1=delt1, advtyp=advtyp, nstep=step)
    torch.cuda.synchronize()
    ctx.close()
    return f


def _oracle_layers(g, case, k0, k1, advtyp, delt1, steps):
    h = {k: np.ascontiguousarray(getattr(case, k)[:, k0:k1].cpu().numpy()) for k in ("temp", "saln", "th3d", "dp")}
    for k in ("uflx", "vflx"):
        h[k] = np.ascontiguousarray(getattr(case, k)[k0:k1].cpu().numpy())
    for step in range(1, steps + 1):
        m, n = levels(step)
        g.tsadvc(m, n, temp=h["temp"], saln=h["saln"], th3d=h["th3d"], uflx=h["uflx"], vflx=h["vflx"], dp=h["dp"],
                 delt1=delt1, advtyp=advtyp, nstep=step)
    return h


@pytest.mark.parametrize("advtyp,nlayers", [(2, 41), (4, CHUNK), (1, CHUNK)])
def test_c1_tsadvc_equals_oracle(cuda, c1, advtyp, nlayers):
    wl, b, masks, nreg, case, g = c1
    steps = 2
    got = _gpu_tsadvc(case, masks, nreg, b, nlayers, advtyp, wl["delt1"], steps)
    moved = False
    for k0 in range(0, nlayers, CHUNK):
        k1 = min(nlayers, k0 + CHUNK)
        want = _oracle_layers(g, case, k0, k1, advtyp, wl["delt1"], steps)
        for k in ("temp", "saln"):
            a = got[k][:, k0:k1].cpu().numpy()
            assert same(a, want[k]), f"advtyp {advtyp} {k} layers {k0 + 1}-{k1}: max |diff| " \
                                     f"{np.nanmax(np.abs(a - want[k]))}"
            moved |= not np.array_equal(want[k], case_layers(case, k, k0, k1))
    assert moved
    del got


def case_layers(case, k, k0, k1):
    return getattr(case, k)[:, k0:k1].cpu().numpy()
