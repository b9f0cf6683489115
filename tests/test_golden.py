"""Golden fixtures (tests/golden/*.npz, written by make_golden.py with the
oracle on x86-64): the oracle must reproduce them on any host (CPU test), and
the CUDA path must reproduce them through the C ABI (GPU test), bit for bit."""
import glob
import os

import numpy as np
import pytest

from helpers import levels, same

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz")))


def load(path):
    z = np.load(path)
    nx, ny, kdm, ntracr, advtyp, steps, nreg, nbdy = (int(x) for x in z["meta"])
    return z, dict(nx=nx, ny=ny, kdm=kdm, ntracr=ntracr, advtyp=advtyp, steps=steps, nreg=nreg, nbdy=nbdy,
                   delt1=float(z["delt1"][0]))


def test_golden_files_present():
    assert len(GOLD) >= 4


@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(p)[:-4] for p in GOLD])
def test_oracle_reproduces_golden(path):
    from oracle import oracle as O

    z, m = load(path)
    depth = np.where(z["mask_ip"] != 0, 100.0, 0.0)
    g = O.Grid(depth, z["in_scp2"], z["in_scp2i"], nbdy=m["nbdy"])
    assert g.nreg == m["nreg"]
    for k in ("ip", "iu", "iv"):
        assert np.array_equal(g.masks[k], z[f"mask_{k}"])
    c = {k: z[f"in_{k}"].copy() for k in ("temp", "saln", "uflx", "vflx", "dp", "tracer")}
    for s in range(1, m["steps"] + 1):
        mm, nn = levels(s)
        g.tsadvc(mm, nn, temp=c["temp"], saln=c["saln"], th3d=c["temp"].copy(), uflx=c["uflx"], vflx=c["vflx"],
                 dp=c["dp"], delt1=m["delt1"], advtyp=m["advtyp"], tracer=c["tracer"],
                 trcflg=np.zeros(m["ntracr"], np.int32), nstep=s)
    for k in ("temp", "saln", "tracer", "uflx", "vflx"):
        assert same(c[k], z[f"out_{k}"]), k


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(p)[:-4] for p in GOLD])
def test_cuda_reproduces_golden(cuda, path):
    import torch

    import hycadv

    z, m = load(path)
    ctx = hycadv.Context(m["nx"], m["ny"], m["kdm"], m["nbdy"], m["nreg"], z["mask_ip"], z["mask_iu"],
                         z["mask_iv"], z["in_scp2"], z["in_scp2i"])
    ctx.set_stream(torch.cuda.current_stream())
    t = {k: torch.from_numpy(z[f"in_{k}"].copy()).to(cuda) for k in ("temp", "saln", "uflx", "vflx", "dp", "tracer")}
    for k, v in t.items():
        ctx.bind(k, v)
    for s in range(1, m["steps"] + 1):
        mm, nn = levels(s)
        ctx.tsadvc(mm, nn, delt1=m["delt1"], advtyp=m["advtyp"], ntracr=m["ntracr"],
                   trcflg=np.zeros(m["ntracr"], np.int32), nstep=s)
    torch.cuda.synchronize()
    for k in ("temp", "saln", "tracer", "uflx", "vflx"):
        assert same(t[k].cpu().numpy(), z[f"out_{k}"]), k
    ctx.close()
