"""Golden fixtures (tests/golden/*.npz, written by make_golden.py with the
oracle on x86-64): the oracle must reproduce them on any host (CPU test), and
the CUDA path must reproduce them through the C ABI (GPU test), bit for bit.
Kinds: the advection schemes through tsadvc; a whole tracer step
(asselin_save, tsadvc, its diffusion block, asselin_filter); cnuity."""
import glob
import os
import sys

import numpy as np
import pytest

from helpers import levels, same

HERE = os.path.dirname(os.path.abspath(__file__))
ALL_GOLD = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def kind_of(path):
    z = np.load(path)
    return str(z["kind"][0]) if "kind" in z.files else "tsadvc"


GOLD = [p for p in ALL_GOLD if kind_of(p) == "tsadvc"]
GOLD_ROWS = [p for p in ALL_GOLD if kind_of(p) != "tsadvc"]


def golden_module():
    sys.path.insert(0, os.path.join(HERE, "golden"))
    try:
        import make_golden
    finally:
        sys.path.pop(0)
    return make_golden


def load(path):
    z = np.load(path)
    nx, ny, kdm, ntracr, advtyp, steps, nreg, nbdy = (int(x) for x in z["meta"])
    return z, dict(nx=nx, ny=ny, kdm=kdm, ntracr=ntracr, advtyp=advtyp, steps=steps, nreg=nreg, nbdy=nbdy,
                   delt1=float(z["delt1"][0]))


def test_golden_files_present():
    assert len(GOLD) >= 4
    assert sorted(kind_of(p) for p in GOLD_ROWS) == ["cnuity", "cnuity", "step", "step"]


def expected(z, key):
    """The stored output, or (not stored: unchanged) the input."""
    return z[f"out_{key}"] if f"out_{key}" in z.files else z[f"in_{key}"]


def inputs(z):
    return {k[3:]: z[k].copy() for k in z.files if k.startswith("in_") and k not in ("in_scp2", "in_scp2i")}


def oracle_grid_of(z, nbdy, nreg):
    from oracle import oracle as O

    depth = np.where(z["mask_ip"] != 0, 100.0, 0.0)
    g = O.Grid(depth, z["in_scp2"], z["in_scp2i"], nbdy=nbdy)
    assert g.nreg == nreg
    for k in ("ip", "iu", "iv"):
        assert np.array_equal(g.masks[k], z[f"mask_{k}"])
    return g


@pytest.mark.parametrize("path", GOLD_ROWS, ids=[os.path.basename(p)[:-4] for p in GOLD_ROWS])
def test_oracle_reproduces_golden_rows(path):
    """The tracer step (Robert-Asselin save, advection, diffusion, filter)
    and the continuity equation, replayed by the oracle on this host."""
    mg = golden_module()
    z = np.load(path)
    nx, ny, kdm, a4, a5, steps, nreg, nbdy = (int(x) for x in z["meta"])
    g = oracle_grid_of(z, nbdy, nreg)
    a = inputs(z)
    if kind_of(path) == "step":
        ntracr = a4
        a.setdefault("tracer", None)
        a.setdefault("otracer", None)
        d = {k[5:]: z[k] for k in z.files if k.startswith("grid_")}
        for s in range(1, steps + 1):
            mg.run_step(g, a, d, s, ntracr)
    else:
        thkdf, btrmas = a4, bool(a5)
        from oracle import oracle as O

        arrs = {k: a.get(k) for k in O.CNUITY_ARRAYS}
        mins = []
        for s in range(1, steps + 1):
            m, n = ((s + 1) % 2) + 1, (s % 2) + 1
            mins.append(g.cnuity(m, n, arrs, delt1=float(z["delt1"][0]), nstep=s, btrmas=btrmas,
                                 thkdf4=thkdf == 4, thkdf2=thkdf == 2))
        assert same(np.stack(mins), z["out_dpkmin"])
    for k, v in a.items():
        if v is not None:
            assert same(v, expected(z, k)), k


@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(p)[:-4] for p in GOLD])
def test_oracle_reproduces_golden(path):
    z, m = load(path)
    g = oracle_grid_of(z, m["nbdy"], m["nreg"])
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


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLD_ROWS, ids=[os.path.basename(p)[:-4] for p in GOLD_ROWS])
def test_cuda_reproduces_golden_rows(cuda, path):
    """The same replay through the C ABI on device-resident fields."""
    import torch

    import hycadv

    mg = golden_module()
    z = np.load(path)
    nx, ny, kdm, a4, a5, steps, nreg, nbdy = (int(x) for x in z["meta"])
    masks = {k: z[f"mask_{k}"] for k in ("ip", "iu", "iv")}
    ctx = hycadv.Context.from_masks(masks, z["in_scp2"], z["in_scp2i"], kdm=kdm, nreg=nreg, nbdy=nbdy)
    ctx.set_stream(torch.cuda.current_stream())
    a = inputs(z)
    grid_keys = ("scuy", "scvx", "depthu", "depthv", "thkdfu", "thkdfv")
    t = {k: torch.from_numpy(v).to(cuda) for k, v in a.items() if k in hycadv.FIELDS}
    for k, v in t.items():
        ctx.bind(k, v)
    delt1 = float(z["delt1"][0])
    if kind_of(path) == "step":
        ntracr, P = a4, mg.STEP_PARAMS
        ctx.set_diffusion_grid(**{k[5:]: z[k] for k in z.files if k.startswith("grid_")})
        for s in range(1, steps + 1):
            m, n = levels(s)
            ctx.asselin_save(m, n, oneta0=P["oneta0"], ntracr=ntracr)
            ctx.tsadvc(m, n, delt1=delt1, advtyp=2, ntracr=ntracr, trcflg=np.zeros(max(ntracr, 1), np.int32),
                       nstep=s)
            ctx.tsdff(m, n, delt1=delt1, temdf2=P["temdf2"], thbase=P["thbase"], ntracr=ntracr)
            ctx.asselin_filter(m, n, ra2fac=P["ra2fac"], oneta0=P["oneta0"], thbase=P["thbase"], ntracr=ntracr)
    else:
        thkdf, btrmas = a4, bool(a5)
        ctx.set_cnuity_grid(*[a.get(k) for k in grid_keys])
        mins = []
        for s in range(1, steps + 1):
            m, n = ((s + 1) % 2) + 1, (s % 2) + 1
            mins.append(ctx.cnuity(m, n, delt1=delt1, nstep=s, btrmas=btrmas, thkdf=thkdf, want_dpkmin=True))
        assert same(np.stack(mins), z["out_dpkmin"])
    torch.cuda.synchronize()
    for k, v in t.items():
        assert same(v.cpu().numpy(), expected(z, k)), k
    ctx.close()
