"""Size-independent properties at the full size of the benchmark basin
(4500x3298x41, periodic in x, T+S, FCT2, Courant 0.8, delt1 240 s); the
comparisons with the oracle at this size are in test_gpu_oracle_c1.py and
test_gpu_oracle_c2c3.py:

* FP64 ensemble step: tracer content conserved to 1e-13 and no value
  outside the inputs' range (FCT keeps new extrema out);
* FP32-mixed step from the same inputs: within 1e-6 of the FP64 one
  (relative to each tracer's max |value|), content within 1e-10, range kept
  up to FP32 rounding;
* the continuity equation (cnuity) at full size: the column restored to
  pbot and the layer fluxes summing to the high-order flux.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c1(cuda):
    import bench

    wl = dict(bench.WORKLOADS["c1"])
    b, masks, nreg, case = bench.make_workload(wl, cuda)
    yield wl, b, masks, nreg, case
    import torch

    del case
    torch.cuda.empty_cache()


def _spec(b, masks, nreg, kdm):
    sc, si = b.metrics()
    return dict(idm=b.nx, jdm=b.ny, kdm=kdm, nbdy=b.nbdy, nreg=nreg, ntr=2, ip=masks["ip"], iu=masks["iu"],
                iv=masks["iv"], scp2=sc, scp2i=si)


def test_fullsize_fp64_and_mixed_step(cuda, c1):
    import torch

    import hycadv

    wl, b, masks, nreg, case = c1
    kdm = wl["kdm"]
    nb = b.nbdy
    sea = torch.from_numpy(np.asarray(masks["ip"]) != 0).to(cuda)
    sea[:nb] = False
    sea[-nb:] = False
    sea[:, :nb] = False
    sea[:, -nb:] = False
    old = torch.stack([case.temp[1], case.saln[1]]).contiguous()
    cur = torch.stack([case.temp[0], case.saln[0]]).contiguous()
    lo = [torch.minimum(old[q][:, sea].min(), cur[q][:, sea].min()).item() for q in range(2)]
    hi = [torch.maximum(old[q][:, sea].max(), cur[q][:, sea].max()).item() for q in range(2)]
    out = {}
    for prec in ("fp64", "mixed"):
        ens = hycadv.Ensemble([_spec(b, masks, nreg, kdm)], precision=prec)
        ens.put(0, "old", old)
        ens.put(0, "cur", cur)
        ens.put(0, "uflx", case.uflx)
        ens.put(0, "vflx", case.vflx)
        ens.put(0, "dp", case.dp[1].contiguous())
        if prec == "mixed":
            ens.set_tile(56, 256)
        c0 = [ens.content(0, q, "old", wl["delt1"]) for q in range(2)]
        ens.step(2, wl["delt1"], 1)
        c1_ = [ens.content(0, q, "cur", wl["delt1"]) for q in range(2)]
        new = torch.empty_like(cur)
        ens.get(0, "cur", new)
        ens.close()
        out[prec] = new
        for q in range(2):
            rel = abs(c1_[q] - c0[q]) / abs(c0[q])
            assert rel <= (1e-13 if prec == "fp64" else 1e-10), (prec, q, rel)
            v = new[q][:, sea]
            span = hi[q] - lo[q]
            tol = 0.0 if prec == "fp64" else 3e-7 * max(abs(lo[q]), abs(hi[q]))
            assert v.min().item() >= lo[q] - tol and v.max().item() <= hi[q] + tol, (prec, q)
            assert span > 0
    for q in range(2):
        a, r = out["mixed"][q][:, sea], out["fp64"][q][:, sea]
        err = ((a - r).abs().max() / r.abs().max()).item()
        assert err < 1e-6, (q, err)


def test_fullsize_cnuity(cuda, c1):
    import torch

    import hycadv

    wl, b, masks, nreg, case = c1
    kdm = wl["kdm"]
    sc, si = b.metrics()
    ctx = hycadv.Context.from_masks(masks, sc, si, kdm=kdm, nreg=nreg, nbdy=b.nbdy)
    dp = case.dp.clone()
    iu = torch.from_numpy(np.asarray(masks["iu"]) != 0).to(cuda)
    iv = torch.from_numpy(np.asarray(masks["iv"]) != 0).to(cuda)
    dx = float(np.sqrt(np.asarray(sc)).max())
    dpu = torch.zeros_like(dp)
    dpv = torch.zeros_like(dp)
    dpu[..., 1:] = 0.5 * (dp[..., 1:] + dp[..., :-1])
    dpv[..., 1:, :] = 0.5 * (dp[..., 1:, :] + dp[..., :-1, :])
    dpu *= iu
    dpv *= iv
    u = torch.zeros_like(dp)
    v = torch.zeros_like(dp)
    u[:] = torch.where(iu, case.uflx / (dpu[0].clamp(min=1.0) * dx), 0.0)
    v[:] = torch.where(iv, case.vflx / (dpv[0].clamp(min=1.0) * dx), 0.0)
    sh = tuple(dp.shape[-2:])
    f64 = dict(dtype=torch.float64, device=cuda)
    pbot = dp[0].sum(dim=0)
    p = torch.zeros((kdm + 1,) + sh, **f64)
    p[1:] = torch.cumsum(dp[0], dim=0)
    f = dict(dp=dp, dpo=torch.zeros_like(dp), dpu=dpu, dpv=dpv, u=u, v=v, ubavg=torch.zeros((3,) + sh, **f64),
             vbavg=torch.zeros((3,) + sh, **f64), pbot=pbot, p=p, uflx=torch.zeros((kdm,) + sh, **f64),
             vflx=torch.zeros((kdm,) + sh, **f64))
    for k, t in f.items():
        ctx.bind(k, t)
    pb = pbot.cpu().numpy()
    du = np.zeros_like(pb)
    dv = np.zeros_like(pb)
    du[:, 1:] = np.minimum(pb[:, 1:], pb[:, :-1])
    dv[1:, :] = np.minimum(pb[1:, :], pb[:-1, :])
    dxa = np.sqrt(np.asarray(sc, dtype=np.float64))
    ctx.set_cnuity_grid(dxa, dxa, du, dv)
    scuy = torch.from_numpy(dxa).to(cuda)
    high = ((u[0] + 0.0) * scuy * dpu[0]).sum(dim=0)  # (u + ubavg)*scuy*dpu(m)*oneta_u, ubavg = 0, m = 1
    ctx.cnuity(1, 2, delt1=wl["delt1"], nstep=1, ra2fac=0.125)
    torch.cuda.synchronize()
    nb = b.nbdy
    ip = torch.from_numpy(np.asarray(masks["ip"]) != 0).to(cuda)
    inner = torch.zeros_like(ip)
    inner[nb:-nb, nb:-nb] = True
    s = ip & inner
    rel = ((p[-1][s] - pbot[s]).abs() / pbot[s]).max().item()
    assert rel < 1e-13, rel
    face = iu & inner
    got = f["uflx"].sum(dim=0)
    err = ((got[face] - high[face]).abs().max() / high[face].abs().max()).item()
    assert err < 1e-10, err
    ctx.close()


def test_fullsize_tsdff_conserves(cuda, c1):
    """Lateral diffusion of T and S over all 41 layers of the full basin:
    sum over sea points of f*dp*oneta*scp2 per field unchanged to 1e-13,
    th3d = sig(T,S) - thbase wherever it was recomputed."""
    import torch

    import hycadv

    wl, b, masks, nreg, case = c1
    kdm = wl["kdm"]
    sc, si = b.metrics()
    ctx = hycadv.Context.from_masks(masks, sc, si, kdm=kdm, nreg=nreg, nbdy=b.nbdy)
    t = {k: getattr(case, k).clone() for k in ("temp", "saln", "th3d", "dp")}
    oneta = torch.ones((2,) + tuple(t["dp"].shape[-2:]), dtype=torch.float64, device=cuda)
    for k, v in t.items():
        ctx.bind(k, v)
    ctx.bind("oneta", oneta)
    dxa = np.sqrt(np.asarray(sc, dtype=np.float64))
    one = np.ones_like(dxa)
    ctx.set_diffusion_grid(one, one, dxa, dxa)
    nb = b.nbdy
    ip = torch.from_numpy(np.asarray(masks["ip"]) != 0).to(cuda)
    inner = torch.zeros_like(ip)
    inner[nb:-nb, nb:-nb] = True
    s = ip & inner
    scp2 = torch.from_numpy(np.asarray(sc, dtype=np.float64)).to(cuda)
    n = 2  # level n = 2 (index 1)

    def content(f):
        return (f[n - 1] * t["dp"][n - 1] * scp2)[:, s].sum().item()

    before = [content(t["temp"]), content(t["saln"])]
    t0 = t["temp"].clone()
    ctx.tsdff(1, n, delt1=wl["delt1"], temdf2=0.5)
    torch.cuda.synchronize()
    after = [content(t["temp"]), content(t["saln"])]
    for x, y in zip(before, after):
        assert abs(y - x) <= 1e-13 * abs(x), (x, y)
    assert not torch.equal(t["temp"], t0)
    ctx.close()
