"""The precision and batching forms against the oracle at the configured
sizes.

* Precision form (the 4500x3298x41 basin with T, S and 8 passive tracers,
  log-uniform in [1e-6, 1e2] with step fronts): one FP32-mixed step
  (FP32 fluxes, limiter and update; FP64 thickness prep and dp) through the
  ensemble API, every tracer within 1e-6 of the oracle's FP64 tsadvc
  relative to the tracer's max |value|; the RMS error is printed.
* Batching form: the largest and the smallest member of the 96-basin
  ensemble (seeded uneven sizes, 2-6 tracers) advanced together in one
  ensemble: FP64 bit for bit with the oracle, FP32-mixed within 1e-6.

The oracle runs on the host on runs of 8 layers (the advection of tsadvc
treats each layer on its own), the GPU on whole basins.
"""
import numpy as np
import pytest

from helpers import levels, same

pytestmark = pytest.mark.gpu

CHUNK = 8
KINDS = ("temp", "saln")


def _sea(b, masks):
    ip = np.asarray(masks["ip"]) != 0
    inner = np.zeros_like(ip)
    inner[b.J, b.I] = True
    return ip & inner


def _make(member, wl, dev, periodic):
    """Basin, masks, spec, flow and tracer levels (FP64, on the device)."""
    import hycadv
    from hycadv import synth

    b = synth.make_basin(member["nx"], member["ny"], periodic, member["seed"])
    _, masks, nreg = hycadv.bigrid(b.depth, b.nbdy)
    sc, si = b.metrics()
    kdm, ntr = member["kdm"], member["ntr"]
    spec = dict(idm=b.nx, jdm=b.ny, kdm=kdm, nbdy=b.nbdy, nreg=nreg, ntr=ntr, ip=masks["ip"], iu=masks["iu"],
                iv=masks["iv"], scp2=sc, scp2i=si)
    dp, uflx, vflx = synth.flow_fields(b, masks, kdm, member["seed"], wl["courant"], wl["delt1"], dev)
    trc = [synth.tracer_levels(b, KINDS[q] if q < 2 else "passive", kdm, member["seed"], q=max(q - 2, 0),
                               device=dev) for q in range(ntr)]
    return dict(b=b, masks=masks, spec=spec, dp=dp, uflx=uflx, vflx=vflx, trc=trc)


def _put(ens, i, d):
    m, n = levels(1)  # level n holds t-1 on entry
    ens.put(i, "uflx", d["uflx"])
    ens.put(i, "vflx", d["vflx"])
    ens.put(i, "dp", d["dp"][n - 1].contiguous())
    kdm = d["spec"]["kdm"]
    for q, lv in enumerate(d["trc"]):
        ens.put(i, "old", lv[n - 1].contiguous(), s0=q * kdm, ns=kdm)
        ens.put(i, "cur", lv[m - 1].contiguous(), s0=q * kdm, ns=kdm)


def _oracle_new(d, wl, k0, k1, dparams=None):
    """The oracle's new level (t+1) of every tracer for layers k0..k1-1;
    with dparams (temdf2 and the grid arrays), tsadvc's diffusion block after
    the advection."""
    from oracle import oracle

    b = d["b"]
    sc, si = b.metrics()
    g = oracle.Grid(b.depth, sc, si, nbdy=b.nbdy)
    assert np.array_equal(g.masks["ip"], np.asarray(d["masks"]["ip"]))
    h = lambda t: np.ascontiguousarray(t.cpu().numpy())
    temp, saln = h(d["trc"][0][:, k0:k1]), h(d["trc"][1][:, k0:k1])
    ntr = len(d["trc"])
    tracer = np.ascontiguousarray(np.stack([h(t[:, k0:k1]) for t in d["trc"][2:]])) if ntr > 2 else None
    dp = h(d["dp"][:, k0:k1])
    m, n = levels(1)
    g.tsadvc(m, n, temp=temp, saln=saln, th3d=np.zeros_like(temp), uflx=h(d["uflx"][k0:k1]),
             vflx=h(d["vflx"][k0:k1]), dp=dp, delt1=wl["delt1"], advtyp=2, tracer=tracer,
             trcflg=np.zeros(max(ntr - 2, 1), np.int32), nstep=1)
    if dparams is not None:
        g.tsdff(m, n, temp=temp, saln=saln, th3d=np.zeros_like(temp), dp=dp, oneta=np.ones((2, b.ld2, b.ld1)),
                delt1=wl["delt1"], tracer=tracer, **dparams)
    out = [temp[n - 1], saln[n - 1]] + ([tracer[q, n - 1] for q in range(ntr - 2)] if ntr > 2 else [])
    return out


def _compare(ens, i, d, wl, exact, label, dparams=None):
    """Per tracer (max rel err, rms rel err) of the ensemble's new level against
    the oracle, over interior sea cells, layer runs of CHUNK."""
    import torch

    b, kdm, ntr = d["b"], d["spec"]["kdm"], d["spec"]["ntr"]
    sea = _sea(b, d["masks"])
    dmax = np.zeros(ntr)
    sq = np.zeros(ntr)
    scale = np.zeros(ntr)
    count = 0
    buf = torch.empty((CHUNK, b.ld2, b.ld1), dtype=torch.float64)
    for k0 in range(0, kdm, CHUNK):
        k1 = min(kdm, k0 + CHUNK)
        want = _oracle_new(d, wl, k0, k1, dparams)
        for q in range(ntr):
            got = buf[:k1 - k0]
            ens.get(i, "cur", got, s0=q * kdm + k0, ns=k1 - k0)
            a, w = got.numpy()[:, sea], want[q][:, sea]
            if exact:
                assert same(a, w), f"{label}: tracer {q} layers {k0 + 1}-{k1}"
            diff = np.abs(a - w)
            dmax[q] = max(dmax[q], diff.max())
            sq[q] += float((diff ** 2).sum())
            scale[q] = max(scale[q], np.abs(w).max())
        count += (k1 - k0) * int(sea.sum())
    return dmax / scale, np.sqrt(sq / count) / scale


def test_c2_precision_form_each_tracer_within_1e6_of_oracle(cuda):
    import torch

    import bench
    import hycadv

    torch.cuda.empty_cache()  # the ensemble allocates outside torch's cache
    wl = dict(bench.WORKLOADS["c2"])
    d = _make(dict(nx=wl["nx"], ny=wl["ny"], kdm=wl["kdm"], ntr=wl["ntr"], seed=wl["seed"]), wl, cuda, True)
    ens = hycadv.Ensemble([d["spec"]], precision="mixed")
    assert ens.option("prep64") == 1
    _put(ens, 0, d)
    ens.step(2, wl["delt1"], 1)
    torch.cuda.synchronize()
    mx, rms = _compare(ens, 0, d, wl, False, "c2")
    ens.close()
    for q in range(wl["ntr"]):
        print(f"c2 tracer {q}: max rel err {mx[q]:.2e}, rms rel err {rms[q]:.2e}")
        assert mx[q] < 1e-6, (q, mx[q])


def test_c3_extreme_members_against_oracle(cuda):
    import torch

    import bench
    import hycadv

    wl = dict(bench.WORKLOADS["c3"])
    members = bench.c3_members(wl)
    size = [m["nx"] * m["ny"] * m["kdm"] * m["ntr"] for m in members]
    pick = [members[int(np.argmax(size))], members[int(np.argmin(size))]]
    data = [_make(m, wl, cuda, wl["periodic"]) for m in pick]
    for prec in ("fp64", "mixed"):
        ens = hycadv.Ensemble([d["spec"] for d in data], precision=prec)
        for i, d in enumerate(data):
            _put(ens, i, d)
        ens.step(2, wl["delt1"], 1)
        torch.cuda.synchronize()
        for i, d in enumerate(data):
            s = d["spec"]
            mx, rms = _compare(ens, i, d, wl, prec == "fp64", f"c3 {prec} member {s['idm']}x{s['jdm']}")
            print(f"c3 {prec} {s['idm']}x{s['jdm']}x{s['kdm']} ntr {s['ntr']}: max rel err {mx.max():.2e}")
            assert mx.max() < 1e-6
        ens.close()


def test_c1_fused_diffusion_against_oracle(cuda):
    """The precision form with the diffusion epilogue on the 4500x3298 basin
    (T and S, 8 layers): within 1e-6 of the oracle's tsadvc followed by its
    diffusion block (mod_tsadvc.F90:2138-2230) on a uniform grid."""
    import torch

    import bench
    import hycadv

    torch.cuda.empty_cache()
    wl = dict(bench.WORKLOADS["c1"])
    d = _make(dict(nx=wl["nx"], ny=wl["ny"], kdm=CHUNK, ntr=2, seed=wl["seed"]), wl, cuda, True)
    dx = np.sqrt(d["b"].metrics()[0])
    grid = dict(aspux=np.ones_like(dx), aspvy=np.ones_like(dx), scuy=dx, scvx=dx)
    ens = hycadv.Ensemble([d["spec"]], precision="mixed")
    ens.set_diffusion(0, bench.TEMDF2, **grid)
    _put(ens, 0, d)
    ens.step(2, wl["delt1"], 1)
    torch.cuda.synchronize()
    mx, rms = _compare(ens, 0, d, wl, False, "c1 diffusion", dparams=dict(temdf2=bench.TEMDF2, **grid))
    ens.close()
    for q in range(2):
        print(f"c1 with diffusion, tracer {q}: max rel err {mx[q]:.2e}, rms rel err {rms[q]:.2e}")
        assert mx[q] < 1e-6, (q, mx[q])
