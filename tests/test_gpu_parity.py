"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

The FP64 kernels keep the reference's operation order without FMA
contraction and divide exactly, so results are compared bit for bit
(values equal, -0.0 == +0.0).
"""
import os

import numpy as np
import pytest

import hycadv
from helpers import basin, levels, np_case, oracle_grid, same

pytestmark = pytest.mark.gpu
SCHEMES = [0, 1, 2, 4]


def torchify(c, dev):
    import torch

    return {k: (torch.from_numpy(v.copy()).to(dev) if isinstance(v, np.ndarray) else v) for k, v in c.items()}


def make_ctx(b, g, kdm, tile=None):
    import torch

    old = os.environ.get("HYC_TILE")
    if tile:
        os.environ["HYC_TILE"] = tile
    try:
        sc, si = b.metrics()
        ctx = hycadv.Context.from_masks(g.masks, sc, si, kdm=kdm, nreg=g.nreg, nbdy=b.nbdy)
    finally:
        if tile:
            if old is None:
                del os.environ["HYC_TILE"]
            else:
                os.environ["HYC_TILE"] = old
    ctx.set_stream(torch.cuda.current_stream())
    return ctx


def bind_all(ctx, t, extra=()):
    for k in ("temp", "saln", "th3d", "uflx", "vflx", "dp") + tuple(extra):
        ctx.bind(k, t[k])
    if t.get("tracer") is not None:
        ctx.bind("tracer", t["tracer"])


def oracle_steps(g, c, steps, advtyp, trcflg=None, **kw):
    for step in steps:
        m, n = levels(step)
        g.tsadvc(m, n, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], uflx=c["uflx"], vflx=c["vflx"],
                 dp=c["dp"], delt1=c["delt1"], advtyp=advtyp, tracer=c["tracer"], trcflg=trcflg, nstep=step, **kw)


def gpu_steps(ctx, c, steps, advtyp, ntracr=0, trcflg=None, **kw):
    for step in steps:
        m, n = levels(step)
        ctx.tsadvc(m, n, delt1=c["delt1"], advtyp=advtyp, ntracr=ntracr, trcflg=trcflg, nstep=step, **kw)


def compare(c_np, c_gpu, keys=("temp", "saln", "tracer")):
    for k in keys:
        if c_np.get(k) is None:
            continue
        got = c_gpu[k].cpu().numpy()
        assert same(got, c_np[k]), f"{k}: max |diff| = {np.nanmax(np.abs(got - c_np[k]))}"


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("advtyp", SCHEMES)
@pytest.mark.parametrize("periodic", [False, True])
def test_advem_slice_host_pointers(cuda, advtyp, periodic):
    b = basin(77, 45, periodic, seed=101)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=1, ntracr=0, seed=101, courant=0.7, delt1=600.0)
    ctx = make_ctx(b, g, 1)
    m, n = 1, 2
    fld = c["temp"][n - 1, 0].copy()
    fldc = c["temp"][m - 1, 0].copy()
    u, v = c["uflx"][0].copy(), c["vflx"][0].copy()
    for a in (fld, fldc, u, v):
        g.xctilr(a, 5, 5)
    dpn = c["dp"][n - 1, 0]
    fd = np.zeros_like(dpn)
    fd[:-1, :-1] = ((u[:-1, 1:] - u[:-1, :-1]) + (v[1:, :-1] - v[:-1, :-1])) * 600.0 * c["scp2i"][:-1, :-1]
    fco = np.maximum(dpn + fd, 0.0)
    fcn = np.maximum(dpn, 0.0)
    ref = fld.copy()
    g.advem(advtyp, ref, fldc, u, v, fco, fcn, 256.0, c["scp2"], c["scp2i"], 600.0)
    got = fld.copy()
    ctx.advem(advtyp, got, fldc, u, v, fco, fcn, 256.0, c["scp2"], c["scp2i"], 600.0)
    assert same(got, ref)
    assert not np.array_equal(got, fld)  # something moved


@pytest.mark.parametrize("advtyp", SCHEMES)
def test_advem_slice_device_pointers(cuda, advtyp):
    import torch

    b = basin(64, 70, True, seed=102)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=1, ntracr=1, seed=102, courant=0.8, delt1=240.0)
    ctx = make_ctx(b, g, 1)
    fld = c["tracer"][0, 1, 0].copy()
    fldc = c["tracer"][0, 0, 0].copy()
    u, v = c["uflx"][0].copy(), c["vflx"][0].copy()
    for a in (fld, fldc, u, v):
        g.xctilr(a, 5, 5)
    fco = np.maximum(c["dp"][1, 0] * 1.01, 0.0)
    fcn = c["dp"][1, 0].copy()
    ref = fld.copy()
    g.advem(advtyp, ref, fldc, u, v, fco, fcn, 0.0, c["scp2"], c["scp2i"], 240.0)
    T = [torch.from_numpy(a.copy()).to(cuda) for a in (fld, fldc, u, v, fco, fcn, c["scp2"], c["scp2i"])]
    ctx.advem(advtyp, T[0], T[1], T[2], T[3], T[4], T[5], 0.0, T[6], T[7], 240.0)
    torch.cuda.synchronize()
    assert same(T[0].cpu().numpy(), ref)


@pytest.mark.parametrize("periodic", [False, True])
def test_advem_fct2c_slice(cuda, periodic):
    """advem_fct2c (FCT2 with btrmas, mod_tsadvc.F90:999-1368) on one slice:
    five sub-cycled donor-cell passes with the halo refreshed between them,
    at a Courant number that makes cells sub-cycle; bit for bit."""
    b = basin(77, 45, periodic, seed=131)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=1, ntracr=0, seed=131, courant=1.4, delt1=1800.0)
    ctx = make_ctx(b, g, 1)
    fld = c["saln"][1, 0].copy()
    fldc = c["saln"][0, 0].copy()
    u, v = c["uflx"][0].copy(), c["vflx"][0].copy()
    for a in (fld, fldc, u, v):
        g.xctilr(a, 5, 5)
    dpn = c["dp"][1, 0]
    fd = np.zeros_like(dpn)
    fd[:-1, :-1] = ((u[:-1, 1:] - u[:-1, :-1]) + (v[1:, :-1] - v[:-1, :-1])) * 1800.0 * c["scp2i"][:-1, :-1]
    fco = np.maximum(dpn + fd, 0.0)
    fcn = np.maximum(dpn, 0.0)
    ref = fld.copy()
    g.advem(2, ref, fldc, u, v, fco, fcn, 0.0, c["scp2"], c["scp2i"], 1800.0, btrmas=True)
    got = fld.copy()
    ctx.advem(2, got, fldc, u, v, fco, fcn, 0.0, c["scp2"], c["scp2i"], 1800.0, btrmas=True)
    assert same(got, ref)
    assert not np.array_equal(got, fld)


@pytest.mark.parametrize("periodic", [False, True])
def test_tsadvc_fct2c_btrmas(cuda, periodic):
    """tsadvc with btrmas (onetamas != 1 scales the thickness, :1804-1810;
    every field goes through advem_fct2c) bit for bit over three steps,
    T, S and a passive tracer."""
    b = basin(90, 60, periodic, seed=31)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=3, ntracr=1, seed=31, courant=1.2, delt1=1800.0)
    c["delt1"] = 1800.0
    rng = np.random.default_rng(31)
    c["oneta"] = 1.0 + 0.05 * rng.standard_normal((2,) + c["dp"].shape[2:])
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, 3)
    bind_all(ctx, t, extra=("oneta",))
    tf = np.array([0], np.int32)
    oracle_steps(g, c, range(1, 4), 2, trcflg=tf, btrmas=True, oneta=c["oneta"])
    gpu_steps(ctx, t, range(1, 4), 2, ntracr=1, trcflg=tf, btrmas=True)
    compare(c, t)


def test_tsadvc_c0_fct2_twenty_steps(cuda):
    """257x193x10 closed basin, T and S, FCT2, dt 1800 s, Courant 0.5, 20 steps."""
    b = basin(257, 193, False, seed=7)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=10, ntracr=0, seed=7, courant=0.5, delt1=1800.0)
    c["delt1"] = 1800.0
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, 10)
    bind_all(ctx, t)
    for s0 in range(1, 21, 5):
        steps = range(s0, s0 + 5)
        oracle_steps(g, c, steps, 2)
        gpu_steps(ctx, t, steps, 2)
        compare(c, t, keys=("temp", "saln", "th3d", "uflx", "vflx"))


@pytest.mark.parametrize("advtyp", SCHEMES)
def test_tsadvc_periodic_tracers(cuda, advtyp):
    """Periodic-x basin with a temperature-like tracer and passive tracers."""
    b = basin(150, 90, True, seed=8)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=4, ntracr=3, seed=8, courant=0.8, delt1=240.0)
    c["delt1"] = 240.0
    c["tracer"][0] = c["temp"]
    tf = np.array([2, 0, 0], np.int32)
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, 4)
    bind_all(ctx, t)
    oracle_steps(g, c, range(1, 5), advtyp, trcflg=tf)
    gpu_steps(ctx, t, range(1, 5), advtyp, ntracr=3, trcflg=tf)
    compare(c, t)
    got = t["tracer"].cpu().numpy()
    ip = g.masks["ip"] != 0
    assert same(got[0][..., ip], t["temp"].cpu().numpy()[..., ip])  # mod_pipe.F90:1516-1534


@pytest.mark.parametrize("tile", ["16x16", "32x16", "32x32"])
@pytest.mark.parametrize("nx,ny", [(37, 29), (8, 7), (100, 17)])
def test_tsadvc_ragged_sizes_and_tiles(cuda, tile, nx, ny):
    b = basin(nx, ny, False, seed=9) if (nx, ny) != (8, 7) else basin(8, 7, False, seed=9)
    if (nx, ny) == (8, 7):
        b.depth[:] = 0.0
        b.depth[b.nbdy + 2:b.nbdy + 5, b.nbdy + 2:b.nbdy + 6] = 100.0  # 4x3 sea box inside the wall
    g = oracle_grid(b)
    c = np_case(b, g, kdm=2, ntracr=1, seed=9, courant=0.6, delt1=900.0)
    c["delt1"] = 900.0
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, 2, tile=tile)
    bind_all(ctx, t)
    tf = np.array([0], np.int32)
    oracle_steps(g, c, range(1, 4), 2, trcflg=tf)
    gpu_steps(ctx, t, range(1, 4), 2, ntracr=1, trcflg=tf)
    compare(c, t)


def test_tsadvc_many_tracers_chunked(cuda):
    """More advected fields than one launch takes (temp, saln + 20 tracers)."""
    b = basin(48, 40, True, seed=10)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=2, ntracr=20, seed=10, courant=0.8, delt1=240.0)
    c["delt1"] = 240.0
    tf = np.zeros(20, np.int32)
    tf[5] = 2
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, 2)
    bind_all(ctx, t)
    oracle_steps(g, c, range(1, 3), 2, trcflg=tf)
    gpu_steps(ctx, t, range(1, 3), 2, ntracr=20, trcflg=tf)
    compare(c, t)


@pytest.mark.parametrize("advtyp", [1, 2])
def test_tsadvc_th3d_hybrid_layers_and_mxlmy(cuda, advtyp):
    """advflg=1 (th3d and saln), nhybrd < kdm (saln only below), q2/q2l."""
    b = basin(60, 50, False, seed=11)
    g = oracle_grid(b)
    kdm = 4
    c = np_case(b, g, kdm=kdm, ntracr=0, seed=11, courant=0.5, delt1=1800.0)
    c["delt1"] = 1800.0
    rng = np.random.default_rng(11)
    q2 = (0.01 + rng.random((2, kdm + 2, b.ld2, b.ld1)) * 0.1)
    q2l = (0.1 + rng.random((2, kdm + 2, b.ld2, b.ld1)))
    c["q2"], c["q2l"] = q2, q2l
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, kdm)
    bind_all(ctx, t, extra=("q2", "q2l"))
    kw = dict(advflg=1, nhybrd=2, mxlmy=True)
    oracle_steps(g, c, range(1, 4), advtyp, q2=c["q2"], q2l=c["q2l"], **kw)
    gpu_steps(ctx, t, range(1, 4), advtyp, **kw)
    compare(c, t, keys=("temp", "saln", "th3d", "q2", "q2l"))


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("mh,nh", [(5, 5), (2, 3), (6, 6), (0, 4)])
def test_xctilr_device(cuda, periodic, mh, nh):
    import torch

    b = basin(41, 33, periodic, seed=12)
    g = oracle_grid(b)
    ctx = make_ctx(b, g, 1)
    a = np.random.default_rng(1).standard_normal((3, b.ld2, b.ld1))
    ref = a.copy()
    g.xctilr(ref, mh, nh)
    T = torch.from_numpy(a.copy()).to(cuda)
    ctx.xctilr(T, mh, nh)
    torch.cuda.synchronize()
    assert same(T.cpu().numpy(), ref)
    h = a.copy()
    ctx.xctilr(h, mh, nh)  # host pointer path
    assert same(h, ref)


def test_salinity_range_diagnostic(cuda):
    b = basin(80, 60, False, seed=13)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=3, ntracr=0, seed=13, courant=0.5, delt1=1800.0)
    c["delt1"] = 1800.0
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, 3)
    bind_all(ctx, t)
    m, n = levels(3)
    xmin, xmax = g.tsadvc(m, n, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], uflx=c["uflx"], vflx=c["vflx"],
                          dp=c["dp"], delt1=1800.0, advtyp=2, nstep=3)
    r = ctx.tsadvc(m, n, delt1=1800.0, advtyp=2, nstep=3, range_diag=True)
    assert r is not None
    assert np.array_equal(r[0], xmin) and np.array_equal(r[1], xmax)
    assert ctx.tsadvc(m, n, delt1=1800.0, advtyp=2, nstep=4, range_diag=True) is None  # mod(nstep,3) != 0


def test_mass_sum_compensated_and_reproducible(cuda):
    import math

    import torch

    b = basin(120, 90, False, seed=14)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=1, ntracr=1, seed=14, courant=0.5, delt1=1800.0)
    ctx = make_ctx(b, g, 1)
    fld = torch.from_numpy(c["tracer"][0, 0, 0].copy()).to(cuda)
    fc = torch.from_numpy(c["dp"][0, 0].copy()).to(cuda)
    s1 = ctx.mass_sum(fld, fc)
    s2 = ctx.mass_sum(fld, fc)
    assert s1 == s2
    msk = (g.masks["ip"] != 0)
    inner = np.zeros_like(msk)
    inner[b.J, b.I] = True
    f, h, sc = c["tracer"][0, 0, 0], c["dp"][0, 0], c["scp2"]
    terms = (f * (h + 9806.e-12) * sc)[msk & inner]
    exact = math.fsum(terms.tolist())
    assert abs(s1 - exact) <= 1e-15 * abs(exact)


def test_error_paths(cuda):
    import torch

    b = basin(40, 30, False, seed=15)
    g = oracle_grid(b)
    ctx = make_ctx(b, g, 2)
    with pytest.raises(hycadv.HycError) as e:
        ctx.tsadvc(1, 2, delt1=100.0)  # nothing bound
    assert e.value.code == -6
    c = np_case(b, g, kdm=2, ntracr=0, seed=15, courant=0.5, delt1=100.0)
    t = torchify(c, cuda)
    bind_all(ctx, t)
    with pytest.raises(hycadv.HycError) as e:
        ctx.tsadvc(1, 2, delt1=100.0, advtyp=3)  # mod_tsadvc.F90:159-165
    assert e.value.code == -2
    with pytest.raises(hycadv.HycError) as e:
        ctx.tsadvc(1, 2, delt1=100.0, advtyp=2, btrmas=True)
    assert e.value.code in (-6, -8)
    with pytest.raises(hycadv.HycError) as e:  # isopycnic mode has no hybrid layers (nhybrd = 0)
        ctx.tsadvc(1, 2, delt1=100.0, isopyc=True)
    assert e.value.code == -1
    with pytest.raises(hycadv.HycError) as e:
        ctx.tsadvc(0, 2, delt1=100.0)
    assert e.value.code == -1
    # a failed call leaves the context usable
    ctx.tsadvc(1, 2, delt1=100.0, advtyp=2)
    torch.cuda.synchronize()


def test_za_read_into_device_memory(cuda, tmp_path):
    """A .a record read straight into a device array (HYC_DEVICE) equals the
    host read; with a mask the unmasked device points are kept."""
    import torch

    from hycadv import za

    idm, jdm, nb = 61, 47, 6
    rng = np.random.default_rng(3)
    f = rng.normal(5.0, 2.0, (jdm, idm)).astype(np.float32).astype(np.float64)
    a = str(tmp_path / "d.a")
    za.write_record_file(a, [f, 2 * f], idm, jdm)
    host = np.full((jdm + 2 * nb, idm + 2 * nb), -1.0)
    dev = torch.full(host.shape, -1.0, dtype=torch.float64, device=cuda)
    assert za.read_record(a, 2, idm, jdm, nb, host) == za.read_record(a, 2, idm, jdm, nb, dev)
    assert np.array_equal(dev.cpu().numpy(), host)
    mask = np.zeros(host.shape, np.int32)
    mask[nb:nb + 10, nb:nb + 20] = 1
    dev.fill_(-3.0)
    za.read_record(a, 1, idm, jdm, nb, dev, mask=mask)
    got = dev.cpu().numpy()
    assert np.array_equal(got[mask != 0], f[:10, :20].ravel())
    assert np.all(got[mask == 0] == -3.0)


@pytest.mark.parametrize("advtyp", SCHEMES)
@pytest.mark.parametrize("periodic", [False, True])
def test_tsadvc_isopycnic_bit_for_bit(cuda, advtyp, periodic):
    """Isopycnic mode (nhybrd = 0, mod_tsadvc.F90:1855-1897): layer 1
    advects th3d and saln with the smoothed mixed-layer fluxes, its tracers
    (and q2, q2l) with the layer's own fluxes and the thickness factors of
    the smoothed ones; deeper layers advect saln and the tracers only."""
    b = basin(83, 61, periodic, seed=131)
    g = oracle_grid(b)
    kdm = 3
    c = np_case(b, g, kdm=kdm, ntracr=2, seed=131, courant=0.7, delt1=600.0)
    c["delt1"] = 600.0
    rng = np.random.default_rng(131)
    c["q2"] = 0.01 + rng.random((2, kdm + 2, b.ld2, b.ld1)) * 0.1
    c["q2l"] = 0.1 + rng.random((2, kdm + 2, b.ld2, b.ld1))
    tf = np.array([0, 2], np.int32)
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, kdm)
    bind_all(ctx, t, extra=("q2", "q2l"))
    kw = dict(isopyc=True, nhybrd=0, mxlmy=True)
    temp0 = c["temp"].copy()
    oracle_steps(g, c, range(1, 4), advtyp, trcflg=tf, q2=c["q2"], q2l=c["q2l"], **kw)
    gpu_steps(ctx, t, range(1, 4), advtyp, ntracr=2, trcflg=tf, **kw)
    compare(c, t, keys=("temp", "saln", "th3d", "tracer", "q2", "q2l"))
    # temperature is not advected in isopycnic mode (its halo is refreshed)
    assert np.array_equal(c["temp"][..., b.J, b.I], temp0[..., b.J, b.I])
    # the smoothing changes layer 1: the same step with hybrid layers differs
    c2 = np_case(b, g, kdm=kdm, ntracr=0, seed=131, courant=0.7, delt1=600.0)
    c2["delt1"] = 600.0
    c2["tracer"] = None
    oracle_steps(g, c2, [1], advtyp, advflg=1)
    t2 = np_case(b, g, kdm=kdm, ntracr=0, seed=131, courant=0.7, delt1=600.0)
    t2["delt1"] = 600.0
    t2["tracer"] = None
    oracle_steps(g, t2, [1], advtyp, isopyc=True, nhybrd=0)
    assert not np.array_equal(c2["th3d"][1, 0], t2["th3d"][1, 0])


def test_tsadvc_isopycnic_rejects_fct2c(cuda):
    b = basin(40, 30, False, seed=132)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=2, ntracr=0, seed=132, courant=0.5, delt1=600.0)
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, 2)
    bind_all(ctx, t, extra=())
    with pytest.raises(hycadv.HycError):
        ctx.tsadvc(1, 2, delt1=600.0, advtyp=2, btrmas=True, isopyc=True, nhybrd=0)
    with pytest.raises(hycadv.HycError):
        ctx.tsadvc(1, 2, delt1=600.0, advtyp=2, isopyc=True, nhybrd=2)


@pytest.mark.parametrize("advtyp", SCHEMES)
def test_tsadvc_lconserve_bit_for_bit(cuda, advtyp):
    """advem's explicit conservation rescale (lconserve, mod_tsadvc.F90:168-203):
    xcsum-ordered content sums before and after each advem, new values at
    sea points scaled by 1 + (old-new)/new; equal to the oracle bit for bit,
    and different from the run without it."""
    b = basin(70, 52, True, seed=141)
    g = oracle_grid(b)
    g.set_conserve(True)
    c = np_case(b, g, kdm=3, ntracr=1, seed=141, courant=0.7, delt1=600.0)
    c["delt1"] = 600.0
    tf = np.array([0], np.int32)
    plain = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in c.items()}
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, 3)
    ctx.set_conserve(True)
    bind_all(ctx, t)
    oracle_steps(g, c, range(1, 4), advtyp, trcflg=tf)
    gpu_steps(ctx, t, range(1, 4), advtyp, ntracr=1, trcflg=tf)
    compare(c, t)
    g.set_conserve(False)
    oracle_steps(g, plain, range(1, 4), advtyp, trcflg=tf)
    assert not np.array_equal(plain["saln"], c["saln"])


def test_advem_lconserve_slice(cuda):
    """hyc_advem on one slice with the rescale, host pointers, FCT2."""
    b = basin(64, 48, False, seed=142)
    g = oracle_grid(b)
    g.set_conserve(True)
    c = np_case(b, g, kdm=1, ntracr=0, seed=142, courant=0.7, delt1=600.0)
    ctx = make_ctx(b, g, 1)
    ctx.set_conserve(True)
    fld = c["temp"][1, 0].copy()
    fldc = c["temp"][0, 0].copy()
    u, v = c["uflx"][0].copy(), c["vflx"][0].copy()
    for a in (fld, fldc, u, v):
        g.xctilr(a, 5, 5)
    fco = np.maximum(c["dp"][1, 0] * 1.02, 0.0)
    fcn = c["dp"][1, 0].copy()
    ref = fld.copy()
    g.advem(2, ref, fldc, u, v, fco, fcn, 0.0, c["scp2"], c["scp2i"], 600.0)
    got = fld.copy()
    ctx.advem(2, got, fldc, u, v, fco, fcn, 0.0, c["scp2"], c["scp2i"], 600.0)
    assert same(got, ref)
    with pytest.raises(hycadv.HycError):  # advem_fct2c forms no content arrays
        ctx.advem(2, got, fldc, u, v, fco, fcn, 0.0, c["scp2"], c["scp2i"], 600.0, btrmas=True)
