"""Ensemble (batched) form on the GPU: FP64 bit for bit against the oracle,
FP32-mixed within its error budget, graph replay equal to eager launches,
tuning leaves the state unchanged, tracer content conserved."""
import numpy as np
import pytest

import hycadv
from helpers import basin, levels, np_case, oracle_grid, same

pytestmark = pytest.mark.gpu

SPECS = [  # nx, ny, periodic, kdm, ntr, seed, courant, delt1
    (60, 45, False, 3, 2, 401, 0.5, 1800.0),
    (70, 40, True, 2, 3, 402, 0.8, 1800.0),
    (33, 27, False, 4, 1, 403, 0.6, 1800.0),
]
DELT1 = 1800.0


def make_members(specs=SPECS, delt1=DELT1):
    out = []
    for nx, ny, per, kdm, ntr, seed, cour, _ in specs:
        b = basin(nx, ny, per, seed)
        g = oracle_grid(b)
        c = np_case(b, g, kdm=kdm, ntracr=max(ntr - 1, 0), seed=seed, courant=cour, delt1=delt1)
        # ensemble tracers: 0 -> saln, 1.. -> the oracle's tracer array
        trc = np.concatenate([c["saln"][None]] + ([c["tracer"]] if ntr > 1 else []), axis=0)  # (ntr, 2, kdm, ...)
        out.append(dict(b=b, g=g, c=c, ntr=ntr, kdm=kdm, trc=trc))
    return out


def spec_of(m):
    b, g = m["b"], m["g"]
    sc, si = b.metrics()
    return dict(idm=b.nx, jdm=b.ny, kdm=m["kdm"], nbdy=b.nbdy, nreg=g.nreg, ntr=m["ntr"], ip=g.masks["ip"],
                iu=g.masks["iu"], iv=g.masks["iv"], scp2=sc, scp2i=si)


def load(ens, members, first_step=1):
    for i, m in enumerate(members):
        mm, nn = levels(first_step)
        old = np.ascontiguousarray(m["trc"][:, nn - 1])
        cur = np.ascontiguousarray(m["trc"][:, mm - 1])
        ens.put(i, "old", old)
        ens.put(i, "cur", cur)
        ens.put(i, "uflx", np.ascontiguousarray(m["c"]["uflx"]))
        ens.put(i, "vflx", np.ascontiguousarray(m["c"]["vflx"]))
        ens.put(i, "dp", np.ascontiguousarray(m["c"]["dp"][nn - 1]))


def oracle_step(m, step, advtyp):
    c = m["c"]
    mm, nn = levels(step)
    g = m["g"]
    g.tsadvc(mm, nn, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], uflx=c["uflx"], vflx=c["vflx"], dp=c["dp"],
             delt1=DELT1, advtyp=advtyp, tracer=c["tracer"] if m["ntr"] > 1 else None,
             trcflg=np.zeros(max(m["ntr"] - 1, 1), np.int32), nhybrd=0, nstep=step)
    trc = np.concatenate([c["saln"][None]] + ([c["tracer"]] if m["ntr"] > 1 else []), axis=0)
    return np.ascontiguousarray(trc[:, nn - 1])  # the new level


def sea_interior(m):
    """Sea cells of the interior: the halo of a new level is refreshed by the
    ensemble at once and by tsadvc only at its next call."""
    b = m["b"]
    msk = np.zeros_like(m["g"].masks["ip"], dtype=bool)
    msk[b.J, b.I] = True
    return msk & (m["g"].masks["ip"] != 0)


def get_cur(ens, i, m):
    out = np.zeros((m["ntr"], m["kdm"], m["b"].ld2, m["b"].ld1))
    return ens.get(i, "cur", out)


@pytest.mark.parametrize("advtyp", [2, 4])
def test_fp64_ensemble_bitwise(cuda, advtyp):
    members = make_members()
    ens = hycadv.Ensemble([spec_of(m) for m in members], precision="fp64")
    load(ens, members)
    for step in range(1, 5):
        ens.step(advtyp, DELT1, 1)
        for i, m in enumerate(members):
            want = oracle_step(m, step, advtyp)
            got = get_cur(ens, i, m)
            ip = sea_interior(m)
            assert same(got[..., ip], want[..., ip]), f"basin {i} step {step}"
            # dp is constant here, but every step reads dp(:,:,k,n) of its own n
            mm, nn = levels(step + 1)
            ens.put(i, "dp", np.ascontiguousarray(m["c"]["dp"][nn - 1]))
    ens.close()


def test_graph_replay_equals_eager(cuda):
    results = []
    for prec in ("fp64", "mixed"):
        per = []
        for graph in (False, True):
            members = make_members(SPECS[:2])
            ens = hycadv.Ensemble([spec_of(m) for m in members], precision=prec)
            load(ens, members)
            ens.step(2, DELT1, 3, graph=graph)
            per.append([get_cur(ens, i, m) for i, m in enumerate(members)])
            ens.close()
        for a, b in zip(per[0], per[1]):
            assert np.array_equal(a, b)
        results.append(per)


def test_tune_keeps_state(cuda):
    members = make_members(SPECS[:2])
    ens = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
    load(ens, members)
    before = [get_cur(ens, i, m) for i, m in enumerate(members)]
    tx, ty, ms = ens.tune(2, DELT1)
    assert tx == 56 and ty in (32, 64, 128, 256, 512, 1024, 2048)
    assert ms > 0
    after = [get_cur(ens, i, m) for i, m in enumerate(members)]
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    ens.close()


@pytest.mark.parametrize("prep64", [True, False])
def test_mixed_one_step_error(cuda, prep64):
    """From identical inputs, one FP32-mixed step is within 1e-6 (relative to
    each tracer's max |value|) of the FP64 oracle, with the thickness prep in
    FP64 or in compensated FP32."""
    members = make_members()
    ens = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
    ens.set_prep64(prep64)
    load(ens, members)
    ens.step(2, DELT1, 1)
    for i, m in enumerate(members):
        want = oracle_step(m, 1, 2)
        got = get_cur(ens, i, m)
        ip = sea_interior(m)
        for q in range(m["ntr"]):
            err = np.abs(got[q][..., ip] - want[q][..., ip]).max() / np.abs(want[q][..., ip]).max()
            assert err < 1e-6, (i, q, err)
    ens.close()


@pytest.mark.parametrize("prec,prep64,cons_tol,err_tol,advtyp",
                         [("fp64", True, 1e-13, 0.0, 2), ("mixed", True, 1e-6, 1e-4, 2), ("mixed", False, 1e-6, 1e-4, 2),
                          ("mixed", False, 1e-6, 1e-4, 4)])
def test_ensemble_multistep_conservation_extrema(cuda, prec, prep64, cons_tol, err_tol, advtyp):
    """20 steps of FCT2 or FCT4: tracer content conserved (FP64 to round-off),
    no new extrema, and the FP32-mixed drift from the oracle stays within
    the envelope of the leapfrog-FCT dynamics (an FP64 run perturbed by one
    FP32 rounding of its inputs already drifts ~1e-6 to 1e-5 in 20 steps,
    FCT2 and FCT4 alike)."""
    members = make_members()
    ens = hycadv.Ensemble([spec_of(m) for m in members], precision=prec)
    if prec == "mixed":
        ens.set_prep64(prep64)
        if advtyp == 4:
            ens.set_tile(56, 64)
    load(ens, members)
    nsteps = 20
    start = [(m["trc"][..., m["g"].masks["ip"] != 0].min(), m["trc"][..., m["g"].masks["ip"] != 0].max())
             for m in members]
    worst_cons = 0.0
    for step in range(1, nsteps + 1):
        for i, m in enumerate(members):
            mm, nn = levels(step)
            ens.put(i, "dp", np.ascontiguousarray(m["c"]["dp"][nn - 1]))
        c_old = [[ens.content(i, q, "old", DELT1) for q in range(m["ntr"])] for i, m in enumerate(members)]
        ens.step(advtyp, DELT1, 1)
        c_new = [[ens.content(i, q, "cur", DELT1) for q in range(m["ntr"])] for i, m in enumerate(members)]
        for i, m in enumerate(members):
            for q in range(m["ntr"]):
                worst_cons = max(worst_cons, abs(c_new[i][q] - c_old[i][q]) / abs(c_old[i][q]))
            oracle_step(m, step, advtyp)
    print(f"{prec} advtyp {advtyp}: worst relative content change in one step {worst_cons:.2e}")
    assert worst_cons < cons_tol
    for i, m in enumerate(members):
        mm, nn = levels(nsteps)
        c = m["c"]
        want = np.concatenate([c["saln"][None]] + ([c["tracer"]] if m["ntr"] > 1 else []), axis=0)[:, nn - 1]
        got = get_cur(ens, i, m)
        ip = sea_interior(m)
        for q in range(m["ntr"]):
            err = np.abs(got[q][..., ip] - want[q][..., ip]).max() / np.abs(want[q][..., ip]).max()
            print(f"{prec}: basin {i} tracer {q}: max rel err after {nsteps} steps {err:.2e}")
            assert err <= err_tol
        lo, hi = start[i]
        assert got[..., ip].min() >= lo - 1e-6 * abs(lo) and got[..., ip].max() <= hi + 1e-6 * abs(hi)
    ens.close()


@pytest.mark.parametrize("prep64", [True, False])
def test_mixed_strip_shapes_agree(cuda, prep64):
    """The strip kernel gives the same update for every segment height (the
    overlap rows of a segment are recomputed from the same inputs by the same
    code: bit for bit) and for one or two tracers per pass (within 1e-6:
    the compiler may contract the two instantiations differently)."""
    outs = {}
    modes = ("32-2", "64-2", "128-2", "256-2", "512-2", "2048-2", "64-1", "512-1")
    for mode in modes:
        ty, nq = (int(x) for x in mode.split("-"))
        members = make_members()
        ens = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
        ens.set_prep64(prep64)
        ens.set_tile(56, ty)
        ens.set_strip_tracers(nq)
        assert ens.option("strip_tracers") == nq
        load(ens, members)
        ens.step(2, DELT1, 2)
        outs[mode] = [get_cur(ens, i, m) for i, m in enumerate(members)]
        ens.close()
    members = make_members()
    for i, m in enumerate(members):
        ip = sea_interior(m)
        for mode in modes[1:6]:
            assert np.array_equal(outs[mode][i], outs["32-2"][i]), (i, mode)
        assert np.array_equal(outs["512-1"][i], outs["64-1"][i]), i
        ref = outs["32-2"][i][..., ip]
        d = np.abs(outs["64-1"][i][..., ip] - ref).max() / np.abs(ref).max()
        assert d < 1e-6, (i, d)


def test_mixed_precision_forms_agree(cuda):
    """The FP64 thickness prep and the compensated-FP32 prep of the strip
    kernel give the same step within 1e-6 (relative to each tracer's max)."""
    res = []
    for prep64 in (True, False):
        members = make_members()
        ens = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
        ens.set_prep64(prep64)
        assert ens.option("prep64") == int(prep64)
        load(ens, members)
        ens.step(2, DELT1, 1)
        res.append([get_cur(ens, i, m) for i, m in enumerate(members)])
        ens.close()
    members = make_members()
    for i, m in enumerate(members):
        ip = sea_interior(m)
        for q in range(m["ntr"]):
            a, b = res[0][i][q][..., ip], res[1][i][q][..., ip]
            assert np.abs(a - b).max() / np.abs(a).max() < 1e-6, (i, q)


def test_put_get_slices(cuda):
    """Moving one tracer (or a run of layers) at a time equals moving the
    whole field; ranges outside the field are rejected."""
    members = make_members(SPECS[:2])
    whole = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
    part = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
    load(whole, members)
    for i, m in enumerate(members):
        mm, nn = levels(1)
        kdm, ntr = m["kdm"], m["ntr"]
        for q in range(ntr):
            part.put(i, "old", np.ascontiguousarray(m["trc"][q, nn - 1]), s0=q * kdm, ns=kdm)
            part.put(i, "cur", np.ascontiguousarray(m["trc"][q, mm - 1]), s0=q * kdm, ns=kdm)
        for what in ("uflx", "vflx"):
            f = np.ascontiguousarray(m["c"][what])
            part.put(i, what, np.ascontiguousarray(f[:1]), s0=0, ns=1)
            if kdm > 1:
                part.put(i, what, np.ascontiguousarray(f[1:]), s0=1, ns=kdm - 1)
        part.put(i, "dp", np.ascontiguousarray(m["c"]["dp"][nn - 1]))
        with pytest.raises(hycadv.HycError):
            part.put(i, "old", np.zeros((kdm, m["b"].ld2, m["b"].ld1)), s0=ntr * kdm - 1, ns=kdm)
        with pytest.raises(hycadv.HycError):
            part.get(i, "cur", np.zeros((kdm, m["b"].ld2, m["b"].ld1)), s0=-1, ns=kdm)
    whole.step(2, DELT1, 2)
    part.step(2, DELT1, 2)
    for i, m in enumerate(members):
        a = get_cur(whole, i, m)
        kdm = m["kdm"]
        for q in range(m["ntr"]):
            one = np.zeros((kdm, m["b"].ld2, m["b"].ld1))
            part.get(i, "cur", one, s0=q * kdm, ns=kdm)
            assert np.array_equal(one, a[q])
    whole.close()
    part.close()


def test_put_follows_torch_stream(cuda):
    """A device tensor torch is still writing when put is called arrives
    whole: the wrapper queues the library's copy behind torch's stream."""
    import torch

    b = basin(1000, 800, False, 409)
    g = oracle_grid(b)
    m = dict(b=b, g=g, kdm=8, ntr=2)
    ens = hycadv.Ensemble([spec_of(m)], precision="fp64")
    dev = torch.device("cuda", 0)
    shape = (2 * m["kdm"], b.ld2, b.ld1)
    for trial in range(3):
        x = torch.linspace(0.0, 1.0, int(np.prod(shape)), dtype=torch.float64, device=dev).reshape(shape)
        for _ in range(20):  # keep torch's stream busy while the put is issued
            x = torch.sin(x * 1.0001 + trial)
        ens.put(0, "cur", x)
        out = torch.empty_like(x)
        ens.get(0, "cur", out)
        assert torch.equal(out[:, b.J, b.I], x[:, b.J, b.I])
    ens.close()

def make_ts_members(specs=SPECS[:2], delt1=DELT1):
    """Members whose tracers are temp (posdef 256 under MPDATA) and saln."""
    out = []
    for nx, ny, per, kdm, ntr, seed, cour, _ in specs:
        b = basin(nx, ny, per, seed)
        g = oracle_grid(b)
        c = np_case(b, g, kdm=kdm, ntracr=0, seed=seed, courant=cour, delt1=delt1)
        trc = np.stack([c["temp"], c["saln"]])  # (2, 2, kdm, ...)
        out.append(dict(b=b, g=g, c=c, ntr=2, kdm=kdm, trc=trc))
    return out


def oracle_ts_step(m, step, advtyp):
    c = m["c"]
    mm, nn = levels(step)
    # hybrid layers (nhybrd = kdm, advflg = 0): temp and saln are advected (mod_tsadvc.F90:1855, :1969-1981)
    m["g"].tsadvc(mm, nn, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], uflx=c["uflx"], vflx=c["vflx"],
                  dp=c["dp"], delt1=DELT1, advtyp=advtyp, nstep=step)
    return np.stack([c["temp"][nn - 1], c["saln"][nn - 1]])


@pytest.mark.parametrize("advtyp", [0, 1])
def test_fp64_ensemble_pcm_mpdata_bitwise(cuda, advtyp):
    """FP64 ensemble PCM and MPDATA (temp with posdef 256) equal the oracle's
    tsadvc bit for bit over three steps, closed and periodic basins."""
    members = make_ts_members()
    ens = hycadv.Ensemble([spec_of(m) for m in members], precision="fp64")
    for i in range(len(members)):
        ens.set_posdef(i, 0, 256.0)
    load(ens, members)
    for step in range(1, 4):
        ens.step(advtyp, DELT1, 1)
        for i, m in enumerate(members):
            want = oracle_ts_step(m, step, advtyp)
            got = get_cur(ens, i, m)
            ip = sea_interior(m)
            assert same(got[..., ip], want[..., ip]), f"basin {i} step {step}"
            mm, nn = levels(step + 1)
            ens.put(i, "dp", np.ascontiguousarray(m["c"]["dp"][nn - 1]))
    ens.close()


@pytest.mark.parametrize("prep64,nq", [(True, 2), (False, 2), (True, 1), (False, 1)])
def test_mixed_mpdata_one_step_error(cuda, prep64, nq):
    """One FP32-mixed MPDATA step (strip kernel, posdef handled outside the
    FP32 values; nq tracers per pass) is within 1e-6 of the FP64 oracle
    relative to each tracer's max |value|, for temp (posdef 256) and saln
    (posdef 0)."""
    members = make_ts_members()
    ens = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
    ens.set_prep64(prep64)
    ens.set_strip_tracers(nq)
    for i in range(len(members)):
        ens.set_posdef(i, 0, 256.0)
    load(ens, members)
    ens.step(1, DELT1, 1)
    for i, m in enumerate(members):
        want = oracle_ts_step(m, 1, 1)
        got = get_cur(ens, i, m)
        ip = sea_interior(m)
        for q in range(2):
            err = np.abs(got[q][..., ip] - want[q][..., ip]).max() / np.abs(want[q][..., ip]).max()
            print(f"mpdata prep64={prep64} basin {i} tracer {q}: {err:.2e}")
            assert err < 1e-6, (i, q, err)
    ens.close()


@pytest.mark.parametrize("advtyp", [1, 2, 4])
def test_mixed_form_runs_the_strip_kernel(cuda, advtyp):
    """The mixed form has one kernel, the strip kernel: cell tiles are
    refused, PCM is not offered, and the tuner picks a strip shape."""
    members = make_ts_members(SPECS[:1])
    ens = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
    load(ens, members)
    with pytest.raises(hycadv.HycError):
        ens.set_tile(32, 16)
    with pytest.raises(hycadv.HycError):
        ens.step(0, DELT1, 1)
    tx, ty, _ = ens.tune(advtyp, DELT1)
    assert tx == 56
    ens.step(advtyp, DELT1, 1)
    ens.close()


@pytest.mark.parametrize("prep64,nq", [(True, 2), (False, 2), (False, 1)])
def test_mixed_fct4_one_step_error(cuda, prep64, nq):
    """One FP32-mixed FCT4 step (two-column strip kernel: 4th-order
    antidiffusive fluxes, 2nd order next to closed faces,
    mod_tsadvc.F90:1534-1555) is within 1e-6 of the FP64 oracle relative to
    each tracer's max |value|, closed and periodic basins, 1 to 3 tracers."""
    members = make_members()
    ens = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
    ens.set_prep64(prep64)
    ens.set_tile(56, 64)
    ens.set_strip_tracers(nq)
    load(ens, members)
    ens.step(4, DELT1, 1)
    for i, m in enumerate(members):
        want = oracle_step(m, 1, 4)
        got = get_cur(ens, i, m)
        ip = sea_interior(m)
        for q in range(m["ntr"]):
            err = np.abs(got[q][..., ip] - want[q][..., ip]).max() / np.abs(want[q][..., ip]).max()
            print(f"fct4 prep64={prep64} nq={nq} basin {i} tracer {q}: {err:.2e}")
            assert err < 1e-6, (i, q, err)
    # FCT4 differs from FCT2 on these inputs (the 4th-order stencil is live)
    members = make_members()
    ens2 = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
    ens2.set_prep64(prep64)
    ens2.set_tile(56, 64)
    ens2.set_strip_tracers(nq)
    load(ens2, members)
    ens2.step(2, DELT1, 1)
    assert any(not np.array_equal(get_cur(ens, i, m), get_cur(ens2, i, m)) for i, m in enumerate(members))
    ens.close()
    ens2.close()


def test_get_async_overlaps_and_equals_get(cuda):
    """hyc_ens_get_async: after wait() the host buffers hold what a synchronous
    get returns, for outputs of consecutive steps whose copies overlap the
    next step's puts; pinned host memory and device destinations."""
    import torch

    members = make_members(SPECS[:2])
    ens = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
    load(ens, members)
    outs, want = [], []
    for s in range(3):
        ens.step(2, DELT1, 1)
        for i, m in enumerate(members):
            shape = (m["ntr"] * m["kdm"], m["b"].ld2, m["b"].ld1)
            pinned = torch.zeros(shape, dtype=torch.float64).pin_memory()
            dev = torch.zeros(shape, dtype=torch.float64, device=cuda)
            ens.get_async(i, "cur", pinned)
            ens.get_async(i, "cur", dev)
            ref = np.zeros(shape)
            ens.get(i, "cur", ref)
            outs.append((pinned, dev))
            want.append(ref)
        for i, m in enumerate(members):  # re-put the inputs while the copies run
            c = m["c"]
            ens.put(i, "uflx", np.ascontiguousarray(c["uflx"]))
    ens.wait()
    torch.cuda.synchronize()
    for (pinned, dev), ref in zip(outs, want):
        assert np.array_equal(pinned.numpy(), ref)
        assert np.array_equal(dev.cpu().numpy(), ref)
    ens.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_all_land_basin_beside_a_sea_basin(cuda, prec):
    """A basin with no sea point (masks all zero) in the same ensemble as an
    ordinary one: its levels pass through unchanged, and the other basin's
    step equals the step it takes alone, bit for bit."""
    members = make_members(SPECS[:1])
    land = members[0]
    b = land["b"]
    spec_land = dict(spec_of(land), ip=np.zeros_like(land["g"].masks["ip"]), iu=np.zeros_like(land["g"].masks["iu"]),
                     iv=np.zeros_like(land["g"].masks["iv"]))
    both = hycadv.Ensemble([spec_land, spec_of(members[0])], precision=prec)
    alone = hycadv.Ensemble([spec_of(members[0])], precision=prec)
    for ens, idx in ((both, [0, 1]), (alone, [0])):
        for i in idx:
            mm, nn = levels(1)
            m = members[0]
            ens.put(i, "old", np.ascontiguousarray(m["trc"][:, nn - 1]))
            ens.put(i, "cur", np.ascontiguousarray(m["trc"][:, mm - 1]))
            ens.put(i, "uflx", np.ascontiguousarray(m["c"]["uflx"]))
            ens.put(i, "vflx", np.ascontiguousarray(m["c"]["vflx"]))
            ens.put(i, "dp", np.ascontiguousarray(m["c"]["dp"][nn - 1]))
        ens.step(2, DELT1, 1)
    m = members[0]
    shape = (m["ntr"] * m["kdm"], b.ld2, b.ld1)
    got_land, got_sea, want = np.zeros(shape), np.zeros(shape), np.zeros(shape)
    both.get(0, "cur", got_land)
    both.get(1, "cur", got_sea)
    alone.get(0, "cur", want)
    mm, _ = levels(1)
    cur = m["trc"][:, mm - 1].reshape(shape)
    if prec == "mixed":  # stored in FP32
        cur = cur.astype(np.float32).astype(np.float64)
    inner = np.zeros((b.ld2, b.ld1), bool)
    inner[b.J, b.I] = True
    assert np.array_equal(got_land[:, inner], cur[:, inner])
    assert np.array_equal(got_sea, want)
    both.close()
    alone.close()
