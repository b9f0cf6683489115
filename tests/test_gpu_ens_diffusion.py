"""Lateral diffusion fused into the FP32-mixed step kernel
(hyc_ens_set_diffusion): one step of advection plus the diffusion block of
tsadvc (mod_tsadvc.F90:2138-2230, tsdff_2x/tsdff_1x :2262-2492) within 1e-6
of the oracle's tsadvc followed by its tsdff, relative to each tracer's max
|value|, for FCT2, FCT4 and MPDATA, one and two tracers per pass, closed and
periodic basins split into several strips and row segments."""
import numpy as np
import pytest

import hycadv
from helpers import basin, diff_grid, levels, np_case, oracle_grid, same
from test_gpu_ensemble import DELT1, get_cur, load, sea_interior, spec_of

pytestmark = pytest.mark.gpu

TEMDF2 = 0.3
# nx, ny, periodic, kdm, passive tracers, seed, courant: wider than one strip
# and, with 32-row segments, taller than one segment
DSPECS = [(150, 100, False, 3, 1, 611, 0.7), (121, 70, True, 2, 0, 612, 0.8)]


def make(specs=DSPECS):
    out = []
    for nx, ny, per, kdm, npas, seed, cour in specs:
        b = basin(nx, ny, per, seed)
        g = oracle_grid(b)
        c = np_case(b, g, kdm=kdm, ntracr=npas, seed=seed, courant=cour, delt1=DELT1)
        trc = np.concatenate([np.stack([c["temp"], c["saln"]])] + ([c["tracer"]] if npas else []), axis=0)
        out.append(dict(b=b, g=g, c=c, ntr=2 + npas, npas=npas, kdm=kdm, trc=trc, d=diff_grid(b, seed)))
    return out


def oracle_step(m, advtyp, diffuse=True):
    """tsadvc (hybrid layers: temp, saln and the tracers advected) and its
    diffusion block on copies of the member's levels; the new level of
    every tracer."""
    c = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in m["c"].items()}
    mm, nn = levels(1)
    npas = m["npas"]
    tracer = c["tracer"] if npas else None
    tf = np.zeros(max(npas, 1), np.int32)
    m["g"].tsadvc(mm, nn, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], uflx=c["uflx"], vflx=c["vflx"],
                  dp=c["dp"], delt1=DELT1, advtyp=advtyp, tracer=tracer, trcflg=tf, nstep=1)
    if diffuse:
        oneta = np.ones((2, m["b"].ld2, m["b"].ld1))
        m["g"].tsdff(mm, nn, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], dp=c["dp"], oneta=oneta,
                     delt1=DELT1, temdf2=TEMDF2, tracer=tracer, **m["d"])
    new = [c["temp"][nn - 1], c["saln"][nn - 1]] + [tracer[q, nn - 1] for q in range(npas)]
    return np.stack(new)


def ensemble(members, advtyp, nq=2, diffuse=(True, True), tile=(56, 32)):
    ens = hycadv.Ensemble([spec_of(m) for m in members], precision="mixed")
    ens.set_strip_tracers(nq)
    for i, m in enumerate(members):
        if advtyp == 1:
            ens.set_posdef(i, 0, 256.0)  # temp (mod_tsadvc.F90:1761-1763)
        if diffuse[i]:
            ens.set_diffusion(i, TEMDF2, **m["d"])
    load(ens, members)
    ens.set_tile(*tile)
    return ens


@pytest.mark.parametrize("advtyp,nq", [(2, 2), (2, 1), (4, 2), (1, 2), (1, 1)])
def test_fused_diffusion_within_1e6_of_oracle(cuda, advtyp, nq):
    members = make()
    ens = ensemble(members, advtyp, nq)
    ens.step(advtyp, DELT1, 1)
    for i, m in enumerate(members):
        want = oracle_step(m, advtyp)
        plain = oracle_step(m, advtyp, diffuse=False)
        got = get_cur(ens, i, m)
        ip = sea_interior(m)
        for q in range(m["ntr"]):
            scale = np.abs(want[q][..., ip]).max()
            err = np.abs(got[q][..., ip] - want[q][..., ip]).max() / scale
            effect = np.abs(plain[q][..., ip] - want[q][..., ip]).max() / scale
            print(f"advtyp {advtyp} nq {nq} basin {i} tracer {q}: err {err:.2e}, diffusion {effect:.2e}")
            assert err < 1e-6, (i, q, err)
            assert effect > 100 * err, (i, q, effect)  # the diffusion is far above the error
    ens.close()


def test_basin_without_diffusion_is_unchanged(cuda):
    """In an ensemble where one basin diffuses, the other basin's step equals
    the step of an ensemble without diffusion bit for bit, and turning the
    diffusion off gives the plain step back."""
    members = make()
    a = ensemble(members, 2, diffuse=(True, False))
    b = ensemble(members, 2, diffuse=(False, False))
    a.step(2, DELT1, 1)
    b.step(2, DELT1, 1)
    ip = sea_interior(members[1])
    ga, gb = get_cur(a, 1, members[1]), get_cur(b, 1, members[1])
    assert same(ga[..., ip], gb[..., ip])
    c = ensemble(members, 2, diffuse=(True, True))
    c.set_diffusion(0, 0.0)
    c.set_diffusion(1, 0.0)
    c.step(2, DELT1, 1)
    for i, m in enumerate(members):
        ip = sea_interior(m)
        assert same(get_cur(c, i, m)[..., ip], get_cur(b, i, m)[..., ip]), i
    for e in (a, b, c):
        e.close()


def test_fused_diffusion_graph_replay_equals_eager(cuda):
    members = make()
    a = ensemble(members, 2)
    b = ensemble(members, 2)
    a.step(2, DELT1, 3)
    b.step(2, DELT1, 3, graph=True)
    for i, m in enumerate(members):
        assert same(get_cur(a, i, m), get_cur(b, i, m)), i
    a.close()
    b.close()


def test_diffusion_errors(cuda):
    members = make(DSPECS[:1])
    m = members[0]
    f64 = hycadv.Ensemble([spec_of(m)], precision="fp64")
    with pytest.raises(hycadv.HycError) as e:
        f64.set_diffusion(0, TEMDF2, **m["d"])
    assert e.value.code == -8  # HYC_ERR_UNSUPPORTED: the FP64 form diffuses with hyc_tsdff
    f64.close()
    ens = ensemble(members, 2)
    with pytest.raises(hycadv.HycError) as e:
        ens.set_diffusion(0, -1.0, **m["d"])
    assert e.value.code == -1
    ens.set_prep64(False)
    with pytest.raises(hycadv.HycError) as e:
        ens.step(2, DELT1, 1)
    assert e.value.code == -8  # the epilogue exists with the FP64 thickness prep only
    ens.close()
