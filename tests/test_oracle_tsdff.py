"""CPU oracle of the diffusion block of tsadvc (mod_tsadvc.F90:2138-2230:
tsdff_1x/tsdff_2x and the density update through the 17-term equation of
state): known answers and invariants."""
import numpy as np
import pytest

from helpers import basin, diff_grid, np_case, oneta_field, oracle_grid
from oracle import oracle as O


def setup(periodic, seed, kdm=3, ntracr=3):
    b = basin(64, 48, periodic, seed)
    g = oracle_grid(b, threads=1)
    c = np_case(b, g, kdm=kdm, ntracr=ntracr, seed=seed, courant=0.5, delt1=1800.0)
    c["oneta"] = oneta_field(b, seed)
    return b, g, c, diff_grid(b, seed)


def run(g, c, d, n=2, temdf2=0.5, thbase=34.0):
    g.tsdff(1, n, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], dp=c["dp"], oneta=c["oneta"], delt1=1800.0,
            temdf2=temdf2, thbase=thbase, tracer=c["tracer"], **d)


def content(b, g, c, fld, n=2):
    """sum over interior sea cells and layers of fld*dp*oneta*scp2 (level n)."""
    sea = np.zeros((b.ld2, b.ld1), bool)
    sea[b.J, b.I] = True
    sea &= g.masks["ip"] != 0
    h = c["dp"][n - 1] * c["oneta"][n - 1][None]
    return float(np.sum((fld[n - 1] * h * c["scp2"][None])[:, sea]))


def test_sig_is_a_density():
    s = [O.sig(t, 35.0) for t in (0.0, 10.0, 20.0, 30.0)]
    assert all(25.0 < x < 40.0 for x in s) and s == sorted(s, reverse=True)  # lighter when warmer
    assert O.sig(10.0, 36.0) > O.sig(10.0, 34.0)                            # heavier when saltier


@pytest.mark.parametrize("periodic", [False, True])
def test_diffusion_conserves_content(periodic):
    b, g, c, d = setup(periodic, 41)
    before = [content(b, g, c, c[k]) for k in ("temp", "saln")] + [content(b, g, c, c["tracer"][q]) for q in range(3)]
    t0 = c["temp"].copy()
    run(g, c, d)
    after = [content(b, g, c, c[k]) for k in ("temp", "saln")] + [content(b, g, c, c["tracer"][q]) for q in range(3)]
    for x, y in zip(before, after):
        assert abs(y - x) <= 1e-13 * abs(x)
    assert not np.array_equal(c["temp"], t0)  # something diffused


def test_constant_field_unchanged_and_density_consistent():
    b, g, c, d = setup(False, 42)
    c["saln"][1] = 35.0
    run(g, c, d, thbase=34.0)
    sea = np.zeros((b.ld2, b.ld1), bool)
    sea[b.J, b.I] = True
    sea &= g.masks["ip"] != 0
    assert np.all(c["saln"][1][:, sea] == 35.0)
    t, s, h = c["temp"][1][:, sea], c["saln"][1][:, sea], c["th3d"][1][:, sea]
    want = np.array([O.sig(x, y) - 34.0 for x, y in zip(t.ravel()[:200], s.ravel()[:200])])
    assert np.array_equal(h.ravel()[:200], want)


def test_variance_decays():
    b, g, c, d = setup(True, 43, ntracr=1)
    sea = np.zeros((b.ld2, b.ld1), bool)
    sea[b.J, b.I] = True
    sea &= g.masks["ip"] != 0
    v0 = np.var(c["tracer"][0, 1][:, sea])
    for _ in range(5):
        run(g, c, d, temdf2=0.2)
    assert np.var(c["tracer"][0, 1][:, sea]) < v0


def test_rejects_isopycnal_layers():
    b, g, c, d = setup(False, 44)
    with pytest.raises(O.OracleError):
        g.tsdff(1, 2, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], dp=c["dp"], oneta=c["oneta"], delt1=1800.0,
                temdf2=0.5, nhybrd=1, **d)


def tsdff_numpy(g, flds, h, temdf2, delt1, aspux, aspvy, scuy, scvx, scp2):
    """tsdff_2x/tsdff_1x (mod_tsadvc.F90:2262-2440) restated apart from the
    oracle, as whole-slice numpy: face factors temdf2*asp*sc*harmonc(h_w, h)
    (:2274-2287, harmonc :1770-1771) at margin 1, fluxes zero at closed faces,
    then fld += div(flux)*(-delt1/(scp2*max(h, eps_har))) at the sea points
    of the interior (:2313-2323).  h = dp*onetamas of the layer."""
    from test_oracle_schemes_numpy import Slice

    S = Slice(g, h.shape)
    sh = S.sh
    eps = 1.0e-20
    harmz = lambda a, b: 2.0 * a * b / np.maximum(a + b, 2.0 * eps)  # noqa: E731
    harmc = lambda a, b: harmz(np.maximum(a, 0.0), np.maximum(b, 0.0))  # noqa: E731
    with np.errstate(invalid="ignore"):
        fu = temdf2 * aspux * scuy * harmc(sh(h, -1, 0), h)
        fv = temdf2 * aspvy * scvx * harmc(sh(h, 0, -1), h)
    factor = -delt1 / (scp2 * np.maximum(h, eps))
    mu, mv, mp = S.region(1) & S.iu, S.region(1) & S.iv, S.region(0) & S.ip
    for fld in flds:
        uf, vf = np.zeros_like(fld), np.zeros_like(fld)
        uf[mu] = (fu * (sh(fld, -1, 0) - fld))[mu]
        vf[mv] = (fv * (sh(fld, 0, -1) - fld))[mv]
        util = ((sh(uf, 1, 0) - uf) + (sh(vf, 0, 1) - vf)) * factor
        fld[mp] = (fld + util)[mp]


@pytest.mark.parametrize("periodic,seed", [(False, 71), (True, 72)])
def test_diffusion_numpy_equals_oracle(periodic, seed):
    """Known answer: the numpy restatement of the diffusion block (T and S
    through tsdff_2x, three tracers as a pair and a single, th3d from the
    17-term sig of the new T and S) equals the oracle bit for bit."""
    b, g, c, d = setup(periodic, seed)
    n, kdm, thbase = 2, c["temp"].shape[1], 34.0
    want = {k: c[k].copy() for k in ("temp", "saln", "th3d", "tracer")}
    for k in ("temp", "saln", "th3d"):  # :2139-2152, mdf = 2
        g.xctilr(want[k][n - 1], 2, 2)
    for q in range(want["tracer"].shape[0]):
        g.xctilr(want["tracer"][q, n - 1], 2, 2)
    sea = np.zeros((b.ld2, b.ld1), bool)
    sea[b.J, b.I] = True
    sea &= g.masks["ip"] != 0
    for k in range(kdm):
        h = c["dp"][n - 1, k] * c["oneta"][n - 1]
        flds = [want["temp"][n - 1, k], want["saln"][n - 1, k]] + [want["tracer"][q, n - 1, k]
                                                                     for q in range(want["tracer"].shape[0])]
        tsdff_numpy(g, flds, h, 0.5, 1800.0, d["aspux"], d["aspvy"], d["scuy"], d["scvx"], c["scp2"])
        t, s = want["temp"][n - 1, k], want["saln"][n - 1, k]
        want["th3d"][n - 1, k][sea] = [O.sig(a, bb) - thbase for a, bb in zip(t[sea], s[sea])]
    before = c["temp"][n - 1].copy()
    run(g, c, d, n=n, thbase=thbase)
    for k in ("temp", "saln", "th3d", "tracer"):
        assert np.array_equal(c[k][..., sea], want[k][..., sea]), k
    assert not np.array_equal(c["temp"][n - 1][:, sea], before[:, sea])  # the diffusion changed level n
