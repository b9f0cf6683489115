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
