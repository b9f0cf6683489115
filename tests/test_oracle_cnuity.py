"""CPU oracle of the continuity equation (cnuity.F90): invariants of the
flux-corrected transport of layer thickness, the barotropic restoration, the
bottom-pressure restoring, the interface-depth diffusion and the
Robert-Asselin filter of dp."""
import numpy as np
import pytest

from helpers import basin, cnuity_case, oracle_grid
from oracle import oracle as O


def sea(b, g):
    s = np.zeros((b.ld2, b.ld1), bool)
    s[b.J, b.I] = True
    return s & (g.masks["ip"] != 0)


def run(g, c, m=1, n=2, **kw):
    kw.setdefault("delt1", 1800.0)
    return g.cnuity(m, n, c, **kw)


@pytest.mark.parametrize("periodic", [False, True])
def test_column_restored_and_fluxes_nondivergent(periodic):
    """Not btrmas: after the barotropic correction the layer fluxes add up to
    the high-order flux sum_k (u_k+ubavg)*scuy*dpu_k (:583-590), and the
    bottom-pressure restoring makes p(kdm+1) = pbot."""
    b = basin(60, 45, periodic, 81)
    g = oracle_grid(b, threads=1)
    c = cnuity_case(b, g, kdm=3)
    m, n = 1, 2
    u0, ub0, dpu0 = c["u"].copy(), c["ubavg"].copy(), c["dpu"].copy()
    run(g, c, m, n)
    s = sea(b, g)
    assert np.allclose(c["p"][-1][s], c["pbot"][s], rtol=1e-13, atol=0)
    iu = g.masks["iu"] != 0
    face = np.zeros_like(iu)
    face[b.J, b.I] = True
    face &= iu
    high = ((u0[m - 1] + ub0[m - 1][None]) * c["scuy"][None] * dpu0[m - 1]).sum(axis=0)
    got = c["uflx"].sum(axis=0)
    assert np.allclose(got[face], high[face], rtol=1e-10, atol=1e-6 * np.abs(high).max())


def test_zero_velocity_keeps_thickness():
    b = basin(50, 40, False, 82)
    g = oracle_grid(b, threads=1)
    c = cnuity_case(b, g, kdm=3, umax=0.0)
    m, n = 1, 2
    c["dp"][n - 1] = c["dp"][m - 1]
    d0 = c["dp"].copy()
    run(g, c, m, n, ra2fac=0.125)
    s = sea(b, g)
    assert np.array_equal(c["dp"][n - 1][:, s], d0[n - 1][:, s])
    assert np.allclose(c["dp"][m - 1][:, s], d0[m - 1][:, s], rtol=1e-15)  # RA of three equal levels
    assert np.array_equal(c["dpo"][m - 1][:, s], d0[m - 1][:, s])
    assert np.all(c["uflx"][:, g.masks["iu"] != 0] == 0.0)


def test_btrmas_restores_column():
    """btrmas: no barotropic correction; the column is rescaled by
    1/onetacnt = pbot/p(kdm+1) (:1350-1385), so p(kdm+1) = pbot after."""
    b = basin(60, 45, False, 83)
    g = oracle_grid(b, threads=1)
    c = cnuity_case(b, g, kdm=3, btrmas=True)
    run(g, c, 1, 2, btrmas=True)
    s = sea(b, g)
    cnt = c["onetacnt"][s]
    assert np.all(cnt > 0.5) and np.all(cnt < 1.5)
    assert np.allclose(c["p"][-1][s], c["pbot"][s], rtol=1e-13, atol=0)


@pytest.mark.parametrize("kind", ["thkdf4", "thkdf2"])
@pytest.mark.parametrize("nstep", [1, 2])
def test_interface_diffusion_keeps_column(kind, nstep):
    """Interface-depth diffusion moves interfaces 2..kdm only: the column
    p(kdm+1) stays pbot, interfaces stay ordered (dp >= 0)."""
    b = basin(60, 45, True, 84)
    g = oracle_grid(b, threads=1)
    c = cnuity_case(b, g, kdm=4, thkdf=True)
    run(g, c, 1, 2, nstep=nstep, **{kind: True})
    s = sea(b, g)
    assert np.allclose(c["p"][-1][s], c["pbot"][s], rtol=1e-13, atol=0)
    assert np.all(c["dp"][1][:, s] >= 0.0)


def test_fatal_negative_thickness():
    """A Courant number far above one empties cells: fatal when nstep%3 == 0."""
    b = basin(40, 30, False, 85)
    g = oracle_grid(b, threads=1)
    c = cnuity_case(b, g, kdm=2, umax=400.0)
    with pytest.raises(O.OracleError) as e:
        run(g, c, 1, 2, nstep=3)
    assert e.value.code == O.ERR_NEGDP
    c = cnuity_case(b, g, kdm=2, umax=400.0)
    dpkmin = run(g, c, 1, 2, nstep=1)
    assert dpkmin[2:].min() < -10.0 * 9806.0
