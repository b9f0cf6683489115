"""A second, independent restatement of advem_fct2 (mod_tsadvc.F90:645-997)
in vectorised numpy — whole-array stages over the reference's margins
instead of the oracle's cell loops — checked against the C oracle bit for
bit on small basins with coasts, islands and a periodic channel.  This is
the known-answer test of the FCT2 scheme: two restatements written apart
must agree on every value, the Zalesak limiter's coastal ipip1/ipjp1 quirk
and the section-edge zeroing included."""
import numpy as np
import pytest

from helpers import basin, np_case, oracle_grid

ONEMU = 9806.e-12  # mod_tsadvc.F90:671


def sections(ip_row, nb, n):
    """Sea segments (first, last) of one row, Fortran indices 1-nb..n+nb."""
    out, start = [], None
    for k, v in enumerate(ip_row):
        i = k - nb + 1
        if v and start is None:
            start = i
        if not v and start is not None:
            out.append((start, i - 1))
            start = None
    if start is not None:
        out.append((start, n + nb))
    return out


def fct2_numpy(g, fld, fldc, u, v, fco, fcn, scal, scali, dt2):
    nb, ii, jj = g.nbdy, g.idm, g.jdm
    ip, iu, iv = (g.masks[k] != 0 for k in ("ip", "iu", "iv"))
    shp = fld.shape
    jg, ig = np.meshgrid(np.arange(shp[0]) - nb + 1, np.arange(shp[1]) - nb + 1, indexing="ij")  # Fortran j, i

    def region(m):
        return (ig >= 1 - m) & (ig <= ii + m) & (jg >= 1 - m) & (jg <= jj + m)

    def sh(a, di, dj):  # a(i+di, j+dj), NaN off the array
        out = np.full_like(a, np.nan)
        ys, yd = (slice(dj, None), slice(None, -dj)) if dj > 0 else (slice(None, dj or None), slice(-dj, None))
        xs, xd = (slice(di, None), slice(None, -di)) if di > 0 else (slice(None, di or None), slice(-di, None))
        out[yd, xd] = a[ys, xs]
        return out

    # sea-only neighbours (bigrid.F90:316-333) as gathers
    col = lambda k: np.clip(g.masks[k] + nb - 1, 0, shp[1] - 1)
    row = lambda k: np.clip(g.masks[k] + nb - 1, 0, shp[0] - 1)
    J, I = np.indices(shp)
    at_i = lambda a, k: a[J, col(k)]
    at_j = lambda a, k: a[row(k), I]

    def five(a, op):
        return op(op(op(op(a, at_i(a, "ipim1")), at_i(a, "ipip1")), at_j(a, "ipjm1")), at_j(a, "ipjp1"))

    def zero_edges(fx, fy, m):
        for j in range(1 - m, jj + m + 1):
            for f, l in sections(ip[j + nb - 1], nb, ii):
                if f >= 1 - m:
                    fx[j + nb - 1, f + nb - 1] = 0.0
                if l < ii + m:
                    fx[j + nb - 1, l + nb] = 0.0
        for i in range(1 - m, ii + m + 1):
            for f, l in sections(ip[:, i + nb - 1], nb, jj):
                if f >= 1 - m:
                    fy[f + nb - 1, i + nb - 1] = 0.0
                if l < jj + m:
                    fy[l + nb, i + nb - 1] = 0.0

    nan = lambda: np.full(shp, np.nan)
    flx, fly, fmx, fmn = nan(), nan(), nan(), nan()
    r = region(4)
    m = r & iu
    flx[m] = (u * np.where(u >= 0.0, sh(fld, -1, 0), fld))[m]
    m = r & iv
    fly[m] = (v * np.where(v >= 0.0, sh(fld, 0, -1), fld))[m]
    m = r & ip
    fmx[m] = five(fld, np.maximum)[m]
    fmn[m] = five(fld, np.minimum)[m]
    zero_edges(flx, fly, 4)
    fldlo, fmxlo, fmnlo = nan(), nan(), nan()
    m = region(3) & ip
    flxdiv = ((sh(flx, 1, 0) - flx) + (sh(fly, 0, 1) - fly)) * dt2 * scali
    q = fld * (fco + ONEMU) - flxdiv
    lo = np.maximum(fmn, np.minimum(fmx, q / (fcn + ONEMU)))
    fldlo[m] = lo[m]
    fmxlo[m] = np.maximum(np.maximum(fld, fldc), lo)[m]
    fmnlo[m] = np.minimum(np.minimum(fld, fldc), lo)[m]
    fax, fay = nan(), nan()
    m = region(3) & iu
    fax[m] = (u * 0.5 * (fldc + sh(fldc, -1, 0)) - flx)[m]
    m = region(3) & iv
    fay[m] = (v * 0.5 * (fldc + sh(fldc, 0, -1)) - fly)[m]
    zero_edges(fax, fay, 3)
    rp, rm = nan(), nan()
    m = region(2) & ip
    fqmax, fqmin = five(fmxlo, np.maximum), five(fmnlo, np.minimum)
    faxb, fayb = at_i(fax, "ipip1"), at_j(fay, "ipjp1")  # the coastal quirk: ib = i where i+1 is land
    pos, neg = (lambda a: np.maximum(0.0, a)), (lambda a: np.minimum(0.0, a))
    famax = ((pos(fax) - neg(faxb)) + pos(fay)) - neg(fayb)
    famin = ((pos(faxb) - neg(fax)) + pos(fayb)) - neg(fay)
    qdt2 = 1.0 / dt2
    qp = (fqmax - fldlo) * fcn * scal * qdt2
    qm = (fldlo - fqmin) * fcn * scal * qdt2
    with np.errstate(divide="ignore", invalid="ignore"):
        rpv = np.where(famax > 0.0, np.where(qp < famax, qp / famax, 1.0), 0.0)
        rmv = np.where(famin > 0.0, np.where(qm < famin, qm / famin, 1.0), 0.0)
    rp[m], rm[m] = rpv[m], rmv[m]
    fmx[m], fmn[m] = fqmax[m], fqmin[m]
    m = region(1) & iu
    fact = np.where(fax < 0.0, np.minimum(sh(rp, -1, 0), rm), np.minimum(rp, sh(rm, -1, 0)))
    fax[m] = (fact * fax)[m]
    m = region(1) & iv
    fact = np.where(fay < 0.0, np.minimum(sh(rp, 0, -1), rm), np.minimum(rp, sh(rm, 0, -1)))
    fay[m] = (fact * fay)[m]
    out = fld.copy()
    m = region(0) & ip
    flxdiv = ((sh(fax, 1, 0) - fax) + (sh(fay, 0, 1) - fay)) * dt2 * scali
    out[m] = np.maximum(fmn, np.minimum(fmx, fldlo - flxdiv / (fcn + ONEMU)))[m]
    return out


@pytest.mark.parametrize("nx,ny,periodic,seed", [(23, 17, False, 41), (30, 20, True, 42), (19, 24, False, 43)])
def test_fct2_numpy_equals_oracle(nx, ny, periodic, seed):
    b = basin(nx, ny, periodic, seed)
    g = oracle_grid(b, threads=1)
    c = np_case(b, g, kdm=1, ntracr=0, seed=seed, courant=0.7, delt1=1800.0)
    rng = np.random.default_rng(seed)
    fld = np.ascontiguousarray(c["saln"][1, 0])
    fldc = np.ascontiguousarray(c["saln"][0, 0] + 0.01 * rng.standard_normal(fld.shape))
    u, v = np.ascontiguousarray(c["uflx"][0]), np.ascontiguousarray(c["vflx"][0])
    fcn = np.ascontiguousarray(c["dp"][1, 0])
    fco = np.ascontiguousarray(fcn * (1.0 + 0.05 * rng.standard_normal(fld.shape)))
    g.xctilr(fld, 5, 5)
    g.xctilr(fldc, 5, 5)
    g.xctilr(u, 5, 5)
    g.xctilr(v, 5, 5)
    want = fct2_numpy(g, fld, fldc, u, v, fco, fcn, c["scp2"], c["scp2i"], 1800.0)
    got = fld.copy()
    g.advem(2, got, fldc, u, v, fco, fcn, 0.0, c["scp2"], c["scp2i"], 1800.0)
    inner = np.zeros(fld.shape, bool)
    inner[b.J, b.I] = True
    sea = inner & (g.masks["ip"] != 0)
    assert np.array_equal(got[sea], want[sea])
    assert not np.array_equal(got[sea], fld[sea])  # the step moved something
