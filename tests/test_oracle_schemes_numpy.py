"""A second, independent restatement of advem_fct2 (mod_tsadvc.F90:645-997),
advem_fct4 (:1370-1706), advem_mpdata (:207-493) and advem_pcm (:495-643)
in vectorised numpy -- whole-array stages over the reference's margins
instead of the oracle's cell loops -- checked against the C oracle bit for
bit on small basins with coasts, islands and a periodic channel.  These are
the known-answer tests of the four schemes: two restatements written apart
must agree on every value, the Zalesak limiter's coastal ipip1/ipjp1
quirk, the section-edge zeroing, FCT4's fall back to 2nd order next to
closed faces and MPDATA's posdef offset included."""
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


class Slice:
    """Whole-slice stencil operations in the reference layout (python index
    (j+nb-1, i+nb-1) for Fortran (i, j))."""

    def __init__(self, g, shape):
        self.g, self.shape = g, shape
        self.nb, self.ii, self.jj = g.nbdy, g.idm, g.jdm
        self.ip, self.iu, self.iv = (g.masks[k] != 0 for k in ("ip", "iu", "iv"))
        nb = self.nb
        self.jg, self.ig = np.meshgrid(np.arange(shape[0]) - nb + 1, np.arange(shape[1]) - nb + 1, indexing="ij")
        self.J, self.I = np.indices(shape)

    def region(self, m):
        """Fortran 1-m..ii+m x 1-m..jj+m."""
        return (self.ig >= 1 - m) & (self.ig <= self.ii + m) & (self.jg >= 1 - m) & (self.jg <= self.jj + m)

    @staticmethod
    def sh(a, di, dj):
        """a(i+di, j+dj), NaN off the array."""
        out = np.full_like(a, np.nan)
        ys, yd = (slice(dj, None), slice(None, -dj)) if dj > 0 else (slice(None, dj or None), slice(-dj, None))
        xs, xd = (slice(di, None), slice(None, -di)) if di > 0 else (slice(None, di or None), slice(-di, None))
        out[yd, xd] = a[ys, xs]
        return out

    def at_i(self, a, k):
        """a(ipim1/ipip1(i,j), j): the sea-only neighbour (bigrid.F90:316-333)."""
        return a[self.J, np.clip(self.g.masks[k] + self.nb - 1, 0, self.shape[1] - 1)]

    def at_j(self, a, k):
        return a[np.clip(self.g.masks[k] + self.nb - 1, 0, self.shape[0] - 1), self.I]

    def five(self, a, op):
        return op(op(op(op(a, self.at_i(a, "ipim1")), self.at_i(a, "ipip1")), self.at_j(a, "ipjm1")),
                  self.at_j(a, "ipjp1"))

    def zero_edges(self, fx, fy, m):
        """Face values at the first and past the last point of every sea
        section set to 0 (mod_tsadvc.F90:738-758)."""
        nb, ii, jj = self.nb, self.ii, self.jj
        for j in range(1 - m, jj + m + 1):
            for f, l in sections(self.ip[j + nb - 1], nb, ii):
                if f >= 1 - m:
                    fx[j + nb - 1, f + nb - 1] = 0.0
                if l < ii + m:
                    fx[j + nb - 1, l + nb] = 0.0
        for i in range(1 - m, ii + m + 1):
            for f, l in sections(self.ip[:, i + nb - 1], nb, jj):
                if f >= 1 - m:
                    fy[f + nb - 1, i + nb - 1] = 0.0
                if l < jj + m:
                    fy[l + nb, i + nb - 1] = 0.0

    def nan(self):
        return np.full(self.shape, np.nan)


pos = lambda a: np.maximum(0.0, a)  # noqa: E731
neg = lambda a: np.minimum(0.0, a)  # noqa: E731


def fct2_numpy(g, fld, fldc, u, v, fco, fcn, scal, scali, dt2, order=2):
    S = Slice(g, fld.shape)
    sh, ip, iu, iv = S.sh, S.ip, S.iu, S.iv
    flx, fly, fmx, fmn = S.nan(), S.nan(), S.nan(), S.nan()
    r = S.region(4)
    m = r & iu
    flx[m] = (u * np.where(u >= 0.0, sh(fld, -1, 0), fld))[m]
    m = r & iv
    fly[m] = (v * np.where(v >= 0.0, sh(fld, 0, -1), fld))[m]
    m = r & ip
    fmx[m] = S.five(fld, np.maximum)[m]
    fmn[m] = S.five(fld, np.minimum)[m]
    S.zero_edges(flx, fly, 4)
    fldlo, fmxlo, fmnlo = S.nan(), S.nan(), S.nan()
    m = S.region(3) & ip
    flxdiv = ((sh(flx, 1, 0) - flx) + (sh(fly, 0, 1) - fly)) * dt2 * scali
    q = fld * (fco + ONEMU) - flxdiv
    lo = np.maximum(fmn, np.minimum(fmx, q / (fcn + ONEMU)))
    fldlo[m] = lo[m]
    fmxlo[m] = np.maximum(np.maximum(fld, fldc), lo)[m]
    fmnlo[m] = np.minimum(np.minimum(fld, fldc), lo)[m]
    fax, fay = S.nan(), S.nan()
    fhx = u * 0.5 * (fldc + sh(fldc, -1, 0))
    fhy = v * 0.5 * (fldc + sh(fldc, 0, -1))
    if order == 4:  # :1534-1555, 4th order where both neighbouring faces are open
        ft14, ft24 = 7.0 / 12.0, -1.0 / 12.0
        hx4 = u * (ft14 * (fldc + sh(fldc, -1, 0)) + ft24 * (sh(fldc, 1, 0) + sh(fldc, -2, 0)))
        hy4 = v * (ft14 * (fldc + sh(fldc, 0, -1)) + ft24 * (sh(fldc, 0, 1) + sh(fldc, 0, -2)))
        iuf, ivf = iu.astype(float), iv.astype(float)
        x4 = (sh(iuf, -1, 0) == 1) & (sh(iuf, 1, 0) == 1)
        y4 = (sh(ivf, 0, -1) == 1) & (sh(ivf, 0, 1) == 1)
        with np.errstate(invalid="ignore"):
            fhx = np.where(x4, hx4, fhx)
            fhy = np.where(y4, hy4, fhy)
    m = S.region(3) & iu
    fax[m] = (fhx - flx)[m]
    m = S.region(3) & iv
    fay[m] = (fhy - fly)[m]
    S.zero_edges(fax, fay, 3)
    rp, rm = S.nan(), S.nan()
    m = S.region(2) & ip
    fqmax, fqmin = S.five(fmxlo, np.maximum), S.five(fmnlo, np.minimum)
    faxb, fayb = S.at_i(fax, "ipip1"), S.at_j(fay, "ipjp1")  # the coastal quirk: ib = i where i+1 is land
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
    m = S.region(1) & iu
    fact = np.where(fax < 0.0, np.minimum(sh(rp, -1, 0), rm), np.minimum(rp, sh(rm, -1, 0)))
    fax[m] = (fact * fax)[m]
    m = S.region(1) & iv
    fact = np.where(fay < 0.0, np.minimum(sh(rp, 0, -1), rm), np.minimum(rp, sh(rm, 0, -1)))
    fay[m] = (fact * fay)[m]
    out = fld.copy()
    m = S.region(0) & ip
    flxdiv = ((sh(fax, 1, 0) - fax) + (sh(fay, 0, 1) - fay)) * dt2 * scali
    out[m] = np.maximum(fmn, np.minimum(fmx, fldlo - flxdiv / (fcn + ONEMU)))[m]
    return out


def mpdata_numpy(g, fld, u, v, fco, fcn, posdef, scal, scali, dt2):
    """advem_mpdata (mod_tsadvc.F90:207-493): donor cell on fld+posdef, the
    antidiffusive velocity's fluxes, limited by min(1, rp, rm)."""
    S = Slice(g, fld.shape)
    sh, ip, iu, iv = S.sh, S.ip, S.iu, S.iv
    tx1, ty1, flx, fly, fmx, fmn = (S.nan() for _ in range(6))
    r = S.region(4)  # :249-281
    m = r & iu
    fw = sh(fld, -1, 0)
    tx1[m] = (0.5 * np.abs(u) * (fld - fw))[m]
    flx[m] = (u * (np.where(u >= 0.0, fw, fld) + posdef))[m]
    m = r & iv
    fs = sh(fld, 0, -1)
    ty1[m] = (0.5 * np.abs(v) * (fld - fs))[m]
    fly[m] = (v * (np.where(v >= 0.0, fs, fld) + posdef))[m]
    m = r & ip
    fmx[m] = (S.five(fld, np.maximum) + posdef)[m]
    fmn[m] = (S.five(fld, np.minimum) + posdef)[m]
    S.zero_edges(flx, fly, 4)  # :301-325 (tx1, ty1 are not zeroed)
    fldlo, flxdiv = S.nan(), S.nan()
    m = S.region(3) & ip  # :345-353
    fd = ((sh(flx, 1, 0) - flx) + (sh(fly, 0, 1) - fly)) * dt2 * scali
    q = (fld + posdef) * (fco + ONEMU) - fd
    flxdiv[m] = fd[m]
    fldlo[m] = np.maximum(fmn, np.minimum(fmx, q / (fcn + ONEMU)))[m]
    m = S.region(3) & iu  # :369-392
    ax = tx1 - u * (flxdiv + sh(flxdiv, -1, 0)) / (((fco + sh(fco, -1, 0)) + (fcn + sh(fcn, -1, 0))) + ONEMU)
    flx[m] = ax[m]
    m = S.region(3) & iv
    ay = ty1 - v * (flxdiv + sh(flxdiv, 0, -1)) / (((fco + sh(fco, 0, -1)) + (fcn + sh(fcn, 0, -1))) + ONEMU)
    fly[m] = ay[m]
    rp, rm = S.nan(), S.nan()
    m = S.region(2) & ip  # :405-423
    fe, fn = sh(flx, 1, 0), sh(fly, 0, 1)
    flxdp, flxdn = neg(fe) - pos(flx), pos(fe) - neg(flx)
    flydp, flydn = neg(fn) - pos(fly), pos(fn) - neg(fly)
    rp[m] = ((fmx - fldlo) * (fcn * scal) / ((ONEMU - (flxdp + flydp)) * dt2))[m]
    rm[m] = ((fldlo - fmn) * (fcn * scal) / ((ONEMU + (flxdn + flydn)) * dt2))[m]
    lim = lambda a, b: np.minimum(np.minimum(1.0, a), b)  # noqa: E731  min(1.0, a, b)
    m = S.region(1) & iu  # :433-449
    lx = pos(flx) * lim(rp, sh(rm, -1, 0)) + neg(flx) * lim(sh(rp, -1, 0), rm)
    m2 = S.region(1) & iv
    ly = pos(fly) * lim(rp, sh(rm, 0, -1)) + neg(fly) * lim(sh(rp, 0, -1), rm)
    flx[m], fly[m2] = lx[m], ly[m2]
    out = fld.copy()
    m = S.region(0) & ip  # :465-486
    fd = ((sh(flx, 1, 0) - flx) + (sh(fly, 0, 1) - fly)) * dt2 * scali
    out[m] = (np.maximum(fmn, np.minimum(fmx, fldlo - fd / (fcn + ONEMU))) - posdef)[m]
    return out


def pcm_numpy(g, fld, u, v, fco, fcn, scal, scali, dt2):
    """advem_pcm (mod_tsadvc.F90:495-643): donor cell, clipped to the sea-only
    5-point extrema; margins 1 and 0 (mbdy = 2)."""
    S = Slice(g, fld.shape)
    sh, ip, iu, iv = S.sh, S.ip, S.iu, S.iv
    flx, fly, fmx, fmn = S.nan(), S.nan(), S.nan(), S.nan()
    r = S.region(1)
    m = r & iu
    flx[m] = (u * np.where(u >= 0.0, sh(fld, -1, 0), fld))[m]
    m = r & iv
    fly[m] = (v * np.where(v >= 0.0, sh(fld, 0, -1), fld))[m]
    m = r & ip
    fmx[m] = S.five(fld, np.maximum)[m]
    fmn[m] = S.five(fld, np.minimum)[m]
    S.zero_edges(flx, fly, 1)
    out = fld.copy()
    m = S.region(0) & ip
    fd = ((sh(flx, 1, 0) - flx) + (sh(fly, 0, 1) - fly)) * dt2 * scali
    q = fld * (fco + ONEMU) - fd
    out[m] = np.maximum(fmn, np.minimum(fmx, q / (fcn + ONEMU)))[m]
    return out


def slice_case(nx, ny, periodic, seed):
    b = basin(nx, ny, periodic, seed)
    g = oracle_grid(b, threads=1)
    c = np_case(b, g, kdm=1, ntracr=0, seed=seed, courant=0.7, delt1=1800.0)
    rng = np.random.default_rng(seed)
    fld = np.ascontiguousarray(c["saln"][1, 0])
    fldc = np.ascontiguousarray(c["saln"][0, 0] + 0.01 * rng.standard_normal(fld.shape))
    u, v = np.ascontiguousarray(c["uflx"][0]), np.ascontiguousarray(c["vflx"][0])
    fcn = np.ascontiguousarray(c["dp"][1, 0])
    fco = np.ascontiguousarray(fcn * (1.0 + 0.05 * rng.standard_normal(fld.shape)))
    for a in (fld, fldc, u, v):
        g.xctilr(a, 5, 5)
    inner = np.zeros(fld.shape, bool)
    inner[b.J, b.I] = True
    sea = inner & (g.masks["ip"] != 0)
    return b, g, c, fld, fldc, u, v, fco, fcn, sea


CASES = [(23, 17, False, 41), (30, 20, True, 42), (19, 24, False, 43)]


@pytest.mark.parametrize("order", [2, 4])
@pytest.mark.parametrize("nx,ny,periodic,seed", CASES)
def test_fct_numpy_equals_oracle(nx, ny, periodic, seed, order):
    b, g, c, fld, fldc, u, v, fco, fcn, sea = slice_case(nx, ny, periodic, seed)
    want = fct2_numpy(g, fld, fldc, u, v, fco, fcn, c["scp2"], c["scp2i"], 1800.0, order)
    got = fld.copy()
    g.advem(order, got, fldc, u, v, fco, fcn, 0.0, c["scp2"], c["scp2i"], 1800.0)
    assert np.array_equal(got[sea], want[sea])
    assert not np.array_equal(got[sea], fld[sea])  # the step moved something
    if order == 4:  # the 4th-order stencil was live
        assert not np.array_equal(got[sea], fct2_numpy(g, fld, fldc, u, v, fco, fcn, c["scp2"], c["scp2i"], 1800.0)[sea])


@pytest.mark.parametrize("posdef", [0.0, 256.0])
@pytest.mark.parametrize("nx,ny,periodic,seed", CASES)
def test_mpdata_numpy_equals_oracle(nx, ny, periodic, seed, posdef):
    b, g, c, fld, fldc, u, v, fco, fcn, sea = slice_case(nx, ny, periodic, seed)
    want = mpdata_numpy(g, fld, u, v, fco, fcn, posdef, c["scp2"], c["scp2i"], 1800.0)
    got = fld.copy()
    g.advem(1, got, fldc, u, v, fco, fcn, posdef, c["scp2"], c["scp2i"], 1800.0)
    assert np.array_equal(got[sea], want[sea])
    assert not np.array_equal(got[sea], fld[sea])


@pytest.mark.parametrize("nx,ny,periodic,seed", CASES)
def test_pcm_numpy_equals_oracle(nx, ny, periodic, seed):
    b, g, c, fld, fldc, u, v, fco, fcn, sea = slice_case(nx, ny, periodic, seed)
    want = pcm_numpy(g, fld, u, v, fco, fcn, c["scp2"], c["scp2i"], 1800.0)
    got = fld.copy()
    g.advem(0, got, fldc, u, v, fco, fcn, 0.0, c["scp2"], c["scp2i"], 1800.0)
    assert np.array_equal(got[sea], want[sea])
    assert not np.array_equal(got[sea], fld[sea])
