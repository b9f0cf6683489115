"""CPU oracle of the Robert-Asselin filter (mod_asselin.F90: asselin_save
:28-82, asselin_filter :84-268): known answers and invariants."""
import numpy as np
import pytest

from helpers import basin, np_case, oracle_grid
from oracle import oracle as O


def assel_case(b, g, kdm=3, ntracr=2, mxlmy=False, seed=61):
    """Level t-1 (n) and t (m) of every scalar, the thickness copies dpo and
    the barotropic pressure, as they stand when asselin_save runs."""
    c = np_case(b, g, kdm=kdm, ntracr=ntracr, seed=seed, courant=0.5, delt1=1800.0)
    rng = np.random.default_rng(seed)
    sh = (b.ld2, b.ld1)
    a = {k: c[k] for k in ("temp", "saln", "th3d", "dp")}
    a["tracer"] = c["tracer"]
    a["dpo"] = np.ascontiguousarray(c["dp"] * (1.0 + 0.01 * rng.standard_normal(c["dp"].shape)))
    a["pbot"] = np.ascontiguousarray(4.0e7 * (0.5 + rng.random(sh)))
    a["pbavg"] = np.ascontiguousarray(1.0e4 * rng.standard_normal((3,) + sh))
    a["oneta"] = np.ones((2,) + sh)
    a["onetao"] = np.ones((2,) + sh)
    a["otemp"] = np.zeros((kdm,) + sh)
    a["osaln"] = np.zeros((kdm,) + sh)
    a["oth3d"] = np.zeros((kdm,) + sh)
    a["otracer"] = np.zeros((ntracr, kdm) + sh) if ntracr else None
    if mxlmy:
        a["q2"] = 0.01 + 0.1 * rng.random((2, kdm + 2) + sh)
        a["q2l"] = 0.1 + rng.random((2, kdm + 2) + sh)
        a["oq2"] = np.zeros((kdm + 2,) + sh)
        a["oq2l"] = np.zeros((kdm + 2,) + sh)
    return a


def advance(a, n, rng):
    """Stand-in for the step between save and filter: new level n values."""
    for k in ("temp", "saln") + (("q2", "q2l") if "q2" in a else ()):
        a[k][n - 1] += 0.05 * rng.standard_normal(a[k][n - 1].shape)
    if a["tracer"] is not None:
        a["tracer"][:, n - 1] = np.abs(a["tracer"][:, n - 1] + 0.05 * rng.standard_normal(a["tracer"][:, n - 1].shape))
    a["dp"][n - 1] *= 1.0 + 0.01 * rng.standard_normal(a["dp"][n - 1].shape)
    a["pbavg"][n - 1] += 100.0 * rng.standard_normal(a["pbavg"][n - 1].shape)


def sea_of(b, g):
    sea = np.zeros((b.ld2, b.ld1), bool)
    sea[b.J, b.I] = True
    return sea & (g.masks["ip"] != 0)


def test_save_copies_level_n_and_sets_oneta():
    b = basin(50, 40, False, 61)
    g = oracle_grid(b, threads=1)
    a = assel_case(b, g, mxlmy=True)
    m, n = 1, 2
    g.asselin_save(m, n, a, oneta0=0.1)
    sea = sea_of(b, g)
    interior = np.zeros_like(sea)
    interior[b.J, b.I] = True
    assert np.array_equal(a["otemp"][:, interior], a["temp"][n - 1][:, interior])
    assert np.array_equal(a["otracer"][:, :, interior], a["tracer"][:, n - 1][:, :, interior])
    assert np.array_equal(a["oq2"][1:-1][:, interior], a["q2"][n - 1][1:-1][:, interior])
    want = np.maximum(0.1, 1.0 + a["pbavg"][n - 1] / a["pbot"])
    assert np.array_equal(a["oneta"][n - 1][sea], want[sea])
    assert np.array_equal(a["onetao"], a["oneta"])


@pytest.mark.parametrize("mxlmy", [False, True])
def test_filter_smooths_thickness_weighted_scalars(mxlmy):
    """dpmidn*S(m) = dpmid*S(m) + ra2fac/2*(dpold*S(t-1) + dpnew*S(n) - 2*dpmid*S(m)),
    th3d(m) = sig(T(m),S(m)) - thbase, tracers stay within their three values."""
    b = basin(60, 45, True, 62)
    g = oracle_grid(b, threads=1)
    a = assel_case(b, g, mxlmy=mxlmy)
    m, n = 2, 1
    rng = np.random.default_rng(62)
    g.asselin_save(m, n, a, oneta0=0.1)
    old = {k: (None if v is None else v.copy()) for k, v in a.items()}
    advance(a, n, rng)
    before = {k: (None if v is None else v.copy()) for k, v in a.items()}
    ra2fac = 0.125
    g.asselin_filter(m, n, a, ra2fac=ra2fac, oneta0=0.1, thbase=34.0)
    sea = sea_of(b, g)
    on = np.maximum(0.1, 1.0 + before["pbavg"][n - 1] / before["pbot"])
    om = np.maximum(0.1, 1.0 + before["pbavg"][m - 1] / before["pbot"])
    dpold = before["dpo"][n - 1] * before["onetao"][n - 1]
    dpmid = before["dpo"][m - 1] * before["onetao"][m - 1]
    dpnew = before["dp"][n - 1] * on
    dpmidn = dpmid + 0.5 * ra2fac * (dpold + dpnew - 2 * dpmid)
    assert np.allclose(a["dp"][m - 1][:, sea], (dpmidn / om)[:, sea], rtol=1e-14, atol=0)
    for k, o in (("saln", "osaln"), ("temp", "otemp")):
        lhs = dpmidn * a[k][m - 1]
        rhs = dpmid * before[k][m - 1] + 0.5 * ra2fac * (dpold * a[o] + dpnew * before[k][n - 1]
                                                          - 2 * dpmid * before[k][m - 1])
        assert np.allclose(lhs[:, sea], rhs[:, sea], rtol=1e-12, atol=1e-9 * np.abs(rhs).max())
    t, s, h = a["temp"][m - 1][:, sea].ravel(), a["saln"][m - 1][:, sea].ravel(), a["th3d"][m - 1][:, sea].ravel()
    for idx in range(0, t.size, max(1, t.size // 50)):
        assert h[idx] == O.sig(t[idx], s[idx]) - 34.0
    tr, lo = a["tracer"][:, m - 1], np.minimum(np.minimum(a["otracer"], before["tracer"][:, m - 1]),
                                               before["tracer"][:, n - 1])
    assert np.all(tr[..., sea] >= lo[..., sea])
    land = ~sea
    assert np.array_equal(a["temp"][m - 1][:, land], before["temp"][m - 1][:, land])
    if mxlmy:
        assert not np.array_equal(a["q2"][m - 1], before["q2"][m - 1])
    assert old["otemp"] is not None


def test_constant_fields_stay_constant():
    b = basin(40, 30, False, 63)
    g = oracle_grid(b, threads=1)
    a = assel_case(b, g)
    a["saln"][:] = 35.0
    a["tracer"][:] = 2.0
    m, n = 1, 2
    g.asselin_save(m, n, a, oneta0=0.1)
    advance(a, n, np.random.default_rng(63))
    a["saln"][:] = 35.0
    a["tracer"][:] = 2.0
    g.asselin_filter(m, n, a, ra2fac=0.25, oneta0=0.1)
    sea = sea_of(b, g)
    assert np.all(a["saln"][m - 1][:, sea] == 35.0)
    assert np.all(a["tracer"][:, m - 1][..., sea] == 2.0)


def test_rejects_th3d_advection():
    b = basin(40, 30, False, 64)
    g = oracle_grid(b, threads=1)
    a = assel_case(b, g, ntracr=0)
    with pytest.raises(O.OracleError):
        g.asselin_filter(1, 2, a, ra2fac=0.125, oneta0=0.1, advflg=1)


def asselin_numpy(g, b, a, m, n, ra2fac, oneta0, thbase):
    """asselin_save then asselin_filter (mod_asselin.F90:28-82, :84-268,
    hybrid layers advecting temperature, no mxlmy) restated apart from the
    oracle as whole-slice numpy, in place on a copy of the arrays."""
    mm, nn = m - 1, n - 1
    inner = np.zeros((b.ld2, b.ld1), bool)
    inner[b.J, b.I] = True
    sea = inner & (g.masks["ip"] != 0)
    for lv in (nn, mm):  # :46-51
        a["oneta"][lv][sea] = np.maximum(oneta0, 1.0 + a["pbavg"][lv] / a["pbot"])[sea]
        a["onetao"][lv][sea] = a["oneta"][lv][sea]
    for k, o in (("temp", "otemp"), ("saln", "osaln"), ("th3d", "oth3d")):  # :53-60
        a[o][:, inner] = a[k][nn][:, inner]
    if a["tracer"] is not None:
        a["otracer"][:, :, inner] = a["tracer"][:, nn][:, :, inner]
    g.xctilr(a["oneta"], 6, 6)  # :77-78
    g.xctilr(a["onetao"], 6, 6)
    return sea


def asselin_filter_numpy(a, sea, m, n, ra2fac, oneta0, thbase):
    from oracle import oracle as O

    mm, nn = m - 1, n - 1
    for lv in (nn, mm):  # :110-115
        a["oneta"][lv][sea] = np.maximum(oneta0, 1.0 + a["pbavg"][lv] / a["pbot"])[sea]
    onezm = 9806.e-20
    kdm = a["temp"].shape[1]
    for k in range(kdm):
        dpold = a["dpo"][nn, k] * a["onetao"][nn]
        dpmid = a["dpo"][mm, k] * a["onetao"][mm]
        dpnew = a["dp"][nn, k] * a["oneta"][nn]
        q = 0.5 * ra2fac * ((dpold + dpnew) - 2.0 * dpmid)
        dpmidn = dpmid + q
        with np.errstate(divide="ignore", invalid="ignore"):  # land cells carry zeros
            a["dp"][mm, k][sea] = (dpmidn / a["oneta"][mm])[sea]
            qd = 1.0 / dpmidn
        live = sea & (dpmidn > onezm)

        def filt(old, mid, new):  # :140-156, :170-178, :205-213
            smin = np.minimum(np.minimum(old, mid), new)
            so, sm, sn = dpold * (old - smin), dpmid * (mid - smin), dpnew * (new - smin)
            with np.errstate(invalid="ignore"):
                return smin + (sm + 0.5 * ra2fac * ((so + sn) - 2.0 * sm)) * qd

        a["saln"][mm, k][live] = filt(a["osaln"][k], a["saln"][mm, k], a["saln"][nn, k])[live]
        a["temp"][mm, k][live] = filt(a["otemp"][k], a["temp"][mm, k], a["temp"][nn, k])[live]
        t, s = a["temp"][mm, k][live], a["saln"][mm, k][live]
        a["th3d"][mm, k][live] = [O.sig(x, y) - thbase for x, y in zip(t, s)]
        if a["tracer"] is not None:
            for q_ in range(a["tracer"].shape[0]):
                tr = a["tracer"][q_]
                tr[mm, k][live] = filt(a["otracer"][q_, k], tr[mm, k], tr[nn, k])[live]


@pytest.mark.parametrize("periodic,ntracr", [(False, 2), (True, 0)])
def test_asselin_numpy_equals_oracle(periodic, ntracr):
    """Known answer: save, a new level n, filter -- the numpy restatement
    equals the oracle bit for bit (dp(m), T, S, th3d, tracers, oneta)."""
    b = basin(46, 34, periodic, 63)
    g = oracle_grid(b, threads=1)
    a = assel_case(b, g, kdm=3, ntracr=ntracr, seed=63)
    rng = np.random.default_rng(63)
    m, n = 1, 2
    w = {k: (None if v is None else v.copy()) for k, v in a.items()}
    g.asselin_save(m, n, a, oneta0=0.1)
    sea = asselin_numpy(g, b, w, m, n, 0.125, 0.1, 34.0)
    advance(a, n, rng)  # the same new level n for both
    for k in ("temp", "saln", "dp", "pbavg"):
        w[k][n - 1] = a[k][n - 1]
    if a["tracer"] is not None:
        w["tracer"][:, n - 1] = a["tracer"][:, n - 1]
    g.asselin_filter(m, n, a, ra2fac=0.125, oneta0=0.1, thbase=34.0)
    asselin_filter_numpy(w, sea, m, n, 0.125, 0.1, 34.0)
    for k in ("dp", "temp", "saln", "th3d", "tracer", "oneta", "onetao", "otemp", "osaln", "oth3d"):
        if a[k] is not None:
            assert np.array_equal(a[k], w[k]), k
    assert not np.array_equal(a["temp"][m - 1], assel_case(b, g, kdm=3, ntracr=ntracr, seed=63)["temp"][m - 1])
