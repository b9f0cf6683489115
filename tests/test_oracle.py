"""CPU checks of the oracle against the reference's own run-time invariants.

The reference ships no golden vectors for this path (parity unpinned); these
are the checks its mod_pipe harness applies (mod_pipe.F90:1516-1546,
:55-75, README.src/README.src.OpenMP) plus analytic known answers.
"""
import numpy as np
import pytest

from helpers import basin, levels, max_rel, np_case, oracle_grid, same
from oracle import oracle as O

SCHEMES = [0, 1, 2, 4]


@pytest.fixture(scope="module")
def closed():
    b = basin(61, 47, False, seed=3)
    g = oracle_grid(b)
    return b, g


@pytest.fixture(scope="module")
def periodic():
    b = basin(64, 40, True, seed=5)
    g = oracle_grid(b)
    return b, g


def run_steps(g, c, nsteps, advtyp, trcflg=None, threads=0):
    if threads:
        g.set_threads(threads)
    for step in range(1, nsteps + 1):
        m, n = levels(step)
        g.tsadvc(m, n, temp=c["temp"], saln=c["saln"], th3d=c["th3d"], uflx=c["uflx"], vflx=c["vflx"],
                 dp=c["dp"], delt1=c["delt1"], advtyp=advtyp, tracer=c["tracer"], trcflg=trcflg, nstep=step)
    return c


def test_bigrid_masks(closed, periodic):
    b, g = closed
    assert g.nreg == 0
    b2, g2 = periodic
    assert g2.nreg == 1
    for gg in (g, g2):
        ip, iu, iv = gg.masks["ip"], gg.masks["iu"], gg.masks["iv"]
        # iu = ip(i-1)*ip(i), iv = ip(j-1)*ip(j) everywhere (bigrid.F90:216-252 + halo)
        assert np.array_equal(iu[:, 1:], ip[:, 1:] * ip[:, :-1])
        assert np.array_equal(iv[1:, :], ip[1:, :] * ip[:-1, :])
    # periodic halo columns are copies of the interior (xctilr on depth)
    ip = g2.masks["ip"]
    nb = b2.nbdy
    assert np.array_equal(ip[:, nb - 5:nb], ip[:, nb + b2.nx - 5:nb + b2.nx])


def test_xctilr_known_answer(closed, periodic):
    for (b, g) in (closed, periodic):
        rng = np.random.default_rng(0)
        a = rng.standard_normal((2, b.ld2, b.ld1))
        a0 = a.copy()
        g.xctilr(a, 5, 5)
        nb = b.nbdy
        I = slice(nb, nb + b.nx)
        J = slice(nb, nb + b.ny)
        assert np.array_equal(a[:, J, I], a0[:, J, I])  # interior untouched
        assert np.all(a[:, nb - 5:nb, :][:, :, nb - 5:nb + b.nx + 5] == 0.0)  # closed in y
        if g.nreg == 0:
            assert np.all(a[:, J, nb - 5:nb] == 0.0)
        else:
            assert np.array_equal(a[:, J, nb - 5:nb], a0[:, J, nb + b.nx - 5:nb + b.nx])
            assert np.array_equal(a[:, J, nb + b.nx:nb + b.nx + 5], a0[:, J, nb:nb + 5])
        # the 6th halo ring is not touched (mh = nh = 5 < nbdy)
        assert np.array_equal(a[:, 0, :], a0[:, 0, :])


@pytest.mark.parametrize("advtyp", SCHEMES)
def test_constant_field_stays_constant(closed, advtyp):
    b, g = closed
    c = np_case(b, g, kdm=3, ntracr=1, seed=11, courant=0.5, delt1=1800.0)
    c["delt1"] = 1800.0
    c["tracer"][:] = 7.25
    run_steps(g, c, 2, advtyp, trcflg=np.array([0], np.int32))
    ip = g.masks["ip"] != 0
    assert np.all(c["tracer"][0][..., ip] == 7.25)


@pytest.mark.parametrize("advtyp", SCHEMES)
def test_temperature_tracer_equals_temp(periodic, advtyp):
    """mod_pipe.F90:1516-1534: a trcflg=2 tracer advected like temp is temp, bit for bit."""
    b, g = periodic
    c = np_case(b, g, kdm=3, ntracr=2, seed=12, courant=0.8, delt1=240.0)
    c["delt1"] = 240.0
    c["tracer"][0] = c["temp"]
    run_steps(g, c, 3, advtyp, trcflg=np.array([2, 0], np.int32))
    ip = g.masks["ip"] != 0
    assert same(c["tracer"][0][..., ip], c["temp"][..., ip])


@pytest.mark.parametrize("advtyp", SCHEMES)
def test_passive_tracers_non_negative(closed, advtyp):
    """mod_pipe.F90:1536-1544: passive tracers stay >= 0."""
    b, g = closed
    c = np_case(b, g, kdm=2, ntracr=2, seed=13, courant=0.5, delt1=1800.0)
    c["delt1"] = 1800.0
    run_steps(g, c, 4, advtyp, trcflg=np.array([0, 0], np.int32))
    ip = g.masks["ip"] != 0
    assert np.all(c["tracer"][..., ip] >= 0.0)


@pytest.mark.parametrize("advtyp", [2, 4])
def test_thread_count_invariance(advtyp):
    """README.src/README.src.OpenMP: results are identical for any thread count."""
    out = []
    for thr in (1, 4):
        b = basin(53, 41, True, seed=21)
        g = oracle_grid(b)
        c = np_case(b, g, kdm=2, ntracr=1, seed=21, courant=0.8, delt1=240.0)
        c["delt1"] = 240.0
        run_steps(g, c, 2, advtyp, trcflg=np.array([0], np.int32), threads=thr)
        out.append(c)
    for k in ("temp", "saln", "tracer"):
        assert same(out[0][k], out[1][k])


@pytest.mark.parametrize("advtyp", SCHEMES)
def test_conservation_one_step(closed, advtyp):
    """sum fld*(fc+onemu)*scp2 is conserved by the flux form (mod_tsadvc.F90:788, :976)."""
    b, g = closed
    c = np_case(b, g, kdm=2, ntracr=0, seed=14, courant=0.5, delt1=1800.0)
    m, n = levels(1)
    k = 0
    fld = c["saln"][n - 1, k].copy()
    fldc = c["saln"][m - 1, k].copy()
    u, v = c["uflx"][k].copy(), c["vflx"][k].copy()
    g.xctilr(u, 5, 5)
    g.xctilr(v, 5, 5)
    g.xctilr(fld, 5, 5)
    g.xctilr(fldc, 5, 5)
    dpn = c["dp"][n - 1, k]
    sc, si = c["scp2"], c["scp2i"]
    fd = np.zeros_like(dpn)
    fd[:-1, :-1] = ((u[:-1, 1:] - u[:-1, :-1]) + (v[1:, :-1] - v[:-1, :-1])) * 1800.0 * si[:-1, :-1]
    fco = np.maximum(dpn + fd, 0.0)
    fcn = np.maximum(dpn, 0.0)
    ip = g.masks["ip"] != 0
    nb = b.nbdy
    inner = np.zeros_like(ip)
    inner[nb:nb + b.ny, nb:nb + b.nx] = True
    msk = ip & inner
    onemu = 9806.e-12
    before = np.sum((fld * (fco + onemu) * sc)[msk])
    posdef = 0.0
    g.advem(advtyp, fld, fldc, u, v, fco, fcn, posdef, sc, si, 1800.0)
    after = np.sum((fld * (fcn + onemu) * sc)[msk])
    assert abs(after - before) / abs(before) < 1e-13


@pytest.mark.parametrize("advtyp", [2, 4])
def test_fct_no_new_extrema(periodic, advtyp):
    b, g = periodic
    c = np_case(b, g, kdm=2, ntracr=2, seed=15, courant=0.8, delt1=240.0)
    c["delt1"] = 240.0
    ip = g.masks["ip"] != 0
    lo = min(c["tracer"][..., ip].min(), c["temp"][..., ip].min())
    hi_t = c["temp"][..., ip].max()
    hi_c = c["tracer"][..., ip].max()
    lo_c = c["tracer"][..., ip].min()
    run_steps(g, c, 3, advtyp, trcflg=np.array([0, 0], np.int32))
    assert c["temp"][..., ip].max() <= hi_t
    assert c["tracer"][..., ip].max() <= hi_c
    assert c["tracer"][..., ip].min() >= lo_c
    del lo


def test_periodic_shift_invariance():
    """PIPE_SHIFT (mod_pipe.F90:55-61): shifting a periodic basin shifts the result."""
    b = basin(48, 36, True, seed=31)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=2, ntracr=1, seed=31, courant=0.8, delt1=240.0)
    c["delt1"] = 240.0
    s = 17
    nb = b.nbdy
    I = slice(nb, nb + b.nx)

    def shift(a):
        a = a.copy()
        a[..., I] = np.roll(a[..., I], s, axis=-1)
        return a

    b2 = basin(48, 36, True, seed=31)
    b2.depth = shift(b.depth)
    g2 = oracle_grid(b2)
    c2 = {k: (shift(v) if isinstance(v, np.ndarray) else v) for k, v in c.items()}
    # tsadvc expects an up-to-date dp halo (mod_tsadvc.F90:1828)
    g.xctilr(c["dp"], 6, 6)
    g2.xctilr(c2["dp"], 6, 6)
    run_steps(g, c, 2, 2, trcflg=np.array([0], np.int32))
    run_steps(g2, c2, 2, 2, trcflg=np.array([0], np.int32))
    J = slice(nb, nb + b.ny)
    for k in ("temp", "saln", "tracer"):
        assert same(shift(c[k])[..., J, I], c2[k][..., J, I])


def test_transpose_symmetry():
    """PIPE_SYM transpose test (mod_pipe.F90:68-75): swap i/j and u/v.

    Exact symmetry does not hold in floating point (sums such as
    famax = ((a-b)+c)-d are re-associated by the transpose), so the check is
    to 1e-12 of the field range."""
    b = basin(40, 40, False, seed=41)
    b.depth = np.ascontiguousarray(np.maximum(b.depth, b.depth.T))  # symmetric land
    g = oracle_grid(b)
    bt = basin(40, 40, False, seed=41)
    bt.depth = b.depth.T.copy()
    gt = oracle_grid(bt)
    c = np_case(b, g, kdm=1, ntracr=0, seed=41, courant=0.5, delt1=1800.0)
    c["delt1"] = 1800.0
    ct = {k: (np.ascontiguousarray(np.swapaxes(v, -1, -2)) if isinstance(v, np.ndarray) else v)
          for k, v in c.items()}
    # u(i,j) on the west face maps to v(j,i) on the south face
    ct["uflx"], ct["vflx"] = ct["vflx"], ct["uflx"]
    run_steps(g, c, 1, 2)
    run_steps(gt, ct, 1, 2)
    ip = g.masks["ip"] != 0
    assert max_rel(np.swapaxes(ct["saln"], -1, -2), c["saln"], ip) < 1e-12


def test_pcm_unit_courant_translation():
    """Donor cell at Courant 1 in a periodic channel of uniform thickness
    moves the field one cell per step (to ~onemu/h relative)."""
    nx, ny, nb = 32, 9, 6
    from hycadv import synth

    b = synth.Basin(nx=nx, ny=ny, periodic=True, seed=0)
    d = np.zeros((b.ld2, b.ld1))
    d[nb + 2:nb + ny - 2, nb:nb + nx] = 1000.0
    b.depth = d
    g = oracle_grid(b)
    assert g.nreg == 1
    h = 100.0 * 9806.0
    dt = 3600.0
    sc, si = b.metrics()
    U = b.dx / dt * h * b.dy  # Courant 1
    u = np.where(g.masks["iu"] != 0, U, 0.0)
    v = np.zeros_like(u)
    x = np.arange(b.ld1)
    fld = np.tile(np.sin(2 * np.pi * (x - nb + 1) / nx), (b.ld2, 1))
    fld0 = fld.copy()
    fco = np.full_like(fld, h)
    fcn = np.full_like(fld, h)
    g.xctilr(fld, 5, 5)
    g.advem(0, fld, fld.copy(), u, v, fco, fcn, 0.0, sc, si, dt)
    J = slice(nb + 2, nb + ny - 2)
    I = slice(nb, nb + nx)
    expect = np.roll(fld0[J, I], 1, axis=-1)
    assert np.abs(fld[J, I] - expect).max() < 1e-12


def test_oracle_rejects_bad_advtyp(closed):
    b, g = closed
    a = np.zeros((b.ld2, b.ld1))
    with pytest.raises(O.OracleError):
        g.advem(3, a, a, a, a, a, a, 0.0, a, a, 1.0)


def test_oracle_lconserve_restores_content():
    """With advem's rescale (lconserve) the content sum(fld*fcn*scp2) after a
    step equals the sum(fld*fco*scp2) before it to round-off (the FCT2 step
    alone conserves only to its own round-off plus the coastal-quirk
    imbalance); the rescale is a sea-point scaling by one factor."""
    import numpy as np

    from helpers import basin, np_case, oracle_grid

    b = basin(60, 45, False, seed=143)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=1, ntracr=0, seed=143, courant=0.7, delt1=600.0)
    fld = c["saln"][1, 0].copy()
    fldc = c["saln"][0, 0].copy()
    u, v = c["uflx"][0].copy(), c["vflx"][0].copy()
    for a in (fld, fldc, u, v):
        g.xctilr(a, 5, 5)
    dpn = c["dp"][1, 0]
    fd = np.zeros_like(dpn)
    fd[:-1, :-1] = ((u[:-1, 1:] - u[:-1, :-1]) + (v[1:, :-1] - v[:-1, :-1])) * 600.0 * c["scp2i"][:-1, :-1]
    fco = np.maximum(dpn + fd, 0.0)
    fcn = np.maximum(dpn, 0.0)
    ip = g.masks["ip"]
    before = g.xcsum(fld * fco * c["scp2"], ip)
    plain = fld.copy()
    g.advem(2, plain, fldc, u, v, fco, fcn, 0.0, c["scp2"], c["scp2i"], 600.0)
    g.set_conserve(True)
    fixed = fld.copy()
    g.advem(2, fixed, fldc, u, v, fco, fcn, 0.0, c["scp2"], c["scp2i"], 600.0)
    after = g.xcsum(fixed * fcn * c["scp2"], ip)
    assert abs(after - before) <= 1e-14 * abs(before)
    sea = ip != 0
    ratio = fixed[sea] / plain[sea]
    assert np.allclose(ratio, ratio[0], rtol=0, atol=1e-15)
    assert np.array_equal(fixed[~sea], plain[~sea])
