"""Seeded synthetic basins and fields for the tracer-advection path.

HYCOM's benchmark regions are not available here, so every workload is a
seeded synthetic stand-in with the shapes, units and value distributions of
the reference's model state (mod_cb_arrays.F90):

* thickness ``dp`` in pressure units, ``onem = 9806`` Pa per metre
  (mod_cb_arrays.F90:843-851);
* mass fluxes ``uflx``/``vflx`` in Pa*m^2/s on the Arakawa C-grid faces,
  zero on faces that are not between two sea cells;
* ``scp2 = dx*dy`` and ``scp2i = 1/scp2`` (geopar.F90:315,320).

All 2-D slices use the reference's memory layout: the Fortran array
``a(1-nbdy:idm+nbdy, 1-nbdy:jdm+nbdy)`` is stored column-major, which is a
C-order array of shape ``(jdm+2*nbdy, idm+2*nbdy)`` indexed ``[j, i]``.
Element ``(i, j)`` (Fortran index, i from 1-nbdy) is ``a[j+nbdy-1, i+nbdy-1]``,
so the interior i=1..idm is ``a[..., nbdy:nbdy+idm]``.
Multi-level fields ``a(:,:,k,t)`` are C-order ``(2, kdm, ld2, ld1)``.

Every random quantity comes from its own ``numpy.random.SeedSequence`` keyed
by (master seed, basin, layer, field), so any slice regenerates
independently.  Random *parameters* are drawn on the CPU; the fields are
evaluated from them with torch, on whatever device is asked for, using
separable sums of sines and Gaussians (outer products), so a 4500x3298x41
basin is generated on the GPU in seconds.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

NBDY = 6
ONEM = 9806.0  # Pa per metre, mod_cb_arrays.F90:846


def _rng(*key: int) -> np.random.Generator:
    return np.random.default_rng(np.random.SeedSequence([int(k) & 0xFFFFFFFF for k in key]))


@dataclass
class Basin:
    """Geometry of one basin (single tile, ii=idm, jj=jdm)."""

    nx: int
    ny: int
    periodic: bool
    seed: int
    nbdy: int = NBDY
    dx: float = 10.0e3
    dy: float = 10.0e3
    depth: np.ndarray = field(default=None, repr=False)  # (ld2, ld1) metres, halo zero

    @property
    def ld1(self) -> int:
        return self.nx + 2 * self.nbdy

    @property
    def ld2(self) -> int:
        return self.ny + 2 * self.nbdy

    @property
    def I(self) -> slice:
        """Array index range of the interior columns i=1..nx (i maps to i+nbdy-1)."""
        return slice(self.nbdy, self.nbdy + self.nx)

    @property
    def J(self) -> slice:
        return slice(self.nbdy, self.nbdy + self.ny)

    def interior(self, a):
        """View of the interior (j=1..ny, i=1..nx) of a (..., ld2, ld1) array."""
        return a[..., self.J, self.I]

    def metrics(self):
        """scp2, scp2i as (ld2, ld1) float64 arrays (uniform dx*dy grid)."""
        scp2 = np.full((self.ld2, self.ld1), self.dx * self.dy, dtype=np.float64)
        scp2i = 1.0 / np.maximum(scp2, 1.0e-20)
        return scp2, scp2i


def _fill_one_point_seas(land: np.ndarray, periodic: bool) -> np.ndarray:
    """Turn sea cells with four land neighbours into land, repeatedly.

    bigrid.F90:156-191 stops the model on such cells, so the generator
    never produces them.
    """
    land = land.copy()
    while True:
        sea = ~land
        if periodic:
            w = np.roll(land, 1, axis=1)
            e = np.roll(land, -1, axis=1)
        else:
            w = np.pad(land, ((0, 0), (1, 0)), constant_values=True)[:, :-1]
            e = np.pad(land, ((0, 0), (0, 1)), constant_values=True)[:, 1:]
        s = np.pad(land, ((1, 0), (0, 0)), constant_values=True)[:-1, :]
        n = np.pad(land, ((0, 1), (0, 0)), constant_values=True)[1:, :]
        bad = sea & w & e & s & n
        if not bad.any():
            return land
        land[bad] = True


def make_closed_basin(nx: int, ny: int, seed: int, n_islands: int = 6) -> Basin:
    """Closed rectangular basin: 2-cell coastal wall plus seeded islands."""
    rng = _rng(seed, 1)
    land = np.zeros((ny, nx), dtype=bool)
    land[:2, :] = True
    land[-2:, :] = True
    land[:, :2] = True
    land[:, -2:] = True
    for _ in range(n_islands):
        w = int(rng.integers(3, max(4, nx // 8)))
        h = int(rng.integers(3, max(4, ny // 8)))
        i0 = int(rng.integers(4, max(5, nx - w - 4)))
        j0 = int(rng.integers(4, max(5, ny - h - 4)))
        land[j0:j0 + h, i0:i0 + w] = True
    land = _fill_one_point_seas(land, periodic=False)
    b = Basin(nx=nx, ny=ny, periodic=False, seed=seed)
    depth = np.zeros((b.ld2, b.ld1), dtype=np.float64)
    b.interior(depth)[...] = np.where(land, 0.0, 4000.0)
    b.depth = depth
    return b


def make_periodic_basin(nx: int, ny: int, seed: int, land_frac: float = 0.30) -> Basin:
    """Periodic-in-x, closed-in-y basin; land from thresholded smooth noise."""
    rng = _rng(seed, 2)
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    noise = np.zeros((ny, nx))
    for _ in range(12):
        kx = int(rng.integers(1, 9))  # integer wavenumbers keep it periodic in x
        ky = float(rng.uniform(0.5, 8.0))
        ph = rng.uniform(0, 2 * np.pi, size=2)
        amp = 1.0 / (kx + ky)
        noise += amp * np.outer(np.sin(2 * np.pi * ky * y + ph[1]), np.sin(2 * np.pi * kx * x + ph[0]))
    thr = np.quantile(noise, 1.0 - land_frac)
    land = noise > thr
    land[:2, :] = True
    land[-2:, :] = True
    land = _fill_one_point_seas(land, periodic=True)
    if land[:, -1].all():  # periodicity is detected from sea in column nx (bigrid.F90:25-33)
        land[2:-2, -1] = False
        land = _fill_one_point_seas(land, periodic=True)
    b = Basin(nx=nx, ny=ny, periodic=True, seed=seed)
    depth = np.zeros((b.ld2, b.ld1), dtype=np.float64)
    b.interior(depth)[...] = np.where(land, 0.0, 4000.0)
    b.depth = depth
    return b


# ----------------------------------------------------------------------
# smooth random fields, evaluated with torch
# ----------------------------------------------------------------------


def _coords(b: Basin, device, stagger_x=0.0, stagger_y=0.0):
    import torch

    i = torch.arange(1 - b.nbdy, b.nx + b.nbdy + 1, device=device, dtype=torch.float64)
    j = torch.arange(1 - b.nbdy, b.ny + b.nbdy + 1, device=device, dtype=torch.float64)
    x = (i - 0.5 + stagger_x) / b.nx  # fraction of the domain
    y = (j - 0.5 + stagger_y) / b.ny
    return x, y


def _sines(b: Basin, rng: np.random.Generator, nterm: int, kmin: float, kmax: float, device,
           stagger_x=0.0, stagger_y=0.0):
    """sum_m a_m sin(2pi(kx x + ky y) + phi), separable; normalised to max|.|=1."""
    import torch

    x, y = _coords(b, device, stagger_x, stagger_y)
    out = torch.zeros((b.ld2, b.ld1), dtype=torch.float64, device=device)
    for _ in range(nterm):
        if b.periodic:
            kx = float(rng.integers(max(1, int(kmin)), max(2, int(kmax) + 1)))
        else:
            kx = float(rng.uniform(kmin, kmax))
        ky = float(rng.uniform(kmin, kmax))
        ph = float(rng.uniform(0, 2 * np.pi))
        a = float(rng.uniform(0.5, 1.0)) / (1.0 + 0.2 * (kx + ky))
        ax = 2 * np.pi * kx * x + ph
        ay = 2 * np.pi * ky * y
        out += a * (torch.outer(torch.cos(ay), torch.sin(ax)) + torch.outer(torch.sin(ay), torch.cos(ax)))
    m = out.abs().max()
    return out / torch.clamp(m, min=1e-30)


def _eddies(b: Basin, rng: np.random.Generator, n: int, rmin: float, rmax: float, device):
    """Sum of n signed Gaussian eddies (separable), radii in cells."""
    import torch

    i = torch.arange(1 - b.nbdy, b.nx + b.nbdy + 1, device=device, dtype=torch.float64)
    j = torch.arange(1 - b.nbdy, b.ny + b.nbdy + 1, device=device, dtype=torch.float64)
    out = torch.zeros((b.ld2, b.ld1), dtype=torch.float64, device=device)
    for _ in range(n):
        ci = float(rng.uniform(1, b.nx))
        cj = float(rng.uniform(1, b.ny))
        r = float(rng.uniform(rmin, rmax))
        s = float(rng.choice([-1.0, 1.0])) * float(rng.uniform(0.5, 1.0))
        di = i - ci
        if b.periodic:
            di = torch.remainder(di + b.nx / 2, b.nx) - b.nx / 2
        out += s * torch.outer(torch.exp(-((j - cj) / r) ** 2), torch.exp(-(di / r) ** 2))
    return out


@dataclass
class LayerForcing:
    dp: object  # (ld2, ld1) float64 torch, Pa, new thickness dp(:,:,k,n)
    u: object  # (ld2, ld1) float64 torch, m/s at u-faces
    v: object  # (ld2, ld1) float64 torch, m/s at v-faces


def make_layer(b: Basin, k: int, kdm: int, seed: int, courant: float, delt1: float,
               device="cpu", div_frac: float = 0.05, step_sign: float = 1.0) -> LayerForcing:
    """Thickness and face velocities of one layer.

    dp: smooth field in [10, 500] m (column sums are capped later by
    :func:`cap_columns`).  Velocity: curl of an 8-sine streamfunction (exactly
    non-divergent on the C-grid) plus a small divergent part of relative size
    ``div_frac`` and sign ``step_sign``, scaled so that the 2-D Courant
    number (max|u| + max|v|) * delt1 / dx equals courant.  :func:`mass_fluxes` turns it into
    uflx/vflx.
    """
    import torch

    r_dp = _rng(seed, 10, k)
    s = _sines(b, r_dp, 3, 0.5, 3.0, device)
    dp_m = 10.0 + 490.0 * (0.5 + 0.5 * s)
    dp = dp_m * ONEM

    r_psi = _rng(seed, 11, k)
    psi = _sines(b, r_psi, 8, 1.0, 8.0, device, stagger_x=-0.5, stagger_y=-0.5)  # q-points
    r_chi = _rng(seed, 12, k)
    chi = _sines(b, r_chi, 4, 1.0, 6.0, device)  # p-points
    u = torch.zeros_like(psi)
    v = torch.zeros_like(psi)
    u[:-1, :] = -(psi[1:, :] - psi[:-1, :])  # u(i,j) = -(psi(i,j+1)-psi(i,j))
    v[:, :-1] = psi[:, 1:] - psi[:, :-1]  # v(i,j) = psi(i+1,j)-psi(i,j)
    ud = torch.zeros_like(chi)
    vd = torch.zeros_like(chi)
    ud[:, 1:] = chi[:, 1:] - chi[:, :-1]  # face i between cells i-1 and i
    vd[1:, :] = chi[1:, :] - chi[:-1, :]
    umax = torch.clamp(torch.maximum(u.abs().max(), v.abs().max()), min=1e-30)
    dmax = torch.clamp(torch.maximum(ud.abs().max(), vd.abs().max()), min=1e-30)
    u = u / umax + step_sign * div_frac * ud / dmax
    v = v / umax + step_sign * div_frac * vd / dmax
    # 2-D Courant number: max|u|*dt/dx + max|v|*dt/dy = courant, so that the
    # donor-cell outflow of any cell stays below its content
    smax = torch.clamp(u.abs().max() + v.abs().max(), min=1e-30)
    vel = courant * b.dx / delt1 / smax  # m/s per unit
    return LayerForcing(dp=dp, u=u * vel, v=v * vel)


def mass_fluxes(b: Basin, masks: dict, dp, u, v):
    """uflx = u * dp_face * dy on sea-sea faces (iu != 0), else 0; likewise vflx."""
    import torch

    dpu = torch.zeros_like(dp)
    dpv = torch.zeros_like(dp)
    dpu[:, 1:] = 0.5 * (dp[:, 1:] + dp[:, :-1])
    dpv[1:, :] = 0.5 * (dp[1:, :] + dp[:-1, :])
    iu = torch.as_tensor(masks["iu"], device=dp.device) != 0
    iv = torch.as_tensor(masks["iv"], device=dp.device) != 0
    uflx = torch.where(iu, u * dpu * b.dy, torch.zeros_like(u))
    vflx = torch.where(iv, v * dpv * b.dx, torch.zeros_like(v))
    return uflx, vflx


def cap_columns(dp_layers, max_depth_m: float = 4000.0):
    """Scale each column so that sum_k dp <= max_depth (in place, list of (ld2,ld1))."""
    import torch

    tot = torch.zeros_like(dp_layers[0])
    for d in dp_layers:
        tot += d
    fac = torch.clamp(max_depth_m * ONEM / torch.clamp(tot, min=1e-30), max=1.0)
    for d in dp_layers:
        d.mul_(fac)


def make_tracer_layer(b: Basin, kind: str, k: int, kdm: int, seed: int, tracer_index: int = 0,
                      device="cpu"):
    """One (ld2, ld1) float64 slice of temperature, salinity or a passive tracer.

    kind 'temp': [-2, 30] degC, layer mean decreasing with depth plus eddies.
    kind 'saln': [30, 38] psu.
    kind 'passive': log-uniform concentrations in [1e-6, 1e2] in piecewise
    constant patches separated by sharp fronts.
    """
    import torch

    if kind == "temp":
        r = _rng(seed, 20, k)
        base = 28.0 - 26.0 * (k - 1) / max(1, kdm - 1)
        t = base + 3.0 * _eddies(b, r, 12, 3.0, 20.0, device) + 0.5 * _sines(b, r, 3, 1.0, 4.0, device)
        return torch.clamp(t, -2.0, 30.0)
    if kind == "saln":
        r = _rng(seed, 21, k)
        base = 34.0 + 1.0 * (k - 1) / max(1, kdm - 1)
        s = base + 0.8 * _eddies(b, r, 10, 3.0, 20.0, device) + 0.3 * _sines(b, r, 3, 1.0, 4.0, device)
        return torch.clamp(s, 30.0, 38.0)
    if kind == "passive":
        r = _rng(seed, 22, k, tracer_index)
        x, y = _coords(b, device)
        th = float(r.uniform(0, np.pi))
        wl = float(r.uniform(0.05, 0.25))
        proj = (torch.outer(torch.ones_like(y), torch.cos(torch.tensor(th, dtype=torch.float64)) * x)
                + torch.outer(torch.sin(torch.tensor(th, dtype=torch.float64)) * y, torch.ones_like(x)))
        band = torch.floor(proj / wl)
        # per-band exponent in [-6, 2] from a hash of the band index
        h = torch.frac(torch.sin(band * 12.9898 + float(r.uniform(0, 100))) * 43758.5453)
        e = -6.0 + 8.0 * torch.abs(h)
        return torch.pow(10.0, e)
    raise ValueError(kind)


def perturb_old(fld, seed: int, k: int, tag: int, rel: float, b: Basin, device="cpu"):
    """fld(n) (time t-1) = fld(m) plus a small smooth perturbation."""
    r = _rng(seed, 30, k, tag)
    s = _sines(b, r, 2, 1.0, 5.0, device)
    return fld * (1.0 + rel * s)


@dataclass
class Case:
    """Full tsadvc input state of one basin, reference layout, torch tensors.

    temp/saln/th3d/dp: (2, kdm, ld2, ld1); tracer: (ntracr, 2, kdm, ld2, ld1);
    uflx/vflx: (kdm, ld2, ld1); scp2/scp2i: (ld2, ld1).  Time level index 0
    is the reference's level 1 and holds time t (the "center" field); level
    index 1 holds t-1.  So the first step is m=1, n=2.
    """

    basin: Basin
    kdm: int
    ntracr: int
    delt1: float
    temp: object
    saln: object
    th3d: object
    tracer: object
    uflx: object
    vflx: object
    dp: object
    scp2: object
    scp2i: object


def flow_fields(b: Basin, masks: dict, kdm: int, seed: int, courant: float, delt1: float, device="cpu"):
    """Layer thickness at both levels and the mass fluxes: (dp, uflx, vflx),
    dp (2, kdm, ld2, ld1) with index 1 the generated thickness and index 0
    its perturbed copy; uflx/vflx (kdm, ld2, ld1)."""
    import torch

    f64 = dict(dtype=torch.float64, device=device)
    dp = torch.empty((2, kdm, b.ld2, b.ld1), **f64)
    uflx = torch.empty((kdm, b.ld2, b.ld1), **f64)
    vflx = torch.empty((kdm, b.ld2, b.ld1), **f64)
    layers = [make_layer(b, k, kdm, seed, courant, delt1, device) for k in range(1, kdm + 1)]
    cap_columns([lf.dp for lf in layers])
    for k, lf in enumerate(layers):
        dp[1, k] = lf.dp
        dp[0, k] = perturb_old(lf.dp, seed, k + 1, 99, 0.02, b, device)
        uflx[k], vflx[k] = mass_fluxes(b, masks, lf.dp, lf.u, lf.v)
    return dp, uflx, vflx


TRACER_TAGS = {"temp": (1, 0.01), "saln": (2, 0.002)}


def tracer_levels(b: Basin, kind: str, kdm: int, seed: int, q: int = 0, device="cpu", like=None):
    """Both time levels of one tracer, (2, kdm, ld2, ld1): index 0 at time t,
    index 1 at t-1.  kind 'temp', 'saln' or 'passive' (passive tracer q);
    like='temp' gives a passive tracer that copies temperature."""
    import torch

    out = torch.empty((2, kdm, b.ld2, b.ld1), dtype=torch.float64, device=device)
    tag, rel = TRACER_TAGS.get(kind, (10 + q, 0.01))
    for k in range(kdm):
        src = like or kind
        c = make_tracer_layer(b, src, k + 1, kdm, seed, tracer_index=q, device=device)
        out[0, k] = c
        out[1, k] = perturb_old(c, seed, k + 1, tag, rel, b, device)
    return out


def build_case(b: Basin, masks: dict, kdm: int, ntracr: int, seed: int, courant: float, delt1: float,
               device="cpu", passive: bool = True) -> Case:
    """Generate every field of a tsadvc call for basin ``b`` (masks from bigrid)."""
    import torch

    dp, uflx, vflx = flow_fields(b, masks, kdm, seed, courant, delt1, device)
    temp = tracer_levels(b, "temp", kdm, seed, device=device)
    saln = tracer_levels(b, "saln", kdm, seed, device=device)
    th3d = torch.empty_like(temp)
    for k in range(kdm):
        th3d[0, k] = 20.0 + 0.1 * (k + 1) + 0.01 * temp[0, k]
        th3d[1, k] = perturb_old(th3d[0, k], seed, k + 1, 3, 0.001, b, device)
    tracer = torch.empty((max(ntracr, 0), 2, kdm, b.ld2, b.ld1), dtype=torch.float64, device=device)
    for q in range(ntracr):
        tracer[q] = tracer_levels(b, "passive", kdm, seed, q=q, device=device, like=None if passive else "temp")
    scp2, scp2i = b.metrics()
    return Case(basin=b, kdm=kdm, ntracr=ntracr, delt1=delt1, temp=temp, saln=saln, th3d=th3d,
                tracer=tracer, uflx=uflx, vflx=vflx, dp=dp,
                scp2=torch.as_tensor(scp2, device=device), scp2i=torch.as_tensor(scp2i, device=device))


# Workload presets (sizes and physics of the reference's synthetic configurations).
PRESETS = {
    # closed 257x193x10, T and S, Courant 0.5, dt 1800 s, 20 steps
    "c0": dict(nx=257, ny=193, kdm=10, ntracr=0, periodic=False, courant=0.5, delt1=1800.0, steps=20),
    # periodic-x 4500x3298x41, T and S, Courant 0.8, dt 240 s, 50 steps
    "c1": dict(nx=4500, ny=3298, kdm=41, ntracr=0, periodic=True, courant=0.8, delt1=240.0, steps=50),
}


def make_basin(nx: int, ny: int, periodic: bool, seed: int) -> Basin:
    return make_periodic_basin(nx, ny, seed) if periodic else make_closed_basin(nx, ny, seed)
