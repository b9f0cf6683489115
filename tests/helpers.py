"""Shared builders for the tests: synthetic basins, oracle grids, cases."""
from __future__ import annotations

import numpy as np

from hycadv import synth
from oracle import oracle as O


def basin(nx, ny, periodic, seed):
    return synth.make_basin(nx, ny, periodic, seed)


def oracle_grid(b, threads=0):
    scp2, scp2i = b.metrics()
    return O.Grid(b.depth, scp2, scp2i, nbdy=b.nbdy, threads=threads)


def np_case(b, g, kdm, ntracr, seed, courant, delt1, passive=True):
    """Case as numpy arrays (CPU), keyed like the oracle's tsadvc arguments."""
    c = synth.build_case(b, g.masks, kdm=kdm, ntracr=ntracr, seed=seed, courant=courant, delt1=delt1,
                         device="cpu", passive=passive)
    out = {k: getattr(c, k).numpy().copy() for k in ("temp", "saln", "th3d", "uflx", "vflx", "dp")}
    out["tracer"] = c.tracer.numpy().copy() if ntracr > 0 else None
    out["scp2"] = c.scp2.numpy().copy()
    out["scp2i"] = c.scp2i.numpy().copy()
    return out


def levels(step):
    """(m, n) of HYCOM_Run for a step counted from 1 (mod_hycom.F90:2254-2255),
    shifted so that the first step reads level 1 as time t."""
    m = ((step + 1) % 2) + 1
    n = (step % 2) + 1
    return m, n


def same(a, b):
    """Bitwise-equal values (treating -0.0 == +0.0) and identical NaN positions."""
    a = np.asarray(a)
    b = np.asarray(b)
    return bool(np.array_equal(np.isnan(a), np.isnan(b)) and np.all((a == b) | (np.isnan(a) & np.isnan(b))))


def max_rel(a, b, mask=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if mask is not None:
        a = a[..., mask]
        b = b[..., mask]
    den = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / den)


def noise(b, rng, shape):
    """Gaussian noise, periodic in i on a periodic basin (the halo columns copy
    the interior ones, as a halo refresh would leave them)."""
    a = rng.standard_normal(shape)
    if b.periodic:
        cols = (np.arange(b.ld1) - b.nbdy) % b.nx + b.nbdy
        a = a[..., cols]
    return a


def diff_grid(b, seed):
    """Diffusion metrics aspux, aspvy, scuy, scvx of a 10 km grid, perturbed so
    every factor matters."""
    rng = np.random.default_rng(seed)
    shape = (b.ld2, b.ld1)
    one = lambda a: np.ascontiguousarray(1.0 + a * noise(b, rng, shape))
    return dict(aspux=one(0.05), aspvy=one(0.05), scuy=1.0e4 * one(0.02), scvx=1.0e4 * one(0.02))


def oneta_field(b, seed):
    """oneta(ld1,ld2,2) = 1 + pbavg/pbot, a few percent from 1."""
    rng = np.random.default_rng(seed + 1)
    return np.ascontiguousarray(1.0 + 0.02 * noise(b, rng, (2, b.ld2, b.ld1)))


def cnuity_case(b, g, kdm=3, seed=81, delt1=1800.0, umax=0.5, btrmas=False, thkdf=False):
    """Inputs of cnuity(m,n) in the reference layout (numpy): thicknesses of
    both levels, u-/v-point thicknesses and velocities of level m, barotropic
    velocities, the bottom pressure and u/v-point depths, the interface
    pressures p(:,:,1:kdm+1) and the metrics.  Velocities reach umax m/s, so
    the Courant number is umax*delt1/1e4."""
    rng = np.random.default_rng(seed)
    sh = (b.ld2, b.ld1)
    ip = g.masks["ip"] != 0
    onem = 9.806 / (1.0 / 1000.0)

    def smooth(amp, shape):
        return amp * noise(b, rng, shape)

    dp = np.zeros((2, kdm) + sh)
    for k in range(kdm):
        dp[0, k] = (20.0 + 5.0 * k) * onem * (1.0 + 0.2 * np.tanh(smooth(1.0, sh)))
    dp[1] = dp[0] * (1.0 + 0.01 * np.tanh(smooth(1.0, (kdm,) + sh)))
    dp *= ip
    pbot = dp[0].sum(axis=0)
    c = {"dp": np.ascontiguousarray(dp)}
    c["dpo"] = np.zeros((2, kdm) + sh)
    dpu = np.zeros((2, kdm) + sh)
    dpv = np.zeros((2, kdm) + sh)
    dpu[..., 1:] = 0.5 * (dp[..., 1:] + dp[..., :-1])
    dpv[..., 1:, :] = 0.5 * (dp[..., 1:, :] + dp[..., :-1, :])
    c["dpu"], c["dpv"] = dpu * (g.masks["iu"] != 0), dpv * (g.masks["iv"] != 0)
    c["u"] = np.ascontiguousarray(smooth(umax * 0.6, (2, kdm) + sh) * (g.masks["iu"] != 0))
    c["v"] = np.ascontiguousarray(smooth(umax * 0.6, (2, kdm) + sh) * (g.masks["iv"] != 0))
    c["ubavg"] = np.ascontiguousarray(smooth(umax * 0.3, (3,) + sh) * (g.masks["iu"] != 0))
    c["vbavg"] = np.ascontiguousarray(smooth(umax * 0.3, (3,) + sh) * (g.masks["iv"] != 0))
    c["pbot"] = np.ascontiguousarray(pbot)
    du = np.zeros(sh)
    dv = np.zeros(sh)
    du[:, 1:] = np.minimum(pbot[:, 1:], pbot[:, :-1])
    dv[1:, :] = np.minimum(pbot[1:, :], pbot[:-1, :])
    c["depthu"], c["depthv"] = du, dv
    c["oneta"] = np.ascontiguousarray(1.0 + 0.01 * noise(b, rng, (2,) + sh)) if btrmas else None
    c["scuy"] = np.full(sh, 1.0e4)
    c["scvx"] = np.full(sh, 1.0e4)
    if thkdf:
        c["thkdfu"] = np.full(sh, 0.02 * 1.0e4 ** 3 / 1.0e8 * 0.05)
        c["thkdfv"] = np.full(sh, 0.02 * 1.0e4 ** 3 / 1.0e8 * 0.05)
    p = np.zeros((kdm + 1,) + sh)
    p[1:] = np.cumsum(dp[0], axis=0)
    c["p"] = p
    c["uflx"] = np.zeros((kdm,) + sh)
    c["vflx"] = np.zeros((kdm,) + sh)
    c["uflxav"] = np.zeros((kdm,) + sh)
    c["vflxav"] = np.zeros((kdm,) + sh)
    c["dpav"] = np.zeros((kdm,) + sh)
    c["onetacnt"] = np.zeros(sh) if btrmas else None
    return {k: (None if v is None else np.ascontiguousarray(v)) for k, v in c.items()}
