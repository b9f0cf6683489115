"""Write the golden fixtures in this folder (run from the repository root).

Each fixture is a small case: the inputs (masks, metrics, fields) and the
fields after a few steps as computed by the CPU oracle (oracle/), FP64, no
FMA contraction.  Kinds: tsadvc (the advection schemes); step (a tracer
step as HYCOM_Run orders it: asselin_save, tsadvc FCT2, the diffusion
block of tsadvc, asselin_filter); cnuity (the continuity equation).  For
the step and cnuity kinds an output array is stored only where it differs
from its input (out_<name>; otherwise the input must come back unchanged).
The reference itself cannot be run here (Fortran, no compiler), so these
vectors pin the oracle across machines (the GPU host is aarch64, this one
x86-64) and the CUDA path against a fixed answer.

    python tests/golden/make_golden.py [tsadvc] [step] [cnuity]
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "hycom-src_gb300"), os.path.join(ROOT, "tests")]

from helpers import basin, cnuity_case, diff_grid, levels, np_case, oracle_grid  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = [
    # name, nx, ny, periodic, kdm, ntracr, advtyp, steps, courant, delt1, seed
    ("fct2_closed", 34, 26, False, 1, 1, 2, 3, 0.5, 1800.0, 201),
    ("fct4_periodic", 40, 22, True, 1, 1, 4, 3, 0.8, 240.0, 202),
    ("mpdata_periodic", 32, 24, True, 1, 1, 1, 3, 0.8, 240.0, 203),
    ("pcm_closed", 30, 22, False, 1, 1, 0, 3, 0.5, 1800.0, 204),
]


def make(name, nx, ny, periodic, kdm, ntracr, advtyp, steps, courant, delt1, seed):
    b = basin(nx, ny, periodic, seed)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=kdm, ntracr=ntracr, seed=seed, courant=courant, delt1=delt1)
    trcflg = np.zeros(ntracr, np.int32)
    inp = {k: c[k].copy() for k in ("temp", "saln", "uflx", "vflx", "dp", "tracer", "scp2", "scp2i")}
    for s in range(1, steps + 1):
        m, n = levels(s)
        g.tsadvc(m, n, temp=c["temp"], saln=c["saln"], th3d=c["temp"].copy(), uflx=c["uflx"], vflx=c["vflx"], dp=c["dp"],
                 delt1=delt1, advtyp=advtyp, tracer=c["tracer"], trcflg=trcflg, nstep=s)
    out = {f"in_{k}": v for k, v in inp.items()}
    out.update({f"out_{k}": c[k] for k in ("temp", "saln", "tracer", "uflx", "vflx")})
    out.update({f"mask_{k}": g.masks[k] for k in ("ip", "iu", "iv")})
    out["meta"] = np.array([nx, ny, kdm, ntracr, advtyp, steps, g.nreg, b.nbdy], np.int64)
    out["delt1"] = np.array([delt1])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


STEP_CASES = [
    # name, nx, ny, periodic, kdm, ntracr, steps, seed
    ("step_closed", 24, 18, False, 2, 1, 2, 211),
    ("step_periodic", 26, 16, True, 2, 0, 2, 212),
]
STEP_KEYS = ("temp", "saln", "th3d", "tracer", "uflx", "vflx", "dp", "dpo", "oneta", "onetao", "pbavg", "pbot",
             "otemp", "osaln", "oth3d", "otracer")
STEP_PARAMS = dict(delt1=1800.0, temdf2=0.3, thbase=34.0, ra2fac=0.125, oneta0=0.1)


def step_inputs(b, g, kdm, ntracr, seed):
    """The arrays of a tracer step: tsadvc's fields and the Robert-Asselin
    state (the thickness copy dpo, barotropic pressures, 1+eta, the saved
    level), as they stand when asselin_save runs."""
    c = np_case(b, g, kdm=kdm, ntracr=ntracr, seed=seed, courant=0.5, delt1=STEP_PARAMS["delt1"])
    rng = np.random.default_rng(seed)
    sh = (b.ld2, b.ld1)
    a = {k: c[k] for k in ("temp", "saln", "th3d", "uflx", "vflx", "dp")}
    a["tracer"] = c["tracer"] if ntracr else None
    a["dpo"] = np.ascontiguousarray(c["dp"] * (1.0 + 0.01 * rng.standard_normal(c["dp"].shape)))
    a["pbot"] = np.ascontiguousarray(4.0e7 * (0.5 + rng.random(sh)))
    a["pbavg"] = np.ascontiguousarray(1.0e4 * rng.standard_normal((3,) + sh))
    a["oneta"] = np.ones((2,) + sh)
    a["onetao"] = np.ones((2,) + sh)
    for k in ("otemp", "osaln", "oth3d"):
        a[k] = np.zeros((kdm,) + sh)
    a["otracer"] = np.zeros((ntracr, kdm) + sh) if ntracr else None
    return a


def run_step(g, a, d, step, ntracr):
    """One tracer step on the oracle, in place (mod_hycom.F90:2517, :2536, :2645)."""
    P = STEP_PARAMS
    m, n = levels(step)
    assel = {k: a[k] for k in STEP_KEYS if k not in ("uflx", "vflx")}
    g.asselin_save(m, n, assel, oneta0=P["oneta0"])
    g.tsadvc(m, n, temp=a["temp"], saln=a["saln"], th3d=a["th3d"], uflx=a["uflx"], vflx=a["vflx"], dp=a["dp"],
             delt1=P["delt1"], advtyp=2, tracer=a["tracer"], trcflg=np.zeros(max(ntracr, 1), np.int32), nstep=step)
    g.tsdff(m, n, temp=a["temp"], saln=a["saln"], th3d=a["th3d"], dp=a["dp"], oneta=a["oneta"], delt1=P["delt1"],
            temdf2=P["temdf2"], thbase=P["thbase"], tracer=a["tracer"], **d)
    g.asselin_filter(m, n, assel, ra2fac=P["ra2fac"], oneta0=P["oneta0"], thbase=P["thbase"])


def make_step(name, nx, ny, periodic, kdm, ntracr, steps, seed):
    b = basin(nx, ny, periodic, seed)
    g = oracle_grid(b)
    a = step_inputs(b, g, kdm, ntracr, seed)
    d = diff_grid(b, seed)
    sc, si = b.metrics()
    out = {f"in_{k}": v.copy() for k, v in a.items() if v is not None}
    for s in range(1, steps + 1):
        run_step(g, a, d, s, ntracr)
    out.update({f"out_{k}": v for k, v in a.items() if v is not None and not np.array_equal(v, out[f"in_{k}"])})
    out.update({f"grid_{k}": v for k, v in d.items()})
    out.update({"in_scp2": sc, "in_scp2i": si})
    out.update({f"mask_{k}": g.masks[k] for k in ("ip", "iu", "iv")})
    out["kind"] = np.array(["step"])
    out["meta"] = np.array([nx, ny, kdm, ntracr, 2, steps, g.nreg, b.nbdy], np.int64)
    out["delt1"] = np.array([STEP_PARAMS["delt1"]])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


CNUITY_CASES = [
    # name, nx, ny, periodic, kdm, thkdf (4 biharmonic, 2 Laplacian), btrmas, steps, seed
    ("cnuity_periodic", 26, 20, True, 3, 4, False, 2, 221),
    ("cnuity_btrmas_closed", 24, 18, False, 2, 2, True, 2, 222),
]


def make_cnuity(name, nx, ny, periodic, kdm, thkdf, btrmas, steps, seed):
    b = basin(nx, ny, periodic, seed)
    g = oracle_grid(b)
    c = cnuity_case(b, g, kdm=kdm, seed=seed, btrmas=btrmas, thkdf=thkdf != 0)
    sc, si = b.metrics()
    out = {f"in_{k}": v.copy() for k, v in c.items() if v is not None}
    mins = []
    for s in range(1, steps + 1):
        m, n = ((s + 1) % 2) + 1, (s % 2) + 1
        mins.append(g.cnuity(m, n, c, delt1=1800.0, nstep=s, btrmas=btrmas, thkdf4=thkdf == 4, thkdf2=thkdf == 2))
    out.update({f"out_{k}": v for k, v in c.items() if v is not None and not np.array_equal(v, out[f"in_{k}"])})
    out["out_dpkmin"] = np.stack(mins)
    out.update({"in_scp2": sc, "in_scp2i": si})
    out.update({f"mask_{k}": g.masks[k] for k in ("ip", "iu", "iv")})
    out["kind"] = np.array(["cnuity"])
    out["meta"] = np.array([nx, ny, kdm, thkdf, int(btrmas), steps, g.nreg, b.nbdy], np.int64)
    out["delt1"] = np.array([1800.0])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


if __name__ == "__main__":
    which = sys.argv[1:] or ["tsadvc", "step", "cnuity"]
    for kind, cases, fn in (("tsadvc", CASES, make), ("step", STEP_CASES, make_step), ("cnuity", CNUITY_CASES, make_cnuity)):
        if kind in which:
            for c in cases:
                fn(*c)
                print("wrote", c[0])
