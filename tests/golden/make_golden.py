"""Write the golden fixtures in this folder (run from the repository root).

Each fixture is a small tsadvc case: the inputs (masks, metrics, fields) and
the fields after a few steps as computed by the CPU oracle (oracle/), FP64,
no FMA contraction.  The reference itself cannot be run here (Fortran, no
compiler), so these vectors pin the oracle across machines (the GPU host is
aarch64, this one x86-64) and the CUDA path against a fixed answer.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "hycom-src_gb300"), os.path.join(ROOT, "tests")]

from helpers import basin, levels, np_case, oracle_grid  # noqa: E402

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
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), f"{name}.npz"), **out)


if __name__ == "__main__":
    for c in CASES:
        make(*c)
        print("wrote", c[0])
