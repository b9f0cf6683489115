#!/usr/bin/env python
"""Benchmark of the tracer-advection hot path (tsadvc/advem) on GB300.

Workload (default): periodic-in-x ocean basin 4500 x 3298 x 41 layers,
temperature and salinity, FCT2 (advtyp=2), plain FP64, max Courant 0.8,
delt1 = 240 s -- seeded synthetic fields with HYCOM's units and layouts
(no real region data exists here).  One step = one tsadvc(m,n) call over
all layers and both fields (leapfrog levels alternate).  The metric counts
dense interior cell*layer*tracer updates per step.

Arms:
  default            the CUDA library through its C ABI, fields resident on
                     the GPU (value), plus an end-to-end run with host
                     buffers copied in and out every step (e2e) and the CPU
                     oracle timed on a bounded sample (cpu_baseline).
  --impl reference   the reference's algorithm on the host cores: the CPU
                     restatement of mod_tsadvc (oracle/), OpenMP over all
                     cores, on a bounded sample of the same workload.

Multi-GPU (torchrun): every rank advects its own basin replica (basins are
independent, no data-path collective), so scaling is weak; the timed region
is bracketed by barriers and the max time over ranks is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "hycom-src_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "cell·layer·tracer updates/s, FP32-mixed batched vs FP64 plain @≤1e-6 err; %HBM"
UNIT = "updates/s"
WORKLOADS = {
    # periodic-x basin, T+S, FCT2/FCT4/MPDATA, FP64
    "c1": dict(nx=4500, ny=3298, kdm=41, periodic=True, courant=0.8, delt1=240.0, seed=1),
    # closed basin 257x193x10, T+S, FCT2, FP64 (CPU-sized case)
    "c0": dict(nx=257, ny=193, kdm=10, periodic=False, courant=0.5, delt1=1800.0, seed=7),
    # precision form: the c1 basin with T, S and 8 passive tracers (log-uniform, sharp fronts)
    "c2": dict(nx=4500, ny=3298, kdm=41, periodic=True, courant=0.8, delt1=240.0, seed=1, ntr=10),
    # batching form: 96 closed basins, nx 120-1500, ny 90-1100, kdm 22/32/41, 2-6 tracers
    "c3": dict(nbasin=96, periodic=False, courant=0.5, delt1=1800.0, seed=3, steps=30),
    # combined: 48 closed regional basins 800x600 .. 3000x2000, kdm 41, T, S + 8 passive tracers,
    # FP32-mixed FCT2 and MPDATA, Courant 0.9, 100 steps; more state than HBM, so resident waves
    "c4": dict(nbasin=48, periodic=False, courant=0.9, delt1=1800.0, seed=4, steps=100, kdm=41, ntr=10),
}
SCHEME_NAMES = {0: "PCM", 1: "MPDATA", 2: "FCT2", 4: "FCT4"}
FALLBACK_HBM_GBS = 6800.0


def bytes_per_update(s_t: int, s_f: int, s_dp: int, ntr: int, kdm: int, nlev: int = 3) -> float:
    """Minimal DRAM bytes per cell*layer*tracer update: read fld(n), fld(m),
    write fld(n) per tracer (nlev = 2 for PCM and MPDATA, which read no
    centre level); uflx, vflx, dp(n) per cell-layer shared by the tracers;
    scp2, scp2i (8+8) and the ip/iu/iv masks (1 byte each) per cell."""
    return nlev * s_t + (2 * s_f + s_dp) / ntr + 19.0 / (kdm * ntr)


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(kernel_key: str):
    """DRAM bytes per launch recorded in profiles/ by an ncu capture, or None."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for fn in sorted(os.listdir(d)):
        if not fn.endswith((".txt", ".md")):
            continue
        try:
            lines = open(os.path.join(d, fn)).read().splitlines()
        except Exception:
            continue
        for ln in lines:
            ln = ln.strip().strip("`")
            if ln.startswith(f"traffic_bytes_per_launch[{kernel_key}]:"):
                try:
                    return float(ln.split(":", 1)[1].split()[0])
                except Exception:
                    return None
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(self.idx)], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p is not None:
            time.sleep(0.25)
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()
                self.out = ""

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in (self.out or "").splitlines():
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_workload(wl: dict, device):
    """Basin, masks (product bigrid) and the full tsadvc state on device."""
    import hycadv
    from hycadv import synth

    b = synth.make_basin(wl["nx"], wl["ny"], wl["periodic"], wl["seed"])
    depth, masks, nreg = hycadv.bigrid(b.depth, b.nbdy)
    case = synth.build_case(b, masks, kdm=wl["kdm"], ntracr=0, seed=wl["seed"], courant=wl["courant"],
                            delt1=wl["delt1"], device=device)
    return b, masks, nreg, case


def run_cpu_sample(wl: dict, nlayers: int, min_seconds: float, steps_max: int, warmup: int, advtyp: int,
                   threads: int, gen_device, min_steps: int = 1):
    """Time the CPU oracle (OpenMP, `threads`) on the workload's basin with
    `nlayers` layers; returns (updates/s, description, steps timed)."""
    import numpy as np

    from hycadv import synth
    from oracle import oracle

    b = synth.make_basin(wl["nx"], wl["ny"], wl["periodic"], wl["seed"])
    sc, si = b.metrics()
    g = oracle.Grid(b.depth, sc, si, nbdy=b.nbdy, threads=threads)
    c = synth.build_case(b, g.masks, kdm=nlayers, ntracr=0, seed=wl["seed"], courant=wl["courant"],
                         delt1=wl["delt1"], device=gen_device)
    h = {k: getattr(c, k).cpu().numpy().copy() for k in ("temp", "saln", "th3d", "uflx", "vflx", "dp")}
    del c
    ups = b.nx * b.ny * nlayers * 2

    def step(s):
        m, n = ((s + 1) % 2) + 1, (s % 2) + 1
        g.tsadvc(m, n, temp=h["temp"], saln=h["saln"], th3d=h["th3d"], uflx=h["uflx"], vflx=h["vflx"], dp=h["dp"],
                 delt1=wl["delt1"], advtyp=advtyp, nstep=s)

    for s in range(1, warmup + 1):
        step(s)
    t0 = time.perf_counter()
    n = 0
    while n < steps_max and (n < min_steps or time.perf_counter() - t0 < min_seconds):
        n += 1
        step(warmup + n)
    dt = time.perf_counter() - t0
    desc = (f"{b.nx}x{b.ny} basin of the workload, {nlayers} of {wl['kdm']} layers, T+S, "
            f"{SCHEME_NAMES[advtyp]}, {n} timed steps after {warmup} warm-up")
    return ups * n / dt, desc, n, dt


def reference_arm(args, wl):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    import torch

    from oracle import oracle

    oracle.build()
    threads = os.cpu_count() or 1
    gen_dev = "cuda:0" if torch.cuda.is_available() else "cpu"
    rate, desc, n, dt = run_cpu_sample(wl, nlayers=args.ref_layers, min_seconds=0.0, steps_max=args.steps,
                                       warmup=args.warmup, advtyp=args.advtyp, threads=threads, gen_device=gen_dev,
                                       min_steps=args.steps)
    line = {
        "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": ws, "steps": n, "warmup": args.warmup,
        "ms_per_step": dt * 1e3 / max(n, 1), "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator, HYCOM units/layout)", "impl": "reference",
        "config": config_of(args, wl, "reference CPU restatement (oracle), FP64"),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


ENS_FORMS = {  # form -> (precision, FP64 thickness prep, advtyp)
    "fp64": ("fp64", True, 2),
    "mixed": ("mixed", True, 2),
    "mixed-fp32prep": ("mixed", False, 2),
    "fp64-fct4": ("fp64", True, 4),
    "mixed-fct4": ("mixed", True, 4),
    "fp64-mpdata": ("fp64", True, 1),
    "mixed-mpdata": ("mixed", True, 1),
    "mixed-diff": ("mixed", True, 2),  # with tsadvc's lateral diffusion fused into the step kernel
}
DIFF_FORMS = {"mixed-diff"}
FP64_REF = {2: "fp64", 4: "fp64-fct4", 1: "fp64-mpdata"}  # the FP64 form each mixed form is checked against
# the ncu capture (profiles/) whose DRAM traffic a form's strip kernel launch is quoted with
TRAFFIC_KEY = {"mixed": "col2_mixed", "mixed-fp32prep": "col2_mixed_fp32prep", "mixed-fct4": "col2_mixed_fct4",
               "mixed-mpdata": "col2_mixed_mpdata", "fp64": "fct2_fp64_ens", "mixed-diff": "col2_mixed_diff"}
KERNEL_OF_FORM = {"mixed": "mix_col2_kernel<FCT2,2,PREP64>", "mixed-fp32prep": "mix_col2_kernel<FCT2,2,FP32 prep>",
                  "mixed-fct4": "mix_col2_kernel<FCT4,2,PREP64>", "mixed-mpdata": "mix_col2_kernel<MPDATA,2,PREP64>",
                  "mixed-diff": "mix_col2_kernel<FCT2,2,PREP64,DIFF>"}


def make_ensemble(spec, form, stream):
    import hycadv

    prec, prep64, adv = ENS_FORMS[form]
    ens = hycadv.Ensemble([spec], precision=prec)
    if adv == 1:
        ens.set_posdef(0, 0, 256.0)  # temperature (mod_tsadvc.F90:1761)
    if prec == "mixed":
        ens.set_prep64(prep64)
    if form in DIFF_FORMS:
        # the diffusion block of tsadvc (temdf2 = TEMDF2) on a uniform grid:
        # aspux = aspvy = 1, scuy = scvx = sqrt(scp2)
        import numpy as np

        dx = np.sqrt(np.asarray(spec["scp2"], dtype=np.float64))
        one = np.ones_like(dx)
        ens.set_diffusion(0, TEMDF2, one, one, dx, dx)
    ens.set_stream(stream)  # graphs are recorded on the library's own stream and replayed here
    return ens


def put_basin(ens, case, kdm):
    """Leapfrog levels t-1 (old) and t (cur) of T and S, the mass fluxes and
    dp(:,:,k,n) of one tsadvc call (time level n = 2 of the generated case)."""
    import torch

    ens.put(0, "old", torch.stack([case.temp[1], case.saln[1]]).contiguous())
    ens.put(0, "cur", torch.stack([case.temp[0], case.saln[0]]).contiguous())
    ens.put(0, "uflx", case.uflx)
    ens.put(0, "vflx", case.vflx)
    ens.put(0, "dp", case.dp[1].contiguous())


def run_ensemble_forms(args, wl, b, masks, spec, case, dev, stream, dist, local, forms):
    """The basin through the ensemble (batched) API in each form (FCT2, FCT4
    or MPDATA): load, tune, one step from the inputs (an FP32-mixed form's is
    compared with the FP64 form of its scheme, which runs first), then W
    warm-up steps and K timed steps replayed from one CUDA graph, bracketed by
    barriers; content of each tracer before and after one step."""
    import torch

    kdm = wl["kdm"]
    ups_step = wl["nx"] * wl["ny"] * kdm * 2
    peak, _ = peak_hbm()
    out, first = {}, {}
    sea = sea_mask(b, masks, dev)
    for form in forms:
        prec, _, adv = ENS_FORMS[form]
        ens = make_ensemble(spec, form, stream)
        put_basin(ens, case, kdm)
        if args.tile and prec == "mixed":  # fixed shape (profiling): no tuner launches
            tx, ty, nq_ = args.tile
            ens.set_tile(tx, ty)
            ens.set_strip_tracers(nq_)
        else:
            tx, ty, _ = ens.tune(adv, wl["delt1"])
        nq = ens.option("strip_tracers") if prec == "mixed" else None
        c_old = [ens.content(0, q, "old", wl["delt1"]) for q in range(2)]
        ens.step(adv, wl["delt1"], 1)  # from the inputs: compare one step
        c_new = [ens.content(0, q, "cur", wl["delt1"]) for q in range(2)]
        got = torch.empty((2, kdm, b.ld2, b.ld1), dtype=torch.float64, device=dev)
        ens.get(0, "cur", got)
        first[form] = got[:, :, sea].clone()
        del got
        for _ in range(args.warmup):
            ens.step(adv, wl["delt1"], 1)
        ens.step(adv, wl["delt1"], args.steps, graph=True)  # capture (and one more warm pass)
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            e0.record(stream)
            ens.step(adv, wl["delt1"], args.steps, graph=True)
            e1.record(stream)
            torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()
        ms = e0.elapsed_time(e1)
        if dist:
            t = torch.tensor([ms], device=dev, dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        ms /= args.steps
        ws = dist.get_world_size() if dist else 1
        s_t = 8 if prec == "fp64" else 4  # fluxes as the tracers; dp is FP64 in every form
        # MPDATA reads no centre level: 2 tracer slices per update instead of 3
        bpu = bytes_per_update(s_t, s_t, 8, 2, kdm, 2 if adv == 1 else 3)
        ach = ups_step * bpu / (ms / 1e3) / 1e9
        tkey = TRAFFIC_KEY.get(form)
        out[form] = {"value": ws * ups_step / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "advtyp": adv,
                     "traffic_bytes_per_launch": profile_traffic(f"{tkey}_{args.workload}") if tkey else None,
                     "tile": [tx, ty],
                     "tracers_per_pass": nq, "kernel": KERNEL_OF_FORM.get(form, "fct tile/queue kernel (FP64)"),
                     "algorithmic_bytes_per_update": bpu, "achieved_GBs": ach, "frac_of_measured_hbm": ach / peak,
                     "graph_steps": args.steps, "clocks": clk.summary(),
                     "content_change_one_step": {n: abs(c_new[q] - c_old[q]) / abs(c_old[q])
                                                 for q, n in enumerate(("temp", "saln"))}}
        ens.close()
        del ens
        torch.cuda.empty_cache()
    for form in first:
        if form in DIFF_FORMS:
            # checked against the oracle's tsadvc + tsdff by the GPU tests; here the
            # size of the diffusion against the same step without it
            if "mixed" in first:
                out[form]["diffusion_change_one_step"] = {
                    name: float((first[form][q] - first["mixed"][q]).abs().max() / first["mixed"][q].abs().max())
                    for q, name in enumerate(("temp", "saln"))}
                out[form]["time_vs_mixed"] = out[form]["ms_per_step"] / out["mixed"]["ms_per_step"]
            continue
        rf = FP64_REF[ENS_FORMS[form][2]]
        if form == rf or rf not in first:
            continue
        ref = first[rf]
        errs = {}
        for q, name in enumerate(("temp", "saln")):
            d = first[form][q] - ref[q]
            scale = ref[q].abs().max()
            errs[name] = {"max_rel": float(d.abs().max() / scale),
                          "rms_rel": float(d.pow(2).mean().sqrt() / scale)}
        out[form]["vs_fp64_one_step"] = errs
        out[form]["speedup_vs_fp64_ensemble"] = out[form]["value"] / out[rf]["value"]
    return out


TEMDF2 = 0.015  # diffusion velocity (m/s) of the full form, a typical blkdat temdf2
RA2FAC = 0.125  # Robert-Asselin weight of the full form (blkdat ra2fac)
ONETA0 = 0.1    # minimum 1+eta (blkdat oneta0)


def run_tsadvc_fp64(args, wl, b, masks, nreg, sc, si, case, dev, stream, dist, local, advtyp=None, full=False,
                    btrmas=False):
    """FP64 plain form through the reference-layout C ABI (hyc_tsadvc on
    resident fields), timed over K steps after W warm-up steps.  With full,
    every step is the tracer part of a HYCOM step: asselin_save, tsadvc, its
    diffusion block (hyc_tsdff, temdf2 = TEMDF2, on a uniform grid: aspux =
    aspvy = 1, scuy = scvx = sqrt(scp2)) and asselin_filter (ra2fac =
    RA2FAC; dpo = the initial dp, pbot = 4e7 Pa, pbavg = 0, so oneta = 1).
    With btrmas, tsadvc runs with the barotropic mass flux (onetamas = 1 +
    a seeded 1 % perturbation), so FCT2 is advem_fct2c."""
    advtyp = args.advtyp if advtyp is None else advtyp
    import numpy as np
    import torch

    import hycadv

    kdm = wl["kdm"]
    ctx = hycadv.Context.from_masks(masks, sc, si, kdm=kdm, nreg=nreg, nbdy=b.nbdy, device=local)
    ctx.set_stream(stream)
    for k in ("temp", "saln", "th3d", "uflx", "vflx"):
        ctx.bind(k, getattr(case, k))
    # the Robert-Asselin filter rewrites dp(m): the full form works on a copy
    # so that dp stays consistent with uflx/vflx for the forms after it
    dpb = case.dp.clone() if full else case.dp
    ctx.bind("dp", dpb)
    keep = [dpb]
    if full:
        sh2 = tuple(case.dp.shape[-2:])
        f64 = dict(dtype=torch.float64, device=dev)
        extra = {"oneta": torch.ones((2,) + sh2, **f64), "onetao": torch.ones((2,) + sh2, **f64),
                 "pbavg": torch.zeros((3,) + sh2, **f64), "pbot": torch.full(sh2, 4.0e7, **f64),
                 "dpo": dpb.clone(), "otemp": torch.empty_like(case.temp[0]),
                 "osaln": torch.empty_like(case.saln[0]), "oth3d": torch.empty_like(case.th3d[0])}
        for k, v in extra.items():
            ctx.bind(k, v)
        keep.append(extra)
        dx = np.sqrt(np.asarray(sc, dtype=np.float64))
        one = np.ones_like(dx)
        ctx.set_diffusion_grid(one, one, dx, dx)
    if btrmas:
        sh2 = tuple(case.dp.shape[-2:])
        g = torch.Generator(device=dev).manual_seed(wl["seed"] + 77)
        oneta = 1.0 + 0.01 * torch.rand((2,) + sh2, dtype=torch.float64, device=dev, generator=g)
        ctx.bind("oneta", oneta)
        keep.append(oneta)

    def step(s):
        m, n = ((s + 1) % 2) + 1, (s % 2) + 1
        if full:
            ctx.asselin_save(m, n, oneta0=ONETA0)
        ctx.tsadvc(m, n, delt1=wl["delt1"], advtyp=advtyp, nstep=s, btrmas=btrmas)
        if full:
            ctx.tsdff(m, n, delt1=wl["delt1"], temdf2=TEMDF2)
            ctx.asselin_filter(m, n, ra2fac=RA2FAC, oneta0=ONETA0)

    for s in range(1, args.warmup + 1):
        step(s)
    torch.cuda.synchronize(dev)
    ctx.enable_timers(True)
    ctx.stats(reset=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for s in range(args.warmup + 1, args.warmup + args.steps + 1):
            step(s)
        e1.record(stream)
        torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    st = ctx.stats(reset=True)
    ctx.enable_timers(False)
    ctx.close()
    if dist:
        t = torch.tensor([ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ws = dist.get_world_size() if dist else 1
    ups_step = wl["nx"] * wl["ny"] * kdm * 2
    adv_ms, adv_calls = st["advect"]
    bpu = bytes_per_update(8, 8, 8, 2, kdm)
    peak, peak_kind = peak_hbm()
    res = {"value": ws * ups_step * args.steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / args.steps,
           "scheme": SCHEME_NAMES[advtyp] + (" + Laplacian diffusion + Robert-Asselin filter" if full else "")
           + (" with btrmas (advem_fct2c)" if btrmas else ""),
           "gpu_launches": int(st["launches"]), "clocks": clk.summary(),
           "timers_ms": {k: v for k, v in st.items() if k != "launches"}}
    if adv_calls > 0:
        # the advection kernels' device time per tsadvc call (one timed span per call, or one
        # per batch of (field, layer) pairs for advem_fct2c)
        ts_calls = max(st["tsadvc"][1], 1)
        avg_s = adv_ms / ts_calls / 1e3
        achieved = ups_step * bpu / avg_s / 1e9
        res["roofline"] = {"bound": "fp64-alu (hbm fraction shown)", "achieved": achieved, "peak": peak,
                           "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                           "kernel": ("fct2c_* stage kernels" if btrmas and advtyp == 2 else
                                      "fct_tile_kernel" if advtyp in (2, 4) else "advect_tile_kernel"),
                           "algorithmic_bytes_per_update": bpu,
                           "advect_ms_per_step": adv_ms / ts_calls, "advect_spans_per_step": adv_calls / ts_calls,
                           "share_of_step": adv_ms / max(st["tsadvc"][0], 1e-9),
                           "traffic": None if btrmas else
                           profile_traffic(f"{SCHEME_NAMES[advtyp].lower()}_fp64_{args.workload}")}
    df_ms, df_calls = st["tsdff"]
    if df_calls > 0:
        # diffusion alone: T and S updated per cell and layer; algorithmic
        # bytes = read T, S, dp and write T, S, th3d (FP64) per cell and layer
        avg_s = df_ms / df_calls / 1e3
        bpc = 6 * 8
        cells = wl["nx"] * wl["ny"] * kdm
        achieved = cells * bpc / avg_s / 1e9
        res["tsdff"] = {"value": ups_step / avg_s, "unit": UNIT, "ms_per_call": df_ms / df_calls,
                        "share_of_step": df_ms / max(ms, 1e-9),
                        "roofline": {"bound": "fp64-alu (hbm fraction shown)", "achieved": achieved, "peak": peak,
                                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                                     "kernel": "tsdff_tile_kernel + tsdff_store_kernel",
                                     "algorithmic_bytes_per_cell_layer": bpc,
                                     "traffic": profile_traffic(f"tsdff_fp64_{args.workload}")}}
    ra_ms, ra_calls = st["asselin"]
    if ra_calls > 0:
        # save + filter per step: cell-layer updates of T and S; algorithmic
        # bytes per cell and layer: save reads T, S, th3d (n) and writes the
        # three copies; filter reads dpo (2), dp (n, m), the copies of T, S
        # and T, S at both levels, writes dp, T, S, th3d (m)
        bpc = 8 * (6 + 13)
        cells = wl["nx"] * wl["ny"] * kdm
        avg_s = ra_ms / ra_calls * 2 / 1e3
        achieved = cells * bpc / avg_s / 1e9
        res["asselin"] = {"value": ups_step / avg_s, "unit": UNIT, "ms_per_step": ra_ms / ra_calls * 2,
                          "share_of_step": ra_ms / max(ms, 1e-9),
                          "roofline": {"bound": "fp64-alu (hbm fraction shown)", "achieved": achieved, "peak": peak,
                                       "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                                       "kernel": "asselin_save_kernel + asselin_filter_kernel",
                                       "algorithmic_bytes_per_cell_layer": bpc,
                                       "traffic": profile_traffic(f"asselin_fp64_{args.workload}")}}
    del keep
    return res


THKDF4 = 0.02  # biharmonic interface-diffusion velocity (m/s), a typical blkdat thkdf4


def run_cnuity(args, wl, b, masks, nreg, sc, si, case, dev, stream, dist, local):
    """cnuity (hyc_cnuity, FP64) on the workload's basin, resident fields,
    K steps after W warm-up steps: the layer thicknesses of the tsadvc case,
    velocities u = uflx/(dpu*scuy) (so the Courant number is the case's),
    ubavg = vbavg = 0, pbot = the column, biharmonic interface diffusion
    thkdf4*dx^3, not btrmas, ra2fac = RA2FAC."""
    import numpy as np
    import torch

    import hycadv

    kdm = wl["kdm"]
    ctx = hycadv.Context.from_masks(masks, sc, si, kdm=kdm, nreg=nreg, nbdy=b.nbdy, device=local)
    ctx.set_stream(stream)
    f64 = dict(dtype=torch.float64, device=dev)
    iu = torch.from_numpy(np.asarray(masks["iu"]) != 0).to(dev)
    iv = torch.from_numpy(np.asarray(masks["iv"]) != 0).to(dev)
    dx = float(np.sqrt(np.asarray(sc, dtype=np.float64)).max())
    dp = case.dp.clone()  # cnuity rewrites dp; the other forms keep the case's
    f = {"dp": dp, "dpo": torch.zeros_like(dp)}
    dpu = torch.zeros_like(dp)
    dpv = torch.zeros_like(dp)
    dpu[..., 1:] = 0.5 * (dp[..., 1:] + dp[..., :-1])
    dpv[..., 1:, :] = 0.5 * (dp[..., 1:, :] + dp[..., :-1, :])
    dpu *= iu
    dpv *= iv
    f["dpu"], f["dpv"] = dpu, dpv
    u = torch.zeros_like(dp)
    v = torch.zeros_like(dp)
    for t in range(2):
        u[t] = torch.where(iu, case.uflx / (dpu[0].clamp(min=1.0) * dx), 0.0)
        v[t] = torch.where(iv, case.vflx / (dpv[0].clamp(min=1.0) * dx), 0.0)
    f["u"], f["v"] = u, v
    sh = tuple(dp.shape[-2:])
    f["ubavg"] = torch.zeros((3,) + sh, **f64)
    f["vbavg"] = torch.zeros((3,) + sh, **f64)
    pbot = dp[0].sum(dim=0)
    f["pbot"] = pbot
    p = torch.zeros((kdm + 1,) + sh, **f64)
    p[1:] = torch.cumsum(dp[0], dim=0)
    f["p"] = p
    f["uflx"] = torch.zeros((kdm,) + sh, **f64)
    f["vflx"] = torch.zeros((kdm,) + sh, **f64)
    for k, t in f.items():
        ctx.bind(k, t)
    pb = pbot.cpu().numpy()
    du = np.zeros_like(pb)
    dv = np.zeros_like(pb)
    du[:, 1:] = np.minimum(pb[:, 1:], pb[:, :-1])
    dv[1:, :] = np.minimum(pb[1:, :], pb[:-1, :])
    dxa = np.sqrt(np.asarray(sc, dtype=np.float64))
    th = THKDF4 * dxa ** 3
    ctx.set_cnuity_grid(dxa, dxa, du, dv, th, th)
    del iu, iv

    def step(s):
        m, n = ((s + 1) % 2) + 1, (s % 2) + 1
        ctx.cnuity(m, n, delt1=wl["delt1"], nstep=s, thkdf=4, ra2fac=RA2FAC)

    for s in range(1, args.warmup + 1):
        step(s)
    torch.cuda.synchronize(dev)
    ctx.enable_timers(True)
    ctx.stats(reset=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for s in range(args.warmup + 1, args.warmup + args.steps + 1):
            step(s)
        e1.record(stream)
        torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    st = ctx.stats(reset=True)
    ctx.close()
    del f
    torch.cuda.empty_cache()
    ws = dist.get_world_size() if dist else 1
    cells = wl["nx"] * wl["ny"] * kdm
    # algorithmic bytes per cell and layer: read dp(n), dp(m), u, v, dpu, dpv;
    # write dp(n), dp(m), dpo(n), dpo(m), uflx, vflx, p (FP64)
    bpc = 13 * 8
    peak, peak_kind = peak_hbm()
    achieved = cells * bpc / (ms / args.steps / 1e3) / 1e9
    return {"value": ws * cells * args.steps / (ms / 1e3), "unit": "cell·layer updates/s",
            "ms_per_step": ms / args.steps, "gpu_launches": int(st["launches"]), "clocks": clk.summary(),
            "config": "FCT continuity + barotropic restoration + bottom restoring + biharmonic interface "
                      "diffusion + RA of dp, FP64, bit-identical to the oracle",
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "kernel": "cnuity sweeps (cn_*)",
                         "algorithmic_bytes_per_cell_layer": bpc,
                         "traffic": profile_traffic(f"cnuity_fp64_{args.workload}")}}


def run_e2e(args, wl, b, spec, case, form, tile, nq, dev, stream, dist):
    """The headline form end to end through the C ABI with host buffers: per
    step hyc_ens_put of T and S (levels t-1 and t), uflx, vflx and dp from
    pinned host memory (FP64, reference layout), hyc_ens_step, and
    hyc_ens_get_async of the new level of T and S back to pinned host memory
    (whose copy overlaps the next step's puts; hyc_ens_wait ends the run)."""
    import torch

    kdm = wl["kdm"]
    host = {}
    host["old"] = torch.stack([case.temp[1], case.saln[1]]).to("cpu").pin_memory()
    host["cur"] = torch.stack([case.temp[0], case.saln[0]]).to("cpu").pin_memory()
    for k in ("uflx", "vflx"):
        host[k] = getattr(case, k).to("cpu").pin_memory()
    host["dp"] = case.dp[1].contiguous().to("cpu").pin_memory()
    out = torch.empty_like(host["cur"]).pin_memory()
    h2d = sum(t.numel() * 8 for t in host.values())
    d2h = out.numel() * 8
    ens = make_ensemble(spec, form, stream)
    if ENS_FORMS[form][0] == "mixed":
        ens.set_tile(*tile)
        if nq:
            ens.set_strip_tracers(nq)

    phases = {"put_ms": 0.0, "step_ms": 0.0, "get_ms": 0.0}

    def e2e_step():
        t0 = time.perf_counter()
        for k in ("old", "cur", "uflx", "vflx", "dp"):
            ens.put(0, k, host[k])  # synchronous: the host buffer is free again on return
        t1 = time.perf_counter()
        ens.step(ENS_FORMS[form][2], wl["delt1"], 1)
        t2 = time.perf_counter()
        # staged on the device after the step; the copy to host overlaps the
        # next step's puts (the timed region ends with ens.wait())
        ens.get_async(0, "cur", out)
        t3 = time.perf_counter()
        phases["put_ms"] += (t1 - t0) * 1e3
        phases["step_ms"] += (t2 - t1) * 1e3
        phases["get_ms"] += (t3 - t2) * 1e3

    e2e_step()
    ens.wait()
    torch.cuda.synchronize(dev)
    for k in phases:
        phases[k] = 0.0
    ens.enable_timers(True)
    ens.stats(reset=True)
    if dist:
        dist.barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.e2e_steps):
        e2e_step()
    ens.wait()
    f1.record(stream)
    torch.cuda.synchronize(dev)
    ems = f0.elapsed_time(f1)
    est = ens.stats(reset=True)
    if dist:
        t = torch.tensor([ems], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ems = float(t.item())
    ens.close()
    K = args.e2e_steps
    device_ms = {"host_link_copies": est["copy_ms"] / K, "halo_and_repitch": est["stage_kernels_ms"] / K,
                 "step": est["step_ms"] / K}
    ws = dist.get_world_size() if dist else 1
    ups_step = wl["nx"] * wl["ny"] * kdm * 2
    return {"value": ws * ups_step * args.e2e_steps / (ems / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "steps": args.e2e_steps, "form": form,
            "host_ms_per_step": {k: v / args.e2e_steps for k, v in phases.items()},
            "device_ms_per_step": device_ms,
            "host_link_GBs": (h2d + d2h) / max(device_ms["host_link_copies"], 1e-9) / 1e6,
            "note": "per step: hyc_ens_put of T,S (t-1, t), uflx, vflx, dp from pinned host FP64 arrays "
                    "(reference layout), hyc_ens_step, hyc_ens_get_async of the new T,S level (its copy to "
                    "host overlaps the next step's puts; the timed region ends after hyc_ens_wait); "
                    "host_link_copies sums the device time of both directions' copies, which overlap"}


def c3_members(wl):
    """Seeded sizes of the 96-basin ensemble (uneven nx, ny, kdm, tracers)."""
    import numpy as np

    rng = np.random.default_rng(wl["seed"])
    out = []
    for bi in range(wl["nbasin"]):
        out.append(dict(nx=int(rng.integers(120, 1501)), ny=int(rng.integers(90, 1101)),
                        kdm=int(rng.choice([22, 32, 41])), ntr=int(rng.integers(2, 7)), seed=1000 + bi))
    return out


TRACER_KINDS = ("temp", "saln")


def member_geometry(m, wl):
    """Basin, bigrid masks and the ensemble spec of one member (host only)."""
    import hycadv
    from hycadv import synth

    b = synth.make_basin(m["nx"], m["ny"], wl["periodic"], m["seed"])
    _, masks, nreg = hycadv.bigrid(b.depth, b.nbdy)
    sc, si = b.metrics()
    spec = dict(idm=b.nx, jdm=b.ny, kdm=m["kdm"], nbdy=b.nbdy, nreg=nreg, ntr=m["ntr"], ip=masks["ip"],
                iu=masks["iu"], iv=masks["iv"], scp2=sc, scp2i=si)
    return b, masks, spec


def load_member(ens, i, m, geo, wl, dev):
    """Generate member i's flow and tracers on the device and put them one
    tracer at a time (T, S, then passive tracers); returns each tracer's
    (min, max) over sea cells of both input levels."""
    import torch

    from hycadv import synth

    b, masks, spec = geo
    kdm = spec["kdm"]
    dp, uflx, vflx = synth.flow_fields(b, masks, kdm, m["seed"], wl["courant"], wl["delt1"], dev)
    ens.put(i, "uflx", uflx)
    ens.put(i, "vflx", vflx)
    ens.put(i, "dp", dp[1].contiguous())
    del dp, uflx, vflx
    sea = sea_mask(b, masks, dev)
    bounds = []
    for q in range(spec["ntr"]):
        kind = TRACER_KINDS[q] if q < 2 else "passive"
        lv = synth.tracer_levels(b, kind, kdm, m["seed"], q=max(q - 2, 0), device=dev)
        ens.put(i, "old", lv[1].contiguous(), s0=q * kdm, ns=kdm)
        ens.put(i, "cur", lv[0].contiguous(), s0=q * kdm, ns=kdm)
        vals = lv[:, :, sea]
        bounds.append((float(vals.min()), float(vals.max())))
        del lv, vals
    return bounds


def sea_mask(b, masks, dev):
    import torch

    ip = torch.as_tensor(masks["ip"], device=dev) != 0
    inner = torch.zeros_like(ip)
    inner[b.J, b.I] = True
    return ip & inner


def run_ensemble_workload(args, wl, dev):
    """c2 (precision form) and c3 (batching form) through the ensemble API,
    printed as their own bench line (see ensemble_workload)."""
    import torch

    ws, rank, local = dist_setup()
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    torch.cuda.set_device(local)
    dev = torch.device(f"cuda:{local}")
    forms = [f for f in args.ens_forms.split(",") if f]
    t_start = time.perf_counter()
    out = ensemble_workload(args, wl, args.workload, dev, dist, forms)
    res, desc, ups, steps = out["forms"], out["workload"], out["updates_per_step"], out["steps"]
    peak, peak_kind = peak_hbm()
    head_form = "mixed" if "mixed" in res else forms[-1]
    head = res[head_form]
    line = {"metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": ws, "steps": steps,
            "warmup": 1, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-mixed" if head_form != "fp64" else "f64",
            "data": "synthetic (seeded generator, HYCOM units/layout)", "impl": f"ensemble-{args.workload}",
            "config": {"workload": desc, "form": head_form, "updates_per_step": ups,
                       "l2": "inputs larger than L2 (state resident in HBM)"},
            "roofline": {"bound": "hbm", "achieved": head["achieved_GBs"], "peak": peak, "unit": "GB/s",
                         "frac": head["frac_of_measured_hbm"], "traffic": None, "peak_kind": peak_kind},
            "clocks": head["clocks"], "wall_seconds": time.perf_counter() - t_start, "forms": res}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def ensemble_workload(args, wl, workload, dev, dist, forms, fp64_steps=None):
    """c2 (precision form) or c3 (batching form) through the ensemble API.

    Every form (FP64 plain, FP32-mixed with FP64 thickness prep, FP32-mixed
    with compensated FP32 prep) is loaded from the same seeded inputs,
    advanced one step and compared, tracer by tracer over sea cells, with
    the FP64 form's step (which is bit-identical to the oracle's): max and
    RMS error relative to the tracer's max |value|, the one-step change of
    tracer content, and the new level against the inputs' extrema.  Then
    it is timed over K steps replayed from one CUDA graph.  Tile shapes come
    from the library's autotuner.

    Under torchrun (N ranks, one GPU each) the 96 basins of c3 are sharded
    over the ranks (longest-processing-time order, hycadv.shard) and each
    rank advances its own; c2's single basin is replicated.  Nothing is
    exchanged in the data path: the timed region is bracketed by barriers,
    its time is the max over ranks, updates are summed, error metrics are
    the max over ranks."""
    import torch

    import hycadv
    from hycadv import shard as hshard

    ws, rank, local = dist_setup()

    def reduce(vals, op):
        if not dist:
            return vals
        t = torch.tensor(vals, dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=op)
        return t.tolist()

    if workload == "c3":
        members = c3_members(wl)
        if args.layers:
            for m in members:
                m["kdm"] = args.layers
        nbasin_all = len(members)
        if ws > 1:
            mine = hshard.shard([m["nx"] * m["ny"] * m["kdm"] * m["ntr"] for m in members], ws)[rank]
            members = [members[i] for i in mine]
        steps = max(args.steps, wl["steps"])
    else:
        members = [dict(nx=wl["nx"], ny=wl["ny"], kdm=args.layers or wl["kdm"], ntr=wl["ntr"], seed=wl["seed"])]
        nbasin_all = ws
        steps = args.steps
    if "fp64" in forms and forms[0] != "fp64":
        raise SystemExit("--ens-forms: fp64 (the reference the others are compared with) must come first")
    t_start = time.perf_counter()
    geos = [member_geometry(m, wl) for m in members]
    specs = [g[2] for g in geos]
    ups_rank = sum(s["idm"] * s["jdm"] * s["kdm"] * s["ntr"] for s in specs)
    ups = reduce([float(ups_rank)], dist.ReduceOp.SUM if dist else None)[0]
    peak, peak_kind = peak_hbm()
    res, refs = {}, {}
    for form in forms:
        prec = "fp64" if form == "fp64" else "mixed"
        ens = hycadv.Ensemble(specs, precision=prec)
        if prec == "mixed":
            ens.set_prep64(form == "mixed")
        t0 = time.perf_counter()
        bounds = [load_member(ens, i, m, geos[i], wl, dev) for i, m in enumerate(members)]
        torch.cuda.synchronize(dev)
        torch.cuda.empty_cache()
        t_load = time.perf_counter() - t0
        tx, ty, _ = ens.tune(2, wl["delt1"])
        c_old = [[ens.content(i, q, "old", wl["delt1"]) for q in range(s["ntr"])] for i, s in enumerate(specs)]
        ens.step(2, wl["delt1"], 1)
        ntr_max = max(s["ntr"] for s in specs)
        per_q = [{"max_rel": 0.0, "sq": 0.0, "n": 0, "cons": 0.0, "extrema_excess": 0.0} for _ in range(ntr_max)]
        for i, s in enumerate(specs):
            b, masks, _ = geos[i]
            sea = sea_mask(b, masks, dev)
            kdm = s["kdm"]
            buf = torch.empty((kdm, b.ld2, b.ld1), dtype=torch.float64, device=dev)
            for q in range(s["ntr"]):
                ens.get(i, "cur", buf, s0=q * kdm, ns=kdm)
                new = buf[:, sea]
                lo, hi = bounds[i][q]
                acc = per_q[q]
                acc["extrema_excess"] = max(acc["extrema_excess"], float(max(lo - new.min(), new.max() - hi, 0.0))
                                            / max(abs(lo), abs(hi)))
                c_new = ens.content(i, q, "cur", wl["delt1"])
                acc["cons"] = max(acc["cons"], abs(c_new - c_old[i][q]) / abs(c_old[i][q]))
                if form == "fp64":
                    refs[(i, q)] = new.clone()
                elif (i, q) in refs:
                    ref = refs[(i, q)]
                    scale = float(ref.abs().max())
                    d = new - ref
                    acc["max_rel"] = max(acc["max_rel"], float(d.abs().max()) / scale)
                    acc["sq"] += float(d.pow(2).sum()) / scale ** 2
                    acc["n"] += d.numel()
                del new
            del buf
        torch.cuda.empty_cache()
        names = ["temp", "saln"] + [f"passive{q - 1}" for q in range(2, 6 if workload == "c3" else ntr_max)]
        while len(per_q) < len(names):  # every rank reports the same tracer slots
            per_q.append({"max_rel": 0.0, "sq": 0.0, "n": 0, "cons": 0.0, "extrema_excess": 0.0})
        if dist:
            mx = reduce([v for a in per_q for v in (a["max_rel"], a["cons"], a["extrema_excess"])], dist.ReduceOp.MAX)
            sm = reduce([v for a in per_q for v in (a["sq"], float(a["n"]))], dist.ReduceOp.SUM)
            for q, a in enumerate(per_q):
                a["max_rel"], a["cons"], a["extrema_excess"] = mx[3 * q:3 * q + 3]
                a["sq"], a["n"] = sm[2 * q], int(sm[2 * q + 1])
        rep = {}
        for q, acc in enumerate(per_q):
            r = {"content_change_one_step": acc["cons"], "new_extrema_rel": acc["extrema_excess"]}
            if form != "fp64":
                r["max_rel_err_vs_fp64"] = acc["max_rel"]
                r["rms_rel_err_vs_fp64"] = (acc["sq"] / max(acc["n"], 1)) ** 0.5
            rep[names[q]] = r
        fsteps = fp64_steps if (form == "fp64" and fp64_steps) else steps
        ens.step(2, wl["delt1"], fsteps, graph=True)  # capture (and warm up)
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        st = torch.cuda.current_stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            e0.record(st)
            ens.step(2, wl["delt1"], fsteps, graph=True)
            e1.record(st)
            torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()
        ms = reduce([e0.elapsed_time(e1) / fsteps], dist.ReduceOp.MAX if dist else None)[0]
        s_t = 8 if prec == "fp64" else 4
        nbytes = sum(s["idm"] * s["jdm"] * s["kdm"] * s["ntr"] * bytes_per_update(s_t, s_t, 8, s["ntr"], s["kdm"])
                     for s in specs)
        nbytes = reduce([nbytes], dist.ReduceOp.SUM if dist else None)[0]
        ach = nbytes / (ms / 1e3) / 1e9
        res[form] = {"value": ups / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "tile": [tx, ty],
                     "graph_steps": fsteps, "achieved_GBs": ach, "frac_of_measured_hbm": ach / peak,
                     "algorithmic_bytes_per_step": nbytes, "load_seconds": t_load, "per_tracer": rep,
                     "clocks": clk.summary()}
        ens.close()
        del ens
        torch.cuda.empty_cache()
    refs.clear()
    for f in forms[1:]:
        if "fp64" in res:
            res[f]["speedup_vs_fp64"] = res[f]["value"] / res["fp64"]["value"]
    if workload == "c3":
        desc = (f"c3: {nbasin_all} closed basins, nx 120-1500, ny 90-1100, kdm 22/32/41, 2-6 tracers (T, S, "
                f"passive), FCT2, max Courant {wl['courant']}, delt1 {wl['delt1']} s, {steps}-step CUDA graph"
                + (f", sharded over {ws} GPUs" if ws > 1 else ""))
    else:
        desc = (f"c2: periodic-x basin {wl['nx']}x{wl['ny']}x{members[0]['kdm']}, T+S+8 passive tracers "
                f"(log-uniform 1e-6..1e2 with fronts), FCT2, max Courant {wl['courant']}, delt1 {wl['delt1']} s")
    return {"forms": res, "workload": desc, "updates_per_step": ups, "steps": steps,
            "wall_seconds": time.perf_counter() - t_start}


def c4_members(wl, layers=0):
    """Seeded sizes of the 48-basin combined workload."""
    import numpy as np

    rng = np.random.default_rng(wl["seed"])
    return [dict(nx=int(rng.integers(800, 3001)), ny=int(rng.integers(600, 2001)), kdm=layers or wl["kdm"],
                 ntr=wl["ntr"], seed=2000 + bi) for bi in range(wl["nbasin"])]


def mixed_state_bytes(spec):
    """Device bytes of one FP32-mixed ensemble basin (three tracer levels,
    fluxes, dp, masks, metrics and the per-cell words)."""
    ld1 = (spec["idm"] + 2 * spec["nbdy"] + 3) // 4 * 4
    sl = ld1 * (spec["jdm"] + 2 * spec["nbdy"])
    return sl * spec["kdm"] * (3 * spec["ntr"] * 4 + 2 * 4 + 8) + sl * (1 + 8 + 8 + 8)


def run_c4(args, wl, dev):
    """Combined workload: FP32-mixed FCT2 and MPDATA (the precision form)
    over 48 basins advanced in resident waves (each wave: load, then all
    steps replayed from a 10-step CUDA graph).  The error against the FP64
    form, the content change and the new-extrema check come from one step of
    the smallest basin; the FP64 form's rate from the same basin; the CPU
    baseline from the oracle on that basin with 4 layers."""
    import torch

    import hycadv

    t_start = time.perf_counter()
    members = c4_members(wl, args.layers)
    steps = args.c4_steps
    gsteps = min(10, steps)
    reps = max(1, steps // gsteps)
    geos = [member_geometry(m, wl) for m in members]
    specs = [g[2] for g in geos]
    free, _ = torch.cuda.mem_get_info(dev)
    budget = 0.75 * free - 24e9  # room for generating one basin in FP64
    waves, cur, tot = [], [], 0.0
    for i, sp in enumerate(specs):
        nbytes = mixed_state_bytes(sp)
        if cur and tot + nbytes > budget:
            waves.append(cur)
            cur, tot = [], 0.0
        cur.append(i)
        tot += nbytes
    waves.append(cur)
    ups_step = sum(sp["idm"] * sp["jdm"] * sp["kdm"] * sp["ntr"] for sp in specs)
    peak, peak_kind = peak_hbm()
    small = min(range(len(specs)), key=lambda i: specs[i]["idm"] * specs[i]["jdm"])
    schemes = {"fct2": 2, "mpdata": 1}
    res = {}
    for name, adv in schemes.items():
        # accuracy on the smallest basin: FP64 ensemble vs FP32-mixed, one step from the same inputs
        acc = {}
        refs = {}
        for prec in ("fp64", "mixed"):
            ens = hycadv.Ensemble([specs[small]], precision=prec)
            ens.set_posdef(0, 0, 256.0)
            bounds = load_member(ens, 0, members[small], geos[small], wl, dev)
            ens.tune(adv, wl["delt1"])
            sp = specs[small]
            c_old = [ens.content(0, q, "old", wl["delt1"]) for q in range(sp["ntr"])]
            ens.step(adv, wl["delt1"], 1)
            b, masks, _ = geos[small]
            sea = sea_mask(b, masks, dev)
            buf = torch.empty((sp["kdm"], b.ld2, b.ld1), dtype=torch.float64, device=dev)
            per = []
            for q in range(sp["ntr"]):
                ens.get(0, "cur", buf, s0=q * sp["kdm"], ns=sp["kdm"])
                new = buf[:, sea].clone()
                lo, hi = bounds[q]
                r = {"content_change_one_step": abs(ens.content(0, q, "cur", wl["delt1"]) - c_old[q]) / abs(c_old[q]),
                     "new_extrema_rel": float(max(lo - new.min(), new.max() - hi, 0.0)) / max(abs(lo), abs(hi))}
                if prec == "fp64":
                    refs[q] = new
                else:
                    d = new - refs[q]
                    scale = float(refs[q].abs().max())
                    r["max_rel_err_vs_fp64"] = float(d.abs().max()) / scale
                    r["rms_rel_err_vs_fp64"] = float(d.pow(2).mean().sqrt()) / scale
                per.append(r)
            if prec == "fp64":  # the FP64 form's rate on this basin
                ens.step(adv, wl["delt1"], 3, graph=True)
                torch.cuda.synchronize(dev)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                st = torch.cuda.current_stream(dev)
                e0.record(st)
                ens.step(adv, wl["delt1"], 3, graph=True)
                e1.record(st)
                torch.cuda.synchronize(dev)
                acc["fp64_rate_smallest_basin"] = sp["idm"] * sp["jdm"] * sp["kdm"] * sp["ntr"] * 3 / (
                    e0.elapsed_time(e1) / 1e3)
            acc[prec] = per
            ens.close()
            del ens, buf
            torch.cuda.empty_cache()
        refs.clear()
        # throughput over all basins, wave by wave
        t_ms, t_ups, load_s, tile, nq, clk_all = 0.0, 0.0, 0.0, None, None, []
        for wv in waves:
            ens = hycadv.Ensemble([specs[i] for i in wv], precision="mixed")
            for j in range(len(wv)):
                ens.set_posdef(j, 0, 256.0)
            t0 = time.perf_counter()
            for j, i in enumerate(wv):
                load_member(ens, j, members[i], geos[i], wl, dev)
            torch.cuda.synchronize(dev)
            torch.cuda.empty_cache()
            load_s += time.perf_counter() - t0
            if tile is None:
                tx, ty, _ = ens.tune(adv, wl["delt1"])
                tile, nq = (tx, ty), ens.option("strip_tracers")
            else:
                ens.set_tile(*tile)
                ens.set_strip_tracers(nq)
            ens.step(adv, wl["delt1"], gsteps, graph=True)  # capture + warm-up
            torch.cuda.synchronize(dev)
            st = torch.cuda.current_stream(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with ClockSampler(0) as clk:
                e0.record(st)
                for _ in range(reps):
                    ens.step(adv, wl["delt1"], gsteps, graph=True)
                e1.record(st)
                torch.cuda.synchronize(dev)
            clk_all.append(clk.summary())
            t_ms += e0.elapsed_time(e1)
            t_ups += sum(specs[i]["idm"] * specs[i]["jdm"] * specs[i]["kdm"] * specs[i]["ntr"] for i in wv) * gsteps * reps
            ens.close()
            del ens
            torch.cuda.empty_cache()
        rate = t_ups / (t_ms / 1e3)
        nbytes = sum(sp["idm"] * sp["jdm"] * sp["kdm"] * sp["ntr"] *
                     (bytes_per_update(4, 4, 8, sp["ntr"], sp["kdm"]) - (4 if adv == 1 else 0)) for sp in specs)
        ach = nbytes * (t_ups / ups_step) / (t_ms / 1e3) / 1e9
        res[name] = {"value": rate, "unit": UNIT, "ms_per_step_all_basins": t_ms / (gsteps * reps), "tile": list(tile),
                     "tracers_per_pass": nq, "achieved_GBs": ach, "frac_of_measured_hbm": ach / peak,
                     "waves": len(waves), "load_seconds": load_s, "steps_per_wave": gsteps * reps,
                     "accuracy_smallest_basin": acc, "clocks": clk_all[0]}
    # CPU baseline: the oracle on the smallest basin, 4 layers, T, S + 8 tracers
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        from oracle import oracle

        from hycadv import synth

        m = members[small]
        b, masks, _ = geos[small]
        sc, si = b.metrics()
        g = oracle.Grid(b.depth, sc, si, nbdy=b.nbdy, threads=threads)
        c = synth.build_case(b, g.masks, kdm=4, ntracr=8, seed=m["seed"], courant=wl["courant"], delt1=wl["delt1"],
                             device=dev)
        h = {k: getattr(c, k).cpu().numpy().copy() for k in ("temp", "saln", "th3d", "uflx", "vflx", "dp", "tracer")}
        del c
        import numpy as np

        tf = np.zeros(8, np.int32)
        n, t0 = 0, time.perf_counter()
        while n < 2 or time.perf_counter() - t0 < args.cpu_seconds:
            n += 1
            mm, nn = ((n + 1) % 2) + 1, (n % 2) + 1
            g.tsadvc(mm, nn, temp=h["temp"], saln=h["saln"], th3d=h["th3d"], uflx=h["uflx"], vflx=h["vflx"],
                     dp=h["dp"], delt1=wl["delt1"], advtyp=2, tracer=h["tracer"], trcflg=tf, nstep=n)
        dt = time.perf_counter() - t0
        cpu = {"value": b.nx * b.ny * 4 * 10 * n / dt, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"smallest basin {b.nx}x{b.ny}, 4 of 41 layers, T, S + 8 tracers, FCT2, {n} steps"}
    head = res["fct2"]
    desc = (f"c4: {len(members)} closed basins 800x600..3000x2000, kdm {members[0]['kdm']}, T, S + 8 passive tracers, "
            f"FP32-mixed FCT2 and MPDATA, max Courant {wl['courant']}, delt1 {wl['delt1']} s, {steps} steps per basin, "
            f"{len(waves)} resident waves")
    line = {"metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": gsteps,
            "ms_per_step": head["ms_per_step_all_basins"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-mixed", "data": "synthetic (seeded generator, HYCOM units/layout)",
            "impl": "ensemble-c4",
            "config": {"workload": desc, "form": "mixed", "updates_per_step": ups_step,
                       "l2": "inputs larger than L2 (state resident in HBM)"},
            "roofline": {"bound": "hbm", "achieved": head["achieved_GBs"], "peak": peak, "unit": "GB/s",
                         "frac": head["frac_of_measured_hbm"], "traffic": None, "peak_kind": peak_kind},
            "cpu_baseline": cpu, "clocks": head["clocks"], "forms": res, "wall_seconds": time.perf_counter() - t_start}
    print(json.dumps(line), flush=True)
    return 0


def config_of(args, wl, form):
    kind = "periodic-x" if wl["periodic"] else "closed"
    return {"workload": f"{args.workload}: {kind} basin {wl['nx']}x{wl['ny']}x{wl['kdm']}, T+S, "
                        f"{SCHEME_NAMES[args.advtyp]} (advtyp={args.advtyp}), max Courant {wl['courant']}, "
                        f"delt1 {wl['delt1']} s",
            "form": form, "updates_per_step": wl["nx"] * wl["ny"] * wl["kdm"] * 2,
            "l2": "inputs larger than L2 (state resident in HBM, >20 GB)" if args.workload == "c1"
            else "small case, fits in L2", "parallelism": "independent basin replica per GPU (replicas only)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="c1", choices=sorted(WORKLOADS))
    ap.add_argument("--advtyp", type=int, default=2, choices=[0, 1, 2, 4])
    ap.add_argument("--layers", type=int, default=0, help="override kdm (smaller profiling case)")
    ap.add_argument("--form", default="mixed", choices=sorted(ENS_FORMS),
                    help="headline form (ensemble API): mixed = the precision form (FP32 fluxes, limiter and "
                         "update; FP64 thickness prep and dp), mixed-fp32prep = the same with the thickness "
                         "factors in compensated FP32, fp64 = the FP64 form")
    ap.add_argument("--forms", default="tsadvc,tsadvc-fct4,tsadvc-mpdata,tsadvc-full,tsadvc-btrmas,cnuity,fp64,"
                                       "mixed-fp32prep,fp64-fct4,mixed-fct4,fp64-mpdata,mixed-mpdata,mixed-diff,c3",
                    help="forms measured beside the headline (tsadvc[-fct4|-mpdata|-pcm] = FP64 plain through "
                         "hyc_tsadvc, FCT2 unless named; tsadvc-full = asselin_save + tsadvc + its "
                         "diffusion + asselin_filter; cnuity = the continuity equation; fp64[-fct4|-mpdata], "
                         "mixed[-fp32prep|-fct4|-mpdata] = the ensemble API, FCT2 unless named; c3 = the "
                         "96-basin batched workload, FP64 and mixed)")
    ap.add_argument("--e2e-steps", type=int, default=6)
    ap.add_argument("--c4-steps", type=int, default=100, help="c4: steps per basin")
    ap.add_argument("--tile", default="", help="mixed forms: fixed tile 'tx,ty,tracers_per_pass' instead of the tuner")
    ap.add_argument("--ref-layers", type=int, default=0, help="layers in the CPU sample (0: all of the workload's)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--ens-forms", default="fp64,mixed-fp32prep,mixed",
                    help="c2/c3: ensemble forms to run, fp64 first")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.ref_layers <= 0:
        args.ref_layers = args.layers or WORKLOADS[args.workload].get("kdm", 41)
    args.tile = tuple(int(x) for x in args.tile.split(",")) if args.tile else None
    wl = dict(WORKLOADS[args.workload])
    if args.layers > 0:
        wl["kdm"] = args.layers
    if args.impl == "reference":
        return reference_arm(args, wl)

    import torch

    if args.workload in ("c2", "c3", "c4"):
        import build as hbuild

        hbuild.build()
        if args.workload == "c4":
            return run_c4(args, wl, torch.device("cuda:0"))
        return run_ensemble_workload(args, wl, None)
    ws, rank, local = dist_setup()
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    torch.cuda.set_device(local)
    dev = torch.device(f"cuda:{local}")

    import build as hbuild

    hbuild.build()
    t_start = time.perf_counter()
    b, masks, nreg, case = make_workload(wl, dev)
    sc, si = b.metrics()
    kdm = wl["kdm"]
    stream = torch.cuda.current_stream(dev)
    spec = dict(idm=b.nx, jdm=b.ny, kdm=kdm, nbdy=b.nbdy, nreg=nreg, ntr=2, ip=masks["ip"], iu=masks["iu"],
                iv=masks["iv"], scp2=sc, scp2i=si)
    others = [f for f in args.forms.split(",") if f]
    # sea-only count beside the dense interior one (interior cells with ip = 1)
    nb = b.nbdy
    sea_cells = int((np.asarray(masks["ip"])[nb:nb + b.ny, nb:nb + b.nx] != 0).sum())
    tsadvc = None
    if "tsadvc" in others:
        tsadvc = run_tsadvc_fp64(args, wl, b, masks, nreg, sc, si, case, dev, stream, dist, local)
    schemes = {}
    for f, adv in (("tsadvc-fct4", 4), ("tsadvc-mpdata", 1), ("tsadvc-pcm", 0)):
        if f in others:
            schemes[f] = run_tsadvc_fp64(args, wl, b, masks, nreg, sc, si, case, dev, stream, dist, local, adv)
    if "tsadvc-btrmas" in others:
        schemes["tsadvc-btrmas"] = run_tsadvc_fp64(args, wl, b, masks, nreg, sc, si, case, dev, stream, dist, local,
                                                   2, btrmas=True)
    if "tsadvc-full" in others:
        schemes["tsadvc-full"] = run_tsadvc_fp64(args, wl, b, masks, nreg, sc, si, case, dev, stream, dist, local,
                                                 2, full=True)
    if "cnuity" in others:
        schemes["cnuity"] = run_cnuity(args, wl, b, masks, nreg, sc, si, case, dev, stream, dist, local)
    ens_forms = [f for f in others if f in ENS_FORMS and f != args.form]
    # the FP64 references of the error checks run first
    ens_forms = [f for f in ens_forms if ENS_FORMS[f][0] == "fp64"] + [f for f in ens_forms if ENS_FORMS[f][0] != "fp64"]
    ens_forms = ens_forms + [args.form]
    forms = run_ensemble_forms(args, wl, b, masks, spec, case, dev, stream, dist, local, ens_forms)
    head = forms[args.form]

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, wl, b, spec, case, args.form, head["tile"], head["tracers_per_pass"], dev, stream, dist)
    del case
    torch.cuda.empty_cache()

    c3 = None
    if "c3" in others:  # the batched workload: FP64 (3 graph steps) and the precision form (K steps)
        c3 = ensemble_workload(args, dict(WORKLOADS["c3"]), "c3", dev, dist, ["fp64", "mixed"], fp64_steps=3)
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, desc, n, _ = run_cpu_sample(wl, nlayers=args.ref_layers, min_seconds=args.cpu_seconds, steps_max=20,
                                          warmup=1, advtyp=args.advtyp, threads=threads, gen_device=dev,
                                          min_steps=2)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc}

    if rank == 0:
        peak, peak_kind = peak_hbm()
        prec = ENS_FORMS[args.form][0]
        key = TRAFFIC_KEY.get(args.form)
        roof = {"bound": "hbm", "achieved": head["achieved_GBs"], "peak": peak, "unit": "GB/s",
                "frac": head["frac_of_measured_hbm"],
                "traffic": profile_traffic(f"{key}_{args.workload}") if key else None,
                "peak_kind": peak_kind, "kernel": head["kernel"],
                "algorithmic_bytes_per_update": head["algorithmic_bytes_per_update"],
                "avg_launch_ms": head["ms_per_step"], "tile": head["tile"],
                "tracers_per_pass": head["tracers_per_pass"]}
        others_out = {k: v for k, v in forms.items() if k != args.form}
        for f, r in schemes.items():
            others_out[f"fp64-{f}"] = r
        if tsadvc:
            others_out["fp64-tsadvc"] = tsadvc
            head["speedup_vs_fp64_tsadvc"] = head["value"] / tsadvc["value"]
        if c3:
            others_out["c3"] = c3
        # the specification's conservation target against the headline's one-step content change
        cc = head.get("content_change_one_step") or {}
        head["conservation"] = {
            "target_rel_per_step": 1e-13, "max_rel_change_one_step": max(cc.values()) if cc else None,
            "met": bool(cc) and max(cc.values()) <= 1e-13,
            "note": "FP32 tracer storage rounds each cell's content by up to 6e-8 relative; the FP64 forms "
                    "conserve to round-off" if prec == "mixed" else "FP64 form"}
        # one compact line of the figures the forms below hold in full
        summary = {f: round(r["value"] / 1e9, 2) for f, r in others_out.items()
                   if isinstance(r, dict) and "value" in r}
        if c3:
            for f, r in c3["forms"].items():
                summary[f"c3-{f}"] = round(r["value"] / 1e9, 2)
                summary[f"c3-{f}-frac_hbm"] = round(r["frac_of_measured_hbm"], 3)
        line = {
            "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-mixed" if prec == "mixed" else "f64",
            "data": "synthetic (seeded generator, HYCOM units/layout)",
            "config": dict(config_of(args, wl, f"ensemble-{args.form}"), tile=head["tile"],
                           tracers_per_pass=head["tracers_per_pass"],
                           sea_updates_per_step=sea_cells * wl["kdm"] * 2),
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": args.steps,
            "clocks": head["clocks"], "gupdates_per_s": summary,
            "headline": {k: v for k, v in head.items() if k != "clocks"},
            "forms": others_out, "wall_seconds": time.perf_counter() - t_start,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
