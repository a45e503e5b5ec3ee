#!/usr/bin/env python
"""Benchmark: FWI shot-gradients/s and Gcell-updates/s on one GB300.

Default workload: batched acoustic FWI gradient with FP32 stencils and FP64
misfit/gradient accumulation, 1000 x 500 cells (PML 40 inside), h = 10 m,
dt = 0.8 ms, 3000 steps, 64 shots with 15 Hz Ricker sources and 500 receivers
each, forward checkpoints every 100 steps, seeded folded-layer model (synthetic
data: observed traces are simulated on the true model, the gradient is taken at
a smoothed start model).  One step = one full gradient of all shots (forward,
misfit, checkpointed adjoint, gradient assembly) with everything resident in HBM.

Also reported: the plain FP64 path on the same per-shot geometry (one shot per
call, no batching), the end-to-end rate through the C ABI with host buffers,
the roofline of the dominant kernel from CUDA events recorded inside the time
loops, SM clocks sampled during the timed region, and the CPU baseline.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FWI shot-gradients/s & Gcell-updates/s, FP32-batched vs FP64-plain, 1 GB300"
UNIT = "shot-gradients/s"

# algorithmic bytes per interior cell-step (each array counted once per step)
BYTES = {
    ("fwd", "f32"): 36,   # increment form: read u, d, phi, psi, c; write u', d', phi', psi'
    ("fwd", "f64"): 64,   # read w, w_old, phi, psi, c; write u, phi', psi'

    ("adj", "f32"): 52,   # adjoint state 32 + forward w 4 + FP64 grad_c RMW 16
    ("adj", "f64"): 88,   # 64 + 8 + 16
}


# DRAM bytes (read + write) of one step of each kernel on the bench geometry
# at 16 shots, from ncu --set full captures of both launches of a step
TRAFFIC_16SHOT = {"k_ac_fwd": 148.9e6, "k_ac_adj": 245.3e6}


def workload(nstep=3000, nshots=64, seed=1234):
    """The C3 workload (adseismic_gb300.configs.c3_batched)."""
    import __graft_entry__ as g

    ads = g.load_package()
    from adseismic_gb300 import configs

    cfg, shots, vp_true, vp0 = configs.c3_batched(nshots=nshots, nstep=nstep, seed=seed)
    return ads, cfg, shots, vp_true, vp0, np.random.default_rng(seed)


class ClockSampler:
    """nvidia-smi samples during the timed region (read-only queries)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, n in enumerate(names):
                if len(r) > 4 + k and r[4 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_sample(cfg, shot, vp, steps, reps=1, use_ref=False):
    """Acoustic gradient of one shot over a bounded number of steps on one core:
    the oracle port, or (use_ref) the reference's own compiled CPU operators
    driven by the restated loop.  Returns seconds per run."""
    import oracle

    oracle.build(ref=False)
    MX, MY, h, dt = cfg["MX"], cfg["MY"], cfg["h"], cfg["dt"]
    sx, ty = oracle.acoustic_pml(MX, MY, h, h, cfg["npml"], cfg["vp_ref"])
    srcv = np.asarray(shot["srcv"])[:steps]
    obs = np.zeros((steps + 1, len(shot["rcvi"])))
    best = math.inf
    for _ in range(reps):
        t0 = time.perf_counter()
        oracle.acoustic_gradient(MX, MY, steps, dt, h, h, sx, ty, vp.reshape(-1), shot["srci"],
                                 shot["srcj"], srcv, shot["rcvi"], shot["rcvj"], obs,
                                 use_ref=use_ref)
        best = min(best, time.perf_counter() - t0)
    return best


def _cpu_worker(args):
    cfg, shot, vp, steps, use_ref = args
    return cpu_sample(cfg, shot, vp, steps, use_ref=use_ref)


def cpu_baseline(cfg, shots, vp, nstep, cores=1, steps=40, use_ref=False):
    """Shot-gradients/s on `cores` processes (one shot each), from a bounded
    sample of `steps` time steps scaled linearly to nstep."""
    if cores == 1:
        t = cpu_sample(cfg, shots[0], vp, steps, use_ref=use_ref)
    else:
        import multiprocessing as mp

        ctx = mp.get_context("spawn")
        with ctx.Pool(cores) as pool:
            ts = pool.map(_cpu_worker, [(cfg, shots[k % len(shots)], vp, steps, use_ref)
                                        for k in range(cores)])
        t = max(ts)
    per_shot = t * (nstep - 1) / (steps - 1)
    return cores / per_shot, t


def run_reference(args):
    """--impl reference: the reference's CPU operators (compiled from the
    reference checkout when present, else the oracle's bit-identical port) timed
    on all host cores over bounded samples of the same workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle

    ads, cfg, shots, vp_true, vp0, _ = workload()
    cores = os.cpu_count() or 1
    use_ref = oracle.ref_available()
    kind = "reference" if use_ref else "port"
    steps = 40
    vals = []
    for k in range(args.warmup + args.steps):
        v, t = cpu_baseline(cfg, shots, vp0, 3000, cores=cores, steps=steps, use_ref=use_ref)
        if k >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "acoustic FWI gradient 1000x500 (PML 40), 3000 steps, "
                               "64 shots x 500 receivers"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"{cores} shots in parallel, {steps} of 3000 steps each "
                                   "(forward + full-history adjoint), scaled linearly"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def _timed(fn, steps, warmup):
    """Device time per call (ms) of `fn` on the current stream."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def _line(metric, value, unit, args, ms, dtype, workload, extra):
    out = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
           "config": {"workload": workload}}
    out.update(extra)
    print(json.dumps(out))


def measure_c1(steps, warmup, with_cpu=True):
    """Plain FP64 acoustic forward (C1): 200x200 interior plus a 20-cell PML, h = 10 m,
    dt = 1 ms, 1000 steps, one 10 Hz Ricker source 20 cells below the PML, 200
    receivers 5 cells below it (the reference CPU operators' own configuration).
    Returns the measured figures (value in Gcell-updates/s)."""
    import torch
    import __graft_entry__ as g

    ads = g.load_package()
    from adseismic_gb300 import configs

    cfg, shot, vp = configs.c1_forward()
    NX, NY, npml, T, h, dt = cfg["MX"], cfg["MY"], cfg["npml"], cfg["nstep"], cfg["h"], cfg["dt"]
    plan = ads.AcousticPlan(NX, NY, h, h, dt, [shot], npml=npml, vp_ref=cfg["vp_ref"],
                            precision="f64")
    vdev = torch.tensor(vp, device="cuda")
    ms = _timed(lambda: plan.forward(vdev), steps, warmup)
    cells = NX * NY * (T - 1)
    vh = torch.tensor(vp).pin_memory()
    th = torch.empty(plan.trace_count, dtype=torch.float64).pin_memory()

    def e2e():
        vdev.copy_(vh, non_blocking=True)
        th.copy_(plan.forward(vdev), non_blocking=True)

    ms_e2e = _timed(e2e, steps, 1)
    out = {"value": cells / (ms / 1e3) / 1e9, "unit": "Gcell-updates/s", "ms_per_step": ms,
           "dtype": "f64",
           "workload": "acoustic forward 240x240 (200x200 + PML 20), 1000 steps, 1 shot, "
                       "200 receivers",
           "e2e": {"value": cells / (ms_e2e / 1e3) / 1e9, "unit": "Gcell-updates/s",
                   "h2d_bytes_per_step": vp.size * 8,
                   "d2h_bytes_per_step": plan.trace_count * 8},
           "gpu_launches": int(plan.launches_forward)}
    plan.close()
    if with_cpu:
        import oracle

        oracle.build(ref=False)
        sx, ty = oracle.acoustic_pml(NX, NY, h, h, npml, cfg["vp_ref"])
        t0 = time.perf_counter()
        oracle.acoustic_forward(NX, NY, T, dt, h, h, sx, ty, vp.reshape(-1), shot["srci"],
                                shot["srcj"], shot["srcv"], shot["rcvi"], shot["rcvj"],
                                use_ref=oracle.ref_available())
        t_cpu = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": cells / t_cpu / 1e9, "unit": "Gcell-updates/s",
                               "cores": 1,
                               "kind": "reference" if oracle.ref_available() else "port",
                               "sample": "the full forward, one core"}
    return out


def run_acoustic_fwd_f64(args):
    r = measure_c1(args.steps, args.warmup)
    _line("acoustic forward Gcell-updates/s, plain FP64 drop-in", r["value"], r["unit"], args,
          r["ms_per_step"], "f64", r["workload"],
          {k: r[k] for k in ("e2e", "cpu_baseline", "gpu_launches")})


def measure_c2(steps, warmup, nstep=2000, rows=0):
    """Plain FP64 acoustic FWI gradient (C2): 400x400 incl. PML 30, nstep steps, 8 shots
    20 cells below the PML at the centres of 8 equal segments, one receiver per
    interior column 5 cells below the PML, observed data from the true model,
    gradient at a Gaussian-smoothed (20 cells) start model."""
    import torch
    import __graft_entry__ as g

    ads = g.load_package()
    from adseismic_gb300 import configs

    cfg, shots, vt, v0 = configs.c2_fwi(nstep=nstep)
    NX, NY, T = cfg["MX"], cfg["MY"], cfg["nstep"]
    # rows > 0 fixes the item tiling (the autotuner's timings mean nothing under a profiler)
    plan = configs.acoustic_plan(ads, cfg, shots, "f64", autotune=rows <= 0,
                                 rows_per_thread=max(rows, 0))
    obs = plan.forward(torch.tensor(vt, device="cuda")).clone()
    vdev = torch.tensor(v0, device="cuda")
    ms = _timed(lambda: plan.gradient(vdev, obs), steps, warmup)
    cells = 2 * len(shots) * NX * NY * (T - 1)
    out = {"value": len(shots) / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "dtype": "f64",
           "workload": f"acoustic FWI gradient 400x400 (PML 30), {T} steps, 8 shots",
           "gcell_updates_per_s": cells / (ms / 1e3) / 1e9,
           "gpu_launches": int(plan.launches_gradient),
           "rows_per_warp": dict(zip(("fwd", "adj", "fwd_pml", "adj_pml"), plan.rows))}
    plan.close()
    return out


def run_fwi_f64(args):
    r = measure_c2(args.steps, args.warmup, nstep=args.nstep if args.nstep != 3000 else 2000,
                   rows=args.rows)
    _line("FWI shot-gradients/s, FP64 plan", r["value"], r["unit"], args,
          r["ms_per_step"], "f64", r["workload"],
          {k: r[k] for k in ("gcell_updates_per_s", "gpu_launches", "rows_per_warp")})


def elastic_workload(ads, nshots=32, T=4000):
    from adseismic_gb300 import configs

    return configs.c4_elastic(nshots=nshots, T=T)


def elastic_measure(steps, warmup, nshots=32, T=4000, with_rel_err=True, autotune=True,
                    adjoint_passes=0, ckpt_every=100, resident_pct=92):
    """Elastic CPML FWI gradient w.r.t. lambda, mu, rho (C4): 600x300 incl. CPML
    30, T steps, FP32 stencils with FP64 accumulation, explosive shots (sigma_xx
    and sigma_yy, 10 Hz Ricker), 300 two-component receivers.  Returns the
    measured figures as a dict (value in shot-gradients/s)."""
    import torch
    import __graft_entry__ as g

    ads = g.load_package()
    from adseismic_gb300 import configs

    p, shots, lam, mu, rho = elastic_workload(ads, nshots=nshots, T=T)
    t = lambda a: torch.tensor(a.reshape(-1), device="cuda")
    # the last checkpoint segments' adjoint inputs stay resident in HBM (up to
    # 92% of the memory free after the plan's other buffers)
    plan = ads.ElasticPlan(p, shots, precision="f32", ckpt_every=ckpt_every,
                           resident_segments=-1 if resident_pct < 0 else 0,
                           resident_mem_pct=max(resident_pct, 0), autotune=autotune,
                           adjoint_passes=adjoint_passes)
    obs = plan.forward(t(lam), t(mu), t(rho)).clone()
    l0, m0, r0 = (t(a) for a in configs.c4_start_model(lam, mu, rho))
    ms = _timed(lambda: plan.gradient(l0, m0, r0, obs), steps, warmup)
    n = len(shots)
    cells = 2 * n * p.NX * p.NY * p.NSTEP
    # roofline: algorithmic bytes per cell-update, forward (13 + 16 f_pml) x 4 B
    # (5 fields read + written, lambda / mu / rho, 8 memory variables in CPML
    # cells); the forward step that stores the adjoint's inputs writes 5 more
    # fields (+20 B); adjoint step = forward + 20 B (the stored strains and
    # accelerations) + 24 B (the FP32 lambda / mu / rho partials, read and
    # written)
    f_pml = 1 - (p.NX - 2 * p.NPOINTS_PML) * (p.NY - 2 * p.NPOINTS_PML) / (p.NX * p.NY)
    b_fwd = (13 + 16 * f_pml) * 4
    b_adj = b_fwd + 20 + 24
    prof = plan.profile(l0, m0, r0)
    peak, peak_kind = measured_peak()
    fwd_ms, st_ms = prof["step"][0], prof["step_store"][0]
    adj_ms = prof["adj1"][0] + prof["adj2"][0] + prof["adj3"][0]
    c1 = prof["step"][1]
    adj_name = ("k_el_adj_rows" if prof["adj2"][0] == 0 else
                "k_el_adj1_rows+k_el_adj2_rows+k_el_adj3_rows")
    groups = {
        "k_el_step_rows": (fwd_ms, b_fwd * c1),
        "k_el_step_rows (storing)": (st_ms, (b_fwd + 20) * c1),
        adj_name: (adj_ms, b_adj * c1),
    }
    kern = {k: {"ms_per_step": round(tt, 4), "achieved_gbs": round(b / (tt / 1e3) / 1e9, 1),
                "frac": round(b / (tt / 1e3) / 1e9 / peak, 4)} for k, (tt, b) in groups.items()}
    kern.update({k: {"ms_per_launch": round(v[0], 4)} for k, v in prof.items()})
    dom = adj_name
    tt, b = groups[dom]
    # the whole gradient: algorithmic bytes of all its steps over its measured
    # time (forward steps without / with stores, the recompute, the adjoint)
    K, res = ckpt_every, plan.resident_segments
    nseg = -(-p.NSTEP // K)
    cps = n * p.NX * p.NY
    n_store = min(res * K, p.NSTEP) + max(nseg - res, 0) * K
    job_b = cps * (b_fwd * max(p.NSTEP - res * K, 0) + (b_fwd + 20) * n_store + b_adj * p.NSTEP)
    job = {"bytes": job_b, "achieved_gbs": round(job_b / (ms / 1e3) / 1e9, 1),
           "frac": round(job_b / (ms / 1e3) / 1e9 / peak, 4),
           "steps": {"forward": p.NSTEP, "storing": n_store, "adjoint": p.NSTEP}}
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(b / (tt / 1e3) / 1e9, 1),
                "peak": peak, "unit": "GB/s", "frac": round(b / (tt / 1e3) / 1e9 / peak, 4),
                "peak_source": peak_kind, "traffic": None, "bytes_per_launch": b,
                "bytes_per_cell": {"forward": round(b_fwd, 2), "forward_storing": round(b_fwd + 20, 2),
                                   "adjoint": round(b_adj, 2), "f_pml": round(f_pml, 4)},
                "kernels": kern, "gradient": job}
    out = {"value": n / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": steps,
           "warmup": warmup, "dtype": "f32",
           "workload": f"elastic CPML gradient {p.NX}x{p.NY} (CPML {p.NPOINTS_PML}), "
                       f"{p.NSTEP} steps, {n} explosive shots x 300 two-component receivers, "
                       f"checkpoints every {ckpt_every}, the last {plan.resident_segments} of "
                       f"{-(-p.NSTEP // ckpt_every)} segments resident in HBM",
           "gcell_updates_per_s": cells / (ms / 1e3) / 1e9, "roofline": roofline,
           "device_bytes": plan.device_bytes, "gpu_launches": int(plan.launches_gradient),
           "tiling": {"rows_per_adjoint_strip": plan.rows_per_warp,
                      "rows_per_fused_tile": plan.rows_per_tile, "autotuned": bool(autotune)}}
    plan.close()
    if with_rel_err:
        out["rel_err"] = elastic_rel_err(ads, p, [shots[3], shots[n // 2 + 4]], lam, mu, rho,
                                         (l0, m0, r0))
    return out


def elastic_rel_err(ads, p, pick, lam, mu, rho, start):
    """FP32 plan against the FP64 plan (pinned to the oracle at 1e-12) on `pick`:
    rel-L2 of each gradient field and of every receiver trace."""
    import torch
    from adseismic_gb300 import configs

    t = lambda a: torch.tensor(a.reshape(-1), device="cuda")
    p64 = ads.ElasticPlan(p, pick, precision="f64", ckpt_every=100)
    obs = p64.forward(t(lam), t(mu), t(rho)).clone()
    o64 = p64.gradient(*start, obs, want_traces=True)
    torch.cuda.synchronize()
    p64.close()
    p32 = ads.ElasticPlan(p, pick, precision="f32", ckpt_every=100)
    o32 = p32.gradient(*start, obs.float(), want_traces=True)
    torch.cuda.synchronize()
    p32.close()
    rel = lambda a, b: float(torch.linalg.vector_norm(a.double() - b) / torch.linalg.vector_norm(b))
    nt = p.NSTEP + 1
    tr32, tr64 = o32[4].double().cpu().numpy(), o64[4].cpu().numpy()
    per, n0 = [], 0
    for s in pick:
        n = len(s["rcvi"])
        a = tr32[n0:n0 + n * nt].reshape(n, nt).T
        b = tr64[n0:n0 + n * nt].reshape(n, nt).T
        per.append(configs.per_trace_rel(a, b, n))
        n0 += n * nt
    per = np.concatenate(per)
    return {"grad_lambda": rel(o32[1], o64[1]), "grad_mu": rel(o32[2], o64[2]),
            "grad_rho": rel(o32[3], o64[3]), "traces": rel(o32[4], o64[4]),
            "trace_max": float(per.max()), "trace_median": float(np.median(per)),
            "traces_compared": int(per.size), "shots": len(pick),
            "reference": "FP64 plan, pinned to the oracle at rel-L2 1e-12"}


def acoustic_rel_err(ads, cfg, pick, vp_true, vp0):
    """The FP32 plan (the benchmark's settings) against the FP64 plan (pinned to
    the oracle at 1e-12) on the shots `pick`: rel-L2 of the gradient, of all
    traces and of every receiver trace (traces with signal, see per_trace_rel)."""
    import torch
    from adseismic_gb300 import configs

    vt = torch.tensor(vp_true, device="cuda")
    v0 = torch.tensor(vp0, device="cuda")
    p64 = configs.acoustic_plan(ads, cfg, pick, "f64", ckpt_every=100)
    obs = p64.forward(vt).clone()
    l64, g64, tr64 = p64.gradient(v0, obs, want_traces=True)
    torch.cuda.synchronize()
    p64.close()
    p32 = configs.acoustic_plan(ads, cfg, pick, "f32", ckpt_every=100, autotune=True)
    l32, g32, tr32 = p32.gradient(v0, obs.float(), want_traces=True)
    torch.cuda.synchronize()
    offs = p32.trace_offsets
    p32.close()
    rel = lambda a, b: float(torch.linalg.vector_norm(a.double() - b) / torch.linalg.vector_norm(b))
    a, b = tr32.double().cpu().numpy(), tr64.cpu().numpy()
    per = []
    for k, s in enumerate(pick):
        n = (s["nstep"] + 1) * len(s["rcvi"])
        per.append(configs.per_trace_rel(a[offs[k]:offs[k] + n], b[offs[k]:offs[k] + n],
                                         len(s["rcvi"])))
    per = np.concatenate(per)
    return {"grad": rel(g32, g64), "traces": rel(tr32, tr64), "trace_max": float(per.max()),
            "trace_median": float(np.median(per)), "traces_compared": int(per.size),
            "loss": abs(float(l32) - float(l64)) / float(l64), "shots": len(pick),
            "reference": "FP64 plan, pinned to the oracle at rel-L2 1e-12"}


def run_elastic_fwi(args):
    """The elastic C4 gradient as its own bench line."""
    nshots = args.shots if args.shots != 64 else 32
    T = args.nstep if args.nstep != 3000 else 4000
    r = elastic_measure(args.steps, args.warmup, nshots=nshots, T=T,
                        with_rel_err=not args.no_fp64, autotune=not args.no_elastic_autotune,
                        adjoint_passes=args.elastic_adjoint_passes,
                        ckpt_every=args.ckpt_every, resident_pct=args.resident_pct)
    _line("elastic FWI shot-gradients/s (FP32 stencils, FP64 accumulation)", r["value"],
          "shot-gradients/s", args, r["ms_per_step"], "f32", r["workload"],
          {k: r[k] for k in ("gcell_updates_per_s", "roofline", "device_bytes", "gpu_launches",
                             "rel_err", "tiling") if k in r})


def measure_c5(steps, warmup, nshots=128):
    """Uneven batched acoustic FWI gradient (C5): 4000 x 2000 model, 128 shots, each
    with its own window of 400-1200 columns (PML 40 inside), 200-1200 receivers
    and 2000-6000 steps drawn from the seed; FP32 stencils, FP64 accumulation."""
    import torch
    import __graft_entry__ as g

    ads = g.load_package()
    from adseismic_gb300 import configs

    cfg, shots, vt, v0 = configs.c5_uneven(nshots=nshots)
    MY = cfg["MY"]
    plan = configs.acoustic_plan(ads, cfg, shots, "f32", ckpt_every=100)
    obs = plan.forward(torch.tensor(vt, device="cuda")).clone()
    vdev = torch.tensor(v0, device="cuda")
    ms = _timed(lambda: plan.gradient(vdev, obs), steps, warmup)
    cells = 2 * sum(s["nx"] * MY * (s["nstep"] - 1) for s in shots)
    out = {"value": len(shots) / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "dtype": "f32",
           "workload": f"uneven acoustic FWI gradient on a 4000x2000 model, {len(shots)} shots, "
                       "windows 400-1200, 200-1200 receivers, 2000-6000 steps, PML 40 per window",
           "gcell_updates_per_s": cells / (ms / 1e3) / 1e9, "device_bytes": plan.device_bytes,
           "resident_segments": plan.resident_segments,
           "gpu_launches": int(plan.launches_gradient)}
    plan.close()
    return out


def run_fwi_uneven(args):
    r = measure_c5(args.steps, args.warmup, nshots=args.shots if args.shots != 64 else 128)
    _line("FWI shot-gradients/s & Gcell-updates/s, FP32-batched uneven shots", r["value"],
          r["unit"], args, r["ms_per_step"], "f32", r["workload"],
          {k: r[k] for k in ("gcell_updates_per_s", "device_bytes", "gpu_launches")})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="fwi-batched",
                    choices=["fwi-batched", "acoustic-fwd-f64", "fwi-f64", "elastic-fwi",
                             "fwi-uneven"])
    ap.add_argument("--shots", type=int, default=64)
    ap.add_argument("--nstep", type=int, default=3000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-elastic", action="store_true")
    ap.add_argument("--no-elastic-autotune", action="store_true")
    ap.add_argument("--no-configs", action="store_true")
    ap.add_argument("--rows", type=int, default=0,
                    help="fwi-f64: rows per warp of the step items instead of the autotuner")
    ap.add_argument("--elastic-adjoint-passes", type=int, default=0, choices=(0, 1, 3))
    # elastic-fwi workload only: checkpoint interval and the resident share of
    # the free device memory in percent (-1: no resident segments), for small
    # profiler captures
    ap.add_argument("--ckpt-every", type=int, default=100)
    ap.add_argument("--resident-pct", type=int, default=92)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    other = {"acoustic-fwd-f64": run_acoustic_fwd_f64, "fwi-f64": run_fwi_f64,
             "elastic-fwi": run_elastic_fwi, "fwi-uneven": run_fwi_uneven}
    if args.workload in other:
        return other[args.workload](args) or 0

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)

    ads, cfg, shots, vp_true, vp0, rng = workload(nstep=args.nstep, nshots=args.shots,
                                                  seed=1234 + rank)
    nstep, MX, MY = args.nstep, cfg["MX"], cfg["MY"]
    mk = lambda prec, sh, **kw: ads.AcousticPlan(MX, MY, cfg["h"], cfg["h"], cfg["dt"], sh,
                                                 npml=cfg["npml"], vp_ref=cfg["vp_ref"],
                                                 precision=prec, ckpt_every=100, **kw)
    t_setup = time.perf_counter()
    # the last checkpoint segments' wavefields stay resident in HBM (up to 92%
    # of the memory free after the plan's other buffers): the reverse sweep
    # recomputes only the others
    plan = mk("f32", shots, autotune=True, resident_mem_pct=92)
    vt = torch.tensor(vp_true, device=dev)
    v0 = torch.tensor(vp0, device=dev)
    obs = plan.forward(vt).clone()
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t_setup

    from adseismic_gb300.distributed import allreduce_loss_grad

    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        loss, grad = plan.gradient(v0, obs)
        if dist:
            allreduce_loss_grad(loss, grad)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    n0 = ads.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            loss, grad = plan.gradient(v0, obs)
            if dist:
                allreduce_loss_grad(loss, grad)
        e1.record(stream)
        torch.cuda.synchronize()
    launches = ads.launch_count() - n0
    ms = e0.elapsed_time(e1) / args.steps
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t)
    total_shots = args.shots * world
    value = total_shots / (ms / 1e3)
    cell_steps = sum(s["nx"] * MY * (s["nstep"] - 1) for s in shots) * world
    gcell = 2 * cell_steps / (ms / 1e3) / 1e9  # forward + adjoint updates per second
    timing = plan.profile(v0, obs)

    # roofline: kernels timed by CUDA events recorded inside the time loops
    peak, peak_kind = measured_peak()
    fwd_ms, fwd_n, fwd_cells = timing["forward"]
    rc_ms, rc_n, rc_cells = timing["recompute"]
    adj_ms, adj_n, adj_cells = timing["adjoint"]
    nseg = math.ceil((nstep - 1) / 100)
    # a step is two launches of each kernel (interior items, PML items); the
    # timed ranges hold whole steps, so per-launch means cover both
    cells_per_step = sum(s["nx"] * MY for s in shots)
    kern = {
        "k_ac_fwd": dict(ms_per_launch=fwd_ms / fwd_n, bytes=BYTES[("fwd", "f32")] * fwd_cells / fwd_n,
                         launches=fwd_n + rc_n * (nseg - plan.resident_segments),
                         launches_per_step=fwd_n / (fwd_cells / cells_per_step)),
        "k_ac_adj": dict(ms_per_launch=adj_ms / adj_n, bytes=BYTES[("adj", "f32")] * adj_cells / adj_n,
                         launches=adj_n * nseg,
                         launches_per_step=adj_n / (adj_cells / cells_per_step)),
    }
    for k, v in kern.items():
        v["achieved_gbs"] = v["bytes"] / (v["ms_per_launch"] / 1e3) / 1e9
        v["total_ms"] = v["ms_per_launch"] * v["launches"]
    dom = max(kern, key=lambda k: kern[k]["total_ms"])
    d = kern[dom]
    # DRAM read + write bytes of one step (both launches) from ncu --set full
    # captures of the same workload at 16 shots, scaled by the shots a step
    # processes here (traffic grows with the shot count), per launch like achieved
    per_shot_step = {"k_ac_fwd": TRAFFIC_16SHOT["k_ac_fwd"] / 16,
                     "k_ac_adj": TRAFFIC_16SHOT["k_ac_adj"] / 16}
    traffic = (round(per_shot_step[dom] * args.shots / d["launches_per_step"], -5)
               if MX == 1000 and MY == 500 and dom in per_shot_step else None)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(d["achieved_gbs"], 1),
                "peak": peak, "unit": "GB/s", "frac": round(d["achieved_gbs"] / peak, 4),
                "peak_source": peak_kind, "traffic": traffic,
                "bytes_per_launch": d["bytes"], "ms_per_launch": d["ms_per_launch"],
                "launches_per_step": round(d["launches_per_step"], 2),
                "kernels": {k: {"achieved_gbs": round(v["achieved_gbs"], 1),
                                "ms_per_launch": round(v["ms_per_launch"], 4),
                                "launches_per_step": round(v["launches_per_step"], 2),
                                "share_of_step": round(v["total_ms"] / ms, 3)}
                            for k, v in kern.items()}}
    # the whole gradient: algorithmic bytes of its forward, recompute and
    # adjoint cell-updates over its measured time
    rc_cu = rc_cells * max(nseg - plan.resident_segments, 0)
    job_b = (BYTES[("fwd", "f32")] * (cell_steps / world + rc_cu) +
             BYTES[("adj", "f32")] * cell_steps / world)
    roofline["gradient"] = {"bytes": job_b, "achieved_gbs": round(job_b / (ms / 1e3) / 1e9, 1),
                            "frac": round(job_b / (ms / 1e3) / 1e9 / peak, 4),
                            "cell_updates": {"forward": cell_steps // world, "recompute": rc_cu,
                                             "adjoint": cell_steps // world}}

    # e2e through the C ABI with host buffers (pinned), copies inside the timed region
    vp_host = torch.tensor(vp0).pin_memory()
    obs_host = obs.cpu().pin_memory()
    grad_host = torch.empty_like(vp_host).pin_memory()
    loss_host = torch.empty(1, dtype=torch.float64).pin_memory()
    vdev = torch.empty_like(v0)
    odev = torch.empty_like(obs)
    torch.cuda.synchronize()
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        vdev.copy_(vp_host, non_blocking=True)
        odev.copy_(obs_host, non_blocking=True)
        l, g = plan.gradient(vdev, odev)
        grad_host.copy_(g, non_blocking=True)
        loss_host.copy_(l.reshape(1), non_blocking=True)
        torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": args.shots / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": vp_host.numel() * 8 + obs_host.numel() * 4,
           "d2h_bytes_per_step": grad_host.numel() * 8 + 8}

    resident = plan.resident_segments
    plan.close()  # its resident wavefields free the memory the FP64 paths need

    # accuracy of the timed FP32 path: two of the shots against the FP64 plan
    rel_err = None
    if not args.no_fp64:
        rel_err = acoustic_rel_err(ads, cfg, [shots[0], shots[len(shots) // 2]], vp_true, vp0)
        rel_err["shot_indices"] = [0, len(shots) // 2]

    # plain FP64 on the same per-shot geometry, one shot per call
    fp64 = None
    if not args.no_fp64:
        p64 = mk("f64", shots[:1], autotune=True)
        o64 = p64.forward(vt).clone()
        p64.gradient(v0, o64)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        reps = 2
        for _ in range(reps):
            p64.gradient(v0, o64)
        b.record(stream)
        torch.cuda.synchronize()
        ms64 = a.elapsed_time(b) / reps
        t64 = p64.profile(v0, o64)
        fwd64 = t64["forward"]
        plan64 = {"value": 1e3 / ms64, "unit": UNIT, "ms_per_shot_gradient": ms64,
                  "gcell_updates_per_s": 2 * shots[0]["nx"] * MY * (nstep - 1) / (ms64 / 1e3) / 1e9,
                  "k_ac_fwd_f64_gbs": BYTES[("fwd", "f64")] * fwd64[2] / (fwd64[0] / 1e3) / 1e9,
                  "fp32_batched_over_this": value / world / (1e3 / ms64)}
        p64.close()
        # the plain FP64 drop-in: the reference's operator chain, one C-ABI call
        # per operator and step, full history on the device, one shot
        s0 = shots[0]
        prm = ads.AcousticPropagatorParams(NX=MX, NY=MY, NSTEP=nstep, DELTAX=cfg["h"],
                                           DELTAY=cfg["h"], DELTAT=cfg["dt"],
                                           NPOINTS_PML=cfg["npml"], vp_ref=cfg["vp_ref"],
                                           PropagatorKernel=1)  # the custom operators
        src = ads.AcousticSource(np.asarray(s0["srci"]), np.asarray(s0["srcj"]),
                                 np.asarray(s0["srcv"]))
        rcv = ads.AcousticReceiver(s0["rcvi"], s0["rcvj"])
        ads.dropin_loss_and_grad(prm, src, rcv, o64, vp0)
        torch.cuda.synchronize()
        a.record(stream)
        ads.dropin_loss_and_grad(prm, src, rcv, o64, vp0)
        b.record(stream)
        torch.cuda.synchronize()
        msd = a.elapsed_time(b)
        fp64 = {"value": 1e3 / msd, "unit": UNIT, "ms_per_shot_gradient": msd,
                "path": "FP64 drop-in operator chain (step, ScatterAdd, Gather and their "
                        "gradients per time step, full history), one shot",
                "gcell_updates_per_s": 2 * s0["nx"] * MY * (nstep - 1) / (msd / 1e3) / 1e9,
                "fp32_batched_over_fp64_plain": value / world / (1e3 / msd),
                "fp64_plan_one_shot": plan64}
        torch.cuda.empty_cache()

    # the elastic C4 gradient (32 shots, 4000 steps), measured in the same run
    elastic = None
    if not args.no_elastic and rank == 0:
        elastic = elastic_measure(min(args.steps, 3), min(max(args.warmup, 1), 3))
        torch.cuda.empty_cache()

    # the other configurations, briefly, in the same run
    other = None
    if not args.no_configs and rank == 0:
        other = {"C1": measure_c1(min(args.steps, 5), min(max(args.warmup, 1), 3),
                                  with_cpu=not args.no_cpu),
                 "C2": measure_c2(min(args.steps, 3), min(max(args.warmup, 1), 2))}
        torch.cuda.empty_cache()
        other["C5"] = measure_c5(min(args.steps, 2), 1)
        torch.cuda.empty_cache()

    cpu = None
    if not args.no_cpu and rank == 0:
        v, t = cpu_baseline(cfg, shots, vp0, nstep, cores=1, steps=100)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"one shot, 100 of {nstep} steps (forward + full-history adjoint, "
                         f"{t:.1f} s), scaled linearly to {nstep} steps"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"acoustic FWI gradient {MX}x{MY} (PML {cfg['npml']}), "
                                   f"{nstep} steps, {args.shots} shots x 500 receivers per GPU, "
                                   "15 Hz Ricker, folded-layer model, checkpoints every 100, "
                                   f"the last {resident} of {nseg} segments resident in HBM "
                                   "(no recompute)",
                       "precision": "FP32 stencils, FP64 misfit and gradient accumulation",
                       "l2": f"working set {plan.device_bytes / 1e9:.1f} GB per GPU >> 126 MB L2",
                       "parallelism": f"shots sharded over {world} GPU(s), gradient all-reduce"},
            "gcell_updates_per_s": gcell,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "rel_err": rel_err,
            "fp64_plain": fp64,
            "elastic": elastic,
            "configs": other,
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "loss": float(loss),
            "setup_s": t_setup,
        }
        print(json.dumps(line))
    plan.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
