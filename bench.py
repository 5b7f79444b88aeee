#!/usr/bin/env python3
"""Benchmark of the explicit hot path on one GB300 (or N replicas).

A *step* is one explicit cycle of the whole model (every element group ->
PARITH/ON assembly -> time step -> nodal update) with the model resident in
HBM.  ``value`` is element-updates/s (elements x cycles / device seconds,
CUDA events on the library's stream); ``e2e`` is the same metric through the
FORINT-level C-ABI call with host buffers (X, V uploaded and assembled
forces + STIFN downloaded every step).  The headline form is the plain FP64
path; the mixed FP32-element / FP64-nodal form is reported beside it.

``--impl reference`` times the reference algorithm's CPU path -- the CPU
restatement under oracle/ (the reference engine itself cannot be built
without a Fortran compiler) -- on all host cores, on the same workload.

Multi-GPU: replicas only (independent models, weak scaling, barrier and
max-over-ranks timing), launched by torchrun.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from openradioss_gb300 import model as M  # noqa: E402

WORKLOADS = {
    # square crash box of Belytschko-Tsay shells, 60x60 mm section, 300 mm
    # long, 308 x 390 = 120,120 elements, t = 1.2 mm, NPT = 5, Johnson-Cook,
    # seeded imperfection U[-0.1t, 0.1t], planar rigid wall hit at 15 m/s
    "crash_box_120k_jc": lambda: M.crash_box(n_side=77, n_len=390),
    # JC hexa block, 128^3 one-point hexas (2,097,152 elements), seeded
    # velocity 20 m/s + N(0, 0.5): the largest single-GPU hexa configuration.
    "hexa_block_128_jc": lambda: M.large_block(n=128),
    # steel bar impact, 20^3 LAW1 (the CPU-runnable case)
    "bar_impact_20_law1": lambda: M.bar_impact(n=20),
}
DEFAULT_WORKLOAD = "crash_box_120k_jc"
# full run length of each configuration (the "job")
JOB_CYCLES = {"crash_box_120k_jc": 20000, "hexa_block_128_jc": 2000, "bar_impact_20_law1": 1000}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 5 + i and s[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def reduce_max(x, device):
    """Max of a per-rank scalar over the process group (replica timing: the
    slowest rank sets the step time)."""
    import torch
    import torch.distributed as tdist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, world, seconds):
    """Whole-job throughput of N replicas: every rank processed
    units_per_rank units in the (max over ranks) time."""
    return world * units_per_rank / seconds


def element_bytes(model, prec):
    """Algorithmic DRAM bytes of one element-kernel launch over the model,
    and per node of one node-kernel launch, from the implemented arrays
    (each node record read once per pass: ideal reuse).  Returns
    (bytes per element, bytes per node, kernel key)."""
    nn = model.numnod
    er = 8 if prec == 0 else 4
    slot = 32 if prec == 0 else 16
    if model.hexa:
        ne = model.numels
        law = model.hexa[0].mat["mtn"]
        # reads NC, IADS (8 int32 each), OFF, SIG(6), QVIS (ER), EINT, RHO,
        # VOL0, EHOU (FP64), [PLA, EPSD]; node X4, V4 (32 B each)
        rd = 32 + 32 + er * (1 + 6 + 1) + 8 * 4 + (2 * er if law == 2 else 0) + 64.0 * nn / ne
        # writes SIG, QVIS, EINT, RHO, EHOU, [PLA, EPSD], 8 slots
        wr = er * (6 + 1) + 8 * 3 + (2 * er if law == 2 else 0) + 8 * slot
        spn = 8.0 * ne / nn
        # ADSKY, slots, X4 V4 (+ D4 in FP64) read + written; mixed: FP32
        # position copy XF read + written, velocity copy VF written
        node = 4 + spn * slot + (3 * 32 * 2 if prec == 0 else 2 * 32 * 2 + 64 + 16)
        return rd + wr, node, "hexa"
    nc = model.numelc
    npt = model.shells[0].npt
    # reads IX, IADC (4 int32 each), DEGEN, OFF, THKE (ER), THK (FP64),
    # FOR(5), MOM(3), HOUR(5), GSTR(8) (ER), EINT(2), EHOU (FP64),
    # per point SIG(5), PLA, EPSD (ER); node X4, V4, VR4 (32 B each)
    rd = 16 + 16 + 4 + 2 * er + 8 + 21 * er + 24 + npt * 7 * er + 96.0 * nn / nc
    # writes GSTR(8), EPSDG, THK, EINT(2), FOR(5), MOM(3), HOUR(5), EHOU,
    # per point SIG(5), PLA, EPSD; 4 slots of forces + 4 of moments
    wr = 22 * er + 8 + 16 + 8 + npt * 7 * er + 4 * 2 * slot
    spn = 4.0 * nc / nn
    # ADSKY, force + moment slots, X4 V4 VR4 (+ D4 in FP64) read + written;
    # mixed: XF read + written, VF VRF written
    node = 4 + spn * 2 * slot + (4 * 32 * 2 if prec == 0 else 3 * 32 * 2 + 64 + 32)
    return rd + wr, node, "shell"


def fp64_roofline(kkey, ne, ms, device):
    """The plain form's element kernel against the FP64 pipe: FP64
    instructions per launch over its time, against the measured FMA rate."""
    pk = fp64_peak(device)
    n = FP64_INSTR_PER_ELEMENT.get(kkey)
    if not pk or not n:
        return None
    ach = n * ne / (ms * 1e-3)
    return {"bound": "fp64 pipe", "achieved": ach, "peak": pk, "unit": "FP64 thread instr/s",
            "frac": ach / pk, "instr_per_element": n,
            "peak_kind": "measured (rg_fp64_peak: dependent FMA chains, all SMs)"}


# DRAM bytes of one launch of the workload's element kernel
# (dram__bytes_read.sum + dram__bytes_write.sum), from the ncu captures whose
# commands and figures are in profiles/shell_kernel_crash_box_120k.md and
# profiles/hexa_kernel_block128_jc.md
NCU_TRAFFIC = {
    "crash_box_120k_jc": {"f64": 73.9e6 + 33.6e6, "mixed": 42.9e6 + 0.9e6},
    "hexa_block_128_jc": {"f64": 506.7e6 + 685.1e6, "mixed": 388.4e6 + 354.4e6},
}


def run_ours(args, rank, world, local_rank):
    from openradioss_gb300.engine import Engine, RG_PREC_FP64, RG_PREC_MIXED
    wl = args.workload
    model = WORKLOADS[wl]()
    ne = model.numels + model.numelc
    hbm_peak, peak_kind = peaks()
    out = {}
    dist = world > 1
    if dist:
        import torch
        import torch.distributed as tdist

    def barrier():
        if dist:
            tdist.barrier()

    def max_over_ranks(x):
        return reduce_max(x, "cuda:%d" % local_rank) if dist else x

    forms = [RG_PREC_FP64, RG_PREC_MIXED] if args.forms == "both" else (
        [RG_PREC_FP64] if args.forms == "f64" else [RG_PREC_MIXED])
    def fresh(prec):
        # every measurement starts from the same state: W cycles after set-up
        e = Engine(model, device=local_rank, precision=prec)
        e.cycle(args.warmup)
        e.sync()
        return e

    for prec in forms:
        eng = fresh(prec)
        barrier()
        with Clocks(local_rank) as clk:
            # every timed cycle starts from cold L2 (256 MB written before it)
            ms = eng.time_cycles_cold(args.steps, L2_FLUSH_BYTES)
        ms = max_over_ranks(ms)
        st = eng.status()
        eng.close()
        eng = fresh(prec)
        ms_warm = eng.time_cycles(args.steps)
        eng.close()
        # per-kernel times (event-bracketed launches, same stream, cold L2)
        eng = fresh(prec)
        eng.time_cycles_cold(0, L2_FLUSH_BYTES)
        eng.set_timing(True)
        eng.cycle(max(3, min(args.steps, 20)))
        kt = eng.kernel_times()
        eng.set_timing(False)
        st |= eng.status()
        eng.close()
        eb, nb, kkey = element_bytes(model, prec)
        out[prec] = dict(ms=ms, ms_warm=ms_warm, clocks=clk.summary(), kt=kt, status=st,
                         elem_bytes=eb, node_bytes=nb, kkey=kkey)
    # e2e: FORINT-level call with pinned host buffers (headline form), from
    # the same state
    eng = fresh(forms[0])
    nd = eng.nodes()
    x = np.ascontiguousarray(nd["X"].T)
    v = np.ascontiguousarray(nd["V"].T)
    f = np.empty((model.numnod, 3))
    stf = np.empty(model.numnod)
    bufs = [x, v, f, stf]
    vr = fr = stfr = None
    if model.shells:
        vr = np.ascontiguousarray(nd["VR"].T)
        fr = np.empty((model.numnod, 3))
        stfr = np.empty(model.numnod)
        bufs += [vr, fr, stfr]
    for a in bufs:
        eng.host_register(a)
    dt1 = eng.time()["dt2"]
    for _ in range(max(1, args.warmup)):
        eng.forint_step(x, v, dt1, vr=vr, f=f, stifn=stf, fr=fr, stifr=stfr)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.forint_step(x, v, dt1, vr=vr, f=f, stifn=stf, fr=fr, stifr=stfr)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    for a in bufs:
        eng.host_unregister(a)
    dev_bytes = eng.info()["device_bytes"]
    eng.close()
    # the whole job of the configuration (its full cycle count, back to back
    # graph launches, state evolving: contact, plasticity)
    jobs = {}
    if not args.no_job and args.forms == "both" and JOB_CYCLES.get(wl):
        for prec in forms:
            e = Engine(model, device=local_rank, precision=prec)
            # the whole job is seconds long: its clock record has many samples
            with Clocks(local_rank) as jclk:
                jms = e.time_cycles(JOB_CYCLES[wl])
            jobs[prec] = dict(cycles=JOB_CYCLES[wl], seconds=jms * 1e-3,
                              element_updates_s=ne * JOB_CYCLES[wl] / (jms * 1e-3),
                              status=e.status(), clocks=jclk.summary())
            e.close()

    if args.forms != "both":
        res = out[forms[0]]
        line = {"metric": "element-updates/s", "forms": args.forms,
                "value": world * ne * args.steps / (res["ms"] * 1e-3),
                "kernel_ms": res["kt"], "e2e_s": e2e_s}
        return line
    res64, res32 = out[RG_PREC_FP64], out[RG_PREC_MIXED]
    value = replica_value(ne * args.steps, world, res64["ms"] * 1e-3)
    value32 = replica_value(ne * args.steps, world, res32["ms"] * 1e-3)
    kk = res64["kkey"]
    k64 = res64["kt"][kk]
    ach = res64["elem_bytes"] * ne / (k64 * 1e-3) / 1e9
    k32 = res32["kt"][kk]
    ach32 = res32["elem_bytes"] * ne / (k32 * 1e-3) / 1e9
    traffic = NCU_TRAFFIC.get(wl, {}).get("f64")
    traffic32 = NCU_TRAFFIC.get(wl, {}).get("mixed")
    line = {
        "metric": "element-updates/s",
        "value": value,
        "unit": "element-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": res64["ms"] / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded mesh and velocity field of the named shape)",
        "config": {"workload": wl, "elements": ne, "nodes": model.numnod,
                   "law": "LAW2 Johnson-Cook" if (model.shells or model.hexa[0].mat["mtn"] == 2)
                   else "LAW1",
                   "formulation": ("one-point hexa Isolid=1 Iframe=1 Ismstr=4, viscous "
                                   "hourglass" if model.hexa else
                                   "Belytschko-Tsay shell Ishell=1 Ismstr=4 Ithick=1 NPT=5 "
                                   "Iplas=1, planar sliding rigid wall") + ", PARITH/ON",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "L2 flushed (256 MB written) before every timed cycle; model "
                         "state %.2f GB" % (dev_bytes / 1e9),
                   "state": "every measurement starts %d cycles after set-up" % args.warmup},
        "e2e": {"value": world * ne * args.steps / e2e_s, "unit": "element-updates/s",
                "transfer": "inputs: registered host buffers read in place by the upload "
                            "kernel; outputs: DMA copies from the device staging buffer",
                "h2d_bytes_per_step": (3 if model.shells else 2) * 3 * 8 * model.numnod,
                "d2h_bytes_per_step": (8 if model.shells else 4) * 8 * model.numnod},
        "gpu_launches": (len(model.hexa) + len(model.shells) + 2) * args.steps,
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                     "frac": ach / hbm_peak, "traffic": traffic, "traffic_unit": "bytes per launch (ncu)",
                     "kernel": "%s_kernel<double>" % kk,
                     "bytes_per_element": res64["elem_bytes"], "ms_per_launch": k64,
                     "peak_kind": peak_kind,
                     "note": "FP64 form is FP64-pipe bound on GB300; see fp64_roofline"},
        "fp64_roofline": fp64_roofline(kk, ne, k64, local_rank),
        "kernel_ms": res64["kt"],
        "l2_warm_back_to_back": {"f64": world * ne * args.steps / (res64["ms_warm"] * 1e-3),
                                 "mixed": world * ne * args.steps / (res32["ms_warm"] * 1e-3)},
        "mixed_f32_f64": {"value": value32, "speedup_vs_f64": value32 / value,
                          "kernel_ms": res32["kt"],
                          "roofline": {"bound": "hbm", "achieved": ach32, "peak": hbm_peak,
                                       "unit": "GB/s", "frac": ach32 / hbm_peak,
                                       "traffic": traffic32,
                                       "bytes_per_element": res32["elem_bytes"]}},
        "clocks": res64["clocks"],
        "device_status": [res64["status"], res32["status"]],
    }
    if jobs:
        line["job"] = {("f64" if p == RG_PREC_FP64 else "mixed"): j for p, j in jobs.items()}
        if len(jobs) == 2:
            line["job"]["mixed_speedup"] = jobs[RG_PREC_FP64]["seconds"] / jobs[RG_PREC_MIXED]["seconds"]
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(wl, args.cpu_sample)
    return line


L2_FLUSH_BYTES = 256 << 20  # twice the GB300 L2

# FP64 thread instructions per element of the plain form's element kernels at
# the benchmark's state (5 cycles after set-up), counted with ncu
# (smsp__sass_thread_inst_executed_op_fp64_pred_on / elements per launch).
FP64_INSTR_PER_ELEMENT = {"shell": 967.0, "hexa": 1030.0}


def fp64_peak(device=0):
    """Measured FP64 fused multiply-add rate of the device (thread instr/s)."""
    import ctypes as C
    from openradioss_gb300 import _lib
    v = C.c_double()
    r = _lib.lib().rg_fp64_peak(device, C.byref(v))
    return v.value if r == 0 else None

SWEEP_JOBS = 64
SWEEP_CYCLES_PER_JOB = 2000


def run_sweep(args, njobs=SWEEP_JOBS, timed_cycles=None, device=0):
    """Batched crash-box sweep: njobs seeded variants (5k-60k shells each)
    stepped together in one persistent kernel per cycle (autotuned launch
    shape), against the same jobs run one after another, alone, in the plain
    FP64 form.  A job is SWEEP_CYCLES_PER_JOB cycles; the timed region is
    timed_cycles cycles of every job and jobs/h is scaled from it."""
    from openradioss_gb300.batch import Batch
    from openradioss_gb300.engine import Engine
    models = M.crash_box_sweep(njobs)
    K = timed_cycles or args.steps
    ne = sum(m.numels + m.numelc for m in models)
    hbm_peak, peak_kind = peaks()
    seq = {}
    for prec in (0, 1):
        tot = 0.0
        for m in models:
            e = Engine(m, device=device, precision=prec)
            e.cycle(args.warmup)
            tot += e.time_cycles(K)
            e.close()
        seq[prec] = tot
    bat = {}
    for prec in (0, 1):
        es = [Engine(m, device=device, precision=prec) for m in models]
        b = Batch(device)
        for e in es:
            b.add(e)
        b.cycle(args.warmup)
        b.sync()
        cfg = b.autotune(trial_cycles=3)
        b.cycle(args.warmup)
        with Clocks(device) as clk:
            ms = b.time_cycles(K)
        prog, st = b.progress()
        bat[prec] = dict(ms=ms, cfg=cfg, status=st, clocks=clk.summary(),
                         status_jobs=sum(e.status() for e in es))
        b.close()
        for e in es:
            e.close()

    def jobs_h(ms):
        return njobs * 3600.0 / (ms * 1e-3 * SWEEP_CYCLES_PER_JOB / K)

    eb32 = sum(element_bytes(m, 1)[0] * m.numelc for m in models)
    ach = eb32 / (bat[1]["ms"] * 1e-3 / K) / 1e9
    return {
        "metric": "jobs/h",
        "value": jobs_h(bat[1]["ms"]),
        "unit": "jobs/h",
        "n_gpus": 1,
        "steps": K,
        "warmup": args.warmup,
        "ms_per_step": bat[1]["ms"] / K,
        "higher_is_better": True,
        "dtype": "f32 element / f64 nodal",
        "data": "synthetic (64 seeded crash-box variants)",
        "config": {"workload": "crash_box_sweep_64", "jobs": njobs, "elements": ne,
                   "elements_per_job": [min(m.numelc for m in models),
                                        max(m.numelc for m in models)],
                   "cycles_per_job": SWEEP_CYCLES_PER_JOB,
                   "note": "jobs/h scaled from %d timed cycles of every job" % K},
        "batched_mixed": {"jobs_h": jobs_h(bat[1]["ms"]),
                          "element_updates_s": ne * K / (bat[1]["ms"] * 1e-3),
                          "autotuned": bat[1]["cfg"]},
        "batched_fp64": {"jobs_h": jobs_h(bat[0]["ms"]),
                         "element_updates_s": ne * K / (bat[0]["ms"] * 1e-3),
                         "autotuned": bat[0]["cfg"]},
        "sequential_fp64": {"jobs_h": jobs_h(seq[0]),
                            "element_updates_s": ne * K / (seq[0] * 1e-3)},
        "sequential_mixed": {"jobs_h": jobs_h(seq[1]),
                             "element_updates_s": ne * K / (seq[1] * 1e-3)},
        "speedup_vs_sequential_plain": seq[0] / bat[1]["ms"],
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                     "frac": ach / hbm_peak, "peak_kind": peak_kind,
                     "note": "batched mixed cycle: shell element-phase algorithmic bytes "
                             "over the whole cycle time"},
        "clocks": bat[1]["clocks"],
        "device_status": [bat[0]["status"], bat[1]["status"], bat[0]["status_jobs"],
                          bat[1]["status_jobs"]],
    }


SERVE_JOBS = 32
SERVE_RATE = 4.0          # Poisson arrivals, jobs/s
SERVE_BUDGET = 48 << 30   # HBM budget of the serving loop (bytes)


def run_serving(args, njobs=SERVE_JOBS, device=0):
    """Serving stream: njobs seeded requests (50/50 shell crash boxes of
    2k-150k elements and hexa impact blocks of 2k-200k elements, 2,000-20,000
    cycles each) arriving as a Poisson process of SERVE_RATE jobs/s, admitted
    by HBM budget into a continuously batched mixed-form run.  Beside it, the
    same jobs as sequential plain FP64 runs alone (GPU time of each job from a
    timed 50-cycle sample scaled to its cycle count)."""
    from openradioss_gb300.engine import Engine
    from openradioss_gb300.serving import Server, poisson_arrivals
    jobs = [M.serving_job(k) for k in range(njobs)]
    arr = poisson_arrivals(njobs, SERVE_RATE, seed=7)
    seq = 0.0
    for m, n in jobs:
        e = Engine(m, device=device, precision=0)
        e.cycle(3)
        seq += e.time_cycles(50) * 1e-3 * n / 50.0
        e.close()
    srv = Server(SERVE_BUDGET, max_jobs=64, precision=1, step_cycles=100, device=device)
    with Clocks(device) as clk:
        st = srv.run([(k, m, n, float(a)) for k, ((m, n), a) in enumerate(zip(jobs, arr))])
    bad = sum(1 for r in srv.done if r.result.get("status", 0))
    srv.close()
    seq_jobs_h = 3600.0 * njobs / seq
    ne = [m.numels + m.numelc for m, _ in jobs]
    return {
        "metric": "jobs/h",
        "value": st["jobs_per_h"],
        "unit": "jobs/h",
        "n_gpus": 1,
        "higher_is_better": True,
        "dtype": "f32 element / f64 nodal",
        "data": "synthetic (seeded serving stream)",
        "config": {"workload": "serving_mix", "jobs": njobs, "arrival_rate_per_s": SERVE_RATE,
                   "elements_per_job": [min(ne), max(ne)],
                   "cycles_per_job": [min(n for _, n in jobs), max(n for _, n in jobs)],
                   "hbm_budget_gb": SERVE_BUDGET / 2 ** 30, "step_cycles": 100},
        "p50_latency_s": st["p50_latency_s"],
        "p99_latency_s": st["p99_latency_s"],
        "mean_latency_s": st["mean_latency_s"],
        "makespan_s": st["makespan_s"],
        "element_updates_s": st["element_updates"] / st["makespan_s"],
        "max_used_gb": st["max_used_bytes"] / 2 ** 30,
        "sequential_fp64_jobs_h": seq_jobs_h,
        "speedup_vs_sequential_plain": st["jobs_per_h"] / seq_jobs_h,
        "jobs_with_device_status": bad,
        "clocks": clk.summary(),
    }


def cpu_baseline(wl, sample_s, threads=None):
    """Time the CPU restatement (oracle/) on the host cores: a bounded
    sample of the same workload."""
    from oracle.oracle import OracleModel
    model = WORKLOADS[wl]()
    nt = threads or os.cpu_count() or 1
    o = OracleModel(model, nthreads=nt)
    t0 = time.perf_counter()
    o.cycle(1)
    t1 = time.perf_counter() - t0
    # bounded sample: about sample_s seconds of CPU work
    n = max(3, min(5000, int(sample_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    o.cycle(n)
    dt = time.perf_counter() - t0
    ne = model.numels + model.numelc
    return {"value": ne * n / dt, "unit": "element-updates/s", "cores": nt,
            "kind": "port", "sample": "%s, %d cycles after 1 warm-up cycle (%.1f s)" % (wl, n, dt)}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    from oracle.oracle import OracleModel
    wl = args.workload
    model = WORKLOADS[wl]()
    nt = os.cpu_count() or 1
    o = OracleModel(model, nthreads=nt)
    o.cycle(1)
    # each step: one cycle of the workload (bounded sample)
    for _ in range(args.warmup):
        o.cycle(1)
    t0 = time.perf_counter()
    o.cycle(args.steps)
    dt = time.perf_counter() - t0
    v = (model.numels + model.numelc) * args.steps / dt
    return {"metric": "element-updates/s", "value": v, "unit": "element-updates/s",
            "impl": "reference", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl, "elements": model.numels + model.numelc,
                       "nodes": model.numnod},
            "cpu_baseline": {"value": v, "unit": "element-updates/s", "cores": nt, "kind": "port",
                             "sample": "%s, %d cycles" % (wl, args.steps)},
            "e2e": {"value": v, "unit": "element-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "reference engine not buildable here (no Fortran compiler); "
                    "timed: the CPU restatement of its algorithm (oracle/, g++ -O3 "
                    "-ffp-contract=off, OpenMP over element groups and node ranges)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    choices=sorted(WORKLOADS) + ["crash_box_sweep_64", "serving_mix"])
    ap.add_argument("--no-job", action="store_true",
                    help="skip the full-length job runs of the configuration")
    ap.add_argument("--no-sweep", action="store_true",
                    help="skip the batched-sweep and serving summaries of the default run")
    ap.add_argument("--cpu-sample", type=float, default=15.0,
                    help="seconds of CPU work in the cpu_baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--forms", default="both", choices=["both", "f64", "mixed"],
                    help="arithmetic forms to run (profiling runs pick one)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local_rank)
        tdist.init_process_group("nccl")
    if args.workload in ("crash_box_sweep_64", "serving_mix"):
        line = (run_sweep(args, device=local_rank) if args.workload == "crash_box_sweep_64"
                else run_serving(args, device=local_rank))
        line["n_gpus"] = world
        if rank == 0:
            print(json.dumps(line, default=float), flush=True)
        return
    line = run_ours(args, rank, world, local_rank)
    if rank == 0 and world == 1 and not args.no_sweep:
        sw = run_sweep(args, timed_cycles=20)
        line["batched_sweep"] = {k: sw[k] for k in (
            "batched_mixed", "batched_fp64", "sequential_fp64", "sequential_mixed",
            "speedup_vs_sequential_plain", "config", "device_status")}
        sv = run_serving(args)
        line["serving"] = {k: sv[k] for k in (
            "value", "unit", "p50_latency_s", "p99_latency_s", "sequential_fp64_jobs_h",
            "speedup_vs_sequential_plain", "element_updates_s", "config",
            "jobs_with_device_status")}
    if rank == 0:
        print(json.dumps(line, default=float), flush=True)
    if world > 1:
        import torch.distributed as tdist
        tdist.barrier()
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
