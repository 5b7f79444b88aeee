#!/usr/bin/env python3
"""Benchmark of the explicit hot path on one GB300 (or N replicas).

A *step* is one explicit cycle of the whole model (every element group ->
PARITH/ON assembly -> time step -> nodal update) with the model resident in
HBM.  ``value`` is element-updates/s (elements x cycles / device seconds,
CUDA events on the library's stream, every cycle from cold L2) of the plain
FP64 form on the crash box of 120,120 shells; the mixed FP32-element /
FP64-nodal form is reported beside it.  ``e2e`` is the same metric through
the library's whole-cycle call with host node buffers (rg_cycle_host: X, V,
VR read from pinned host memory, X, V, VR, D written back, every step).

The same line carries, for the other single-GPU configurations, summaries
measured in the same run: the 20^3 bar impact (LAW1, 1,000 cycles) and the
128^3 Johnson-Cook block (2,000 cycles), each with both forms' full-length
job runs and the mixed form's error against the FP64 run (displacement,
peak force, internal energy and its growth); the batched sweep of 64
crash-box variants and the Poisson serving stream, both against sequential
runs of the same jobs, all at full length.

``--impl reference`` times the reference algorithm's CPU path -- the CPU
restatement under oracle/ (the reference engine itself cannot be built
without a Fortran compiler) -- on all host cores, on the same workload and
the same cycle window as the GPU's timed region.

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
# printouts of a job run (forces, energies, displacement) for the error curve
JOB_PRINTOUTS = 40
L2_FLUSH_BYTES = 256 << 20  # twice the GB300 L2


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def profile_json(name):
    p = os.path.join(ROOT, "profiles", name)
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return {}
    return {}


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


def workload_config(wl, model, world):
    """The workload as both arms describe it (the same dict in the GPU line
    and in the reference arm's line)."""
    hexa = bool(model.hexa)
    law2 = bool(model.shells) or model.hexa[0].mat["mtn"] == 2
    return {"workload": wl, "elements": model.numels + model.numelc, "nodes": model.numnod,
            "law": "LAW2 Johnson-Cook" if law2 else "LAW1",
            "formulation": ("one-point hexa Isolid=1 Iframe=1 Ismstr=4, viscous hourglass"
                            if hexa else
                            "Belytschko-Tsay shell Ishell=1 Ismstr=4 Ithick=1 NPT=5 Iplas=1, "
                            "planar sliding rigid wall") + ", PARITH/ON",
            "parallelism": "replicas" if world > 1 else "single GPU",
            "window": "each arm times cycles W+1 .. W+K of a fresh model (W warm-up cycles)"
                      + ("; at W=5, K=20 the box is still moving to the wall (elastic): the "
                         "full 20,000-cycle job (contact, buckling, plasticity) is timed in "
                         "'job'" if not hexa else ""),
            "l2": "GPU arm: L2 flushed (256 MB written) before every timed cycle"}


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
        # VOL0, EHOU (FP64), [PLA, EPSD]; node records X4, V4 (32 B each;
        # mixed: the FP32 copies XF 32 B, VF 16 B)
        gather = 64.0 if prec == 0 else 48.0
        rd = 32 + 32 + er * (1 + 6 + 1) + 8 * 4 + (2 * er if law == 2 else 0) + gather * nn / ne
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
    # per point SIG(5), PLA, EPSD (ER); node records X4, V4, VR4 (32 B
    # each; mixed: the FP32 copies XF 32 B, VF and VRF 16 B)
    gather = 96.0 if prec == 0 else 64.0
    rd = 16 + 16 + 4 + 2 * er + 8 + 21 * er + 24 + npt * 7 * er + gather * nn / nc
    # writes GSTR(8), EPSDG, THK, EINT(2), FOR(5), MOM(3), HOUR(5), EHOU,
    # per point SIG(5), PLA, EPSD; 4 slots of forces + 4 of moments
    wr = 22 * er + 8 + 16 + 8 + npt * 7 * er + 4 * 2 * slot
    spn = 4.0 * nc / nn
    # ADSKY, force + moment slots, X4 V4 VR4 (+ D4 in FP64) read + written;
    # mixed: XF read + written, VF VRF written
    node = 4 + spn * 2 * slot + (4 * 32 * 2 if prec == 0 else 3 * 32 * 2 + 64 + 32)
    return rd + wr, node, "shell"


def fp64_peak(device=0):
    """Measured FP64 fused multiply-add rate of the device (thread instr/s)."""
    import ctypes as C
    from openradioss_gb300 import _lib
    v = C.c_double()
    r = _lib.lib().rg_fp64_peak(device, C.byref(v))
    return v.value if r == 0 else None


def fp64_roofline(wl, kkey, ne, ms, device):
    """The plain form's element kernel against the FP64 pipe, from
    algorithmic operation counts: the FP64 flops per element the reference
    algorithm performs in the timed window (op-counting build of the CPU
    oracle, committed in profiles/fp64_op_counts.json) x elements over the
    kernel's measured time, against twice the measured FMA instruction rate
    (an FMA is two flops).  The FP64 instructions the kernel executes per
    element (ncu) are given beside, with their ratio to the algorithmic
    operations."""
    pk = fp64_peak(device)
    cnt = profile_json("fp64_op_counts.json").get("windows", {}).get(wl, {}).get(kkey)
    if not pk or not cnt:
        return None
    flops = cnt["flops"]
    ach = flops * ne / (ms * 1e-3)
    out = {"bound": "fp64 pipe", "achieved": ach, "peak": 2.0 * pk, "unit": "FP64 flop/s",
           "frac": ach / (2.0 * pk), "flops_per_element": flops,
           "ops_per_element": {k: cnt[k] for k in ("add", "mul", "div", "sqrt", "pow", "log",
                                                   "exp", "cmp", "minmax")},
           "counts_from": "profiles/fp64_op_counts.json (python oracle/opcount_report.py)",
           "peak_kind": "measured: 2 x rg_fp64_peak (dependent FMA chains on all SMs)"}
    ex = profile_json("element_kernel_ncu.json").get(wl, {}).get("f64", {})
    if ex.get("fp64_instr_per_element"):
        n = ex["fp64_instr_per_element"]
        algo = sum(cnt[k] for k in ("add", "mul", "div", "sqrt", "pow", "log", "exp", "cmp",
                                    "minmax"))
        out["executed_fp64_instr_per_element"] = n
        out["executed_over_algorithmic_ops"] = n / algo
        out["fp64_pipe_frac_executed"] = n * ne / (ms * 1e-3) / pk
    return out


def ncu_traffic(wl, form):
    d = profile_json("element_kernel_ncu.json").get(wl, {}).get(form)
    return (d["dram_read"] + d["dram_write"]) if d else None


def support_nodes(model):
    """Nodes whose summed internal force is the model's impact force: the
    fixed face of a hexa model, the row of a crash box at the wall."""
    if model.hexa:
        return np.nonzero(model.icodt != 0)[0]
    z = model.X[2]
    return np.nonzero(z <= z.min() + 1e-9)[0]


def job_run(model, prec, cycles, device, printouts=JOB_PRINTOUTS):
    """The configuration's full-length run (back-to-back graph launches, the
    state evolving through contact and plasticity) in printout chunks, each
    chunk timed with CUDA events on the library's stream (the printouts --
    forces, energies, displacements -- fall between the timed spans)."""
    from openradioss_gb300.engine import Engine
    e = Engine(model, device=device, precision=prec)
    sup = support_nodes(model)
    every = max(1, cycles // printouts)
    # displacements are kept at every dstride-th printout and the last
    dstride = max(1, printouts // 10)
    ms, curve, done, i = 0.0, [], 0, 0
    with Clocks(device) as clk:
        while done < cycles:
            k = min(every, cycles - done)
            ms += e.time_cycles(k)
            done += k
            f = e.forces()["F"]
            en = e.energy()
            keep_d = (i % dstride == dstride - 1) or done >= cycles
            curve.append({"cycle": done, "reaction": float(abs(f[2, sup].sum())),
                          "fmax": float(np.max(np.linalg.norm(f, axis=0))),
                          "eint": en["eint"], "d": e.displacement() if keep_d else None})
            i += 1
    ne = model.numels + model.numelc
    out = dict(cycles=cycles, seconds=ms * 1e-3, element_updates_s=ne * cycles / (ms * 1e-3),
               status=e.status(), clocks=clk.summary(), printout_every=every)
    e.close()
    return out, curve


def one_ulp(model):
    """The model with every initial coordinate moved by one ulp: its FP64 run
    against the unperturbed one measures the problem's own sensitivity to
    round-off, the yardstick of the mixed form's error."""
    import copy
    mp = copy.deepcopy(model)
    mp.X = np.nextafter(model.X, np.inf)
    return mp


def job_pair(model, cycles, device):
    """Full-length FP64 and mixed runs of a configuration, and an FP64 run
    from the one-ulp-perturbed start: times, and the mixed form's error
    beside the FP64 form's own round-off drift."""
    from openradioss_gb300.engine import RG_PREC_FP64, RG_PREC_MIXED
    j64, c64 = job_run(model, RG_PREC_FP64, cycles, device)
    j32, c32 = job_run(model, RG_PREC_MIXED, cycles, device)
    _, c64p = job_run(one_ulp(model), RG_PREC_FP64, cycles, device)
    return {"f64": j64, "mixed": j32, "mixed_speedup": j64["seconds"] / j32["seconds"],
            "mixed_error_vs_f64": mixed_error(c64, c32),
            "fp64_one_ulp_drift": mixed_error(c64, c64p),
            "note": "fp64_one_ulp_drift: the FP64 run from coordinates moved by one ulp "
                    "against the FP64 run -- the round-off sensitivity of the problem"}


def mixed_error(c64, c32):
    """Mixed-form error against the FP64 run of the same job: relative
    displacement error (final, and its largest over the printouts), peak
    impact-force and peak nodal-force errors over the printouts, largest
    internal-energy error, and the growth of the errors printout by
    printout (all relative to the FP64 quantity's largest magnitude)."""
    dmax = max(float(np.max(np.abs(c["d"]))) for c in c64 if c["d"] is not None) or 1.0
    emax = max(abs(c["eint"]) for c in c64) or 1.0
    rmax = max(c["reaction"] for c in c64) or 1.0
    growth = []
    for a, b in zip(c64, c32):
        dd = (float(np.max(np.abs(b["d"] - a["d"]))) / dmax if a["d"] is not None
              else None)
        growth.append([a["cycle"], dd, abs(b["eint"] - a["eint"]) / emax,
                       abs(b["reaction"] - a["reaction"]) / rmax])
    p64r, p32r = max(c["reaction"] for c in c64), max(c["reaction"] for c in c32)
    p64f, p32f = max(c["fmax"] for c in c64), max(c["fmax"] for c in c32)
    return {"displacement_final": growth[-1][1],
            "displacement_max": max(g[1] for g in growth if g[1] is not None),
            "peak_impact_force": abs(p32r - p64r) / p64r if p64r else None,
            "peak_nodal_force": abs(p32f - p64f) / p64f if p64f else None,
            "internal_energy_max": max(g[2] for g in growth),
            "peak_impact_force_n": p64r,
            "growth_columns": ["cycle", "displacement", "internal_energy", "impact_force"],
            "growth": [[g[0]] + [None if x is None else "%.3e" % x for x in g[1:]]
                       for g in growth]}


def measure_forms(wl, model, args, world, local_rank, forms, barrier, max_over_ranks):
    """Cold-L2 timed cycles, warm back-to-back cycles and per-kernel times
    of each arithmetic form, every measurement from the same state (W cycles
    after set-up)."""
    from openradioss_gb300.engine import Engine

    def fresh(prec):
        e = Engine(model, device=local_rank, precision=prec)
        e.cycle(args.warmup)
        e.sync()
        return e

    out = {}
    for prec in forms:
        eng = fresh(prec)
        barrier()
        with Clocks(local_rank) as clk:
            ms = eng.time_cycles_cold(args.steps, L2_FLUSH_BYTES)
        ms = max_over_ranks(ms)
        st = eng.status()
        dev_bytes = eng.info()["device_bytes"]
        eng.close()
        eng = fresh(prec)
        ms_warm = eng.time_cycles(args.steps)
        eng.close()
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
                         elem_bytes=eb, node_bytes=nb, kkey=kkey, dev_bytes=dev_bytes)
    return out


def e2e_cycle_host(model, prec, args, local_rank, barrier, max_over_ranks):
    """Whole cycles through rg_cycle_host with registered host buffers:
    every step X, V (VR) go host -> device and X, V (VR), D come back.
    Returns (seconds for K steps, h2d bytes, d2h bytes per step)."""
    from openradioss_gb300.engine import Engine
    e = Engine(model, device=local_rank, precision=prec)
    e.cycle(args.warmup)
    nd = e.nodes()
    n = model.numnod
    x = np.ascontiguousarray(nd["X"].T)
    v = np.ascontiguousarray(nd["V"].T)
    vr = np.ascontiguousarray(nd["VR"].T) if model.shells else None
    d = np.empty((n, 3))
    bufs = [a for a in (x, v, vr, d) if a is not None]
    for a in bufs:
        e.host_register(a)
    for _ in range(3):
        e.cycle_host(x, v, vr, x_out=x, v_out=v, vr_out=vr, d_out=d)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e.cycle_host(x, v, vr, x_out=x, v_out=v, vr_out=vr, d_out=d)
    s = max_over_ranks(time.perf_counter() - t0)
    for a in bufs:
        e.host_unregister(a)
    e.close()
    nin = 3 if model.shells else 2
    return s, nin * 24 * n, (nin + 1) * 24 * n


def e2e_forint(model, prec, args, local_rank):
    """The FORINT-level drop-in call (elements + PARITH/ON assembly; the
    engine keeps its nodal update) with registered host buffers: seconds for
    K calls."""
    from openradioss_gb300.engine import Engine
    eng = Engine(model, device=local_rank, precision=prec)
    eng.cycle(args.warmup)
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
    for _ in range(3):
        eng.forint_step(x, v, dt1, vr=vr, f=f, stifn=stf, fr=fr, stifr=stfr)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.forint_step(x, v, dt1, vr=vr, f=f, stifn=stf, fr=fr, stifr=stfr)
    s = time.perf_counter() - t0
    for a in bufs:
        eng.host_unregister(a)
    eng.close()
    return s


def workload_summary(wl, args, device, with_jobs=True):
    """One single-GPU configuration measured in both forms (cold-L2 cycles,
    kernel times, element-kernel roofline) and, with_jobs, its full-length
    job runs with the mixed form's error against the FP64 run."""
    from openradioss_gb300.engine import RG_PREC_FP64, RG_PREC_MIXED
    model = WORKLOADS[wl]()
    ne = model.numels + model.numelc
    hbm_peak, peak_kind = peaks()
    res = measure_forms(wl, model, args, 1, device, [RG_PREC_FP64, RG_PREC_MIXED],
                        lambda: None, lambda x: x)
    out = {"config": workload_config(wl, model, 1)}
    for prec, name in ((RG_PREC_FP64, "f64"), (RG_PREC_MIXED, "mixed")):
        r = res[prec]
        k = r["kt"][r["kkey"]]
        ach = r["elem_bytes"] * ne / (k * 1e-3) / 1e9
        out[name] = {"element_updates_s": ne * args.steps / (r["ms"] * 1e-3),
                     "ms_per_step": r["ms"] / args.steps, "kernel_ms": r["kt"],
                     "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm_peak,
                                  "unit": "GB/s", "frac": ach / hbm_peak,
                                  "traffic": ncu_traffic(wl, name),
                                  "kernel": "%s_kernel<%s>" % (r["kkey"], "double" if prec == 0
                                                               else "float"),
                                  "bytes_per_element": r["elem_bytes"], "peak_kind": peak_kind},
                     "status": r["status"]}
    out["mixed_speedup"] = out["mixed"]["element_updates_s"] / out["f64"]["element_updates_s"]
    kk = res[RG_PREC_FP64]["kkey"]
    out["fp64_roofline"] = fp64_roofline(wl, kk, ne, res[RG_PREC_FP64]["kt"][kk], device)
    if with_jobs and JOB_CYCLES.get(wl):
        out["job"] = job_pair(model, JOB_CYCLES[wl], device)
    return out


def run_ours(args, rank, world, local_rank):
    from openradioss_gb300.engine import RG_PREC_FP64, RG_PREC_MIXED
    wl = args.workload
    model = WORKLOADS[wl]()
    ne = model.numels + model.numelc
    hbm_peak, peak_kind = peaks()
    dist = world > 1
    if dist:
        import torch.distributed as tdist

    def barrier():
        if dist:
            tdist.barrier()

    def max_over_ranks(x):
        return reduce_max(x, "cuda:%d" % local_rank) if dist else x

    forms = [RG_PREC_FP64, RG_PREC_MIXED] if args.forms == "both" else (
        [RG_PREC_FP64] if args.forms == "f64" else [RG_PREC_MIXED])
    out = measure_forms(wl, model, args, world, local_rank, forms, barrier, max_over_ranks)
    if args.forms != "both":
        res = out[forms[0]]
        return {"metric": "element-updates/s", "forms": args.forms,
                "value": world * ne * args.steps / (res["ms"] * 1e-3), "kernel_ms": res["kt"]}
    # e2e: whole cycles with host node buffers, both forms (headline: FP64)
    e2e = {}
    for prec in forms:
        s, hb, db = e2e_cycle_host(model, prec, args, local_rank, barrier, max_over_ranks)
        e2e[prec] = dict(s=s, h2d=hb, d2h=db)
    forint_s = e2e_forint(model, RG_PREC_FP64, args, local_rank)
    jobs = {}
    if not args.no_job and JOB_CYCLES.get(wl):
        jobs = job_pair(model, JOB_CYCLES[wl], local_rank)
    res64, res32 = out[RG_PREC_FP64], out[RG_PREC_MIXED]
    value = replica_value(ne * args.steps, world, res64["ms"] * 1e-3)
    value32 = replica_value(ne * args.steps, world, res32["ms"] * 1e-3)
    kk = res64["kkey"]
    k64 = res64["kt"][kk]
    ach = res64["elem_bytes"] * ne / (k64 * 1e-3) / 1e9
    k32 = res32["kt"][kk]
    ach32 = res32["elem_bytes"] * ne / (k32 * 1e-3) / 1e9
    groups = len(model.hexa) + len(model.shells)
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
        "config": workload_config(wl, model, world),
        "e2e": {"value": world * ne * args.steps / e2e[RG_PREC_FP64]["s"],
                "unit": "element-updates/s",
                "call": "rg_cycle_host: whole cycle (elements, PARITH/ON assembly, time step, "
                        "nodal update) with host node buffers",
                "transfer": "inputs X, V, VR read in place from registered (pinned) host "
                            "buffers by the upload kernel; outputs X, V, VR, D written in "
                            "place into registered host buffers by one kernel (16-byte "
                            "stores)",
                "h2d_bytes_per_step": e2e[RG_PREC_FP64]["h2d"],
                "d2h_bytes_per_step": e2e[RG_PREC_FP64]["d2h"],
                "mixed": world * ne * args.steps / e2e[RG_PREC_MIXED]["s"],
                "forint_level_f64": world * ne * args.steps / forint_s},
        # per timed cycle: one element kernel per group + one node kernel
        "gpu_launches": (groups + 1) * args.steps,
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                     "frac": ach / hbm_peak, "traffic": ncu_traffic(wl, "f64"),
                     "traffic_unit": "DRAM bytes per launch (ncu capture, profiles/)",
                     "kernel": "%s_kernel<double>" % kk,
                     "bytes_per_element": res64["elem_bytes"], "ms_per_launch": k64,
                     "peak_kind": peak_kind,
                     "note": "the FP64 form is bound by the FP64 pipe on GB300: fp64_roofline"},
        "fp64_roofline": fp64_roofline(wl, kk, ne, k64, local_rank),
        "kernel_ms": res64["kt"],
        "l2_warm_back_to_back": {"f64": world * ne * args.steps / (res64["ms_warm"] * 1e-3),
                                 "mixed": world * ne * args.steps / (res32["ms_warm"] * 1e-3)},
        "mixed_f32_f64": {"value": value32, "speedup_vs_f64": value32 / value,
                          "kernel_ms": res32["kt"],
                          "roofline": {"bound": "hbm", "achieved": ach32, "peak": hbm_peak,
                                       "unit": "GB/s", "frac": ach32 / hbm_peak,
                                       "traffic": ncu_traffic(wl, "mixed"),
                                       "bytes_per_element": res32["elem_bytes"]}},
        "device_bytes": res64["dev_bytes"],
        "clocks": res64["clocks"],
        "device_status": [res64["status"], res32["status"]],
    }
    if jobs:
        line["job"] = jobs
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        # the baseline legs: the CPU restatement on the host cores, and (shell
        # workloads) the reference's own CUDA shell path on this GPU
        line["cpu_baseline"] = cpu_baseline(wl, args.warmup, args.steps)
        if model.shells:
            try:
                line["reference_gpu_shell"] = reference_gpu_shell(model, args, local_rank,
                                                                  res64["kt"])
            except Exception as ex:  # the comparator is optional
                line["reference_gpu_shell"] = {"unavailable": repr(ex)[:200]}
    return line


SWEEP_JOBS = 64
SWEEP_CYCLES_PER_JOB = 2000


def run_sweep(args, njobs=SWEEP_JOBS, cycles=SWEEP_CYCLES_PER_JOB, device=0):
    """Crash-box sweep: njobs seeded variants (5k-60k shells each) advanced
    together -- as concurrent single-model graphs on their own streams (the
    line's value), and in one persistent batched kernel per cycle (autotuned
    launch shape) -- against the same jobs run one after another alone, each
    form at full length (cycles per job, from a fresh model)."""
    from openradioss_gb300.batch import Batch
    from openradioss_gb300.engine import Engine
    models = M.crash_box_sweep(njobs)
    ne = sum(m.numels + m.numelc for m in models)
    hbm_peak, peak_kind = peaks()
    seq = {}
    for prec in (0, 1):
        tot = 0.0
        for m in models:
            e = Engine(m, device=device, precision=prec)
            tot += e.time_cycles(cycles)
            e.close()
        seq[prec] = tot
    bat = {}
    for prec in (0, 1):
        # autotune on a throw-away copy of the jobs, then time fresh jobs
        es = [Engine(m, device=device, precision=prec) for m in models]
        b = Batch(device)
        for e in es:
            b.add(e)
        cfg = b.autotune(trial_cycles=3)
        b.close()
        for e in es:
            e.close()
        es = [Engine(m, device=device, precision=prec) for m in models]
        b = Batch(device)
        for e in es:
            b.add(e, cycles)
        b.set_config(cfg["ktile"], cfg["knode"], cfg["blocks_per_sm"], cfg["schedule"])
        with Clocks(device) as clk:
            ms = b.time_cycles(cycles)
        prog, st = b.progress()
        bat[prec] = dict(ms=ms, cfg=cfg, status=st, clocks=clk.summary(),
                         status_jobs=sum(e.status() for e in es),
                         all_at_target=all(p == cycles for p in prog.values()))
        b.close()
        for e in es:
            e.close()

    # the same jobs as concurrent single-model graphs, each on its own
    # stream (the serving loop's streams executor), launched in interleaved
    # chunks of 100 cycles; wall time from the first launch to the last
    # job's completion
    from openradioss_gb300.batch import run_concurrent
    conc = {}
    for prec in (0, 1):
        es = [Engine(m, device=device, precision=prec) for m in models]
        for e in es:
            e.sync()
        t0 = time.perf_counter()
        run_concurrent(es, cycles, chunk=100)
        conc[prec] = (time.perf_counter() - t0) * 1e3
        assert all(e.time()["ncycle"] == cycles and e.status() == 0 for e in es)
        for e in es:
            e.close()

    def jobs_h(ms):
        return njobs * 3600.0 / (ms * 1e-3)

    eb32 = sum(element_bytes(m, 1)[0] * m.numelc for m in models)
    ach = eb32 / (conc[1] * 1e-3 / cycles) / 1e9
    return {
        "metric": "jobs/h",
        "value": jobs_h(conc[1]),
        "unit": "jobs/h",
        "n_gpus": 1,
        "steps": cycles,
        "warmup": 0,
        "ms_per_step": conc[1] / cycles,
        "higher_is_better": True,
        "dtype": "f32 element / f64 nodal",
        "data": "synthetic (64 seeded crash-box variants)",
        "config": {"workload": "crash_box_sweep_64", "jobs": njobs, "elements": ne,
                   "elements_per_job": [min(m.numelc for m in models),
                                        max(m.numelc for m in models)],
                   "cycles_per_job": cycles,
                   "timing": "every job run at full length from a fresh model, in every "
                             "arm; device time (CUDA events) for the sequential and batched "
                             "arms, wall time for the concurrent arm"},
        "batched_mixed": {"jobs_h": jobs_h(bat[1]["ms"]),
                          "element_updates_s": ne * cycles / (bat[1]["ms"] * 1e-3),
                          "autotuned": bat[1]["cfg"], "all_at_target": bat[1]["all_at_target"]},
        "batched_fp64": {"jobs_h": jobs_h(bat[0]["ms"]),
                         "element_updates_s": ne * cycles / (bat[0]["ms"] * 1e-3),
                         "autotuned": bat[0]["cfg"], "all_at_target": bat[0]["all_at_target"]},
        "sequential_fp64": {"jobs_h": jobs_h(seq[0]),
                            "element_updates_s": ne * cycles / (seq[0] * 1e-3)},
        "sequential_mixed": {"jobs_h": jobs_h(seq[1]),
                             "element_updates_s": ne * cycles / (seq[1] * 1e-3)},
        "concurrent_streams_fp64": {"jobs_h": jobs_h(conc[0]), "gain_vs_sequential": seq[0] / conc[0]},
        "concurrent_streams_mixed": {"jobs_h": jobs_h(conc[1]), "gain_vs_sequential": seq[1] / conc[1],
                                     "note": "the line's value: each job its own graph and stream "
                                             "(batch.run_concurrent), interleaved chunks of 100 "
                                             "cycles; wall time"},
        "batching_gain_fp64": seq[0] / bat[0]["ms"],
        "batching_gain_mixed": seq[1] / bat[1]["ms"],
        "speedup_vs_sequential_plain": seq[0] / conc[1],
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                     "frac": ach / hbm_peak, "peak_kind": peak_kind,
                     "note": "concurrent mixed cycles: shell element-phase algorithmic bytes "
                             "over the whole run's time"},
        "clocks": bat[1]["clocks"],
        "device_status": [bat[0]["status"], bat[1]["status"], bat[0]["status_jobs"],
                          bat[1]["status_jobs"]],
    }


SERVE_JOBS = 32
SERVE_RATE = 4.0          # Poisson arrivals, jobs/s
SERVE_BUDGET = 48 << 30   # HBM budget of the serving loop (bytes)
SERVE_ELEMENTS = 400_000  # elements in flight of the least-work-first batched policy
SERVE_STREAM_ELEMENTS = 400_000  # elements in flight of the streams executor


def run_serving(args, njobs=SERVE_JOBS, device=0):
    """Serving stream: njobs seeded requests (50/50 shell crash boxes and
    hexa impact blocks of 21k-180k elements, 3,000-20,000 cycles each)
    arriving as a Poisson process of SERVE_RATE jobs/s, admitted by HBM
    budget and served in the mixed form -- each job on its own graph and
    stream (the line's value), and by the batched kernel under two policies.
    Beside it the same jobs run alone one after another at full length, in
    the plain FP64 form and in the mixed form (device time of every job)."""
    from openradioss_gb300.engine import Engine
    from openradioss_gb300.serving import Server, poisson_arrivals
    jobs = [M.serving_job(k) for k in range(njobs)]
    arr = poisson_arrivals(njobs, SERVE_RATE, seed=7)
    seq, per_job = {}, {}
    for prec in (0, 1):
        ts = []
        for m, n in jobs:
            e = Engine(m, device=device, precision=prec)
            ts.append(e.time_cycles(n) * 1e-3)
            e.close()
        per_job[prec] = ts
        seq[prec] = sum(ts)

    def fifo_latency(ts):
        """Latencies of a server running one job at a time, first come first
        served, on the same arrivals (each job taking its measured time)."""
        free, lat = 0.0, []
        for a, t in sorted(zip(arr, ts)):
            start = max(free, float(a))
            free = start + t
            lat.append(free - float(a))
        return float(np.percentile(lat, 50)), float(np.percentile(lat, 99))
    reqs = [(k, m, n, float(a)) for k, ((m, n), a) in enumerate(zip(jobs, arr))]

    def serve(**kw):
        srv = Server(SERVE_BUDGET, max_jobs=64, precision=1, step_cycles=100, device=device,
                     **kw)
        st = srv.run(reqs)
        st["bad"] = sum(1 for r in srv.done if r.result.get("status", 0)) + len(srv.failed)
        srv.close()
        return st
    # the served line: each job its own single-model graph and stream (these
    # jobs fill the GPU alone: the batched kernel gains them nothing), first
    # come first served, at most SERVE_STREAM_ELEMENTS elements in flight
    with Clocks(device) as clk:
        st = serve(policy="fifo", max_elements=SERVE_STREAM_ELEMENTS, executor="streams")
    # the batched executor on the same stream: every arrived job admitted
    # (arrival order, HBM budget only), and least work first under an
    # element cap
    st_all = serve(executor="batch")
    st_sjf = serve(policy="sjf", max_elements=SERVE_ELEMENTS, executor="batch")
    bad = st["bad"] + st_all["bad"] + st_sjf["bad"]
    seq_jobs_h = {p: 3600.0 * njobs / seq[p] for p in seq}
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
                   "hbm_budget_gb": SERVE_BUDGET / 2 ** 30, "step_cycles": 100,
                   "policy": "each job its own graph and stream, first come first served, "
                             "at most %d elements in flight" % SERVE_STREAM_ELEMENTS,
                   "sequential": "every job run alone at full length (device time)"},
        "completed": st["completed"], "failed": st["failed"],
        "p50_latency_s": st["p50_latency_s"],
        "p99_latency_s": st["p99_latency_s"],
        "mean_latency_s": st["mean_latency_s"],
        "makespan_s": st["makespan_s"],
        "element_updates_s": st["element_updates"] / st["makespan_s"],
        "max_used_gb": st["max_used_bytes"] / 2 ** 30,
        "sequential_fp64_jobs_h": seq_jobs_h[0],
        "sequential_mixed_jobs_h": seq_jobs_h[1],
        "batched_admit_all_arrival_order": {"jobs_h": st_all["jobs_per_h"],
                                            "p50_latency_s": st_all["p50_latency_s"],
                                            "p99_latency_s": st_all["p99_latency_s"]},
        "batched_least_work_first": {"jobs_h": st_sjf["jobs_per_h"],
                                     "p50_latency_s": st_sjf["p50_latency_s"],
                                     "p99_latency_s": st_sjf["p99_latency_s"],
                                     "policy": "at most %d elements in flight" % SERVE_ELEMENTS},
        "fifo_one_at_a_time_latency_s": {
            "fp64": dict(zip(("p50", "p99"), fifo_latency(per_job[0]))),
            "mixed": dict(zip(("p50", "p99"), fifo_latency(per_job[1]))),
            "note": "the same arrivals served one job at a time, first come first served, "
                    "each job taking its measured solo device time"},
        "speedup_vs_sequential_plain": st["jobs_per_h"] / seq_jobs_h[0],
        "speedup_vs_sequential_mixed": st["jobs_per_h"] / seq_jobs_h[1],
        "jobs_with_device_status": bad,
        "clocks": clk.summary(),
    }


def reference_gpu_shell(model, args, device, ours_kt):
    """Baseline leg: the reference's own CUDA shell path (its unmodified
    shell_*_kernel.cu and shell_gpu_driver.cu, built for sm_103a in double
    precision; oracle/ref_gpu.py) timed on this GPU on the same shells and
    node state as ours -- a speed comparator, not a parity check.  Two
    states, each held fixed for W + K steps as in a FORINT-level call: the
    state of the timed window (W cycles after set-up) and the same with a
    seeded N(0, 2 m/s) velocity perturbation, under which the points go
    plastic.  Beside each: our FORINT-level call (rg_forint_step: the same
    uploads, elements with PARITH/ON assembly, the same downloads) on the
    same state, and our element kernel's device time per cycle."""
    import tempfile
    from openradioss_gb300.engine import Engine
    from oracle import ref_gpu
    why = ref_gpu.available()
    if why:
        return {"unavailable": why}
    g = model.shells[0]
    mt = g.mat
    e = Engine(model, device=device, precision=0)
    e.cycle(args.warmup)
    nd = e.nodes()
    dt = e.time()["dt2"]
    e.close()
    pm = mt["pm"]
    rng = np.random.default_rng(11)
    out = {"what": "reference CUDA shell path (shell_gpu_driver.h:302-477, MYREAL8, ISMSTR=2, "
                   "IPLA=1, NPT=5) vs ours on the same shells and fixed node state",
           "numelc": model.numelc, "steps": args.steps}
    for name, dv in (("window_state", 0.0), ("perturbed_plastic", 2.0)):
        X = np.ascontiguousarray(nd["X"].T)
        V = np.ascontiguousarray(nd["V"].T + (rng.normal(0.0, dv, nd["V"].T.shape) if dv else 0.0))
        VR = np.ascontiguousarray(nd["VR"].T)
        req = dict(ixc4=(g.ixc[1:5] - 1).astype(np.int32), thk=g.thk, X=X, V=V, VR=VR,
                   # E, nu, rho; Johnson-Cook A, B, n, C, eps0 (mat_param%uparam 1-3, 6-7)
                   mat=np.array([pm[19], pm[20], pm[0], mt["uparam"][0], mt["uparam"][1],
                                 mt["uparam"][2], mt["uparam"][5], mt["uparam"][6]]),
                   # membrane, flexural, rotational hourglass (GEO(13:15))
                   hg=np.array([g.geo[12], g.geo[13], g.geo[14]]), dt=dt, nwarm=args.warmup,
                   nsteps=args.steps)
        with tempfile.TemporaryDirectory() as td:
            fn = os.path.join(td, "req.npz")
            np.savez(fn, **req)
            r = subprocess.run([sys.executable, "-m", "oracle.ref_gpu", fn], cwd=ROOT,
                               capture_output=True, text=True, timeout=900)
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
        if r.returncode != 0 or not lines:
            out[name] = {"unavailable": "reference comparator exited %d: %s" % (
                r.returncode, (r.stderr or r.stdout).strip().splitlines()[-1:])}
            continue
        ref = json.loads(lines[-1])
        # ours: the FORINT-level call on the same fixed state
        e = Engine(model, device=device, precision=0)
        e.cycle(args.warmup)
        f, fr = np.empty_like(X), np.empty_like(X)
        st, sr = np.empty(model.numnod), np.empty(model.numnod)
        bufs = [X, V, VR, f, fr, st, sr]
        for a in bufs:
            e.host_register(a)
        for _ in range(args.warmup):
            e.forint_step(X, V, dt, vr=VR, f=f, stifn=st, fr=fr, stifr=sr)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e.forint_step(X, V, dt, vr=VR, f=f, stifn=st, fr=fr, stifr=sr)
        ours_ms = 1e3 * (time.perf_counter() - t0) / args.steps
        for a in bufs:
            e.host_unregister(a)
        e.close()
        d = {"reference_kernels_ms_per_step": ref["kernels_ms_per_step"],
             "reference_full_step_ms": ref["full_step_ms"],
             "ours_forint_step_ms": ours_ms,
             "speedup_full_step": ref["full_step_ms"] / ours_ms}
        if name == "window_state":
            # the reference's kernels include the (atomic) assembly; ours
            # assembles in the node kernel, which also does the nodal update
            both = ours_kt["shell"] + ours_kt["node"]
            d["ours_shell_kernel_ms"] = ours_kt["shell"]
            d["ours_shell_plus_node_kernel_ms"] = both
            d["speedup_kernels"] = ref["kernels_ms_per_step"] / both
        out[name] = d
    return out


def cpu_window(wl, warmup, steps, threads=None):
    """Time the CPU restatement (oracle/) on the host cores over the GPU's
    timed window: a fresh model, W warm-up cycles, then K timed cycles."""
    from oracle.oracle import OracleModel
    model = WORKLOADS[wl]()
    nt = threads or os.cpu_count() or 1
    o = OracleModel(model, nthreads=nt)
    o.cycle(warmup)
    t0 = time.perf_counter()
    o.cycle(steps)
    dt = time.perf_counter() - t0
    ne = model.numels + model.numelc
    return model, nt, dt, ne * steps / dt


def cpu_baseline(wl, warmup, steps):
    model, nt, dt, v = cpu_window(wl, warmup, steps)
    return {"value": v, "unit": "element-updates/s", "cores": nt, "kind": "port",
            "sample": "%s, cycles %d-%d of a fresh model (the GPU's timed window), %.1f s"
                      % (wl, warmup + 1, warmup + steps, dt)}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    wl = args.workload
    model, nt, dt, v = cpu_window(wl, args.warmup, args.steps)
    return {"metric": "element-updates/s", "value": v, "unit": "element-updates/s",
            "impl": "reference", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh and velocity "
            "field of the named shape)",
            "config": workload_config(wl, model, world),
            "cpu_baseline": {"value": v, "unit": "element-updates/s", "cores": nt, "kind": "port",
                             "sample": "%s, cycles %d-%d of a fresh model" % (
                                 wl, args.warmup + 1, args.warmup + args.steps)},
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
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other single-GPU configurations' summaries")
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
    if rank == 0 and world == 1 and args.forms == "both":
        if not args.no_configs:
            line["configs"] = {w: workload_summary(w, args, local_rank, not args.no_job)
                               for w in WORKLOADS if w != args.workload}
        if not args.no_sweep:
            sw = run_sweep(args)
            line["batched_sweep"] = {k: sw[k] for k in (
                "value", "unit", "batched_mixed", "batched_fp64", "sequential_fp64",
                "sequential_mixed", "batching_gain_fp64", "batching_gain_mixed",
                "concurrent_streams_fp64", "concurrent_streams_mixed",
                "speedup_vs_sequential_plain", "config", "device_status", "roofline")}
            sv = run_serving(args)
            line["serving"] = {k: sv[k] for k in (
                "value", "unit", "completed", "failed", "p50_latency_s", "p99_latency_s",
                "sequential_fp64_jobs_h", "sequential_mixed_jobs_h",
                "fifo_one_at_a_time_latency_s", "batched_admit_all_arrival_order",
                "batched_least_work_first",
                "speedup_vs_sequential_plain", "speedup_vs_sequential_mixed",
                "element_updates_s", "makespan_s", "config", "jobs_with_device_status")}
    if rank == 0:
        print(json.dumps(line, default=float), flush=True)
    if world > 1:
        import torch.distributed as tdist
        tdist.barrier()
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
