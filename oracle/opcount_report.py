"""Algorithmic FP64 operation counts of the explicit cycle -- MEASUREMENT
INFRASTRUCTURE (test / benchmark support, never part of the product).

Runs the op-counting build of the oracle (rg_opcount.h: the oracle's own
sources with every double replaced by a counting scalar, one thread) and
writes, per element (hexa / shell phases) and per node (assembly + nodal
update), the number of FP64 additions/subtractions, multiplications,
divisions, square roots, pow / log / exp calls, comparisons and min/max
selections the reference algorithm performs, for

* the benchmark windows: the cycles bench.py times (5 cycles after set-up,
  then 20) on the crash box of 120,120 shells and the 128^3 hexa block, and
  the 1,000-cycle bar impact;
* one branch at a time, on small cases where every element is in it:
  hexa LAW1, hexa LAW2 elastic and plastic, shell NPT=5 Iplas=1 elastic and
  plastic.

flops = add + mul + div + sqrt + pow + log + exp (each one operation, the
usual convention); comparisons and min/max are listed apart.  Output:
profiles/fp64_op_counts.json (read by bench.py for its FP64-pipe roofline).

Usage: python oracle/opcount_report.py [--quick]
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from openradioss_gb300 import model as M  # noqa: E402
from oracle.oracle import OracleModel, count_lib  # noqa: E402

OPS = ["add", "mul", "div", "sqrt", "pow", "log", "exp", "trig", "cmp", "minmax"]
FLOP_OPS = ["add", "mul", "div", "sqrt", "pow", "log", "exp", "trig"]
PHASES = ["other", "hexa", "shell", "nodes"]


def counts():
    L = count_lib()
    a = np.zeros(len(PHASES) * len(OPS), np.int64)
    L.or_opcount_get(a.ctypes.data)
    return a.reshape(len(PHASES), len(OPS))


def window(model, warm, ncyc, plastic_fraction=None):
    """Counts over cycles warm+1 .. warm+ncyc of the model, per unit."""
    L = count_lib()
    o = OracleModel(model, nthreads=1, library=L)
    o.cycle(warm)
    L.or_opcount_reset()
    t0 = time.time()
    o.cycle(ncyc)
    c = counts()
    out = {"cycles": [warm + 1, warm + ncyc], "seconds": round(time.time() - t0, 1)}
    for ph, units in (("hexa", model.numels), ("shell", model.numelc), ("nodes", model.numnod)):
        if units == 0:
            continue
        row = c[PHASES.index(ph)] / float(units * ncyc)
        d = {op: round(float(row[i]), 3) for i, op in enumerate(OPS)}
        d["flops"] = round(float(sum(row[OPS.index(k)] for k in FLOP_OPS)), 3)
        out[ph] = d
    if model.numels:
        pla = o.hexa_state(5)
        out["plastic_elements"] = round(float(np.mean(pla > 0)), 4)
    if model.numelc:
        npt = model.shells[0].npt
        pla = o.shell_state(6, npt * model.numelc)
        out["plastic_points"] = round(float(np.mean(pla > 0)), 4)
    return out


def branch_cases(quick):
    n = 6 if quick else 10
    cases = {}
    cases["hexa_law1"] = window(M.bar_impact(n=n), 5, 10)
    cases["hexa_law2_elastic"] = window(M.large_block(n=n, vmean=1.0, vstd=0.01, seed=2), 5, 10)
    cases["hexa_law2_plastic"] = window(M.large_block(n=n, vmean=150.0, vstd=30.0, seed=2), 40, 10)
    cases["shell_npt5_iplas1_elastic"] = window(
        M.crash_box(n_side=4, n_len=8, v0=0.5, vpert=0.01), 5, 10)
    cases["shell_npt5_iplas1_plastic"] = window(
        M.crash_box(n_side=4, n_len=8, v0=40.0, vpert=60.0), 60, 10)
    return cases


def main():
    quick = "--quick" in sys.argv
    rep = {"what": "algorithmic FP64 operations per unit of the reference algorithm "
                   "(op-counting build of the CPU oracle, one thread)",
           "command": "python oracle/opcount_report.py",
           "flops": "add + mul + div + sqrt + pow + log + exp + trig, one each",
           "windows": {}, "branches": branch_cases(quick)}
    if not quick:
        rep["windows"]["crash_box_120k_jc"] = window(M.crash_box(n_side=77, n_len=390), 5, 20)
        rep["windows"]["hexa_block_128_jc"] = window(M.large_block(n=128), 5, 20)
        rep["windows"]["bar_impact_20_law1"] = window(M.bar_impact(n=20), 5, 20)
    out = os.path.join(ROOT, "profiles", "fp64_op_counts.json")
    if not quick:
        with open(out, "w") as f:
            json.dump(rep, f, indent=1)
            f.write("\n")
    print(json.dumps(rep, indent=1))


if __name__ == "__main__":
    main()
