"""The reference's own CUDA shell path as a speed comparator -- TEST /
BENCHMARK INFRASTRUCTURE, never part of the product and never a parity
oracle.

``python -m oracle.ref_gpu <request.npz>`` builds (make ref_gpu: the
reference's unmodified shell_*_kernel.cu / shell_gpu_driver.cu, copied into
the git-ignored oracle/_ref/src by make ref_src, with our timing harness
ref_shell_gpu_harness.cu) and runs it on the node state and shells of the
request, printing one JSON line: device ms per step of the reference's
kernels (zeroing, geometry, strain and material, forces with atomic
assembly) and wall ms per full step (upload of X, V, VR -> kernels ->
download of the force record).  It runs as its own process because the
reference's error checks call exit().
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libref_shell_gpu.so")
SRC = os.path.join(HERE, "_ref", "src", "shell_gpu_driver.cu")


def available():
    """Why the comparator cannot run, or None."""
    if not os.path.exists(SRC) and not os.path.exists(LIB):
        return "reference CUDA shell sources not staged (make -C oracle ref_src)"
    return None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "ref_gpu"], check=True, capture_output=True)
    return LIB


def run(req):
    L = C.CDLL(build())
    f = L.refgpu_shell_time
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 7 + [C.c_double, C.c_int, C.c_int,
                                                        C.c_void_p]
    ixc4 = np.ascontiguousarray(req["ixc4"], np.int32)
    nc = ixc4.shape[1]
    X, V, VR = (np.ascontiguousarray(req[k], np.float64) for k in ("X", "V", "VR"))
    nn = X.shape[0]
    thk = np.ascontiguousarray(req["thk"], np.float64)
    mat = np.ascontiguousarray(req["mat"], np.float64)
    hg = np.ascontiguousarray(req["hg"], np.float64)
    out = np.zeros(3)
    r = f(nc, nn, ixc4.ctypes.data, thk.ctypes.data, X.ctypes.data, V.ctypes.data,
          VR.ctypes.data, mat.ctypes.data, hg.ctypes.data, float(req["dt"]),
          int(req["nwarm"]), int(req["nsteps"]), out.ctypes.data)
    return {"rc": r, "kernels_ms_per_step": out[0], "full_step_ms": out[1],
            "sum_abs_f": out[2], "numelc": nc, "numnod": nn}


if __name__ == "__main__":
    req = dict(np.load(sys.argv[1]))
    print(json.dumps(run(req)), flush=True)
