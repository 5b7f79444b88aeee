"""Build librg.so (the CUDA hot path + C ABI) in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel with one -gencode (sm_103a),
then linked as a shared library next to this file.  No CMake, no torch
extension machinery: the product is a plain C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librg.so")
SOURCES = ["rg_api.cu", "rg_hexa.cu", "rg_shell.cu", "rg_batch.cu", "rg_noalloc.cu", "rg_parts.cu"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-O2", "--expt-relaxed-constexpr"]
# per-source flags: the shell unit's FP32 (mixed-form) arithmetic uses the
# fast single-precision division, square root and transcendentals (38.9 ->
# 36.9 us per crash-box cycle, errors against the FP64 form still within the
# mixed form's bound); its FP64 kernels are unchanged by these flags, which
# apply to single precision only (the FP64 results are bitwise the same)
TU_FLAGS = {"rg_shell.cu": ["--use_fast_math"]}


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librg.so")
    return p


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
               if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "rg_api.h"))
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _newer(o, [s] + headers + [os.path.abspath(__file__)]):
            cmd = [nvcc()] + GENCODE + FLAGS + TU_FLAGS.get(src, []) + ["-c", s, "-o", o]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
        for j, f in zip(jobs, futs):
            r = f.result()
            if verbose or ptxas_info:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(j), r.stderr))
    if force or jobs or _newer(LIB, objs):
        cmd = [nvcc()] + GENCODE + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr)
    return LIB


def build_fortran(fc=None):
    """Compile the Fortran ISO_C_BINDING module include/rg_api_mod.F90 (the
    interface a Fortran engine uses) when asked (RG_FORTRAN=1) and a Fortran
    compiler is present ($FC, else gfortran / flang / ifx / nvfortran).
    Returns the object file, or None when skipped."""
    if os.environ.get("RG_FORTRAN") != "1":
        return None
    fc = fc or os.environ.get("FC") or next(
        (c for c in ("gfortran", "flang", "ifx", "nvfortran") if shutil.which(c)), None)
    if not fc:
        raise RuntimeError("RG_FORTRAN=1 but no Fortran compiler found")
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "..", "include", "rg_api_mod.F90")
    obj = os.path.join(OUT, "rg_api_mod.o")
    subprocess.run([fc, "-c", src, "-o", obj, "-J" if "gfortran" in fc else "-module", OUT],
                   check=True)
    return obj


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                ptxas_info="--ptxas" in sys.argv))
