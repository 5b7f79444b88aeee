"""Python host mirror of the batched-jobs C ABI (rg_batch_* in
include/rg_api.h).

A :class:`Batch` advances many :class:`~openradioss_gb300.engine.Engine`
models of one arithmetic form together -- one persistent cooperative kernel
per cycle on the GPU, captured in a CUDA graph -- each with its own time step
and cycle target.  Launch shapes come from :meth:`Batch.autotune`, which
times candidate configurations on the batch's own jobs (state saved and
restored) and keeps the fastest; :func:`tuned_config` caches the choice per
workload signature in a JSON file.

:func:`run_concurrent` is the other way to advance many jobs: each job's own
single-model CUDA graph on its own stream, launched in interleaved chunks so
that the GPU runs the jobs' kernels side by side.  On GB300 it is the faster
of the two for a sweep of 5k-60k-element crash boxes (the batched kernel
keeps its results independent of the batch's composition and launch shape
bit for bit; concurrent graphs give each job exactly its solo results).
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from . import _lib
from .engine import RgError

ST_BARRIER = 16


class Batch:
    """Jobs (Engines) advanced together on one GPU."""

    def __init__(self, device=0):
        self.L = _lib.lib()
        h = C.c_void_p()
        r = self.L.rg_batch_create(device, C.byref(h))
        if r != 0:
            raise RgError("rg_batch_create failed (%d): no usable CUDA device %d" % (r, device))
        self.h = h
        self.slots = {}  # slot -> Engine

    def _chk(self, r, what):
        if r < 0:
            raise RgError("%s failed (%d): %s" % (what, r,
                                                  self.L.rg_batch_last_error(self.h).decode()))
        return r

    def add(self, engine, target_ncycle=-1):
        """Add a job; it advances until its cycle count reaches
        target_ncycle (< 0: no target).  Returns its slot."""
        s = self._chk(self.L.rg_batch_add(self.h, engine.h, int(target_ncycle)), "rg_batch_add")
        self.slots[s] = engine
        return s

    def remove(self, slot):
        self._chk(self.L.rg_batch_remove(self.h, slot), "rg_batch_remove")
        return self.slots.pop(slot)

    def set_target(self, slot, target_ncycle):
        self._chk(self.L.rg_batch_set_target(self.h, slot, int(target_ncycle)),
                  "rg_batch_set_target")

    def set_config(self, ktile=1, knode=1, blocks_per_sm=0, schedule=0):
        self._chk(self.L.rg_batch_set_config(self.h, ktile, knode, blocks_per_sm, schedule),
                  "rg_batch_set_config")

    def config(self):
        c = (C.c_int * 5)()
        self._chk(self.L.rg_batch_get_config(self.h, c), "rg_batch_get_config")
        return dict(ktile=c[0], knode=c[1], blocks_per_sm=c[2], schedule=c[3],
                    max_blocks_per_sm=c[4])

    def cycle(self, n=1):
        self._chk(self.L.rg_batch_cycle(self.h, int(n)), "rg_batch_cycle")

    def sync(self):
        self._chk(self.L.rg_batch_synchronize(self.h), "rg_batch_synchronize")

    def time_cycles(self, n):
        ms = C.c_double()
        self._chk(self.L.rg_batch_time_cycles(self.h, int(n), C.byref(ms)), "rg_batch_time_cycles")
        return ms.value

    def progress(self):
        """{slot: cycle count} of the jobs and the batch status word."""
        n = max(self.slots) + 1 if self.slots else 1
        nc = np.full(n, -1, np.int32)
        st = C.c_int()
        self._chk(self.L.rg_batch_progress(self.h, nc.ctypes.data_as(C.c_void_p), n,
                                           C.byref(st)), "rg_batch_progress")
        return {s: int(nc[s]) for s in self.slots}, st.value

    def job_status(self):
        """{slot: status word} of the jobs' own contexts (RG_ST_* bits),
        read after the queued cycles and left set."""
        n = max(self.slots) + 1 if self.slots else 1
        st = np.zeros(n, np.int32)
        self._chk(self.L.rg_batch_job_status(self.h, st.ctypes.data_as(C.c_void_p), n),
                  "rg_batch_job_status")
        return {s: int(st[s]) for s in self.slots}

    def set_barrier_test(self, spin_limit=0, late_block=-1, late_us=0):
        """Test hook of the bounded grid barrier (see rg_batch_set_barrier_test);
        the defaults switch it off."""
        self._chk(self.L.rg_batch_set_barrier_test(self.h, int(spin_limit), int(late_block),
                                                    int(late_us)), "rg_batch_set_barrier_test")

    def autotune(self, trial_cycles=5, candidates=None):
        """Time candidate launch configurations ({ktile, knode,
        blocks_per_sm, schedule} rows; None = the built-in list) on this
        batch and keep the fastest.  Returns the chosen configuration."""
        best = (C.c_int * 5)()
        if candidates is None:
            r = self.L.rg_batch_autotune(self.h, trial_cycles, None, 0, best)
        else:
            a = np.ascontiguousarray(np.asarray(candidates, np.int32).reshape(-1, 4))
            r = self.L.rg_batch_autotune(self.h, trial_cycles, a.ctypes.data_as(C.c_void_p),
                                         a.shape[0], best)
        self._chk(r, "rg_batch_autotune")
        return dict(ktile=best[0], knode=best[1], blocks_per_sm=best[2], schedule=best[3],
                    us_per_cycle=best[4])

    def close(self):
        if getattr(self, "h", None):
            self.L.rg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_concurrent(engines, ncycles, chunk=100):
    """Advance every engine by ncycles cycles, each on its own stream with its
    own graph (rg_cycle, asynchronous), in interleaved chunks of at most
    chunk cycles so that all jobs progress together; returns after all of
    them finished.  Each job's results are those of the job run alone."""
    left = int(ncycles)
    while left > 0:
        n = min(chunk, left)
        for e in engines:
            e.cycle(n, sync=False)
        left -= n
    for e in engines:
        e.sync()


def signature(models, precision):
    """Workload signature used as the autotuner cache key: arithmetic form,
    element kinds, job count and total elements rounded to 2 significant
    digits."""
    kinds = sorted({("hexa%d" % g.mat["mtn"]) for m in models for g in m.hexa} |
                   {("shell%d" % g.npt) for m in models for g in m.shells})
    ne = sum(m.numels + m.numelc for m in models)
    return "p%d|%s|jobs%d|ne%.1e" % (precision, ",".join(kinds), len(models), float("%.2g" % ne))


def tuned_config(batch, models, precision, cache_path=None, trial_cycles=5):
    """Autotune ``batch`` once per workload signature; later calls reuse the
    configuration stored in the JSON cache file."""
    key = signature(models, precision)
    cache = {}
    if cache_path and os.path.exists(cache_path):
        try:
            cache = json.load(open(cache_path))
        except Exception:
            cache = {}
    if key in cache:
        c = cache[key]
        batch.set_config(c["ktile"], c["knode"], c["blocks_per_sm"], c["schedule"])
        return dict(c, cached=True)
    c = batch.autotune(trial_cycles)
    if cache_path:
        cache[key] = c
        tmp = cache_path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, cache_path)
    return dict(c, cached=False)
