"""Serving loop: simulation jobs admitted by HBM budget and advanced together
(continuous batching) on one GPU.

Requests (a model plus a cycle count) arrive over time.  Between two steps
of ``step_cycles`` cycles the loop

* admits waiting requests, in arrival order, while a job slot is free and
  the job's estimated device bytes fit the remaining HBM budget -- the job's
  model is uploaded to the device (its state then stays there) and it joins
  the running jobs with its own cycle target;
* retires the jobs whose cycle count reached their target: their results are
  read back, their device memory is released, and the freed slot and bytes go
  to the next waiting requests;
* retires as failed, at once, a job whose own device status word is raised
  (negative volume, non-finite acceleration, time step below its minimum:
  the conditions on which the reference engine stops its run) -- the other
  jobs share no data with it and go on unchanged.  A batch-level failure (a
  grid barrier that gave up) voids the step for every running job: they are
  all retired as failed, and the server goes on with the waiting requests.

While the GPU runs a step, the host prepares the next admissions (upload
and set-up), so requests that arrive while others are on the GPU overlap
with them.  With the streams executor each job's results are bit for bit
those of the job run alone; with the batch executor they equal them within
the parity tolerance (the batched kernel runs the same element and node
functions; the compiler may contract multiply-adds differently in the two
kernels) and are bitwise the same whatever the batch's launch configuration
or neighbours -- all of which the tests check.

With preemption on, a request may carry a priority: when an arrived request
does not fit (slot or budget) and jobs of lower priority are running, the
lowest-priority running jobs (the most cycles left first) are preempted --
their whole device state is snapshotted to host memory (rg_snapshot), their
device memory released -- until it fits; a preempted job waits in the queue
with its snapshot and resumes from it (rg_restore) bit for bit, the batched
kernel's results not depending on what else is in the batch.

Two executors.  "streams" (the default) advances each running job with its
own single-model CUDA graph on its own stream (rg_cycle, asynchronous): jobs
large enough to fill the GPU by themselves run at their solo speed, and the
kernels of concurrent jobs overlap where one leaves SMs idle.  "batch"
advances the running jobs together in one batched persistent kernel per
cycle, a job's results then not depending on what else runs beside it.  Admission, retirement, failure
isolation and preemption are the same in both.

The latency of a job is its completion time minus its arrival time; the
loop reports jobs/h and the p50 / p99 latencies.
"""
from __future__ import annotations

import heapq
import time
from dataclasses import dataclass, field

import numpy as np

from .batch import Batch
from .engine import Engine, RG_PREC_MIXED


def estimate_device_bytes(model, precision=RG_PREC_MIXED):
    """Upper estimate of the device bytes an Engine of this model holds
    (element state, connectivity, skyline slots, node records, staging).
    Admission uses it before the job is uploaded."""
    er = 8 if precision == 0 else 4
    slot = 32 if precision == 0 else 16
    nn = model.numnod
    b = 0
    if model.numels:
        ne = model.numels
        # SIG 6, QVIS, OFF, PLA, EPSD (ER); EINT, RHO, VOL0, EHOU (FP64);
        # NC, IADS (8 int32 each), user id, slots, dt partials
        b += ne * (er * 10 + 8 * 4 + 64 + 4 + 8 * slot + 4) + (ne // 128 + 1) * 12
    if model.numelc:
        nc = model.numelc
        npt = model.shells[0].npt
        # FOR 5, MOM 3, HOUR 5, GSTR 8, OFF, THKE, EPSDG (ER), THK, EINT 2,
        # EHOU (FP64), per point SIG 5, PLA, EPSD; IX, IADC, DEGEN; 2x4 slots
        b += nc * (er * (24 + 7 * npt) + 8 * 4 + 36 + 8 * slot + 4) + (nc // 128 + 1) * 12
    rot = model.numelc > 0
    # X4 V4 D4 (+VR4 DR4), FP32 copies, ADSKY, wall index, staging 12 doubles
    b += nn * (96 + (64 if rot else 0) + (48 + (16 if rot else 0) if precision else 0)
               + 4 + 4 + 96)
    return int(1.15 * b) + (1 << 20)


@dataclass(order=True)
class Request:
    arrival: float
    key: int
    model: object = field(compare=False)
    ncycles: int = field(compare=False)
    priority: int = field(default=0, compare=False)
    snapshot: object = field(default=None, compare=False)   # preempted job's state
    record: object = field(default=None, compare=False)     # its JobRecord


@dataclass
class JobRecord:
    key: int
    arrival: float
    admitted: float = 0.0
    finished: float = 0.0
    ncycles: int = 0
    elements: int = 0
    device_bytes: int = 0
    result: dict = field(default_factory=dict)
    failed: bool = False
    status: int = 0
    priority: int = 0
    preemptions: int = 0
    ncycles_done: int = 0   # cycles done when last preempted

    @property
    def latency(self):
        return self.finished - self.arrival


class Server:
    """Continuous-batching server of explicit simulation jobs on one GPU."""

    def __init__(self, hbm_budget_bytes, max_jobs=64, precision=RG_PREC_MIXED,
                 step_cycles=100, device=0, config=None, keep_results=False,
                 result_fn=None, preempt=False, policy="fifo", max_elements=None,
                 executor="streams"):
        """policy: admission order among arrived requests of equal priority,
        "fifo" (arrival) or "sjf" (least work first: elements x cycles
        left).  max_elements: cap on the elements of the running jobs -- a
        single large model already fills the GPU, and admitting more only
        shares it (every job slower) where waiting would finish the first
        ones sooner; a job is always admitted when nothing runs.
        executor: "streams" (each job its own graph and stream; the faster
        on GB300 for every measured workload) or "batch" (one batched
        kernel for all running jobs: results independent of the batch's
        composition bit for bit)."""
        self.budget = int(hbm_budget_bytes)
        self.max_jobs = max_jobs
        self.precision = precision
        self.step_cycles = step_cycles
        self.device = device
        if executor not in ("batch", "streams"):
            raise ValueError("executor must be 'batch' or 'streams'")
        self.executor = executor
        self.batch = Batch(device) if executor == "batch" else None
        if config and self.batch is not None:
            self.batch.set_config(**config)
        self.next_slot = 0
        self.cycles_done = {}  # streams executor: slot -> cycles launched
        self.keep_results = keep_results
        self.result_fn = result_fn
        self.used = 0
        self.preempt = preempt
        if policy not in ("fifo", "sjf"):
            raise ValueError("policy must be 'fifo' or 'sjf'")
        self.policy = policy
        self.max_elements = max_elements
        self.running = {}     # slot -> (Engine, JobRecord, reserved bytes, Request)
        self.waiting = []     # heap of Request not yet arrived (arrival order)
        self.queue = []       # heap of arrived requests: priority, then arrival
        self.done = []
        self.failed = []
        self.max_used = 0

    def submit(self, key, model, ncycles, arrival, priority=0):
        heapq.heappush(self.waiting, Request(arrival, key, model, ncycles, priority))

    def _enqueue(self, req):
        work = 0.0
        if self.policy == "sjf":
            left = req.ncycles - (req.record.ncycles_done if req.record else 0)
            work = float(req.model.numels + req.model.numelc) * max(left, 0)
        heapq.heappush(self.queue, (-req.priority, work, req.arrival, req.key, req))

    def _elements_running(self):
        return sum(r[1].elements for r in self.running.values())

    # ---- executor: the batched kernel or one graph per job ----
    def _sync(self):
        if self.batch is not None:
            self.batch.sync()
        else:
            for e, _, _, _ in self.running.values():
                e.sync()

    def _join(self, e, req):
        if self.batch is not None:
            return self.batch.add(e, req.ncycles)
        slot = self.next_slot
        self.next_slot += 1
        self.cycles_done[slot] = e.time()["ncycle"]
        return slot

    def _leave(self, slot):
        if self.batch is not None:
            self.batch.remove(slot)
        else:
            self.cycles_done.pop(slot, None)

    def _step(self):
        if self.batch is not None:
            self.batch.cycle(self.step_cycles)
            return
        for s, (e, rec, _, _) in self.running.items():
            n = min(self.step_cycles, rec.ncycles - self.cycles_done[s])
            if n > 0:
                e.cycle(n, sync=False)
                self.cycles_done[s] += n

    def _progress(self):
        """({slot: cycles done}, {slot: job status}, batch status)."""
        if self.batch is not None:
            prog, st = self.batch.progress()
            return prog, self.batch.job_status(), st
        self._sync()
        return (dict(self.cycles_done),
                {s: e.status() for s, (e, _, _, _) in self.running.items()}, 0)

    def _victims(self, req, need):
        """Running jobs of lower priority than req whose preemption frees a
        slot and enough budget for it (lowest priority, most cycles left
        first), or None when that is not possible."""
        cands = sorted((s for s, r in self.running.items() if r[3].priority < req.priority),
                       key=lambda s: (self.running[s][3].priority,
                                      -(self.running[s][1].ncycles -
                                        self.running[s][0].time()["ncycle"])))
        out, free, slots = [], self.budget - self.used, self.max_jobs - len(self.running)
        for s in cands:
            if free >= need and slots >= 1:
                break
            out.append(s)
            free += self.running[s][2]
            slots += 1
        return out if (free >= need and slots >= 1) else None

    def _preempt(self, slot):
        """Snapshot a running job to host memory, release its device memory
        and put it back in the queue."""
        self._sync()
        e, rec, need, req = self.running.pop(slot)
        self._leave(slot)
        req.snapshot = e.snapshot()
        req.record = rec
        rec.preemptions += 1
        rec.ncycles_done = e.time()["ncycle"]
        e.close()
        self.used -= need
        self._enqueue(req)

    def _admit(self, now):
        n = 0
        while self.waiting and self.waiting[0].arrival <= now:
            self._enqueue(heapq.heappop(self.waiting))
        while self.queue:
            req = self.queue[0][-1]
            need = estimate_device_bytes(req.model, self.precision)
            if self.running and self.max_elements is not None and \
                    self._elements_running() + req.model.numels + req.model.numelc > \
                    self.max_elements:
                break
            if self.used + need > self.budget or len(self.running) >= self.max_jobs:
                if not self.running and self.used + need > self.budget:
                    raise RuntimeError("job %d needs %d bytes, more than the whole budget %d"
                                       % (req.key, need, self.budget))
                vict = self._victims(req, need) if self.preempt else None
                if not vict:
                    break
                for s in vict:
                    self._preempt(s)
            heapq.heappop(self.queue)
            e = Engine(req.model, device=self.device, precision=self.precision)
            if req.snapshot is not None:
                e.restore(req.snapshot)   # resume where it was preempted
                req.snapshot = None
                rec = req.record
            else:
                rec = JobRecord(req.key, req.arrival, admitted=self._clock(),
                                ncycles=req.ncycles,
                                elements=req.model.numels + req.model.numelc,
                                device_bytes=e.info()["device_bytes"], priority=req.priority)
            slot = self._join(e, req)
            self.running[slot] = (e, rec, need, req)
            self.used += need
            self.max_used = max(self.max_used, self.used)
            n += 1
        return n

    def _retire(self, prog):
        fin = [s for s, (e, rec, need, _) in self.running.items()
               if prog.get(s, -1) >= rec.ncycles]
        if not fin:
            return 0
        self._sync()
        now = self._clock()
        for s in fin:
            e, rec, need, _ = self.running.pop(s)
            self._leave(s)
            rec.finished = now
            if self.result_fn is not None:
                rec.result = self.result_fn(e)
            elif self.keep_results:
                nd = e.nodes()
                rec.result = dict(X=nd["X"], V=nd["V"], time=e.time(), energy=e.energy(),
                                  status=e.status())
            else:
                rec.result = dict(time=e.time(), energy=e.energy(), status=e.status())
            e.close()
            self.used -= need
            self.done.append(rec)
        return len(fin)

    def _retire_failed(self, jstat, bstatus):
        """Retire, as failed, every job whose status word is raised (every
        running job when the batch status is): removed from the batch,
        memory released, record kept with its status."""
        bad = [s for s in self.running if bstatus or jstat.get(s, 0)]
        if not bad:
            return 0
        self._sync()
        now = self._clock()
        for s in bad:
            e, rec, need, _ = self.running.pop(s)
            self._leave(s)
            rec.finished = now
            rec.failed = True
            rec.status = int(jstat.get(s, 0)) | int(bstatus)
            rec.result = dict(time=e.time(), status=rec.status)
            e.status()  # clear the word the job's context kept
            e.close()
            self.used -= need
            self.failed.append(rec)
        return len(bad)

    def _clock(self):
        return time.perf_counter() - self.t0

    def run(self, requests):
        """Serve ``requests`` -- (key, model, ncycles, arrival seconds) --
        arriving on the wall clock from now; returns the statistics."""
        for r in requests:
            self.submit(*r)
        total = len(self.waiting)
        self.t0 = time.perf_counter()
        steps = 0
        while len(self.done) + len(self.failed) < total:
            now = self._clock()
            if self.running:
                # launch a step; admissions prepared meanwhile overlap with it
                self._step()
                steps += 1
                self._admit(self._clock())
                prog, jst, st = self._progress()
                self._retire_failed(jst, st)
                self._retire(prog)
            else:
                if not self.queue and self.waiting and self.waiting[0].arrival > now:
                    time.sleep(min(0.05, self.waiting[0].arrival - now))
                self._admit(self._clock())
        makespan = self._clock()
        lat = np.array([r.latency for r in self.done]) if self.done else np.zeros(1)
        ok = len(self.done)
        return dict(jobs=total, completed=ok, failed=len(self.failed), makespan_s=makespan,
                    jobs_per_h=3600.0 * ok / makespan,
                    p50_latency_s=float(np.percentile(lat, 50)),
                    p99_latency_s=float(np.percentile(lat, 99)),
                    mean_latency_s=float(lat.mean()), steps=steps,
                    max_used_bytes=self.max_used, budget_bytes=self.budget,
                    element_updates=float(sum(r.elements * r.ncycles for r in self.done)))

    def close(self):
        for s, (e, rec, need, _) in list(self.running.items()):
            self._leave(s)
            e.close()
        self.running.clear()
        if self.batch is not None:
            self.batch.close()


def poisson_arrivals(n, rate, seed=7):
    """n arrival times of a Poisson process of the given rate (1/s)."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))
