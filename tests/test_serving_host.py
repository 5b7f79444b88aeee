"""Host logic of the serving loop (admission by HBM budget, arrival order,
retirement, latency statistics) with stand-in engine and batch objects: no
GPU, no library calls."""
import numpy as np
import pytest

from openradioss_gb300 import model as M
from openradioss_gb300 import serving as S


class FakeEngine:
    live = 0
    # model name -> (cycle at which the job's status word is raised, bits)
    fail_at = {}

    def __init__(self, model, device=0, precision=1):
        self.model = model
        self.nc = 0
        self.word = 0
        FakeEngine.live += 1

    def info(self):
        return {"device_bytes": S.estimate_device_bytes(self.model, 1) // 2}

    def time(self):
        return {"ncycle": self.nc}

    def energy(self):
        return {}

    def status(self):
        w, self.word = self.word, 0
        return w

    def snapshot(self):
        return {"nc": self.nc}

    def restore(self, snap):
        self.nc = snap["nc"]

    def cycle(self, n, sync=True):
        # the streams executor's solo graph launches
        if FakeBatch.step_s:
            import time
            time.sleep(FakeBatch.step_s / 4)
        self.nc += n
        f = FakeEngine.fail_at.get(self.model.name)
        if f and self.nc >= f[0]:
            self.word |= f[1]

    def sync(self):
        pass

    def close(self):
        FakeEngine.live -= 1


class FakeBatch:
    def __init__(self, device=0):
        self.slots = {}
        self.max_live = 0

    def set_config(self, **k):
        pass

    def add(self, e, target):
        s = 0
        while s in self.slots:
            s += 1
        self.slots[s] = (e, target)
        self.max_live = max(self.max_live, len(self.slots))
        return s

    def remove(self, s):
        self.slots.pop(s)

    bstatus = 0
    step_s = 0.0   # wall time a step takes (arrivals during running steps)

    def cycle(self, n):
        if FakeBatch.step_s:
            import time
            time.sleep(FakeBatch.step_s)
        for e, t in self.slots.values():
            e.nc = min(t, e.nc + n)
            f = FakeEngine.fail_at.get(e.model.name)
            if f and e.nc >= f[0]:
                e.word |= f[1]

    def progress(self):
        st, FakeBatch.bstatus = FakeBatch.bstatus, 0
        return {s: e.nc for s, (e, t) in self.slots.items()}, st

    def job_status(self):
        return {s: e.word for s, (e, t) in self.slots.items()}

    def sync(self):
        pass

    def close(self):
        pass


@pytest.fixture
def fakes(monkeypatch):
    monkeypatch.setattr(S, "Engine", FakeEngine)
    monkeypatch.setattr(S, "Batch", FakeBatch)
    FakeEngine.live = 0
    FakeEngine.fail_at = {}
    FakeBatch.bstatus = 0
    FakeBatch.step_s = 0.0
    yield
    FakeBatch.step_s = 0.0


def small_jobs():
    return [(k, M.crash_box(n_side=3 + k % 3, n_len=4 + k, seed=k), 50 * (k + 1), 0.0)
            for k in range(6)]


def test_admission_respects_budget(fakes):
    jobs = small_jobs()
    need = [S.estimate_device_bytes(m, 1) for _, m, _, _ in jobs]
    budget = max(need) + min(need)
    srv = S.Server(budget, max_jobs=8, step_cycles=50, executor="batch")
    st = srv.run(jobs)
    assert st["jobs"] == 6 and len(srv.done) == 6
    assert st["max_used_bytes"] <= budget
    assert srv.used == 0 and FakeEngine.live == 0
    assert srv.batch.max_live < 6  # the budget forced waiting


def test_slot_limit_and_order(fakes):
    jobs = small_jobs()
    srv = S.Server(1 << 40, max_jobs=2, step_cycles=50, executor="batch")
    srv.run(jobs)
    assert srv.batch.max_live == 2
    adm = sorted(srv.done, key=lambda r: r.admitted)
    assert [r.key for r in adm] == sorted(r.key for r in adm)  # FIFO admission


def test_failed_job_is_retired_and_others_finish(fakes):
    """A job whose status word is raised (here a non-finite acceleration at
    its cycle 100) is retired as failed at the end of that step, its memory
    released, and every other job still reaches its target."""
    jobs = small_jobs()
    for k, m, n, a in jobs:
        m.name = "job%d" % k
    FakeEngine.fail_at = {"job3": (100, 2)}
    srv = S.Server(1 << 40, max_jobs=8, step_cycles=50, executor="batch")
    st = srv.run(jobs)
    assert st["failed"] == 1 and st["completed"] == 5
    assert [r.key for r in srv.failed] == [3]
    assert srv.failed[0].status == 2 and srv.failed[0].failed
    assert srv.failed[0].result["time"]["ncycle"] == 100
    assert sorted(r.key for r in srv.done) == [0, 1, 2, 4, 5]
    assert all(r.result["time"]["ncycle"] == jobs[r.key][2] for r in srv.done)
    assert srv.used == 0 and FakeEngine.live == 0


def test_batch_failure_retires_the_running_jobs(fakes):
    """A batch-level failure (grid barrier gave up) voids the step of every
    running job: they are retired as failed and the server serves the
    requests that arrive afterwards."""
    jobs = small_jobs()[:2] + [(9, M.crash_box(n_side=3, n_len=4, seed=9), 100, 0.3)]

    class OnceBatch(FakeBatch):
        fired = False

        def cycle(self, n):
            super().cycle(n)
            if not OnceBatch.fired:
                OnceBatch.fired = True
                FakeBatch.bstatus = 16

    S.Batch = OnceBatch
    srv = S.Server(1 << 40, max_jobs=8, step_cycles=50, executor="batch")
    st = srv.run(jobs)
    assert sorted(r.key for r in srv.failed) == [0, 1]
    assert all(r.status & 16 for r in srv.failed)
    assert [r.key for r in srv.done] == [9]
    assert st["completed"] == 1 and srv.used == 0 and FakeEngine.live == 0


def test_priority_request_preempts_and_preempted_job_resumes(fakes):
    """With preemption on, a high-priority request that does not fit the
    budget evicts the lowest-priority running job with the most cycles
    left: that job is snapshotted, its memory released, and it resumes from
    the snapshot later, reaching exactly its cycle count (no work redone)."""
    lo1 = M.crash_box(n_side=4, n_len=8, seed=1)
    lo2 = M.crash_box(n_side=4, n_len=8, seed=2)
    hi = M.crash_box(n_side=4, n_len=8, seed=3)
    need = S.estimate_device_bytes(lo1, 1)
    jobs = [(0, lo1, 2000, 0.0, 0), (1, lo2, 1500, 0.0, 0), (2, hi, 200, 0.05, 5)]
    FakeBatch.step_s = 0.005
    srv = S.Server(2 * need + need // 2, max_jobs=8, step_cycles=50, preempt=True,
                   executor="batch")
    st = srv.run(jobs)
    assert st["completed"] == 3 and st["failed"] == 0
    recs = {r.key: r for r in srv.done}
    assert recs[0].preemptions == 1 and recs[1].preemptions == 0  # most cycles left
    assert recs[2].finished < recs[0].finished
    assert all(r.result["time"]["ncycle"] == jobs[r.key][2] for r in srv.done)
    assert srv.used == 0 and FakeEngine.live == 0
    # without preemption the high-priority job waits for a retirement
    srv2 = S.Server(2 * need + need // 2, max_jobs=8, step_cycles=50, preempt=False,
                    executor="batch")
    srv2.run(jobs)
    r2 = {r.key: r for r in srv2.done}
    assert all(r.preemptions == 0 for r in srv2.done)
    assert r2[2].finished > r2[1].finished


def test_sjf_admits_least_work_first_under_an_element_cap(fakes):
    """With policy sjf and an element cap, arrived requests are admitted in
    order of their work (elements x cycles), never more elements at once than
    the cap (except a single job), and every job completes."""
    big = M.crash_box(n_side=6, n_len=20, seed=1)
    small = [M.crash_box(n_side=3, n_len=4, seed=k) for k in range(2, 5)]
    jobs = [(0, big, 3000, 0.0)] + [(k + 1, m, 200, 0.0) for k, m in enumerate(small)]
    cap = big.numelc  # room for the big job alone, or for the small ones
    srv = S.Server(1 << 40, max_jobs=8, step_cycles=50, policy="sjf", max_elements=cap,
                   executor="batch")
    seen = []
    orig = srv._admit

    def spy(now):
        n = orig(now)
        seen.append(srv._elements_running())
        return n
    srv._admit = spy
    st = srv.run(jobs)
    assert st["completed"] == 4
    assert max(seen) <= cap
    adm = sorted(srv.done, key=lambda r: r.admitted)
    assert adm[-1].key == 0  # the large job goes last
    fin = {r.key: r.finished for r in srv.done}
    assert max(fin[k] for k in (1, 2, 3)) < fin[0]


def test_oversize_job_is_refused(fakes):
    jobs = small_jobs()[:1]
    srv = S.Server(1000, max_jobs=2, executor="batch")
    with pytest.raises(RuntimeError):
        srv.run(jobs)


def test_estimate_grows_with_size():
    a = S.estimate_device_bytes(M.crash_box(n_side=4, n_len=8), 1)
    b = S.estimate_device_bytes(M.crash_box(n_side=8, n_len=16), 1)
    c = S.estimate_device_bytes(M.crash_box(n_side=8, n_len=16), 0)
    assert b > a and c > b


def test_poisson_arrivals_seeded():
    a = S.poisson_arrivals(1000, 4.0, seed=7)
    assert np.all(np.diff(a) > 0)
    assert abs(1000 / a[-1] - 4.0) < 0.4
    assert np.array_equal(a, S.poisson_arrivals(1000, 4.0, seed=7))


def test_streams_executor(fakes):
    """Each job on its own graph: the same admission by budget, every job
    done with exactly its cycle count, a failed job retired alone."""
    jobs = small_jobs()
    FakeEngine.fail_at = {jobs[2][1].name: (60, 8)}
    need = [S.estimate_device_bytes(m, 1) for _, m, _, _ in jobs]
    budget = max(need) + min(need)
    srv = S.Server(budget, max_jobs=8, step_cycles=40, executor="streams", keep_results=False)
    assert srv.batch is None
    st = srv.run(jobs)
    assert st["completed"] == 5 and st["failed"] == 1
    assert st["max_used_bytes"] <= budget
    assert [r.key for r in srv.failed] == [2] and srv.failed[0].status == 8
    for r in srv.done:
        assert r.result["time"]["ncycle"] == r.ncycles
    assert srv.used == 0 and FakeEngine.live == 0


def test_streams_executor_preemption(fakes):
    FakeBatch.step_s = 0.02
    lo = [(0, M.crash_box(n_side=5, n_len=10, seed=1), 4000, 0.0, 0),
          (1, M.crash_box(n_side=5, n_len=11, seed=2), 4000, 0.0, 0)]
    hi = (2, M.crash_box(n_side=5, n_len=10, seed=3), 200, 0.05, 1)
    need = max(S.estimate_device_bytes(j[1], 1) for j in lo + [hi])
    srv = S.Server(int(2.5 * need), max_jobs=8, step_cycles=40, executor="streams",
                   preempt=True)
    st = srv.run(lo + [hi])
    assert st["completed"] == 3
    recs = {r.key: r for r in srv.done}
    assert recs[0].preemptions + recs[1].preemptions >= 1
    assert recs[2].finished < max(recs[0].finished, recs[1].finished)
    for r in srv.done:
        assert r.result["time"]["ncycle"] == r.ncycles
