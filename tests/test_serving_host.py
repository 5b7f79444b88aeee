"""Host logic of the serving loop (admission by HBM budget, arrival order,
retirement, latency statistics) with stand-in engine and batch objects: no
GPU, no library calls."""
import numpy as np
import pytest

from openradioss_gb300 import model as M
from openradioss_gb300 import serving as S


class FakeEngine:
    live = 0

    def __init__(self, model, device=0, precision=1):
        self.model = model
        self.nc = 0
        FakeEngine.live += 1

    def info(self):
        return {"device_bytes": S.estimate_device_bytes(self.model, 1) // 2}

    def time(self):
        return {"ncycle": self.nc}

    def energy(self):
        return {}

    def status(self):
        return 0

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

    def cycle(self, n):
        for e, t in self.slots.values():
            e.nc = min(t, e.nc + n)

    def progress(self):
        return {s: e.nc for s, (e, t) in self.slots.items()}, 0

    def sync(self):
        pass

    def close(self):
        pass


@pytest.fixture
def fakes(monkeypatch):
    monkeypatch.setattr(S, "Engine", FakeEngine)
    monkeypatch.setattr(S, "Batch", FakeBatch)
    FakeEngine.live = 0
    yield


def small_jobs():
    return [(k, M.crash_box(n_side=3 + k % 3, n_len=4 + k, seed=k), 50 * (k + 1), 0.0)
            for k in range(6)]


def test_admission_respects_budget(fakes):
    jobs = small_jobs()
    need = [S.estimate_device_bytes(m, 1) for _, m, _, _ in jobs]
    budget = max(need) + min(need)
    srv = S.Server(budget, max_jobs=8, step_cycles=50)
    st = srv.run(jobs)
    assert st["jobs"] == 6 and len(srv.done) == 6
    assert st["max_used_bytes"] <= budget
    assert srv.used == 0 and FakeEngine.live == 0
    assert srv.batch.max_live < 6  # the budget forced waiting


def test_slot_limit_and_order(fakes):
    jobs = small_jobs()
    srv = S.Server(1 << 40, max_jobs=2, step_cycles=50)
    srv.run(jobs)
    assert srv.batch.max_live == 2
    adm = sorted(srv.done, key=lambda r: r.admitted)
    assert [r.key for r in adm] == sorted(r.key for r in adm)  # FIFO admission


def test_oversize_job_is_refused(fakes):
    jobs = small_jobs()[:1]
    srv = S.Server(1000, max_jobs=2)
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
