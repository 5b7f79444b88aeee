"""Checkpoint / restart of a model on the GPU (rg_snapshot / rg_restore), the
device-resident counterpart of the engine's restart file (WRRESTP,
engine/source/output/restart/wrrestp.F:161):

* a run restored from a snapshot -- into the same context, or into a fresh
  one built from the same model (a restart in another process) -- repeats
  the uninterrupted run bit for bit, in both arithmetic forms, for shells
  (with a rigid wall) and hexas;
* a snapshot of another model is refused;
* a served job preempted by a higher-priority request (snapshot, device
  memory released, resumed later) ends bitwise where the same job ends when
  it is served without interruption.
"""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu


def state(e, m):
    nd = e.nodes()
    out = [nd["X"], nd["V"], nd["VR"], e.forces()["F"]]
    if m.numelc:
        out += [e.shell_state(k, s * m.numelc) for k, s in ((0, 5), (2, 1), (6, 5))]
    if m.numels:
        out += [e.hexa_state(0), e.hexa_state(5)]
    t = e.time()
    out.append(np.array([t["tt"], t["dt2"], t["ncycle"], t["neltst"]]))
    return out


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("kind", ["shell", "hexa"])
def test_restore_resumes_bit_for_bit(kind, prec):
    from openradioss_gb300.engine import Engine
    m = (M.crash_box(n_side=6, n_len=16, v0=20.0, vpert=1.0) if kind == "shell"
         else M.hexa_impact_block(3000, seed=4, law="law2"))
    e = Engine(m, precision=prec)
    e.cycle(30)
    snap = e.snapshot()
    e.cycle(40)
    a = state(e, m)
    e.restore(snap)
    e.cycle(40)
    b = state(e, m)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    # restart in a fresh context built from the same model
    e2 = Engine(m, precision=prec)
    e2.restore(snap)
    e2.cycle(40)
    c = state(e2, m)
    for x, y in zip(a, c):
        assert np.array_equal(x, y)
    assert e.status() == 0 and e2.status() == 0


def test_restore_refuses_another_model():
    from openradioss_gb300.engine import Engine, RgError
    e = Engine(M.crash_box(n_side=6, n_len=16))
    snap = e.snapshot()
    other = Engine(M.crash_box(n_side=6, n_len=18))
    with pytest.raises(RgError):
        other.restore(snap)
    mixed = Engine(M.crash_box(n_side=6, n_len=16), precision=1)
    with pytest.raises(RgError):
        mixed.restore(snap)


def test_preempted_served_job_equals_uninterrupted():
    from openradioss_gb300.serving import Server, estimate_device_bytes
    # three jobs of about the same device footprint in a budget of 2.5 of
    # them: the high-priority arrival finds both low-priority jobs running
    # (each takes seconds) and can only start by preempting one of them
    lo0 = M.crash_box(n_side=5, n_len=10, seed=31)
    lo1 = M.crash_box(n_side=5, n_len=11, seed=32)
    hi = M.crash_box(n_side=5, n_len=10, seed=33)
    sizes = [estimate_device_bytes(x, 1) for x in (lo0, lo1, hi)]
    need = max(sizes)
    assert sum(sizes) > 2.5 * need and sizes[0] + sizes[1] <= 2.5 * need
    jobs = [(0, lo0, 120000, 0.0, 0), (1, lo1, 100000, 0.0, 0), (2, hi, 3000, 0.2, 1)]
    res = {}
    for pre in (True, False):
        srv = Server(int(2.5 * need), max_jobs=8, precision=1, step_cycles=25,
                     keep_results=True, preempt=pre, executor="batch")
        st = srv.run(jobs)
        srv.close()
        assert st["completed"] == 3
        res[pre] = {r.key: r for r in srv.done}
    assert res[True][0].preemptions + res[True][1].preemptions >= 1
    assert all(r.preemptions == 0 for r in res[False].values())
    for k in (0, 1, 2):
        a, b = res[True][k].result, res[False][k].result
        assert a["time"]["ncycle"] == b["time"]["ncycle"] == jobs[k][2]
        assert np.array_equal(a["X"], b["X"]) and np.array_equal(a["V"], b["V"]), k
