"""Batched jobs (one persistent kernel per cycle over many models): every
job's results are bitwise those of the same model stepped alone, under any
launch configuration and schedule, with per-job cycle targets, jobs joining
a running batch, and autotuning (which must leave the state untouched)."""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu


def models_mix():
    return [M.crash_box(n_side=5, n_len=14, v0=12.0, seed=3),
            M.hexa_impact_block(3000, seed=4, law="law2"),
            M.crash_box(n_side=8, n_len=9, v0=18.0, seed=5, thk=1.6e-3),
            M.hexa_impact_block(1500, seed=6, law="law1")]


def state(e):
    nd = e.nodes()
    t = e.time()
    return nd["X"], nd["V"], nd["VR"], t["dt2"], t["ncycle"], t["tt"]


def same(a, b):
    for x, y in zip(a, b):
        if isinstance(x, np.ndarray):
            if not np.array_equal(x, y):
                return False
        elif x != y:
            return False
    return True


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("cfg", [(1, 1, 0, 0), (2, 4, 1, 0), (4, 1, 0, 1), (1, 2, 2, 1)])
def test_batch_equals_alone(prec, cfg):
    from openradioss_gb300.batch import Batch
    from openradioss_gb300.engine import Engine
    ms = models_mix()
    n = 40
    alone = []
    for m in ms:
        e = Engine(m, precision=prec)
        e.cycle(n)
        alone.append(state(e))
    b = Batch()
    b.set_config(*cfg)
    es = [Engine(m, precision=prec) for m in ms]
    for e in es:
        b.add(e)
    b.cycle(n)
    b.sync()
    prog, st = b.progress()
    assert st == 0
    for i, e in enumerate(es):
        assert prog[i] == n
        assert same(state(e), alone[i]), i
        assert e.status() == 0


def test_batch_targets_and_late_join():
    """Jobs stop exactly at their own targets; a job added to a running
    batch advances from its own start and matches its solo run."""
    from openradioss_gb300.batch import Batch
    from openradioss_gb300.engine import Engine
    ms = models_mix()
    tg = [10, 35, 20, 50]
    b = Batch()
    es = [Engine(m, precision=1) for m in ms[:3]]
    for e, t in zip(es, tg):
        b.add(e, t)
    b.cycle(15)
    late = Engine(ms[3], precision=1)
    s3 = b.add(late, tg[3])
    b.cycle(60)
    b.sync()
    prog, st = b.progress()
    assert st == 0
    assert [prog[i] for i in range(3)] == tg[:3]
    assert prog[s3] == tg[3]
    for m, e, t in zip(ms, es + [late], tg):
        ref = Engine(m, precision=1)
        ref.cycle(t)
        assert same(state(e), state(ref))


def test_autotune_leaves_state_unchanged():
    from openradioss_gb300.batch import Batch
    from openradioss_gb300.engine import Engine
    ms = models_mix()
    b = Batch()
    es = [Engine(m, precision=1) for m in ms]
    for e in es:
        b.add(e)
    b.cycle(5)
    cfg = b.autotune(trial_cycles=2, candidates=[[1, 1, 0, 0], [2, 1, 1, 1], [1, 4, 0, 0]])
    assert cfg["ktile"] in (1, 2) and cfg["schedule"] in (0, 1)
    b.cycle(20)
    b.sync()
    for m, e in zip(ms, es):
        ref = Engine(m, precision=1)
        ref.cycle(25)
        assert same(state(e), state(ref))
