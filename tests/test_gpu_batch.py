"""Batched jobs (one persistent kernel per cycle over many models).

* Within the batched kernel, results are bitwise the same under every launch
  configuration and schedule, with jobs joining a running batch, and after
  autotuning (which must leave the state untouched).
* Against the same model stepped alone (the single-model kernels, compiled
  separately: their multiply-add contraction may differ), every job agrees
  within 1e-10 (FP64 form) / 1e-4 (mixed form) relative to its displacement
  and velocity scales, and reaches exactly its own cycle target."""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu

TOL = {0: 1e-10, 1: 1e-4}


def models_mix():
    return [M.crash_box(n_side=5, n_len=14, v0=12.0, seed=3),
            M.hexa_impact_block(3000, seed=4, law="law2"),
            M.crash_box(n_side=8, n_len=9, v0=18.0, seed=5, thk=1.6e-3),
            M.hexa_impact_block(1500, seed=6, law="law1")]


def state(e):
    nd = e.nodes()
    t = e.time()
    return dict(X=nd["X"], V=nd["V"], VR=nd["VR"], D=nd["D"], dt2=t["dt2"],
                ncycle=t["ncycle"], tt=t["tt"])


def bitwise(a, b):
    return all(np.array_equal(a[k], b[k]) if isinstance(a[k], np.ndarray) else a[k] == b[k]
               for k in a)


def close(a, b, tol):
    """b (reference) against a: displacement, velocities and time step."""
    if a["ncycle"] != b["ncycle"]:
        return False
    sd = max(np.max(np.abs(b["D"])), 1e-30)
    sv = max(np.max(np.abs(b["V"])), 1e-30)
    svr = max(np.max(np.abs(b["VR"])), 1e-30)
    return (np.max(np.abs(a["D"] - b["D"])) <= tol * sd and
            np.max(np.abs(a["V"] - b["V"])) <= tol * sv and
            np.max(np.abs(a["VR"] - b["VR"])) <= tol * max(svr, 1e-30) + 0.0 and
            abs(a["dt2"] - b["dt2"]) <= tol * b["dt2"])


def run_batch(ms, prec, n, cfg=None):
    from openradioss_gb300.batch import Batch
    from openradioss_gb300.engine import Engine
    b = Batch()
    if cfg:
        b.set_config(*cfg)
    es = [Engine(m, precision=prec) for m in ms]
    for e in es:
        b.add(e)
    b.cycle(n)
    b.sync()
    prog, st = b.progress()
    assert st == 0
    assert all(prog[i] == n for i in range(len(ms)))
    assert all(e.status() == 0 for e in es)
    return [state(e) for e in es]


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_matches_alone(prec):
    from openradioss_gb300.engine import Engine
    ms = models_mix()
    n = 40
    got = run_batch(ms, prec, n)
    for i, m in enumerate(ms):
        e = Engine(m, precision=prec)
        e.cycle(n)
        assert close(got[i], state(e), TOL[prec]), i


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_bitwise_across_configs(prec):
    ms = models_mix()
    ref = run_batch(ms, prec, 30, (1, 1, 0, 0))
    for cfg in [(2, 4, 1, 0), (4, 1, 0, 1), (1, 2, 2, 1)]:
        got = run_batch(ms, prec, 30, cfg)
        for i in range(len(ms)):
            assert bitwise(got[i], ref[i]), (cfg, i)


def test_batch_targets_and_late_join():
    """Jobs stop exactly at their own targets; a job added to a running
    batch advances from its own start: bitwise equal to the same job in a
    batch from the start, close to its solo run."""
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
        b2 = Batch()
        r = Engine(m, precision=1)
        b2.add(r, t)
        b2.cycle(t + 5)
        b2.sync()
        assert bitwise(state(e), state(r))
        solo = Engine(m, precision=1)
        solo.cycle(t)
        assert close(state(e), state(solo), TOL[1])


def test_autotune_leaves_state_unchanged():
    from openradioss_gb300.batch import Batch
    from openradioss_gb300.engine import Engine
    ms = models_mix()
    ref = run_batch(ms, 1, 25)
    b = Batch()
    es = [Engine(m, precision=1) for m in ms]
    for e in es:
        b.add(e)
    b.cycle(5)
    cfg = b.autotune(trial_cycles=2, candidates=[[1, 1, 0, 0], [2, 1, 1, 1], [1, 4, 0, 0]])
    assert cfg["ktile"] in (1, 2) and cfg["schedule"] in (0, 1)
    b.cycle(20)
    b.sync()
    for i, e in enumerate(es):
        assert bitwise(state(e), ref[i]), i


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_corotational_hexa(prec):
    """Hexa jobs in the co-rotational frame (JCVT = 1, the starter's default
    for Lagrangian bricks) share a batch with Jaumann-rate hexas and shells:
    each agrees with the same model stepped alone, and the batch is bitwise
    the same under another launch configuration."""
    from openradioss_gb300.engine import Engine
    corot = []
    for seed, law in ((21, "law2"), (22, "law1")):
        m = M.hexa_impact_block(2000, seed=seed, law=law)
        for g in m.hexa:
            g.jcvt = 1
        corot.append(m)
    ms = corot + [M.crash_box(n_side=5, n_len=10, seed=23), M.hexa_impact_block(1500, seed=24)]
    n = 40
    got = run_batch(ms, prec, n)
    for i, m in enumerate(ms):
        e = Engine(m, precision=prec)
        e.cycle(n)
        assert close(got[i], state(e), TOL[prec]), i
    other = run_batch(ms, prec, n, (2, 4, 1, 1))
    for i in range(len(ms)):
        assert bitwise(other[i], got[i]), i


@pytest.mark.parametrize("prec", [0, 1])
def test_run_concurrent_equals_alone_bitwise(prec):
    """batch.run_concurrent advances every job on its own stream with its own
    graph: each ends bit for bit where the job run alone ends, with exactly
    its cycle count."""
    from openradioss_gb300.batch import run_concurrent
    from openradioss_gb300.engine import Engine
    ms = models_mix()
    es = [Engine(m, precision=prec) for m in ms]
    run_concurrent(es, 130, chunk=40)
    for m, e in zip(ms, es):
        alone = Engine(m, precision=prec)
        alone.cycle(130)
        assert bitwise(state(e), state(alone))
        assert e.status() == 0
        alone.close()
        e.close()
