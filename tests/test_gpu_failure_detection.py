"""Failure detection on the GPU, every failure made on the host (no GPU fault,
no trap, no unbounded wait):

* an element folded inside out by the coordinates handed to the FORINT-level
  call raises RG_ST_NEGVOL and that element is switched off (OFF = 0), as
  SCHKJAB3 does (engine/source/elements/solid/solide/schkjab3.F:39);
* a minimum time step above the computed one raises RG_ST_DTMIN
  (DTNODA's DTMIN1 test, engine/source/time_step/dtnoda.F:258-266);
* a non-finite initial velocity raises RG_ST_NAN;
* the batched kernel's grid barrier, given a short wait limit while one block
  is made to arrive late, gives up: RG_ST_BARRIER is recorded, the kernel
  returns, and the next cycle runs clean;
* the serving loop retires a job whose status is raised as failed while the
  other jobs finish with the results they have alone.
"""
import time

import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu

ST_NEGVOL, ST_NAN, ST_DTMIN, ST_BARRIER = 1, 2, 8, 16


@pytest.mark.parametrize("prec", [0, 1])
def test_folded_element_raises_negvol_and_is_switched_off(prec):
    from openradioss_gb300.engine import Engine
    m = M.bar_impact(n=3)
    e = Engine(m, precision=prec)
    e.cycle(2)
    assert e.status() == 0
    nd = e.nodes()
    x = np.ascontiguousarray(nd["X"].T)
    v = np.ascontiguousarray(nd["V"].T)
    # node 1 belongs to element 1 only: move it past the element's far corner
    x[0] = [0.012, 0.012, 0.012]
    e.forint_step(x, v, e.time()["dt2"])
    assert e.status() & ST_NEGVOL
    off = e.hexa_state(4)
    assert off[0] == 0.0
    assert np.all(off[1:] == 1.0)
    assert e.status() == 0  # the read cleared the word


@pytest.mark.parametrize("shell", [False, True])
def test_step_below_dtmin_raises_status(shell):
    from openradioss_gb300.engine import Engine
    m = M.crash_box(n_side=4, n_len=6) if shell else M.bar_impact(n=4)
    m.nodal_dt = (0.9, 1.0)  # DTMIN1(11) = 1 s: far above any step of the model
    e = Engine(m)
    e.cycle(1)
    assert e.status() & ST_DTMIN
    m.nodal_dt = (0.9, 0.0)
    e2 = Engine(m)
    e2.cycle(3)
    assert e2.status() == 0


@pytest.mark.parametrize("prec", [0, 1])
def test_nan_velocity_raises_status(prec):
    from openradioss_gb300.engine import Engine
    m = M.bar_impact(n=4)
    m.V[0, 40] = np.nan
    e = Engine(m, precision=prec)
    e.cycle(2)
    assert e.status() & ST_NAN


def test_grid_barrier_gives_up_and_batch_stays_usable():
    from openradioss_gb300.batch import Batch
    from openradioss_gb300.engine import Engine
    es = [Engine(M.crash_box(n_side=4, n_len=8, seed=3)),
          Engine(M.hexa_impact_block(1200, seed=4, law="law1"))]
    b = Batch(0)
    for e in es:
        b.add(e)
    b.set_config(ktile=1, knode=1, blocks_per_sm=0, schedule=0)  # one cooperative launch
    b.cycle(1)
    b.sync()
    assert b.progress()[1] == 0
    # ~1 ms wait limit; block 0 arrives 20 ms late at each barrier
    b.set_barrier_test(spin_limit=1 << 10, late_block=0, late_us=20000)
    t0 = time.perf_counter()
    b.cycle(1)
    b.sync()
    assert time.perf_counter() - t0 < 30.0
    assert b.progress()[1] & ST_BARRIER
    b.set_barrier_test()
    b.cycle(2)
    b.sync()
    assert b.progress()[1] == 0
    b.close()
    for e in es:
        e.close()


def test_serving_retires_failed_job_and_others_match_alone():
    from openradioss_gb300.engine import Engine
    from openradioss_gb300.serving import Server
    bad = M.hexa_impact_block(2000, seed=22, law="law2")
    bad.V[2, 100] = np.nan
    jobs = [(0, M.crash_box(n_side=5, n_len=10, seed=21), 100, 0.0),
            (1, bad, 100, 0.0),
            (2, M.hexa_impact_block(1500, seed=23, law="law1"), 75, 0.0)]
    srv = Server(1 << 34, max_jobs=8, precision=1, step_cycles=25, keep_results=True,
                 executor="batch")
    st = srv.run(jobs)
    srv.close()
    assert st["failed"] == 1 and st["completed"] == 2
    assert [r.key for r in srv.failed] == [1] and srv.failed[0].status & ST_NAN
    for rec in srv.done:
        _, m, n, _ = jobs[rec.key]
        ref = Engine(m, precision=1)
        ref.cycle(n)
        nd = ref.nodes()
        assert rec.result["time"]["ncycle"] == n
        sd = np.max(np.abs(nd["X"] - m.X))
        assert np.max(np.abs(rec.result["X"] - nd["X"])) <= 1e-4 * sd, rec.key
        assert np.max(np.abs(rec.result["V"] - nd["V"])) <= 1e-4 * np.max(np.abs(nd["V"]))
        assert rec.result["status"] == 0
