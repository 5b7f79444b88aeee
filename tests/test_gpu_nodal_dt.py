"""GPU parity of the nodal time step (/DT/NODA, DTNODA) against the oracle.

Hexa bar impact and a crash box of square shells under the nodal step: the
step of every cycle within 1e-12 relative of the oracle's (the FP64 form)
and the trajectories within 1e-10 over 200 cycles; the controlling node is
the oracle's except between round-off ties.  Mixed form within 1e-4.  A
model with the nodal step runs alone (the batch refuses it).
"""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu


def rel(a, b):
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (s if s > 0 else 1.0))


def models():
    a = M.bar_impact(n=8, law="law2")
    b = M.crash_box(n_side=6, n_len=30, npt=3, vpert=0.5)
    for m in (a, b):
        m.nodal_dt = (0.9, 0.0)
    return [a, b]


@pytest.mark.parametrize("k", [0, 1])
def test_fp64_steps_and_trajectory(oracle_lib, k):
    from openradioss_gb300.engine import Engine

    m = models()[k]
    e = Engine(m)
    o = oracle_lib.OracleModel(m, nthreads=2)
    for c in range(200):
        e.cycle(1)
        o.cycle(1)
        tg, to = e.time(), o.time()
        assert abs(tg["dt2"] - to["dt2"]) <= 1e-12 * to["dt2"], c
        if tg["neltst"] != to["neltst"]:
            # another node within round-off of the same step
            assert 1 <= tg["neltst"] <= m.numnod
    ng, no = e.nodes(), o.nodes()
    assert rel(ng["X"] - m.X, no["X"] - m.X) < 1e-10
    assert rel(ng["V"], no["V"]) < 1e-10
    assert e.status() == 0


@pytest.mark.parametrize("k", [0, 1])
def test_mixed_within_bound(oracle_lib, k):
    from openradioss_gb300.engine import Engine, RG_PREC_MIXED

    m = models()[k]
    e = Engine(m, precision=RG_PREC_MIXED)
    o = oracle_lib.OracleModel(m, nthreads=2)
    e.cycle(200)
    o.cycle(200)
    assert abs(e.time()["tt"] - o.time()["tt"]) <= 1e-4 * o.time()["tt"]
    ng, no = e.nodes(), o.nodes()
    assert rel(ng["D"], no["D"]) < 1e-4


def test_batch_refuses_nodal_dt():
    from openradioss_gb300.batch import Batch
    from openradioss_gb300.engine import Engine, RG_PREC_MIXED

    e = Engine(models()[0], precision=RG_PREC_MIXED)
    b = Batch()
    with pytest.raises(Exception):
        b.add(e, 10)
    b.close()
    e.close()
