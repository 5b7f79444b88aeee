"""Time-step actions of /DT on the GPU (rg_set_dtmin) against the oracle:

* shells, IDTMIN(3) = 2 (cdt3.F:93-109): the same elements are deleted in
  the same cycles (OFF arrays equal at every printout) and the run follows
  the oracle's (FP64 form, trajectories within 1e-10 of the largest
  displacement); the mixed form deletes elements too and keeps its step
  above DTMIN1(3);
* shells, IDTMIN(3) = 1: RG_ST_DTMIN is raised, nothing is deleted;
* nodal time step, IDTMIN(11) = 3 (dtnoda.F:268-305): the nodal masses
  after scaling equal the oracle's to round-off, the added mass shows in
  the energy balance (mass error > 0) and the trajectories follow the
  oracle's;
* refused actions (IDTMIN(3) = 3, IDTMIN(11) = 4) and a batch job with an
  action are refused.
"""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu

DTMIN_SHELL = 1.7386e-6


def box(idtmin):
    m = M.crash_box(n_side=6, n_len=16, v0=20.0, vpert=1.0)
    m.dtmin_actions = {3: (idtmin, DTMIN_SHELL)}
    return m


def test_shell_deletion_matches_oracle():
    from openradioss_gb300.engine import Engine
    from oracle.oracle import OracleModel
    m = box(2)
    e, o = Engine(m, precision=0), OracleModel(m)
    counts = []
    for _ in range(8):
        e.cycle(200)
        o.cycle(200)
        og = e.shell_state(4, m.numelc)
        oo = o.shell_state(4, m.numelc)
        assert np.array_equal(og == 0, oo == 0)
        counts.append(int((og == 0).sum()))
        xg, xo = e.nodes()["X"], o.nodes()["X"]
        d = np.max(np.abs(xo - m.X))
        assert np.max(np.abs(xg - xo)) <= 1e-10 * max(d, 1e-30)
        assert e.time()["dt2"] > DTMIN_SHELL
    assert 0 < counts[0] < counts[-1] < m.numelc
    assert e.status() == 0


def test_shell_deletion_mixed_form():
    from openradioss_gb300.engine import Engine
    m = box(2)
    e = Engine(m, precision=1)
    e.cycle(1000)
    off = e.shell_state(4, m.numelc)
    assert 0 < int((off == 0).sum()) < m.numelc
    assert e.time()["dt2"] > DTMIN_SHELL
    assert e.status() == 0


def test_shell_stop_flag():
    from openradioss_gb300.engine import ST_DTMIN, Engine
    for prec in (0, 1):
        e = Engine(box(1), precision=prec)
        e.cycle(5)
        assert e.status() & ST_DTMIN
        assert (e.shell_state(4, e.model.numelc) != 0).all()


def test_nodal_mass_scaling_matches_oracle():
    from openradioss_gb300.engine import Engine
    from oracle.oracle import OracleModel
    m0 = M.hexa_impact_block(3000, seed=4, law="law2")
    m0.nodal_dt = (0.9, 0.0)
    o0 = OracleModel(m0)
    o0.cycle(1)
    dtmin = 1.001 * o0.time()["dt2"]
    m = M.hexa_impact_block(3000, seed=4, law="law2")
    m.nodal_dt = (0.9, dtmin)
    m.dtmin_actions = {11: (3, dtmin)}
    e, o = Engine(m, precision=0), OracleModel(m)
    mass0 = float(m.MS.sum())
    for _ in range(4):
        e.cycle(50)
        o.cycle(50)
        b = e.energy_balance()
        ms = o.mass()[0]
        assert abs(b["mass"] - ms.sum()) <= 1e-12 * ms.sum()
        assert b["mass_error"] > 0.0
        assert abs(b["mass_error"] - (ms.sum() - mass0) / mass0) <= 1e-9
        xg, xo = e.nodes()["X"], o.nodes()["X"]
        d = np.max(np.abs(xo - m.X))
        assert np.max(np.abs(xg - xo)) <= 1e-10 * d
    assert e.status() == 0
    em = Engine(m, precision=1)
    em.cycle(200)
    assert em.energy_balance()["mass_error"] > 0.0 and em.status() == 0


def test_refused_actions():
    from openradioss_gb300.engine import Engine, RgError
    for acts in ({3: (3, 1e-6)}, {11: (4, 1e-6)}, {7: (2, 1e-6)}):
        m = M.crash_box(n_side=6, n_len=16)
        m.dtmin_actions = acts
        with pytest.raises(RgError):
            Engine(m)


def test_batch_refuses_dtmin_action():
    from openradioss_gb300.batch import Batch
    from openradioss_gb300.engine import Engine, RgError
    b = Batch()
    e = Engine(box(2), precision=1)
    with pytest.raises(RgError):
        b.add(e, 100)
    b.close()
