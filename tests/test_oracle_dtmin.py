"""Time-step actions of /DT in the oracle (CPU): IDTMIN(3) for shells
(engine/source/elements/shell/coque/cdt3.F:77-141) and IDTMIN(11) for the
nodal time step (engine/source/time_step/dtnoda.F:258-305, 459-500).

* IDTMIN(3) = 2: every element whose step reaches DTMIN1(3) is deleted --
  OFF = 0 from then on, never switched back -- and the cycle's step is the
  minimum over the remaining elements, so it stays above DTMIN1(3);
* IDTMIN(3) = 1: the same elements only flag the stop (error bit 8), none
  is deleted;
* IDTMIN(11) = 3: nodes below DTMIN1(11) take the mass of a step DTMIN1(11)
  (1/2 STIFN (DTMIN1/DTFAC1)^2 * 1.00001): mass is added, only ever added,
  and from the cycle after the scaling the nodal step is back at or above
  DTMIN1(11) up to the stiffness change of one cycle.
"""
import numpy as np

from openradioss_gb300 import model as M

DTMIN_SHELL = 1.7386e-6


def test_shell_deletion():
    from oracle.oracle import OracleModel
    m = M.crash_box(n_side=6, n_len=16, v0=20.0, vpert=1.0)
    m.dtmin_actions = {3: (2, DTMIN_SHELL)}
    o = OracleModel(m)
    dead = np.zeros(m.numelc, bool)
    counts = []
    for _ in range(10):
        o.cycle(200)
        off = o.shell_state(4, m.numelc)
        now = off == 0
        assert not (dead & ~now).any()      # deleted elements stay deleted
        dead = now
        counts.append(int(dead.sum()))
        assert o.time()["dt2"] > DTMIN_SHELL
    assert 0 < counts[0] < counts[-1] < m.numelc
    assert o.error() == 0


def test_shell_stop_flag_deletes_nothing():
    from oracle.oracle import OracleModel
    m = M.crash_box(n_side=6, n_len=16, v0=20.0, vpert=1.0)
    m.dtmin_actions = {3: (1, DTMIN_SHELL)}
    o = OracleModel(m)
    o.cycle(5)
    assert o.error() & 8
    assert (o.shell_state(4, m.numelc) != 0).all()


def test_nodal_mass_scaling():
    from oracle.oracle import OracleModel
    m = M.hexa_impact_block(3000, seed=4, law="law2")
    m.nodal_dt = (0.9, 0.0)
    o = OracleModel(m)
    o.cycle(1)
    dtmin = 1.001 * o.time()["dt2"]
    m = M.hexa_impact_block(3000, seed=4, law="law2")
    m.nodal_dt = (0.9, dtmin)
    m.dtmin_actions = {11: (3, dtmin)}
    o = OracleModel(m)
    ms0 = o.mass()[0].copy()
    prev = ms0
    for k in range(5):
        o.cycle(40)
        ms = o.mass()[0]
        assert (ms >= prev).all()
        prev = ms.copy()
        assert o.time()["dt2"] > 0.999 * dtmin
    assert (ms > ms0).sum() > m.numnod // 2
    assert 0 < (ms.sum() - ms0.sum()) / ms0.sum() < 1e-2
    assert o.error() == 0
