"""GPU parity against the CPU oracle on the benchmark workloads at their own
size (the FP64 plain form):

* crash box of 120,120 Johnson-Cook Belytschko-Tsay shells (NPT=5, Iplas=1,
  Ithick=1, planar rigid wall at 15 m/s): assembled forces, moments and nodal
  stiffness of each of the first 3 cycles within 1e-12; after 200 cycles the
  coordinates, velocities, rotational velocities, thickness and plastic
  strain within 1e-10, time step within 1e-12 and the controlling element
  equal;
* block of 128^3 = 2,097,152 Johnson-Cook one-point hexas (seeded velocity
  20 m/s + N(0, 0.5)): forces and stiffness of each of the first 3 cycles
  within 1e-12, coordinates and velocities after 20 cycles within 1e-10,
  stresses and time step likewise.

Relative errors are taken against the largest magnitude of each quantity,
as in the other parity tests (cforc3.F:85 / sforc3.F:60 are the routines
checked).  The oracle runs these sizes in seconds on the host's cores.
"""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu

TOL_FORCE = 1e-12
TOL_TRAJ = 1e-10


def rel(a, b):
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (s if s > 0 else 1.0))


def test_crash_box_120k_matches_oracle(oracle_lib):
    from openradioss_gb300.engine import Engine

    m = M.crash_box(n_side=77, n_len=390)
    assert m.numelc == 120120 and m.shells[0].npt == 5
    e = Engine(m)
    o = oracle_lib.OracleModel(m)
    for k in range(3):
        e.cycle(1)
        o.cycle(1)
        fg, fo = e.forces(), o.nodes()
        errs = (rel(fg["F"], fo["F"]), rel(fg["FR"], fo["FR"]), rel(fg["STIFN"], fo["STIFN"]))
        print("crash box cycle %d: F %.2e FR %.2e STIFN %.2e" % (k + 1, *errs))
        assert max(errs) < TOL_FORCE, (k, errs)
    e.cycle(197)
    o.cycle(197)
    ng, no = e.nodes(), o.nodes()
    nc = m.numelc
    errs = {
        "X": rel(ng["X"] - m.X, no["X"] - m.X),
        "V": rel(ng["V"], no["V"]),
        "VR": rel(ng["VR"], no["VR"]),
        "THK": rel(e.shell_state(2, nc) - m.shells[0].thk, o.shell_state(2, nc) - m.shells[0].thk),
        "PLA": rel(e.shell_state(6, 5 * nc), o.shell_state(6, 5 * nc)),
    }
    print("crash box after 200 cycles:", {k: "%.2e" % v for k, v in errs.items()})
    assert o.shell_state(6, 5 * nc).max() > 0.0, "the box must yield at the wall"
    for k, v in errs.items():
        assert v < TOL_TRAJ, (k, v)
    tg, to = e.time(), o.time()
    assert tg["ncycle"] == to["ncycle"] == 200
    assert abs(tg["dt2"] - to["dt2"]) <= 1e-12 * to["dt2"]
    assert tg["neltst"] == to["neltst"]
    assert e.status() == 0


def test_hexa_block_128_matches_oracle(oracle_lib):
    from openradioss_gb300.engine import Engine

    m = M.large_block(n=128)
    assert m.numels == 2097152
    e = Engine(m)
    o = oracle_lib.OracleModel(m)
    for k in range(3):
        e.cycle(1)
        o.cycle(1)
        fg, fo = e.forces(), o.nodes()
        errs = (rel(fg["F"], fo["F"]), rel(fg["STIFN"], fo["STIFN"]))
        print("hexa block cycle %d: F %.2e STIFN %.2e" % (k + 1, *errs))
        assert max(errs) < TOL_FORCE, (k, errs)
    e.cycle(17)
    o.cycle(17)
    ng, no = e.nodes(), o.nodes()
    errs = {"X": rel(ng["X"] - m.X, no["X"] - m.X), "V": rel(ng["V"], no["V"]),
            "SIG": rel(e.hexa_state(0), o.hexa_state(0))}
    print("hexa block after 20 cycles:", {k: "%.2e" % v for k, v in errs.items()})
    for k, v in errs.items():
        assert v < TOL_TRAJ, (k, v)
    tg, to = e.time(), o.time()
    assert tg["ncycle"] == to["ncycle"] == 20
    assert abs(tg["dt2"] - to["dt2"]) <= 1e-12 * to["dt2"]
    assert tg["neltst"] == to["neltst"]
    assert e.status() == 0
