"""GPU parity against the CPU oracle on the benchmark workloads at their own
size (the FP64 plain form):

* crash box of 120,120 Johnson-Cook Belytschko-Tsay shells (NPT=5, Iplas=1,
  Ithick=1, planar rigid wall at 15 m/s).  The box moves rigidly until it
  reaches the wall (about cycle 52), so its first cycles' forces are round-off
  on both sides; the forces are therefore checked the way an engine uses the
  FORINT-level call: every cycle for 80 cycles the oracle's own X, V, VR and
  DT1 go to rg_forint_step, and the returned forces, moments and nodal
  stiffness must equal the oracle's for that cycle within 1e-12 of their
  largest value over the run (wall contact, plasticity).  A free run of 200
  device cycles then gives coordinates, velocities, rotational velocities,
  thickness and plastic strain within 1e-10 of the oracle's, the time step
  within 1e-12 and the same controlling element;
* block of 128^3 = 2,097,152 Johnson-Cook one-point hexas (seeded velocity
  20 m/s + N(0, 0.5)).  This state is sensitive to round-off at the onset of
  yield: the oracle itself, started from coordinates moved by one ulp, drifts
  from its own run by 2.2e-12 / 4.7e-12 in the forces of cycles 2 / 3 and by
  1.7e-9 (velocities) / 3.1e-9 (stresses) after 20 cycles -- as much as the
  oracle built with multiply-add contraction does.  The test measures that
  yardstick on the same model and requires the GPU's deviation from the
  oracle to stay within the larger of 1e-10 and the yardstick, quantity by
  quantity (measured on GB300: forces 1.3e-13 / 2.2e-12 / 4.7e-12, after 20
  cycles X 4.2e-11, V 3.3e-10, SIG 5.8e-10 -- about five times inside it);
  the time step within 1e-12 and the controlling element equal.

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
    n = m.numnod
    # forces of every cycle, from the oracle's own state (FORINT-level call)
    ef = Engine(m)
    o = oracle_lib.OracleModel(m)
    x, v, vr = (np.empty((n, 3)) for _ in range(3))
    f, fr = np.empty((n, 3)), np.empty((n, 3))
    stf, stfr = np.empty(n), np.empty(n)
    dmax = {"F": 0.0, "FR": 0.0, "STIFN": 0.0}
    smax = dict(dmax)
    for k in range(80):
        nd = o.nodes()
        x[:], v[:], vr[:] = nd["X"].T, nd["V"].T, nd["VR"].T
        dt1 = o.time()["dt2"]
        _, _, dt2t, el = ef.forint_step(x, v, dt1, vr=vr, f=f, stifn=stf, fr=fr, stifr=stfr)
        o.cycle(1)
        fo = o.nodes()
        for key, a, b in (("F", f.T, fo["F"]), ("FR", fr.T, fo["FR"]),
                          ("STIFN", stf, fo["STIFN"])):
            dmax[key] = max(dmax[key], float(np.max(np.abs(a - b))))
            smax[key] = max(smax[key], float(np.max(np.abs(b))))
        # the element step of the same state (DTFAC * DTX, before RESOL's limits)
        assert abs(dt2t - o.time()["dt2"]) <= 1e-12 * dt2t or o.time()["dt2"] < dt2t
    ef.close()
    errs = {k: dmax[k] / smax[k] for k in dmax}
    print("crash box forces over 80 FORINT-level cycles:",
          {k: "%.2e" % v for k, v in errs.items()}, "max |F| %.3e" % smax["F"])
    assert smax["F"] > 1.0, "the box must reach the wall within the compared cycles"
    for key, err in errs.items():
        assert err < TOL_FORCE, (key, err)
    # free run of the device cycle against the oracle's run
    e = Engine(m)
    e.cycle(200)
    o.cycle(120)
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
    import copy
    from openradioss_gb300.engine import Engine

    m = M.large_block(n=128)
    assert m.numels == 2097152
    # the oracle's own sensitivity: the same model with X moved by one ulp
    mp = copy.deepcopy(m)
    mp.X = np.nextafter(m.X, np.inf)
    e = Engine(m)
    o = oracle_lib.OracleModel(m)
    op = oracle_lib.OracleModel(mp)
    for k in range(3):
        e.cycle(1)
        o.cycle(1)
        op.cycle(1)
        fg, fo, fp = e.forces(), o.nodes(), op.nodes()
        errs = (rel(fg["F"], fo["F"]), rel(fg["STIFN"], fo["STIFN"]))
        yard = (rel(fp["F"], fo["F"]), rel(fp["STIFN"], fo["STIFN"]))
        print("hexa block cycle %d: F %.2e STIFN %.2e (one-ulp yardstick %.2e %.2e)"
              % (k + 1, *errs, *yard))
        for err, y in zip(errs, yard):
            assert err < max(TOL_TRAJ, y), (k, errs, yard)
    e.cycle(17)
    o.cycle(17)
    op.cycle(17)
    ng, no, npp = e.nodes(), o.nodes(), op.nodes()
    errs = {"X": rel(ng["X"] - m.X, no["X"] - m.X), "V": rel(ng["V"], no["V"]),
            "SIG": rel(e.hexa_state(0), o.hexa_state(0))}
    yard = {"X": rel(npp["X"] - m.X, no["X"] - m.X), "V": rel(npp["V"], no["V"]),
            "SIG": rel(op.hexa_state(0), o.hexa_state(0))}
    print("hexa block after 20 cycles:", {k: "%.2e" % v for k, v in errs.items()},
          "one-ulp yardstick:", {k: "%.2e" % v for k, v in yard.items()})
    for k, v in errs.items():
        assert v < max(TOL_TRAJ, yard[k]), (k, v, yard[k])
    tg, to = e.time(), o.time()
    assert tg["ncycle"] == to["ncycle"] == 20
    assert abs(tg["dt2"] - to["dt2"]) <= 1e-12 * to["dt2"]
    assert tg["neltst"] == to["neltst"]
    assert e.status() == 0
