"""FP64 shell groups larger than one wave of resident blocks (GPU).

A crash box of 41,600 shells (more than the 152 SMs x 2 blocks x 128
threads of one wave of the FP64 shell kernel, so blocks are scheduled in
several rounds) against the oracle -- forces of the first cycles within
1e-12, trajectories within 1e-10, time step and controlling element equal --
the same model stepped by the batched kernel (which writes the job's
time-step partials in its own tile layout) within 1e-10 of the single
model, and the FORINT-level call equal bit for bit to the device cycle.
"""
import numpy as np
import pytest

from openradioss_gb300 import model as M
from test_gpu_batch import close, run_batch, state

pytestmark = pytest.mark.gpu


def model():
    return M.crash_box(n_side=20, n_len=520, npt=5, vpert=0.5)


def rel(a, b):
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (s if s > 0 else 1.0))


def test_balanced_fp64_launch_matches_oracle(oracle_lib):
    from openradioss_gb300.engine import Engine

    m = model()
    assert m.numelc > 152 * 2 * 128
    e = Engine(m)
    o = oracle_lib.OracleModel(m)
    for _ in range(3):
        e.cycle(1)
        o.cycle(1)
        assert rel(e.forces()["F"], o.nodes()["F"]) < 1e-12
    e.cycle(20)
    o.cycle(20)
    ng, no = e.nodes(), o.nodes()
    assert rel(ng["X"] - m.X, no["X"] - m.X) < 1e-10
    assert rel(ng["V"], no["V"]) < 1e-10
    tg, to = e.time(), o.time()
    assert abs(tg["dt2"] - to["dt2"]) <= 1e-12 * to["dt2"]
    assert tg["neltst"] == to["neltst"]
    assert e.status() == 0


def test_batch_with_a_job_larger_than_one_wave():
    from openradioss_gb300.engine import Engine

    ms = [model(), M.hexa_impact_block(1500, seed=6, law="law1")]
    got = run_batch(ms, 0, 10)
    for i, m in enumerate(ms):
        e = Engine(m)
        e.cycle(10)
        assert close(got[i], state(e), 1e-10), i


def test_forint_step_matches_device_cycle_beyond_one_wave():
    """The FORINT-level call (warp tasks on the same layout) returns the
    device-resident cycle's assembled forces, moments, stiffness and element
    step bit for bit on the model larger than one wave."""
    from openradioss_gb300.engine import Engine

    m = model()
    e1 = Engine(m)
    e1.cycle(5)
    nd = e1.nodes()
    t = e1.time()
    e1.cycle(1)
    ref = e1.forces()
    e2 = Engine(m)
    e2.cycle(5)
    x = np.ascontiguousarray(nd["X"].T)
    v = np.ascontiguousarray(nd["V"].T)
    vr = np.ascontiguousarray(nd["VR"].T)
    fr = np.empty_like(x)
    sr = np.empty(m.numnod)
    f, st, dt2t, el = e2.forint_step(x, v, t["dt2"], vr=vr, fr=fr, stifr=sr)
    assert np.array_equal(f.T, ref["F"])
    assert np.array_equal(fr.T, ref["FR"])
    assert np.array_equal(st, ref["STIFN"])
    assert el == e1.time()["neltst"] and dt2t > 0
    e1.close()
    e2.close()
