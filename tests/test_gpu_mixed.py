"""Mixed form (FP32 element / material, FP64 nodal + energies) against the
FP64 GPU path: relative error of displacement, peak force and internal
energy within 1e-4 (the mixed form's stated tolerance)."""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu

TOL = 1e-4


def run(model, prec, ncycle, every):
    from openradioss_gb300.engine import Engine
    e = Engine(model, precision=prec)
    peak, eint = 0.0, []
    for _ in range(ncycle // every):
        e.cycle(every)
        f = e.forces()["F"]
        peak = max(peak, float(np.max(np.linalg.norm(f, axis=0))))
        eint.append(e.energy()["eint"])
    return e, peak, np.array(eint)


@pytest.mark.parametrize("wl", ["jc_block", "elastic_bar"])
def test_mixed_vs_fp64(wl):
    if wl == "jc_block":
        m = M.large_block(n=20, seed=1)
        ncyc = 600
    else:
        m = M.bar_impact(n=16)
        ncyc = 800
    e64, p64, ei64 = run(m, 0, ncyc, 50)
    e32, p32, ei32 = run(m, 1, ncyc, 50)
    d64, d32 = e64.nodes()["D"], e32.nodes()["D"]
    err_d = np.max(np.abs(d32 - d64)) / np.max(np.abs(d64))
    err_p = abs(p32 - p64) / p64
    err_e = np.max(np.abs(ei32 - ei64)) / np.max(np.abs(ei64))
    print(wl, "displacement %.2e peak force %.2e internal energy %.2e" % (err_d, err_p, err_e))
    assert err_d < TOL
    assert err_p < TOL
    assert err_e < TOL
    assert e32.status() == 0 and e64.status() == 0


def test_mixed_forint_step_tracks_cycle():
    """FORINT-level call in the mixed form: fed, call after call, the X, V
    and DT1 of a device-resident mixed run, it returns that run's assembled
    forces within the mixed tolerance (the element volume is re-anchored to
    the host coordinates on every call)."""
    from openradioss_gb300.engine import Engine
    m = M.large_block(n=10, seed=3)
    e1 = Engine(m, precision=1)
    e2 = Engine(m, precision=1)
    e1.cycle(20)
    e2.cycle(20)
    for _ in range(3):
        nd = e1.nodes()
        t = e1.time()
        e1.cycle(1)
        f_ref = e1.forces()["F"]
        x = np.ascontiguousarray(nd["X"].T)
        v = np.ascontiguousarray(nd["V"].T)
        f, st, dt2t, el = e2.forint_step(x, v, t["dt2"])
        err = np.max(np.abs(f.T - f_ref)) / np.max(np.abs(f_ref))
        assert err < TOL, err
