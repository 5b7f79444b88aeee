"""Mixed form (FP32 element / FP64 nodal) against the plain FP64 form over
5,000 cycles, with printouts every 250 cycles: relative error of the final
displacement, of the peak impact force (the summed internal force of the
supported or wall-side nodes, the largest over the printouts), of the peak
nodal force and of the internal energy (largest over the printouts).

* elastic bar impact (16^3 LAW1 hexas, a smooth wave problem): every error
  within 1e-4;
* Johnson-Cook crash box of 8,000 shells hitting a rigid wall (buckling):
  this problem is sensitive to round-off -- the FP64 run itself, started
  from coordinates moved by one ulp, drifts from the unperturbed FP64 run.
  That drift is measured here too, and the mixed form's error must stay
  within 1e-4 or within three times the FP64 drift, whichever is larger.
"""
import copy

import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu

NCYC = 5000
EVERY = 250


def support(model):
    if model.hexa:
        return np.nonzero(model.icodt != 0)[0]
    z = model.X[2]
    return np.nonzero(z <= z.min() + 1e-9)[0]


def run(model, prec):
    from openradioss_gb300.engine import Engine
    e = Engine(model, precision=prec)
    sup = support(model)
    imp, fmax, eint = [], [], []
    for _ in range(NCYC // EVERY):
        e.cycle(EVERY)
        f = e.forces()["F"]
        imp.append(abs(float(f[2, sup].sum())))
        fmax.append(float(np.max(np.linalg.norm(f, axis=0))))
        eint.append(e.energy()["eint"])
    d = e.displacement()
    assert e.status() == 0
    e.close()
    return d, np.array(imp), np.array(fmax), np.array(eint)


def errors(a, b):
    """Relative errors of run b against run a."""
    da, ia, fa, ea = a
    db, ib, fb, eb = b
    return {"displacement": float(np.max(np.abs(db - da)) / np.max(np.abs(da))),
            "peak_impact_force": abs(ib.max() - ia.max()) / ia.max(),
            "peak_nodal_force": abs(fb.max() - fa.max()) / fa.max(),
            "internal_energy": float(np.max(np.abs(eb - ea)) / np.max(np.abs(ea)))}


def test_mixed_elastic_bar_5000_cycles():
    m = M.bar_impact(n=16)
    err = errors(run(m, 0), run(m, 1))
    print("bar 16^3, 5000 cycles, mixed vs FP64:", {k: "%.2e" % v for k, v in err.items()})
    for k, v in err.items():
        assert v <= 1e-4, (k, v)


def test_mixed_crash_box_5000_cycles_within_fp64_sensitivity():
    m = M.crash_box(n_side=20, n_len=100)
    mp = copy.deepcopy(m)
    mp.X = np.nextafter(m.X, np.inf)
    r64 = run(m, 0)
    err = errors(r64, run(m, 1))
    sens = errors(r64, run(mp, 0))
    print("crash box 8,000 shells, 5000 cycles, mixed vs FP64:",
          {k: "%.2e" % v for k, v in err.items()},
          "FP64 one-ulp drift:", {k: "%.2e" % v for k, v in sens.items()})
    for k, v in err.items():
        assert v <= max(1e-4, 3.0 * sens[k]), (k, v, sens[k])
