"""The no-allocation kinetic-energy entry point (rg_kinetic_energy_noalloc)
called through the C ABI on device arrays: equal, within 1e-12 relative
(different fixed summation order), to the kinetic energy rg_energy reports
for the same model state, on two calls in a row (the shared scratch is
reused), and refusing sizes above its fixed scratch.  After the first call
(which may load the library's module onto the device) a further call leaves
the device's free memory unchanged: the point of the entry point is that it
allocates nothing.  Collected last so that it also runs after every other
test in the same process."""
import ctypes as C

import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu

TOL = 1e-12


def test_kinetic_energy_noalloc_matches_rg_energy():
    import torch
    from openradioss_gb300 import _lib
    from openradioss_gb300.engine import Engine
    L = _lib.lib()
    m = M.bar_impact(n=12)
    e = Engine(m)
    e.cycle(30)
    ref = e.energy()["ekin"]
    nd = e.nodes()
    assert ref > 0.0
    v = torch.tensor(np.ascontiguousarray(nd["V"].T).reshape(-1), dtype=torch.float64,
                     device="cuda:0")
    ms = torch.tensor(np.ascontiguousarray(m.MS, np.float64), dtype=torch.float64,
                      device="cuda:0")
    torch.cuda.synchronize()
    free = []
    for _ in range(2):
        out = C.c_double(-1.0)
        r = L.rg_kinetic_energy_noalloc(0, m.numnod, C.c_void_p(v.data_ptr()),
                                        C.c_void_p(ms.data_ptr()), C.byref(out))
        assert r == 0
        assert abs(out.value - ref) <= TOL * abs(ref), (out.value, ref)
        free.append(torch.cuda.mem_get_info(0)[0])
    # the second call took no device memory
    assert free[1] == free[0], free


def test_kinetic_energy_noalloc_refuses_oversize():
    from openradioss_gb300 import _lib
    L = _lib.lib()
    out = C.c_double(0.0)
    too_many = 65536 * 1024 + 1
    assert L.rg_kinetic_energy_noalloc(0, too_many, None, None, C.byref(out)) == -7
