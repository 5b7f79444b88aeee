"""FORINT-level call (rg_forint_step) with registered host buffers -- the
inputs read in place by the upload kernel, the outputs written in place by
the assembly -- against the same call with ordinary pageable buffers (staged
copies): bitwise equal forces, moments, stiffnesses and time step, for a
shell model (rotational slots) and a hexa model (its moments and rotational
stiffness come back zero), in both arithmetic forms."""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("kind", ["shell", "hexa"])
def test_forint_registered_equals_staged(kind, prec):
    from openradioss_gb300.engine import Engine
    m = (M.crash_box(n_side=5, n_len=10, vpert=1.0) if kind == "shell"
         else M.large_block(n=8, seed=2))
    runs = []
    for register in (False, True):
        e = Engine(m, precision=prec)
        e.cycle(10)
        nd = e.nodes()
        dt1 = e.time()["dt2"]
        n = m.numnod
        x = np.ascontiguousarray(nd["X"].T)
        v = np.ascontiguousarray(nd["V"].T)
        vr = np.ascontiguousarray(nd["VR"].T) if kind == "shell" else None
        f, st = np.full((n, 3), np.nan), np.full(n, np.nan)
        fr = np.full((n, 3), np.nan)
        sr = np.full(n, np.nan)
        bufs = [a for a in (x, v, vr, f, st, fr, sr) if a is not None]
        if register:
            for a in bufs:
                e.host_register(a)
        out = e.forint_step(x, v, dt1, vr=vr, f=f, stifn=st, fr=fr, stifr=sr)
        if register:
            for a in bufs:
                e.host_unregister(a)
        runs.append((f.copy(), st.copy(), None if fr is None else fr.copy(),
                     None if sr is None else sr.copy(), out[2], out[3]))
    a, b = runs
    assert np.all(np.isfinite(a[0])) and np.max(np.abs(a[0])) > 0
    for i in range(4):
        if a[i] is not None:
            assert np.array_equal(a[i], b[i]), i
    assert a[4] == b[4] and a[5] == b[5]
    if kind == "hexa":
        assert (a[2] == 0).all() and (a[3] == 0).all()


@pytest.mark.parametrize("registered", [True, False, "unaligned"])
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("kind", ["shell", "hexa"])
def test_cycle_host_equals_device_cycle(kind, prec, registered):
    """The whole-cycle call with host node buffers (rg_cycle_host), fed each
    cycle with its own previous output, follows the device-resident cycle:
    bitwise in the FP64 form (the upload writes back the same values),
    within the mixed form's tolerance there (its element volumes are
    re-anchored to the given coordinates), over 20 cycles, with the same
    time step sequence (FP64).  Registered buffers are read and written in
    place by the upload and download kernels; pageable ones go through the
    staging copies, and so do the outputs of registered buffers that are not
    16-byte aligned -- all give the same results."""
    from openradioss_gb300.engine import Engine
    m = (M.crash_box(n_side=5, n_len=10, vpert=1.0) if kind == "shell"
         else M.large_block(n=8, seed=2))
    n = m.numnod
    e1 = Engine(m, precision=prec)
    e2 = Engine(m, precision=prec)
    e1.cycle(5)
    e2.cycle(5)
    nd = e2.nodes()
    def buf(init):
        if registered != "unaligned":
            return np.ascontiguousarray(init)
        raw = np.empty(3 * n + 2)
        off = 1 if raw.ctypes.data % 16 == 0 else 0  # 8 bytes past a 16-byte boundary
        a = raw[off:off + 3 * n].reshape(n, 3)
        a[:] = init
        return a

    x = buf(nd["X"].T)
    v = buf(nd["V"].T)
    vr = buf(nd["VR"].T) if kind == "shell" else None
    d = buf(np.zeros((n, 3)))
    if registered == "unaligned":
        assert x.ctypes.data % 16 == 8
    bufs = [a for a in (x, v, vr, d) if a is not None] if registered else []
    for a in bufs:
        e2.host_register(a)
    for _ in range(20):
        e1.cycle(1)
        dt2 = e2.cycle_host(x, v, vr, x_out=x, v_out=v, vr_out=vr, d_out=d)
        if prec == 0:
            assert dt2 == e1.time()["dt2"]
    for a in bufs:
        e2.host_unregister(a)
    n1 = e1.nodes()
    if prec == 0:
        assert np.array_equal(x.T, n1["X"]) and np.array_equal(v.T, n1["V"])
        assert np.array_equal(d.T, n1["D"])
        if kind == "shell":
            assert np.array_equal(vr.T, n1["VR"])
    else:
        sd = np.max(np.abs(n1["X"] - m.X))
        assert np.max(np.abs(x.T - n1["X"])) <= 1e-4 * sd
        assert np.max(np.abs(v.T - n1["V"])) <= 1e-4 * np.max(np.abs(n1["V"]))
    assert e2.time()["ncycle"] == e1.time()["ncycle"] == 25
    assert e1.status() == 0 and e2.status() == 0
