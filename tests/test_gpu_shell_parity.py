"""GPU parity of the Belytschko-Tsay shell path (CFORC3 chain, LAW2,
PARITH/ON with rotational slots, sliding rigid wall) against the CPU oracle.
Tolerances as for the hexa path: forces of a cycle 1e-12, trajectories over
N cycles 1e-10 (relative to the max magnitude)."""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu


def rel(a, b):
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (s if s > 0 else 1.0))


@pytest.fixture(scope="module")
def Engine():
    from openradioss_gb300.engine import Engine
    return Engine


def test_shell_skyline_matches_oracle(Engine, oracle_lib):
    m = M.crash_box(n_side=4, n_len=6)
    e = Engine(m)
    o = oracle_lib.OracleModel(m, nthreads=2)
    a1, _, c1, l1 = e.skyline()
    a2, _, c2, l2 = o.skyline()
    assert l1 == l2 == 4 * m.numelc
    assert np.array_equal(a1, a2) and np.array_equal(c1, c2)


@pytest.mark.parametrize("iplas", [1, 0])
def test_crash_box_first_cycles(Engine, oracle_lib, iplas):
    # seeded velocity perturbation: the shells deform from the first cycle
    # (a rigid translation would leave only round-off forces to compare)
    m = M.crash_box(n_side=5, n_len=12, v0=40.0, vpert=2.0)
    m.shells[0].geo[38] = iplas
    e = Engine(m)
    o = oracle_lib.OracleModel(m, nthreads=2)
    for _ in range(3):
        e.cycle(1)
        o.cycle(1)
        fg, fo = e.forces(), o.nodes()
        assert rel(fg["F"], fo["F"]) < 1e-12
        assert rel(fg["FR"], fo["FR"]) < 1e-12
        assert rel(fg["STIFN"], fo["STIFN"]) < 1e-12
    tg, to = e.time(), o.time()
    assert abs(tg["dt2"] - to["dt2"]) <= 1e-12 * to["dt2"]
    assert tg["neltst"] == to["neltst"]


def test_crash_box_trajectory(Engine, oracle_lib):
    """Small crash box against the rigid wall, 400 cycles: plastic hinges
    form at the impacted end; trajectories, rotations, thickness, plastic
    strain and energies within 1e-10 / 1e-9."""
    m = M.crash_box(n_side=6, n_len=16, v0=15.0)
    e = Engine(m)
    o = oracle_lib.OracleModel(m, nthreads=2)
    for k in range(4):
        e.cycle(100)
        o.cycle(100)
        ng, no = e.nodes(), o.nodes()
        assert rel(ng["X"] - m.X, no["X"] - m.X) < 1e-10, k
        assert rel(ng["V"], no["V"]) < 1e-10, k
        assert rel(ng["VR"], no["VR"]) < 1e-9, k
    nc = m.numelc
    assert rel(e.shell_state(2, nc), o.shell_state(2, nc)) < 1e-10
    pg, po = e.shell_state(6, 5 * nc), o.shell_state(6, 5 * nc)
    assert po.max() > 0.0
    assert rel(pg, po) < 1e-8
    eg, eo = e.energy(), o.energy()
    for key in ("eint", "ekin", "ekinr", "ehour"):
        assert abs(eg[key] - eo[key]) <= 1e-9 * max(abs(eo[key]), 1e-12), key
    assert e.status() == 0


def test_shell_mixed_vs_fp64(Engine):
    """Mixed form on the crash box: displacement, peak force and internal
    energy within 1e-4 of the FP64 GPU path."""
    m = M.crash_box(n_side=8, n_len=24, v0=15.0)
    res = {}
    for prec in (0, 1):
        e = Engine(m, precision=prec)
        peak, eint = 0.0, []
        for _ in range(8):
            e.cycle(100)
            f = e.forces()["F"]
            peak = max(peak, float(np.max(np.linalg.norm(f, axis=0))))
            eint.append(e.energy()["eint"])
        res[prec] = (e.nodes()["D"], peak, np.array(eint))
    d64, p64, e64 = res[0]
    d32, p32, e32 = res[1]
    err_d = np.max(np.abs(d32 - d64)) / np.max(np.abs(d64))
    err_p = abs(p32 - p64) / p64
    err_e = np.max(np.abs(e32 - e64)) / np.max(np.abs(e64))
    print("shell mixed: displacement %.2e peak force %.2e internal energy %.2e" % (err_d, err_p, err_e))
    assert err_d < 1e-4 and err_p < 1e-4 and err_e < 1e-4


@pytest.mark.parametrize("ishfram,ithk,iplas,npt", [
    (2, 1, 1, 5), (2, 0, 0, 3), (0, 0, 1, 3), (2, 1, 0, 1), (0, 1, 1, 2)])
def test_formulation_combinations(Engine, oracle_lib, ishfram, ithk, iplas, npt):
    """The shell options one at a time and together (local frame 0 / 2,
    current / initial thickness, iterative / radial-return plasticity, 1-5
    points), on a deforming crash box against the oracle: first-cycle forces
    1e-12, 150-cycle trajectories 1e-10."""
    m = M.crash_box(n_side=5, n_len=12, v0=40.0, vpert=2.0, npt=npt)
    m.ishfram = ishfram
    g = m.shells[0]
    g.ithk = ithk
    g.geo[38] = iplas
    e = Engine(m)
    o = oracle_lib.OracleModel(m, nthreads=2)
    e.cycle(1)
    o.cycle(1)
    fg, fo = e.forces(), o.nodes()
    assert rel(fg["F"], fo["F"]) < 1e-12
    assert rel(fg["FR"], fo["FR"]) < 1e-12
    e.cycle(149)
    o.cycle(149)
    ng, no = e.nodes(), o.nodes()
    assert rel(ng["X"] - m.X, no["X"] - m.X) < 1e-10
    assert rel(ng["VR"], no["VR"]) < 1e-10
    # thickness (updated in both ITHK modes by the material)
    assert rel(e.shell_state(2, m.numelc), o.shell_state(2, m.numelc)) < 1e-10


@pytest.mark.parametrize("iplas,fisokin,rhocp,cc", [
    (2, 0.0, 0.0, 0.022),      # IPLA = 2: normal projection + radial return
    (0, 0.5, 0.0, 0.022),      # mixed hardening, radial return
    (1, 0.5, 0.0, 0.022),      # mixed hardening, plane-stress Newton
    (2, 1.0, 0.0, 0.0),        # kinematic hardening, IPLA = 2, no rate effect
    (1, 0.0, 3.6e5, 0.022),    # adiabatic heating and thermal softening
    (0, 0.3, 3.6e5, 0.0),      # heating without strain rate, with mixed hardening
])
def test_m2cplr_branches(Engine, oracle_lib, iplas, fisokin, rhocp, cc):
    """The M2CPLR branches beyond the benchmark's (IPLA = 2, kinematic and
    mixed hardening, Johnson-Cook thermal softening with adiabatic heating;
    m2cplr.F:115-121, 146-180, 289-490, sigeps02c.F:125, 226-229) on a
    deforming crash box against the oracle: first-cycle forces and moments
    1e-12, 150-cycle trajectories, thickness, back stress and temperature
    1e-10 (plastic strain 1e-8, as in the other shell tests)."""
    m = M.crash_box(n_side=5, n_len=12, v0=40.0, vpert=3.0, npt=5)
    g = m.shells[0]
    g.mat = M.law2(7850.0, 210e9, 0.3, 350e6, 275e6, 0.36, c=cc, eps0=1.0,
                   fisokin=fisokin, rhocp=rhocp, tmelt=800.0 if rhocp else 0.0)
    g.geo[38] = iplas
    e = Engine(m)
    o = oracle_lib.OracleModel(m, nthreads=2)
    e.cycle(1)
    o.cycle(1)
    fg, fo = e.forces(), o.nodes()
    assert rel(fg["F"], fo["F"]) < 1e-12
    assert rel(fg["FR"], fo["FR"]) < 1e-12
    e.cycle(149)
    o.cycle(149)
    ng, no = e.nodes(), o.nodes()
    nc = m.numelc
    assert rel(ng["X"] - m.X, no["X"] - m.X) < 1e-10
    assert rel(ng["VR"], no["VR"]) < 1e-10
    assert rel(e.shell_state(2, nc), o.shell_state(2, nc)) < 1e-10
    pg, po = e.shell_state(6, 5 * nc), o.shell_state(6, 5 * nc)
    assert po.max() > 0.0, "the case must yield"
    assert rel(pg, po) < 1e-8
    if fisokin > 0.0:
        bg, bo = e.shell_state(8, 15 * nc), o.shell_state(8, 15 * nc)
        assert np.max(np.abs(bo)) > 0.0
        assert rel(bg, bo) < 1e-10
    if rhocp > 0.0:
        tg, to = e.shell_state(9, 5 * nc), o.shell_state(9, 5 * nc)
        assert to.max() > 300.0 + 1.0, "adiabatic heating must raise the temperature"
        assert rel(tg - 300.0, to - 300.0) < 1e-10
    assert e.status() == 0
