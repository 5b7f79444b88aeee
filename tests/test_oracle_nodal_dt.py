"""Known answers of the nodal time step (/DT/NODA, DTNODA) in the oracle
(CPU).

With /DT/NODA the elements give only stiffness (hexa STI of MQVISCB, shell
STI / STIR of CHVIS3's nodal branch) and the step is the minimum over nodes
of DTFAC1(11)*sqrt(2*MS/STIFN) (and 2*IN/STIFR for shell nodes):

* regular hexa mesh: every node's step equals the element step
  DTFAC*DELTAX/SSP_EQ (each node collects MS = sum rho V / 8 and
  STIFN = sum STI / 4 with the same STI = rho V / DTX^2), so the first
  cycle's step is the element one (to round-off);
* regular flat shell mesh (first cycle, no hourglass term): STI = t A11 / 2
  per element, so every node's step is DTFAC * h * sqrt(rho (1 - nu^2) / E),
  the plate wave speed -- sqrt(1 - nu^2) of the element step -- and the
  rotational step is the same;
* the run stays energy-bounded under the nodal step (see the last test for
  elongated shells).
"""
import numpy as np
import pytest

from openradioss_gb300 import model as M


@pytest.fixture(scope="module")
def O():
    from oracle.oracle import OracleModel
    return OracleModel


def flat_plate(n=6, h=0.01, t=0.002, rho=7850.0, E=210e9, nu=0.3, npt=3):
    """n x n square shells of side h in the z=0 plane, at rest."""
    g = np.arange(n + 1)
    gy, gx = np.meshgrid(g, g, indexing="ij")
    X = np.stack([h * gx.ravel(), h * gy.ravel(), np.zeros(gx.size)]).astype(np.float64)
    nid = lambda i, j: j * (n + 1) + i
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    ii, jj = ii.ravel(), jj.ravel()
    conn = np.stack([nid(ii, jj), nid(ii + 1, jj), nid(ii + 1, jj + 1), nid(ii, jj + 1)])
    nel = conn.shape[1]
    ixc = np.zeros((7, nel), np.int32)
    ixc[0] = 1
    ixc[1:5] = conn + 1
    ixc[5] = 1
    ixc[6] = np.arange(1, nel + 1)
    thk = np.full(nel, t)
    mat = M.law2(rho, E, nu, 350e6, 275e6, 0.36)
    ms, inr = M.shell_mass_inertia(X, ixc, thk, rho)
    m = M.Model("plate", X, np.zeros_like(X), ms, np.zeros(X.shape[1], np.int32),
                shells=[M.ShellGroupSpec(ixc, mat, M.shell_prop(t), thk, npt)], IN=inr)
    return m


def test_hexa_regular_mesh_nodal_equals_element(O):
    a = O(M.bar_impact(n=4), nthreads=1)
    m = M.bar_impact(n=4)
    m.nodal_dt = (0.9, 0.0)
    b = O(m, nthreads=1)
    a.cycle(1)
    b.cycle(1)
    ta, tb = a.time(), b.time()
    assert abs(tb["dt2"] - ta["dt2"]) <= 1e-13 * ta["dt2"]
    # the controlling entity is a node (equal steps up to round-off)
    assert 1 <= tb["neltst"] <= m.numnod
    assert b.error() == 0


def test_shell_regular_plate_plate_wave_speed(O):
    h, rho, E, nu = 0.01, 7850.0, 210e9, 0.3
    m = flat_plate(h=h, rho=rho, E=E, nu=nu)
    m.nodal_dt = (0.9, 0.0)
    o = O(m, nthreads=1)
    o.cycle(1)
    t = o.time()
    expect = 0.9 * h * np.sqrt(rho * (1.0 - nu * nu) / E)
    assert abs(t["dt2"] - expect) <= 1e-12 * expect
    assert 1 <= t["neltst"] <= m.numnod
    # the element step of the same plate is sqrt(1 - nu^2) larger
    e = O(flat_plate(h=h, rho=rho, E=E, nu=nu), nthreads=1)
    e.cycle(1)
    assert abs(t["dt2"] / e.time()["dt2"] - np.sqrt(1.0 - nu * nu)) <= 1e-12
    assert o.error() == 0


def test_nodal_dt_run_is_stable(O):
    """Energy stays bounded: hexa bar and a crash box of square shells at
    DTFAC 0.9; a crash box of 1.5-aspect shells at DTFAC 0.6 (the shell nodal
    stiffness max(B1,B2) t A11 / A gives an a x b element the step
    a b sqrt(2 / (a^2 + b^2)) / c, above the element step for aspect ratios
    past about 1.3, and at DTFAC 0.9 that box gains energy)."""
    cases = ((M.bar_impact(n=6, law="law2"), 0.9),
             (M.crash_box(n_side=6, n_len=30, npt=3, vpert=0.5), 0.9),
             (M.crash_box(n_side=6, n_len=20, npt=3, vpert=0.5), 0.6))
    for m, dtfac in cases:
        m.nodal_dt = (dtfac, 0.0)
        o = O(m, nthreads=2)
        e0 = o.energy()
        tot0 = e0["ekin"] + e0["ekinr"]
        o.cycle(400)
        e = o.energy()
        assert o.error() == 0
        assert np.isfinite(e["ekin"]) and e["eint"] + e["ekin"] <= 1.05 * tot0 + 1e-9
