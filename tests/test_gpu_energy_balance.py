"""Energy balance of the listing's cycle line (rg_energy_balance), the
counterpart of ECRIT (engine/source/output/ecrit.F:501-517) with the rigid
walls' external work of RGWAL0 (engine/source/constraints/general/rwall/
rgwal0.F, TFEXT), against the oracle run on the same model:

* internal, kinetic and rotational energy, the walls' external work WFEXT,
  mass and momentum agree with the oracle's to round-off of the summation
  order (FP64 form);
* ENTOT = IE + KE + KE-R, the energy error 100 (ENTOT / (ENTOT0 + WFEXT) - 1)
  with ENTOT0 taken at rg_finalize, and the mass error (zero here: no mass
  is added) follow from those values as in ECRIT;
* the wall does negative work on the crash box (it takes kinetic energy
  out), and the balance stays within a few percent;
* the balance survives a snapshot / restore unchanged.
"""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu


def oracle_balance(o, m, entot0, mass0):
    en = o.energy()
    nd = o.nodes()
    ms = m.MS
    entot = en["eint"] + en["ekin"] + en["ekinr"]
    w = o.wfext()
    return dict(eint=en["eint"], ekin=en["ekin"], ekinr=en["ekinr"], ehour=en["ehour"],
                wfext=w, entot=entot, error_pct=100.0 * (entot / (entot0 + w) - 1.0),
                mass=float(ms.sum()), mass_error=(float(ms.sum()) - mass0) / mass0,
                xmom=float((ms * nd["V"][0]).sum()), ymom=float((ms * nd["V"][1]).sum()),
                zmom=float((ms * nd["V"][2]).sum()))


@pytest.mark.parametrize("kind", ["shell", "hexa"])
def test_energy_balance_matches_oracle(kind):
    from openradioss_gb300.engine import Engine
    from oracle.oracle import OracleModel
    m = (M.crash_box(n_side=6, n_len=16, v0=20.0, vpert=1.0) if kind == "shell"
         else M.hexa_impact_block(3000, seed=4, law="law2"))
    e = Engine(m, precision=0)
    o = OracleModel(m)
    b0 = e.energy_balance()
    en0 = o.energy()
    entot0 = en0["eint"] + en0["ekin"] + en0["ekinr"]
    mass0 = float(m.MS.sum())
    assert abs(b0["entot"] - entot0) <= 1e-12 * entot0
    assert b0["wfext"] == 0.0 and b0["error_pct"] == 0.0 and b0["mass_error"] == 0.0
    for _ in range(6):
        e.cycle(300)
        o.cycle(300)
        g = e.energy_balance()
        r = oracle_balance(o, m, entot0, mass0)
        tt = o.time()["tt"]
        assert abs(g["tt"] - tt) <= 1e-12 * tt
        for k in ("eint", "ekin", "ekinr", "ehour", "entot", "mass"):
            assert abs(g[k] - r[k]) <= 1e-10 * max(abs(r[k]), 1e-30 + 1e-6 * entot0), (k, g[k], r[k])
        assert abs(g["wfext"] - r["wfext"]) <= 1e-10 * entot0, (g["wfext"], r["wfext"])
        assert abs(g["error_pct"] - r["error_pct"]) <= 1e-8
        assert g["mass_error"] == 0.0
        pnorm = float(np.sqrt(2.0 * mass0 * entot0))
        for k in ("xmom", "ymom", "zmom"):
            assert abs(g[k] - r[k]) <= 1e-10 * pnorm, (k, g[k], r[k])
        # ECRIT's ENTOT leaves out the hourglass energy: the viscous
        # hourglass of the randomly moving block dissipates a few percent
        assert abs(g["error_pct"]) < 10.0
    if kind == "shell":
        assert g["wfext"] < 0.0
    assert e.status() == 0


def test_energy_balance_survives_restore():
    from openradioss_gb300.engine import Engine
    m = M.crash_box(n_side=6, n_len=16, v0=20.0, vpert=1.0)
    e = Engine(m, precision=1)
    e.cycle(200)
    snap = e.snapshot()
    e.cycle(200)
    a = e.energy_balance()
    e2 = Engine(m, precision=1)
    e2.restore(snap)
    e2.cycle(200)
    b = e2.energy_balance()
    assert a == b
