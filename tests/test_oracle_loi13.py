"""The oracle's Johnson-Cook hexa path against the reference engine's outputs
for its QA deck LOI13/solide (CPU).

LOI13 (qa-tests/miniqa/LOIS/LOI13/solide): a block of 464 one-point hexas of
/MAT/PLAS_JOHNS (LAW2, no strain-rate term; Isolid = 1, Iframe = 2: the
co-rotational frame, viscous hourglass h = 0.1, qa = 1.1, qb = 0.05) with
three /MAT/RIGID (LAW13) parts that the starter turns into rigid-material
bodies; the block's bottom is fixed and 44 top nodes follow an imposed
velocity ramp (/IMPVEL, 0 -> 5 over 100 time units) that crushes it
plastically: the internal energy reaches 3.1e5 over 1636 cycles (t = 8.01).
This is the Johnson-Cook radial return of the solid element (M2LAW,
engine/source/materials/mat/mat002/m2law.F:38-580) pinned to outputs of the
reference engine.  What the reference wrote and the oracle must reproduce:

* the starter's rigid-material bodies (RIGID_MAT: mass and centre of mass of
  each) and the total mass;
* every printed cycle of the engine listing to its printed digits: time,
  time step, controlling element, internal, kinetic and rotational kinetic
  energy, external work (the imposed velocity's), mass and energy error;
* the time history every 0.01: energies (hourglass energy included), time
  step and mass within 1e-6 relative, momenta within 1e-6 of their norm.

To run the deck the oracle restates, as test infrastructure only, the
rigid-material bodies (RIGID_MAT + ININODE_RM in the model builder; RMATPON,
RMATACCE, CONDRMAT in the oracle) and the imposed velocity (FIXVEL,
VINTERDP).  Planted changes (the Jaumann rate instead of the co-rotational
frame; a 2 % lower yield stress) must break the match.
"""
import numpy as np
import pytest

from loi13_common import check_printed, check_time_history, load_deck, run
from openradioss_gb300 import model as M


@pytest.fixture(scope="module")
def deck():
    return load_deck()


def oracle_run(deck, edit=None):
    from oracle.oracle import OracleModel

    m = M.rigid_jc_model_from_deck(deck, "loi13")
    if edit:
        edit(m)
    o = OracleModel(m, nthreads=2)
    o.set_record(True)

    def step():
        o.cycle(1)
        return o.record()

    recs = run(deck, step, lambda: o.time()["tt"])
    assert o.error() == 0
    return m, recs, o.time()


@pytest.fixture(scope="module")
def result(deck):
    return oracle_run(deck)


def test_starter_rigid_material_bodies(deck):
    m = M.rigid_jc_model_from_deck(deck, "loi13")
    off = deck["rm_offsets"]
    listed = [set(deck["rm_nodes"][off[k]:off[k + 1]].tolist()) for k in range(len(off) - 1)]
    assert len(m.rmats) == len(listed) == 3
    for nodes, xg, mass, axes, inertia in m.rmats:
        k = listed.index(set(int(deck["node_id"][n - 1]) for n in nodes))
        assert abs(mass - deck["rm_mass"][k]) <= 1e-6 * mass
        assert np.allclose(xg, deck["rm_com"][k], rtol=1e-6)
        assert np.allclose(axes @ axes.T, np.eye(3), atol=1e-14) and np.linalg.det(axes) > 0
        assert (inertia > 0).all()
    assert abs(m.MS.sum() - float(deck["starter_total_mass"])) <= 1e-12 * m.MS.sum()


def test_printed_table(deck, result):
    m, recs, _ = result
    check_printed(deck, m, recs)


def test_time_history(deck, result):
    _, recs, _ = result
    check_time_history(deck, recs)


def test_cycle_count(deck, result):
    _, recs, t = result
    assert t["ncycle"] == 1636 and t["tt"] >= float(deck["run_tstop"])


@pytest.mark.parametrize("change", ["jaumann", "yield"])
def test_planted_change_breaks_match(deck, change):
    def edit(m):
        for g in m.hexa:
            if change == "jaumann":
                g.jcvt = 0
            else:
                g.mat["pm"][37] *= 0.98
                g.mat["uparam"][0] *= 0.98
    m, recs, _ = oracle_run(deck, edit)
    with pytest.raises(AssertionError):
        check_printed(deck, m, recs)
