"""The oracle's hexa path against the reference engine's outputs for its QA
deck H101 (CPU).

H101 (qa-tests/miniqa/SOLIDES/nv_elts/poutre_flex/flexion/H101): six elastic
cantilevers of one-point hexas (LAW1; Isolid = 1, co-rotational frame
Iframe = 2, viscous hourglass h = 0.1, qa = 1.1, qb = 0.05), meshed with 1,
2, 2, 5, 20 and 80 bricks, each with a rigid body at its free end loaded by a
constant 40000 along z; deflections reach 70 % of the span by the end of the
run (t = 0.002, 848 cycles).  What the reference wrote and the oracle must
reproduce:

* the starter's rigid-body set-up (main node moved to the centre of mass,
  mass, inertia tensor, principal inertia) and the total mass;
* every printed cycle of the engine listing to its printed digits: time,
  time step, internal, kinetic and rotational kinetic energy, external work,
  mass and the energy error;
* the time history every 1e-5: global energies (hourglass energy included),
  time step, mass, z momentum within 1e-6 relative, and the displacement and
  velocity of the six loaded main nodes within 1e-6 of their largest value.

Planted formulation changes (made in the oracle's input model: Jaumann rate
instead of the co-rotational frame, half the hourglass coefficient) must
break the match, so the deck pins those parts of the element.
"""
import numpy as np
import pytest

from h101_common import check_printed, check_time_history, load_deck, run
from openradioss_gb300 import model as M


@pytest.fixture(scope="module")
def deck():
    return load_deck()


def oracle_run(deck, edit=None):
    from oracle.oracle import OracleModel

    m = M.hexa_model_from_deck(deck, "h101")
    if edit:
        edit(m)
    o = OracleModel(m, nthreads=2)
    o.set_record(True)
    mains = np.array([b[0] for b in m.rbodies]) - 1

    def nodes_of():
        nd = o.nodes()
        return nd["D"][:, mains], nd["V"][:, mains]

    def step():
        o.cycle(1)
        return o.record()

    recs, nodes = run(deck, step, nodes_of, lambda: o.time()["tt"])
    assert o.error() == 0
    return m, recs, nodes, o.time()


@pytest.fixture(scope="module")
def result(deck):
    return oracle_run(deck)


def test_starter_rigid_bodies(deck):
    m = M.hexa_model_from_deck(deck, "h101")
    cols = [str(c) for c in deck["starter_rbody_columns"]]
    for (main, nodes, axes, inertia), row in zip(m.rbodies, deck["starter_rbody"]):
        r = dict(zip(cols, row))
        k = main - 1
        assert np.allclose(m.X[:, k], [r["x"], r["y"], r["z"]], rtol=1e-6, atol=1e-15)
        assert abs(m.MS[k] - r["mass"]) <= 1e-6 * r["mass"]
        assert np.allclose(np.sort(inertia)[::-1], [r["I1"], r["I2"], r["I3"]], rtol=1e-6)
        assert abs(m.IN[k] - min(r["I1"], r["I2"], r["I3"])) <= 1e-6 * m.IN[k]
        assert np.allclose(axes @ axes.T, np.eye(3), atol=1e-14) and np.linalg.det(axes) > 0
    # the listing's total mass counts each body once (its main node)
    sec = np.concatenate([b[1] for b in m.rbodies]) - 1
    total = m.MS.sum() - m.MS[sec].sum()
    assert abs(total - float(deck["starter_total_mass"])) <= 1e-9 * total


def test_printed_table(deck, result):
    m, recs, _, _ = result
    check_printed(deck, m, recs)


def test_time_history(deck, result):
    _, recs, nodes, _ = result
    check_time_history(deck, recs, nodes)


def test_cycle_count(deck, result):
    # 847 cycles carry the time past the end time; the reference's count of
    # 848 includes its final output pass at that time
    _, recs, _, t = result
    assert t["ncycle"] == 847 and t["tt"] >= float(deck["run_tstop"])


@pytest.mark.parametrize("change", ["jaumann", "hourglass"])
def test_planted_change_breaks_match(deck, change):
    def edit(m):
        for g in m.hexa:
            if change == "jaumann":
                g.jcvt = 0
            else:
                g.geo[12] = 0.05

    m, recs, nodes, _ = oracle_run(deck, edit)
    with pytest.raises(AssertionError):
        check_printed(deck, m, recs)
    with pytest.raises(AssertionError):
        check_time_history(deck, recs, nodes)


def test_external_forces_hook(deck):
    """or_set_forces (the hook the CUDA path's FORINT-level call feeds, see
    tests/test_gpu_h101.py): a second oracle that takes the first one's
    assembled element forces and element step every cycle instead of
    computing its own follows it bit for bit through the rigid bodies and
    loads."""
    from oracle.oracle import OracleModel

    a = OracleModel(M.hexa_model_from_deck(deck, "h101"), nthreads=1)
    m = M.hexa_model_from_deck(deck, "h101")
    b = OracleModel(m, nthreads=1)
    loaded = np.array([c[0] for c in m.cloads]) - 1
    for _ in range(200):
        a.cycle(1)
        nd, t = a.nodes(), a.time()
        f = nd["F"].T.copy()
        f[loaded] = 0.0          # F holds the loads; b adds its own
        b.set_forces(f, nd["STIFN"], t["dt2"], t["neltst"])
        b.cycle(1)
    na, nb = a.nodes(), b.nodes()
    assert np.array_equal(na["X"], nb["X"]) and np.array_equal(na["V"], nb["V"])
    assert np.array_equal(na["VR"], nb["VR"])
    assert a.time()["tt"] == b.time()["tt"]


def test_cuda_engine_refuses_rigid_bodies(deck):
    """The CUDA path does not run rigid bodies or concentrated loads: an
    Engine for such a model is refused unless it is opened for the
    FORINT-level call only (the caller runs the nodal update)."""
    from openradioss_gb300.engine import Engine, RgError

    with pytest.raises(RgError):
        Engine(M.hexa_model_from_deck(deck, "h101"))
