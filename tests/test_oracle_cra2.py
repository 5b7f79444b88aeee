"""The oracle against the reference engine's own QA results (CPU).

Deck: the OpenRadioss QA model CRA2V44 (qa-tests/miniqa/RESTART/cra2), held
as numbers in tests/golden/cra2.npz by tests/golden/make_cra2.py: a U-section
channel of 768 Belytschko-Tsay shells (LAW2 Johnson-Cook, NPT = 3 radial
return, Ithick = 0, /SHFRA/V4 frame) crushed by a rigidly linked end with an
added mass of 500 t, run to t = 2.5 with the link and restarted to t = 5
without it (3375 cycles).

The reference values are what the reference engine wrote for that deck: its
printed cycle table (4 significant digits, every 100 cycles) and its time
history files (float32, every 0.05).  The oracle must reproduce the printed
table to the last printed digit, the controlling element of every printed
cycle and the time histories to within the tolerances below, which are a few
times the differences seen (IE 4e-7, KE 4e-8, DT 6e-7 relative; node
displacements 1.3e-5, velocities 9e-4 absolute, on values of order 10), and
the per-part time histories of the three parts (PART_TOL in cra2_common).
"""
import numpy as np
import pytest

from cra2_common import (check_part_history, check_printed, check_time_history, load_deck,
                         printed_ok, run_both)
from openradioss_gb300 import model as M


@pytest.fixture(scope="module")
def deck():
    return load_deck()


def test_deck_masses_match_starter(deck):
    m = M.model_from_deck(deck, "cra2")
    assert m.numelc == 768 and m.numnod == 850
    # total nodal mass: shell lumping + 500 t added mass, to the starter's
    # printed 13 digits
    assert abs(m.MS.sum() - float(deck["starter_total_mass"])) <= 1e-9 * float(deck["starter_total_mass"])
    for g, ref in zip(m.shells, deck["starter_part_mass"]):
        n = g.ixc[1:5] - 1
        p = [m.X[:, n[k]] for k in range(4)]
        area = 0.5 * np.linalg.norm(np.cross((p[2] - p[0]).T, (p[3] - p[1]).T), axis=1)
        mass = (g.mat["pm"][0] * g.thk * area).sum()
        assert abs(mass - ref) <= 1e-10 * ref
    # starter decisions for this deck
    assert all(g.npt == 3 and g.ithk == 0 and g.ismstr == 2 for g in m.shells)
    assert all(int(g.geo[38]) == 0 for g in m.shells)  # Iplas 0: radial return
    assert m.ishfram == 2 and len(m.rlinks) == 1 and m.rlinks[0][1] == 7


@pytest.fixture(scope="module")
def run(deck):
    """Both engine runs of the deck through the oracle."""
    from oracle.oracle import OracleModel

    o = OracleModel(M.model_from_deck(deck, "cra2"))
    o.set_record(True)

    def step():
        o.cycle(1)
        assert o.error() == 0
        r = o.record()
        r["parts"] = o.part_sums()
        return r

    def nodes_of():
        nd = o.nodes()
        return nd["D"], nd["V"]

    return run_both(deck, step, o.clear_links, nodes_of, lambda: o.time()["tt"])


def test_first_cycle_time_step(deck, run):
    recs, _ = run
    # starter: smallest shell time step; engine cycle 0: DTFAC 0.9 times it
    assert abs(recs[0][0]["dt2"] - 0.9 * float(deck["starter_shell_dt"])) <= 1e-12
    assert recs[0][0]["neltst"] == 1


def test_cycle_counts(deck, run):
    recs, _ = run
    # the restart run starts where the first one stopped: its cycle 0 is
    # printed at t = 2.501, and 1800 more printed cycles reach t = 4.987
    assert printed_ok(recs[1][0]["tt"], deck["out2"][0, 1])
    assert len(recs[1]) > int(deck["out2"][-1, 0])


@pytest.mark.parametrize("phase", [0, 1])
def test_printed_table(deck, run, phase):
    check_printed(deck, run[0], phase)


@pytest.mark.parametrize("phase", [0, 1])
def test_time_history(deck, run, phase):
    check_time_history(deck, run[0], run[1], phase)


@pytest.mark.parametrize("phase", [0, 1])
def test_part_time_history(deck, run, phase):
    """The per-part sums (CBILAN's PARTSAV with CHVIS3's hourglass energy)
    against the reference's /TH/PART outputs of the three parts: IE, KE,
    momentum, mass and hourglass energy at every time-history time."""
    check_part_history(deck, run[0], phase)


def test_part_history_detects_wrong_part_map(deck):
    """Planted in the oracle on the CPU: the shells' part numbers rotated
    (part p's elements counted in part p + 1) no longer match the
    reference's per-part outputs."""
    from oracle.oracle import OracleModel

    m = M.model_from_deck(deck, "cra2")
    o = OracleModel(m)
    o.set_record(True)
    part = np.concatenate([np.full(g.ixc.shape[1], (k + 1) % 3, np.int32)
                           for k, g in enumerate(m.shells)])
    o.set_parts(3, None, part)
    th_t, th_p = deck["th1_time"], deck["th1_part"]
    recs = []
    while o.time()["tt"] < float(th_t[3]) + 1e-9:
        o.cycle(1)
        r = o.record()
        r["parts"] = o.part_sums()
        recs.append(r)
    short = dict(deck)
    short["th1_time"], short["th1_part"] = th_t[:4], th_p[:4]
    with pytest.raises(AssertionError):
        check_part_history(short, (recs, []), 0)


def _printed_misses(deck, mutate, ncyc=1501):
    from oracle.oracle import OracleModel

    m = M.model_from_deck(deck, "cra2")
    mutate(m)
    o = OracleModel(m)
    o.set_record(True)
    table = deck["out1"]
    miss = 0
    for c in range(ncyc):
        o.cycle(1)
        row = table[table[:, 0] == c]
        if len(row):
            r = o.record()
            for key, col in (("tt", 1), ("dt2", 2), ("eint", 4), ("ekin", 5), ("ekinr", 6)):
                miss += not printed_ok(r[key], row[0][col])
    return miss


def _frame0(m):
    m.ishfram = 0


def _iterative_plasticity(m):
    for g in m.shells:
        g.geo[38] = 1.0


@pytest.mark.parametrize("mutate", [_frame0, _iterative_plasticity])
def test_table_detects_formulation_change(deck, mutate):
    """Planted in the oracle on the CPU: the symmetric frame instead of
    /SHFRA/V4, or iterative instead of radial-return plasticity, no longer
    reproduces the printed table -- the comparison has teeth."""
    assert _printed_misses(deck, mutate) >= 10
