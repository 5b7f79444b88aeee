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
displacements 1.3e-5, velocities 9e-4 absolute, on values of order 10).
"""
import os

import numpy as np
import pytest

from openradioss_gb300 import model as M

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "cra2.npz")


@pytest.fixture(scope="module")
def deck():
    return dict(np.load(FIX))


def printed_ok(ours, ref):
    """ours rounds to the 4-significant-digit printed value ref."""
    if ref == 0.0:
        return abs(ours) < 5e-4
    e = np.floor(np.log10(abs(ref)))
    half_unit = 0.5 * 10.0 ** (e - 3)
    return abs(ours - ref) <= half_unit * 1.02


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
    """Both engine runs of the deck through the oracle: per cycle the
    listing record and, before it, the nodal D and V (what the time history
    samples at that cycle)."""
    from oracle.oracle import OracleModel

    m = M.model_from_deck(deck, "cra2")
    o = OracleModel(m)
    o.set_record(True)
    tstop1, tstop2 = (float(t) for t in deck["run_tstop"])
    nid = deck["th_node_ids"] - 1
    recs = ([], [])
    nodes = ([], [])
    phase = 0
    while True:
        tt = o.time()["tt"]
        if phase == 0 and tt >= tstop1:
            o.clear_links()  # the restart deck has no /VEL card
            phase = 1
        if phase == 1 and tt >= tstop2:
            break
        nd = o.nodes()
        o.cycle(1)
        assert o.error() == 0
        recs[phase].append(o.record())
        nodes[phase].append(np.concatenate([nd["D"][:, nid].T, nd["V"][:, nid].T], axis=1))
    return recs, nodes


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
    recs, _ = run
    table = deck["out1" if phase == 0 else "out2"]
    for row in table:
        c = int(row[0])
        r = recs[phase][c]
        for key, col in (("tt", 1), ("dt2", 2), ("eint", 4), ("ekin", 5), ("ekinr", 6)):
            assert printed_ok(r[key], row[col]), (phase, c, key, r[key], row[col])
        assert r["neltst"] == int(row[3]), (phase, c, r["neltst"], row[3])


@pytest.mark.parametrize("phase", [0, 1])
def test_time_history(deck, run, phase):
    recs, nodes = run
    pre = "th1" if phase == 0 else "th2"
    th_t, th_g, th_n = deck[pre + "_time"], deck[pre + "_glob"], deck[pre + "_node"]
    tts = np.array([r["tt"] for r in recs[phase]], np.float32)
    cols = [str(c) for c in deck["th_glob_columns"]]
    tol = dict(IE=2e-6, KE=2e-7, XMOM=2e-7, MASS=1e-7, DT=3e-6, RKE=1e-4, HE=1e-5)
    key = dict(IE="eint", KE="ekin", XMOM="xmom", MASS="mass", DT="dt2", RKE="ekinr", HE="ehour")
    matched = 0
    for k, t in enumerate(th_t):
        # the time-history cycle: the one whose time matches the recorded
        # one (times agree to a small fraction of a step)
        c = int(np.argmin(np.abs(tts.astype(np.float64) - float(t))))
        assert abs(float(tts[c]) - float(t)) <= 1e-3 * recs[phase][c]["dt2"], (phase, k, t, tts[c])
        r = recs[phase][c]
        for name, rel in tol.items():
            ref = float(th_g[k][cols.index(name)])
            if ref != 0.0:
                assert abs(r[key[name]] - ref) <= rel * abs(ref), (phase, k, name, r[key[name]], ref)
        dn = np.abs(nodes[phase][c] - th_n[k])
        assert dn[:, :3].max() <= 5e-5, (phase, k, dn[:, :3].max())
        assert dn[:, 3:].max() <= 5e-3, (phase, k, dn[:, 3:].max())
        matched += 1
    assert matched == len(th_t) == 50


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
